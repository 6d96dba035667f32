/*
 * fastkpm_gb300.h -- C ABI of the GB300 stochastic Chebyshev (KPM) engine.
 *
 * Plain C types only: opaque handles, pointers, sizes, int status codes. Host
 * buffers are caller-owned and only read/written during the call; device
 * buffers are owned by the engine. Every call returns FK_OK or an FK_ERR_*
 * code; nothing aborts. fk_engine_last_error() gives a one-line reason.
 *
 * Value arrays are real doubles, or interleaved (re, im) double pairs when the
 * engine was created with FK_COMPLEX. Probe matrices are column-major n x s
 * (the layout of arma::Mat<T> R, reference src/fastkpm.h:188). BSR blocks are
 * column-major b x b (reference src/fastkpm.h:64-65).
 *
 * The reference has no C ABI of its own; its hot path is the C++ class
 * fkpm::Engine<T> (reference src/fastkpm.h:185-234). Each entry point below
 * names the Engine<T> member it carries out; include/fastkpm.h implements
 * Engine<T> on top of these calls.
 */
#ifndef FASTKPM_GB300_H
#define FASTKPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define FK_OK              0
#define FK_ERR_ARG         1   /* invalid argument (size, order, pointer)                 */
#define FK_ERR_OOM         2   /* device allocation failed / admission refused by memory   */
#define FK_ERR_PATTERN     3   /* malformed BSR pattern (unsorted, out of range, asymmetric D) */
#define FK_ERR_TIMEOUT     4   /* bounded wait expired                                      */
#define FK_ERR_CUDA        5   /* CUDA runtime error                                        */
#define FK_ERR_STATE       6   /* call order violated (e.g. autodiff without moments(M))    */
#define FK_ERR_NODEV       7   /* no usable CUDA device                                     */
#define FK_ERR_UNSUPPORTED 8   /* valid request outside what this library implements        */

/* ---- value kinds at the boundary ---- */
#define FK_REAL    0   /* double                          */
#define FK_COMPLEX 1   /* complex double, (re, im) pairs  */

/* ---- recursion precision (what the kernels store and compute in) ---- */
#define FK_PREC_FP64 0   /* native IEEE double                                              */
#define FK_PREC_FP32 1   /* float vectors and SpMM; FP64 moment sums and D accumulation      */
#define FK_PREC_DS   2   /* double-single (float-float, ~48-bit) on the FP32 pipe; FP64 sums */

/* ---- kernel kinds for profiling ---- */
#define FK_KERNEL_STEP    0   /* fused Chebyshev step (+ moments / stochastic sum)          */
#define FK_KERNEL_ADJOINT 1   /* fused reverse-mode step (+ outer-product epilogue)         */
#define FK_KERNEL_OUTER   2   /* sparsity-restricted outer product                          */
#define FK_KERNEL_HELPER  3   /* layout, scaling, reduction and symmetrize helpers          */

typedef struct fk_engine fk_engine;

/* Library / device queries */
const char* fk_version(void);
const char* fk_status_string(int status);
int fk_device_count(int* count);
/* Measured multiply-add throughput of `device` in TFLOP/s (2 flops per FMA), FP64 (fp64 != 0) or
 * FP32: a few milliseconds of independent FMA chains with no memory traffic, timed with CUDA
 * events. The denominator of the FP64 engine's compute roofline. No reference counterpart. */
int fk_device_fma_rate(int device, int fp64, double* tflops);
/* Free and total device memory of `device` in bytes (admission control of the serving loop). */
int fk_device_memory(int device, size_t* free_bytes, size_t* total_bytes);

/* mk_engine<T>() / mk_engine_cuSPARSE<T>(devices) (reference src/engine.cpp:124-131,
 * src/engine_cusparse.cpp:1170-1215): one engine bound to one device and one stream. */
int  fk_engine_create(int device, int kind, int precision, fk_engine** out);
int  fk_engine_destroy(fk_engine* e);
const char* fk_engine_last_error(const fk_engine* e);
/* Run on a caller-provided cudaStream_t (NULL: the engine's own stream). */
int  fk_engine_set_stream(fk_engine* e, void* cuda_stream);
int  fk_engine_synchronize(fk_engine* e);
/* Engine options: FK_OPT_* below. */
#define FK_OPT_FUSE_D      0   /* fuse the outer product into the adjoint step when D's pattern is H's: 1 or 2 (default) yes, 0 never */
#define FK_OPT_NP          1   /* packets per lane: 0 auto, or 1, 2, 4                                           */
#define FK_OPT_CTAS_PER_SM 2   /* 0 auto (occupancy), else a cap on CTAs per SM                                   */
#define FK_OPT_STAGE_H     3   /* 1: stage H blocks in shared memory, 0: never, 2 (default): not in FP32 kernels */
#define FK_OPT_GRAPHS      4   /* 1: capture the M-step recursions in CUDA graphs and replay them                 */
#define FK_OPT_NP_STEP     5   /* packets per lane of the step kernel only (0: FK_OPT_NP / default)               */
#define FK_OPT_NP_ADJOINT  6   /* ... of the adjoint kernel only                                                  */
#define FK_OPT_NP_OUTER    7   /* ... of the outer-product kernel only                                            */
#define FK_OPT_TMA         8   /* step kernel gathers: 0 (default) per-thread loads; when the per-tile gather lists
                                * fit shared memory, 1 stages them with TMA bulk copies (mbarrier completion),
                                * 2 with per-thread 16-byte cp.async copies; reading the option returns the mode
                                * in use                                                                         */
#define FK_OPT_UPLOAD      9   /* set_R: 0 (default) the layout kernel reads R in place when the GPU can (pinned
                                * memory, or any host memory on systems with pageable-memory access); 1 always
                                * copy through device staging buffers                                          */
#define FK_OPT_ADJ_SPLIT  11   /* reverse step: 0 one pass over the blocks, 1 two passes (alpha, then beta + D),
                                * 2 (default): by configuration                                           */
#define FK_OPT_PIPE       12   /* FP32 / float-float step and adjoint kernels: 1 double-buffer each thread's
                                * gathers in shared memory with cp.async, 0 plain loads, 2 (default): by
                                * configuration; reading it back returns whether the configured step uses it */
#define FK_OPT_PRIORITY   10   /* CUDA priority of the engine's own stream (0 default; more negative = more urgent,
                                * clamped to the device's range); FK_ERR_STATE on a caller-set stream   */
#define FK_OPT_ACC64      13   /* FP32 engines: 1 (default) each thread's moment sums and the D accumulator across
                                * the reverse recursion are FP64 (doubles, DADD / DFMA); 0 float-float pairs on
                                * the FP32 pipe, D converted to double once at the end. Batches (fk_batch_*)
                                * default to 0: there the FP64 additions cost 21% (narrow rows). Reads back 1
                                * for FP64 engines and 0 for float-float (DS) engines                         */
#define FK_OPT_CTA_WAVES  14   /* launch grids of this many times the CTAs an SM set holds at once (1 .. 64; 1 the
                                * default: every CTA walks its share of tiles for the whole launch). Larger values
                                * make each CTA shorter-lived, so that launches of a higher-priority stream on the
                                * same GPU start sooner (the serving loop's short solves); moment sums are then
                                * added over more CTA partials (last-bit differences, deterministic)          */
#define FK_OPT_WARP_ROWS  15   /* 1 (default): when a warp serves each block row (32 lanes), every column
                                * chunk is whole and D's pattern is H's (fused epilogue), the FP32 and
                                * float-float reverse steps run the warp-per-row kernel (a three-slot copy
                                * ring, compile-time offsets) and the FP64 b=2 complex one its warp-per-row form (fewer FP64
                                * additions in the D reduction); 0 the general kernels. Results agree to the
                                * last bits of rounding                                               */
#define FK_OPT_ADJ_SWEEP  16   /* the warp-per-row FP32 / float-float reverse step: 1 one launch per column chunk
                                * (D's entries read and written per launch, gathered rows kept in L2 a whole
                                * lattice plane later), 0 one launch over whole rows, 2 (default) float-float
                                * engines sweep when the rows moved between a row's first and last gathers
                                * exceed half of L2 (FP32 engines: one launch, faster at cubic L=64).
                                * Same results either way (each D entry adds its chunks in the same order);
                                * reads back whether the configured reverse step sweeps              */
int  fk_engine_set_option(fk_engine* e, int option, int value);
int  fk_engine_get_option(const fk_engine* e, int option, int* value);

/* Engine<T>::set_H(H, es) (reference src/engine_cusparse.cpp:701-730, src/engine_cpu.cpp:53-61):
 * Hs = (H - avg I)/mag with avg = (lo+hi)/2, mag = (hi-lo)/2. n_b block rows of b x b blocks;
 * row_ptr[n_b+1], col_idx[nnzb] sorted within each row; val[nnzb*b*b] column-major blocks.
 * Rows without a stored diagonal block receive one. b must be 1 or 2. */
int  fk_engine_set_H(fk_engine* e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
                     const double* val, double es_lo, double es_hi);
/* Engine<T>::transfer_R() (reference src/engine_cusparse.cpp:675-699): upload the column-major
 * n x s probe block R. s must be >= 1 (the reference exits on an empty R). */
int  fk_engine_set_R(fk_engine* e, int n, int s, const double* R);
/* The same probe block given by its nonzeros, k per row (the structure set_R_correlated produces,
 * reference src/engine.cpp:76-116: one entry per row and realisation): R[i, cols[i*k+q]] += vals[i*k+q]
 * (complex: interleaved pairs), every other entry zero. Uploads ~(4 + 8 or 16) k bytes per row
 * instead of s values. Columns must lie in [0, s) (FK_ERR_ARG otherwise). */
int  fk_engine_set_R_sparse(fk_engine* e, int n, int s, int k, const int* cols, const double* vals);
/* Read back the device copy of R (column-major n x s), converted to double. */
int  fk_engine_get_R(fk_engine* e, double* R);

/* Engine<T>::moments(M) (reference src/engine_cusparse.cpp:755-791, src/engine_cpu.cpp:63-84):
 * mu[M] for even M >= 2. Leaves alpha_{M/2-1}, alpha_{M/2} on the device for autodiff. */
int  fk_engine_moments(fk_engine* e, int M, double* mu);
/* Same work, enqueued only; fk_engine_fetch_moments() waits and copies mu[M] out. */
int  fk_engine_moments_async(fk_engine* e, int M);
int  fk_engine_fetch_moments(fk_engine* e, double* mu);

/* Engine<T>::stoch_matrix(c, D) (reference src/engine_cusparse.cpp:910-953, src/engine_cpu.cpp:229-253):
 * D = (R xi^dag + xi R^dag)/2 on D's BSR pattern, xi = sum_{m<M} c_m T_m(Hs) R.
 * D pattern: d_n_b block rows (= H's), d_nnzb blocks, row_ptr/col_idx; D_val[d_nnzb*b*b] out. */
int  fk_engine_stoch_matrix(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb,
                            const int* d_row_ptr, const int* d_col_idx, double* D_val);
/* Engine<T>::autodiff_matrix(c, D) (reference src/engine_cusparse.cpp:955-1039,
 * src/engine_cpu.cpp:255-304): reverse-mode derivative of tr g, symmetrized and divided by
 * the energy scale. Requires fk_engine_moments with the same M first (FK_ERR_STATE otherwise).
 * D's pattern must be symmetric (FK_ERR_PATTERN otherwise). */
int  fk_engine_autodiff_matrix(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb,
                               const int* d_row_ptr, const int* d_col_idx, double* D_val);
/* Enqueue-only forms of the two D calls; fk_engine_fetch_D waits and copies D_val out. */
int  fk_engine_stoch_matrix_async(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb,
                                  const int* d_row_ptr, const int* d_col_idx);
int  fk_engine_autodiff_matrix_async(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb,
                                     const int* d_row_ptr, const int* d_col_idx);
int  fk_engine_fetch_D(fk_engine* e, double* D_val);

/* Engine<T>::energy_scale(H, extend, iters) (reference src/engine_cusparse.cpp:598-673,
 * src/engine_cpu.cpp:14-51): Lanczos on the device (iters SpMV steps from the start vector
 * v0[n], or a seeded start when v0 is NULL), extremal eigenvalues of the tridiagonal by
 * bisection, widened by extend*(max-min) on each side. */
int  fk_engine_energy_scale(fk_engine* e, int n_b, int b, int nnzb, const int* row_ptr,
                            const int* col_idx, const double* val, double extend, int iters,
                            const double* v0, double* lo, double* hi);

/* expansion_coefficients(M, Mq, f, es) with f = fermi_density(., kT, mu) (f_kind 0) or
 * fermi_energy(., kT, mu) (f_kind 1) and the Jackson kernel (reference src/fastkpm.cpp:13-78,
 * :375-393), computed in FP64 on the engine's device: T_m at the Mq Chebyshev nodes as
 * cos(m theta_i), node sums reduced in a fixed order. out[M] on the host. */
int  fk_engine_expansion_coefficients(fk_engine* e, int M, int Mq, int f_kind, double kT, double mu,
                                      double es_lo, double es_hi, double* out);

/* Engine<T>::moments2_v1(M, j1, j2, a_chunk_ncols, R_chunk_ncols) (reference
 * src/engine_cusparse.cpp:793-902, src/engine_cpu.cpp:86-160): second-order moments
 * mu[m1][m2] = sum_k <T_m1(Hs) r_k, j2 T_m2(Hs) j1 r_k> ~ tr(j1 T_m1(Hs) j2 T_m2(Hs)) over the
 * probe columns r_k of R. j1, j2: BSR operators with H's block rows and block size (values as
 * for set_H, not scaled). mu[2*(m1*M + m2) + {0,1}] = (re, im), M even. Chebyshev vectors in
 * the engine's precision, reduction in FP64 over double panels (this library's split-contraction
 * product kernels).
 * R_chunk_ncols > 0: probe columns per pass (default all); a_chunk_ncols >= 3: Chebyshev orders
 * per panel (default: as many as fit 60% of free device memory). Overwrites the recursion state
 * that moments() leaves for autodiff_matrix(). */
int  fk_engine_moments2_v1(fk_engine* e, int M, int j1_nnzb, const int* j1_row_ptr, const int* j1_col_idx,
                           const double* j1_val, int j2_nnzb, const int* j2_row_ptr, const int* j2_col_idx,
                           const double* j2_val, int a_chunk_ncols, int R_chunk_ncols, double* mu);

/* Engine<T>::moments2_v2(M, j1, j2) (reference src/engine_cpu.cpp:162-209; the reference's GPU
 * engine exits there, src/engine_cusparse.cpp:904-908): with a second probe block R2 (column-
 * major n x s like R; NULL: R2 = R), A_i = R^dag T_i(Hs) j2 R2 and B_i = R2^dag T_i(Hs) j1 R,
 * mu[m1][m2] = tr(A_m1 B_m2); mu[2*(m1*M + m2) + {0,1}] = (re, im). Projections and the
 * trace are FP64 products in this library's kernels; holds 2 M ld^2 projected values on the
 * device. Overwrites
 * the recursion state that moments() leaves for autodiff_matrix(). */
int  fk_engine_moments2_v2(fk_engine* e, int M, int j1_nnzb, const int* j1_row_ptr, const int* j1_col_idx,
                           const double* j1_val, int j2_nnzb, const int* j2_row_ptr, const int* j2_col_idx,
                           const double* j2_val, const double* R2, double* mu);

/* KPM post-processing of the last moments(M) on the device, with no host round trip after
 * the moments: gamma = moment_transform(mu, Mq) (reference src/fastkpm.cpp:236-256), the
 * chemical potential mu_F = filling_to_mu(gamma, es, kT, filling, delta_filling) (:418-432:
 * thermal smearing kT' = max(kT, 0.1 mag / Mq), the same bracket, root by bisection where
 * the reference uses toms748 to 30 bits, so the two agree to that tolerance), and
 * E = electronic_energy(gamma, es, kT, filling, mu_F) (:452-456). result[3] = {mu_F, E, n_tot}
 * with n_tot = density_product(gamma, 1) (:314-322); gamma[Mq] out when not NULL.
 * Needs 0 < filling - delta_filling, filling + delta_filling < 1, Mq >= M. No reference C entry
 * point: it replaces the caller's host calls between moments() and autodiff_matrix(). */
int  fk_engine_kpm_filling(fk_engine* e, int Mq, double kT, double filling, double delta_filling,
                           double* result, double* gamma);
/* The fixed-filling solve of a Kondo-lattice caller in one call, every stage on the device:
 * moments(M); mu_F, E as fk_engine_kpm_filling; c = expansion_coefficients(M, Mq,
 * fermi_energy(., kT, mu_F), es); autodiff_matrix(c, D). D_val, result[3], gamma (optional). */
int  fk_engine_solve_filling(fk_engine* e, int M, int Mq, double kT, double filling, double delta_filling,
                             int d_n_b, int d_nnzb, const int* d_row_ptr, const int* d_col_idx,
                             double* D_val, double* result, double* gamma);

/* Profiling: when on, each kernel launch is bracketed by CUDA events on the engine's stream. */
int  fk_engine_set_profiling(fk_engine* e, int on);
int  fk_engine_profile_read(fk_engine* e, int kernel_kind, long long* launches, double* total_ms);
int  fk_engine_profile_reset(fk_engine* e);
/* Device-side timing on the engine's stream: start records a CUDA event; stop records a
 * second one, waits for it and returns the elapsed milliseconds. */
int  fk_engine_timer_start(fk_engine* e);
int  fk_engine_timer_stop(fk_engine* e, double* ms);
/* Page-lock (pin) a caller-owned host buffer so uploads from it run at full copy speed;
 * fk_host_unregister undoes it. */
int  fk_host_register(void* ptr, size_t bytes);
int  fk_host_unregister(void* ptr);
/* Device memory the engine holds, in bytes. */
int  fk_engine_memory(const fk_engine* e, size_t* bytes);

/* ---- batched engine: many Hamiltonians of uneven size in one launch per Chebyshev step ----
 * No reference counterpart: the reference solves one Hamiltonian per Engine<T> call; this is the
 * batched form of Engine<T>::moments (reference src/engine_cusparse.cpp:755-791) over independent
 * systems that share the block size b; their probe counts s may differ (each system's rows use the
 * widest system's row stride and the kernels walk only that system's own columns). */
typedef struct fk_batch fk_batch;
int  fk_batch_create(int device, int kind, int precision, fk_batch** out);
int  fk_batch_destroy(fk_batch* bt);
const char* fk_batch_last_error(const fk_batch* bt);
/* Add one system (its H as in fk_engine_set_H and its column-major (n_b*b) x s probe block R);
 * *index receives its position. Takes effect at the next fk_batch_commit. */
int  fk_batch_add(fk_batch* bt, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
                  const double* val, double es_lo, double es_hi, int s, const double* R, int* index);
/* Upload every added system and build the launch tables. */
int  fk_batch_commit(fk_batch* bt);
/* mu[index * M + m] for every system, even M >= 2: M/2 launches, each covering all systems,
 * replayed from a CUDA graph when FK_OPT_GRAPHS is on. */
int  fk_batch_moments(fk_batch* bt, int M, double* mu);
/* Engine<T>::autodiff_matrix(c, D) (reference src/engine_cpu.cpp:255-304) for every system of the
 * batch in the same launches, after fk_batch_moments with the same M (FK_ERR_STATE otherwise).
 * c[sys*M + m]: each system's coefficients. D_val: each system's D on its own H pattern (as added),
 * systems in index order, b*b (complex: interleaved) values per block; symmetrized and divided by
 * that system's energy scale. H patterns must be symmetric (FK_ERR_PATTERN). */
int  fk_batch_autodiff_matrix(fk_batch* bt, int M, const double* c, double* D_val);
int  fk_batch_set_option(fk_batch* bt, int option, int value);
int  fk_batch_get_option(const fk_batch* bt, int option, int* value);
/* Choose lanes per block row, packets per lane, CTA cap and H staging by timing trial_steps
 * Chebyshev steps of this batch per candidate; the fastest is kept (and remembered per batch
 * shape for later batches in this process). Returns the chosen mapping and its step time. */
int  fk_batch_autotune(fk_batch* bt, int trial_steps, int* lanes_per_row, int* packets_per_lane,
                       int* ctas_per_sm, int* stage_h, double* ms_per_step);
/* moments(M) of the batch once with direct launches, each step launch bracketed by CUDA events on
 * the batch's stream: *kernel_ms = the sum of the launch times, *launches = their number. Set
 * against the time of the same moments(M) replayed from a CUDA graph, it gives the share of the
 * graph's time spent between kernels. Leaves the moments state like fk_batch_moments. */
int  fk_batch_profile_moments(fk_batch* bt, int M, double* kernel_ms, int* launches);
int  fk_batch_timer_start(fk_batch* bt);
int  fk_batch_timer_stop(fk_batch* bt, double* ms);
int  fk_batch_info(const fk_batch* bt, int* n_systems, long long* total_rows, size_t* device_bytes);

/* ---- moments without device allocation ----
 * No counterpart in the reference (its engines cudaMalloc inside every call). For callers
 * that cannot allocate device memory: their device memory is owned by another allocator
 * (a host application's pool, or a fixed reservation made at start-up that nothing else may
 * grow), or they must not trigger the device-wide synchronisation that cudaFree implies while
 * their other streams run. Same result as fk_engine_moments in native FP64, on buffers the
 * caller already holds; the kernels' scratch (moment partials, per-step sums, launch tables)
 * is one static device array of under 300 KiB in the library, held by every GPU that loads it
 * until the process exits. Nothing is allocated: no cudaMalloc, cudaFree or allocating library
 * routine is called.
 *   d_row_ptr[n_b+1], d_col_idx[nnzb] (each < 2^30), d_hs_val[nnzb*b*b]: the SCALED matrix
 *     Hs = (H - avg I)/mag as device BSR (column-major b x b blocks; interleaved (re, im) for
 *     FK_COMPLEX); the pattern is trusted, not checked. d_hs_val must be aligned to a whole
 *     element (16 bytes for FK_COMPLEX, 8 for FK_REAL), d_row_ptr and d_col_idx to 4 bytes.
 *   d_R: device, row-major (n_b*b) x ld doubles (complex: pairs), zero in columns s..ld-1;
 *     ld a multiple of 2 for FK_REAL; 16-byte aligned.  d_work: device, 2 * (n_b*b) * ld
 *     elements for the two recursion vectors (overwritten).  mu: host, M doubles out.
 *   stream: a cudaStream_t or NULL (the legacy default stream); the call waits for it.
 * Limits: even M with 2 <= M <= 32768; larger M returns FK_ERR_UNSUPPORTED (the static
 * scratch holds 16384 steps); malformed arguments return FK_ERR_ARG.
 * Every call looks up the array's device address on the current device (cudaGetSymbolAddress,
 * which allocates nothing); the first lookup on a device loads the library's device code, so
 * make the first call on each device before any stream capture. The launch tables in the array
 * are rewritten on `stream` at the start of every call. All calls share the array and it keeps
 * the last call's contents, so calls that overlap on the GPU (from different streams or
 * threads) race with each other: serialise them. */
int  fk_moments_noalloc(int kind, int n_b, int b, const int* d_row_ptr, const int* d_col_idx,
                        const double* d_hs_val, long long ld, int s, const double* d_R, double* d_work,
                        int M, double* mu, void* stream);

/* ---- host helpers of the drop-in layer (no device work) ---- */
/* SpMatBsr::build (reference src/spmat.cpp:46-129): sort blocks by (row, col), sum duplicates.
 * Out arrays sized for n_elems blocks; returns FK_OK and *nnzb_out. */
int  fk_bsr_build(int kind, int n_rows, int b, int n_elems, const int* row_idx, const int* col_idx,
                  const double* val, int* row_ptr_out, int* row_idx_out, int* col_idx_out,
                  double* val_out, int* nnzb_out);
/* SpMatBsr::symmetrize (reference src/spmat.cpp:171-190) */
int  fk_bsr_symmetrize(int kind, int n_rows, int b, int nnzb, const int* row_ptr, const int* row_idx,
                       const int* col_idx, double* val);
/* Probe generation (reference src/engine.cpp:34-116) with std::mt19937 master generator
 * state given as (seed, draws already taken). R column-major n x (j_end - j_start). */
int  fk_probe_identity(int kind, int n, int j_start, int j_end, double* R);
int  fk_probe_uncorrelated(int kind, int n, int s, uint32_t seed, unsigned long long discard,
                           int j_start, int j_end, double* R);
int  fk_probe_correlated(int kind, int n, const int* groups, uint32_t seed, unsigned long long discard,
                         int j_start, int j_end, double* R);
/* KPM coefficients (reference src/fastkpm.cpp:13-78, :375-393): f = fermi_density(., kT, mu)
 * for f_kind 0 and fermi_energy(., kT, mu) for f_kind 1, expanded on [es_lo, es_hi]. */
int  fk_jackson_kernel(int M, double* out);
int  fk_expansion_coefficients(int M, int Mq, int f_kind, double kT, double mu, double es_lo,
                               double es_hi, double* out);

#ifdef __cplusplus
}
#endif
#endif /* FASTKPM_GB300_H */
