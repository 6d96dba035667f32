/*
 * kpm_oracle.h -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * CPU restatement of FastKPM's reference CPU engine and host helpers, used only
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, to check
 * results. Nothing in fastkpm_gb300/ links, loads or calls this library.
 *
 * PARITY UNPINNED against the reference itself: the reference ships no tests,
 * fixtures or golden vectors, and it cannot be compiled here (its public
 * header includes <armadillo>; Armadillo and Boost are mandatory and absent).
 * The oracle is instead pinned against analytic known answers in tests/
 * (exact traces with identity probes, closed-form lattice moments, dense
 * eigendecomposition, finite differences of the moment sum).
 *
 * Value layout: every `double*` value array holds real doubles, or interleaved
 * (re, im) pairs when the engine / call was created with cplx != 0.
 * Probe matrices R are column-major n x s, exactly like arma::Mat<T> R in
 * src/fastkpm.h:188. BSR blocks are column-major b x b (src/fastkpm.h:64-65).
 */
#ifndef KPM_ORACLE_H
#define KPM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_engine orc_engine;

/* Engine_CPU<T> (src/engine_cpu.cpp:6-305); nthreads <= 0 -> all usable cores */
orc_engine* orc_engine_create(int cplx, int nthreads);
void orc_engine_destroy(orc_engine* e);
int  orc_engine_threads(const orc_engine* e);
/* set_H (src/engine_cpu.cpp:53-61): Hs = (H - avg I) / mag */
int  orc_set_H(orc_engine* e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
               const double* val, double es_lo, double es_hi);
/* R (column-major n x s), as left in Engine<T>::R by set_R_* */
int  orc_set_R(orc_engine* e, int n, int s, const double* R);
/* moments (src/engine_cpu.cpp:63-84) */
int  orc_moments(orc_engine* e, int M, double* mu);
/* stoch_matrix (src/engine_cpu.cpp:229-253); D pattern given by row/col idx */
int  orc_stoch_matrix(orc_engine* e, int M, const double* c, int nnzb, const int* D_row_idx,
                      const int* D_col_idx, double* D_val);
/* autodiff_matrix (src/engine_cpu.cpp:255-304); needs orc_moments(M) first */
int  orc_autodiff_matrix(orc_engine* e, int M, const double* c, int n_b, int nnzb,
                         const int* D_row_ptr, const int* D_row_idx, const int* D_col_idx,
                         double* D_val);
/* Lanczos energy_scale (src/engine_cpu.cpp:14-51) with a caller-given start vector
 * (the reference draws arma::randn, which is not reproducible without Armadillo) and
 * Sturm-bisection eigenvalues of the tridiagonal matrix in place of arma::eig_sym. */
int  orc_energy_scale(orc_engine* e, int n_b, int b, int nnzb, const int* row_ptr,
                      const int* col_idx, const double* val, double extend, int iters,
                      const double* v_start, double* lo, double* hi);
/* Extreme eigenvalues of the symmetric tridiagonal (alpha[0..n), beta[1..n)) by bisection */
void orc_tridiag_extremes(int n, const double* alpha, const double* beta, double* emin, double* emax);

/* Probe generation (src/engine.cpp:7-116). The master generator is
 * std::mt19937(seed) advanced by `discard` draws. */
int  orc_R_identity(int cplx, int n, int j_start, int j_end, double* R);
int  orc_R_uncorrelated(int cplx, int n, int s, uint32_t seed, unsigned long long discard,
                        int j_start, int j_end, double* R);
int  orc_R_correlated(int cplx, int n, const int* groups, uint32_t seed, unsigned long long discard,
                      int j_start, int j_end, double* R);

/* SpMatBsr::build (src/spmat.cpp:46-129): returns the number of unique blocks;
 * out arrays sized for n_elems blocks (row_ptr: n_rows + 1). */
int  orc_bsr_build(int cplx, int n_rows, int b, int n_elems, const int* row_idx, const int* col_idx,
                   const double* val, int* out_row_ptr, int* out_row_idx, int* out_col_idx,
                   double* out_val);
/* SpMatBsr::symmetrize + scale (src/spmat.cpp:171-198) */
int  orc_bsr_symmetrize(int cplx, int n_rows, int b, int nnzb, const int* row_ptr,
                        const int* row_idx, const int* col_idx, double* val);

/* KPM host math (src/fastkpm.cpp) */
void   orc_jackson_kernel(int M, double* out);
void   orc_chebyshev_fill_array(double x, int M, int kind, double* out);
double orc_fermi_density(double x, double kT, double mu);
double orc_fermi_energy(double x, double kT, double mu);
/* expansion_coefficients, non-FFTW branch (src/fastkpm.cpp:41-78); f = fermi_density(., kT, mu)
 * when kind == 0, fermi_energy(., kT, mu) when kind == 1 */
void   orc_expansion_coefficients(int M, int Mq, int kind, double kT, double mu,
                                  double es_lo, double es_hi, double* out);
double orc_moment_product(int M, const double* c, const double* mu);
/* moments2_v1 (src/engine_cpu.cpp:86-160): mu[m1*M + m2] (complex, interleaved) =
 * sum_k cdot(T_m1(Hs) r_k, j2 T_m2(Hs) j1 r_k); j1, j2 BSR with H's block structure, unscaled */
int    orc_moments2_v1(orc_engine* e, int M, int n_b, int b, const int* rp1, const int* ci1, const double* v1,
                       const int* rp2, const int* ci2, const double* v2, double* mu);
/* moments2_v2 (src/engine_cpu.cpp:162-209): mu[m1*M + m2] = tr(A_m1 B_m2), A_i = R^dag T_i j2 R2,
 * B_i = R2^dag T_i j1 R; R2 column-major n x s like R, or NULL for R2 = R */
int    orc_moments2_v2(orc_engine* e, int M, int n_b, int b, const int* rp1, const int* ci1, const double* v1,
                       const int* rp2, const int* ci2, const double* v2, const double* R2, double* mu);
/* electrical_conductivity_coefficients, direct-sum branch (src/fastkpm.cpp:80-233):
 * out[2*(m1*M + m2) + {0,1}]; 1 on the reference's assertion failures */
int    orc_electrical_conductivity_coefficients(int M, int Mq, double kT, double mu, double omega, double lo,
                                                double hi, const double* kernel, double* out);
/* moment_transform, mu_to_filling, filling_to_mu, electronic_energy (src/fastkpm.cpp:236-256,
 * :395-400, :418-432, :452-456); es = [lo, hi] */
void   orc_moment_transform(int M, const double* mu, int Mq, double* gamma);
double orc_mu_to_filling(int Mq, const double* gamma, double lo, double hi, double kT, double mu);
double orc_filling_to_mu(int Mq, const double* gamma, double lo, double hi, double kT, double filling,
                         double delta_filling);
double orc_electronic_energy(int Mq, const double* gamma, double lo, double hi, double kT, double filling,
                             double mu);

#ifdef __cplusplus
}
#endif
#endif
