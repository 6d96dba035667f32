// fk_engine.cu -- the C ABI of include/fastkpm_gb300.h: engine state, device
// buffers, launch configuration and the call sequences of moments,
// stoch_matrix, autodiff_matrix and energy_scale.
//
// Device layout and buffer plan (one engine = one Hamiltonian on one device):
//   R (n x ld, row-major, precision of the engine) and four work vectors V0..V3
//   of the same shape. moments: a_{m+1} overwrites a_{m-1} in place (the step
//   kernel reads z and writes y at the same position only), so only two work
//   vectors rotate. stoch_matrix: two rotating vectors plus xi. autodiff: the
//   two moment vectors (alpha) plus two beta vectors, all updated in place by
//   the fused adjoint kernel. No allocation happens inside any recursion.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/fastkpm_gb300.h"
#include "fk_dispatch.h"
#include "fk_gram.cuh"
#include "fk_post.cuh"
#include "fk_prep.h"

using fk::SysDesc;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && p) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; bytes = 0; }
        if (need == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, need);
        if (e == cudaSuccess) bytes = need;
        else { p = nullptr; cudaGetLastError(); }
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; bytes = 0; }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct KCfg {
    int Gp = 1, NP = 1, slices = 1, W = 1;   // lanes per row, packets per lane, column slices, packets per slice
    int stage_cap = 0;
    size_t smem = 0;
    int ctas = 1;
    DevBuf sys, cta_sys;
    bool valid = false;
    bool staged = false;   // step kind only: TMA-staged gathers (k_cheb_step_staged)
    bool split = false;    // adjoint kind only: two passes over the blocks (k_adjoint_split)
    bool pipe = false;     // step kind only: double-buffered gathers (k_cheb_step_pipe, FP32)
    bool warp = false;     // adjoint kind: the warp-per-row kernel (k_adjoint_warp)
    int umax = 0;          // largest per-tile gather list
};

struct ProfEvent { int kind; cudaEvent_t a, b; };

int next_pow2(int v) { int p = 1; while (p < v) p <<= 1; return p; }

// FMA pipe throughput probe: kFmaChains independent multiply-add chains per thread, no memory
// traffic; the sum is stored only when it equals an impossible value, so nothing is optimised out.
constexpr int kFmaChains = 8;
constexpr int kFmaThreads = 256;
template <class T>
__global__ void __launch_bounds__(kFmaThreads) k_fma_rate(double* sink, int iters, T seed) {
    T v[kFmaChains];
#pragma unroll
    for (int q = 0; q < kFmaChains; q++) v[q] = seed + (T)(threadIdx.x + q);
    const T mul = (T)0.9999999, add = (T)1e-7;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < kFmaChains; q++) v[q] = fma(v[q], mul, add);
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < kFmaChains; q++) s += v[q];
    if (s == (T)-1.0) *sink = (double)s;
}

}  // namespace

struct fk_engine {
    int device = 0;
    int cplx = 0;
    int prec = fk::kF64;
    int num_sms = 1;
    long long l2_bytes = 0;   // the device's L2 cache
    long long gather_dist = 0;   // 90th percentile of H's block-column distances |j - i| (set_H)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int opt_priority = 0;   // CUDA priority of the engine's own stream
    std::string err;

    // options
    int opt_fuse_d = 2, opt_np = 0, opt_ctas_per_sm = 0, opt_stage = 2, opt_graphs = 0;
    int opt_np_kind[3] = {0, 0, 0};   // per kernel kind (step, adjoint, outer); 0 = opt_np / default
    // Stage the step kernel's gathers with TMA bulk copies when they fit. Off by default: on the
    // cubic L=64 workload the per-copy cost of its 512-byte row chunks made it 2-3x slower than
    // per-thread gathers, whose DRAM traffic is already at the algorithmic minimum.
    int opt_tma = 0;
    DevBuf d_t_uoff, d_t_ucol, d_t_own, d_t_kslot, d_t_base, d_err;   // per-tile gather lists, error flag

    // H (scaled, augmented with diagonal blocks)
    int n_b = 0, b = 0, nnzb = 0;
    double es_lo = 0, es_hi = 0;
    std::vector<int> h_row_ptr, h_col;
    DevBuf d_row_ptr, d_colc, d_hval;
    DevBuf d_row_hsum;   // float-float engines: per row, identity blocks of one value (fk_prep.h)

    // probes and work vectors
    int n = 0, s = 0;
    long long ld = 0;
    int P = 0;
    DevBuf d_R, d_V[4];

    // moment state: which buffers hold alpha_{M/2-1}, alpha_{M/2} (-1 = R)
    int mom_M = 0, mom_a0 = -2, mom_a1 = -2;
    int pending_M = 0;       // moments enqueued, not yet fetched

    // D pattern cache
    int d_nb = -1, d_nnzb = -1;
    std::vector<int> dh_row_ptr, dh_col;
    bool d_same_as_H = false;
    bool d_symmetric = false;
    DevBuf dd_row_ptr, dd_colc, dd_rows, dd_pair, dd_acc;

    // scratch
    DevBuf d_partials, d_raw, d_coef, d_stage;
    // R upload: a copy stream and events so the next chunk's host-to-device copy overlaps
    // the layout kernel of the current one (two halves of d_stage)
    cudaStream_t copy_stream = nullptr;
    int pageable_access = 0;   // the GPU reads any host memory (cudaDevAttrPageableMemoryAccess)
    int opt_upload = 0;        // FK_OPT_UPLOAD: 0 read device-readable host R directly, 1 staging copies
    int opt_adj_split = 2;     // FK_OPT_ADJ_SPLIT: 0 one pass, 1 two passes, 2 (default) by configuration
    int opt_pipe = 2;          // FK_OPT_PIPE: 0 plain step, 1 double-buffered gathers (FP32), 2 (default) by configuration
    int opt_acc64 = 1;         // FK_OPT_ACC64 (FP32 engines): 1 FP64 moment sums and D accumulator, 0 float-float
    int opt_waves = 1;         // FK_OPT_CTA_WAVES: grids of this many times the resident CTAs (shorter-lived CTAs)
    int opt_warp = 1;          // FK_OPT_WARP_ROWS: warp-per-row kernels where a warp serves each block row
    int opt_sweep = 2;         // FK_OPT_ADJ_SWEEP: 0 one launch, 1 a launch per column chunk, 2 (default) by size
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_consumed[2] = {nullptr, nullptr};
    DevBuf d_post;   // post-processing: [mu M][gamma Mq][energies Mq][result 4][coefficients M]
    int post_M = 0, post_Mq = 0;

    // second-order moments (moments2_v1): operators j1, j2 in the engine's format, the two
    // double panels of Chebyshev vectors, a scratch vector, the M x M result, and the split
    // partial tiles of the FP64 products (fk_gram.cuh) that reduce the panels
    struct Op { DevBuf row_ptr, colc, hval; };
    Op d_j[2];
    DevBuf d_panel[2], d_tmp, d_mu2, d_R2, d_gram;
    std::vector<double> h_raw;

    KCfg cfg[fk::kNumKinds];

    // timer
    cudaEvent_t t_start = nullptr, t_stop = nullptr;

    // captured launch sequences (FK_OPT_GRAPHS), keyed by call kind and shape; each keeps the
    // buffer addresses and launch shapes it was captured with and is recaptured when they change
    struct GraphEntry { std::vector<long long> sig; cudaGraphExec_t exec = nullptr; };
    std::map<long long, GraphEntry> graphs;

    // profiling
    bool profiling = false;
    std::vector<ProfEvent> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
    long long prof_launches[fk::kNumKinds] = {0, 0, 0, 0};
    double prof_ms[fk::kNumKinds] = {0, 0, 0, 0};

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t ce, const char* what) {
        cudaGetLastError();
        return fail(ce == cudaErrorMemoryAllocation ? FK_ERR_OOM : FK_ERR_CUDA, "%s: %s", what,
                    cudaGetErrorString(ce));
    }
    size_t esize() const { return (size_t)fk::elem_bytes(prec, cplx); }
    int epp() const { return fk::elems_per_packet(prec, cplx); }
    size_t hsize() const { return esize(); }   // H entries use the element type
    size_t vec_bytes() const { return (size_t)n * ld * esize(); }
    void* V(int id) const { return id < 0 ? d_R.p : d_V[id].p; }
};

namespace {

#define FK_TRY(expr, what)                                   \
    do {                                                     \
        cudaError_t _ce = (expr);                            \
        if (_ce != cudaSuccess) return e->cuda_fail(_ce, what); \
    } while (0)

cudaError_t prec_launch_step(fk_engine* e, int NP, const fk::StepArgs& a, const fk::Launch& l) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_step_f64(e->cplx, e->b, NP, a, l);
        case fk::kF32: return e->opt_acc64 ? fk::launch_step_f32a(e->cplx, e->b, NP, a, l)
                                           : fk::launch_step_f32(e->cplx, e->b, NP, a, l);
        default: return fk::launch_step_ds(e->cplx, e->b, NP, a, l);
    }
}
cudaError_t prec_launch_adjoint(fk_engine* e, int NP, const fk::AdjArgs& a, const fk::Launch& l) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_adjoint_f64(e->cplx, e->b, NP, a, l);
        case fk::kF32: return e->opt_acc64 ? fk::launch_adjoint_f32a(e->cplx, e->b, NP, a, l)
                                           : fk::launch_adjoint_f32(e->cplx, e->b, NP, a, l);
        default: return fk::launch_adjoint_ds(e->cplx, e->b, NP, a, l);
    }
}
cudaError_t prec_launch_outer(fk_engine* e, int NP, const fk::OuterArgs& a, const fk::Launch& l) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_outer_f64(e->cplx, e->b, NP, a, l);
        case fk::kF32: return e->opt_acc64 ? fk::launch_outer_f32a(e->cplx, e->b, NP, a, l)
                                           : fk::launch_outer_f32(e->cplx, e->b, NP, a, l);
        default: return fk::launch_outer_ds(e->cplx, e->b, NP, a, l);
    }
}
cudaError_t prec_occupancy(fk_engine* e, int kind, int NP, size_t smem, int* n) {
    switch (e->prec) {
        case fk::kF64: return fk::occupancy_f64(kind, e->cplx, e->b, NP, smem, n);
        case fk::kF32: return e->opt_acc64 ? fk::occupancy_f32a(kind, e->cplx, e->b, NP, smem, n)
                                           : fk::occupancy_f32(kind, e->cplx, e->b, NP, smem, n);
        default: return fk::occupancy_ds(kind, e->cplx, e->b, NP, smem, n);
    }
}
cudaError_t prec_load_colmajor(fk_engine* e, const double* src, long long n, int ncols, int c0, void* dst) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_load_colmajor_f64(e->cplx, src, n, ncols, c0, e->ld, dst, e->stream);
        case fk::kF32: return fk::launch_load_colmajor_f32(e->cplx, src, n, ncols, c0, e->ld, dst, e->stream);
        default: return fk::launch_load_colmajor_ds(e->cplx, src, n, ncols, c0, e->ld, dst, e->stream);
    }
}
cudaError_t prec_expand_sparse(fk_engine* e, const int* cols, const double* vals, long long n, int k, void* dst) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_expand_sparse_f64(e->cplx, cols, vals, n, k, e->ld, dst, e->stream);
        case fk::kF32: return fk::launch_expand_sparse_f32(e->cplx, cols, vals, n, k, e->ld, dst, e->stream);
        default: return fk::launch_expand_sparse_ds(e->cplx, cols, vals, n, k, e->ld, dst, e->stream);
    }
}
cudaError_t prec_store_colmajor(fk_engine* e, const void* src, long long n, int ncols, double* dst) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_store_colmajor_f64(e->cplx, src, n, ncols, e->ld, dst, e->stream);
        case fk::kF32: return fk::launch_store_colmajor_f32(e->cplx, src, n, ncols, e->ld, dst, e->stream);
        default: return fk::launch_store_colmajor_ds(e->cplx, src, n, ncols, e->ld, dst, e->stream);
    }
}
// ---- profiling ----
cudaEvent_t prof_event(fk_engine* e) {
    if (!e->prof_pool.empty()) { cudaEvent_t ev = e->prof_pool.back(); e->prof_pool.pop_back(); return ev; }
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    return ev;
}
struct ProfScope {
    fk_engine* e; int kind; cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(fk_engine* e_, int k) : e(e_), kind(k) {
        if (e->profiling) { a = prof_event(e); b = prof_event(e); cudaEventRecord(a, e->stream); }
    }
    ~ProfScope() {
        if (e->profiling) { cudaEventRecord(b, e->stream); e->prof_pending.push_back({kind, a, b}); }
    }
};
// y = (*c_dev) x, the factor read on the device (graph replays see new values)
cudaError_t prec_scale(fk_engine* e, const void* x, void* y, const double* c_dev) {
    const long long ne = (long long)e->n * e->ld;
    ProfScope ps(e, fk::kHelper);
    switch (e->prec) {
        case fk::kF64: return fk::launch_scale_f64(e->cplx, x, y, ne, 0.0, c_dev, e->stream);
        case fk::kF32: return fk::launch_scale_f32(e->cplx, x, y, ne, 0.0, c_dev, e->stream);
        default: return fk::launch_scale_ds(e->cplx, x, y, ne, 0.0, c_dev, e->stream);
    }
}

// Graph capture of a fixed launch sequence (FK_OPT_GRAPHS): captured on first use per key,
// replayed afterwards. Keys encode the call kind and every value baked into the launches.
long long graph_key(int kind, int M, long long extra) {
    return ((long long)kind << 56) ^ ((long long)M << 24) ^ extra;
}
// Everything a captured sequence bakes in besides its key: buffer addresses, sizes and launch shapes.
std::vector<long long> graph_signature(const fk_engine* e) {
    std::vector<long long> s;
    auto addr = [&](const void* p) { s.push_back((long long)(uintptr_t)p); };
    addr(e->stream);
    for (const DevBuf* b : {&e->d_row_ptr, &e->d_colc, &e->d_hval, &e->d_R, &e->d_V[0], &e->d_V[1], &e->d_V[2],
                            &e->d_V[3], &e->dd_row_ptr, &e->dd_colc, &e->dd_rows, &e->dd_pair, &e->dd_acc,
                            &e->d_partials, &e->d_raw, &e->d_coef, &e->d_row_hsum})
        addr(b->p);
    for (long long v : {(long long)e->n_b, (long long)e->b, (long long)e->nnzb, (long long)e->n, (long long)e->s, e->ld,
                        (long long)e->P, (long long)e->d_nnzb, (long long)e->opt_acc64})
        s.push_back(v);
    long long mag_bits;
    const double mag = (e->es_hi - e->es_lo) / 2.0;
    std::memcpy(&mag_bits, &mag, sizeof mag);
    s.push_back(mag_bits);
    for (const KCfg& c : e->cfg) {
        for (long long v : {(long long)c.Gp, (long long)c.NP, (long long)c.slices, (long long)c.W,
                            (long long)c.stage_cap, (long long)c.smem, (long long)c.ctas, (long long)c.valid})
            s.push_back(v);
        addr(c.sys.p);
        addr(c.cta_sys.p);
    }
    return s;
}
void drop_graphs(fk_engine* e) {
    for (auto& g : e->graphs) cudaGraphExecDestroy(g.second.exec);
    e->graphs.clear();
}
// Run a call's launch sequence directly, or (FK_OPT_GRAPHS) replay it as a CUDA graph captured on
// first use. Not used while profiling (per-launch events) or with the staged step kernel.
template <class F>
int run_launches(fk_engine* e, long long key, F&& launches) {
    if (!e->opt_graphs || e->profiling || e->cfg[fk::kStep].staged) return launches();
    std::vector<long long> sig = graph_signature(e);
    auto it = e->graphs.find(key);
    if (it != e->graphs.end() && it->second.sig != sig) {
        cudaGraphExecDestroy(it->second.exec);
        e->graphs.erase(it);
        it = e->graphs.end();
    }
    if (it == e->graphs.end()) {
        cudaGraph_t g = nullptr;
        FK_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        const int rc = launches();
        const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if (rc != FK_OK) { if (g) cudaGraphDestroy(g); return rc; }
        if (ce != cudaSuccess) return e->cuda_fail(ce, "end capture");
        cudaGraphExec_t ge = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return e->cuda_fail(ie, "instantiate graph");
        fk_engine::GraphEntry ent;
        ent.sig = std::move(sig);
        ent.exec = ge;
        it = e->graphs.emplace(key, std::move(ent)).first;
    }
    FK_TRY(cudaGraphLaunch(it->second.exec, e->stream), "graph launch");
    return FK_OK;
}
void prof_flush(fk_engine* e) {
    for (auto& p : e->prof_pending) {
        float ms = 0.f;
        cudaEventSynchronize(p.b);
        cudaEventElapsedTime(&ms, p.a, p.b);
        e->prof_launches[p.kind] += 1;
        e->prof_ms[p.kind] += ms;
        e->prof_pool.push_back(p.a);
        e->prof_pool.push_back(p.b);
    }
    e->prof_pending.clear();
}

// ---- launch configuration ----

// Staged (TMA bulk-copy) step kernel: build the per-tile gather lists for this Gp and pick
// the widest column chunk whose double buffer keeps two CTAs on an SM (or one, at most).
int configure_staged(fk_engine* e, KCfg& c, int Gp, int nk_max, size_t per_blk) {
    fk::TileTables t;
    if (!fk::append_tile_tables(e->h_row_ptr.data(), e->h_col.data(), e->n_b, Gp, 0, 0, t)) return FK_OK;
    const int hs = (int)e->hsize();
    int NP = 0;
    size_t smem = 0;
    for (int np : {2, 1}) {
        if (np == 2 && Gp >= e->P) continue;   // one chunk already covers the row
        const size_t s = fk::staged_smem_bytes(t.umax, e->b, Gp * np, nk_max, hs);
        const size_t tx = (size_t)t.umax * e->b * Gp * np * 16;
        if (tx < (1u << 20) && s <= (np == 2 ? 110u * 1024 : 200u * 1024)) { NP = np; smem = s; break; }
    }
    if (NP == 0) return FK_OK;
    const size_t tiles = t.own.size();
    FK_TRY(e->d_t_uoff.ensure(sizeof(int) * t.uoff.size()), "alloc gather lists");
    FK_TRY(e->d_t_ucol.ensure(sizeof(int) * std::max<size_t>(t.ucol.size(), 1)), "alloc gather lists");
    FK_TRY(e->d_t_own.ensure(sizeof(int) * std::max<size_t>(tiles, 1)), "alloc gather lists");
    FK_TRY(e->d_t_kslot.ensure(sizeof(unsigned short) * std::max<size_t>(t.kslot.size(), 1)), "alloc gather lists");
    FK_TRY(e->d_t_base.ensure(sizeof(int)), "alloc gather lists");
    FK_TRY(e->d_err.ensure(sizeof(int)), "alloc error flag");
    FK_TRY(cudaMemcpy(e->d_t_uoff.p, t.uoff.data(), sizeof(int) * t.uoff.size(), cudaMemcpyHostToDevice), "upload lists");
    FK_TRY(cudaMemcpy(e->d_t_ucol.p, t.ucol.data(), sizeof(int) * t.ucol.size(), cudaMemcpyHostToDevice), "upload lists");
    FK_TRY(cudaMemcpy(e->d_t_own.p, t.own.data(), sizeof(int) * tiles, cudaMemcpyHostToDevice), "upload lists");
    FK_TRY(cudaMemcpy(e->d_t_kslot.p, t.kslot.data(), sizeof(unsigned short) * t.kslot.size(), cudaMemcpyHostToDevice),
           "upload lists");
    FK_TRY(cudaMemset(e->d_t_base.p, 0, sizeof(int)), "clear tile base");
    FK_TRY(cudaMemset(e->d_err.p, 0, sizeof(int)), "clear error flag");
    c.staged = true;
    c.NP = NP;
    c.stage_cap = nk_max;
    c.smem = smem;
    c.umax = t.umax;
    (void)per_blk;
    return FK_OK;
}

fk::StageTables stage_tables(fk_engine* e, const KCfg& c) {
    return fk::StageTables{e->d_t_base.as<int>(), e->d_t_uoff.as<int>(), e->d_t_ucol.as<int>(), e->d_t_own.as<int>(),
                           e->d_t_kslot.as<unsigned short>(), c.umax, e->d_err.as<int>()};
}

// A staged kernel that ran out of its bounded wait left a mark: report and clear it.
int check_staged_error(fk_engine* e) {
    if (!e->cfg[fk::kStep].staged || !e->d_err.p) return FK_OK;
    int flag = 0;
    FK_TRY(cudaMemcpy(&flag, e->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (flag) {
        cudaMemset(e->d_err.p, 0, sizeof(int));
        return e->fail(FK_ERR_TIMEOUT, "a staged step kernel gave up waiting for its row copies");
    }
    return FK_OK;
}

// Packets per lane when no option sets them, for rows of P 16-byte packets (measured on GB300;
// FP32 on 10^6-site and DS / FP64 on 3x10^5-site cubic lattices, b=1 real and b=2 complex, S=32..128,
// and cubic L=64 S=256 for the widest rows):
//  * step: 4 from P = 16 (FP32) or 32 (FP64, DS) up, else 2. FP32 b=2 S=64 (P=32): 0.85 ms vs 1.34
//    with 2; FP64 b=2 S=32 (P=32): 0.96 vs 1.85; FP32 b=1 S=32 (P=8): 0.107 with 2 vs 0.142 with 4.
//  * outer product: 4 from P = 16 up (DS b=1 S=32: 0.10 vs 0.16 ms; FP64 b=2 S=32: 1.87 vs 2.31).
//  * adjoint: FP64 4 from P = 16 up (b=2 S=32: 3.74 vs 5.07 ms); DS 4 for b=1 from P = 16 up
//    (S=128: 0.60 vs 0.74), 2 for b=2 (S=64: 1.61 vs 2.53; cubic L=64 S=256: 5.9 vs 9.3); FP32 4 for
//    P = 32..64 (b=1 S=128: 0.97 vs 1.11; b=2 S=64: 3.16 vs 3.38), else 2 (b=2 S=32: 1.67 vs 1.95;
//    cubic L=64 S=256 fused: 3.24 vs 3.52).
int default_np(int kind, int prec, int P, int b) {
    if (P < 2) return 1;
    if (kind == fk::kStep) return P >= (prec == fk::kF32 ? 16 : 32) ? 4 : 2;
    if (kind == fk::kOuter) return P >= 16 ? 4 : 2;
    if (prec == fk::kF64) return P >= 16 ? 4 : 2;
    if (prec == fk::kDS) return b == 1 && P >= 16 ? 4 : 2;
    return P >= 32 && P <= 64 ? 4 : 2;
}

// FK_OPT_ADJ_SPLIT: the two-pass adjoint kernel (fewer live registers, 3 CTAs per SM) or the
// one-pass kernel. Default: two passes for b=1 rows wider than the light configurations in FP32
// and float-float (10^6-site cubic, S=128: FP32 0.77 vs 0.81 ms, DS 0.78 vs 0.82); one pass for
// b=2 and FP64 (cubic L=64, S=256: FP32 3.17 vs 3.05 ms, DS 11.6 vs 10.7).
bool use_adjoint_split(const fk_engine* e, int NP) {
    if (e->opt_adj_split != 2) return e->opt_adj_split != 0;
    const bool light = e->b * NP <= 2;   // a lane's slice of a block row is at most 32 bytes (kLightStep)
    return e->b == 1 && e->prec != fk::kF64 && !light;
}

// FK_OPT_ADJ_SWEEP 2 (default): float-float engines sweep the columns when a launch over whole
// rows would put more through L2 between a row's first and last gathers than half of L2 holds
// (FP32 engines run one launch: see configure): six vectors
// (alpha_m, beta_{m+1} gathered; alpha_{m+1}, beta_{m+2} read and written) per block row, over
// twice the block-column distance |j - i| that 90% of H's blocks keep within (periodic lattices:
// the few wrap-around bonds do not count; cubic: L^2 sites).
bool use_sweeps(const fk_engine* e, int NP) {
    if (e->P % (32 * NP) != 0 || e->P / (32 * NP) < 2) return false;
    if (e->opt_sweep != 2) return e->opt_sweep != 0;
    if (e->prec != fk::kDS) return false;
    const double window = 2.0 * (double)e->gather_dist * e->b * 6.0 * (double)e->P * 16.0;
    return e->l2_bytes > 0 && window > 0.5 * (double)e->l2_bytes;
}
// the block-column distance |j - i| that 90% of the blocks keep within
long long gather_distance(const std::vector<int>& row_ptr, const std::vector<int>& col, int n_b) {
    if (col.empty()) return 0;
    std::vector<int> d(col.size());
    for (int i = 0; i < n_b; i++)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) d[k] = std::abs(col[k] - i);
    const size_t q = (d.size() * 9) / 10;
    std::nth_element(d.begin(), d.begin() + q, d.end());
    return d[q];
}

// FK_OPT_PIPE: step / adjoint kernels with double-buffered gathers (FP32, float-float). FP32: the
// step kernel for b=2 (cubic L=64, S=256: 0.67 vs 0.85 ms; 10^6-site cubic S=128: 1.34 vs
// 1.59; b=1 S=128 stays plain: 0.301 vs 0.293); the adjoint kernel except for light rows
// (cubic L=64 S=256 fused: 2.44 vs 2.83 ms; 10^6-site cubic b=2 S=128: 4.41 vs 5.85, b=1
// S=128: 0.75 vs 0.79; b=1 S=32, light, stays plain: 0.39 vs 0.43).
bool use_pipe(const fk_engine* e, int kind, int NP) {
    if (e->prec == fk::kF64) return false;
    if (e->opt_pipe != 2) return e->opt_pipe != 0;
    // float-float: b=2 only (cubic L=64, S=256: fused adjoint 9.62 vs 10.62 ms, step 2.43 vs 2.54;
    // b=1 S=128 keeps the two-pass adjoint: 0.77 vs 0.79 piped)
    if (e->prec == fk::kDS) return e->b == 2;
    if (kind == fk::kStep) return e->b == 2;
    return e->b * NP > 2;   // not the light configurations
}

int configure(fk_engine* e) {
    for (auto& c : e->cfg) c.valid = false;
    if (e->n_b == 0 || e->s == 0 || e->n != e->n_b * e->b) return FK_OK;   // configured once both are set
    const int P = e->P;
    // Gp lanes per block row, NP packets per lane and column chunk; the kernels walk
    // the row's ceil(P / (Gp * NP)) chunks themselves, so one launch covers all columns.
    // Each kernel kind has its own NP (register use vs. loads in flight, default_np).
    const int slices = 1, W = P;
    const size_t per_blk = (size_t)e->b * e->b * e->hsize() + sizeof(unsigned);
    for (int kind = 0; kind < fk::kHelper; kind++) {
        int NP, Gp;
        const int want = e->opt_np_kind[kind] > 0 ? e->opt_np_kind[kind] : e->opt_np;
        if (want > 0) {
            NP = want;
            Gp = std::min(32, next_pow2((P + NP - 1) / NP));
        } else {
            // the lanes that cover a row in one chunk of NP packets each, at most a warp
            NP = default_np(kind, e->prec, P, e->b);
            // small systems: more lanes per row (fewer packets each) until the launch offers one
            // CTA's worth of (row, lane) items per SM, so that latency-bound solves spread over the
            // GPU (square L=32, S=64 FP64, 1,024 rows: 8 lanes give 32 CTAs; with 32 lanes a
            // moments + stoch_matrix solve takes 2.2 ms instead of 3.4)
            while (NP > 1 && next_pow2((P + NP - 1) / NP) < 32 &&
                   (long long)e->n_b * next_pow2((P + NP - 1) / NP) < (long long)e->num_sms * fk::kThreads)
                NP >>= 1;
            // the double-buffered adjoint keeps 6 x b x NP packets per thread in shared memory:
            // b x NP at most 4 so that two CTAs fit an SM (b=2 S=128 with NP=4: 1 CTA, 8.1 vs 5.8 ms)
            if (kind == fk::kAdjoint && use_pipe(e, fk::kAdjoint, NP) && e->b * NP > 4) NP = 4 / e->b;
            Gp = std::min(32, next_pow2((P + NP - 1) / NP));
        }
        // H blocks per tile of kThreads items: the shared-memory stage size
        const long long items = (long long)e->n_b * Gp;
        const long long tiles = (items + fk::kThreads - 1) / fk::kThreads;
        const int nk_max = fk::max_tile_blocks(e->h_row_ptr.data(), e->n_b, Gp);
        // FK_OPT_STAGE_H 2 (default): stage except in FP32 kernels, where the barrier around the
        // stage costs more than the re-read H blocks (cubic L=64, S=256: step 0.96 vs 1.03 ms,
        // adjoint 3.13 vs 3.24; 10^6-site cubic b=1 S=128 adjoint 0.82 vs 0.97); the FP64 and
        // DS step kernels run 12-25% faster staged.
        const bool stage = e->opt_stage == 2 ? e->prec != fk::kF32 : e->opt_stage != 0;
        const int stage_cap = (stage && nk_max * per_blk <= 48 * 1024) ? nk_max : 0;
        KCfg& c = e->cfg[kind];
        c.Gp = Gp; c.NP = NP; c.slices = slices; c.W = W;
        c.stage_cap = kind == fk::kOuter ? 0 : stage_cap;
        c.smem = c.stage_cap ? ((size_t)c.stage_cap * per_blk + 15) / 16 * 16 : 0;
        c.staged = false;
        const size_t stage_smem = c.smem;
        c.pipe = (kind == fk::kStep && !e->opt_tma && use_pipe(e, fk::kStep, NP)) ||
                 (kind == fk::kAdjoint && use_pipe(e, fk::kAdjoint, NP));
        c.split = kind == fk::kAdjoint && !c.pipe && use_adjoint_split(e, NP);
        // the warp-per-row kernel (FP32 and float-float) keeps a row's block columns one per lane:
        // rows of at most 32 blocks (cubic L=64, S=256: FP32 1.669 vs 2.141 ms, float-float 8.32 vs
        // 9.38 ms against k_adjoint_pipe)
        c.warp = kind == fk::kAdjoint && c.pipe && e->opt_warp && e->prec != fk::kF64 && Gp == 32 &&
                 P % (32 * NP) == 0 && fk::max_row_blocks(e->h_row_ptr.data(), e->n_b) <= 32;
        if (c.warp) c.stage_cap = 0;   // its H entries travel with the units: no per-tile stage
        // column sweeps: the warp-per-row reverse step launched once per column chunk, so that the
        // rows gathered again a bandwidth later are still in L2 (each launch puts a chunk's width
        // of six vectors per row through L2 instead of the whole row's). Cubic L=64, S=256, DRAM
        // bytes per reverse step: float-float 26.2 GB in one launch (1.98x the algorithmic 13.2),
        // 19.4 GB in four (7.98 -> 7.65 ms); FP32 10.3 GB in one (1.52x 6.7), 8.4 GB in two, but
        // 1.620 -> 1.663 ms: a launch over single-chunk rows starts and drains the copy ring once
        // per row and chunk, and FP32 already drew 0.93 of the DRAM peak. D's entries are read and
        // written once per launch.
        if (c.warp && use_sweeps(e, NP)) {
            c.W = 32 * NP;
            c.slices = P / c.W;
        }
        // FP64 b=2 complex: the warp-per-row step (k_adjoint_step_warp), fewer FP64-pipe additions
        // in the D reduction
        if (kind == fk::kAdjoint && !c.pipe && !c.split && e->opt_warp && e->prec == fk::kF64 && e->cplx &&
            e->b == 2 && Gp == 32 && P % (32 * NP) == 0)
            c.warp = true;
        if (c.split) c.smem += 2 * (size_t)fk::kThreads * e->b * NP * 16;   // kept alpha_{m+1}, alpha_{m-1}
        if (c.pipe) c.smem = (c.warp ? 0 : stage_smem) + (kind == fk::kStep ? fk::pipe_smem_bytes(e->b, NP)
                                           : c.warp ? fk::adj_warp_smem_bytes(e->b, NP) : fk::adj_pipe_smem_bytes(e->b, NP));
        if (kind == fk::kStep && e->opt_tma) {
            int rc = configure_staged(e, c, Gp, nk_max, per_blk);
            if (rc != FK_OK) return rc;
        }
        int occ = 0;
        const int okind = c.split ? (int)fk::kAdjointSplit
                        : c.warp ? (int)fk::kAdjointWarp   // (FP64: k_adjoint_step_warp)
                        : c.pipe ? (kind == fk::kStep ? (int)fk::kStepPipe : (int)fk::kAdjointPipe)
                        : !c.staged ? kind : (e->opt_tma == 1 ? (int)fk::kStepStaged : (int)fk::kStepStagedAsync);
        FK_TRY(prec_occupancy(e, okind, c.NP, c.smem, &occ), "occupancy query");
        if (occ < 1) return e->fail(FK_ERR_UNSUPPORTED, "kernel kind %d does not fit on an SM", kind);
        if (e->opt_ctas_per_sm > 0) occ = std::min(occ, e->opt_ctas_per_sm);
        c.ctas = (int)std::max<long long>(1, std::min<long long>(tiles, (long long)occ * e->num_sms * e->opt_waves));
        SysDesc sd{0, e->n_b, 0, c.ctas};
        FK_TRY(c.sys.ensure(sizeof(SysDesc)), "alloc sys table");
        FK_TRY(cudaMemcpy(c.sys.p, &sd, sizeof sd, cudaMemcpyHostToDevice), "upload sys table");
        FK_TRY(c.cta_sys.ensure(sizeof(int) * c.ctas), "alloc cta table");
        FK_TRY(cudaMemset(c.cta_sys.p, 0, sizeof(int) * c.ctas), "clear cta table");
        c.valid = true;
    }
    return FK_OK;
}

int require_ready(fk_engine* e) {
    if (e->n_b == 0) return e->fail(FK_ERR_STATE, "set_H has not been called");
    if (e->s == 0) return e->fail(FK_ERR_STATE, "R has not been set");
    if (e->n != e->n_b * e->b)
        return e->fail(FK_ERR_ARG, "R has %d rows but H has %d scalar rows", e->n, e->n_b * e->b);
    if (!e->cfg[0].valid) {
        int rc = configure(e);
        if (rc != FK_OK) return rc;
    }
    return FK_OK;
}

// One Chebyshev step over every column slice: y = (two?2:1) Hs x - z, optional dots / xi.
int run_step(fk_engine* e, const void* x, const void* z, void* y, bool two, bool want_dots, int xi_mode, void* xi,
             const double* coef_dev, double* partials_step) {
    const KCfg& c = e->cfg[fk::kStep];
    const size_t es = e->esize();
    for (int sl = 0; sl < c.slices; sl++) {
        const long long off = (long long)sl * c.W * e->epp();   // element offset of this slice
        fk::StepArgs a;
        a.sys = c.sys.as<SysDesc>();
        a.cta_sys = c.cta_sys.as<int>();
        a.Gp = c.Gp;
        a.P = std::min(c.W, e->P - sl * c.W);
        a.ld = e->ld;
        a.row_ptr = e->d_row_ptr.as<int>();
        a.colc = e->d_colc.as<unsigned>();
        a.hval = e->d_hval.p;
        a.x = (const char*)x + off * es;
        a.z = z ? (const char*)z + off * es : nullptr;
        a.y = (char*)y + off * es;
        a.xi = xi ? (char*)xi + off * es : nullptr;
        a.coef = coef_dev;
        a.cstride = 2;
        a.two = two; a.has_z = z != nullptr; a.want_dots = want_dots; a.xi_mode = xi_mode;
        a.partials = want_dots ? partials_step + (size_t)sl * c.ctas * 2 : nullptr;
        a.stage_cap = c.stage_cap;
        a.pipe = c.pipe ? 1 : 0;
        ProfScope ps(e, fk::kStep);
        if (c.staged) {
            const fk::StageTables tb = stage_tables(e, c);
            const fk::Launch l{c.ctas, c.smem, e->stream};
            cudaError_t ce;
            switch (e->prec) {
                case fk::kF64: ce = fk::launch_step_staged_f64(e->cplx, e->b, c.NP, e->opt_tma == 1, a, tb, l); break;
                case fk::kF32:
                    ce = e->opt_acc64 ? fk::launch_step_staged_f32a(e->cplx, e->b, c.NP, e->opt_tma == 1, a, tb, l)
                                      : fk::launch_step_staged_f32(e->cplx, e->b, c.NP, e->opt_tma == 1, a, tb, l);
                    break;
                default: ce = fk::launch_step_staged_ds(e->cplx, e->b, c.NP, e->opt_tma == 1, a, tb, l); break;
            }
            FK_TRY(ce, "staged step kernel launch");
        } else {
            FK_TRY(prec_launch_step(e, c.NP, a, fk::Launch{c.ctas, c.smem, e->stream}), "step kernel launch");
        }
    }
    return FK_OK;
}

int run_adjoint(fk_engine* e, const void* A, void* Ap, const void* Bv, void* Bp, const double* coef_dev, double* Dacc) {
    const KCfg& c = e->cfg[fk::kAdjoint];
    const size_t es = e->esize();
    ProfScope ps(e, fk::kAdjoint);   // one reverse step, all its column sweeps
    for (int sl = 0; sl < c.slices; sl++) {
        const long long off = (long long)sl * c.W * e->epp();
        fk::AdjArgs a;
        a.sys = c.sys.as<SysDesc>();
        a.cta_sys = c.cta_sys.as<int>();
        a.Gp = c.Gp;
        a.P = std::min(c.W, e->P - sl * c.W);
        a.ld = e->ld;
        a.row_ptr = e->d_row_ptr.as<int>();
        a.colc = e->d_colc.as<unsigned>();
        a.hval = e->d_hval.p;
        a.A = (const char*)A + off * es;
        a.Ap = (char*)Ap + off * es;
        a.Bv = (const char*)Bv + off * es;
        a.Bp = (char*)Bp + off * es;
        a.coef = coef_dev;
        a.cstride = 3;
        a.Dacc = Dacc;
        a.dscale = 2.0;
        a.stage_cap = c.stage_cap;
        a.split = c.split ? 1 : 0;
        a.pipe = c.pipe ? 1 : 0;
        a.warp = c.warp ? 1 : 0;
        a.row_hsum = (c.warp && e->prec == fk::kDS) ? e->d_row_hsum.as<unsigned char>() : nullptr;
        FK_TRY(prec_launch_adjoint(e, c.NP, a, fk::Launch{c.ctas, c.smem, e->stream}), "adjoint kernel launch");
    }
    return FK_OK;
}

int run_outer(fk_engine* e, const void* A, const void* Bv, double alpha, bool two_terms) {
    const KCfg& c = e->cfg[fk::kOuter];
    const size_t es = e->esize();
    for (int sl = 0; sl < c.slices; sl++) {
        const long long off = (long long)sl * c.W * e->epp();
        fk::OuterArgs a;
        a.sys = c.sys.as<SysDesc>();
        a.cta_sys = c.cta_sys.as<int>();
        a.Gp = c.Gp;
        a.P = std::min(c.W, e->P - sl * c.W);
        a.ld = e->ld;
        a.row_ptr = e->dd_row_ptr.as<int>();
        a.colc = e->dd_colc.as<unsigned>();
        a.A = (const char*)A + off * es;
        a.Bv = (const char*)Bv + off * es;
        a.alpha = alpha;
        a.two_terms = two_terms ? 1 : 0;
        a.Dacc = e->dd_acc.as<double>();
        ProfScope ps(e, fk::kOuter);
        FK_TRY(prec_launch_outer(e, c.NP, a, fk::Launch{c.ctas, 0, e->stream}), "outer kernel launch");
    }
    return FK_OK;
}

int ensure_vectors(fk_engine* e) {
    const size_t vb = e->vec_bytes();
    FK_TRY(e->d_R.ensure(vb), "allocate R");
    for (auto& v : e->d_V) FK_TRY(v.ensure(vb), "allocate work vector");
    return FK_OK;
}

int check_pattern(fk_engine* e, int n_b, int nnzb, const int* row_ptr, const int* col_idx, const char* what) {
    std::string why;
    const int rc = fk::check_bsr_pattern(n_b, nnzb, row_ptr, col_idx, why);
    return rc == FK_OK ? FK_OK : e->fail(rc, "%s: %s", what, why.c_str());
}

// Upload (or reuse) D's pattern. need_pairs: autodiff's symmetrize needs the (j,i) partner of every block.
int set_D_pattern(fk_engine* e, int d_n_b, int d_nnzb, const int* rp, const int* ci, bool need_pairs) {
    if (d_n_b != e->n_b) return e->fail(FK_ERR_ARG, "D has %d block rows, H has %d", d_n_b, e->n_b);
    if (d_nnzb < 0) return e->fail(FK_ERR_ARG, "negative D nnzb");
    const bool same = d_n_b == e->d_nb && d_nnzb == e->d_nnzb &&
                      std::equal(rp, rp + d_n_b + 1, e->dh_row_ptr.begin()) &&
                      (d_nnzb == 0 || std::equal(ci, ci + d_nnzb, e->dh_col.begin()));
    if (!same) {
        int rc = check_pattern(e, d_n_b, d_nnzb, rp, ci, "D pattern");
        if (rc != FK_OK) return rc;
        e->dh_row_ptr.assign(rp, rp + d_n_b + 1);
        e->dh_col.assign(ci, ci + d_nnzb);
        std::vector<int> rows(d_nnzb), pair(d_nnzb, -1);
        bool sym = true;
        for (int i = 0; i < d_n_b; i++) {
            for (int k = rp[i]; k < rp[i + 1]; k++) {
                rows[k] = i;
                const int j = ci[k];
                const int* lo = ci + rp[j];
                const int* hi = ci + rp[j + 1];
                const int* f = std::lower_bound(lo, hi, i);
                if (f != hi && *f == i) pair[k] = (int)(f - ci);
                else sym = false;
            }
        }
        std::vector<unsigned> colc(ci, ci + d_nnzb);
        FK_TRY(e->dd_row_ptr.ensure(sizeof(int) * (d_n_b + 1)), "alloc D row_ptr");
        FK_TRY(e->dd_colc.ensure(sizeof(unsigned) * std::max(d_nnzb, 1)), "alloc D cols");
        FK_TRY(e->dd_rows.ensure(sizeof(int) * std::max(d_nnzb, 1)), "alloc D rows");
        FK_TRY(e->dd_pair.ensure(sizeof(int) * std::max(d_nnzb, 1)), "alloc D pairs");
        FK_TRY(cudaMemcpy(e->dd_row_ptr.p, rp, sizeof(int) * (d_n_b + 1), cudaMemcpyHostToDevice), "upload D row_ptr");
        if (d_nnzb) {
            FK_TRY(cudaMemcpy(e->dd_colc.p, colc.data(), sizeof(unsigned) * d_nnzb, cudaMemcpyHostToDevice), "upload D cols");
            FK_TRY(cudaMemcpy(e->dd_rows.p, rows.data(), sizeof(int) * d_nnzb, cudaMemcpyHostToDevice), "upload D rows");
            FK_TRY(cudaMemcpy(e->dd_pair.p, pair.data(), sizeof(int) * d_nnzb, cudaMemcpyHostToDevice), "upload D pairs");
        }
        e->d_nb = d_n_b;
        e->d_nnzb = d_nnzb;
        e->d_symmetric = sym;
        e->d_same_as_H = d_nnzb == e->nnzb && std::equal(rp, rp + d_n_b + 1, e->h_row_ptr.begin()) &&
                         std::equal(ci, ci + d_nnzb, e->h_col.begin());
    }
    if (need_pairs && !e->d_symmetric)
        return e->fail(FK_ERR_PATTERN, "D pattern is not symmetric: a block (i,j) has no (j,i) partner");
    const size_t dbytes = sizeof(double) * (size_t)std::max(d_nnzb, 1) * e->b * e->b * (e->cplx ? 2 : 1);
    FK_TRY(e->dd_acc.ensure(dbytes), "alloc D accumulator");
    return FK_OK;
}

// DS engines, and FP32 engines without FK_OPT_ACC64, accumulate D as float-float pairs; turn them
// into doubles in place.
int finish_D_accumulator(fk_engine* e, size_t n_reals) {
    if (e->prec == fk::kF64 || (e->prec == fk::kF32 && e->opt_acc64) || n_reals == 0) return FK_OK;
    const int grid = (int)std::max<long long>(1, std::min<long long>(((long long)n_reals + 255) / 256, 152LL * 16));
    ProfScope ps(e, fk::kHelper);
    fk::k_ds_to_double<<<grid, 256, 0, e->stream>>>(e->dd_acc.as<double>(), (long long)n_reals);
    FK_TRY(cudaGetLastError(), "accumulator conversion");
    return FK_OK;
}

int ensure_coef(fk_engine* e, size_t ndoubles) {
    FK_TRY(e->d_coef.ensure(sizeof(double) * std::max<size_t>(ndoubles, 1)), "alloc coefficients");
    return FK_OK;
}

int ensure_partials(fk_engine* e, int nsteps) {
    const KCfg& c = e->cfg[fk::kStep];
    FK_TRY(e->d_partials.ensure(sizeof(double) * 2 * (size_t)nsteps * c.slices * c.ctas), "alloc partials");
    FK_TRY(e->d_raw.ensure(sizeof(double) * 2 * (size_t)nsteps), "alloc moment sums");
    return FK_OK;
}

__global__ void k_reduce_steps(const double* partials, int per_step, double* raw, int nsteps) {
    // one warp per step: fixed-order sum of per_step (= slices * ctas) CTA partials
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nsteps) return;
    const double* p = partials + (size_t)w * per_step * 2;
    double a = 0.0, bsum = 0.0;
    for (int c = lane; c < per_step; c += 32) { a += p[2 * c]; bsum += p[2 * c + 1]; }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        bsum += __shfl_xor_sync(0xffffffffu, bsum, off);
    }
    if (lane == 0) { raw[2 * w] = a; raw[2 * w + 1] = bsum; }
}

int moments_enqueue(fk_engine* e, int M) {
    if (M < 2 || M % 2 != 0) return e->fail(FK_ERR_ARG, "moments: M must be even and >= 2 (got %d)", M);
    int rc = require_ready(e);
    if (rc != FK_OK) return rc;
    const int nsteps = M / 2;
    rc = ensure_partials(e, nsteps);
    if (rc != FK_OK) return rc;
    const KCfg& c = e->cfg[fk::kStep];
    const size_t per_step = (size_t)c.slices * c.ctas * 2;
    double* part = e->d_partials.as<double>();
    auto launches = [&]() -> int {
        // step 0: alpha_1 = Hs R; dots <R,R>, Re<alpha_1,R>
        int r = run_step(e, e->d_R.p, nullptr, e->d_V[0].p, false, true, 0, nullptr, nullptr, part);
        if (r != FK_OK) return r;
        int x = 0, z = -1;   // x = alpha_m, z = alpha_{m-1}  (-1 = R)
        for (int m = 1; m < nsteps; m++) {
            const int y = (z == -1) ? 1 : z;   // never overwrite R
            r = run_step(e, e->V(x), e->V(z), e->V(y), true, true, 0, nullptr, nullptr, part + per_step * m);
            if (r != FK_OK) return r;
            z = x;
            x = y;
        }
        ProfScope ps(e, fk::kHelper);
        k_reduce_steps<<<(nsteps * 32 + 255) / 256, 256, 0, e->stream>>>(part, (int)(per_step / 2), e->d_raw.as<double>(), nsteps);
        FK_TRY(cudaGetLastError(), "moment reduction launch");
        return FK_OK;
    };
    rc = run_launches(e, graph_key(0, M, 0), launches);
    if (rc != FK_OK) return rc;
    // buffer roles after the loop: alpha_{M/2-1} in z, alpha_{M/2} in x
    int x = 0, z = -1;
    for (int m = 1; m < nsteps; m++) {
        const int y = (z == -1) ? 1 : z;
        z = x;
        x = y;
    }
    e->mom_M = M;
    e->mom_a0 = z;
    e->mom_a1 = x;
    e->pending_M = M;
    return FK_OK;
}

int moments_fetch(fk_engine* e, double* mu) {
    if (e->pending_M == 0) return e->fail(FK_ERR_STATE, "no moments enqueued");
    const int M = e->pending_M, nsteps = M / 2;
    e->h_raw.resize(2 * (size_t)nsteps);
    FK_TRY(cudaMemcpyAsync(e->h_raw.data(), e->d_raw.p, sizeof(double) * 2 * nsteps, cudaMemcpyDeviceToHost, e->stream),
           "copy moment sums");
    FK_TRY(cudaStreamSynchronize(e->stream), "moments");
    if (int rc = check_staged_error(e)) return rc;
    // mu_0 = <a0,a0>, mu_1 = Re<a1,a0>, mu_2m = 2<a_m,a_m> - mu_0, mu_2m+1 = 2 Re<a_m+1,a_m> - mu_1
    mu[0] = e->h_raw[0];
    mu[1] = e->h_raw[1];
    for (int m = 1; m < nsteps; m++) {
        mu[2 * m] = 2 * e->h_raw[2 * m] - mu[0];
        mu[2 * m + 1] = 2 * e->h_raw[2 * m + 1] - mu[1];
    }
    if (e->profiling) prof_flush(e);
    return FK_OK;
}

int stoch_enqueue(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb, const int* rp, const int* ci) {
    if (M < 2) return e->fail(FK_ERR_ARG, "stoch_matrix: need at least 2 coefficients (got %d)", M);
    if (!c) return e->fail(FK_ERR_ARG, "stoch_matrix: null coefficients");
    int rc = require_ready(e);
    if (rc != FK_OK) return rc;
    rc = set_D_pattern(e, d_n_b, d_nnzb, rp, ci, false);
    if (rc != FK_OK) return rc;
    rc = ensure_coef(e, 2 * (size_t)M);
    if (rc != FK_OK) return rc;
    std::vector<double> coef(2 * (size_t)M, 0.0);
    coef[0] = c[0];
    coef[1] = c[1];
    for (int m = 2; m < M; m++) coef[2 * m + 1] = c[m];
    FK_TRY(cudaMemcpyAsync(e->d_coef.p, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, e->stream),
           "upload coefficients");
    const double* cd = e->d_coef.as<double>();
    void* xi = e->d_V[2].p;
    const size_t dn = (size_t)d_nnzb * e->b * e->b * (e->cplx ? 2 : 1);
    auto launches = [&]() -> int {
        // m = 1: alpha_1 = Hs R, xi = c0 R + c1 alpha_1
        int r = run_step(e, e->d_R.p, nullptr, e->d_V[0].p, false, false, 1, xi, cd, nullptr);
        if (r != FK_OK) return r;
        int x = 0, z = -1;
        for (int m = 2; m < M; m++) {
            const int y = (z == -1) ? 1 : z;
            r = run_step(e, e->V(x), e->V(z), e->V(y), true, false, 2, xi, cd + 2 * m, nullptr);
            if (r != FK_OK) return r;
            z = x;
            x = y;
        }
        // D = (R xi^dag + xi R^dag)/2 on D's pattern
        FK_TRY(cudaMemsetAsync(e->dd_acc.p, 0, sizeof(double) * std::max<size_t>(dn, 1), e->stream), "clear D");
        if (d_nnzb > 0) {
            r = run_outer(e, e->d_R.p, xi, 0.5, true);
            if (r != FK_OK) return r;
            r = finish_D_accumulator(e, dn);
            if (r != FK_OK) return r;
        }
        return FK_OK;
    };
    rc = run_launches(e, graph_key(1, M, 0), launches);
    if (rc != FK_OK) return rc;
    e->mom_M = 0;   // the recursion state is no longer the one autodiff needs (reference clears a0, a1)
    e->mom_a0 = e->mom_a1 = -2;
    return FK_OK;
}

// c: host coefficients, or (c == null) c_dev: device coefficients (the fixed-filling solve)
int autodiff_enqueue(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb, const int* rp, const int* ci,
                     const double* c_dev = nullptr) {
    if (!c && !c_dev) return e->fail(FK_ERR_ARG, "autodiff_matrix: null coefficients");
    int rc = require_ready(e);
    if (rc != FK_OK) return rc;
    if (e->mom_M == 0 || e->mom_M != M)
        return e->fail(FK_ERR_STATE, "autodiff_matrix(M=%d) needs moments(%d) first (have %d)", M, M, e->mom_M);
    rc = set_D_pattern(e, d_n_b, d_nnzb, rp, ci, true);
    if (rc != FK_OK) return rc;
    const size_t dn = (size_t)d_nnzb * e->b * e->b * (e->cplx ? 2 : 1);
    const int nsteps = M / 2 - 1;
    const size_t nadj = 3 * (size_t)std::max(nsteps, 1);
    rc = ensure_coef(e, nadj + 2);
    if (rc != FK_OK) return rc;
    if (c) {
        double diag = c[1];
        for (int m = 1; m < M / 2; m++) diag -= c[2 * m + 1];
        // per adjoint step q: {4 c_2m, 2 c_2m+1, 2 c_2m-1 or diag}; then the scale factors 2 c_{M-1}, diag
        std::vector<double> coef(nadj + 2, 0.0);
        for (int m = M / 2 - 1, q = 0; m >= 1; m--, q++) {
            coef[3 * q + 0] = 4 * c[2 * m];
            coef[3 * q + 1] = 2 * c[2 * m + 1];
            coef[3 * q + 2] = (m > 1) ? 2 * c[2 * m - 1] : diag;   // m = 1 folds diag * R R^dag into beta_1
        }
        coef[nadj] = 2 * c[M - 1];
        coef[nadj + 1] = diag;
        FK_TRY(cudaMemcpyAsync(e->d_coef.p, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice,
                               e->stream),
               "upload coefficients");
    } else {
        ProfScope ps(e, fk::kHelper);
        fk::k_adjoint_coefs<<<1, fk::kPostThreads, 0, e->stream>>>(c_dev, M, e->d_coef.as<double>());
        FK_TRY(cudaGetLastError(), "coefficient table launch");
    }
    // FK_OPT_FUSE_D: 0 never fuse, otherwise (1, 2 = default) fuse when D's pattern is H's.
    // Measured per reverse step on cubic L=64, S=256 (the fused kernel saves the outer product's
    // two gathered vector reads): FP32 3.10 ms fused vs 3.28 apart, DS 10.66 vs 10.92, FP64
    // 29.2 vs 30.4; 10^6-site cubic b=1 S=128: FP32 0.80 vs 1.00, DS 0.82 vs 0.91.
    const bool fuse_pref = e->opt_fuse_d != 0;
    const bool fuse = fuse_pref && e->d_same_as_H;
    // buffers: alpha_m in A, alpha_{m+1} in Ap (moments left alpha_{M/2-1}, alpha_{M/2})
    const double* scales = e->d_coef.as<double>() + nadj;   // [2 c_{M-1}, diag]
    auto launches = [&]() -> int {
        int A = e->mom_a0, Ap = e->mom_a1;
        int freeb[4], nf = 0;
        for (int q = 0; q < 4; q++) if (q != A && q != Ap) freeb[nf++] = q;
        int Bv = freeb[0], Bp = freeb[1];
        FK_TRY(cudaMemsetAsync(e->dd_acc.p, 0, sizeof(double) * std::max<size_t>(dn, 1), e->stream), "clear D");
        if (M > 2) {
            // beta_{M/2} = 2 c_{M-1} alpha_{M/2-1}, beta_{M/2+1} = 0
            FK_TRY(prec_scale(e, e->V(A), e->V(Bv), scales), "scale kernel");
            FK_TRY(cudaMemsetAsync(e->V(Bp), 0, e->vec_bytes(), e->stream), "clear beta");
            for (int m = M / 2 - 1, q = 0; m >= 1; m--, q++) {
                if (!fuse && d_nnzb > 0) {
                    const int r = run_outer(e, e->V(A), e->V(Bv), 2.0, false);   // D += 2 alpha_m beta_{m+1}^dag
                    if (r != FK_OK) return r;
                }
                const int r = run_adjoint(e, e->V(A), e->V(Ap), e->V(Bv), e->V(Bp), e->d_coef.as<double>() + 3 * q,
                                          fuse ? e->dd_acc.as<double>() : nullptr);
                if (r != FK_OK) return r;
                std::swap(A, Ap);    // A = alpha_{m-1}, Ap = alpha_m
                std::swap(Bv, Bp);   // Bv = beta_m,   Bp = beta_{m+1}
            }
        } else {
            // M = 2: D = diag R R^dag = R (diag R)^dag
            FK_TRY(prec_scale(e, e->V(A), e->V(Bv), scales + 1), "scale kernel");
        }
        // D += alpha_0 (beta_1 + diag alpha_0)^dag, then symmetrize and divide by mag
        if (d_nnzb > 0) {
            int r = run_outer(e, e->V(A), e->V(Bv), 1.0, false);
            if (r != FK_OK) return r;
            r = finish_D_accumulator(e, dn);
            if (r != FK_OK) return r;
            const double mag = (e->es_hi - e->es_lo) / 2.0;
            const long long work = (long long)d_nnzb * e->b * e->b;
            const int grid = (int)std::min<long long>((work + 255) / 256, 152LL * 16);
            ProfScope ps(e, fk::kHelper);
            fk::k_symmetrize_scale<<<std::max(grid, 1), 256, 0, e->stream>>>(
                e->dd_acc.as<double>(), e->dd_rows.as<int>(), e->dd_colc.as<int>(), e->dd_pair.as<int>(), d_nnzb, e->b,
                e->cplx, 1.0 / mag, nullptr);
            FK_TRY(cudaGetLastError(), "symmetrize launch");
        }
        return FK_OK;
    };
    rc = run_launches(e, graph_key(2, M, ((long long)fuse << 40) ^ ((long long)e->mom_a0 + 2) ^ ((long long)d_nnzb << 4)),
                      launches);
    if (rc != FK_OK) return rc;
    e->mom_M = 0;   // alpha state consumed (reference zeroes a_d[0..1])
    e->mom_a0 = e->mom_a1 = -2;
    return FK_OK;
}

int fetch_D(fk_engine* e, double* D) {
    if (e->d_nnzb < 0) return e->fail(FK_ERR_STATE, "no D computed");
    const size_t dn = (size_t)e->d_nnzb * e->b * e->b * (e->cplx ? 2 : 1);
    if (dn) FK_TRY(cudaMemcpyAsync(D, e->dd_acc.p, sizeof(double) * dn, cudaMemcpyDeviceToHost, e->stream), "copy D");
    FK_TRY(cudaStreamSynchronize(e->stream), "D calculation");
    if (int rc = check_staged_error(e)) return rc;
    if (e->profiling) prof_flush(e);
    return FK_OK;
}

// Layout of the post-processing buffer for (M, Mq): [mu M][gamma Mq][energies Mq][result 4][c M]
struct PostLayout {
    double *mu, *gamma, *en, *res, *c;
    static size_t doubles(int M, int Mq) { return 2 * (size_t)M + 2 * (size_t)Mq + 4; }
};
PostLayout post_layout(const fk_engine* e, int M, int Mq) {
    PostLayout l;
    l.mu = e->d_post.as<double>();
    l.gamma = l.mu + M;
    l.en = l.gamma + Mq;
    l.res = l.en + Mq;
    l.c = l.res + 4;
    return l;
}

// Post-processing of the last moments(M) on the device, enqueued behind it: moments from the
// per-step sums, gamma = moment_transform(mu, Mq), {mu_F, energy, n_tot} for the filling and,
// with want_coef, the fermi_energy expansion coefficients at mu_F (kT as given).
int post_enqueue(fk_engine* e, int Mq, double kT, double filling, double delta, bool want_coef) {
    const int M = e->pending_M;
    if (M == 0) return e->fail(FK_ERR_STATE, "kpm post-processing needs moments(M) first");
    if (Mq < M) return e->fail(FK_ERR_ARG, "kpm post-processing: Mq (%d) must be >= M (%d)", Mq, M);
    if (!(filling > 0.0 && filling < 1.0)) return e->fail(FK_ERR_ARG, "kpm post-processing: filling must be in (0, 1)");
    if (!(delta >= 0.0) || filling - delta <= 0.0 || filling + delta >= 1.0)
        return e->fail(FK_ERR_ARG, "kpm post-processing: need 0 <= delta_filling < min(filling, 1 - filling)");
    FK_TRY(e->d_post.ensure(sizeof(double) * PostLayout::doubles(M, Mq)), "alloc post-processing");
    const PostLayout pl = post_layout(e, M, Mq);
    double *mu = pl.mu, *gamma = pl.gamma, *en = pl.en, *res = pl.res, *c = pl.c;
    const double avg = (e->es_hi + e->es_lo) / 2.0, mag = (e->es_hi - e->es_lo) / 2.0;
    ProfScope ps(e, fk::kHelper);
    fk::k_moments_from_raw<<<(M + 255) / 256, 256, 0, e->stream>>>(e->d_raw.as<double>(), M, mu);
    fk::k_moment_transform<<<(Mq + 255) / 256, 256, 0, e->stream>>>(mu, M, Mq, avg, mag, gamma, en);
    fk::k_filling_solve<<<1, fk::kPostThreads, 0, e->stream>>>(gamma, en, Mq, e->es_lo, e->es_hi, kT, filling, delta, res);
    if (want_coef)
        fk::k_expansion_coefficients<<<M, fk::kPostThreads, 0, e->stream>>>(M, Mq, 1, kT, 0.0, res, avg, mag, c);
    FK_TRY(cudaGetLastError(), "post-processing launch");
    e->post_M = M;
    e->post_Mq = Mq;
    return FK_OK;
}

// result[0..3) = {mu_F, energy, n_tot}; gamma (optional) = Mq doubles
int post_fetch(fk_engine* e, double* result, double* gamma) {
    const PostLayout pl = post_layout(e, e->post_M, e->post_Mq);
    FK_TRY(cudaMemcpyAsync(result, pl.res, sizeof(double) * 3, cudaMemcpyDeviceToHost, e->stream), "copy results");
    if (gamma)
        FK_TRY(cudaMemcpyAsync(gamma, pl.gamma, sizeof(double) * e->post_Mq,
                               cudaMemcpyDeviceToHost, e->stream),
               "copy gamma");
    FK_TRY(cudaStreamSynchronize(e->stream), "post-processing");
    return FK_OK;
}

// ---- second-order moments (moments2_v1) ----

cudaError_t prec_export(fk_engine* e, const void* src, long long c0, int w, double* dst) {
    switch (e->prec) {
        case fk::kF64: return fk::launch_export_panel_f64(e->cplx, src, e->n, e->ld, c0, w, dst, e->stream);
        case fk::kF32: return fk::launch_export_panel_f32(e->cplx, src, e->n, e->ld, c0, w, dst, e->stream);
        default: return fk::launch_export_panel_ds(e->cplx, src, e->n, e->ld, c0, w, dst, e->stream);
    }
}

struct M2Mat {
    const int* row_ptr;
    const unsigned* colc;
    const void* hval;
};

// y = (two ? 2 : 1) A x (- z) on the packet columns [c0_el / EPP, + P_sl) of the row-major
// vectors, with the step kernel's launch shape (any BSR A with H's block rows fits it: the H
// stage holds stage_cap blocks and tiles with more blocks read A from global memory).
int m2_step(fk_engine* e, const M2Mat& A, const void* x, const void* z, void* y, bool two, long long c0_el, int P_sl) {
    const KCfg& c = e->cfg[fk::kStep];
    const size_t es = e->esize();
    fk::StepArgs a;
    a.sys = c.sys.as<SysDesc>();
    a.cta_sys = c.cta_sys.as<int>();
    a.Gp = c.Gp;
    a.P = P_sl;
    a.ld = e->ld;
    a.row_ptr = A.row_ptr;
    a.colc = A.colc;
    a.hval = A.hval;
    a.x = (const char*)x + c0_el * es;
    a.z = z ? (const char*)z + c0_el * es : nullptr;
    a.y = (char*)y + c0_el * es;
    a.xi = nullptr;
    a.coef = nullptr;
    a.cstride = 0;
    a.two = two;
    a.has_z = z != nullptr;
    a.want_dots = 0;
    a.xi_mode = 0;
    a.partials = nullptr;
    // the staged (TMA) configuration sizes its shared memory differently: run unstaged then
    a.stage_cap = c.staged ? 0 : c.stage_cap;
    a.pipe = 0;
    ProfScope ps(e, fk::kStep);
    FK_TRY(prec_launch_step(e, c.NP, a, fk::Launch{c.ctas, c.staged ? 0 : c.smem, e->stream}), "moments2 step");
    return FK_OK;
}

// C[i + j ldc] = (accumulate ? C : 0) + sum_k opA(i, k) opB(k, j) in FP64 on the engine's stream
// (fk_gram.cuh): opA(i, k) = A[i a_si + k a_sk] (conjugated when conj_a), opB(k, j) = B[k b_sk +
// j b_sj] (conjugated when conj_b). The contraction is split over enough CTAs to fill the GPU.
int gram(fk_engine* e, int m, int n, long long kdim, const double* A, long long a_si, long long a_sk, bool conj_a,
         const double* B, long long b_sk, long long b_sj, bool conj_b, double* C, long long ldc, bool accumulate,
         const char* what) {
    const size_t elt = e->cplx ? 16 : 8;
    const long long tiles = (long long)((m + fk::kGramTile - 1) / fk::kGramTile) * ((n + fk::kGramTile - 1) / fk::kGramTile);
    const long long want = std::max<long long>(1, (4LL * e->num_sms + tiles - 1) / tiles);   // ~4 CTAs per SM
    long long splits = std::min<long long>(want, std::max<long long>(1, kdim / (4 * fk::kGramDepth)));
    // keep the workspace of partial tiles within 256 MB
    const long long cap = std::max<long long>(1, (256LL << 20) / std::max<long long>(1, (long long)m * n * (long long)elt));
    splits = std::max<long long>(1, std::min<long long>({splits, cap, 65535LL}));
    long long per = (kdim + splits - 1) / splits;
    per = (per + fk::kGramDepth - 1) / fk::kGramDepth * fk::kGramDepth;
    splits = std::max<long long>(1, (kdim + per - 1) / per);
    FK_TRY(e->d_gram.ensure((size_t)splits * m * n * elt), "alloc product workspace");
    fk::GramArgs g{m, n, kdim, per, A, a_si, a_sk, conj_a ? 1 : 0, B, b_sk, b_sj, conj_b ? 1 : 0, e->d_gram.as<double>()};
    const dim3 grid((m + fk::kGramTile - 1) / fk::kGramTile, (n + fk::kGramTile - 1) / fk::kGramTile, (unsigned)splits);
    const int rg = (int)std::max<long long>(1, std::min<long long>(((long long)m * n + 255) / 256, 152LL * 8));
    ProfScope ps(e, fk::kHelper);
    if (e->cplx) {
        fk::k_gram_partial<true><<<grid, fk::kGramThreads, 0, e->stream>>>(g);
        fk::k_gram_reduce<true><<<rg, 256, 0, e->stream>>>(e->d_gram.as<double>(), (int)splits, m, n, C, ldc, accumulate);
    } else {
        fk::k_gram_partial<false><<<grid, fk::kGramThreads, 0, e->stream>>>(g);
        fk::k_gram_reduce<false><<<rg, 256, 0, e->stream>>>(e->d_gram.as<double>(), (int)splits, m, n, C, ldc, accumulate);
    }
    FK_TRY(cudaGetLastError(), what);
    return FK_OK;
}

// Upload operator q (j1 or j2) in the engine's format: H's block rows, unscaled (energy scale
// [-1, 1]), a zero diagonal block inserted where a row has none.
int m2_upload_op(fk_engine* e, int q, int nnzb, const int* rp, const int* ci, const double* val) {
    fk::PreparedH ph;
    std::string why;
    const int rc = fk::prepare_H(e->prec, e->cplx, e->n_b, e->b, nnzb, rp, ci, val, -1.0, 1.0, 0, ph, why);
    if (rc != FK_OK) return e->fail(rc, "moments2_v1: j%d: %s", q + 1, why.c_str());
    fk_engine::Op& op = e->d_j[q];
    FK_TRY(op.row_ptr.ensure(sizeof(int) * ph.row_ptr.size()), "alloc operator");
    FK_TRY(op.colc.ensure(sizeof(unsigned) * std::max<size_t>(ph.colc.size(), 1)), "alloc operator");
    FK_TRY(op.hval.ensure(std::max<size_t>(ph.hval.size(), 16)), "alloc operator");
    FK_TRY(cudaMemcpy(op.row_ptr.p, ph.row_ptr.data(), sizeof(int) * ph.row_ptr.size(), cudaMemcpyHostToDevice),
           "upload operator");
    if (!ph.colc.empty()) {
        FK_TRY(cudaMemcpy(op.colc.p, ph.colc.data(), sizeof(unsigned) * ph.colc.size(), cudaMemcpyHostToDevice),
               "upload operator");
        FK_TRY(cudaMemcpy(op.hval.p, ph.hval.data(), ph.hval.size(), cudaMemcpyHostToDevice), "upload operator");
    }
    return FK_OK;
}

// moments2_v1 (reference src/engine_cpu.cpp:86-160, src/engine_cusparse.cpp:793-902):
//   mu[m1][m2] = sum_k <T_m1(Hs) r_k, j2 T_m2(Hs) j1 r_k>.
// The probe columns run in slices of r_chunk columns (all at once by default); per slice the
// Chebyshev vectors alpha_m = T_m r and j2 atild_m (atild_m = T_m j1 r) are written, K orders
// at a time, as double panels, and mu's K x K blocks are one GEMM each (A^H B over the panel
// rows) instead of the reference's M^2 separate dot products. K = a_chunk when >= 3, else the
// largest that fits 60% of free device memory (K = M: every recursion runs once per slice).
// Each panel of atild restarts its recursion from j1 r, as the reference does.
int moments2_v1(fk_engine* e, int M, const int* nnzb, const int* const* rp, const int* const* ci,
                const double* const* val, int a_chunk, int r_chunk, double* mu_out) {
    if (M < 2 || M % 2 != 0) return e->fail(FK_ERR_ARG, "moments2_v1: M must be even and >= 2 (got %d)", M);
    int rc = require_ready(e);
    if (rc != FK_OK) return rc;
    for (int q = 0; q < 2; q++) {
        rc = m2_upload_op(e, q, nnzb[q], rp[q], ci[q], val[q]);
        if (rc != FK_OK) return rc;
    }
    const int epp = e->epp();
    const int w_el = r_chunk > 0 ? std::min(r_chunk, e->s) : e->s;
    int wp = (w_el + epp - 1) / epp;                                  // packets per column slice
    while (wp > 1 && (long long)e->n * wp * epp >= (1LL << 31)) wp = (wp + 1) / 2;   // GEMM sizes are int
    if ((long long)e->n * wp * epp >= (1LL << 31)) return e->fail(FK_ERR_UNSUPPORTED, "moments2_v1: too many rows");
    const int nsl = (e->P + wp - 1) / wp;
    const long long Lmax = (long long)e->n * wp * epp;
    const size_t elt = e->cplx ? 16 : 8;
    int K;
    if (a_chunk >= 3) {
        K = std::min(a_chunk, M);
    } else {
        size_t fr = 0, tot = 0;
        FK_TRY(cudaMemGetInfo(&fr, &tot), "memory query");
        const size_t per = 2 * (size_t)Lmax * elt;
        K = (int)std::min<size_t>(M, std::max<size_t>(2, fr / 10 * 6 / per));
    }
    FK_TRY(e->d_panel[0].ensure((size_t)K * Lmax * elt), "alloc panel");
    FK_TRY(e->d_panel[1].ensure((size_t)K * Lmax * elt), "alloc panel");
    FK_TRY(e->d_tmp.ensure(e->vec_bytes()), "alloc scratch vector");
    FK_TRY(e->d_mu2.ensure((size_t)M * M * elt), "alloc moments");
    FK_TRY(cudaMemsetAsync(e->d_mu2.p, 0, (size_t)M * M * elt, e->stream), "clear moments");
    const M2Mat hs{e->d_row_ptr.as<int>(), e->d_colc.as<unsigned>(), e->d_hval.p};
    const M2Mat j1{e->d_j[0].row_ptr.as<int>(), e->d_j[0].colc.as<unsigned>(), e->d_j[0].hval.p};
    const M2Mat j2{e->d_j[1].row_ptr.as<int>(), e->d_j[1].colc.as<unsigned>(), e->d_j[1].hval.p};
    void* R = e->d_R.p;
    void* V[4] = {e->d_V[0].p, e->d_V[1].p, e->d_V[2].p, e->d_V[3].p};
    char* PA = e->d_panel[0].as<char>();
    char* PB = e->d_panel[1].as<char>();
    for (int sl = 0; sl < nsl; sl++) {
        const long long c0 = (long long)sl * wp * epp;
        const int P_sl = std::min(wp, e->P - sl * wp);
        const int w = P_sl * epp;
        const long long L = (long long)e->n * w;
        // alpha_m = T_m(Hs) r: alpha_0 = R, then two rotating vectors (never overwriting R)
        const void* aP = nullptr;
        void* aC = nullptr;
        int am = -1;
        auto alpha_next = [&]() -> int {
            const int m = ++am;
            if (m == 0) { aC = R; return FK_OK; }
            void* y = m == 1 ? V[0] : (aP == R ? V[1] : const_cast<void*>(aP));
            const int r = m2_step(e, hs, aC, m == 1 ? nullptr : aP, y, m > 1, c0, P_sl);
            aP = aC;
            aC = y;
            return r;
        };
        for (int a0 = 0; a0 < M; a0 += K) {
            const int Ka = std::min(K, M - a0);
            for (int q = 0; q < Ka; q++) {
                rc = alpha_next();
                if (rc != FK_OK) return rc;
                FK_TRY(prec_export(e, aC, c0, w, reinterpret_cast<double*>(PA + (size_t)q * L * elt)), "export panel");
            }
            // atild_m = T_m(Hs) j1 r, restarted for every alpha panel; panel B holds j2 atild_m
            void* tP = nullptr;
            void* tC = nullptr;
            for (int b0 = 0, tm = -1; b0 < M; b0 += K) {
                const int Kb = std::min(K, M - b0);
                for (int q = 0; q < Kb; q++) {
                    const int m = ++tm;
                    void* y = m == 0 ? V[2] : (m == 1 ? V[3] : tP);
                    rc = m == 0 ? m2_step(e, j1, R, nullptr, y, false, c0, P_sl)
                                : m2_step(e, hs, tC, m == 1 ? nullptr : tP, y, m > 1, c0, P_sl);
                    if (rc != FK_OK) return rc;
                    tP = tC;
                    tC = y;
                    rc = m2_step(e, j2, tC, nullptr, e->d_tmp.p, false, c0, P_sl);
                    if (rc != FK_OK) return rc;
                    FK_TRY(prec_export(e, e->d_tmp.p, c0, w, reinterpret_cast<double*>(PB + (size_t)q * L * elt)),
                           "export panel");
                }
                // mu[a0 .. a0+Ka, b0 .. b0+Kb] += A^H B   (mu column-major M x M on the device):
                // mu[a, b] += sum_l conj(PA[l + a L]) PB[l + b L]
                rc = gram(e, Ka, Kb, L, reinterpret_cast<const double*>(PA), L, 1, true,
                          reinterpret_cast<const double*>(PB), 1, L, false,
                          e->d_mu2.as<double>() + (a0 + (size_t)b0 * M) * (elt / 8), M, true, "moments2 product");
                if (rc != FK_OK) return rc;
            }
        }
    }
    std::vector<double> h((size_t)M * M * (e->cplx ? 2 : 1));
    FK_TRY(cudaMemcpyAsync(h.data(), e->d_mu2.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, e->stream),
           "copy moments");
    FK_TRY(cudaStreamSynchronize(e->stream), "moments2_v1");
    for (int m1 = 0; m1 < M; m1++)
        for (int m2 = 0; m2 < M; m2++) {
            const size_t src = (size_t)m1 + (size_t)m2 * M, dst = (size_t)m1 * M + m2;
            mu_out[2 * dst] = e->cplx ? h[2 * src] : h[src];
            mu_out[2 * dst + 1] = e->cplx ? h[2 * src + 1] : 0.0;
        }
    // the work vectors no longer hold the moments' recursion state
    e->mom_M = 0;
    e->mom_a0 = e->mom_a1 = -2;
    if (e->profiling) prof_flush(e);
    return FK_OK;
}

}  // namespace

// ===================================================================================
// Lanczos energy_scale on the device
// ===================================================================================
namespace {

// alpha_j = sum of the step kernel's per-CTA Re<Hv, v> partials (odd entries), in CTA order
__global__ void k_lanczos_alpha(const double* step_part, int ctas, double* alpha) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0;
    for (int q = 0; q < ctas; q++) a += step_part[2 * q + 1];
    *alpha = a;
}

// beta_j = sqrt(sum of |w|^2 partials) in CTA order, and 1/beta_j (0 once the Krylov space is exhausted)
__global__ void k_lanczos_beta(const double* part, int n, double* beta, double* inv_beta) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int q = 0; q < n; q++) s += part[q];
    const double b = sqrt(s);
    *beta = b;
    *inv_beta = b > 0.0 ? 1.0 / b : 0.0;
}

// w <- w - alpha_j v1 - beta_{j-1} v0 (real or complex doubles), partial |w|^2 per CTA
__global__ void k_lanczos_update(double* w, const double* v1, const double* v0, long long n_dbl, const double* alpha,
                                 const double* beta, double* part) {
    const double al = *alpha, be = *beta;
    double acc = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n_dbl; q += (long long)gridDim.x * blockDim.x) {
        const double v = w[q] - al * v1[q] - be * v0[q];
        w[q] = v;
        acc += v * v;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        part[blockIdx.x] = t;
    }
}

}  // namespace

namespace {
int sturm(int n, const double* a, const double* bt, double x) {
    int cnt = 0;
    double q = a[0] - x;
    if (q < 0) cnt++;
    for (int j = 1; j < n; j++) {
        q = a[j] - x - bt[j] * bt[j] / (q == 0 ? 1e-300 : q);
        if (q < 0) cnt++;
    }
    return cnt;
}
void tridiag_extremes(int n, const double* a, const double* bt, double* emin, double* emax) {
    double glo = 1e300, ghi = -1e300;
    for (int j = 0; j < n; j++) {
        const double r = (j > 0 ? std::fabs(bt[j]) : 0.0) + (j + 1 < n ? std::fabs(bt[j + 1]) : 0.0);
        glo = std::min(glo, a[j] - r);
        ghi = std::max(ghi, a[j] + r);
    }
    auto kth = [&](int k) {
        double l = glo, h = ghi;
        for (int it = 0; it < 200 && h - l > 1e-15 * std::max(1.0, std::fabs(l) + std::fabs(h)); it++) {
            const double mid = 0.5 * (l + h);
            if (sturm(n, a, bt, mid) > k) h = mid; else l = mid;
        }
        return 0.5 * (l + h);
    };
    *emin = kth(0);
    *emax = kth(n - 1);
}
}  // namespace

// ===================================================================================
// C ABI
// ===================================================================================
extern "C" {

const char* fk_version(void) { return "fastkpm_gb300 0.1 (sm_103a)"; }

const char* fk_status_string(int s) {
    switch (s) {
        case FK_OK: return "ok";
        case FK_ERR_ARG: return "invalid argument";
        case FK_ERR_OOM: return "out of device memory";
        case FK_ERR_PATTERN: return "malformed sparsity pattern";
        case FK_ERR_TIMEOUT: return "timeout";
        case FK_ERR_CUDA: return "CUDA error";
        case FK_ERR_STATE: return "invalid call order";
        case FK_ERR_NODEV: return "no CUDA device";
        case FK_ERR_UNSUPPORTED: return "unsupported";
        default: return "unknown status";
    }
}

int fk_device_count(int* count) {
    if (!count) return FK_ERR_ARG;
    int c = 0;
    cudaError_t ce = cudaGetDeviceCount(&c);
    if (ce != cudaSuccess) { cudaGetLastError(); *count = 0; return FK_ERR_NODEV; }
    *count = c;
    return FK_OK;
}

int fk_device_fma_rate(int device, int fp64, double* tflops) {
    if (!tflops) return FK_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { cudaGetLastError(); return FK_ERR_NODEV; }
    if (device < 0 || device >= count) return FK_ERR_ARG;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    double* sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    int rc = FK_OK;
    const int blocks = sms * 8;
    const int iters = fp64 ? 2048 : 65536;
    float ms = 0.f;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess ||
        cudaEventCreate(&b) != cudaSuccess) {
        rc = FK_ERR_CUDA;
    } else {
        for (int rep = 0; rep < 2 && rc == FK_OK; rep++) {   // the first launch warms the clocks up
            cudaEventRecord(a);
            if (fp64) k_fma_rate<double><<<blocks, kFmaThreads>>>(sink, iters, 1.0);
            else k_fma_rate<float><<<blocks, kFmaThreads>>>(sink, iters, 1.0f);
            cudaEventRecord(b);
            if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) rc = FK_ERR_CUDA;
        }
    }
    if (rc == FK_OK) {
        const double flops = 2.0 * kFmaChains * (double)iters * kFmaThreads * (double)blocks;
        *tflops = flops / (ms * 1e-3) / 1e12;
    }
    cudaGetLastError();
    if (sink) cudaFree(sink);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaSetDevice(prev);
    return rc;
}

int fk_device_memory(int device, size_t* free_bytes, size_t* total_bytes) {
    if (!free_bytes || !total_bytes) return FK_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { cudaGetLastError(); return FK_ERR_NODEV; }
    if (device < 0 || device >= count) return FK_ERR_ARG;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaError_t ce = cudaMemGetInfo(free_bytes, total_bytes);
    cudaSetDevice(prev);
    if (ce != cudaSuccess) { cudaGetLastError(); return FK_ERR_CUDA; }
    return FK_OK;
}

int fk_engine_create(int device, int kind, int precision, fk_engine** out) {
    if (!out) return FK_ERR_ARG;
    *out = nullptr;
    if (kind != FK_REAL && kind != FK_COMPLEX) return FK_ERR_ARG;
    if (precision < FK_PREC_FP64 || precision > FK_PREC_DS) return FK_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { cudaGetLastError(); return FK_ERR_NODEV; }
    if (device < 0 || device >= count) return FK_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return FK_ERR_CUDA; }
    fk_engine* e = new fk_engine();
    e->device = device;
    e->cplx = kind;
    e->prec = precision;
    cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device);
    {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device);
        e->l2_bytes = l2;
    }
    if (cudaDeviceGetAttribute(&e->pageable_access, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        cudaGetLastError();
        e->pageable_access = 0;
    }
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete e;
        return FK_ERR_CUDA;
    }
    e->own_stream = true;
    *out = e;
    return FK_OK;
}

int fk_engine_destroy(fk_engine* e) {
    if (!e) return FK_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto& p : e->prof_pending) { e->prof_pool.push_back(p.a); e->prof_pool.push_back(p.b); }
    for (auto ev : e->prof_pool) cudaEventDestroy(ev);
    if (e->t_start) cudaEventDestroy(e->t_start);
    if (e->t_stop) cudaEventDestroy(e->t_stop);
    drop_graphs(e);
    if (e->copy_stream) {
        cudaStreamSynchronize(e->copy_stream);
        cudaStreamDestroy(e->copy_stream);
        for (int q = 0; q < 2; q++) { cudaEventDestroy(e->ev_copied[q]); cudaEventDestroy(e->ev_consumed[q]); }
    }
    for (auto& op : e->d_j) { op.row_ptr.release(); op.colc.release(); op.hval.release(); }
    for (auto& pb : e->d_panel) pb.release();
    e->d_tmp.release();
    e->d_mu2.release();
    e->d_R2.release();
    DevBuf* bufs[] = {&e->d_row_ptr, &e->d_colc, &e->d_hval, &e->d_R, &e->d_V[0], &e->d_V[1], &e->d_V[2], &e->d_V[3],
                      &e->dd_row_ptr, &e->dd_colc, &e->dd_rows, &e->dd_pair, &e->dd_acc, &e->d_partials, &e->d_raw,
                      &e->d_coef, &e->d_stage, &e->d_post, &e->d_t_uoff, &e->d_t_ucol, &e->d_t_own, &e->d_t_kslot,
                      &e->d_t_base, &e->d_err, &e->d_row_hsum};
    for (auto* b : bufs) b->release();
    for (auto& c : e->cfg) { c.sys.release(); c.cta_sys.release(); }
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return FK_OK;
}

const char* fk_engine_last_error(const fk_engine* e) { return e ? e->err.c_str() : "null engine"; }

int fk_engine_set_stream(fk_engine* e, void* st) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    if (e->own_stream && e->stream) { cudaStreamSynchronize(e->stream); cudaStreamDestroy(e->stream); }
    e->opt_priority = 0;
    if (st) { e->stream = (cudaStream_t)st; e->own_stream = false; }
    else {
        if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) return e->fail(FK_ERR_CUDA, "stream create");
        e->own_stream = true;
    }
    return FK_OK;
}

int fk_engine_synchronize(fk_engine* e) {
    if (!e) return FK_ERR_ARG;
    FK_TRY(cudaStreamSynchronize(e->stream), "synchronize");
    return FK_OK;
}

int fk_engine_set_option(fk_engine* e, int option, int value) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    switch (option) {
        case FK_OPT_FUSE_D:
            if (value < 0 || value > 2) return e->fail(FK_ERR_ARG, "FUSE_D must be 0, 1 or 2");
            e->opt_fuse_d = value;
            return FK_OK;
        case FK_OPT_NP:
            if (value != 0 && value != 1 && value != 2 && value != 4) return e->fail(FK_ERR_ARG, "NP must be 0, 1, 2 or 4");
            e->opt_np = value;
            for (int& v : e->opt_np_kind) v = 0;
            return configure(e);
        case FK_OPT_NP_STEP:
        case FK_OPT_NP_ADJOINT:
        case FK_OPT_NP_OUTER:
            if (value != 0 && value != 1 && value != 2 && value != 4) return e->fail(FK_ERR_ARG, "NP must be 0, 1, 2 or 4");
            e->opt_np_kind[option - FK_OPT_NP_STEP] = value;
            return configure(e);
        case FK_OPT_CTAS_PER_SM:
            if (value < 0) return e->fail(FK_ERR_ARG, "negative CTA cap");
            e->opt_ctas_per_sm = value; return configure(e);
        case FK_OPT_STAGE_H:
            if (value < 0 || value > 2) return e->fail(FK_ERR_ARG, "STAGE_H must be 0, 1 or 2");
            e->opt_stage = value;
            return configure(e);
        case FK_OPT_GRAPHS:
            e->opt_graphs = value ? 1 : 0;
            if (!e->opt_graphs) drop_graphs(e);
            return FK_OK;
        case FK_OPT_UPLOAD:
            if (value < 0 || value > 1) return e->fail(FK_ERR_ARG, "UPLOAD must be 0 or 1");
            e->opt_upload = value;
            return FK_OK;
        case FK_OPT_PIPE:
            if (value < 0 || value > 2) return e->fail(FK_ERR_ARG, "PIPE must be 0, 1 or 2");
            e->opt_pipe = value;
            drop_graphs(e);
            return configure(e);
        case FK_OPT_CTA_WAVES:
            if (value < 1 || value > 64) return e->fail(FK_ERR_ARG, "CTA_WAVES must be 1 .. 64");
            e->opt_waves = value;
            drop_graphs(e);
            return configure(e);
        case FK_OPT_ACC64:
            if (value < 0 || value > 1) return e->fail(FK_ERR_ARG, "ACC64 must be 0 or 1");
            e->opt_acc64 = value;   // the kept recursion state stays valid: every D call starts its accumulator anew
            drop_graphs(e);
            return configure(e);
        case FK_OPT_WARP_ROWS:
            if (value < 0 || value > 1) return e->fail(FK_ERR_ARG, "WARP_ROWS must be 0 or 1");
            e->opt_warp = value;
            drop_graphs(e);
            return configure(e);
        case FK_OPT_ADJ_SWEEP:
            if (value < 0 || value > 2) return e->fail(FK_ERR_ARG, "ADJ_SWEEP must be 0, 1 or 2");
            e->opt_sweep = value;
            drop_graphs(e);
            return configure(e);
        case FK_OPT_ADJ_SPLIT:
            if (value < 0 || value > 2) return e->fail(FK_ERR_ARG, "ADJ_SPLIT must be 0, 1 or 2");
            e->opt_adj_split = value;
            drop_graphs(e);
            return configure(e);
        case FK_OPT_PRIORITY: {
            if (!e->own_stream) return e->fail(FK_ERR_STATE, "PRIORITY applies to the engine's own stream, not a caller's");
            int least = 0, greatest = 0;
            FK_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest), "priority range");
            const int p = std::max(greatest, std::min(least, value));
            if (p == e->opt_priority) return FK_OK;
            cudaStream_t ns = nullptr;
            FK_TRY(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, p), "stream create");
            cudaStreamSynchronize(e->stream);
            cudaStreamDestroy(e->stream);
            e->stream = ns;
            e->opt_priority = p;
            return FK_OK;
        }
        case FK_OPT_TMA:
            if (value < 0 || value > 2) return e->fail(FK_ERR_ARG, "TMA must be 0, 1 or 2");
            e->opt_tma = value;
            return configure(e);
        default: return e->fail(FK_ERR_ARG, "unknown option %d", option);
    }
}

int fk_engine_get_option(const fk_engine* e, int option, int* value) {
    if (!e || !value) return FK_ERR_ARG;
    switch (option) {
        case FK_OPT_FUSE_D: *value = e->opt_fuse_d; return FK_OK;
        case FK_OPT_NP: *value = e->cfg[0].valid ? e->cfg[0].NP : e->opt_np; return FK_OK;
        case FK_OPT_NP_STEP:
        case FK_OPT_NP_ADJOINT:
        case FK_OPT_NP_OUTER: {
            const int k = option - FK_OPT_NP_STEP;
            *value = e->cfg[k].valid ? e->cfg[k].NP : e->opt_np_kind[k];
            return FK_OK;
        }
        case FK_OPT_CTAS_PER_SM: *value = e->opt_ctas_per_sm; return FK_OK;
        case FK_OPT_STAGE_H: *value = e->opt_stage; return FK_OK;
        case FK_OPT_GRAPHS: *value = e->opt_graphs; return FK_OK;
        case FK_OPT_UPLOAD: *value = e->opt_upload; return FK_OK;
        case FK_OPT_PRIORITY: *value = e->opt_priority; return FK_OK;
        case FK_OPT_ADJ_SPLIT: *value = e->opt_adj_split; return FK_OK;
        case FK_OPT_PIPE: *value = e->cfg[fk::kStep].valid ? (int)e->cfg[fk::kStep].pipe : e->opt_pipe; return FK_OK;
        case FK_OPT_ACC64: *value = e->prec == fk::kF64 ? 1 : e->prec == fk::kF32 ? e->opt_acc64 : 0; return FK_OK;
        case FK_OPT_CTA_WAVES: *value = e->opt_waves; return FK_OK;
        case FK_OPT_WARP_ROWS: *value = e->cfg[fk::kAdjoint].valid ? (int)e->cfg[fk::kAdjoint].warp : e->opt_warp; return FK_OK;
        case FK_OPT_ADJ_SWEEP: *value = e->cfg[fk::kAdjoint].valid ? (int)(e->cfg[fk::kAdjoint].slices > 1) : e->opt_sweep; return FK_OK;
        case FK_OPT_TMA: *value = e->cfg[fk::kStep].valid ? (e->cfg[fk::kStep].staged ? e->opt_tma : 0) : e->opt_tma; return FK_OK;
        default: return FK_ERR_ARG;
    }
}

int fk_engine_set_H(fk_engine* e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx, const double* val,
                    double es_lo, double es_hi) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    if (n_b > (int)fk::kColMask) return e->fail(FK_ERR_UNSUPPORTED, "set_H: too many block rows");
    fk::PreparedH ph;
    std::string why;
    int rc = fk::prepare_H(e->prec, e->cplx, n_b, b, nnzb, row_ptr, col_idx, val, es_lo, es_hi, 0, ph, why);
    if (rc != FK_OK) return e->fail(rc, "set_H: %s", why.c_str());
    const int nk = (int)ph.col.size();
    FK_TRY(e->d_row_ptr.ensure(sizeof(int) * (n_b + 1)), "alloc H row_ptr");
    FK_TRY(e->d_colc.ensure(sizeof(unsigned) * std::max(nk, 1)), "alloc H columns");
    FK_TRY(e->d_hval.ensure(std::max<size_t>(ph.hval.size(), 16)), "alloc H values");
    FK_TRY(cudaMemcpy(e->d_row_ptr.p, ph.row_ptr.data(), sizeof(int) * (n_b + 1), cudaMemcpyHostToDevice), "upload H row_ptr");
    FK_TRY(cudaMemcpy(e->d_colc.p, ph.colc.data(), sizeof(unsigned) * nk, cudaMemcpyHostToDevice), "upload H columns");
    FK_TRY(cudaMemcpy(e->d_hval.p, ph.hval.data(), ph.hval.size(), cudaMemcpyHostToDevice), "upload H values");
    if (e->prec == fk::kDS) {
        FK_TRY(e->d_row_hsum.ensure(std::max<size_t>(ph.row_hsum.size(), 16)), "alloc H row flags");
        FK_TRY(cudaMemcpy(e->d_row_hsum.p, ph.row_hsum.data(), ph.row_hsum.size(), cudaMemcpyHostToDevice),
               "upload H row flags");
    }
    e->n_b = n_b;
    e->b = b;
    e->nnzb = nk;
    e->es_lo = es_lo;
    e->es_hi = es_hi;
    e->h_row_ptr.swap(ph.row_ptr);
    e->h_col.swap(ph.col);
    e->gather_dist = gather_distance(e->h_row_ptr, e->h_col, n_b);
    e->mom_M = 0;
    e->mom_a0 = e->mom_a1 = -2;
    e->d_nb = -1;   // D pattern comparison against H must be redone
    e->d_nnzb = -1;
    return configure(e);
}

namespace {
// Device address through which kernels can read the host buffer [R, R + bytes), or null.
// Registered (pinned) buffers are read through their device mapping; other host memory is read
// by its own address where the system gives the GPU pageable-memory access.
const double* device_readable(const fk_engine* e, const double* R, size_t bytes) {
    cudaPointerAttributes a0, a1;
    if (cudaPointerGetAttributes(&a0, R) == cudaSuccess &&
        cudaPointerGetAttributes(&a1, (const char*)R + bytes - 1) == cudaSuccess && a0.type == cudaMemoryTypeHost &&
        a1.type == cudaMemoryTypeHost && a0.devicePointer && a1.devicePointer &&
        (const char*)a1.devicePointer - (const char*)a0.devicePointer == (ptrdiff_t)(bytes - 1))
        return reinterpret_cast<const double*>(a0.devicePointer);
    cudaGetLastError();
    return e->pageable_access ? R : nullptr;
}
}  // namespace

namespace {
// Column-major n x s host block -> row-major engine vector dst (n x ld, padding already zero),
// synchronously. A host buffer the GPU can read is read in place by the layout kernel;
// otherwise it goes through two staging halves: the copy of chunk q+1 (copy stream)
// overlaps the layout kernel of chunk q (engine stream).
int upload_colmajor(fk_engine* e, const double* src, int n, int s, void* dst) {
    const size_t col_bytes = sizeof(double) * (size_t)n * (e->cplx ? 2 : 1);
    const double* direct = e->opt_upload == 0 ? device_readable(e, src, col_bytes * s) : nullptr;
    if (direct) {
        ProfScope ps(e, fk::kHelper);
        FK_TRY(prec_load_colmajor(e, direct, n, s, 0, dst), "layout kernel");
        FK_TRY(cudaStreamSynchronize(e->stream), "upload");
        return FK_OK;
    }
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)s, (128u << 20) / col_bytes));
    const size_t half = col_bytes * chunk;
    FK_TRY(e->d_stage.ensure(2 * half), "alloc staging buffer");
    if (!e->copy_stream) {
        FK_TRY(cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking), "copy stream");
        for (int q = 0; q < 2; q++) {
            FK_TRY(cudaEventCreateWithFlags(&e->ev_copied[q], cudaEventDisableTiming), "copy event");
            FK_TRY(cudaEventCreateWithFlags(&e->ev_consumed[q], cudaEventDisableTiming), "copy event");
        }
    }
    // the staging halves may still be read by an earlier upload's kernels
    FK_TRY(cudaEventRecord(e->ev_consumed[0], e->stream), "upload order");
    FK_TRY(cudaEventRecord(e->ev_consumed[1], e->stream), "upload order");
    for (int c0 = 0, q = 0; c0 < s; c0 += chunk, q ^= 1) {
        const int nc = std::min(chunk, s - c0);
        char* buf = e->d_stage.as<char>() + q * half;
        FK_TRY(cudaStreamWaitEvent(e->copy_stream, e->ev_consumed[q], 0), "upload order");
        FK_TRY(cudaMemcpyAsync(buf, (const char*)src + col_bytes * c0, col_bytes * nc, cudaMemcpyHostToDevice,
                               e->copy_stream), "upload");
        FK_TRY(cudaEventRecord(e->ev_copied[q], e->copy_stream), "upload order");
        FK_TRY(cudaStreamWaitEvent(e->stream, e->ev_copied[q], 0), "upload order");
        ProfScope ps(e, fk::kHelper);
        FK_TRY(prec_load_colmajor(e, reinterpret_cast<const double*>(buf), n, nc, c0, dst), "layout kernel");
        FK_TRY(cudaEventRecord(e->ev_consumed[q], e->stream), "upload order");
    }
    FK_TRY(cudaStreamSynchronize(e->stream), "upload");
    return FK_OK;
}
}  // namespace

int fk_engine_set_R(fk_engine* e, int n, int s, const double* R) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    if (n <= 0) return e->fail(FK_ERR_ARG, "set_R: n must be positive");
    if (s <= 0) return e->fail(FK_ERR_ARG, "set_R: cannot handle an empty R (s = %d)", s);
    if (!R) return e->fail(FK_ERR_ARG, "set_R: null R");
    const int epp = e->epp();
    e->n = n;
    e->s = s;
    e->ld = ((long long)s + epp - 1) / epp * epp;
    e->P = (int)(e->ld / epp);
    int rc = ensure_vectors(e);
    if (rc != FK_OK) return rc;
    FK_TRY(cudaMemsetAsync(e->d_R.p, 0, e->vec_bytes(), e->stream), "clear R");
    for (auto& v : e->d_V) FK_TRY(cudaMemsetAsync(v.p, 0, e->vec_bytes(), e->stream), "clear work vector");
    rc = upload_colmajor(e, R, n, s, e->d_R.p);
    if (rc != FK_OK) return rc;
    e->mom_M = 0;
    e->mom_a0 = e->mom_a1 = -2;
    return configure(e);
}

int fk_engine_set_R_sparse(fk_engine* e, int n, int s, int k, const int* cols, const double* vals) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    if (n <= 0) return e->fail(FK_ERR_ARG, "set_R_sparse: n must be positive");
    if (s <= 0) return e->fail(FK_ERR_ARG, "set_R_sparse: cannot handle an empty R (s = %d)", s);
    if (k <= 0 || !cols || !vals) return e->fail(FK_ERR_ARG, "set_R_sparse: need k >= 1 entries per row and their arrays");
    const size_t nk = (size_t)n * k;
    for (size_t t = 0; t < nk; t++)
        if (cols[t] < 0 || cols[t] >= s)
            return e->fail(FK_ERR_ARG, "set_R_sparse: column %d of entry %zu outside [0, %d)", cols[t], t, s);
    const int epp = e->epp();
    e->n = n;
    e->s = s;
    e->ld = ((long long)s + epp - 1) / epp * epp;
    e->P = (int)(e->ld / epp);
    int rc = ensure_vectors(e);
    if (rc != FK_OK) return rc;
    FK_TRY(cudaMemsetAsync(e->d_R.p, 0, e->vec_bytes(), e->stream), "clear R");
    for (auto& v : e->d_V) FK_TRY(cudaMemsetAsync(v.p, 0, e->vec_bytes(), e->stream), "clear work vector");
    const size_t cw = e->cplx ? 2 : 1;
    const size_t col_bytes = (sizeof(int) * nk + 15) / 16 * 16;
    FK_TRY(e->d_stage.ensure(col_bytes + sizeof(double) * nk * cw), "alloc probe entries");
    int* d_cols = e->d_stage.as<int>();
    double* d_vals = reinterpret_cast<double*>(e->d_stage.as<char>() + col_bytes);
    FK_TRY(cudaMemcpyAsync(d_cols, cols, sizeof(int) * nk, cudaMemcpyHostToDevice, e->stream), "upload probe columns");
    FK_TRY(cudaMemcpyAsync(d_vals, vals, sizeof(double) * nk * cw, cudaMemcpyHostToDevice, e->stream), "upload probe values");
    {
        ProfScope ps(e, fk::kHelper);
        FK_TRY(prec_expand_sparse(e, d_cols, d_vals, n, k, e->d_R.p), "probe expansion kernel");
    }
    FK_TRY(cudaStreamSynchronize(e->stream), "set_R_sparse");
    e->mom_M = 0;
    e->mom_a0 = e->mom_a1 = -2;
    return configure(e);
}

int fk_engine_get_R(fk_engine* e, double* R) {
    if (!e || !R) return FK_ERR_ARG;
    if (e->s == 0) return e->fail(FK_ERR_STATE, "R has not been set");
    cudaSetDevice(e->device);
    const size_t bytes = sizeof(double) * (size_t)e->n * e->s * (e->cplx ? 2 : 1);
    DevBuf tmp;
    FK_TRY(tmp.ensure(bytes), "alloc readback buffer");
    cudaError_t ce = prec_store_colmajor(e, e->d_R.p, e->n, e->s, tmp.as<double>());
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(R, tmp.p, bytes, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    tmp.release();
    if (ce != cudaSuccess) return e->cuda_fail(ce, "read back R");
    return FK_OK;
}

int fk_engine_moments(fk_engine* e, int M, double* mu) {
    if (!e || !mu) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    int rc = moments_enqueue(e, M);
    if (rc != FK_OK) return rc;
    return moments_fetch(e, mu);
}
int fk_engine_moments_async(fk_engine* e, int M) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    return moments_enqueue(e, M);
}
int fk_engine_fetch_moments(fk_engine* e, double* mu) {
    if (!e || !mu) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    return moments_fetch(e, mu);
}

int fk_engine_stoch_matrix(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb, const int* rp, const int* ci,
                           double* D) {
    if (!e || (!D && d_nnzb > 0)) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    int rc = stoch_enqueue(e, M, c, d_n_b, d_nnzb, rp, ci);
    if (rc != FK_OK) return rc;
    return fetch_D(e, D);
}
int fk_engine_stoch_matrix_async(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb, const int* rp,
                                 const int* ci) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    return stoch_enqueue(e, M, c, d_n_b, d_nnzb, rp, ci);
}
int fk_engine_autodiff_matrix(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb, const int* rp,
                              const int* ci, double* D) {
    if (!e || (!D && d_nnzb > 0)) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    int rc = autodiff_enqueue(e, M, c, d_n_b, d_nnzb, rp, ci);
    if (rc != FK_OK) return rc;
    return fetch_D(e, D);
}
int fk_engine_autodiff_matrix_async(fk_engine* e, int M, const double* c, int d_n_b, int d_nnzb, const int* rp,
                                    const int* ci) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    return autodiff_enqueue(e, M, c, d_n_b, d_nnzb, rp, ci);
}
int fk_engine_fetch_D(fk_engine* e, double* D) {
    if (!e || !D) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    return fetch_D(e, D);
}

namespace {
// moments2_v2 (reference src/engine_cpu.cpp:162-209; the reference's GPU engine exits there,
// src/engine_cusparse.cpp:904-908): with X_i = T_i(Hs) j2 R2 and Y_i = T_i(Hs) j1 R,
//   A_i = R^dag X_i,  B_i = R2^dag Y_i  (s x s),  mu[m1][m2] = tr(A_m1 B_m2).
// Per order i the vector is exported as a double panel and projected by one GEMM:
//   At_i = X_i^T conj(R)  (= A_i transposed),  E_i = R2^T conj(Y_i)  (= conj(B_i)),
// then mu (row-major) = E^H At over the stacked ld^2-long columns, one more GEMM.
int moments2_v2(fk_engine* e, int M, const int* nnzb, const int* const* rp, const int* const* ci,
                const double* const* val, const double* R2_host, double* mu_out) {
    if (M < 2 || M % 2 != 0) return e->fail(FK_ERR_ARG, "moments2_v2: M must be even and >= 2 (got %d)", M);
    int rc = require_ready(e);
    if (rc != FK_OK) return rc;
    for (int q = 0; q < 2; q++) {
        rc = m2_upload_op(e, q, nnzb[q], rp[q], ci[q], val[q]);
        if (rc != FK_OK) return rc;
    }
    const long long ld = e->ld, L = (long long)e->n * ld, ld2 = ld * ld;
    if (L >= (1LL << 31) || (long long)M * ld2 >= (1LL << 31))
        return e->fail(FK_ERR_UNSUPPORTED, "moments2_v2: too many rows or probe columns for the GEMM sizes");
    const size_t elt = e->cplx ? 16 : 8;
    void* R2 = e->d_R.p;
    if (R2_host) {
        FK_TRY(e->d_R2.ensure(e->vec_bytes()), "alloc R2");
        FK_TRY(cudaMemsetAsync(e->d_R2.p, 0, e->vec_bytes(), e->stream), "clear R2");
        rc = upload_colmajor(e, R2_host, e->n, e->s, e->d_R2.p);
        if (rc != FK_OK) return rc;
        R2 = e->d_R2.p;
    }
    FK_TRY(e->d_panel[0].ensure(3 * (size_t)L * elt), "alloc panels");
    FK_TRY(e->d_panel[1].ensure(2 * (size_t)M * ld2 * elt), "alloc projections");
    FK_TRY(e->d_mu2.ensure((size_t)M * M * elt), "alloc moments");
    double* Xp = e->d_panel[0].as<double>();
    double* Rp = Xp + (size_t)L * (elt / 8);
    double* R2p = Rp + (size_t)L * (elt / 8);
    char* At = e->d_panel[1].as<char>();
    char* Ep = At + (size_t)M * ld2 * elt;
    FK_TRY(prec_export(e, e->d_R.p, 0, (int)ld, Rp), "export R");
    FK_TRY(prec_export(e, R2, 0, (int)ld, R2p), "export R2");
    const M2Mat hs{e->d_row_ptr.as<int>(), e->d_colc.as<unsigned>(), e->d_hval.p};
    const M2Mat j1{e->d_j[0].row_ptr.as<int>(), e->d_j[0].colc.as<unsigned>(), e->d_j[0].hval.p};
    const M2Mat j2{e->d_j[1].row_ptr.as<int>(), e->d_j[1].colc.as<unsigned>(), e->d_j[1].hval.p};
    const int n_ld = (int)ld;   // projections: ld x ld GEMMs over the n rows
    for (int side = 0; side < 2; side++) {
        // side 0: X_i = T_i j2 R2 in V0/V1 -> At_i;  side 1: Y_i = T_i j1 R in V2/V3 -> E_i
        void* va = e->d_V[2 * side].p;
        void* vb = e->d_V[2 * side + 1].p;
        void* prev = nullptr;
        void* cur = nullptr;
        for (int m = 0; m < M; m++) {
            void* y = m == 0 ? va : (m == 1 ? vb : prev);
            if (m == 0) rc = m2_step(e, side == 0 ? j2 : j1, side == 0 ? R2 : e->d_R.p, nullptr, y, false, 0, e->P);
            else rc = m2_step(e, hs, cur, m == 1 ? nullptr : prev, y, m > 1, 0, e->P);
            if (rc != FK_OK) return rc;
            prev = cur;
            cur = y;
            FK_TRY(prec_export(e, cur, 0, n_ld, Xp), "export panel");
            char* dst = (side == 0 ? At : Ep) + (size_t)m * ld2 * elt;
            // panels are column-major ld x n (leading dimension ld):
            // dst[p + q ld] = sum_i a[p + i ld] conj(b[q + i ld])
            rc = gram(e, n_ld, n_ld, e->n, side == 0 ? Xp : R2p, 1, ld, false, side == 0 ? Rp : Xp, ld, 1, true,
                      reinterpret_cast<double*>(dst), ld, false, "moments2_v2 projection");
            if (rc != FK_OK) return rc;
        }
    }
    // mu^T (column-major M x M) = mu row-major: (E^H At)(m2, m1) = sum_q conj(E[q, m2]) At[q, m1]
    rc = gram(e, M, M, ld2, reinterpret_cast<const double*>(Ep), ld2, 1, true, reinterpret_cast<const double*>(At), 1, ld2,
              false, e->d_mu2.as<double>(), M, false, "moments2_v2 trace product");
    if (rc != FK_OK) return rc;
    std::vector<double> h((size_t)M * M * (e->cplx ? 2 : 1));
    FK_TRY(cudaMemcpyAsync(h.data(), e->d_mu2.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, e->stream),
           "copy moments");
    FK_TRY(cudaStreamSynchronize(e->stream), "moments2_v2");
    for (size_t q = 0; q < (size_t)M * M; q++) {   // column-major (m2 + m1 M) of mu^T = row-major mu
        mu_out[2 * q] = e->cplx ? h[2 * q] : h[q];
        mu_out[2 * q + 1] = e->cplx ? h[2 * q + 1] : 0.0;
    }
    e->mom_M = 0;
    e->mom_a0 = e->mom_a1 = -2;
    if (e->profiling) prof_flush(e);
    return FK_OK;
}
}  // namespace

int fk_engine_moments2_v2(fk_engine* e, int M, int j1_nnzb, const int* j1_row_ptr, const int* j1_col_idx,
                          const double* j1_val, int j2_nnzb, const int* j2_row_ptr, const int* j2_col_idx,
                          const double* j2_val, const double* R2, double* mu) {
    if (!e || !mu || !j1_row_ptr || !j2_row_ptr) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    const int nnzb[2] = {j1_nnzb, j2_nnzb};
    const int* rp[2] = {j1_row_ptr, j2_row_ptr};
    const int* ci[2] = {j1_col_idx, j2_col_idx};
    const double* val[2] = {j1_val, j2_val};
    return moments2_v2(e, M, nnzb, rp, ci, val, R2, mu);
}

int fk_engine_moments2_v1(fk_engine* e, int M, int j1_nnzb, const int* j1_row_ptr, const int* j1_col_idx,
                          const double* j1_val, int j2_nnzb, const int* j2_row_ptr, const int* j2_col_idx,
                          const double* j2_val, int a_chunk_ncols, int R_chunk_ncols, double* mu) {
    if (!e || !mu || !j1_row_ptr || !j2_row_ptr) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    const int nnzb[2] = {j1_nnzb, j2_nnzb};
    const int* rp[2] = {j1_row_ptr, j2_row_ptr};
    const int* ci[2] = {j1_col_idx, j2_col_idx};
    const double* val[2] = {j1_val, j2_val};
    return moments2_v1(e, M, nnzb, rp, ci, val, a_chunk_ncols, R_chunk_ncols, mu);
}

int fk_engine_kpm_filling(fk_engine* e, int Mq, double kT, double filling, double delta_filling, double* result,
                          double* gamma) {
    if (!e || !result) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    int rc = post_enqueue(e, Mq, kT, filling, delta_filling, false);
    if (rc != FK_OK) return rc;
    return post_fetch(e, result, gamma);
}

int fk_engine_solve_filling(fk_engine* e, int M, int Mq, double kT, double filling, double delta_filling, int d_n_b,
                            int d_nnzb, const int* d_row_ptr, const int* d_col_idx, double* D, double* result,
                            double* gamma) {
    if (!e || !D || !result || !d_row_ptr || (d_nnzb > 0 && !d_col_idx)) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    if (Mq < M) return e->fail(FK_ERR_ARG, "solve_filling: Mq (%d) must be >= M (%d)", Mq, M);
    int rc = moments_enqueue(e, M);
    if (rc != FK_OK) return rc;
    rc = post_enqueue(e, Mq, kT, filling, delta_filling, true);
    if (rc != FK_OK) return rc;
    const double* c_dev = post_layout(e, M, Mq).c;
    rc = autodiff_enqueue(e, M, nullptr, d_n_b, d_nnzb, d_row_ptr, d_col_idx, c_dev);
    if (rc != FK_OK) return rc;
    rc = fetch_D(e, D);
    if (rc != FK_OK) return rc;
    return post_fetch(e, result, gamma);
}

int fk_engine_energy_scale(fk_engine* e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
                           const double* val, double extend, int iters, const double* v0, double* lo, double* hi) {
    if (!e || !lo || !hi) return FK_ERR_ARG;
    if (iters < 1) return e->fail(FK_ERR_ARG, "energy_scale: iters must be >= 1");
    cudaSetDevice(e->device);
    // A scratch FP64 engine holds H unscaled (es = [-1, 1] makes Hs = H) and one probe column.
    fk_engine* t = nullptr;
    int rc = fk_engine_create(e->device, e->cplx, FK_PREC_FP64, &t);
    if (rc != FK_OK) return e->fail(rc, "energy_scale: scratch engine");
    struct Guard { fk_engine* t; ~Guard() { fk_engine_destroy(t); } } guard{t};
    rc = fk_engine_set_H(t, n_b, b, nnzb, row_ptr, col_idx, val, -1.0, 1.0);
    if (rc != FK_OK) return e->fail(rc, "energy_scale: %s", t->err.c_str());
    const int n = n_b * b, cw = e->cplx ? 2 : 1;
    std::vector<double> v(static_cast<size_t>(n) * cw);
    if (v0) std::copy(v0, v0 + v.size(), v.begin());
    else {
        // seeded Gaussian start vector (the reference draws arma::randn)
        unsigned long long st = 0x9e3779b97f4a7c15ull;
        auto u01 = [&]() { st = st * 6364136223846793005ull + 1442695040888963407ull; return ((st >> 11) + 0.5) / 9007199254740992.0; };
        for (auto& x : v) x = std::sqrt(-2.0 * std::log(u01())) * std::cos(6.283185307179586 * u01());
    }
    double nrm = 0;
    for (double x : v) nrm += x * x;
    nrm = std::sqrt(nrm);
    for (auto& x : v) x /= nrm;
    rc = fk_engine_set_R(t, n, 1, v.data());
    if (rc != FK_OK) return e->fail(rc, "energy_scale: %s", t->err.c_str());
    rc = require_ready(t);
    if (rc != FK_OK) return e->fail(rc, "energy_scale: %s", t->err.c_str());
    // vectors: v1 = R buffer copy in V0 (we keep R intact), v0 in V1, w in V2; stride ld (padded) doubles
    const size_t vb = t->vec_bytes();
    FK_TRY(cudaMemcpyAsync(t->d_V[0].p, t->d_R.p, vb, cudaMemcpyDeviceToDevice, t->stream), "lanczos init");
    FK_TRY(cudaMemsetAsync(t->d_V[1].p, 0, vb, t->stream), "lanczos init");
    const long long n_dbl = (long long)vb / sizeof(double);
    // The whole recursion stays on the device: the scalars alpha_j, beta_j, 1/beta_j are
    // reduced into device arrays that the next launches read, so the host waits once, at the
    // end, and then solves the iters x iters tridiagonal problem.
    DevBuf scal, spart, upart;
    const int ugrid = 152 * 4;
    const int ctas = t->cfg[fk::kStep].ctas;   // one column slice
    FK_TRY(scal.ensure(sizeof(double) * 3 * (size_t)(iters + 1)), "lanczos scalars");
    FK_TRY(spart.ensure(sizeof(double) * 2 * (size_t)ctas), "lanczos partials");
    FK_TRY(upart.ensure(sizeof(double) * ugrid), "lanczos partials");
    double* d_alpha = scal.as<double>();
    double* d_beta = d_alpha + (iters + 1);
    double* d_inv = d_beta + (iters + 1);
    FK_TRY(cudaMemsetAsync(scal.p, 0, scal.bytes, t->stream), "lanczos init");
    int v1 = 0, vz = 1, w = 2;
    for (int j = 1; j <= iters; j++) {
        // w = H v1 with the step kernel; alpha_j = <w, v1> from its dots
        rc = run_step(t, t->V(v1), nullptr, t->V(w), false, true, 0, nullptr, nullptr, spart.as<double>());
        if (rc != FK_OK) return e->fail(rc, "energy_scale: %s", t->err.c_str());
        k_lanczos_alpha<<<1, 32, 0, t->stream>>>(spart.as<double>(), ctas, d_alpha + (j - 1));
        FK_TRY(cudaGetLastError(), "lanczos alpha");
        if (j == iters) break;
        k_lanczos_update<<<ugrid, 256, 0, t->stream>>>(t->d_V[w].as<double>(), t->d_V[v1].as<double>(),
                                                       t->d_V[vz].as<double>(), n_dbl, d_alpha + (j - 1), d_beta + (j - 1),
                                                       upart.as<double>());
        FK_TRY(cudaGetLastError(), "lanczos update");
        k_lanczos_beta<<<1, 32, 0, t->stream>>>(upart.as<double>(), ugrid, d_beta + j, d_inv + j);
        FK_TRY(cudaGetLastError(), "lanczos beta");
        // v0 <- v1, v1 <- w / beta_j (w / 0 -> 0 once the Krylov space is exhausted)
        FK_TRY(fk::launch_scale_f64(e->cplx, t->V(w), t->V(vz), (long long)t->n * t->ld, 0.0, d_inv + j, t->stream),
               "lanczos scale");
        std::swap(v1, vz);   // new v1 = scaled w (in old vz), new v0 = old v1
    }
    std::vector<double> alpha(iters + 1), beta(iters + 1);
    FK_TRY(cudaMemcpyAsync(alpha.data(), d_alpha, sizeof(double) * (iters + 1), cudaMemcpyDeviceToHost, t->stream),
           "lanczos");
    FK_TRY(cudaMemcpyAsync(beta.data(), d_beta, sizeof(double) * (iters + 1), cudaMemcpyDeviceToHost, t->stream), "lanczos");
    FK_TRY(cudaStreamSynchronize(t->stream), "lanczos");
    for (int j = 1; j < iters; j++)
        if (!(beta[j] > 0)) { iters = j; break; }   // invariant subspace found at step j
    double emin, emax;
    tridiag_extremes(iters, alpha.data(), beta.data(), &emin, &emax);
    const double slack = extend * (emax - emin);
    *lo = emin - slack;
    *hi = emax + slack;
    scal.release();
    spart.release();
    upart.release();
    return FK_OK;
}

int fk_engine_expansion_coefficients(fk_engine* e, int M, int Mq, int f_kind, double kT, double mu, double es_lo,
                                     double es_hi, double* out) {
    if (!e || !out) return FK_ERR_ARG;
    if (M < 1 || Mq < M || (f_kind != 0 && f_kind != 1) || !(es_hi > es_lo))
        return e->fail(FK_ERR_ARG, "expansion_coefficients: need 1 <= M <= Mq, f_kind 0/1, hi > lo");
    cudaSetDevice(e->device);
    DevBuf d;
    FK_TRY(d.ensure(sizeof(double) * M), "alloc coefficients");
    fk::k_expansion_coefficients<<<M, fk::kPostThreads, 0, e->stream>>>(M, Mq, f_kind, kT, mu, nullptr, (es_hi + es_lo) / 2.0,
                                                       (es_hi - es_lo) / 2.0, d.as<double>());
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(out, d.p, sizeof(double) * M, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    d.release();
    if (ce != cudaSuccess) return e->cuda_fail(ce, "expansion coefficients");
    return FK_OK;
}

int fk_engine_set_profiling(fk_engine* e, int on) {
    if (!e) return FK_ERR_ARG;
    e->profiling = on != 0;
    return FK_OK;
}
int fk_engine_profile_read(fk_engine* e, int kind, long long* launches, double* total_ms) {
    if (!e || kind < 0 || kind >= fk::kNumKinds) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    prof_flush(e);
    if (launches) *launches = e->prof_launches[kind];
    if (total_ms) *total_ms = e->prof_ms[kind];
    return FK_OK;
}
int fk_engine_profile_reset(fk_engine* e) {
    if (!e) return FK_ERR_ARG;
    prof_flush(e);
    for (int k = 0; k < fk::kNumKinds; k++) { e->prof_launches[k] = 0; e->prof_ms[k] = 0; }
    return FK_OK;
}
int fk_host_register(void* ptr, size_t bytes) {
    if (!ptr || bytes == 0) return FK_ERR_ARG;
    cudaError_t ce = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (ce != cudaSuccess) { cudaGetLastError(); return ce == cudaErrorHostMemoryAlreadyRegistered ? FK_OK : FK_ERR_CUDA; }
    return FK_OK;
}
int fk_host_unregister(void* ptr) {
    if (!ptr) return FK_ERR_ARG;
    cudaError_t ce = cudaHostUnregister(ptr);
    if (ce != cudaSuccess) { cudaGetLastError(); return FK_ERR_CUDA; }
    return FK_OK;
}
int fk_engine_timer_start(fk_engine* e) {
    if (!e) return FK_ERR_ARG;
    cudaSetDevice(e->device);
    if (!e->t_start) FK_TRY(cudaEventCreate(&e->t_start), "timer event");
    if (!e->t_stop) FK_TRY(cudaEventCreate(&e->t_stop), "timer event");
    FK_TRY(cudaEventRecord(e->t_start, e->stream), "timer start");
    return FK_OK;
}
int fk_engine_timer_stop(fk_engine* e, double* ms) {
    if (!e || !ms) return FK_ERR_ARG;
    if (!e->t_start) return e->fail(FK_ERR_STATE, "timer not started");
    cudaSetDevice(e->device);
    FK_TRY(cudaEventRecord(e->t_stop, e->stream), "timer stop");
    FK_TRY(cudaEventSynchronize(e->t_stop), "timer wait");
    float f = 0.f;
    FK_TRY(cudaEventElapsedTime(&f, e->t_start, e->t_stop), "timer elapsed");
    *ms = f;
    return FK_OK;
}
int fk_engine_memory(const fk_engine* e, size_t* bytes) {
    if (!e || !bytes) return FK_ERR_ARG;
    size_t t = e->d_row_ptr.bytes + e->d_colc.bytes + e->d_hval.bytes + e->d_R.bytes + e->dd_row_ptr.bytes +
               e->dd_colc.bytes + e->dd_rows.bytes + e->dd_pair.bytes + e->dd_acc.bytes + e->d_partials.bytes +
               e->d_raw.bytes + e->d_coef.bytes + e->d_stage.bytes + e->d_row_hsum.bytes;
    for (auto& v : e->d_V) t += v.bytes;
    *bytes = t;
    return FK_OK;
}

}  // extern "C"
