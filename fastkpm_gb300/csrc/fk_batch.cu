// fk_batch.cu -- batched engine: many Hamiltonians of uneven size share one launch
// per Chebyshev step (the k_cheb_step kernel with a multi-system table), the M/2
// launches of moments(M) are captured once in a CUDA graph and replayed, and the
// (lanes per row, packets per lane, CTAs per SM, H staging) mapping is chosen by
// timing candidates on the batch itself.
//
// Layout: systems' block rows are concatenated; H columns are offset to global
// block rows; R and the two rotating recursion vectors are (sum of rows) x ld.
// CTA counts are per system and depend only on that system's size and the
// mapping, so a system's moments are bit-identical alone or inside any batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/fastkpm_gb300.h"
#include "fk_dispatch.h"
#include "fk_prep.h"

using fk::SysDesc;

namespace {

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && p) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; bytes = 0; }
        if (!need) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, need);
        if (e == cudaSuccess) bytes = need; else { p = nullptr; cudaGetLastError(); }
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; bytes = 0; }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct PendingSystem {
    fk::PreparedH h;
    int n_b, b, s;
    double mag;              // energy-scale half width (autodiff divides D by it)
    std::vector<int> o2a;    // original block -> block of the prepared (diagonal-augmented) pattern
    std::vector<double> R;   // column-major n x s (interleaved complex)
};

struct Mapping {
    int Gp = 0, NP = 0, cap_per_sm = 0;   // 0 = automatic
    int stage = -1;                       // -1 = automatic (off for FP32, as in the single engine)
};

// Process-wide memory of autotuned mappings, keyed by batch shape.
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, long long, int>, Mapping> g_tuned;

__global__ void k_batch_reduce(const double* partials, int grid, int slices, int nsteps, const SysDesc* sys, int n_sys,
                               double* raw) {
    // one warp per (step, system): fixed-order sum over the system's CTAs in every slice
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nsteps * n_sys) return;
    const int step = w / n_sys, s = w - step * n_sys;
    double a = 0.0, b = 0.0;
    for (int sl = 0; sl < slices; sl++) {
        const double* p = partials + ((size_t)step * slices + sl) * grid * 2;
        for (int c = sys[s].cta_base + lane; c < sys[s].cta_base + sys[s].ctas; c += 32) {
            a += p[2 * c];
            b += p[2 * c + 1];
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
    }
    if (lane == 0) { raw[2 * w] = a; raw[2 * w + 1] = b; }
}

int next_pow2(int v) { int p = 1; while (p < v) p <<= 1; return p; }

}  // namespace

struct fk_batch {
    int device = 0, cplx = 0, prec = 0, num_sms = 1;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<PendingSystem> pending;
    // committed state
    int b = 0, s = 0, n_sys = 0, P = 0;   // s, P: the widest system's probe columns and packets per row
    long long ld = 0, total_rows = 0;
    std::vector<int> row_base, n_b;
    std::vector<int> Pk;                  // per system: its packets per row (probe counts may differ)
    std::vector<int> Gpk;                 // per system: its lanes per block row
    int P_launch = 0;                     // the launches' P: P when every system's rows split into whole
                                          // chunks of the mapping (the unmasked kernels), else one that does not
    std::vector<int> h_row_ptr;          // global
    std::vector<int> h_col;              // global block columns of the prepared pattern
    Buf d_row_ptr, d_colc, d_hval, d_R, d_V[4], d_stage;
    // autodiff_matrix over the batch: per-system scale, original-pattern maps, D accumulator
    std::vector<double> mag;
    std::vector<std::vector<int>> o2a;   // per system: original block -> global prepared block
    int mom_M = 0;                       // moments(M) state left in V0/V1 (0: none)
    Buf d_D, d_coef, d_rows, d_cols, d_pair, d_rowscale, d_rowsys, d_rowfac, d_gather, d_Dout;
    bool d_tables = false;
    bool d_gather_identity = true;   // no diagonal blocks were added: D leaves in the prepared order
    long long n_out_blocks = 0;
    // launch tables
    Mapping opt, cur;
    int Gp = 1, NP = 1, slices = 1, W = 1, stage_cap = 0, grid = 0;
    size_t smem = 0;
    std::vector<SysDesc> sysd;
    Buf d_sys, d_cta_sys, d_partials, d_raw;
    std::vector<double> h_raw;
    bool configured = false;
    int opt_graphs = 0;
    // FK_OPT_ACC64 (FP32 batches): 0 (default) float-float per-thread sums, 1 FP64. Measured on the
    // 64 square lattices (b=1, S=32, M=500): 37.8 ms per batch with float-float sums, 45.8 ms with FP64
    // ones (the narrow-row step's per-row FP64 conversions and adds keep this GPU's FP64 pipe 44% busy
    // and double its short-scoreboard stalls); the moments' error against FP64 is 3.0e-7 either way.
    int acc64 = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>>* prof = nullptr;   // events around each step launch
    std::map<int, cudaGraphExec_t> graphs;
    cudaEvent_t t0 = nullptr, t1 = nullptr;

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
        return fail(ce == cudaErrorMemoryAllocation ? FK_ERR_OOM : FK_ERR_CUDA, "%s: %s", what, cudaGetErrorString(ce));
    }
    size_t esize() const { return (size_t)fk::elem_bytes(prec, cplx); }
    int epp() const { return fk::elems_per_packet(prec, cplx); }
    void drop_graphs() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
    }
};

#define BT_TRY(expr, what)                                  \
    do {                                                    \
        cudaError_t _ce = (expr);                           \
        if (_ce != cudaSuccess) return bt->cuda_fail(_ce, what); \
    } while (0)

namespace {

cudaError_t batch_launch_step(fk_batch* bt, const fk::StepArgs& a, const fk::Launch& l) {
    switch (bt->prec) {
        case fk::kF64: return fk::launch_step_f64(bt->cplx, bt->b, bt->NP, a, l);
        case fk::kF32: return bt->acc64 ? fk::launch_step_f32a(bt->cplx, bt->b, bt->NP, a, l)
                                        : fk::launch_step_f32(bt->cplx, bt->b, bt->NP, a, l);
        default: return fk::launch_step_ds(bt->cplx, bt->b, bt->NP, a, l);
    }
}
cudaError_t batch_occupancy(fk_batch* bt, int NP, size_t smem, int* n) {
    switch (bt->prec) {
        case fk::kF64: return fk::occupancy_f64(fk::kStep, bt->cplx, bt->b, NP, smem, n);
        case fk::kF32: return bt->acc64 ? fk::occupancy_f32a(fk::kStep, bt->cplx, bt->b, NP, smem, n)
                                        : fk::occupancy_f32(fk::kStep, bt->cplx, bt->b, NP, smem, n);
        default: return fk::occupancy_ds(fk::kStep, bt->cplx, bt->b, NP, smem, n);
    }
}
cudaError_t batch_load(fk_batch* bt, const double* src, long long n, int ncols, int c0, void* dst) {
    switch (bt->prec) {
        case fk::kF64: return fk::launch_load_colmajor_f64(bt->cplx, src, n, ncols, c0, bt->ld, dst, bt->stream);
        case fk::kF32: return fk::launch_load_colmajor_f32(bt->cplx, src, n, ncols, c0, bt->ld, dst, bt->stream);
        default: return fk::launch_load_colmajor_ds(bt->cplx, src, n, ncols, c0, bt->ld, dst, bt->stream);
    }
}

// Build the launch tables for mapping m (0 fields = automatic).
int batch_configure(fk_batch* bt, const Mapping& m) {
    bt->configured = false;
    bt->mom_M = 0;   // a new mapping (or the autotuner's trial runs) leaves no usable alpha state
    bt->drop_graphs();
    const int P = bt->P;
    // packets per lane: as requested, else by the widest system's packets (narrow rows: two per lane,
    // measured faster than one on b=1, S=32 lattices; wider: enough for 32 lanes, 1, 2 or 4); lanes
    // per row: as requested, else the fewest that cover the row in one chunk (at most 32)
    int NP = m.NP;
    if (NP <= 0) {
        if (P <= 32) NP = P >= 2 ? 2 : 1;
        else NP = (P + 31) / 32 <= 1 ? 1 : (P + 31) / 32 <= 2 ? 2 : 4;
    }
    const int Gp = m.Gp > 0 ? m.Gp : std::min(32, next_pow2((P + NP - 1) / NP));
    if (!(Gp == 1 || Gp == 2 || Gp == 4 || Gp == 8 || Gp == 16 || Gp == 32)) return bt->fail(FK_ERR_ARG, "bad lanes per row %d", Gp);
    if (!(NP == 1 || NP == 2 || NP == 4)) return bt->fail(FK_ERR_ARG, "bad packets per lane %d", NP);
    // the kernel walks the row's column chunks of Gp * NP packets itself: one launch per step
    bt->Gp = Gp;
    bt->NP = NP;
    bt->W = P;
    bt->slices = 1;
    // lanes per row of each system: a forced mapping's for all; else the fewest (a power of two, at
    // most 32) that cover the system's own packets in one chunk of NP each, so that a system's tiles,
    // CTAs and sums depend on its own probe count and not on the widest system in the batch
    bt->Gpk.resize(bt->n_sys);
    for (int k = 0; k < bt->n_sys; k++)
        bt->Gpk[k] = m.Gp > 0 ? Gp : std::min(32, next_pow2((bt->Pk[k] + NP - 1) / NP));
    // shared-memory stage: largest tile over all systems
    int nk_max = 0;
    for (int k = 0; k < bt->n_sys; k++) {
        const int* rp = bt->h_row_ptr.data() + bt->row_base[k];
        std::vector<int> local(rp, rp + bt->n_b[k] + 1);
        for (auto& v : local) v -= rp[0];
        nk_max = std::max(nk_max, fk::max_tile_blocks(local.data(), bt->n_b[k], bt->Gpk[k]));
    }
    const size_t per_blk = (size_t)bt->b * bt->b * bt->esize() + sizeof(unsigned);
    const int stage = m.stage >= 0 ? m.stage : (bt->prec == fk::kF32 ? 0 : 1);
    bt->stage_cap = (stage && nk_max * per_blk <= 48 * 1024) ? nk_max : 0;
    bt->smem = bt->stage_cap ? ((size_t)bt->stage_cap * per_blk + 15) / 16 * 16 : 0;
    int occ = 0;
    BT_TRY(batch_occupancy(bt, NP, bt->smem, &occ), "occupancy query");
    if (occ < 1) return bt->fail(FK_ERR_UNSUPPORTED, "step kernel does not fit on an SM");
    if (m.cap_per_sm > 0) occ = std::min(occ, m.cap_per_sm);
    const long long cap = (long long)occ * bt->num_sms;
    bt->sysd.resize(bt->n_sys);
    bool all_whole = true;
    for (int k = 0; k < bt->n_sys; k++) all_whole = all_whole && bt->Pk[k] % (bt->Gpk[k] * NP) == 0;
    // (the kernels read each system's own P and Gp; the launch's P only selects the unmasked instances)
    bt->P_launch = all_whole || Gp * NP == 1 ? Gp * NP : Gp * NP + 1;
    std::vector<int> cta_sys, order(bt->n_sys);
    std::vector<long long> tiles(bt->n_sys);
    std::vector<int> ctas(bt->n_sys);
    for (int k = 0; k < bt->n_sys; k++) {
        tiles[k] = ((long long)bt->n_b[k] * bt->Gpk[k] + fk::kThreads - 1) / fk::kThreads;
        ctas[k] = (int)std::max<long long>(1, std::min(tiles[k], cap));
        order[k] = k;
    }
    // CTAs are dispatched roughly in index order: give the systems whose CTAs walk the most
    // tiles the lowest indices, so the longest CTAs start first and the launch's tail is short.
    // Only the position of a system's CTA range moves; its CTA count (and so its sums) does not.
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (tiles[a] + ctas[a] - 1) / ctas[a] > (tiles[b] + ctas[b] - 1) / ctas[b];
    });
    int base = 0;
    for (int k : order) {
        bt->sysd[k] = SysDesc{bt->row_base[k], bt->n_b[k], base, ctas[k], bt->Pk[k], bt->Gpk[k]};
        cta_sys.insert(cta_sys.end(), ctas[k], k);
        base += ctas[k];
    }
    bt->grid = base;
    BT_TRY(bt->d_sys.ensure(sizeof(SysDesc) * bt->n_sys), "alloc system table");
    BT_TRY(bt->d_cta_sys.ensure(sizeof(int) * base), "alloc CTA table");
    BT_TRY(cudaMemcpy(bt->d_sys.p, bt->sysd.data(), sizeof(SysDesc) * bt->n_sys, cudaMemcpyHostToDevice), "upload system table");
    BT_TRY(cudaMemcpy(bt->d_cta_sys.p, cta_sys.data(), sizeof(int) * base, cudaMemcpyHostToDevice), "upload CTA table");
    bt->cur = m;   // as requested (automatic fields stay automatic when the tables are rebuilt)
    bt->configured = true;
    return FK_OK;
}

int batch_ensure_partials(fk_batch* bt, int nsteps) {
    BT_TRY(bt->d_partials.ensure(sizeof(double) * 2 * (size_t)nsteps * bt->slices * bt->grid), "alloc partials");
    BT_TRY(bt->d_raw.ensure(sizeof(double) * 2 * (size_t)nsteps * bt->n_sys), "alloc moment sums");
    return FK_OK;
}

// Enqueue the M/2 step launches and the per-system reduction on bt->stream.
int batch_enqueue_moments(fk_batch* bt, int M) {
    const int nsteps = M / 2;
    const size_t es = bt->esize();
    const size_t per_step = (size_t)bt->slices * bt->grid * 2;
    double* part = bt->d_partials.as<double>();
    void* R = bt->d_R.p;
    void* V[2] = {bt->d_V[0].p, bt->d_V[1].p};
    for (int m = 0; m < nsteps; m++) {
        // m = 0: x = R -> V0;  m = 1: x = V0, z = R -> V1;  m >= 2: x = V[(m-1)&1], z = y = V[m&1]
        const void* x = m == 0 ? R : V[(m - 1) & 1];
        const void* z = m == 0 ? nullptr : (m == 1 ? R : V[m & 1]);
        void* y = m == 0 ? V[0] : V[m & 1];
        for (int sl = 0; sl < bt->slices; sl++) {
            const long long off = (long long)sl * bt->W * bt->epp();
            fk::StepArgs a;
            a.sys = bt->d_sys.as<SysDesc>();
            a.cta_sys = bt->d_cta_sys.as<int>();
            a.Gp = bt->Gp;
            a.P = bt->P_launch;   // (one column slice: bt->W == bt->P)
            a.ld = bt->ld;
            a.row_ptr = bt->d_row_ptr.as<int>();
            a.colc = bt->d_colc.as<unsigned>();
            a.hval = bt->d_hval.p;
            a.x = (const char*)x + off * es;
            a.z = z ? (const char*)z + off * es : nullptr;
            a.y = (char*)y + off * es;
            a.xi = nullptr;
            a.coef = nullptr;
            a.cstride = 0;
            a.two = m > 0;
            a.has_z = z != nullptr;
            a.want_dots = 1;
            a.xi_mode = 0;
            a.partials = part + per_step * m + (size_t)sl * bt->grid * 2;
            a.stage_cap = bt->stage_cap;
            a.pipe = 0;
            cudaEvent_t ev0 = nullptr, ev1 = nullptr;
            if (bt->prof) {
                BT_TRY(cudaEventCreate(&ev0), "profile event");
                BT_TRY(cudaEventCreate(&ev1), "profile event");
                BT_TRY(cudaEventRecord(ev0, bt->stream), "profile event");
            }
            BT_TRY(batch_launch_step(bt, a, fk::Launch{bt->grid, bt->smem, bt->stream}), "batched step launch");
            if (bt->prof) {
                BT_TRY(cudaEventRecord(ev1, bt->stream), "profile event");
                bt->prof->push_back({ev0, ev1});
            }
        }
    }
    const int warps = nsteps * bt->n_sys;
    k_batch_reduce<<<(warps * 32 + 255) / 256, 256, 0, bt->stream>>>(part, bt->grid, bt->slices, nsteps, bt->d_sys.as<SysDesc>(),
                                                                    bt->n_sys, bt->d_raw.as<double>());
    BT_TRY(cudaGetLastError(), "batched reduction launch");
    return FK_OK;
}

int batch_run_moments(fk_batch* bt, int M) {
    int rc = batch_ensure_partials(bt, M / 2);
    if (rc != FK_OK) return rc;
    if (!bt->opt_graphs) return batch_enqueue_moments(bt, M);
    auto it = bt->graphs.find(M);
    if (it == bt->graphs.end()) {
        cudaGraph_t g = nullptr;
        BT_TRY(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        rc = batch_enqueue_moments(bt, M);
        cudaError_t ce = cudaStreamEndCapture(bt->stream, &g);
        if (rc != FK_OK) { if (g) cudaGraphDestroy(g); return rc; }
        if (ce != cudaSuccess) return bt->cuda_fail(ce, "end capture");
        cudaGraphExec_t ge = nullptr;
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return bt->cuda_fail(ce, "instantiate graph");
        it = bt->graphs.emplace(M, ge).first;
    }
    BT_TRY(cudaGraphLaunch(it->second, bt->stream), "graph launch");
    return FK_OK;
}

cudaError_t batch_launch_adjoint(fk_batch* bt, const fk::AdjArgs& a, const fk::Launch& l) {
    switch (bt->prec) {
        case fk::kF64: return fk::launch_adjoint_f64(bt->cplx, bt->b, bt->NP, a, l);
        case fk::kF32: return bt->acc64 ? fk::launch_adjoint_f32a(bt->cplx, bt->b, bt->NP, a, l)
                                        : fk::launch_adjoint_f32(bt->cplx, bt->b, bt->NP, a, l);
        default: return fk::launch_adjoint_ds(bt->cplx, bt->b, bt->NP, a, l);
    }
}
cudaError_t batch_launch_outer(fk_batch* bt, const fk::OuterArgs& a, const fk::Launch& l) {
    switch (bt->prec) {
        case fk::kF64: return fk::launch_outer_f64(bt->cplx, bt->b, bt->NP, a, l);
        case fk::kF32: return bt->acc64 ? fk::launch_outer_f32a(bt->cplx, bt->b, bt->NP, a, l)
                                        : fk::launch_outer_f32(bt->cplx, bt->b, bt->NP, a, l);
        default: return fk::launch_outer_ds(bt->cplx, bt->b, bt->NP, a, l);
    }
}
cudaError_t batch_scale_rows(fk_batch* bt, const void* x, void* y, const double* f) {
    switch (bt->prec) {
        case fk::kF64: return fk::launch_scale_rows_f64(bt->cplx, x, y, bt->total_rows, bt->ld, bt->b, bt->d_rowsys.as<int>(), f, bt->stream);
        case fk::kF32: return fk::launch_scale_rows_f32(bt->cplx, x, y, bt->total_rows, bt->ld, bt->b, bt->d_rowsys.as<int>(), f, bt->stream);
        default: return fk::launch_scale_rows_ds(bt->cplx, x, y, bt->total_rows, bt->ld, bt->b, bt->d_rowsys.as<int>(), f, bt->stream);
    }
}

// Tables of the symmetrize step on the prepared pattern: block row, block column and partner
// (j, i) of every block, and 1 / mag of its system per block row.
int batch_d_tables(fk_batch* bt) {
    if (bt->d_tables) return FK_OK;
    const int rows = (int)bt->h_row_ptr.size() - 1;
    const size_t nk = bt->h_col.size();
    std::vector<int> brow(nk), pair(nk);
    std::vector<double> rscale(rows);
    std::vector<int> rsys(rows);
    for (int sys = 0; sys < bt->n_sys; sys++)
        for (int i = bt->row_base[sys]; i < bt->row_base[sys] + bt->n_b[sys]; i++) {
            rscale[i] = 1.0 / bt->mag[sys];
            rsys[i] = sys;
        }
    for (int i = 0; i < rows; i++) {
        for (int k = bt->h_row_ptr[i]; k < bt->h_row_ptr[i + 1]; k++) {
            brow[k] = i;
            const int j = bt->h_col[k];
            const int* lo = bt->h_col.data() + bt->h_row_ptr[j];
            const int* hi = bt->h_col.data() + bt->h_row_ptr[j + 1];
            const int* f = std::lower_bound(lo, hi, i);
            if (f == hi || *f != i)
                return bt->fail(FK_ERR_PATTERN, "batch_autodiff_matrix: H's pattern is not symmetric (block %d, %d)", i, j);
            pair[k] = (int)(f - bt->h_col.data());
        }
    }
    BT_TRY(bt->d_rows.ensure(sizeof(int) * std::max<size_t>(nk, 1)), "alloc D tables");
    BT_TRY(bt->d_cols.ensure(sizeof(int) * std::max<size_t>(nk, 1)), "alloc D tables");
    BT_TRY(bt->d_pair.ensure(sizeof(int) * std::max<size_t>(nk, 1)), "alloc D tables");
    BT_TRY(bt->d_rowscale.ensure(sizeof(double) * rows), "alloc D tables");
    BT_TRY(bt->d_rowsys.ensure(sizeof(int) * rows), "alloc D tables");
    BT_TRY(cudaMemcpy(bt->d_rowsys.p, rsys.data(), sizeof(int) * rows, cudaMemcpyHostToDevice), "upload D tables");
    BT_TRY(cudaMemcpy(bt->d_rows.p, brow.data(), sizeof(int) * nk, cudaMemcpyHostToDevice), "upload D tables");
    BT_TRY(cudaMemcpy(bt->d_cols.p, bt->h_col.data(), sizeof(int) * nk, cudaMemcpyHostToDevice), "upload D tables");
    BT_TRY(cudaMemcpy(bt->d_pair.p, pair.data(), sizeof(int) * nk, cudaMemcpyHostToDevice), "upload D tables");
    BT_TRY(cudaMemcpy(bt->d_rowscale.p, rscale.data(), sizeof(double) * rows, cudaMemcpyHostToDevice), "upload D tables");
    // output order: each system's blocks as added, systems in index order
    std::vector<int> gl;
    for (int sys = 0; sys < bt->n_sys; sys++) gl.insert(gl.end(), bt->o2a[sys].begin(), bt->o2a[sys].end());
    bt->n_out_blocks = (long long)gl.size();
    bt->d_gather_identity = gl.size() == nk;
    for (size_t q = 0; q < gl.size() && bt->d_gather_identity; q++) bt->d_gather_identity = gl[q] == (int)q;
    if (!bt->d_gather_identity) {
        BT_TRY(bt->d_gather.ensure(sizeof(int) * std::max<size_t>(gl.size(), 1)), "alloc D tables");
        BT_TRY(cudaMemcpy(bt->d_gather.p, gl.data(), sizeof(int) * gl.size(), cudaMemcpyHostToDevice), "upload D tables");
    }
    bt->d_tables = true;
    return FK_OK;
}

// autodiff_matrix for every system of the batch at once (the single engine's reverse recursion,
// src/engine_cpu.cpp:255-304, with per-system coefficients c[sys * M + m]): D on each system's
// own H pattern, symmetrized and divided by that system's mag. The adjoint and outer-product
// kernels run with the batch's system tables, so every system's CTAs stay its own.
int batch_autodiff(fk_batch* bt, int M, const double* c, double* D_out) {
    if (M < 2 || M % 2) return bt->fail(FK_ERR_ARG, "batch_autodiff_matrix: M must be even and >= 2");
    if (bt->mom_M != M)
        return bt->fail(FK_ERR_STATE, "batch_autodiff_matrix(M=%d) needs batch_moments(%d) first", M, M);
    int rc = batch_d_tables(bt);
    if (rc != FK_OK) return rc;
    const size_t vb = (size_t)bt->total_rows * bt->ld * bt->esize();
    BT_TRY(bt->d_V[2].ensure(vb), "alloc work vector");
    BT_TRY(bt->d_V[3].ensure(vb), "alloc work vector");
    const int nsys = bt->n_sys;
    const size_t nk = bt->h_col.size(), bb = (size_t)bt->b * bt->b, cw = bt->cplx ? 2 : 1;
    const size_t dn = nk * bb * cw;
    BT_TRY(bt->d_D.ensure(sizeof(double) * std::max<size_t>(dn, 1)), "alloc D");
    BT_TRY(cudaMemsetAsync(bt->d_D.p, 0, sizeof(double) * dn, bt->stream), "clear D");
    // per adjoint step q (m = M/2-1-q) and system: {4 c_2m, 2 c_2m+1, 2 c_2m-1 or diag}
    const int nsteps = M / 2 - 1;
    std::vector<double> coef(3 * (size_t)std::max(nsteps, 1) * nsys, 0.0), fac(nsys);
    for (int sys = 0; sys < nsys; sys++) {
        const double* cs = c + (size_t)sys * M;
        double diag = cs[1];
        for (int m = 1; m < M / 2; m++) diag -= cs[2 * m + 1];
        for (int m = M / 2 - 1, q = 0; m >= 1; m--, q++) {
            double* t = &coef[3 * ((size_t)q * nsys + sys)];
            t[0] = 4 * cs[2 * m];
            t[1] = 2 * cs[2 * m + 1];
            t[2] = m > 1 ? 2 * cs[2 * m - 1] : diag;
        }
        fac[sys] = M > 2 ? 2 * cs[M - 1] : diag;   // beta_{M/2} = fac alpha_{M/2-1}
    }
    BT_TRY(bt->d_coef.ensure(sizeof(double) * coef.size()), "alloc coefficients");
    BT_TRY(bt->d_rowfac.ensure(sizeof(double) * nsys), "alloc factors");
    BT_TRY(cudaMemcpyAsync(bt->d_coef.p, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, bt->stream),
           "upload coefficients");
    BT_TRY(cudaMemcpyAsync(bt->d_rowfac.p, fac.data(), sizeof(double) * nsys, cudaMemcpyHostToDevice, bt->stream),
           "upload factors");
    // moments(M) left alpha_{M/2} in V[(M/2-1)&1] and alpha_{M/2-1} in V[(M/2)&1] (R when M = 2)
    void* V[4] = {bt->d_V[0].p, bt->d_V[1].p, bt->d_V[2].p, bt->d_V[3].p};
    void* A = M / 2 >= 2 ? V[(M / 2) & 1] : bt->d_R.p;
    void* Ap = V[(M / 2 - 1) & 1];
    void* Bv = V[2];
    void* Bp = V[3];
    const bool fuse = true;   // the single engine's default: the D epilogue rides on the adjoint step
    auto outer = [&](const void* a, const void* bv, double alpha) -> int {
        fk::OuterArgs o;
        o.sys = bt->d_sys.as<SysDesc>();
        o.cta_sys = bt->d_cta_sys.as<int>();
        o.Gp = bt->Gp;
        o.P = bt->P_launch;
        o.ld = bt->ld;
        o.row_ptr = bt->d_row_ptr.as<int>();
        o.colc = bt->d_colc.as<unsigned>();
        o.A = a;
        o.Bv = bv;
        o.alpha = alpha;
        o.two_terms = 0;
        o.Dacc = bt->d_D.as<double>();
        BT_TRY(batch_launch_outer(bt, o, fk::Launch{bt->grid, 0, bt->stream}), "batched outer-product launch");
        return FK_OK;
    };
    BT_TRY(batch_scale_rows(bt, A, Bv, bt->d_rowfac.as<double>()), "scale kernel");
    if (M > 2) {
        BT_TRY(cudaMemsetAsync(Bp, 0, vb, bt->stream), "clear beta");
        for (int q = 0; q < nsteps; q++) {
            if (!fuse) {
                rc = outer(A, Bv, 2.0);
                if (rc != FK_OK) return rc;
            }
            fk::AdjArgs a;
            a.sys = bt->d_sys.as<SysDesc>();
            a.cta_sys = bt->d_cta_sys.as<int>();
            a.Gp = bt->Gp;
            a.P = bt->P_launch;
            a.ld = bt->ld;
            a.row_ptr = bt->d_row_ptr.as<int>();
            a.colc = bt->d_colc.as<unsigned>();
            a.hval = bt->d_hval.p;
            a.A = A;
            a.Ap = Ap;
            a.Bv = Bv;
            a.Bp = Bp;
            a.coef = bt->d_coef.as<double>() + 3 * (size_t)q * nsys;
            a.cstride = 3;
            a.Dacc = fuse ? bt->d_D.as<double>() : nullptr;
            a.dscale = 2.0;
            a.stage_cap = bt->stage_cap;
            a.split = 0;
            a.pipe = 0;
            BT_TRY(batch_launch_adjoint(bt, a, fk::Launch{bt->grid, bt->smem, bt->stream}), "batched adjoint launch");
            std::swap(A, Ap);
            std::swap(Bv, Bp);
        }
    }
    rc = outer(A, Bv, 1.0);
    if (rc != FK_OK) return rc;
    if (bt->prec == fk::kDS || (bt->prec == fk::kF32 && !bt->acc64)) {   // float-float accumulator -> double
        const int g = (int)std::max<long long>(1, std::min<long long>(((long long)dn + 255) / 256, 152LL * 16));
        fk::k_ds_to_double<<<g, 256, 0, bt->stream>>>(bt->d_D.as<double>(), (long long)dn);
        BT_TRY(cudaGetLastError(), "accumulator conversion");
    }
    {
        const long long work = (long long)nk * bb;
        const int g = (int)std::max<long long>(1, std::min<long long>((work + 255) / 256, 152LL * 16));
        fk::k_symmetrize_scale<<<g, 256, 0, bt->stream>>>(bt->d_D.as<double>(), bt->d_rows.as<int>(), bt->d_cols.as<int>(),
                                                          bt->d_pair.as<int>(), (int)nk, bt->b, bt->cplx, 0.0,
                                                          bt->d_rowscale.as<double>());
        BT_TRY(cudaGetLastError(), "symmetrize launch");
    }
    // back to each system's own block order on the device, then one copy into the caller's buffer
    const int per = (int)(bb * cw);
    const size_t nout = (size_t)bt->n_out_blocks * per;
    const double* src = bt->d_D.as<double>();
    if (!bt->d_gather_identity) {
        BT_TRY(bt->d_Dout.ensure(sizeof(double) * std::max<size_t>(nout, 1)), "alloc D");
        const int g = (int)std::max<long long>(1, std::min<long long>(((long long)nout + 255) / 256, 152LL * 16));
        fk::k_gather_blocks<<<g, 256, 0, bt->stream>>>(src, bt->d_gather.as<int>(), bt->n_out_blocks, per,
                                                       bt->d_Dout.as<double>());
        BT_TRY(cudaGetLastError(), "gather launch");
        src = bt->d_Dout.as<double>();
    }
    if (nout) BT_TRY(cudaMemcpyAsync(D_out, src, sizeof(double) * nout, cudaMemcpyDeviceToHost, bt->stream), "copy D");
    BT_TRY(cudaStreamSynchronize(bt->stream), "batch autodiff");
    bt->mom_M = 0;   // the alpha state is consumed
    return FK_OK;
}

}  // namespace

extern "C" {

int fk_batch_create(int device, int kind, int precision, fk_batch** out) {
    if (!out) return FK_ERR_ARG;
    *out = nullptr;
    if (kind != FK_REAL && kind != FK_COMPLEX) return FK_ERR_ARG;
    if (precision < FK_PREC_FP64 || precision > FK_PREC_DS) return FK_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) { cudaGetLastError(); return FK_ERR_NODEV; }
    if (device < 0 || device >= count) return FK_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return FK_ERR_CUDA; }
    fk_batch* bt = new fk_batch();
    bt->device = device;
    bt->cplx = kind;
    bt->prec = precision;
    cudaDeviceGetAttribute(&bt->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete bt;
        return FK_ERR_CUDA;
    }
    *out = bt;
    return FK_OK;
}

int fk_batch_destroy(fk_batch* bt) {
    if (!bt) return FK_OK;
    cudaSetDevice(bt->device);
    cudaStreamSynchronize(bt->stream);
    bt->drop_graphs();
    Buf* bufs[] = {&bt->d_row_ptr, &bt->d_colc, &bt->d_hval, &bt->d_R, &bt->d_V[0], &bt->d_V[1], &bt->d_V[2],
                   &bt->d_V[3], &bt->d_stage, &bt->d_sys, &bt->d_cta_sys, &bt->d_partials, &bt->d_raw, &bt->d_D,
                   &bt->d_coef, &bt->d_rows, &bt->d_cols, &bt->d_pair, &bt->d_rowscale, &bt->d_rowfac,
                   &bt->d_rowsys, &bt->d_gather, &bt->d_Dout};
    for (auto* b : bufs) b->release();
    if (bt->t0) cudaEventDestroy(bt->t0);
    if (bt->t1) cudaEventDestroy(bt->t1);
    cudaStreamDestroy(bt->stream);
    delete bt;
    return FK_OK;
}

const char* fk_batch_last_error(const fk_batch* bt) { return bt ? bt->err.c_str() : "null batch"; }

int fk_batch_add(fk_batch* bt, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx, const double* val,
                 double es_lo, double es_hi, int s, const double* R, int* index) {
    if (!bt) return FK_ERR_ARG;
    if (s <= 0 || !R) return bt->fail(FK_ERR_ARG, "batch_add: need a probe block with s >= 1 columns");
    const int ref_b = bt->pending.empty() ? (bt->n_sys ? bt->b : b) : bt->pending.front().b;
    if (b != ref_b) return bt->fail(FK_ERR_ARG, "batch_add: every system needs the same block size b");
    PendingSystem ps;
    std::string why;
    int rc = fk::prepare_H(bt->prec, bt->cplx, n_b, b, nnzb, row_ptr, col_idx, val, es_lo, es_hi, 0, ps.h, why);
    if (rc != FK_OK) return bt->fail(rc, "batch_add: %s", why.c_str());
    ps.n_b = n_b;
    ps.b = b;
    ps.s = s;
    ps.mag = (es_hi - es_lo) / 2.0;
    ps.o2a.resize(nnzb);
    for (int i = 0; i < n_b; i++) {   // the prepared row holds the original blocks in order plus maybe a diagonal
        int a = ps.h.row_ptr[i];
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
            while (ps.h.col[a] != col_idx[k]) a++;
            ps.o2a[k] = a++;
        }
    }
    ps.R.assign(R, R + (size_t)n_b * b * s * (bt->cplx ? 2 : 1));
    bt->pending.push_back(std::move(ps));
    if (index) *index = bt->n_sys + (int)bt->pending.size() - 1;
    return FK_OK;
}

int fk_batch_commit(fk_batch* bt) {
    if (!bt) return FK_ERR_ARG;
    if (bt->pending.empty()) return bt->n_sys ? FK_OK : bt->fail(FK_ERR_STATE, "batch_commit: no systems added");
    if (bt->n_sys) return bt->fail(FK_ERR_UNSUPPORTED, "batch_commit: systems can only be committed once");
    cudaSetDevice(bt->device);
    auto& ps = bt->pending;
    bt->b = ps[0].b;
    bt->s = 0;
    for (const auto& q : ps) bt->s = std::max(bt->s, q.s);
    bt->n_sys = (int)ps.size();
    const int epp = bt->epp();
    bt->ld = ((long long)bt->s + epp - 1) / epp * epp;   // every system's rows use the widest one's stride
    bt->P = (int)(bt->ld / epp);
    bt->Pk.resize(bt->n_sys);
    for (int k = 0; k < bt->n_sys; k++) bt->Pk[k] = (ps[k].s + epp - 1) / epp;
    long long rows = 0, nk = 0;
    bt->row_base.resize(bt->n_sys);
    bt->n_b.resize(bt->n_sys);
    bt->mag.resize(bt->n_sys);
    bt->o2a.resize(bt->n_sys);
    for (int k = 0; k < bt->n_sys; k++) {
        bt->row_base[k] = (int)rows;
        bt->n_b[k] = ps[k].n_b;
        rows += ps[k].n_b;
        nk += (long long)ps[k].h.col.size();
    }
    if (rows > (long long)fk::kColMask || nk >= (1LL << 31)) return bt->fail(FK_ERR_UNSUPPORTED, "batch too large");
    bt->total_rows = rows * bt->b;
    // concatenated H with global columns
    bt->h_row_ptr.assign(rows + 1, 0);
    std::vector<unsigned> colc;
    colc.reserve(nk);
    std::vector<unsigned char> hval;
    for (int k = 0; k < bt->n_sys; k++) {
        const int kb = (int)colc.size();
        for (int i = 0; i < ps[k].n_b; i++) bt->h_row_ptr[bt->row_base[k] + i + 1] = kb + ps[k].h.row_ptr[i + 1];
        for (unsigned cc : ps[k].h.colc) {
            const unsigned cls = cc >> 30, col = cc & fk::kColMask;
            colc.push_back((col + (unsigned)bt->row_base[k]) | (cls << 30));
        }
        bt->mag[k] = ps[k].mag;
        bt->o2a[k] = std::move(ps[k].o2a);
        for (int& v : bt->o2a[k]) v += kb;
        hval.insert(hval.end(), ps[k].h.hval.begin(), ps[k].h.hval.end());
    }
    bt->h_col.resize(colc.size());
    for (size_t q = 0; q < colc.size(); q++) bt->h_col[q] = (int)(colc[q] & fk::kColMask);
    BT_TRY(bt->d_row_ptr.ensure(sizeof(int) * (rows + 1)), "alloc H row_ptr");
    BT_TRY(bt->d_colc.ensure(sizeof(unsigned) * std::max<size_t>(colc.size(), 1)), "alloc H columns");
    BT_TRY(bt->d_hval.ensure(std::max<size_t>(hval.size(), 16)), "alloc H values");
    BT_TRY(cudaMemcpy(bt->d_row_ptr.p, bt->h_row_ptr.data(), sizeof(int) * (rows + 1), cudaMemcpyHostToDevice), "upload H");
    BT_TRY(cudaMemcpy(bt->d_colc.p, colc.data(), sizeof(unsigned) * colc.size(), cudaMemcpyHostToDevice), "upload H");
    BT_TRY(cudaMemcpy(bt->d_hval.p, hval.data(), hval.size(), cudaMemcpyHostToDevice), "upload H");
    const size_t vb = (size_t)bt->total_rows * bt->ld * bt->esize();
    BT_TRY(bt->d_R.ensure(vb), "alloc R");
    BT_TRY(bt->d_V[0].ensure(vb), "alloc work vector");
    BT_TRY(bt->d_V[1].ensure(vb), "alloc work vector");
    BT_TRY(cudaMemsetAsync(bt->d_R.p, 0, vb, bt->stream), "clear R");
    BT_TRY(cudaMemsetAsync(bt->d_V[0].p, 0, vb, bt->stream), "clear");
    BT_TRY(cudaMemsetAsync(bt->d_V[1].p, 0, vb, bt->stream), "clear");
    for (int k = 0; k < bt->n_sys; k++) {
        const long long n = (long long)ps[k].n_b * bt->b;
        const size_t bytes = ps[k].R.size() * sizeof(double);
        BT_TRY(bt->d_stage.ensure(bytes), "alloc staging");
        BT_TRY(cudaMemcpyAsync(bt->d_stage.p, ps[k].R.data(), bytes, cudaMemcpyHostToDevice, bt->stream), "upload R");
        char* dst = (char*)bt->d_R.p + (size_t)bt->row_base[k] * bt->b * bt->ld * bt->esize();
        BT_TRY(batch_load(bt, bt->d_stage.as<double>(), n, ps[k].s, 0, dst), "R layout kernel");
        BT_TRY(cudaStreamSynchronize(bt->stream), "upload R");
    }
    bt->d_stage.release();
    bt->pending.clear();
    // a mapping remembered for this batch shape, else the automatic one
    Mapping m = bt->opt;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(std::make_tuple(bt->prec, bt->cplx, bt->b, bt->P, (long long)bt->total_rows, bt->n_sys));
        if (it != g_tuned.end() && m.Gp == 0 && m.NP == 0 && m.cap_per_sm == 0) m = it->second;
    }
    return batch_configure(bt, m);
}

int fk_batch_moments(fk_batch* bt, int M, double* mu) {
    if (!bt || !mu) return FK_ERR_ARG;
    if (M < 2 || M % 2) return bt->fail(FK_ERR_ARG, "batch_moments: M must be even and >= 2");
    if (!bt->configured) return bt->fail(FK_ERR_STATE, "batch_moments: commit the batch first");
    cudaSetDevice(bt->device);
    int rc = batch_run_moments(bt, M);
    if (rc != FK_OK) return rc;
    bt->mom_M = M;
    const int nsteps = M / 2;
    bt->h_raw.resize(2 * (size_t)nsteps * bt->n_sys);
    BT_TRY(cudaMemcpyAsync(bt->h_raw.data(), bt->d_raw.p, sizeof(double) * bt->h_raw.size(), cudaMemcpyDeviceToHost,
                           bt->stream), "copy moment sums");
    BT_TRY(cudaStreamSynchronize(bt->stream), "batch moments");
    for (int k = 0; k < bt->n_sys; k++) {
        double* out = mu + (size_t)k * M;
        const double* r0 = &bt->h_raw[2 * (size_t)k];
        out[0] = r0[0];
        out[1] = r0[1];
        for (int m = 1; m < nsteps; m++) {
            const double* r = &bt->h_raw[2 * ((size_t)m * bt->n_sys + k)];
            out[2 * m] = 2 * r[0] - out[0];
            out[2 * m + 1] = 2 * r[1] - out[1];
        }
    }
    return FK_OK;
}

int fk_batch_autodiff_matrix(fk_batch* bt, int M, const double* c, double* D_val) {
    if (!bt || !c || !D_val) return FK_ERR_ARG;
    if (!bt->configured) return bt->fail(FK_ERR_STATE, "batch_autodiff_matrix: commit the batch first");
    cudaSetDevice(bt->device);
    return batch_autodiff(bt, M, c, D_val);
}

int fk_batch_set_option(fk_batch* bt, int option, int value) {
    if (!bt) return FK_ERR_ARG;
    cudaSetDevice(bt->device);
    switch (option) {
        case FK_OPT_GRAPHS: bt->opt_graphs = value ? 1 : 0; bt->drop_graphs(); return FK_OK;
        case FK_OPT_NP:
            if (value != 0 && value != 1 && value != 2 && value != 4) return bt->fail(FK_ERR_ARG, "NP must be 0, 1, 2 or 4");
            bt->opt.NP = value;
            bt->opt.Gp = 0;
            break;
        case FK_OPT_CTAS_PER_SM: bt->opt.cap_per_sm = std::max(0, value); break;
        case FK_OPT_STAGE_H: bt->opt.stage = value == 2 ? -1 : (value ? 1 : 0); break;
        case FK_OPT_FUSE_D: return FK_OK;
        case FK_OPT_ACC64:
            if (value < 0 || value > 1) return bt->fail(FK_ERR_ARG, "ACC64 must be 0 or 1");
            bt->acc64 = value;
            bt->drop_graphs();
            // the two kernel families may differ in occupancy: rebuild the launch tables for them
            return bt->configured ? batch_configure(bt, bt->cur) : FK_OK;
        default: return bt->fail(FK_ERR_ARG, "unknown option %d", option);
    }
    if (!bt->n_sys) return FK_OK;
    return batch_configure(bt, bt->opt);   // (lanes per row follow the packets per lane, per system)
}

int fk_batch_get_option(const fk_batch* bt, int option, int* value) {
    if (!bt || !value) return FK_ERR_ARG;
    switch (option) {
        case FK_OPT_GRAPHS: *value = bt->opt_graphs; return FK_OK;
        case FK_OPT_NP: *value = bt->NP; return FK_OK;
        case FK_OPT_CTAS_PER_SM: *value = bt->cur.cap_per_sm; return FK_OK;
        case FK_OPT_STAGE_H: *value = bt->stage_cap > 0; return FK_OK;
        case FK_OPT_ACC64: *value = bt->prec == fk::kF64 ? 1 : bt->prec == fk::kF32 ? bt->acc64 : 0; return FK_OK;
        default: return FK_ERR_ARG;
    }
}

int fk_batch_autotune(fk_batch* bt, int trial_steps, int* lanes, int* np_out, int* cap_out, int* stage_out, double* ms_out) {
    if (!bt) return FK_ERR_ARG;
    if (!bt->configured) return bt->fail(FK_ERR_STATE, "batch_autotune: commit the batch first");
    if (trial_steps < 1) trial_steps = 8;
    cudaSetDevice(bt->device);
    // candidate mappings: packets per lane (each system's lanes per row follow), CTA caps, H staging
    std::vector<Mapping> cands;
    for (int np : {1, 2, 4})
        for (int cap : {0, 1, 2, 3, 4, 6})
            for (int st : {1, 0}) cands.push_back(Mapping{0, np, cap, st});
    const int M = 2 * (trial_steps + 1);
    if (!bt->t0) cudaEventCreate(&bt->t0);
    if (!bt->t1) cudaEventCreate(&bt->t1);
    const int saved_graphs = bt->opt_graphs;
    bt->opt_graphs = 0;
    Mapping best;
    double best_ms = 1e300;
    for (const Mapping& m : cands) {
        int rc = batch_configure(bt, m);
        if (rc != FK_OK) continue;
        rc = batch_ensure_partials(bt, M / 2);
        if (rc != FK_OK) return rc;
        rc = batch_enqueue_moments(bt, M);   // warm-up
        if (rc != FK_OK) return rc;
        BT_TRY(cudaEventRecord(bt->t0, bt->stream), "tune timer");
        rc = batch_enqueue_moments(bt, M);
        if (rc != FK_OK) return rc;
        BT_TRY(cudaEventRecord(bt->t1, bt->stream), "tune timer");
        BT_TRY(cudaEventSynchronize(bt->t1), "tune timer");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, bt->t0, bt->t1);
        const double per_step = ms / (M / 2);
        if (per_step < best_ms) { best_ms = per_step; best = m; }
    }
    bt->opt_graphs = saved_graphs;
    int rc = batch_configure(bt, best);
    if (rc != FK_OK) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[std::make_tuple(bt->prec, bt->cplx, bt->b, bt->P, (long long)bt->total_rows, bt->n_sys)] = best;
    }
    if (lanes) *lanes = bt->Gp;   // (the widest system's; narrower ones take fewer)
    if (np_out) *np_out = best.NP;
    if (cap_out) *cap_out = best.cap_per_sm;
    if (stage_out) *stage_out = best.stage;
    if (ms_out) *ms_out = best_ms;
    return FK_OK;
}

int fk_batch_profile_moments(fk_batch* bt, int M, double* kernel_ms, int* launches) {
    if (!bt || !kernel_ms || !launches) return FK_ERR_ARG;
    if (!bt->configured) return bt->fail(FK_ERR_STATE, "batch_profile_moments: commit the batch first");
    if (M < 2 || M % 2 != 0) return bt->fail(FK_ERR_ARG, "M must be even and >= 2");
    cudaSetDevice(bt->device);
    int rc = batch_ensure_partials(bt, M / 2);
    if (rc != FK_OK) return rc;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    bt->prof = &ev;
    rc = batch_enqueue_moments(bt, M);
    bt->prof = nullptr;
    double total = 0.0;
    cudaError_t ce = cudaStreamSynchronize(bt->stream);
    for (auto& p : ev) {
        float f = 0.f;
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&f, p.first, p.second);
        total += f;
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    if (rc != FK_OK) return rc;
    if (ce != cudaSuccess) return bt->cuda_fail(ce, "batch_profile_moments");
    bt->mom_M = M;
    *kernel_ms = total;
    *launches = (int)ev.size();
    return FK_OK;
}

int fk_batch_timer_start(fk_batch* bt) {
    if (!bt) return FK_ERR_ARG;
    cudaSetDevice(bt->device);
    if (!bt->t0) BT_TRY(cudaEventCreate(&bt->t0), "timer");
    if (!bt->t1) BT_TRY(cudaEventCreate(&bt->t1), "timer");
    BT_TRY(cudaEventRecord(bt->t0, bt->stream), "timer start");
    return FK_OK;
}

int fk_batch_timer_stop(fk_batch* bt, double* ms) {
    if (!bt || !ms) return FK_ERR_ARG;
    if (!bt->t0) return bt->fail(FK_ERR_STATE, "timer not started");
    cudaSetDevice(bt->device);
    BT_TRY(cudaEventRecord(bt->t1, bt->stream), "timer stop");
    BT_TRY(cudaEventSynchronize(bt->t1), "timer wait");
    float f = 0.f;
    BT_TRY(cudaEventElapsedTime(&f, bt->t0, bt->t1), "timer elapsed");
    *ms = f;
    return FK_OK;
}

int fk_batch_info(const fk_batch* bt, int* n_systems, long long* total_rows, size_t* device_bytes) {
    if (!bt) return FK_ERR_ARG;
    if (n_systems) *n_systems = bt->n_sys;
    if (total_rows) *total_rows = bt->total_rows;
    if (device_bytes) {
        size_t t = bt->d_row_ptr.bytes + bt->d_colc.bytes + bt->d_hval.bytes + bt->d_R.bytes + bt->d_V[0].bytes +
                   bt->d_V[1].bytes + bt->d_sys.bytes + bt->d_cta_sys.bytes + bt->d_partials.bytes + bt->d_raw.bytes;
        *device_bytes = t;
    }
    return FK_OK;
}

}  // extern "C"
