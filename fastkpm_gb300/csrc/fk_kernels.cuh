// fk_kernels.cuh -- hand-written sm_103a kernels for the stochastic Chebyshev path.
//
// Data layout in HBM (all kernels):
//   * Probe / recursion vectors: row-major N x ld elements (ld = S rounded up to
//     a whole 16-byte packet, P = ld / EPP packets per row); scalar row
//     r = b*i + bi of block row i. Padding columns hold zeros and stay zero.
//   * H: BSR. row_ptr[n_b+1]; colc[k] = block column | class << 30; hval holds
//     b*b entries per block, column-major (the reference's BSR block order,
//     src/fastkpm.h:64-65). Class 0: general entries, 1: real entries, 2: real
//     multiple of the identity (only the (0,0) entry is read).
//   * Several Hamiltonians ("systems") can share one launch: their block rows
//     are concatenated, columns are global, and SysDesc says which CTAs work on
//     which system. A CTA only ever touches one system, and the number of CTAs a
//     system gets depends on that system alone, so every per-system reduction is
//     the same whether the system runs alone or in a batch.
//
// Thread mapping: a block row is served by Gp lanes (a power of two <= 32,
// aligned inside the warp). Items (row, lane) are cut into tiles of kThreads;
// each CTA walks the tiles of its system with a CTA-count stride, stages the
// tile's H blocks in shared memory once, and then walks the row's columns in
// chunks of W = Gp * NP packets: in chunk c lane g owns packets
// c*W + g + q*Gp (q < NP), so every access is a coalesced 16-byte packet and NP
// sets the registers each thread holds. Sums that span columns (moment dots,
// D entries) are accumulated across chunks in a fixed order by the same thread.
#pragma once
#include "fk_sys.cuh"

namespace fk {

constexpr int kThreads = 256;
constexpr unsigned kColMask = 0x3fffffffu;

struct SysDesc {
    int row_base;    // first global block row
    int n_b;         // block rows
    int cta_base;    // first CTA of this system
    int ctas;        // CTAs assigned to this system
    int P;           // packets per row of this system's probe columns (0: the launch's P); systems of a
                     // batch may have different probe counts and share the row stride of the widest
    int Gp;          // lanes per block row of this system (0: the launch's Gp)
};

struct StepArgs {
    const SysDesc* sys;
    const int* cta_sys;        // CTA -> system index
    int Gp, P;                 // lanes per block row, packets per row
    long long ld;              // elements per scalar row
    const int* row_ptr;
    const unsigned* colc;
    const void* hval;
    const void* x;             // gathered input
    const void* z;             // own-row input (may be null)
    void* y;                   // output (may alias z)
    void* xi;                  // stochastic-sum accumulator (xi_mode != 0)
    const double* coef;        // per system: coef[sys * cstride + ...]
    int cstride;
    int two, has_z, want_dots, xi_mode;   // xi_mode 1: xi = c0 x + c1 y;  2: xi += c1 y
    double* partials;          // 2 doubles per CTA: <x,x>, Re<y,x>
    int stage_cap;             // blocks that fit the shared-memory stage (0: no staging)
    int pipe;                  // FP32 systems: run k_cheb_step_pipe (double-buffered gathers)
};

struct AdjArgs {
    const SysDesc* sys;
    const int* cta_sys;
    int Gp, P;
    long long ld;
    const int* row_ptr;
    const unsigned* colc;
    const void* hval;
    const void* A;        // alpha_m          (gathered)
    void* Ap;             // alpha_{m+1} in,  alpha_{m-1} out
    const void* Bv;       // beta_{m+1}       (gathered)
    void* Bp;             // beta_{m+2} in,   beta_m out
    const double* coef;   // per system: cA, cAp, cAn
    int cstride;
    double* Dacc;         // FP64 D accumulator on H's pattern (null: no fused epilogue)
    double dscale;        // D += dscale * A_i B_j^dagger
    int stage_cap;
    int split;            // run k_adjoint_split (two passes over the blocks) instead of k_adjoint_step
    int pipe;             // FP32 systems: run k_adjoint_pipe (double-buffered gathers)
    int warp = 0;         // with pipe, Gp == 32, whole chunks and the fused epilogue: run k_adjoint_warp
    const unsigned char* row_hsum = nullptr;   // per row (float-float k_adjoint_warp): identity blocks of one value
};

struct OuterArgs {
    const SysDesc* sys;
    const int* cta_sys;
    int Gp, P;
    long long ld;
    const int* row_ptr;        // D pattern
    const unsigned* colc;      // D pattern columns (class bits ignored)
    const void* A;
    const void* Bv;
    double alpha;              // D += alpha (A B^dagger [+ B A^dagger when two_terms])
    int two_terms;
    double* Dacc;
};

template <class E, int EPP>
union Packet {
    uint4 u;
    E e[EPP];
};

// Packets base + g + q*Gp (q < NP) of one row, masked to pk < P (FULL: every chunk of the
// row is whole, P a multiple of Gp * NP, and no mask is needed).
// Gathered rows are read-only for the whole kernel: non-coherent path.
template <class S, int NP, bool FULL = false>
__device__ __forceinline__ void ld_nc(typename S::E (&v)[NP * S::EPP], const typename S::E* row, int base, int g,
                                      int Gp, int P) {
    constexpr int EPP = S::EPP;
#pragma unroll
    for (int q = 0; q < NP; q++) {
        const int pk = base + g + Gp * q;
        Packet<typename S::E, EPP> pkt;
        pkt.u = make_uint4(0u, 0u, 0u, 0u);
        if (FULL || pk < P) pkt.u = __ldg(reinterpret_cast<const uint4*>(row) + pk);
#pragma unroll
        for (int e = 0; e < EPP; e++) v[q * EPP + e] = pkt.e[e];
    }
}
template <class S, int NP, bool FULL = false>
__device__ __forceinline__ void ld_rw(typename S::E (&v)[NP * S::EPP], const typename S::E* row, int base, int g,
                                      int Gp, int P) {
    constexpr int EPP = S::EPP;
#pragma unroll
    for (int q = 0; q < NP; q++) {
        const int pk = base + g + Gp * q;
        Packet<typename S::E, EPP> pkt;
        pkt.u = make_uint4(0u, 0u, 0u, 0u);
        if (FULL || pk < P) pkt.u = reinterpret_cast<const uint4*>(row)[pk];
#pragma unroll
        for (int e = 0; e < EPP; e++) v[q * EPP + e] = pkt.e[e];
    }
}
template <class S, int NP, bool FULL = false>
__device__ __forceinline__ void st(typename S::E* row, const typename S::E (&v)[NP * S::EPP], int base, int g, int Gp,
                                   int P) {
    constexpr int EPP = S::EPP;
#pragma unroll
    for (int q = 0; q < NP; q++) {
        const int pk = base + g + Gp * q;
        Packet<typename S::E, EPP> pkt;
#pragma unroll
        for (int e = 0; e < EPP; e++) pkt.e[e] = v[q * EPP + e];
        if (FULL || pk < P) reinterpret_cast<uint4*>(row)[pk] = pkt.u;
    }
}

// Block-wide sum of two Dot values; thread 0 gets the result.
template <class S>
__device__ __forceinline__ void block_reduce2(typename S::Dot& a, typename S::Dot& b) {
    typedef typename S::Dot Dot;
    __shared__ Dot red[2][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    auto wsum = [&](Dot v) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v = S::dot_shfl_add(v, off);
        return v;
    };
    a = wsum(a);
    b = wsum(b);
    __syncthreads();
    if (lane == 0) { red[0][wid] = a; red[1][wid] = b; }
    __syncthreads();
    if (wid == 0) {
        a = lane < kThreads / 32 ? red[0][lane] : S::dot_zero();
        b = lane < kThreads / 32 ? red[1][lane] : S::dot_zero();
        a = wsum(a);
        b = wsum(b);
    }
}

// Stage H blocks [k_lo, k_lo + nk) into shared memory.
template <class S, int B>
__device__ __forceinline__ void stage_h(unsigned* s_col, typename S::H* s_h, const unsigned* colc,
                                        const typename S::H* hval, int k_lo, int nk) {
    for (int q = threadIdx.x; q < nk; q += blockDim.x) s_col[q] = __ldg(colc + k_lo + q);
    const int nh = nk * B * B;
    const typename S::H* src = hval + (size_t)k_lo * B * B;
    for (int q = threadIdx.x; q < nh; q += blockDim.x) s_h[q] = src[q];
}

// acc[bi] += sum_bj H_k(bi, bj) x[b j + bj] for one block (class-specialised).
template <class S, int B, int NP>
__device__ __forceinline__ void mac_block(typename S::Acc (&acc)[B][NP * S::EPP], unsigned cls, const typename S::H* hk,
                                          const typename S::E (&xv)[NP * S::EPP], int bj) {
    constexpr int EPT = NP * S::EPP;
    if (cls == 2u) {
        const typename S::Hr h = S::hreal(hk[bj * B + bj]);
#pragma unroll
        for (int e = 0; e < EPT; e++) S::mac_re(acc[bj][e], h, xv[e]);
    } else if (!S::CPLX || cls == 1u) {
#pragma unroll
        for (int bi = 0; bi < B; bi++) {
            const typename S::Hr h = S::hreal(hk[bj * B + bi]);
#pragma unroll
            for (int e = 0; e < EPT; e++) S::mac_re(acc[bi][e], h, xv[e]);
        }
    } else {
#pragma unroll
        for (int bi = 0; bi < B; bi++) {
            const typename S::H h = hk[bj * B + bi];
#pragma unroll
            for (int e = 0; e < EPT; e++) S::mac(acc[bi][e], h, xv[e]);
        }
    }
}

// Tile bookkeeping shared by the kernels: rows of tile t0 and their H block range.
struct Tile {
    int k_lo, nk;
    bool staged;
};
__device__ __forceinline__ Tile tile_range(const int* row_ptr, const SysDesc& sd, long long t0, long long items, int Gp,
                                           int stage_cap) {
    Tile t;
    if (stage_cap <= 0) {   // no stage: skip the two row_ptr reads (a memory round trip per tile)
        t.k_lo = 0;
        t.nk = 0;
        t.staged = false;
        return t;
    }
    const int r_lo = sd.row_base + (int)(t0 / Gp);
    const long long t_last = min(t0 + kThreads, items) - 1;
    const int r_hi = sd.row_base + (int)(t_last / Gp);
    t.k_lo = row_ptr[r_lo];
    t.nk = row_ptr[r_hi + 1] - t.k_lo;
    t.staged = t.nk <= stage_cap;
    return t;
}

// ---------------------------------------------------------------------------------
// Chebyshev step: y = (two ? 2 : 1) * Hs x  (- z), fused with the moment partials
// <x,x>, Re<y,x> over own rows and with the stochastic sum xi.
// ---------------------------------------------------------------------------------
// "Light" step threads hold at most 32 bytes of x per block (b=1 and narrow rows, e.g. S=32
// FP32): they are held to <= 40 registers so that 6 CTAs (48 warps) fit an SM (measured on
// 64 square lattices, b=1, S=32: 47 ms vs 53 ms per M=500 batch, a few spilled bytes included).
template <class S, int B, int NP>
constexpr bool kLightStep = B * NP * S::EPP * (int)sizeof(typename S::E) <= 32;

// CTAs per SM each kernel is compiled for (the register cap is 65536 / (256 x CTAs)). Measured
// per launch on GB300 against 2 CTAs (128 registers):
//  * step, FP32 and b=1 float-float at 3: cubic L=64 S=256 b=2 FP32 0.78 vs 0.92 ms; b=2 S=128
//    (10^6 sites) 1.65 vs 2.13; b=1 S=128 FP32 0.31 vs 0.39, float-float 0.32 vs 0.37; b=2
//    float-float stays at 2 (cubic L=64: 3.04 ms at 3 vs 2.65, spills);
//  * outer product, b=1 at 3: S=128 FP32 0.42 vs 0.51 ms, float-float 0.34 vs 0.38; b=2 at 2
//    (FP32 cubic L=64: 1.59 ms at 3 vs 1.36).
template <class S, int B, int NP>
constexpr int kStepCtas = kLightStep<S, B, NP> ? 6 : (S::PREC == 1 || (S::PREC == 2 && B == 1)) ? 3 : 2;
template <class S, int B, int NP>
constexpr int kOuterCtas = (B == 1 && S::PREC != 0) ? 3 : 2;
template <class S, int B, int NP>
constexpr int kAdjointCtas = kLightStep<S, B, NP> ? 4 : 2;
template <class S, int B, int NP>
constexpr int kAdjointSplitCtas = kLightStep<S, B, NP> ? 4 : 3;

template <class S, int B, int NP, bool FULL = false>
__global__ void __launch_bounds__(kThreads, kStepCtas<S, B, NP>) k_cheb_step(StepArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    constexpr int EPT = NP * S::EPP;
    extern __shared__ __align__(16) unsigned char smem[];
    H* s_h = reinterpret_cast<H*>(smem);
    unsigned* s_col = reinterpret_cast<unsigned*>(smem + sizeof(H) * B * B * (size_t)a.stage_cap);

    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const int Gp = sd.Gp > 0 ? sd.Gp : a.Gp, P = sd.P > 0 ? sd.P : a.P, W = Gp * NP;
    const int nch = (P + W - 1) / W;
    const long long items = (long long)sd.n_b * Gp;
    const E* x = reinterpret_cast<const E*>(a.x);
    const E* z = reinterpret_cast<const E*>(a.z);
    E* y = reinterpret_cast<E*>(a.y);
    E* xi = reinterpret_cast<E*>(a.xi);
    const H* hval = reinterpret_cast<const H*>(a.hval);
    const typename S::Coef c0 = S::coef(a.xi_mode ? a.coef[sidx * a.cstride + 0] : 0.0);
    const typename S::Coef c1 = S::coef(a.xi_mode ? a.coef[sidx * a.cstride + 1] : 0.0);

    typename S::Dot dxx = S::dot_zero(), dyx = S::dot_zero();
    for (long long t0 = (long long)lc * kThreads; t0 < items; t0 += (long long)sd.ctas * kThreads) {
        const Tile tl = tile_range(a.row_ptr, sd, t0, items, Gp, a.stage_cap);
        if (tl.staged) {
            __syncthreads();
            stage_h<S, B>(s_col, s_h, a.colc, hval, tl.k_lo, tl.nk);
            __syncthreads();
        }
        const long long t = t0 + threadIdx.x;
        if (t >= items) continue;
        const int il = (int)(t / Gp);
        const int g = (int)(t - (long long)il * Gp);
        const int i = sd.row_base + il;
        const int kb = a.row_ptr[i], ke = a.row_ptr[i + 1];   // (reading these a tile ahead measured slower)
        for (int c = 0; c < nch; c++) {
            const int base = c * W;
            typename S::Acc acc[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++)
#pragma unroll
                for (int e = 0; e < EPT; e++) acc[bi][e] = S::zero();
            // Not unrolled, and not pipelined by hand: unroll factors and a one-block-ahead
            // gather both measured slower (registers, fewer warps), for light (b=1, S=32
            // FP32) and heavy (b=2, S=256 complex) threads alike.
#pragma unroll 1
            for (int k = kb; k < ke; k++) {
                const unsigned cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                const H* hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
                const int j = (int)(cc & kColMask);
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E xv[EPT];
                    ld_nc<S, NP, FULL>(xv, x + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                    mac_block<S, B, NP>(acc, cc >> 30, hk, xv, bj);
                }
            }
            typename S::RowDot rxx = S::rd_zero(), ryx = S::rd_zero();
#pragma unroll
            for (int bi = 0; bi < B; bi++) {
                const size_t roff = (size_t)(B * i + bi) * a.ld;
                E zv[EPT], yv[EPT];
                if (a.has_z) ld_rw<S, NP, FULL>(zv, z + roff, base, g, Gp, P);
                else {
#pragma unroll
                    for (int e = 0; e < EPT; e++) zv[e] = S::to(S::zero());
                }
#pragma unroll
                for (int e = 0; e < EPT; e++) yv[e] = S::fin(acc[bi][e], a.two != 0, a.has_z != 0, zv[e]);
                st<S, NP, FULL>(y + roff, yv, base, g, Gp, P);
                if (a.want_dots || a.xi_mode == 1) {
                    E xo[EPT];
                    ld_nc<S, NP, FULL>(xo, x + roff, base, g, Gp, P);
                    if (a.want_dots) {
#pragma unroll
                        for (int e = 0; e < EPT; e++) { S::rd_nrm(rxx, xo[e]); S::rd_re(ryx, yv[e], xo[e]); }
                    }
                    if (a.xi_mode == 1) {
                        E xv2[EPT];
#pragma unroll
                        for (int e = 0; e < EPT; e++) {
                            typename S::Acc t2 = S::zero();
                            S::axpy(t2, c0, xo[e]);
                            S::axpy(t2, c1, yv[e]);
                            xv2[e] = S::to(t2);
                        }
                        st<S, NP, FULL>(xi + roff, xv2, base, g, Gp, P);
                    }
                }
                if (a.xi_mode == 2) {
                    E xv2[EPT];
                    ld_rw<S, NP, FULL>(xv2, xi + roff, base, g, Gp, P);
#pragma unroll
                    for (int e = 0; e < EPT; e++) {
                        typename S::Acc t2 = S::from(xv2[e]);
                        S::axpy(t2, c1, yv[e]);
                        xv2[e] = S::to(t2);
                    }
                    st<S, NP, FULL>(xi + roff, xv2, base, g, Gp, P);
                }
            }
            if (a.want_dots) { S::dot_add(dxx, rxx); S::dot_add(dyx, ryx); }
        }
    }
    if (a.want_dots) {
        block_reduce2<S>(dxx, dyx);
        if (threadIdx.x == 0) {
            a.partials[2 * blockIdx.x + 0] = S::dot_get(dxx);
            a.partials[2 * blockIdx.x + 1] = S::dot_get(dyx);
        }
    }
}

// Transposed reduction of V = 2^k values over the Gp lanes of a row group: at each of
// the first min(k, log2 Gp) levels a lane keeps one half of its values and adds the
// partner's copy of that half, so the live values halve while the reduction proceeds;
// the remaining levels are plain butterflies. On return v[0..count) holds the complete
// sums of values [first, first + count), and `writer` marks the one lane (of those
// holding the same values) that stores them. The lane that stores a value depends
// only on g, so successive chunks update each D entry from the same thread.
struct Owner {
    int first, count;   // values [first, first + count) of the V end up in this lane
    bool writer;        // the lane that stores them
};
template <int V>
__device__ __forceinline__ Owner transposed_owner(int Gp, int g) {
    int off = Gp >> 1, sel = 0, cur = V;
#pragma unroll
    for (int h = V >> 1; h >= 1; h >>= 1) {
        if (off > 0) {
            sel = (sel << 1) | ((g & off) != 0 ? 1 : 0);
            cur = h;
            off >>= 1;
        }
    }
    const int span = Gp / (V / cur);   // lanes holding the same values
    return Owner{sel * cur, cur, (g & (span - 1)) == 0};
}
template <class S, int V>
__device__ __forceinline__ void group_sum_transposed(typename S::OAcc (&v)[V], int Gp, int g) {
    int off = Gp >> 1, cur = V;
#pragma unroll
    for (int h = V >> 1; h >= 1; h >>= 1) {
        if (off > 0) {
            const bool up = (g & off) != 0;
#pragma unroll
            for (int i = 0; i < h; i++) {
                const typename S::OAcc send = up ? v[i] : v[i + h];
                const typename S::OAcc keep = up ? v[i + h] : v[i];
                v[i] = S::oa_add(keep, S::oa_shfl(send, off));
            }
            cur = h;
            off >>= 1;
        }
    }
    // lanes left over after the transposed levels: those levels ran all log2(V) times, so one
    // value per lane remains (cur == 1) and plain butterflies finish it
    (void)cur;
    for (; off > 0; off >>= 1) v[0] = S::oa_add(v[0], S::oa_shfl(v[0], off));
}

// Early read of the first D entry a writer lane updates for block k (8 bytes per real:
// a double, or a float-float pair for FP32/DS systems), issued before the block's
// gathers so that the read-modify-write does not wait a memory round trip at the end.
template <class S, int B>
__device__ __forceinline__ double2 d_prefetch(const double* Dacc, size_t k, const Owner& o, bool on) {
    double2 v = make_double2(0.0, 0.0);
    if (on) {
        const size_t q = (k * B * B + o.first) * (S::CPLX ? 2 : 1);
        if (S::CPLX) v = *reinterpret_cast<const double2*>(Dacc + q);
        else v.x = Dacc[q];
    }
    return v;
}
__device__ __forceinline__ float2 bits_float2(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return make_float2(__int_as_float((int)(unsigned)(u & 0xffffffffull)), __int_as_float((int)(unsigned)(u >> 32)));
}

// Add a block's reduced D values (the entries [o.first, o.first + o.count) held by this lane)
// to Dacc[k]; `pre` is the d_prefetch of the lane's first entry. FP64 systems accumulate in
// double; FP32 and DS systems keep the accumulator as float-float pairs (same 8 bytes
// per real) on the FP32 pipe and convert it to double once at the end (k_ds_to_double).
template <class S, int B>
__device__ __forceinline__ void d_write(const typename S::OAcc (&of)[B * B], bool has, size_t k, double scale,
                                        float2 scale_ds, double* Dacc, const Owner& o, double2 pre) {
    if (has && o.writer) {
#pragma unroll
        for (int t = 0; t < B * B; t++) {
            if (t < o.count) {
                const size_t q = (k * B * B + o.first + t) * (S::CPLX ? 2 : 1);
                if constexpr (S::DACC_DS) {
                    float2* D2 = reinterpret_cast<float2*>(Dacc);
#pragma unroll
                    for (int comp = 0; comp < (S::CPLX ? 2 : 1); comp++) {
                        float2 cur = t == 0 ? bits_float2(comp ? pre.y : pre.x) : D2[q + comp];
                        ds_mac(cur, scale_ds, S::oa_ds(of[t], comp));
                        D2[q + comp] = ds_norm(cur);
                    }
                } else {
                    const double2 v = S::oa_get(of[t]);
                    const double re = t == 0 ? pre.x : Dacc[q];
                    Dacc[q] = re + scale * v.x;
                    if (S::CPLX) {
                        const double im = t == 0 ? pre.y : Dacc[q + 1];
                        Dacc[q + 1] = im + scale * v.y;
                    }
                }
            }
        }
    }
}

// Reduce a block's per-lane D partials over the row group and add them to Dacc[k].
template <class S, int B>
__device__ __forceinline__ void flush_block(typename S::OAcc (&of)[B * B], int Gp, int g, bool has, size_t k,
                                            double scale, float2 scale_ds, double* Dacc, const Owner& o, double2 pre) {
    group_sum_transposed<S, B * B>(of, Gp, g);
    d_write<S, B>(of, has, k, scale, scale_ds, Dacc, o, pre);
}

// Float-float accumulator -> double, in place (both are 8 bytes per real).
static __global__ void k_ds_to_double(double* D, long long n_reals) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n_reals; q += (long long)gridDim.x * blockDim.x) {
        const float2 v = reinterpret_cast<const float2*>(D)[q];
        D[q] = (double)v.x + (double)v.y;
    }
}

// ---------------------------------------------------------------------------------
// Adjoint (reverse-mode) step of autodiff_matrix, both recursions in one pass:
//   alpha_{m-1} = 2 Hs alpha_m - alpha_{m+1}
//   beta_m      = 2 Hs beta_{m+1} - beta_{m+2} + cA alpha_m + cAp alpha_{m+1} + cAn alpha_{m-1}
// and, when Dacc != null (D's pattern is H's pattern), the outer-product epilogue
//   D_k += dscale * sum_s alpha_m[b i + bi, s] conj(beta_{m+1}[b j + bj, s])
// reusing the gathered beta_{m+1} rows of block k = (i, j).
// ---------------------------------------------------------------------------------
// kAdjointCtas: light configurations (kLightStep) are held to 64 registers, 4 CTAs per SM: on 64 square
// lattices (b=1, S=32, FP32, 7.4M blocks) a reverse step took 0.32 ms against 0.53 ms at the
// 96 registers (2 CTAs) the compiler picks otherwise; 3 and 5 CTAs measured 0.38 and 0.36 ms.
template <class S, int B, int NP, bool FULL = false>
__global__ void __launch_bounds__(kThreads, kAdjointCtas<S, B, NP>) k_adjoint_step(AdjArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    constexpr int EPT = NP * S::EPP;
    extern __shared__ __align__(16) unsigned char smem[];
    H* s_h = reinterpret_cast<H*>(smem);
    unsigned* s_col = reinterpret_cast<unsigned*>(smem + sizeof(H) * B * B * (size_t)a.stage_cap);

    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const int Gp = sd.Gp > 0 ? sd.Gp : a.Gp, P = sd.P > 0 ? sd.P : a.P, W = Gp * NP;
    const int nch = (P + W - 1) / W;
    const long long items = (long long)sd.n_b * Gp;
    const E* A = reinterpret_cast<const E*>(a.A);
    E* Ap = reinterpret_cast<E*>(a.Ap);
    const E* Bv = reinterpret_cast<const E*>(a.Bv);
    E* Bp = reinterpret_cast<E*>(a.Bp);
    const H* hval = reinterpret_cast<const H*>(a.hval);
    const typename S::Coef cA = S::coef(a.coef[sidx * a.cstride + 0]);
    const typename S::Coef cAp = S::coef(a.coef[sidx * a.cstride + 1]);
    const typename S::Coef cAn = S::coef(a.coef[sidx * a.cstride + 2]);
    const bool fuse = a.Dacc != nullptr;
    const float2 dscale_ds = ds_from_double(a.dscale);
    const Owner own = transposed_owner<B * B>(Gp, (int)(threadIdx.x % Gp));   // Gp divides kThreads

    for (long long t0 = (long long)lc * kThreads; t0 < items; t0 += (long long)sd.ctas * kThreads) {
        const Tile tl = tile_range(a.row_ptr, sd, t0, items, Gp, a.stage_cap);
        if (tl.staged) {
            __syncthreads();
            stage_h<S, B>(s_col, s_h, a.colc, hval, tl.k_lo, tl.nk);
            __syncthreads();
        }
        const long long t = t0 + threadIdx.x;
        const bool active = t < items;
        const int il = active ? (int)(t / Gp) : 0;
        const int g = active ? (int)(t - (long long)il * Gp) : (int)(threadIdx.x % Gp);
        const int i = sd.row_base + il;
        const int kb = active ? a.row_ptr[i] : 0;
        const int ke = active ? a.row_ptr[i + 1] : 0;
        // With the epilogue every lane of the warp walks the longest row of the warp so
        // that the group reductions see all 32 lanes; missing blocks contribute zero.
        int nmax = ke - kb;
        if (fuse) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, off));
        } else if (!active) {
            continue;
        }
        for (int c = 0; c < nch; c++) {
            const int base = c * W;
            E Ai[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++) {
                if (active) ld_nc<S, NP, FULL>(Ai[bi], A + (size_t)(B * i + bi) * a.ld, base, g, Gp, P);
                else {
#pragma unroll
                    for (int e = 0; e < EPT; e++) Ai[bi][e] = S::to(S::zero());
                }
            }
            typename S::Acc accA[B][EPT], accB[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++)
#pragma unroll
                for (int e = 0; e < EPT; e++) { accA[bi][e] = S::zero(); accB[bi][e] = S::zero(); }

            for (int kk = 0; kk < nmax; kk++) {
                const int k = kb + kk;
                const bool has = kk < ke - kb;
                unsigned cc = 0;
                const H* hk = hval;
                if (has) {
                    cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                    hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
                }
                const int j = (int)(cc & kColMask);
                const double2 dpre = d_prefetch<S, B>(a.Dacc, (size_t)k, own, fuse && has && own.writer);
                typename S::OAcc of[B * B];
#pragma unroll
                for (int q = 0; q < B * B; q++) of[q] = S::oa_zero();
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E av[EPT], bv[EPT];
                    if (has) {
                        ld_nc<S, NP, FULL>(av, A + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                        ld_nc<S, NP, FULL>(bv, Bv + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                        mac_block<S, B, NP>(accA, cc >> 30, hk, av, bj);
                        mac_block<S, B, NP>(accB, cc >> 30, hk, bv, bj);
                    } else {
#pragma unroll
                        for (int e = 0; e < EPT; e++) bv[e] = S::to(S::zero());
                    }
                    if (fuse) {
#pragma unroll
                        for (int bi = 0; bi < B; bi++) {   // each entry's first product starts it (of is zero): no add to zero
                            of[bj * B + bi] = S::oa_first(Ai[bi][0], bv[0]);
#pragma unroll
                            for (int e = 1; e < EPT; e++) S::oa_mac(of[bj * B + bi], Ai[bi][e], bv[e]);
                        }
                    }
                }
                if (fuse) flush_block<S, B>(of, Gp, g, has, (size_t)k, a.dscale, dscale_ds, a.Dacc, own, dpre);
            }
            if (active) {
#pragma unroll
                for (int bi = 0; bi < B; bi++) {
                    const size_t roff = (size_t)(B * i + bi) * a.ld;
                    E apv[EPT], bpv[EPT], an[EPT], bn[EPT];
                    ld_rw<S, NP, FULL>(apv, Ap + roff, base, g, Gp, P);
                    ld_rw<S, NP, FULL>(bpv, Bp + roff, base, g, Gp, P);
#pragma unroll
                    for (int e = 0; e < EPT; e++) {
                        an[e] = S::fin(accA[bi][e], true, true, apv[e]);
                        typename S::Acc tb = S::from(S::fin(accB[bi][e], true, true, bpv[e]));
                        S::axpy(tb, cA, Ai[bi][e]);
                        S::axpy(tb, cAp, apv[e]);
                        S::axpy(tb, cAn, an[e]);
                        bn[e] = S::to(tb);
                    }
                    st<S, NP, FULL>(Ap + roff, an, base, g, Gp, P);
                    st<S, NP, FULL>(Bp + roff, bn, base, g, Gp, P);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// FP64 reverse step for block rows served by a whole warp (Gp == 32, whole chunks, fused D
// epilogue, b=2 complex): k_adjoint_step's loads and arithmetic, with the D reduction arranged to
// spend fewer FP64-pipe additions, the resource that bounds the FP64 engine:
//  * a lane whose bit 4 is set (sw = 1) holds every block index swapped -- gathered rows
//    b j + (bj ^ sw), own rows b i + (bi ^ sw), accumulators and H entries permuted to match -- so
//    the first transposed level exchanges exactly the entries the partner keeps (no selects);
//  * the third level splits real and imaginary parts (lane bit 2), so 8 writer lanes each finish
//    one real of the block: 9 DADDs and one DFMA per block and chunk instead of 12 and two;
//  * lane offsets are compile-time and every lane of the warp walks the same row (no per-block
//    row test, no zero fill, no warp-wide maximum of the row lengths).
// Results equal k_adjoint_step's up to the order of the two bj terms of a general block in the
// swapped lanes (rounding), and the reduction adds the same partials in the same pairs.
// ---------------------------------------------------------------------------------
template <class S, int NP>
__global__ void __launch_bounds__(kThreads, 2) k_adjoint_step_warp(AdjArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    typedef typename S::OAcc OAcc;
    constexpr int B = 2;
    constexpr int G = 32;
    constexpr int EPT = NP * S::EPP;
    static_assert(S::CPLX && S::PREC == 0, "FP64 complex systems");
    extern __shared__ __align__(16) unsigned char smem[];
    H* s_h = reinterpret_cast<H*>(smem);
    unsigned* s_col = reinterpret_cast<unsigned*>(smem + sizeof(H) * B * B * (size_t)a.stage_cap);

    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const int P = sd.P > 0 ? sd.P : a.P, W = G * NP;
    const int nch = P / W;
    const long long items = (long long)sd.n_b * G;
    const E* A = reinterpret_cast<const E*>(a.A);
    E* Ap = reinterpret_cast<E*>(a.Ap);
    const E* Bv = reinterpret_cast<const E*>(a.Bv);
    E* Bp = reinterpret_cast<E*>(a.Bp);
    const H* hval = reinterpret_cast<const H*>(a.hval);
    const typename S::Coef cA = S::coef(a.coef[sidx * a.cstride + 0]);
    const typename S::Coef cAp = S::coef(a.coef[sidx * a.cstride + 1]);
    const typename S::Coef cAn = S::coef(a.coef[sidx * a.cstride + 2]);
    const int lane = threadIdx.x & 31;
    const int sw = (lane >> 4) & 1;                       // block-index swap of this lane
    const int hx = sw * 3;                                // H entry (bi, bj) -> (bi ^ sw, bj ^ sw)
    const bool im = (lane >> 2) & 1;                      // the part this lane finishes
    const int ent = sw * 2 + ((lane >> 3) & 1);           // the D entry (bj * 2 + bi) it finishes
    const bool writer = (lane & 3) == 0;

    for (long long t0 = (long long)lc * kThreads; t0 < items; t0 += (long long)sd.ctas * kThreads) {
        const Tile tl = tile_range(a.row_ptr, sd, t0, items, G, a.stage_cap);
        if (tl.staged) {
            __syncthreads();
            stage_h<S, B>(s_col, s_h, a.colc, hval, tl.k_lo, tl.nk);
            __syncthreads();
        }
        const long long t = t0 + threadIdx.x;
        if (t >= items) continue;   // items is a multiple of 32: whole warps leave together
        const int i = sd.row_base + (int)(t >> 5);
        const int kb = a.row_ptr[i], ke = a.row_ptr[i + 1];
        for (int c = 0; c < nch; c++) {
            const int base = c * W;
            E Ai[B][EPT];
#pragma unroll
            for (int r = 0; r < B; r++) ld_nc<S, NP, true>(Ai[r], A + (size_t)(B * i + (r ^ sw)) * a.ld, base, lane, G, P);
            typename S::Acc accA[B][EPT], accB[B][EPT];
#pragma unroll
            for (int r = 0; r < B; r++)
#pragma unroll
                for (int e = 0; e < EPT; e++) { accA[r][e] = S::zero(); accB[r][e] = S::zero(); }
            for (int k = kb; k < ke; k++) {
                const unsigned cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                const H* hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
                const int j = (int)(cc & kColMask);
                const size_t dq = ((size_t)k * B * B + ent) * 2 + (im ? 1 : 0);
                const double dpre = writer ? a.Dacc[dq] : 0.0;   // read early: used after the block's work
                OAcc of[B * B];
#pragma unroll
                for (int q = 0; q < B * B; q++) of[q] = S::oa_zero();
                const bool ident = (cc >> 30) == 2u;
#pragma unroll
                for (int rj = 0; rj < B; rj++) {
                    E av[EPT], bv[EPT];
                    ld_nc<S, NP, true>(av, A + (size_t)(B * j + (rj ^ sw)) * a.ld, base, lane, G, P);
                    ld_nc<S, NP, true>(bv, Bv + (size_t)(B * j + (rj ^ sw)) * a.ld, base, lane, G, P);
                    if (ident) {   // real multiple of the identity: H(0,0) = H(1,1)
                        const typename S::Hr h = S::hreal(hk[0]);
#pragma unroll
                        for (int e = 0; e < EPT; e++) { S::mac_re(accA[rj][e], h, av[e]); S::mac_re(accB[rj][e], h, bv[e]); }
                    } else if ((cc >> 30) == 1u) {   // real entries
#pragma unroll
                        for (int r = 0; r < B; r++) {
                            const typename S::Hr h = S::hreal(hk[(rj * B + r) ^ hx]);
#pragma unroll
                            for (int e = 0; e < EPT; e++) { S::mac_re(accA[r][e], h, av[e]); S::mac_re(accB[r][e], h, bv[e]); }
                        }
                    } else {
#pragma unroll
                        for (int r = 0; r < B; r++) {
                            const H h = hk[(rj * B + r) ^ hx];
#pragma unroll
                            for (int e = 0; e < EPT; e++) { S::mac(accA[r][e], h, av[e]); S::mac(accB[r][e], h, bv[e]); }
                        }
                    }
#pragma unroll
                    for (int r = 0; r < B; r++) {   // each entry's first product starts it (of is zero): no add to zero
                        of[rj * B + r] = S::oa_first(Ai[r][0], bv[0]);
#pragma unroll
                        for (int e = 1; e < EPT; e++) S::oa_mac(of[rj * B + r], Ai[r][e], bv[e]);
                    }
                }
                // of[rj * B + r] holds D entry (bj = rj ^ sw, bi = r ^ sw); lane ^ 16 has the other swap
                of[0] = S::oa_add(of[0], S::oa_shfl(of[3], 16));
                of[1] = S::oa_add(of[1], S::oa_shfl(of[2], 16));
                const bool k0 = ((lane >> 3) & 1) == sw;   // lane bit 3 picks bi
                const OAcc keep = k0 ? of[0] : of[1];
                const OAcc send = k0 ? of[1] : of[0];
                const OAcc e2 = S::oa_add(keep, S::oa_shfl(send, 8));
                const double kp = im ? e2.y : e2.x;
                const double sd2 = im ? e2.x : e2.y;
                double v = kp + __shfl_xor_sync(0xffffffffu, sd2, 4);
                v += __shfl_xor_sync(0xffffffffu, v, 2);
                v += __shfl_xor_sync(0xffffffffu, v, 1);
                if (writer) a.Dacc[dq] = dpre + a.dscale * v;
            }
#pragma unroll
            for (int r = 0; r < B; r++) {
                const size_t roff = (size_t)(B * i + (r ^ sw)) * a.ld;
                E apv[EPT], bpv[EPT], an[EPT], bn[EPT];
                ld_rw<S, NP, true>(apv, Ap + roff, base, lane, G, P);
                ld_rw<S, NP, true>(bpv, Bp + roff, base, lane, G, P);
#pragma unroll
                for (int e = 0; e < EPT; e++) {
                    an[e] = S::fin(accA[r][e], true, true, apv[e]);
                    typename S::Acc tb = S::from(S::fin(accB[r][e], true, true, bpv[e]));
                    S::axpy(tb, cA, Ai[r][e]);
                    S::axpy(tb, cAp, apv[e]);
                    S::axpy(tb, cAn, an[e]);
                    bn[e] = S::to(tb);
                }
                st<S, NP, true>(Ap + roff, an, base, lane, G, P);
                st<S, NP, true>(Bp + roff, bn, base, lane, G, P);
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// The same reverse step in two passes over the row's blocks, to hold fewer values in
// registers at a time: pass 1 gathers alpha_m and writes alpha_{m-1} (keeping alpha_{m+1}
// and alpha_{m-1} of the thread's own rows in shared memory, which only that thread
// touches); pass 2 gathers beta_{m+1}, runs the D epilogue and writes beta_m from the kept
// values. Each gathered row is still read once per block; the kept vectors cost
// 2 x kThreads x B x NP packets of shared memory after the H stage.
// ---------------------------------------------------------------------------------
__host__ __device__ inline size_t adj_stage_bytes(int stage_cap, size_t h_block_bytes) {
    return ((h_block_bytes + sizeof(unsigned)) * (size_t)stage_cap + 15) / 16 * 16;
}
template <class S, int B, int NP, bool FULL = false>
__global__ void __launch_bounds__(kThreads, kAdjointSplitCtas<S, B, NP>) k_adjoint_split(AdjArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    constexpr int EPT = NP * S::EPP;
    extern __shared__ __align__(16) unsigned char smem[];
    H* s_h = reinterpret_cast<H*>(smem);
    unsigned* s_col = reinterpret_cast<unsigned*>(smem + sizeof(H) * B * B * (size_t)a.stage_cap);
    E* s_ap = reinterpret_cast<E*>(smem + adj_stage_bytes(a.stage_cap, sizeof(H) * B * B));   // alpha_{m+1}
    E* s_an = s_ap + (size_t)kThreads * B * EPT;                                               // alpha_{m-1}

    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const int Gp = sd.Gp > 0 ? sd.Gp : a.Gp, P = sd.P > 0 ? sd.P : a.P, W = Gp * NP;
    const int nch = (P + W - 1) / W;
    const long long items = (long long)sd.n_b * Gp;
    const E* A = reinterpret_cast<const E*>(a.A);
    E* Ap = reinterpret_cast<E*>(a.Ap);
    const E* Bv = reinterpret_cast<const E*>(a.Bv);
    E* Bp = reinterpret_cast<E*>(a.Bp);
    const H* hval = reinterpret_cast<const H*>(a.hval);
    const typename S::Coef cA = S::coef(a.coef[sidx * a.cstride + 0]);
    const typename S::Coef cAp = S::coef(a.coef[sidx * a.cstride + 1]);
    const typename S::Coef cAn = S::coef(a.coef[sidx * a.cstride + 2]);
    const bool fuse = a.Dacc != nullptr;
    const float2 dscale_ds = ds_from_double(a.dscale);
    const Owner own = transposed_owner<B * B>(Gp, (int)(threadIdx.x % Gp));   // Gp divides kThreads

    for (long long t0 = (long long)lc * kThreads; t0 < items; t0 += (long long)sd.ctas * kThreads) {
        const Tile tl = tile_range(a.row_ptr, sd, t0, items, Gp, a.stage_cap);
        if (tl.staged) {
            __syncthreads();
            stage_h<S, B>(s_col, s_h, a.colc, hval, tl.k_lo, tl.nk);
            __syncthreads();
        }
        const long long t = t0 + threadIdx.x;
        const bool active = t < items;
        const int il = active ? (int)(t / Gp) : 0;
        const int g = active ? (int)(t - (long long)il * Gp) : (int)(threadIdx.x % Gp);
        const int i = sd.row_base + il;
        const int kb = active ? a.row_ptr[i] : 0;
        const int ke = active ? a.row_ptr[i + 1] : 0;
        int nmax = ke - kb;
        if (fuse) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, off));
        } else if (!active) {
            continue;
        }
        for (int c = 0; c < nch; c++) {
            const int base = c * W;
            // pass 1: alpha_{m-1} = 2 Hs alpha_m - alpha_{m+1}
            if (active) {
                typename S::Acc accA[B][EPT];
#pragma unroll
                for (int bi = 0; bi < B; bi++)
#pragma unroll
                    for (int e = 0; e < EPT; e++) accA[bi][e] = S::zero();
#pragma unroll 1
                for (int k = kb; k < ke; k++) {
                    const unsigned cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                    const H* hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
                    const int j = (int)(cc & kColMask);
#pragma unroll
                    for (int bj = 0; bj < B; bj++) {
                        E av[EPT];
                        ld_nc<S, NP, FULL>(av, A + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                        mac_block<S, B, NP>(accA, cc >> 30, hk, av, bj);
                    }
                }
#pragma unroll
                for (int bi = 0; bi < B; bi++) {
                    const size_t roff = (size_t)(B * i + bi) * a.ld;
                    E apv[EPT], an[EPT];
                    ld_rw<S, NP, FULL>(apv, Ap + roff, base, g, Gp, P);
#pragma unroll
                    for (int e = 0; e < EPT; e++) {
                        an[e] = S::fin(accA[bi][e], true, true, apv[e]);
                        s_ap[(size_t)(bi * EPT + e) * kThreads + threadIdx.x] = apv[e];
                        s_an[(size_t)(bi * EPT + e) * kThreads + threadIdx.x] = an[e];
                    }
                    st<S, NP, FULL>(Ap + roff, an, base, g, Gp, P);
                }
            }
            // pass 2: beta_m = 2 Hs beta_{m+1} - beta_{m+2} + cA alpha_m + cAp alpha_{m+1} + cAn alpha_{m-1},
            // with D_k += dscale alpha_m[i] beta_{m+1}[j]^dagger on the gathered beta rows
            E Ai[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++) {
                if (active) ld_nc<S, NP, FULL>(Ai[bi], A + (size_t)(B * i + bi) * a.ld, base, g, Gp, P);
                else {
#pragma unroll
                    for (int e = 0; e < EPT; e++) Ai[bi][e] = S::to(S::zero());
                }
            }
            typename S::Acc accB[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++)
#pragma unroll
                for (int e = 0; e < EPT; e++) accB[bi][e] = S::zero();
            for (int kk = 0; kk < nmax; kk++) {
                const int k = kb + kk;
                const bool has = kk < ke - kb;
                unsigned cc = 0;
                const H* hk = hval;
                if (has) {
                    cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                    hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
                }
                const int j = (int)(cc & kColMask);
                const double2 dpre = d_prefetch<S, B>(a.Dacc, (size_t)k, own, fuse && has && own.writer);
                typename S::OAcc of[B * B];
#pragma unroll
                for (int q = 0; q < B * B; q++) of[q] = S::oa_zero();
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E bv[EPT];
                    if (has) {
                        ld_nc<S, NP, FULL>(bv, Bv + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                        mac_block<S, B, NP>(accB, cc >> 30, hk, bv, bj);
                    } else {
#pragma unroll
                        for (int e = 0; e < EPT; e++) bv[e] = S::to(S::zero());
                    }
                    if (fuse) {
#pragma unroll
                        for (int bi = 0; bi < B; bi++) {   // each entry's first product starts it (of is zero): no add to zero
                            of[bj * B + bi] = S::oa_first(Ai[bi][0], bv[0]);
#pragma unroll
                            for (int e = 1; e < EPT; e++) S::oa_mac(of[bj * B + bi], Ai[bi][e], bv[e]);
                        }
                    }
                }
                if (fuse) flush_block<S, B>(of, Gp, g, has, (size_t)k, a.dscale, dscale_ds, a.Dacc, own, dpre);
            }
            if (active) {
#pragma unroll
                for (int bi = 0; bi < B; bi++) {
                    const size_t roff = (size_t)(B * i + bi) * a.ld;
                    E bpv[EPT], bn[EPT];
                    ld_rw<S, NP, FULL>(bpv, Bp + roff, base, g, Gp, P);
#pragma unroll
                    for (int e = 0; e < EPT; e++) {
                        typename S::Acc tb = S::from(S::fin(accB[bi][e], true, true, bpv[e]));
                        S::axpy(tb, cA, Ai[bi][e]);
                        S::axpy(tb, cAp, s_ap[(size_t)(bi * EPT + e) * kThreads + threadIdx.x]);
                        S::axpy(tb, cAn, s_an[(size_t)(bi * EPT + e) * kThreads + threadIdx.x]);
                        bn[e] = S::to(tb);
                    }
                    st<S, NP, FULL>(Bp + roff, bn, base, g, Gp, P);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Sparsity-restricted outer product on D's pattern (the reference's
// outer_product_kernel role, src/outer_product.cu:38-60, re-designed):
//   D_k(bi,bj) += alpha sum_s ( A[b i+bi, s] conj(B[b j+bj, s])
//                             [+ B[b i+bi, s] conj(A[b j+bj, s])] )
// One row group (Gp lanes) per block row of D; own rows held in registers per
// column chunk, partner rows gathered once per block, transposed reduction over
// the lanes, FP64 accumulation into Dacc.
// ---------------------------------------------------------------------------------
template <class S, int B, int NP, bool FULL = false>
__global__ void __launch_bounds__(kThreads, kOuterCtas<S, B, NP>) k_outer(OuterArgs a) {
    typedef typename S::E E;
    constexpr int EPT = NP * S::EPP;
    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const int Gp = sd.Gp > 0 ? sd.Gp : a.Gp, P = sd.P > 0 ? sd.P : a.P, W = Gp * NP;
    const int nch = (P + W - 1) / W;
    const long long items = (long long)sd.n_b * Gp;
    const E* A = reinterpret_cast<const E*>(a.A);
    const E* Bv = reinterpret_cast<const E*>(a.Bv);
    const bool two_terms = a.two_terms != 0;
    const float2 alpha_ds = ds_from_double(a.alpha);
    const Owner own = transposed_owner<B * B>(Gp, (int)(threadIdx.x % Gp));   // Gp divides kThreads

    for (long long t0 = (long long)lc * kThreads; t0 < items; t0 += (long long)sd.ctas * kThreads) {
        const long long t = t0 + threadIdx.x;
        const bool active = t < items;
        const int il = active ? (int)(t / Gp) : 0;
        const int g = active ? (int)(t - (long long)il * Gp) : (int)(threadIdx.x % Gp);
        const int i = sd.row_base + il;
        const int kb = active ? a.row_ptr[i] : 0;
        const int ke = active ? a.row_ptr[i + 1] : 0;
        int nmax = ke - kb;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, off));
        for (int c = 0; c < nch; c++) {
            const int base = c * W;
            E Ai[B][EPT], Bi[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++) {
                if (active) {
                    ld_nc<S, NP, FULL>(Ai[bi], A + (size_t)(B * i + bi) * a.ld, base, g, Gp, P);
                    if (two_terms) ld_nc<S, NP, FULL>(Bi[bi], Bv + (size_t)(B * i + bi) * a.ld, base, g, Gp, P);
                    else {
#pragma unroll
                        for (int e = 0; e < EPT; e++) Bi[bi][e] = S::to(S::zero());
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < EPT; e++) { Ai[bi][e] = S::to(S::zero()); Bi[bi][e] = Ai[bi][e]; }
                }
            }
            unsigned cc_next = ke > kb ? __ldg(a.colc + kb) : 0u;   // column index one block ahead
            for (int kk = 0; kk < nmax; kk++) {
                const int k = kb + kk;
                const bool has = kk < ke - kb;
                const int j = has ? (int)(cc_next & kColMask) : 0;
                cc_next = kk + 1 < ke - kb ? __ldg(a.colc + k + 1) : 0u;
                const double2 dpre = d_prefetch<S, B>(a.Dacc, (size_t)k, own, has && own.writer);
                typename S::OAcc of[B * B];
#pragma unroll
                for (int q = 0; q < B * B; q++) of[q] = S::oa_zero();
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E bv[EPT], av[EPT];
                    if (has) {
                        ld_nc<S, NP, FULL>(bv, Bv + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                        if (two_terms) ld_nc<S, NP, FULL>(av, A + (size_t)(B * j + bj) * a.ld, base, g, Gp, P);
                        else {
#pragma unroll
                            for (int e = 0; e < EPT; e++) av[e] = S::to(S::zero());
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < EPT; e++) { bv[e] = S::to(S::zero()); av[e] = bv[e]; }
                    }
#pragma unroll
                    for (int bi = 0; bi < B; bi++)
#pragma unroll
                        for (int e = 0; e < EPT; e++) {
                            S::oa_mac(of[bj * B + bi], Ai[bi][e], bv[e]);
                            if (two_terms) S::oa_mac(of[bj * B + bi], Bi[bi][e], av[e]);
                        }
                }
                flush_block<S, B>(of, Gp, g, has, (size_t)k, a.alpha, alpha_ds, a.Dacc, own, dpre);
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------------

// Column-major double (or interleaved complex double) n x ncols block -> row-major vector
// columns [c0, c0+ncols) in system S. src is device memory or host memory the GPU can read
// (pinned, or any host memory on systems with pageable-memory access). 32 x 32 tiles are
// transposed through shared memory so that both the column reads and the row writes are
// contiguous across a warp (launched with 32 x 8 threads).
constexpr int kTransposeTile = 32;
// Sparse probe block -> row-major engine vector (already zeroed): row i holds k entries,
// R[i, cols[i k + q]] += vals[i k + q] (complex: interleaved (re, im) pairs). One thread per
// row, so repeated columns of a row add up without races. Colour (correlated) probes have
// one entry per row and realisation: ~20 bytes per row instead of S elements.
template <class S>
__global__ void k_expand_sparse(const int* cols, const double* vals, long long n, int k, long long ld,
                                typename S::E* dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        for (int q = 0; q < k; q++) {
            const long long t = i * k + q;
            typename S::E* p = dst + i * ld + cols[t];
            const double2 add = S::CPLX ? make_double2(vals[2 * t], vals[2 * t + 1]) : make_double2(vals[t], 0.0);
            const double2 cur = S::to_double2(*p);
            *p = S::from_double2(make_double2(cur.x + add.x, cur.y + add.y));
        }
    }
}

template <class S>
__global__ void k_load_colmajor(const double* src, long long n, int ncols, int c0, long long ld, typename S::E* dst) {
    constexpr int T = kTransposeTile;
    __shared__ double2 tile[T][T + 1];
    const long long ntr = (n + T - 1) / T;
    const int ntc = (ncols + T - 1) / T;
    for (long long tt = blockIdx.x; tt < ntr * ntc; tt += gridDim.x) {
        const long long r0 = (tt / ntc) * T;
        const int cc0 = (int)(tt % ntc) * T;
        for (int j = threadIdx.y; j < T; j += blockDim.y) {
            const int c = cc0 + j;
            const long long r = r0 + threadIdx.x;
            if (c < ncols && r < n) {
                const long long sidx = (long long)c * n + r;
                tile[j][threadIdx.x] = S::CPLX ? make_double2(src[2 * sidx], src[2 * sidx + 1]) : make_double2(src[sidx], 0.0);
            }
        }
        __syncthreads();
        for (int j = threadIdx.y; j < T; j += blockDim.y) {
            const long long r = r0 + j;
            const int c = cc0 + threadIdx.x;
            if (c < ncols && r < n) dst[r * ld + c0 + c] = S::from_double2(tile[threadIdx.x][j]);
        }
        __syncthreads();
    }
}

// Columns [c0, c0 + w) of a row-major vector -> a dense row-major n x w panel of doubles (real) or
// (re, im) double pairs (complex), converted from system S: one column of the GEMM that forms
// the second-order moments.
template <class S>
__global__ void k_export_panel(const typename S::E* src, long long n, long long ld, long long c0, int w, double* dst) {
    const long long total = n * (long long)w;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const long long r = q / w;
        const int c = (int)(q - r * w);
        const double2 v = S::to_double2(src[r * ld + c0 + c]);
        if (S::CPLX) reinterpret_cast<double2*>(dst)[q] = v;
        else dst[q] = v.x;
    }
}

// y[r, :] = f[row_sys[block row of r]] * x[r, :] over rows r < n_rows of row-major n x ld
// vectors (the batched engine's per-system factors; row_sys maps a block row of b rows to its system).
template <class S>
__global__ void k_scale_rows(const typename S::E* x, typename S::E* y, long long n_rows, long long ld, int b,
                             const int* row_sys, const double* f) {
    const long long total = n_rows * ld;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x)
        y[q] = S::scale(S::coef(f[row_sys[(q / ld) / b]]), x[q]);
}

// Row-major device vector -> column-major double host layout (for reading back R / state).
template <class S>
__global__ void k_store_colmajor(const typename S::E* src, long long n, int ncols, long long ld, double* dst) {
    const long long total = n * (long long)ncols;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const long long r = q / ncols;
        const int c = (int)(q - r * ncols);
        const double2 v = S::to_double2(src[r * ld + c]);
        const long long didx = (long long)c * n + r;
        if (S::CPLX) { dst[2 * didx] = v.x; dst[2 * didx + 1] = v.y; }
        else dst[didx] = v.x;
    }
}

// y = c * x over the whole vector (n_elems elements); the factor is *c_dev when given
// (so a replayed CUDA graph picks up new values), else c.
template <class S>
__global__ void k_scale(const typename S::E* x, typename S::E* y, long long n_elems, double c, const double* c_dev) {
    const typename S::Coef cc = S::coef(c_dev ? *c_dev : c);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n_elems; q += (long long)gridDim.x * blockDim.x)
        y[q] = S::scale(cc, x[q]);
}

// dst block q <- src block idx[q] (per doubles each): D of the prepared patterns back to the
// caller's block order, in one pass before the copy to the host.
static __global__ void k_gather_blocks(const double* src, const int* idx, long long n_out, int per, double* dst) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n_out * per; q += (long long)gridDim.x * blockDim.x) {
        const long long blk = q / per;
        dst[q] = src[(size_t)idx[blk] * per + (q - blk * per)];
    }
}

// D <- (D + D^T-pair^dagger)/2 blockwise, then * scale (row_scale[i] per block row when given) (SpMatBsr::symmetrize and
// scale, src/spmat.cpp:171-198, done on the device). pair[k] is the block index of
// (j, i) for k = (i, j). Each unordered pair is handled by the block with i >= j.
static __global__ void k_symmetrize_scale(double* D, const int* rows, const int* cols, const int* pair, int nnzb, int b,
                                          int cplx, double scale_all, const double* row_scale) {
    const int bb = b * b;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)nnzb * bb;
         q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q / bb);
        const int e = (int)(q - (long long)k * bb);
        const int bj = e / b, bi = e - (e / b) * b;
        const int i = rows[k], j = cols[k];
        if (i < j) continue;
        const int kt = pair[k];
        const size_t q1 = (size_t)k * bb + bj * b + bi;    // (bi, bj) of block k
        const size_t q2 = (size_t)kt * bb + bi * b + bj;   // (bj, bi) of block kt
        if (i == j && bi < bj) continue;                   // diagonal block: each entry pair once
        const double scale = row_scale ? row_scale[i] : scale_all;   // per block row (batched systems)
        if (cplx) {
            const double r1 = D[2 * q1], i1 = D[2 * q1 + 1], r2 = D[2 * q2], i2 = D[2 * q2 + 1];
            const double sr = (r1 + r2) / 2.0, si = (i1 - i2) / 2.0;
            D[2 * q1] = sr * scale; D[2 * q1 + 1] = si * scale;
            D[2 * q2] = sr * scale; D[2 * q2 + 1] = -si * scale;
        } else {
            const double s = (D[q1] + D[q2]) / 2.0;
            D[q1] = s * scale;
            D[q2] = s * scale;
        }
    }
}

}  // namespace fk
