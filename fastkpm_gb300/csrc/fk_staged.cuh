// fk_staged.cuh -- step and reverse-step kernels whose neighbour gathers go through
// shared memory, in two designs:
//
//  1. k_cheb_step_staged (FK_OPT_TMA, off by default): a whole tile's gathers staged
//     by TMA bulk / cp.async copies from per-tile column lists (below);
//  2. k_cheb_step_pipe / k_adjoint_pipe (FK_OPT_PIPE, the default for b=2 FP32 and
//     float-float and for the FP32 adjoint): every thread double-buffers its own
//     packets of the next block with 16-byte cp.async copies (end of this file).
//
// The plain kernels gather rows with per-thread loads and stall on their latency
// (long-scoreboard is their top stall; registers cap them at 16-24 warps/SM).
// In design 1 a tile of kThreads (row, lane) items is served from shared memory:
//   * the host lists, per tile, the distinct block columns its rows touch (own
//     rows included), sorted, and for every H block its slot in that list;
//   * per column chunk of W = Gp * NP packets, warp 0 issues one 1-D
//     cp.async.bulk copy per (distinct column, bj) row chunk into one of two
//     shared buffers, completing on that buffer's mbarrier (expect_tx bytes);
//   * while a chunk is computed from shared memory, the next chunk (of this or
//     the CTA's next tile) is already in flight.
// Every wait is bounded: after kWaitLimit polls the CTA records the failure in
// *err and stops (the host turns that into FK_ERR_TIMEOUT).
// All copies start on 16-byte boundaries and move multiples of 16 bytes.
#pragma once
#include "fk_kernels.cuh"

namespace fk {

struct StageTables {
    const int* tile_base;           // per system: global index of its first tile
    const int* uoff;                // [tiles + 1]: offsets into ucol
    const int* ucol;                // distinct global block columns of each tile, sorted
    const int* own;                 // [tiles]: slot of the tile's first own row
    const unsigned short* kslot;    // per H block: slot of its column in its tile's list
    int umax;                       // largest list
    int* err;                       // set to 1 by a CTA whose wait ran out
};

constexpr unsigned kWaitLimit = 1u << 26;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: true when the phase with this parity completed
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
    for (unsigned it = 0; it < kWaitLimit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16-byte asynchronous global -> shared copy (bypasses L1), grouped and waited by the hardware
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Shared-memory bytes the staged step kernel needs.
__host__ __device__ inline size_t staged_smem_bytes(int umax, int B, int W, int stage_cap, int hsize) {
    const size_t buf = (size_t)umax * B * W * 16;
    return 128 + 2 * buf + (size_t)stage_cap * ((size_t)B * B * hsize + 4 + 2) + 16;
}

// TMA = true: warp 0 issues one cp.async.bulk per row chunk, completion on an mbarrier.
// TMA = false: every thread issues 16-byte cp.async copies of its share of the unit's
// row chunks (commit/wait groups); no spin loop at all.
template <class S, int B, int NP, bool TMA>
__global__ void __launch_bounds__(kThreads, 2) k_cheb_step_staged(StepArgs a, StageTables tb) {
    typedef typename S::E E;
    typedef typename S::H H;
    constexpr int EPP = S::EPP;
    constexpr int EPT = NP * EPP;
    extern __shared__ __align__(16) unsigned char smem[];   // dynamic shared memory starts 16-byte aligned or better
    const int Gp = a.Gp, P = a.P, W = Gp * NP;   // (single-engine kernel: one system, the launch's P)
    const int nch = (P + W - 1) / W;
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(smem);
    __shared__ int s_fail;
    uint4* buf0 = reinterpret_cast<uint4*>(smem + 128);
    const size_t buf_packets = (size_t)tb.umax * B * W;
    H* s_h = reinterpret_cast<H*>(smem + 128 + 2 * buf_packets * 16);
    unsigned* s_col = reinterpret_cast<unsigned*>(s_h + (size_t)a.stage_cap * B * B);
    unsigned short* s_slot = reinterpret_cast<unsigned short*>(s_col + a.stage_cap);

    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const long long items = (long long)sd.n_b * Gp;
    const int tiles = (int)((items + kThreads - 1) / kThreads);
    const int my_tiles = lc < tiles ? (tiles - 1 - lc) / sd.ctas + 1 : 0;
    const int n_units = my_tiles * nch;
    const int tbase = tb.tile_base[sidx];
    const E* x = reinterpret_cast<const E*>(a.x);
    const E* z = reinterpret_cast<const E*>(a.z);
    E* y = reinterpret_cast<E*>(a.y);
    E* xi = reinterpret_cast<E*>(a.xi);
    const H* hval = reinterpret_cast<const H*>(a.hval);
    const typename S::Coef c0 = S::coef(a.xi_mode ? a.coef[sidx * a.cstride + 0] : 0.0);
    const typename S::Coef c1 = S::coef(a.xi_mode ? a.coef[sidx * a.cstride + 1] : 0.0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        if constexpr (TMA) {
            mbar_init(&mbar[0], 1);
            mbar_init(&mbar[1], 1);
            mbar_fence_init();
        }
        s_fail = 0;
    }
    __syncthreads();

    // put the row chunks of `unit` in flight into buffer unit & 1
    // (TMA: warp 0 only; cp.async: every thread, then one commit group per thread)
    auto issue = [&](int unit) {
        const int lt = lc + (unit / nch) * sd.ctas;
        const int c = unit % nch;
        const int gt = tbase + lt;
        const int u0 = tb.uoff[gt];
        const int nu = tb.uoff[gt + 1] - u0;
        const int pk = min(W, P - c * W);
        uint4* dstb = buf0 + (size_t)(unit & 1) * buf_packets;
        if constexpr (TMA) {
            const unsigned row_bytes = (unsigned)pk * 16u;
            // the generic-proxy reads of this buffer (two units ago, ordered by the CTA barrier)
            // must precede this lane's async-proxy writes into it
            fence_proxy_async_smem();
            if (lane == 0) mbar_expect_tx(&mbar[unit & 1], row_bytes * (unsigned)(nu * B));
            __syncwarp();
            for (int q = lane; q < nu * B; q += 32) {
                const int ui = q / B, bj = q - (q / B) * B;
                const int col = tb.ucol[u0 + ui];
                const E* src = x + (size_t)(B * col + bj) * a.ld + (size_t)c * W * EPP;
                bulk_g2s(dstb + (size_t)(ui * B + bj) * W, src, row_bytes, &mbar[unit & 1]);
            }
        } else {
            const int per_col = B * pk;   // packets of one distinct column in this chunk
            for (int q = threadIdx.x; q < nu * per_col; q += kThreads) {
                const int ui = q / per_col;
                const int rem = q - ui * per_col;
                const int bj = rem / pk, p = rem - (rem / pk) * pk;
                const int col = tb.ucol[u0 + ui];
                const E* src = x + (size_t)(B * col + bj) * a.ld + (size_t)(c * W + p) * EPP;
                cp_async16(dstb + (size_t)(ui * B + bj) * W + p, src);
            }
            cp_async_commit();
        }
    };

    typename S::Dot dxx = S::dot_zero(), dyx = S::dot_zero();
    if ((TMA ? warp == 0 : true) && n_units > 0) issue(0);
    int k_lo = 0;
    for (int unit = 0; unit < n_units; unit++) {
        const int lt = lc + (unit / nch) * sd.ctas;
        const int c = unit % nch;
        const long long t0 = (long long)lt * kThreads;
        const int r_lo = sd.row_base + (int)(t0 / Gp);
        if ((TMA ? warp == 0 : true) && unit + 1 < n_units) issue(unit + 1);
        if (c == 0) {
            // H blocks, their columns and their slots for this tile
            const long long t_last = min(t0 + kThreads, items) - 1;
            const int r_hi = sd.row_base + (int)(t_last / Gp);
            k_lo = a.row_ptr[r_lo];
            const int nk = a.row_ptr[r_hi + 1] - k_lo;
            for (int q = threadIdx.x; q < nk; q += blockDim.x) {
                s_col[q] = __ldg(a.colc + k_lo + q);
                s_slot[q] = __ldg(tb.kslot + k_lo + q);
            }
            for (int q = threadIdx.x; q < nk * B * B; q += blockDim.x) s_h[q] = hval[(size_t)k_lo * B * B + q];
        }
        if constexpr (TMA) {
            // wait for this unit's row chunks: thread 0 with a bound, then everyone acquires
            if (threadIdx.x == 0 && !mbar_wait_bounded(&mbar[unit & 1], (unsigned)(unit >> 1) & 1u)) s_fail = 1;
            __syncthreads();
            if (s_fail) {
                if (threadIdx.x == 0) {
                    atomicExch(tb.err, 1);
                    // the next unit's copies may be in flight: wait for them (bounded) before leaving
                    if (unit + 1 < n_units) mbar_wait_bounded(&mbar[(unit + 1) & 1], (unsigned)((unit + 1) >> 1) & 1u);
                }
                return;
            }
            mbar_wait_bounded(&mbar[unit & 1], (unsigned)(unit >> 1) & 1u);   // completed: returns at once
        } else {
            // this thread's copies of this unit are done once at most the next unit's group is pending
            if (unit + 1 < n_units) cp_async_wait<1>();
            else cp_async_wait<0>();
            __syncthreads();
        }
        const uint4* sb = buf0 + (size_t)(unit & 1) * buf_packets;
        const long long t = t0 + threadIdx.x;
        if (t < items) {
            const int il = (int)(t / Gp);
            const int g = (int)(t - (long long)il * Gp);
            const int i = sd.row_base + il;
            const int kb = a.row_ptr[i], ke = a.row_ptr[i + 1];
            const int base = c * W;
            typename S::Acc acc[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++)
#pragma unroll
                for (int e = 0; e < EPT; e++) acc[bi][e] = S::zero();
            for (int k = kb; k < ke; k++) {
                const int kk = k - k_lo;
                const unsigned cc = s_col[kk];
                const int slot = s_slot[kk];
                const H* hk = s_h + (size_t)kk * B * B;
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E xv[EPT];
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        Packet<E, EPP> pkt;
                        const int pk = g + Gp * q;
                        pkt.u = make_uint4(0u, 0u, 0u, 0u);
                        if (base + pk < P) pkt.u = sb[(size_t)(slot * B + bj) * W + pk];
#pragma unroll
                        for (int e = 0; e < EPP; e++) xv[q * EPP + e] = pkt.e[e];
                    }
                    mac_block<S, B, NP>(acc, cc >> 30, hk, xv, bj);
                }
            }
            const int own_slot = tb.own[tbase + lt] + (i - r_lo);
            typename S::RowDot rxx = S::rd_zero(), ryx = S::rd_zero();
#pragma unroll
            for (int bi = 0; bi < B; bi++) {
                const size_t roff = (size_t)(B * i + bi) * a.ld;
                E zv[EPT], yv[EPT], xo[EPT];
                if (a.has_z) ld_rw<S, NP>(zv, z + roff, base, g, Gp, P);
                else {
#pragma unroll
                    for (int e = 0; e < EPT; e++) zv[e] = S::to(S::zero());
                }
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    Packet<E, EPP> pkt;
                    const int pk = g + Gp * q;
                    pkt.u = make_uint4(0u, 0u, 0u, 0u);
                    if (base + pk < P) pkt.u = sb[(size_t)(own_slot * B + bi) * W + pk];
#pragma unroll
                    for (int e = 0; e < EPP; e++) xo[q * EPP + e] = pkt.e[e];
                }
#pragma unroll
                for (int e = 0; e < EPT; e++) yv[e] = S::fin(acc[bi][e], a.two != 0, a.has_z != 0, zv[e]);
                st<S, NP>(y + roff, yv, base, g, Gp, P);
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
                    st<S, NP>(xi + roff, xv2, base, g, Gp, P);
                } else if (a.xi_mode == 2) {
                    E xv2[EPT];
                    ld_rw<S, NP>(xv2, xi + roff, base, g, Gp, P);
#pragma unroll
                    for (int e = 0; e < EPT; e++) {
                        typename S::Acc t2 = S::from(xv2[e]);
                        S::axpy(t2, c1, yv[e]);
                        xv2[e] = S::to(t2);
                    }
                    st<S, NP>(xi + roff, xv2, base, g, Gp, P);
                }
            }
            if (a.want_dots) { S::dot_add(dxx, rxx); S::dot_add(dyx, ryx); }
        }
        __syncthreads();   // buffer unit & 1 and the H stage are free again
    }
    if (a.want_dots) {
        block_reduce2<S>(dxx, dyx);
        if (threadIdx.x == 0) {
            a.partials[2 * blockIdx.x + 0] = S::dot_get(dxx);
            a.partials[2 * blockIdx.x + 1] = S::dot_get(dyx);
        }
    }
}

// ---------------------------------------------------------------------------------
// Chebyshev step with each thread's gathers double-buffered in shared memory: while the
// multiply-adds of block k read its x packets from one buffer, 16-byte cp.async copies
// bring block k+1's packets into the other, so the next round trip overlaps this block's
// arithmetic without holding the packets in registers. Every thread copies and reads only
// its own slots (thread-minor layout: conflict-free 16-byte shared accesses), so the only
// synchronisation is cp.async.wait_group on the thread's own copies; no spin loop. Masked
// packets (a ragged last chunk) are never copied and read as zero.
// Shared memory: 2 buffers x B x NP packets per thread after the H stage.
// ---------------------------------------------------------------------------------
__host__ __device__ inline size_t pipe_smem_bytes(int B, int NP) { return 2 * (size_t)kThreads * B * NP * 16; }

template <class S, int B, int NP, bool FULL = false>
__global__ void __launch_bounds__(kThreads, kStepCtas<S, B, NP>) k_cheb_step_pipe(StepArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    constexpr int EPP = S::EPP;
    constexpr int EPT = NP * EPP;
    extern __shared__ __align__(16) unsigned char smem[];
    H* s_h = reinterpret_cast<H*>(smem);
    unsigned* s_col = reinterpret_cast<unsigned*>(smem + sizeof(H) * B * B * (size_t)a.stage_cap);
    uint4* sbuf = reinterpret_cast<uint4*>(smem + ((sizeof(H) * B * B + sizeof(unsigned)) * (size_t)a.stage_cap + 15) / 16 * 16);

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
    // slot of (buffer, bj, q) for this thread
    auto slot = [&](int buf, int bj, int q) -> uint4* { return sbuf + ((size_t)(buf * B + bj) * NP + q) * kThreads + threadIdx.x; };

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
        const int kb = a.row_ptr[i], ke = a.row_ptr[i + 1];
        for (int c = 0; c < nch; c++) {
            const int base = c * W;
            typename S::Acc acc[B][EPT];
#pragma unroll
            for (int bi = 0; bi < B; bi++)
#pragma unroll
                for (int e = 0; e < EPT; e++) acc[bi][e] = S::zero();
            // copies of block k's packets into buffer b
            auto issue = [&](int k, int b) -> unsigned {
                const unsigned cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                const int j = (int)(cc & kColMask);
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    const uint4* row = reinterpret_cast<const uint4*>(x + (size_t)(B * j + bj) * a.ld);
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        const int pk = base + g + Gp * q;
                        if (FULL || pk < P) cp_async16(slot(b, bj, q), row + pk);
                    }
                }
                return cc;
            };
            unsigned cc_next = 0;
            if (kb < ke) cc_next = issue(kb, 0);
            cp_async_commit();
#pragma unroll 1
            for (int k = kb; k < ke; k++) {
                const int b = (k - kb) & 1;
                const unsigned cc = cc_next;
                if (k + 1 < ke) cc_next = issue(k + 1, b ^ 1);
                cp_async_commit();
                cp_async_wait<1>();   // this thread's copies of block k have landed
                const H* hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E xv[EPT];
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        const int pk = base + g + Gp * q;
                        Packet<E, EPP> pkt;
                        pkt.u = make_uint4(0u, 0u, 0u, 0u);
                        if (FULL || pk < P) pkt.u = *slot(b, bj, q);
#pragma unroll
                        for (int e = 0; e < EPP; e++) xv[q * EPP + e] = pkt.e[e];
                    }
                    mac_block<S, B, NP>(acc, cc >> 30, hk, xv, bj);
                }
            }
            cp_async_wait<0>();
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

// ---------------------------------------------------------------------------------
// The reverse (adjoint) step with the same double buffering: block k+1's alpha_m and
// beta_{m+1} packets are copied into shared memory while block k's multiply-adds and D
// epilogue run. Same arithmetic, in the same order, as k_adjoint_step.
// The own rows of alpha_{m+1} and beta_{m+2}, needed only when the row's blocks are done, are
// copied the same way at the start of each column chunk, with the first block's packets.
// Shared memory: (2 buffers x 2 vectors + 2 own rows) x B x NP packets per thread after the H stage.
// ---------------------------------------------------------------------------------
__host__ __device__ inline size_t adj_pipe_smem_bytes(int B, int NP) { return 6 * (size_t)kThreads * B * NP * 16; }

template <class S, int B, int NP, bool FULL = false>
__global__ void __launch_bounds__(kThreads, kAdjointCtas<S, B, NP>) k_adjoint_pipe(AdjArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    constexpr int EPP = S::EPP;
    constexpr int EPT = NP * EPP;
    extern __shared__ __align__(16) unsigned char smem[];
    H* s_h = reinterpret_cast<H*>(smem);
    unsigned* s_col = reinterpret_cast<unsigned*>(smem + sizeof(H) * B * B * (size_t)a.stage_cap);
    uint4* sbuf = reinterpret_cast<uint4*>(smem + ((sizeof(H) * B * B + sizeof(unsigned)) * (size_t)a.stage_cap + 15) / 16 * 16);
    // slot of (buffer, vector v: 0 alpha_m / 1 beta_{m+1}, bj, q) for this thread
    auto slot = [&](int buf, int v, int bj, int q) -> uint4* {
        return sbuf + ((size_t)((buf * 2 + v) * B + bj) * NP + q) * kThreads + threadIdx.x;
    };
    // slot of the own row (v: 0 alpha_{m+1} / 1 beta_{m+2}, bi, q)
    uint4* sown = sbuf + (size_t)4 * B * NP * kThreads;
    auto own_slot = [&](int v, int bi, int q) -> uint4* {
        return sown + ((size_t)(v * B + bi) * NP + q) * kThreads + threadIdx.x;
    };

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
            // copies of block k's alpha_m and beta_{m+1} packets into buffer b (rows of this thread only)
            // FP32 (H not staged): the next block's H entries are read a block ahead like its
            // packets (cubic L=64 S=256: 2.17 vs 2.48 ms); float-float reads its staged H at use
            // (the extra registers cost it 6%)
            constexpr bool kHAhead = S::PREC == 1;
            H hnxt[B * B];
            auto issue = [&](int k, int b) -> unsigned {
                const unsigned cc = tl.staged ? s_col[k - tl.k_lo] : __ldg(a.colc + k);
                const int j = (int)(cc & kColMask);
                if constexpr (kHAhead) {
                    const H* hsrc = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
#pragma unroll
                    for (int q = 0; q < B * B; q++) hnxt[q] = hsrc[q];
                }
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    const uint4* ra = reinterpret_cast<const uint4*>(A + (size_t)(B * j + bj) * a.ld);
                    const uint4* rb = reinterpret_cast<const uint4*>(Bv + (size_t)(B * j + bj) * a.ld);
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        const int pk = base + g + Gp * q;
                        if (FULL || pk < P) {
                            cp_async16(slot(b, 0, bj, q), ra + pk);
                            cp_async16(slot(b, 1, bj, q), rb + pk);
                        }
                    }
                }
                return cc;
            };
            const int nrow = ke - kb;
            // FP32: own rows copied now (cubic L=64: 2.08 vs 2.17 ms); float-float, issue-bound,
            // loads them at the end as the one-pass kernel does (9.77 vs 9.81 ms)
            constexpr bool kOwnAsync = S::PREC == 1;
            if (kOwnAsync && active) {
#pragma unroll
                for (int bi = 0; bi < B; bi++) {
                    const uint4* rap = reinterpret_cast<const uint4*>(Ap + (size_t)(B * i + bi) * a.ld);
                    const uint4* rbp = reinterpret_cast<const uint4*>(Bp + (size_t)(B * i + bi) * a.ld);
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        const int pk = base + g + Gp * q;
                        if (FULL || pk < P) {
                            cp_async16(own_slot(0, bi, q), rap + pk);
                            cp_async16(own_slot(1, bi, q), rbp + pk);
                        }
                    }
                }
            }
            unsigned cc_next = 0;
            if (nrow > 0) cc_next = issue(kb, 0);
            cp_async_commit();
            for (int kk = 0; kk < nmax; kk++) {
                const int k = kb + kk;
                const bool has = kk < nrow;
                const int b = kk & 1;
                const unsigned cc = cc_next;
                H hbuf[B * B];
                const H* hk = hval;
                if constexpr (kHAhead) {
#pragma unroll
                    for (int q = 0; q < B * B; q++) hbuf[q] = hnxt[q];
                    hk = hbuf;
                } else if (has) {
                    hk = tl.staged ? s_h + (size_t)(k - tl.k_lo) * B * B : hval + (size_t)k * B * B;
                }
                if (kk + 1 < nrow) cc_next = issue(k + 1, b ^ 1);
                cp_async_commit();
                cp_async_wait<1>();   // this thread's copies of block k have landed
                const double2 dpre = d_prefetch<S, B>(a.Dacc, (size_t)k, own, fuse && has && own.writer);
                typename S::OAcc of[B * B];
#pragma unroll
                for (int q = 0; q < B * B; q++) of[q] = S::oa_zero();
#pragma unroll
                for (int bj = 0; bj < B; bj++) {
                    E av[EPT], bv[EPT];
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        const int pk = base + g + Gp * q;
                        Packet<E, EPP> pa, pb;
                        pa.u = make_uint4(0u, 0u, 0u, 0u);
                        pb.u = make_uint4(0u, 0u, 0u, 0u);
                        if (has && (FULL || pk < P)) {
                            pa.u = *slot(b, 0, bj, q);
                            pb.u = *slot(b, 1, bj, q);
                        }
#pragma unroll
                        for (int e = 0; e < EPP; e++) { av[q * EPP + e] = pa.e[e]; bv[q * EPP + e] = pb.e[e]; }
                    }
                    if (has) {
                        mac_block<S, B, NP>(accA, cc >> 30, hk, av, bj);
                        mac_block<S, B, NP>(accB, cc >> 30, hk, bv, bj);
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
            cp_async_wait<0>();
            if (active) {
#pragma unroll
                for (int bi = 0; bi < B; bi++) {
                    const size_t roff = (size_t)(B * i + bi) * a.ld;
                    E apv[EPT], bpv[EPT], an[EPT], bn[EPT];
                    if constexpr (kOwnAsync) {
#pragma unroll
                        for (int q = 0; q < NP; q++) {
                            const int pk = base + g + Gp * q;
                            Packet<E, EPP> pa, pb;
                            pa.u = make_uint4(0u, 0u, 0u, 0u);
                            pb.u = make_uint4(0u, 0u, 0u, 0u);
                            if (FULL || pk < P) {
                                pa.u = *own_slot(0, bi, q);
                                pb.u = *own_slot(1, bi, q);
                            }
#pragma unroll
                            for (int e = 0; e < EPP; e++) { apv[q * EPP + e] = pa.e[e]; bpv[q * EPP + e] = pb.e[e]; }
                        }
                    } else {
                        ld_rw<S, NP, FULL>(apv, Ap + roff, base, g, Gp, P);
                        ld_rw<S, NP, FULL>(bpv, Bp + roff, base, g, Gp, P);
                    }
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
// The FP32 / float-float reverse step for block rows served by a whole warp (Gp == 32) whose
// column chunks are all whole: the shape of wide probe blocks (b=2 complex, S >= 128). Same recursions and
// fused D epilogue as k_adjoint_pipe, organised around the fixed shape:
//  * a warp walks one row as a stream of units, chunk by chunk: A (the own alpha_m rows of the
//    chunk), K (one H block: its alpha_m / beta_{m+1} rows, H entries and D entries) for each of
//    the row's blocks, then O (the own alpha_{m+1} / beta_{m+2} rows: the chunk's final update);
//  * every unit's data arrives by cp.async in a ring of three shared-memory slots, issued two units
//    ahead, so two units' copies are in flight while one is computed, also across chunk ends
//    (the general kernel keeps one block ahead and drains at every chunk end);
//  * lane and packet offsets are compile-time (packet q of a lane sits 32 packets after q-1), row
//    addresses are one 32 x 32 -> 64-bit multiply-add; the row's block columns are read once, one
//    per lane (rows of at most 32 blocks, checked by the host), and passed by shuffles;
//  * every lane of a warp walks the same row: no per-block "row has block kk" test, no zero fill;
//    one class branch and one read of the H entries per block;
//  * b=2: a lane whose bit 4 is set (sw = 1) holds every block index swapped -- gathered rows
//    b j + (bj ^ sw), own rows b i + (bi ^ sw), accumulators and H entries permuted to match --
//    so the two D entries it sends at the first transposed reduction level are exactly the two
//    its partner (lane ^ 16, the other swap) keeps, and that level needs no selects.
// It runs with the fused D epilogue only (D's pattern is H's). Results equal k_adjoint_pipe's up to
// the order of the two bj terms of a general block in the swapped lanes (rounding), and the same
// lanes write the same D entries. Float-float blocks carry 64-byte H blocks; each warp's slot part
// holds them with the D entries.
// ---------------------------------------------------------------------------------
template <int V>
struct BufTag { static constexpr int value = V; };

constexpr int kRing = 3;          // shared-memory slots of the unit stream
constexpr int kWarpHBytes = 64;      // per warp and slot: the H block (up to 64 B: 2x2 float-float complex) ...
constexpr int kWarpSlotBytes = 128;  // ... then the 4 writer lanes' D entries (16 B each)

// Shared memory of k_adjoint_warp after the H stage: kRing slots of 2 vectors x B rows x NP packets
// per thread, then the per-warp H / D slots.
__host__ __device__ inline size_t adj_warp_smem_bytes(int B, int NP) {
    return (size_t)kRing * 2 * B * NP * kThreads * 16 + (size_t)(kThreads / 32) * (kRing * kWarpSlotBytes + 32);
}
// cp.async of N = 4, 8 or 16 bytes (N < 16 goes through L1: the .cg form moves 16 bytes only)
template <int N>
__device__ __forceinline__ void cp_async_n(void* dst, const void* src) {
    if constexpr (N == 16) cp_async16(dst, src);
    else asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src), "n"(N) : "memory");
}
// 16-byte cp.async with compile-time offsets on both addresses (folded into the instruction)
template <int DOFF, int SOFF>
__device__ __forceinline__ void cp_async16_at(unsigned dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0+%2], [%1+%3], 16;" ::"r"(dst), "l"(src), "n"(DOFF), "n"(SOFF) : "memory");
}
// An L2 policy that makes the lines it tags the first to be evicted. The own rows of a
// reverse step are read once and overwritten in place (a stream); tagging them keeps L2 for
// the gathered rows, which every neighbouring row reads again: on a cubic lattice with the
// site index running through planes, a row is gathered again two planes later.
__device__ __forceinline__ unsigned long long l2_evict_first() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// cp_async16_at with an L2 cache policy
template <int DOFF, int SOFF>
__device__ __forceinline__ void cp_async16_at_pol(unsigned dst, const void* src, unsigned long long pol) {
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0+%2], [%1+%3], 16, %4;" ::"r"(dst), "l"(src), "n"(DOFF),
                 "n"(SOFF), "l"(pol)
                 : "memory");
}
// 16-byte store with an L2 cache policy
__device__ __forceinline__ void st16_pol(uint4* p, uint4 v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.v4.b32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w), "l"(pol)
                 : "memory");
}
// 16-byte cp.async issued only where `on` holds: a predicated instruction, no branch
__device__ __forceinline__ void cp_async16_if(unsigned dst, const void* src, bool on) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %2, 0;\n\t@p cp.async.cg.shared.global [%0], [%1], 16;\n\t}\n"
        ::"r"(dst), "l"(src), "r"((int)on)
        : "memory");
}
// compile-time loop: f(BufTag<I>()) for I in [I0, N)
template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
    if constexpr (I < N) {
        f(BufTag<I>());
        static_for<I + 1, N>(f);
    }
}
__device__ __forceinline__ const uint4* row_at(const void* base, unsigned row, unsigned row_bytes) {
    return reinterpret_cast<const uint4*>(static_cast<const char*>(base) + (unsigned long long)row * row_bytes);
}

template <class S, int B, int NP>
__global__ void __launch_bounds__(kThreads, kAdjointCtas<S, B, NP>) k_adjoint_warp(AdjArgs a) {
    typedef typename S::E E;
    typedef typename S::H H;
    typedef typename S::OAcc OAcc;
    constexpr int EPP = S::EPP;
    constexpr int EPT = NP * EPP;
    constexpr int G = 32;            // lanes per block row
    constexpr int W = G * NP;        // packets per column chunk
    constexpr int kHBytes = B * B * (int)sizeof(H);
    constexpr int kDBytes = S::CPLX ? 16 : 8;   // one D entry of the accumulator (8 bytes per real)
    static_assert(kHBytes <= kWarpHBytes && B * B * kDBytes <= 64, "per-warp slot sizes");
    extern __shared__ __align__(16) unsigned char smem[];
    uint4* sbuf = reinterpret_cast<uint4*>(smem + ((sizeof(H) * B * B + sizeof(unsigned)) * (size_t)a.stage_cap + 15) / 16 * 16);
    uint4* const mine = sbuf + threadIdx.x;
    // thread-minor ring slots: (slot, vector v, row r, packet q)
    auto slot = [&](int sl, int v, int r, int q) -> uint4* { return mine + (((sl * 2 + v) * B + r) * NP + q) * kThreads; };
    unsigned char* const wbase = reinterpret_cast<unsigned char*>(sbuf + (size_t)kRing * 2 * B * NP * kThreads) +
                                 (threadIdx.x >> 5) * kRing * kWarpSlotBytes;
    // the same places as 32-bit shared addresses, and the strides of the ring slots (bytes)
    const unsigned s_mine = smem_addr(mine), s_warp = smem_addr(wbase);
    // per-warp scratch of 32 bytes after all the warps' slot parts: a row's unit order (float-float)
    unsigned char* const worder = reinterpret_cast<unsigned char*>(sbuf + (size_t)kRing * 2 * B * NP * kThreads) +
                                  (kThreads / 32) * kRing * kWarpSlotBytes + (threadIdx.x >> 5) * 32;
    constexpr int kQStride = kThreads * 16, kRowStride = NP * kQStride, kVecStride = B * kRowStride;
    constexpr unsigned kSlotStride = 2u * kVecStride;
    // complex b=2: the H block is kHP whole 16-byte pieces and a D entry is 16 bytes, so one predicated
    // copy per lane fetches both (lanes 0-1 H, lanes 2-5 the four D entries)
    constexpr int kHP = kHBytes / 16;
    constexpr bool kFast = kHBytes % 16 == 0 && kDBytes == 16 && kHP + B * B <= 32;
    // complex b=2 (FP32: OAcc is a float pair): the last reduction levels split real and imaginary parts
    // (FP32: a float pair; float-float: two float-float values)
    constexpr bool kCompSplit = kFast && B == 2 && S::CPLX && S::PREC != 0;
    auto h_slot = [&](int sl) -> const H* { return reinterpret_cast<const H*>(wbase + sl * kWarpSlotBytes); };

    const int sidx = a.cta_sys[blockIdx.x];
    const SysDesc sd = a.sys[sidx];
    const int lc = blockIdx.x - sd.cta_base;
    const int nch = (sd.P > 0 ? sd.P : a.P) / W;
    const long long items = (long long)sd.n_b * G;
    const unsigned rb = (unsigned)(a.ld * (long long)sizeof(E));   // bytes per scalar row
    const int lane = threadIdx.x & 31;
    const int sw = B == 2 ? (lane >> 4) & 1 : 0;   // block-index swap of this lane
    const int hx = sw * 3;                          // H entry (bi, bj) -> (bi ^ sw, bj ^ sw), column-major b=2
    const H* hval = reinterpret_cast<const H*>(a.hval);
    const typename S::Coef cA = S::coef(a.coef[sidx * a.cstride + 0]);
    const typename S::Coef cAp = S::coef(a.coef[sidx * a.cstride + 1]);
    const typename S::Coef cAn = S::coef(a.coef[sidx * a.cstride + 2]);
    const float2 dscale_ds = ds_from_double(a.dscale);   // a.Dacc is never null here (fused epilogue only)
    const Owner own = transposed_owner<B * B>(G, lane);
    const unsigned long long pol_stream = l2_evict_first();   // alpha_{m+1}, beta_{m+2}: read once, overwritten

    for (long long t0 = (long long)lc * kThreads; t0 < items; t0 += (long long)sd.ctas * kThreads) {
        const long long t = t0 + threadIdx.x;
        if (t >= items) continue;   // items is a multiple of 32: whole warps leave together (no CTA barrier here)
        const int i = sd.row_base + (int)(t >> 5);
        const int kb = a.row_ptr[i];
        const int nrow = a.row_ptr[i + 1] - kb;   // at most 32
        const unsigned ccl = lane < nrow ? __ldg(a.colc + kb + lane) : 0u;   // lane kk: block kb + kk
        const int per = nrow + 2;                  // units per chunk: A, K x nrow, O
        const int U = nch * per;
        // Float-float rows whose identity blocks share one value h (host flag): those blocks come first,
        // their rows are summed (a float-float addition instead of a multiply-add each) and the sum is
        // scaled by h once, before the other blocks add their products. `ord` (lane p): the lane, i.e.
        // block kb + ord, that unit position p takes; n_id: the identity blocks.
        bool hsum = false;
        unsigned ord = lane;
        int n_id = 0;
        if constexpr (S::PREC == 2) {
            hsum = a.row_hsum != nullptr && a.row_hsum[i] != 0;
            if (hsum) {
                const bool isid = lane < nrow && (ccl >> 30) == 2u;
                const unsigned mid = __ballot_sync(0xffffffffu, isid);
                const unsigned mrow = nrow >= 32 ? 0xffffffffu : ((1u << nrow) - 1u);
                const unsigned lt = (1u << lane) - 1u;
                n_id = __popc(mid);
                const int pos = isid ? __popc(mid & lt) : n_id + __popc(mrow & ~mid & lt);
                if (lane < nrow) worder[pos] = (unsigned char)lane;
                __syncwarp();
                ord = lane < nrow ? worder[lane] : lane;
                __syncwarp();
            }
        }

        // ---- issue: put unit (ic, ir) in flight into ring slot sl (one commit group per unit)
        auto issue = [&](int ic, int ir, int sl) {
            const unsigned coff = (unsigned)(ic * W + lane) * 16u;
            const unsigned sdst = s_mine + (unsigned)sl * kSlotStride;   // this thread's part of slot sl
            // the B x NP packets of vector V (slot part) from the rows b r0 + (r ^ sw) of `base`;
            // tag V + 2: the rows are a stream (read once here, overwritten by this warp), copied
            // with the evict-first L2 policy
            auto rows = [&](auto vt, const void* base, unsigned r0) {
                constexpr int V = decltype(vt)::value & 1;
                constexpr bool kStream = decltype(vt)::value >= 2;
                static_for<0, B>([&](auto rt) {
                    constexpr int R = decltype(rt)::value;
                    const uint4* src = row_at(static_cast<const char*>(base) + coff, (unsigned)(B * r0 + (R ^ sw)), rb);
                    static_for<0, NP>([&](auto qt) {
                        constexpr int Q = decltype(qt)::value;
                        if constexpr (kStream)
                            cp_async16_at_pol<V * kVecStride + R * kRowStride + Q * kQStride, Q * G * 16>(sdst, src, pol_stream);
                        else
                            cp_async16_at<V * kVecStride + R * kRowStride + Q * kQStride, Q * G * 16>(sdst, src);
                    });
                });
            };
            if (ir == 0) {                 // A: alpha_m own rows
                rows(BufTag<0>(), a.A, (unsigned)i);
            } else if (ir == per - 1) {    // O: alpha_{m+1}, beta_{m+2} own rows (streams)
                rows(BufTag<2>(), a.Ap, (unsigned)i);
                rows(BufTag<3>(), a.Bp, (unsigned)i);
            } else {                       // K: the block at unit position ir - 1 (identity-first order in hsum rows)
                const int kk = hsum ? (int)__shfl_sync(0xffffffffu, ord, ir - 1) : ir - 1;
                const int k = kb + kk;
                const unsigned cc = __shfl_sync(0xffffffffu, ccl, kk);
                const unsigned j = cc & kColMask;
                const unsigned ws = s_warp + (unsigned)sl * kWarpSlotBytes;
                if constexpr (kFast) {
                    // lanes 0 .. kHP-1: the H block's 16-byte pieces; lanes kHP .. kHP+B*B-1: the D
                    // entries of the block (one per writer lane, read back by it)
                    const bool hl = lane < kHP;
                    const int dl = lane - kHP;
                    const bool dlane = dl >= 0 && dl < B * B;
                    const char* src = hl ? reinterpret_cast<const char*>(hval + (size_t)k * B * B) + lane * 16
                                         : reinterpret_cast<const char*>(a.Dacc + ((size_t)k * B * B + (dlane ? dl : 0)) * 2);
                    cp_async16_if(hl ? ws + lane * 16 : ws + kWarpHBytes + dl * 16, src, hl || dlane);
                } else {
                    constexpr int kPieces = kHBytes >= 16 ? kHBytes / 16 : 1;
                    constexpr int kPiece = kHBytes >= 16 ? 16 : kHBytes;
                    unsigned char* wsp = wbase + sl * kWarpSlotBytes;
                    if (lane < kPieces)
                        cp_async_n<kPiece>(wsp + lane * kPiece, reinterpret_cast<const char*>(hval + (size_t)k * B * B) + lane * kPiece);
                    if (own.writer)   // the D entry this lane will update
                        cp_async_n<kDBytes>(wsp + kWarpHBytes + own.first * kDBytes,
                                            a.Dacc + ((size_t)k * B * B + own.first) * (S::CPLX ? 2 : 1));
                }
                rows(BufTag<0>(), a.A, j);
                rows(BufTag<1>(), a.Bv, j);
            }
            cp_async_commit();
        };

        E Ai[B][EPT];   // alpha_m of the own rows (this lane's order), for the current chunk
        typename S::Acc accA[B][EPT], accB[B][EPT];
        // one block's multiply-adds and epilogue products from ring slot sl; IDENT: a real multiple
        // of the identity (class 2, read from its (0,0) entry), else general (real systems, or complex
        // with class 0 or 1: a class-1 block's zero imaginary parts make the complex product exact)
        // FP32: both rows' multiply-adds, then the epilogue once for every block kind (beta_{m+1}'s
        // packets read from shared memory again): 1.628 vs 1.669 ms at cubic L=64, S=256. Float-float
        // keeps each row's epilogue with its multiply-adds (8.10 vs 8.44 ms split).
        constexpr bool kEpiInside = S::PREC != 1;
        // one block's recursion multiply-adds from ring slot sl (and, kEpiInside, its epilogue
        // products); MODE 0: general (real systems, or complex with class 0 or 1: a class-1 block's
        // zero imaginary parts make the complex product exact), 1: a real multiple of the identity
        // (class 2, its (0,0) entry), 2: an identity block of an hsum row (its rows added; the sum is
        // scaled after the row's last identity block)
        auto body = [&](auto mtag, int sl, OAcc (&of)[B * B]) {
            constexpr int MODE = decltype(mtag)::value;
            const H* hm = h_slot(sl);
            typename S::Hr hd;
            H hr[B * B];
            if constexpr (MODE == 1) hd = S::hreal(hm[0]);
            else if constexpr (MODE == 0) {
#pragma unroll
                for (int q = 0; q < B * B; q++) hr[q] = hm[q ^ hx];   // this lane's order
            }
#pragma unroll
            for (int rj = 0; rj < B; rj++) {
                E av[EPT], bv[EPT];
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    Packet<E, EPP> pa, pb;
                    pa.u = *slot(sl, 0, rj, q);
                    pb.u = *slot(sl, 1, rj, q);
#pragma unroll
                    for (int e = 0; e < EPP; e++) { av[q * EPP + e] = pa.e[e]; bv[q * EPP + e] = pb.e[e]; }
                }
                if constexpr (MODE == 2) {
                    if constexpr (S::PREC == 2) {
#pragma unroll
                        for (int e = 0; e < EPT; e++) { S::acc_add(accA[rj][e], av[e]); S::acc_add(accB[rj][e], bv[e]); }
                    }
                } else if constexpr (MODE == 1) {
#pragma unroll
                    for (int e = 0; e < EPT; e++) { S::mac_re(accA[rj][e], hd, av[e]); S::mac_re(accB[rj][e], hd, bv[e]); }
                } else {
#pragma unroll
                    for (int r = 0; r < B; r++) {
                        const H h = hr[rj * B + r];
                        if constexpr (S::CPLX) {
#pragma unroll
                            for (int e = 0; e < EPT; e++) { S::mac(accA[r][e], h, av[e]); S::mac(accB[r][e], h, bv[e]); }
                        } else {
#pragma unroll
                            for (int e = 0; e < EPT; e++) { S::mac_re(accA[r][e], S::hreal(h), av[e]); S::mac_re(accB[r][e], S::hreal(h), bv[e]); }
                        }
                    }
                }
                if constexpr (kEpiInside) {
#pragma unroll
                    for (int r = 0; r < B; r++) {   // each entry's first product starts it (of is zero): no add to zero
                        of[rj * B + r] = S::oa_first(Ai[r][0], bv[0]);
#pragma unroll
                        for (int e = 1; e < EPT; e++) S::oa_mac(of[rj * B + r], Ai[r][e], bv[e]);
                    }
                }
            }
        };
        // the block's epilogue products after its multiply-adds (FP32): one copy of this code for all
        // block kinds, beta_{m+1}'s packets read from shared memory again
        auto epi = [&](int sl, OAcc (&of)[B * B]) {
#pragma unroll
            for (int rj = 0; rj < B; rj++) {
                E bv[EPT];
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    Packet<E, EPP> pb;
                    pb.u = *slot(sl, 1, rj, q);
#pragma unroll
                    for (int e = 0; e < EPP; e++) bv[q * EPP + e] = pb.e[e];
                }
#pragma unroll
                for (int r = 0; r < B; r++) {   // each entry's first product starts it (of is zero): no add to zero
                    of[rj * B + r] = S::oa_first(Ai[r][0], bv[0]);
#pragma unroll
                    for (int e = 1; e < EPT; e++) S::oa_mac(of[rj * B + r], Ai[r][e], bv[e]);
                }
            }
        };

        issue(0, 0, 0);
        issue(0, 1, 1);                           // per >= 2: unit 1 is (chunk 0, position 1)
        int pc = 0, pr = 0;                       // the unit being processed: chunk, position
        int ic = 2 / per, ir = 2 % per;           // the next unit to issue
        int sl = 0;                               // its ring slot: u % kRing
#pragma unroll 1
        for (int u = 0; u < U; u++) {
            const int sl_next = sl == 0 ? 2 : sl - 1;   // (u + 2) % kRing
            __syncwarp();   // every lane is done with unit u - 1, whose slot unit u + 2 takes
            if (u + 2 < U) {
                issue(ic, ir, sl_next);
                if (++ir == per) { ir = 0; ic++; }
            } else {
                cp_async_commit();   // one group per unit keeps the wait count fixed
            }
            cp_async_wait<2>();   // unit u's copies have landed (units u + 1, u + 2 may be in flight)
            __syncwarp();         // ... and those of the warp's shared H / D entries, copied by other lanes
            if (pr == 0) {        // A: the chunk's alpha_m rows; accumulators start
#pragma unroll
                for (int r = 0; r < B; r++) {
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        Packet<E, EPP> pa;
                        pa.u = *slot(sl, 0, r, q);
#pragma unroll
                        for (int e = 0; e < EPP; e++) Ai[r][q * EPP + e] = pa.e[e];
                    }
#pragma unroll
                    for (int e = 0; e < EPT; e++) { accA[r][e] = S::zero(); accB[r][e] = S::zero(); }
                }
            } else if (pr < per - 1) {   // K: the block at unit position pr - 1
                const int kk = hsum ? (int)__shfl_sync(0xffffffffu, ord, pr - 1) : pr - 1;
                const int k = kb + kk;
                const unsigned cc = __shfl_sync(0xffffffffu, ccl, kk);
                OAcc of[B * B];
#pragma unroll
                for (int q = 0; q < B * B; q++) of[q] = S::oa_zero();
                if ((cc >> 30) == 2u) {
                    bool summed = false;
                    if constexpr (S::PREC == 2) {
                        if (hsum) {
                            body(BufTag<2>(), sl, of);
                            summed = true;
                            if (pr - 1 == n_id - 1) {   // the last identity block: scale the sums by h
                                const typename S::Hr h = S::hreal(h_slot(sl)[0]);
#pragma unroll
                                for (int r = 0; r < B; r++)
#pragma unroll
                                    for (int e = 0; e < EPT; e++) { S::acc_scale(accA[r][e], h); S::acc_scale(accB[r][e], h); }
                            }
                        }
                    }
                    if (!summed) body(BufTag<1>(), sl, of);
                } else {
                    body(BufTag<0>(), sl, of);
                }
                if constexpr (!kEpiInside) epi(sl, of);
                // of[rj * B + r] holds D entry (bj = rj ^ sw, bi = r ^ sw)
                if constexpr (B == 2) {
                    // lane ^ 16 has the other swap: its (1,1) and (1,0) slots are this lane's (0,0), (0,1)
                    of[0] = S::oa_add(of[0], S::oa_shfl(of[3], 16));
                    of[1] = S::oa_add(of[1], S::oa_shfl(of[2], 16));
                    // now of[0] = (bj sw, bi sw), of[1] = (bj sw, bi sw ^ 1); lane bit 3 picks bi
                    const bool k0 = ((lane >> 3) & 1) == sw;
                    const OAcc keep = k0 ? of[0] : of[1];
                    const OAcc send = k0 ? of[1] : of[0];
                    of[0] = S::oa_add(keep, S::oa_shfl(send, 8));
                    if constexpr (kCompSplit) {
                        // third level: lane bit 2 picks the real (0) or imaginary (1) part, so each of the
                        // 8 writer lanes (lane & 3 == 0) finishes and stores one real of the block
                        const bool im = (lane >> 2) & 1;
                        const int ent = sw * 2 + ((lane >> 3) & 1);   // entry bj * 2 + bi
                        const size_t q = ((size_t)k * B * B + ent) * 2 + (im ? 1 : 0);
                        const unsigned char* dp = wbase + sl * kWarpSlotBytes + kWarpHBytes + ent * 16 + (im ? 8 : 0);
                        if constexpr (S::PREC == 2) {   // float-float parts (hi, lo)
                            const float2 kp = im ? make_float2(of[0].z, of[0].w) : make_float2(of[0].x, of[0].y);
                            const float2 sd2 = im ? make_float2(of[0].x, of[0].y) : make_float2(of[0].z, of[0].w);
                            float2 v = kp;
                            ds_add(v, make_float2(__shfl_xor_sync(0xffffffffu, sd2.x, 4), __shfl_xor_sync(0xffffffffu, sd2.y, 4)));
#pragma unroll
                            for (int off = 2; off > 0; off >>= 1)
                                ds_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off)));
                            if ((lane & 3) == 0) {
                                float2 cur2 = *reinterpret_cast<const float2*>(dp);
                                ds_mac(cur2, dscale_ds, v);
                                reinterpret_cast<float2*>(a.Dacc)[q] = ds_norm(cur2);
                            }
                        } else {
                            const float kp = im ? of[0].y : of[0].x;
                            const float sd2 = im ? of[0].x : of[0].y;
                            float v = kp + __shfl_xor_sync(0xffffffffu, sd2, 4);
                            v += __shfl_xor_sync(0xffffffffu, v, 2);
                            v += __shfl_xor_sync(0xffffffffu, v, 1);
                            if ((lane & 3) == 0) {
                                if constexpr (S::DACC_DS) {
                                    float2 cur2 = *reinterpret_cast<const float2*>(dp);
                                    ds_mac(cur2, dscale_ds, make_float2(v, 0.f));
                                    reinterpret_cast<float2*>(a.Dacc)[q] = ds_norm(cur2);
                                } else {
                                    a.Dacc[q] = *reinterpret_cast<const double*>(dp) + a.dscale * (double)v;
                                }
                            }
                        }
                    } else {
#pragma unroll
                        for (int off = 4; off > 0; off >>= 1) of[0] = S::oa_add(of[0], S::oa_shfl(of[0], off));
                    }
                } else {
                    group_sum_transposed<S, B * B>(of, G, lane);
                }
                if constexpr (!kCompSplit) {
                    double2 pre = make_double2(0.0, 0.0);
                    if (own.writer) {   // the D entry, copied with the unit (by lane kHP + first in the fast form)
                        const unsigned char* dp = wbase + sl * kWarpSlotBytes + kWarpHBytes + own.first * kDBytes;
                        if constexpr (S::CPLX) pre = *reinterpret_cast<const double2*>(dp);
                        else pre.x = *reinterpret_cast<const double*>(dp);
                    }
                    d_write<S, B>(of, true, (size_t)k, a.dscale, dscale_ds, a.Dacc, own, pre);
                }
            } else {   // O: alpha_{m-1} and beta_m of the chunk
                const unsigned coff = (unsigned)(pc * W + lane) * 16u;
#pragma unroll
                for (int r = 0; r < B; r++) {
                    E apv[EPT], bpv[EPT], an[EPT], bn[EPT];
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        Packet<E, EPP> pa, pb;
                        pa.u = *slot(sl, 0, r, q);
                        pb.u = *slot(sl, 1, r, q);
#pragma unroll
                        for (int e = 0; e < EPP; e++) { apv[q * EPP + e] = pa.e[e]; bpv[q * EPP + e] = pb.e[e]; }
                    }
#pragma unroll
                    for (int e = 0; e < EPT; e++) {
                        an[e] = S::fin(accA[r][e], true, true, apv[e]);
                        typename S::Acc tb = S::from(S::fin(accB[r][e], true, true, bpv[e]));
                        S::axpy(tb, cA, Ai[r][e]);
                        S::axpy(tb, cAp, apv[e]);
                        S::axpy(tb, cAn, an[e]);
                        bn[e] = S::to(tb);
                    }
                    uint4* rap = const_cast<uint4*>(row_at(static_cast<char*>(a.Ap) + coff, (unsigned)(B * i + (r ^ sw)), rb));
                    uint4* rbp = const_cast<uint4*>(row_at(static_cast<char*>(a.Bp) + coff, (unsigned)(B * i + (r ^ sw)), rb));
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        Packet<E, EPP> pa, pb;
#pragma unroll
                        for (int e = 0; e < EPP; e++) { pa.e[e] = an[q * EPP + e]; pb.e[e] = bn[q * EPP + e]; }
                        st16_pol(rap + q * G, pa.u, pol_stream);
                        st16_pol(rbp + q * G, pb.u, pol_stream);
                    }
                }
            }
            if (++pr == per) { pr = 0; pc++; }
            sl = sl == kRing - 1 ? 0 : sl + 1;
        }
        cp_async_wait<0>();
        __syncwarp();   // the next row's first copies reuse slots the other lanes have just read
    }
}

}  // namespace fk
