// fk_gram.cuh -- FP64 (real or complex) products C = op(A) op(B) with a long contraction
// dimension, for the second-order moments (moments2_v1 / moments2_v2): the mu blocks A^H B
// over Chebyshev panels, the s x s probe projections, and the trace of products.
//
//   C[i + j ldc] (= beta C) + sum_k  opA(i, k) opB(k, j),  i < m, j < n, k < kdim
//   opA(i, k) = A[i a_si + k a_sk]   (conjugated when conj_a)
//   opB(k, j) = B[k b_sk + j b_sj]   (conjugated when conj_b)
//
// The output is small (m, n <= a few thousand) and the contraction long (kdim up to 2^31), so
// the contraction is split across CTAs (grid z): every CTA computes a 64 x 64 tile of C over its
// range of k, staging 16-deep slices of A and B in shared memory, 256 threads with a 4 x 4
// register tile each; partial tiles go to a workspace and a second kernel sums them over the
// splits in a fixed order (deterministic). FP64 arithmetic (DFMA): on this GPU the FP64 tensor
// rate is no higher than the FP64 pipe's, so the kernel is bound by the FP64 pipe.
#pragma once
#include <cuda_runtime.h>

namespace fk {

constexpr int kGramTile = 64;
constexpr int kGramDepth = 16;
constexpr int kGramThreads = 256;

template <bool CPLX>
struct GramT {
    typedef double V;
    __device__ static V zero() { return 0.0; }
    __device__ static V load(const double* p, long long idx) { return p[idx]; }
    __device__ static V conj(V v) { return v; }
    __device__ static void mac(V& c, V a, V b) { c = fma(a, b, c); }
};
template <>
struct GramT<true> {
    typedef double2 V;
    __device__ static V zero() { return make_double2(0.0, 0.0); }
    __device__ static V load(const double* p, long long idx) { return reinterpret_cast<const double2*>(p)[idx]; }
    __device__ static V conj(V v) { return make_double2(v.x, -v.y); }
    __device__ static void mac(V& c, V a, V b) {
        c.x = fma(a.x, b.x, c.x);
        c.x = fma(-a.y, b.y, c.x);
        c.y = fma(a.x, b.y, c.y);
        c.y = fma(a.y, b.x, c.y);
    }
};

struct GramArgs {
    int m, n;
    long long kdim, k_per_split;
    const double* A;
    long long a_si, a_sk;
    int conj_a;
    const double* B;
    long long b_sk, b_sj;
    int conj_b;
    double* work;   // [splits][n][m] partial tiles (V elements)
};

// Partial product of one 64 x 64 tile of C over k in [z k_per_split, (z + 1) k_per_split).
template <bool CPLX>
__global__ void __launch_bounds__(kGramThreads) k_gram_partial(GramArgs g) {
    typedef GramT<CPLX> T;
    typedef typename T::V V;
    __shared__ V sa[kGramDepth][kGramTile + 1];   // +1: the k-fast staging stores spread over banks
    __shared__ V sb[kGramDepth][kGramTile + 1];
    const int i0 = blockIdx.x * kGramTile, j0 = blockIdx.y * kGramTile;
    const long long k_lo = (long long)blockIdx.z * g.k_per_split;
    const long long k_hi = min(g.kdim, k_lo + g.k_per_split);
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    V acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[p][q] = T::zero();
    // loads walk the operand along whichever index has unit stride (coalesced)
    const bool a_k_fast = g.a_sk == 1, b_k_fast = g.b_sk == 1;
    for (long long k0 = k_lo; k0 < k_hi; k0 += kGramDepth) {
#pragma unroll
        for (int r = 0; r < kGramDepth * kGramTile / kGramThreads; r++) {
            const int t = threadIdx.x + r * kGramThreads;
            int kk, ii;
            if (a_k_fast) { kk = t % kGramDepth; ii = t / kGramDepth; }
            else { ii = t % kGramTile; kk = t / kGramTile; }
            const long long k = k0 + kk;
            const int i = i0 + ii;
            V v = T::zero();
            if (k < k_hi && i < g.m) {
                v = T::load(g.A, (long long)i * g.a_si + k * g.a_sk);
                if (g.conj_a) v = T::conj(v);
            }
            sa[kk][ii] = v;
            int kb, jj;
            if (b_k_fast) { kb = t % kGramDepth; jj = t / kGramDepth; }
            else { jj = t % kGramTile; kb = t / kGramTile; }
            const long long kq = k0 + kb;
            const int j = j0 + jj;
            V w = T::zero();
            if (kq < k_hi && j < g.n) {
                w = T::load(g.B, kq * g.b_sk + (long long)j * g.b_sj);
                if (g.conj_b) w = T::conj(w);
            }
            sb[kb][jj] = w;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kGramDepth; kk++) {
            V a[4], b[4];
#pragma unroll
            for (int p = 0; p < 4; p++) a[p] = sa[kk][ty + 16 * p];
#pragma unroll
            for (int q = 0; q < 4; q++) b[q] = sb[kk][tx + 16 * q];
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) T::mac(acc[p][q], a[p], b[q]);
        }
        __syncthreads();
    }
    V* out = reinterpret_cast<V*>(g.work) + (size_t)blockIdx.z * g.m * g.n;
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
            if (i < g.m && j < g.n) out[(size_t)j * g.m + i] = acc[p][q];
        }
}

// C[i + j ldc] = (beta ? C : 0) + sum over splits z = 0, 1, ... of work[z][j][i], in that order.
template <bool CPLX>
__global__ void k_gram_reduce(const double* work, int splits, int m, int n, double* C, long long ldc, int beta) {
    typedef GramT<CPLX> T;
    typedef typename T::V V;
    const long long total = (long long)m * n;
    const V* w = reinterpret_cast<const V*>(work);
    V* c = reinterpret_cast<V*>(C);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % m), j = (int)(q / m);
        V s = beta ? c[i + j * ldc] : T::zero();
        for (int z = 0; z < splits; z++) {
            const V v = w[(size_t)z * total + q];
            if constexpr (CPLX) { s.x += v.x; s.y += v.y; }
            else s += v;
        }
        c[i + j * ldc] = s;
    }
}

}  // namespace fk
