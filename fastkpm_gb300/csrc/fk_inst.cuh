// fk_inst.cuh -- instantiates every kernel of one precision (included once per
// fk_inst_<prec>.cu with FK_PREC_NAME, FK_SYS_R and FK_SYS_C defined).
#pragma once
#include <algorithm>

#include "fk_dispatch.h"

namespace fk {

namespace {
// Rows whose chunks are all whole (P a multiple of Gp * NP, e.g. every power-of-two S) run the
// instance without packet masks: 2-5% faster per launch (float-float cubic L=64 S=256: step
// 2.55 vs 2.65 ms, outer product 5.12 vs 5.39).
inline bool whole_chunks(int P, int Gp, int NP) { return Gp > 0 && P % (Gp * NP) == 0; }
template <class S, int B, int NP, bool FULL>
cudaError_t step_pipe_launch(const StepArgs& a, const Launch& l) {
    if (l.smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)k_cheb_step_pipe<S, B, NP, FULL>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem);
        if (e != cudaSuccess) return e;
    }
    k_cheb_step_pipe<S, B, NP, FULL><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP>
cudaError_t step_one(const StepArgs& a, const Launch& l) {
    const bool whole = whole_chunks(a.P, a.Gp, NP);
    if constexpr (S::PREC != 0) {   // double-buffered gathers: FP32 and float-float systems
        if (a.pipe) return whole ? step_pipe_launch<S, B, NP, true>(a, l) : step_pipe_launch<S, B, NP, false>(a, l);
    }
    if (whole) k_cheb_step<S, B, NP, true><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    else k_cheb_step<S, B, NP, false><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP, bool TMA>
cudaError_t staged_launch(const StepArgs& a, const StageTables& t, const Launch& l) {
    if (l.smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)k_cheb_step_staged<S, B, NP, TMA>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem);
        if (e != cudaSuccess) return e;
    }
    k_cheb_step_staged<S, B, NP, TMA><<<l.grid, kThreads, l.smem, l.stream>>>(a, t);
    return cudaGetLastError();
}
template <class S, int B, int NP>
cudaError_t staged_one(const StepArgs& a, const StageTables& t, const Launch& l, int tma) {
    return tma ? staged_launch<S, B, NP, true>(a, t, l) : staged_launch<S, B, NP, false>(a, t, l);
}
template <class S, int B, int NP, bool FULL>
cudaError_t adj_split_launch(const AdjArgs& a, const Launch& l) {
    if (l.smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)k_adjoint_split<S, B, NP, FULL>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem);
        if (e != cudaSuccess) return e;
    }
    k_adjoint_split<S, B, NP, FULL><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP, bool FULL>
cudaError_t adj_pipe_launch(const AdjArgs& a, const Launch& l) {
    if (l.smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)k_adjoint_pipe<S, B, NP, FULL>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem);
        if (e != cudaSuccess) return e;
    }
    k_adjoint_pipe<S, B, NP, FULL><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP>
cudaError_t adj_warp_launch(const AdjArgs& a, const Launch& l) {
    if (l.smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void*)k_adjoint_warp<S, B, NP>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem);
        if (e != cudaSuccess) return e;
    }
    k_adjoint_warp<S, B, NP><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP>
cudaError_t adj_one(const AdjArgs& a, const Launch& l) {
    const bool whole = whole_chunks(a.P, a.Gp, NP);
    if constexpr (S::PREC != 0) {   // FP32 / float-float rows served by a whole warp
        if (a.pipe && a.warp && whole && a.Gp == 32 && a.Dacc) return adj_warp_launch<S, B, NP>(a, l);
    }
    if constexpr (S::PREC != 0) {   // double-buffered gathers: FP32 and float-float systems
        if (a.pipe) return whole ? adj_pipe_launch<S, B, NP, true>(a, l) : adj_pipe_launch<S, B, NP, false>(a, l);
    }
    if (a.split) return whole ? adj_split_launch<S, B, NP, true>(a, l) : adj_split_launch<S, B, NP, false>(a, l);
    if constexpr (S::PREC == 0 && S::CPLX && B == 2) {   // FP64 complex rows served by a whole warp
        if (a.warp && whole && a.Gp == 32 && a.Dacc) {
            k_adjoint_step_warp<S, NP><<<l.grid, kThreads, l.smem, l.stream>>>(a);
            return cudaGetLastError();
        }
    }
    if (whole) k_adjoint_step<S, B, NP, true><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    else k_adjoint_step<S, B, NP, false><<<l.grid, kThreads, l.smem, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP>
cudaError_t outer_one(const OuterArgs& a, const Launch& l) {
    if (whole_chunks(a.P, a.Gp, NP)) k_outer<S, B, NP, true><<<l.grid, kThreads, 0, l.stream>>>(a);
    else k_outer<S, B, NP, false><<<l.grid, kThreads, 0, l.stream>>>(a);
    return cudaGetLastError();
}
template <class S, int B, int NP>
const void* pipe_fn(int kind) {
    if constexpr (S::PREC != 0) {
        if (kind == kAdjointWarp) return (const void*)k_adjoint_warp<S, B, NP>;
    }
    if constexpr (S::PREC != 0)
        return kind == kStepPipe ? (const void*)k_cheb_step_pipe<S, B, NP, true> : (const void*)k_adjoint_pipe<S, B, NP, true>;
    else return nullptr;
}
template <class S, int B, int NP>
cudaError_t occ_one(int kind, size_t smem, int* n) {
    if constexpr (S::PREC == 0) {
        if (kind == kStepPipe || kind == kAdjointPipe) return cudaErrorInvalidValue;
        if (kind == kAdjointWarp) {
            if constexpr (S::CPLX && B == 2)
                return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, (const void*)k_adjoint_step_warp<S, NP>, kThreads, smem);
            else return cudaErrorInvalidValue;
        }
    }
    const void* f = kind == kStep ? (const void*)k_cheb_step<S, B, NP>
                  : (kind == kStepPipe || kind == kAdjointPipe || kind == kAdjointWarp) ? pipe_fn<S, B, NP>(kind)
                  : kind == kAdjoint ? (const void*)k_adjoint_step<S, B, NP>
                  : kind == kAdjointSplit ? (const void*)k_adjoint_split<S, B, NP, true>
                  : kind == kStepStaged ? (const void*)k_cheb_step_staged<S, B, NP, true>
                  : kind == kStepStagedAsync ? (const void*)k_cheb_step_staged<S, B, NP, false>
                  : (const void*)k_outer<S, B, NP>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, f, kThreads, smem);
}
}  // namespace

// dispatch on (cplx, B, NP) -> template instance
#define FK_DISPATCH(FN, ...)                                                            \
    do {                                                                                \
        const int key = (cplx ? 100 : 0) + B * 10 + NP;                                 \
        switch (key) {                                                                  \
            case 11: return FN<FK_SYS_R, 1, 1>(__VA_ARGS__);                            \
            case 12: return FN<FK_SYS_R, 1, 2>(__VA_ARGS__);                            \
            case 14: return FN<FK_SYS_R, 1, 4>(__VA_ARGS__);                            \
            case 21: return FN<FK_SYS_R, 2, 1>(__VA_ARGS__);                            \
            case 22: return FN<FK_SYS_R, 2, 2>(__VA_ARGS__);                            \
            case 24: return FN<FK_SYS_R, 2, 4>(__VA_ARGS__);                            \
            case 111: return FN<FK_SYS_C, 1, 1>(__VA_ARGS__);                           \
            case 112: return FN<FK_SYS_C, 1, 2>(__VA_ARGS__);                           \
            case 114: return FN<FK_SYS_C, 1, 4>(__VA_ARGS__);                           \
            case 121: return FN<FK_SYS_C, 2, 1>(__VA_ARGS__);                           \
            case 122: return FN<FK_SYS_C, 2, 2>(__VA_ARGS__);                           \
            case 124: return FN<FK_SYS_C, 2, 4>(__VA_ARGS__);                           \
            default: return cudaErrorInvalidValue;                                      \
        }                                                                               \
    } while (0)

#define FK_CAT2(a, b) a##_##b
#define FK_CAT(a, b) FK_CAT2(a, b)

cudaError_t FK_CAT(launch_step, FK_PREC_NAME)(int cplx, int B, int NP, const StepArgs& a, const Launch& l) {
    FK_DISPATCH(step_one, a, l);
}
cudaError_t FK_CAT(launch_step_staged, FK_PREC_NAME)(int cplx, int B, int NP, int tma, const StepArgs& a,
                                                   const StageTables& t, const Launch& l) {
    FK_DISPATCH(staged_one, a, t, l, tma);
}
cudaError_t FK_CAT(launch_adjoint, FK_PREC_NAME)(int cplx, int B, int NP, const AdjArgs& a, const Launch& l) {
    FK_DISPATCH(adj_one, a, l);
}
cudaError_t FK_CAT(launch_outer, FK_PREC_NAME)(int cplx, int B, int NP, const OuterArgs& a, const Launch& l) {
    FK_DISPATCH(outer_one, a, l);
}
cudaError_t FK_CAT(occupancy, FK_PREC_NAME)(int kind, int cplx, int B, int NP, size_t smem, int* n) {
    FK_DISPATCH(occ_one, kind, smem, n);
}

static int helper_grid(long long work) {
    long long g = (work + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (g < 1) g = 1;
    return (int)g;
}

cudaError_t FK_CAT(launch_load_colmajor, FK_PREC_NAME)(int cplx, const double* src, long long n, int ncols, int c0,
                                                     long long ld, void* dst, cudaStream_t st) {
    const long long tiles = ((n + kTransposeTile - 1) / kTransposeTile) * ((ncols + kTransposeTile - 1) / kTransposeTile);
    const int g = (int)std::max<long long>(1, std::min<long long>(tiles, 152LL * 8));
    const dim3 blk(kTransposeTile, 8);
    if (cplx) k_load_colmajor<FK_SYS_C><<<g, blk, 0, st>>>(src, n, ncols, c0, ld, reinterpret_cast<FK_SYS_C::E*>(dst));
    else k_load_colmajor<FK_SYS_R><<<g, blk, 0, st>>>(src, n, ncols, c0, ld, reinterpret_cast<FK_SYS_R::E*>(dst));
    return cudaGetLastError();
}
cudaError_t FK_CAT(launch_store_colmajor, FK_PREC_NAME)(int cplx, const void* src, long long n, int ncols, long long ld,
                                                      double* dst, cudaStream_t st) {
    const int g = helper_grid(n * ncols);
    if (cplx) k_store_colmajor<FK_SYS_C><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_C::E*>(src), n, ncols, ld, dst);
    else k_store_colmajor<FK_SYS_R><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_R::E*>(src), n, ncols, ld, dst);
    return cudaGetLastError();
}
cudaError_t FK_CAT(launch_scale, FK_PREC_NAME)(int cplx, const void* x, void* y, long long n_elems, double c,
                                             const double* c_dev, cudaStream_t st) {
    const int g = helper_grid(n_elems);
    if (cplx) k_scale<FK_SYS_C><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_C::E*>(x), reinterpret_cast<FK_SYS_C::E*>(y), n_elems, c, c_dev);
    else k_scale<FK_SYS_R><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_R::E*>(x), reinterpret_cast<FK_SYS_R::E*>(y), n_elems, c, c_dev);
    return cudaGetLastError();
}
cudaError_t FK_CAT(launch_export_panel, FK_PREC_NAME)(int cplx, const void* src, long long n, long long ld, long long c0,
                                                    int w, double* dst, cudaStream_t st) {
    const int g = helper_grid(n * w);
    if (cplx) k_export_panel<FK_SYS_C><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_C::E*>(src), n, ld, c0, w, dst);
    else k_export_panel<FK_SYS_R><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_R::E*>(src), n, ld, c0, w, dst);
    return cudaGetLastError();
}
cudaError_t FK_CAT(launch_scale_rows, FK_PREC_NAME)(int cplx, const void* x, void* y, long long n_rows, long long ld,
                                                  int b, const int* row_sys, const double* f, cudaStream_t st) {
    const int g = helper_grid(n_rows * ld);
    if (cplx) k_scale_rows<FK_SYS_C><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_C::E*>(x), reinterpret_cast<FK_SYS_C::E*>(y), n_rows, ld, b, row_sys, f);
    else k_scale_rows<FK_SYS_R><<<g, 256, 0, st>>>(reinterpret_cast<const FK_SYS_R::E*>(x), reinterpret_cast<FK_SYS_R::E*>(y), n_rows, ld, b, row_sys, f);
    return cudaGetLastError();
}

cudaError_t FK_CAT(launch_expand_sparse, FK_PREC_NAME)(int cplx, const int* cols, const double* vals, long long n, int k,
                                                     long long ld, void* dst, cudaStream_t st) {
    const int g = helper_grid(n);
    if (cplx) k_expand_sparse<FK_SYS_C><<<g, 256, 0, st>>>(cols, vals, n, k, ld, reinterpret_cast<FK_SYS_C::E*>(dst));
    else k_expand_sparse<FK_SYS_R><<<g, 256, 0, st>>>(cols, vals, n, k, ld, reinterpret_cast<FK_SYS_R::E*>(dst));
    return cudaGetLastError();
}

}  // namespace fk
