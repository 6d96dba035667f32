// fk_dispatch.h -- host-side launch table for the templated kernels.
// Each precision's kernels are instantiated in their own translation unit
// (fk_inst_f64.cu, fk_inst_f32.cu, fk_inst_ds.cu) so the build compiles them in
// parallel; fk_engine.cu reaches them only through these functions.
#pragma once
#include <cuda_runtime.h>
#include "fk_kernels.cuh"
#include "fk_staged.cuh"

namespace fk {

enum Prec { kF64 = 0, kF32 = 1, kDS = 2 };
enum KernelKind { kStep = 0, kAdjoint = 1, kOuter = 2, kHelper = 3, kNumKinds = 4, kStepStaged = 5, kStepStagedAsync = 6,
                  kAdjointSplit = 7, kStepPipe = 8, kAdjointPipe = 9, kAdjointWarp = 10 };

struct Launch {
    int grid;
    size_t smem;
    cudaStream_t stream;
};

// element / H-entry sizes in bytes, elements per 16-byte packet
inline int elem_bytes(int prec, int cplx) {
    static const int t[3][2] = {{8, 16}, {4, 8}, {8, 16}};
    return t[prec][cplx ? 1 : 0];
}
inline int elems_per_packet(int prec, int cplx) { return 16 / elem_bytes(prec, cplx); }

// Per-precision entry points (defined in fk_inst_<prec>.cu)
#define FK_DECLARE_PREC(P)                                                                                  \
    cudaError_t launch_step_##P(int cplx, int B, int NP, const StepArgs& a, const Launch& l);              \
    cudaError_t launch_step_staged_##P(int cplx, int B, int NP, int tma, const StepArgs& a,                \
                                       const StageTables& t, const Launch& l);                            \
    cudaError_t launch_adjoint_##P(int cplx, int B, int NP, const AdjArgs& a, const Launch& l);            \
    cudaError_t launch_outer_##P(int cplx, int B, int NP, const OuterArgs& a, const Launch& l);            \
    cudaError_t occupancy_##P(int kind, int cplx, int B, int NP, size_t smem, int* blocks_per_sm);         \
    cudaError_t launch_load_colmajor_##P(int cplx, const double* src, long long n, int ncols, int c0,      \
                                         long long ld, void* dst, cudaStream_t st);                         \
    cudaError_t launch_store_colmajor_##P(int cplx, const void* src, long long n, int ncols, long long ld, \
                                          double* dst, cudaStream_t st);                                    \
    cudaError_t launch_scale_##P(int cplx, const void* x, void* y, long long n_elems, double c,            \
                                 const double* c_dev, cudaStream_t st);                                     \
    cudaError_t launch_export_panel_##P(int cplx, const void* src, long long n, long long ld, long long c0, \
                                        int w, double* dst, cudaStream_t st);                               \
    cudaError_t launch_scale_rows_##P(int cplx, const void* x, void* y, long long n_rows, long long ld,     \
                                      int b, const int* row_sys, const double* f, cudaStream_t st);        \
    cudaError_t launch_expand_sparse_##P(int cplx, const int* cols, const double* vals, long long n, int k,  \
                                         long long ld, void* dst, cudaStream_t st);
FK_DECLARE_PREC(f64)
FK_DECLARE_PREC(f32)
FK_DECLARE_PREC(f32a)   // FP32 systems with FP64 accumulators (fk_inst_f32a.cu)
FK_DECLARE_PREC(ds)
#undef FK_DECLARE_PREC

}  // namespace fk
