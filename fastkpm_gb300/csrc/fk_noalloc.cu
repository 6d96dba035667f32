// fk_noalloc.cu -- Chebyshev moments for callers that cannot allocate device memory.
//
// Some callers own every byte of device memory through their own allocator (a
// host application's memory pool, or a fixed reservation made at start-up that
// nothing else may grow), or must not trigger the device-wide synchronisation
// that cudaFree implies while their other streams are running. This entry point
// lets them run the fused moment recursion on buffers they already hold: the
// caller passes H, R, the two recursion vectors and the output, and the only
// scratch the kernels need -- per-CTA moment partials, the per-step sums and the
// one-system launch tables -- lives in one file-scope static __device__ array
// (kScratchBytes, under 300 KiB, held by every GPU that loads the library until
// the process exits). No cudaMalloc, cudaFree or allocating library routine is
// called.
//
// The array's name is only a host-side stand-in in host code: every call looks
// up its device address with cudaGetSymbolAddress (the current device's copy; the
// lookup allocates nothing) and passes it to the kernels, so the address is never
// stale, also after a cudaDeviceReset. Every call shares the array and it keeps
// the last call's contents, so calls that overlap on the GPU race with each other.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/fastkpm_gb300.h"
#include "fk_dispatch.h"

namespace {

constexpr int kMaxCtas = 2048;                  // CTAs per step launch (a grid-stride loop covers any size)
constexpr int kMaxSteps = 16384;                // M <= 2 * kMaxSteps = 32768
constexpr size_t kPartialsOff = 0;                                   // kMaxCtas x 2 doubles
constexpr size_t kRawOff = kPartialsOff + sizeof(double) * 2 * kMaxCtas;   // kMaxSteps x 2 doubles
constexpr size_t kSysOff = kRawOff + sizeof(double) * 2 * kMaxSteps;       // one SysDesc (padded)
constexpr size_t kCtaOff = kSysOff + 256;                            // kMaxCtas ints, all zero
constexpr size_t kScratchBytes = kCtaOff + sizeof(int) * kMaxCtas;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The one-system launch tables, written on the caller's stream before the first step of every
// call: the system descriptor, and the CTA -> system table (all zeros: every CTA serves system 0).
__global__ void k_noalloc_sys(fk::SysDesc* sys, int* cta_sys, int n_b, int ctas) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) sys[0] = fk::SysDesc{0, n_b, 0, ctas};
    if (t < kMaxCtas) cta_sys[t] = 0;
}

// Fixed-order sum of one step's CTA partials into raw[0..1].
__global__ void k_noalloc_reduce(const double* partials, int ctas, double* raw) {
    const int lane = threadIdx.x;
    double a = 0.0, b = 0.0;
    for (int c = lane; c < ctas; c += 32) { a += partials[2 * c]; b += partials[2 * c + 1]; }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
    }
    if (lane == 0) { raw[0] = a; raw[1] = b; }
}

// Device address of the scratch array on the current device, looked up on every call.
int scratch_for_current_device(unsigned char** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) { cudaGetLastError(); return FK_ERR_CUDA; }
    *out = (unsigned char*)p;
    return FK_OK;
}

int next_pow2(int v) { int p = 1; while (p < v) p <<= 1; return p; }

}  // namespace

extern "C" int fk_moments_noalloc(int kind, int n_b, int b, const int* d_row_ptr, const int* d_col_idx,
                                  const double* d_hs_val, long long ld, int s, const double* d_R, double* d_work,
                                  int M, double* mu, void* stream) {
    if (kind != FK_REAL && kind != FK_COMPLEX) return FK_ERR_ARG;
    if (n_b <= 0 || (b != 1 && b != 2) || s <= 0 || ld < s) return FK_ERR_ARG;
    if (!d_row_ptr || !d_col_idx || !d_hs_val || !d_R || !d_work || !mu) return FK_ERR_ARG;
    if (M < 2 || M % 2 != 0) return FK_ERR_ARG;
    if (M > 2 * kMaxSteps) return FK_ERR_UNSUPPORTED;   // beyond the static scratch: M <= 32768
    const int cplx = kind == FK_COMPLEX ? 1 : 0;
    const int epp = fk::elems_per_packet(fk::kF64, cplx);
    const size_t esz = (size_t)fk::elem_bytes(fk::kF64, cplx);
    // 16-byte packets: rows of ld elements must start on 16-byte boundaries; H values are read as
    // whole elements (double2 for FK_COMPLEX), row pointers and columns as 4-byte ints
    if (ld % epp != 0 || ((uintptr_t)d_R % 16) || ((uintptr_t)d_work % 16)) return FK_ERR_ARG;
    if (((uintptr_t)d_hs_val % esz) || ((uintptr_t)d_row_ptr % 4) || ((uintptr_t)d_col_idx % 4)) return FK_ERR_ARG;
    unsigned char* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != FK_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    const int P = (int)(ld / epp);
    int NP, Gp;
    if (P <= 32) { NP = 1; Gp = next_pow2(P); }
    else { NP = 4; Gp = std::min(32, next_pow2((P + 3) / 4)); }   // every lane holds packets
    int occ = 0;
    if (fk::occupancy_f64(fk::kStep, cplx, b, NP, 0, &occ) != cudaSuccess || occ < 1) { cudaGetLastError(); return FK_ERR_CUDA; }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = ((long long)n_b * Gp + fk::kThreads - 1) / fk::kThreads;
    long long ctas = tiles;
    if (ctas > (long long)occ * sms) ctas = (long long)occ * sms;
    if (ctas > kMaxCtas) ctas = kMaxCtas;
    if (ctas < 1) ctas = 1;

    fk::SysDesc* sys = reinterpret_cast<fk::SysDesc*>(scratch + kSysOff);
    int* cta_sys = reinterpret_cast<int*>(scratch + kCtaOff);
    double* partials = reinterpret_cast<double*>(scratch + kPartialsOff);
    double* raw = reinterpret_cast<double*>(scratch + kRawOff);
    k_noalloc_sys<<<(kMaxCtas + 255) / 256, 256, 0, st>>>(sys, cta_sys, n_b, (int)ctas);
    if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;

    const size_t vec = (size_t)n_b * b * (size_t)ld;   // elements per vector
    char* W0 = reinterpret_cast<char*>(d_work);
    char* W1 = W0 + vec * esz;
    char* Wv[2] = {W0, W1};
    const int nsteps = M / 2;
    for (int m = 0; m < nsteps; m++) {
        // m = 0: alpha_1 = Hs R -> W0;  m = 1: W0, R -> W1;  m >= 2: x = W[(m-1)&1], z = y = W[m&1]
        fk::StepArgs a;
        a.sys = sys;
        a.cta_sys = cta_sys;
        a.Gp = Gp;
        a.P = P;
        a.ld = ld;
        a.row_ptr = d_row_ptr;
        a.colc = reinterpret_cast<const unsigned*>(d_col_idx);   // no class bits: general blocks
        a.hval = d_hs_val;
        a.x = m == 0 ? (const void*)d_R : (const void*)Wv[(m - 1) & 1];
        a.z = m == 0 ? nullptr : (m == 1 ? (const void*)d_R : (const void*)Wv[m & 1]);
        a.y = m == 0 ? (void*)W0 : (void*)Wv[m & 1];
        a.xi = nullptr;
        a.coef = nullptr;
        a.cstride = 0;
        a.two = m > 0;
        a.has_z = m > 0;
        a.want_dots = 1;
        a.xi_mode = 0;
        a.partials = partials;
        a.stage_cap = 0;
        a.pipe = 0;
        if (fk::launch_step_f64(cplx, b, NP, a, fk::Launch{(int)ctas, 0, st}) != cudaSuccess) { cudaGetLastError(); return FK_ERR_CUDA; }
        k_noalloc_reduce<<<1, 32, 0, st>>>(partials, (int)ctas, raw + 2 * m);
        if (cudaGetLastError() != cudaSuccess) return FK_ERR_CUDA;
    }
    // the per-step sums have mu's layout: mu[2m] = <a_m, a_m>, mu[2m+1] = Re<a_{m+1}, a_m>
    if (cudaMemcpyAsync(mu, raw, sizeof(double) * M, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return FK_ERR_CUDA;
    }
    for (int m = 1; m < nsteps; m++) {
        mu[2 * m] = 2 * mu[2 * m] - mu[0];
        mu[2 * m + 1] = 2 * mu[2 * m + 1] - mu[1];
    }
    return FK_OK;
}
