// fk_post.cuh -- KPM post-processing on the device: moments from the per-step sums,
// the Jackson-damped density on Chebyshev nodes (moment_transform), the chemical
// potential for a filling, the electronic energy, the expansion coefficients at that
// chemical potential and the autodiff coefficient table, so that a fixed-filling solve
// (moments -> filling -> coefficients -> autodiff_matrix) never leaves the device
// between its stages. Each kernel restates a function of the reference's
// src/fastkpm.cpp (lines cited per kernel); all sums run in a fixed order.
#pragma once
#include <cuda_runtime.h>

namespace fk {

constexpr double kPi = 3.141592653589793238463;
constexpr int kPostThreads = 256;

// fermi_density (kind 0) and fermi_energy (kind 1), src/fastkpm.cpp:375-393
__device__ __forceinline__ double dev_fermi(int kind, double x, double kT, double mu) {
    const double a = (x - mu) / fabs(kT);
    if (kT < 1e-15 || fabs(a) > 20) return kind == 0 ? (x < mu ? 1.0 : 0.0) : (x < mu ? (x - mu) : 0.0);
    return kind == 0 ? 1.0 / (exp(a) + 1.0) : -kT * log(1.0 + exp(-a));
}

// Jackson damping g_m, src/fastkpm.cpp:13-20
__device__ __forceinline__ double dev_jackson(int m, int M) {
    const double Mp = M + 1.0;
    return ((Mp - m) * cos(kPi * m / Mp) + sin(kPi * m / Mp) / tan(kPi / Mp)) / Mp;
}

// Fixed-order block sum over kPostThreads threads; every thread gets the result.
__device__ __forceinline__ double post_block_sum(double v, double* red) {
    __syncthreads();
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = kPostThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    return red[0];
}

// mu_0 = <a0,a0>, mu_1 = Re<a1,a0>, mu_2m = 2<a_m,a_m> - mu_0, mu_2m+1 = 2 Re<a_m+1,a_m> - mu_1
// from the per-step sums raw[2m], raw[2m+1] (the reference's moments(), engine_cpu.cpp:63-84).
static __global__ void k_moments_from_raw(const double* raw, int M, double* mu) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int h = m / 2;
    mu[m] = h == 0 ? raw[m] : 2 * raw[m] - raw[m & 1];
}

// gamma_i = sum_m (m == 0 ? 1 : 2) mu_m g_m T_m(x_i), x_i = cos(pi (i + 1/2) / Mq), with T_m from
// the three-term recurrence (moment_transform, src/fastkpm.cpp:236-256; chebyshev_fill_array :30-39).
// E_i = es.unscale(x_i) is stored beside gamma for the filling solve.
static __global__ void k_moment_transform(const double* mu, int M, int Mq, double avg, double mag, double* gamma,
                                          double* energies) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Mq) return;
    const double x = cos(kPi * (i + 0.5) / Mq);
    double t0 = 1.0, t1 = x, acc = 0.0;
    for (int m = 0; m < M; m++) {
        const double T = m == 0 ? 1.0 : (m == 1 ? x : 2 * x * t1 - t0);
        if (m >= 2) { t0 = t1; t1 = T; }
        acc += (m == 0 ? 1.0 : 2.0) * mu[m] * dev_jackson(m, M) * T;
    }
    gamma[i] = acc;
    energies[i] = x * mag + avg;
}

// Chemical potential for a filling and the electronic energy (one CTA of kPostThreads):
//   kT' = max(kT, 0.1 mag / Mq) (thermal smearing), bracket [lo - max(c, 0), hi + max(-c, 0)],
//   c = kT' log(1/filling - 1); root of mu_to_filling(gamma, kT', mu) = filling (+-delta, averaged)
//   by bisection (filling_to_mu, src/fastkpm.cpp:418-432; the reference solves the same bracket
//   with toms748 to 30 bits); energy = electronic_energy(gamma, es, kT, filling, mu) (:452-456).
// out = {mu, energy, n_tot} with n_tot = sum_i gamma_i / Mq.
static __global__ void k_filling_solve(const double* gamma, const double* energies, int Mq, double lo, double hi,
                                       double kT, double filling, double delta, double* out) {
    __shared__ double red[kPostThreads];
    double part = 0.0;
    for (int i = threadIdx.x; i < Mq; i += kPostThreads) part += gamma[i];
    const double tot = post_block_sum(part, red);
    const double mag = (hi - lo) / 2;
    const double kTs = fmax(kT, 0.1 * mag / Mq);
    const double c = kTs * log(1.0 / filling - 1.0);
    const double lo0 = lo - fmax(c, 0.0), hi0 = hi + fmax(-c, 0.0);
    double roots[2];
    const int nroots = delta == 0.0 ? 1 : 2;
    for (int r = 0; r < nroots; r++) {
        const double target = r == 0 ? filling + delta : filling - delta;
        double a = lo0, b = hi0;
        for (int it = 0; it < 200; it++) {
            const double mid = 0.5 * (a + b);
            double occ = 0.0;
            for (int i = threadIdx.x; i < Mq; i += kPostThreads) occ += gamma[i] * dev_fermi(0, energies[i], kTs, mid);
            occ = post_block_sum(occ, red);
            if (occ / tot - target < 0) a = mid; else b = mid;
            if (b - a <= 1e-14 * fmax(1.0, fabs(mid))) break;
        }
        roots[r] = 0.5 * (a + b);
    }
    const double mu = nroots == 1 ? roots[0] : 0.5 * (roots[0] + roots[1]);
    double ge = 0.0;
    for (int i = threadIdx.x; i < Mq; i += kPostThreads) ge += gamma[i] * dev_fermi(1, energies[i], kT, mu);
    ge = post_block_sum(ge, red);
    if (threadIdx.x == 0) {
        out[0] = mu;
        out[1] = ge / Mq + mu * (tot / Mq) * filling;
        out[2] = tot / Mq;
    }
}

// One CTA per order m: c_m = (m == 0 ? 1 : 2) g_m (1/Mq) sum_i f(E_i) T_m(x_i), x_i = cos(pi (i + 1/2) / Mq),
// T_m(x_i) = cos(m pi (i + 1/2) / Mq) (expansion_coefficients, src/fastkpm.cpp:41-78, its non-FFTW
// branch); the node sum is reduced in a fixed order. The chemical potential is *mu_dev when given.
static __global__ void k_expansion_coefficients(int M, int Mq, int kind, double kT, double mu, const double* mu_dev,
                                                double avg, double mag, double* out) {
    const int m = blockIdx.x;
    if (m >= M) return;
    __shared__ double red[kPostThreads];
    const double mu_ = mu_dev ? *mu_dev : mu;
    double acc = 0.0;
    for (int i = threadIdx.x; i < Mq; i += kPostThreads) {
        const double th = kPi * (i + 0.5) / Mq;
        acc += dev_fermi(kind, cos(th) * mag + avg, kT, mu_) * cos(m * th);
    }
    acc = post_block_sum(acc, red);
    if (threadIdx.x == 0) out[m] = (m == 0 ? 1.0 : 2.0) * dev_jackson(m, M) * acc / Mq;
}

// The autodiff coefficient table from device coefficients c[0..M): per adjoint step q
// (m = M/2-1-q): {4 c_2m, 2 c_2m+1, m > 1 ? 2 c_2m-1 : diag}, then {2 c_{M-1}, diag} with
// diag = c_1 - sum_{m=1}^{M/2-1} c_{2m+1} (the reference's autodiff_matrix, engine_cpu.cpp:255-304).
static __global__ void k_adjoint_coefs(const double* c, int M, double* coef) {
    const int nsteps = M / 2 - 1;
    const int nadj = 3 * (nsteps > 1 ? nsteps : 1);
    __shared__ double s_diag;
    if (threadIdx.x == 0) {
        double d = c[1];
        for (int m = 1; m < M / 2; m++) d -= c[2 * m + 1];
        s_diag = d;
        coef[nadj] = 2 * c[M - 1];
        coef[nadj + 1] = d;
        if (nsteps < 1) { coef[0] = coef[1] = coef[2] = 0.0; }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nsteps; q += blockDim.x) {
        const int m = M / 2 - 1 - q;
        coef[3 * q + 0] = 4 * c[2 * m];
        coef[3 * q + 1] = 2 * c[2 * m + 1];
        coef[3 * q + 2] = m > 1 ? 2 * c[2 * m - 1] : s_diag;
    }
}

}  // namespace fk
