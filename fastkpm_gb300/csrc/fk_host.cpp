// fk_host.cpp -- host side of the drop-in: fkpm::SpMatBsr, probe generation,
// KPM helper math, the GB300 Engine<T> (which calls the C ABI in fk_engine.cu),
// its factories, and the host-helper entry points of include/fastkpm_gb300.h.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>

#include "../../include/fastkpm.h"
#include "../../include/fastkpm_gb300.h"

namespace fkpm {

// ============================== SpMatElems / SpMatBsr ==============================
// Semantics of reference src/spmat.cpp:8-198.

template <typename T>
SpMatElems<T>::SpMatElems(int n_rows, int n_cols, int b_len) : n_rows(n_rows), n_cols(n_cols), b_len(b_len) {}
template <typename T>
int SpMatElems<T>::n_blocks() const { return (int)row_idx.size(); }
template <typename T>
void SpMatElems<T>::clear() { row_idx.clear(); col_idx.clear(); val.clear(); }
template <typename T>
void SpMatElems<T>::add(int i, int j, T const* v) {
    if (i < 0 || i >= n_rows || j < 0 || j >= n_cols) throw std::out_of_range("SpMatElems::add: index out of range");
    row_idx.push_back(i);
    col_idx.push_back(j);
    val.insert(val.end(), v, v + b_len * b_len);
}

template <typename T>
SpMatBsr<T>::SpMatBsr() {}
template <typename T>
SpMatBsr<T>::SpMatBsr(SpMatElems<T> const& elems) { build(elems); }

// Blocks ordered by (row, col), duplicates summed in their input order.
template <typename T>
void SpMatBsr<T>::build(SpMatElems<T> const& elems) {
    n_rows = elems.n_rows;
    n_cols = elems.n_cols;
    b_len = elems.b_len;
    const int ne = elems.n_blocks(), bb = b_len * b_len;
    std::vector<int> order(ne);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
        return elems.row_idx[p] != elems.row_idx[q] ? elems.row_idx[p] < elems.row_idx[q]
                                                    : elems.col_idx[p] < elems.col_idx[q];
    });
    row_idx.clear(); col_idx.clear(); val.clear();
    row_ptr.assign(n_rows + 1, 0);
    for (int p : order) {
        const int i = elems.row_idx[p], j = elems.col_idx[p];
        const T* src = &elems.val[size_t(bb) * p];
        if (!row_idx.empty() && row_idx.back() == i && col_idx.back() == j) {
            T* dst = &val[val.size() - bb];
            for (int q = 0; q < bb; q++) dst[q] += src[q];
        } else {
            row_idx.push_back(i);
            col_idx.push_back(j);
            val.insert(val.end(), src, src + bb);
            row_ptr[i + 1]++;
        }
    }
    for (int i = 0; i < n_rows; i++) row_ptr[i + 1] += row_ptr[i];
}

template <typename T>
int SpMatBsr<T>::n_blocks() const { return (int)row_idx.size(); }
template <typename T>
void SpMatBsr<T>::clear() { row_idx.clear(); col_idx.clear(); row_ptr.clear(); val.clear(); }
template <typename T>
int SpMatBsr<T>::find_index(int i, int j) const {
    auto lo = col_idx.begin() + row_ptr[i], hi = col_idx.begin() + row_ptr[i + 1];
    auto it = std::lower_bound(lo, hi, j);
    if (it == hi || *it != j)
        throw std::out_of_range("SpMatBsr: block (" + std::to_string(i) + "," + std::to_string(j) + ") not stored");
    return int(it - col_idx.begin());
}
template <typename T>
T* SpMatBsr<T>::operator()(int i, int j) { return &val[size_t(b_len) * b_len * find_index(i, j)]; }
template <typename T>
T const* SpMatBsr<T>::operator()(int i, int j) const { return &val[size_t(b_len) * b_len * find_index(i, j)]; }
template <typename T>
void SpMatBsr<T>::zeros() { std::fill(val.begin(), val.end(), T(0)); }
template <typename T>
void SpMatBsr<T>::symmetrize() {
    for (int k = 0; k < n_blocks(); k++) {
        const int i = row_idx[k], j = col_idx[k];
        if (i < j) continue;
        T* v1b = &val[size_t(b_len) * b_len * k];
        T* v2b = (*this)(j, i);
        for (int bj = 0; bj < b_len; bj++)
            for (int bi = 0; bi < b_len; bi++) {
                T* v1 = &v1b[bj * b_len + bi];
                T* v2 = &v2b[bi * b_len + bj];
                const T sym = (*v1 + conj(*v2)) / T(2);
                *v1 = sym;
                *v2 = conj(sym);
            }
    }
}
template <typename T>
void SpMatBsr<T>::scale(T alpha) { for (auto& v : val) v *= alpha; }

template class SpMatElems<float>;
template class SpMatElems<double>;
template class SpMatElems<cx_float>;
template class SpMatElems<cx_double>;
template class SpMatBsr<float>;
template class SpMatBsr<double>;
template class SpMatBsr<cx_float>;
template class SpMatBsr<cx_double>;

// ================================== KPM math ==================================
// Reference src/fastkpm.cpp; the expansion uses the direct-sum branch.

Vec<double> jackson_kernel(int M) {
    Vec<double> g(M);
    const double Mp = M + 1.0;
    for (int m = 0; m < M; m++) g[m] = ((Mp - m) * std::cos(Pi * m / Mp) + std::sin(Pi * m / Mp) / std::tan(Pi / Mp)) / Mp;
    return g;
}
Vec<double> lorentz_kernel(int M, double lambda) {
    Vec<double> g(M);
    for (int m = 0; m < M; m++) g[m] = std::sinh(lambda * (1.0 - double(m) / M)) / std::sinh(lambda);
    return g;
}
void chebyshev_fill_array(double x, Vec<double>& ret, int kind) {
    if (kind != 1 && kind != 2) throw std::invalid_argument("chebyshev_fill_array: kind must be 1 or 2");
    if (!ret.empty()) ret[0] = 1.0;
    if (ret.size() > 1) ret[1] = kind * x;
    for (size_t m = 2; m < ret.size(); m++) ret[m] = 2 * x * ret[m - 1] - ret[m - 2];
}
Vec<double> expansion_coefficients(int M, int Mq, std::function<double(double)> f, EnergyScale es) {
    if (Mq < M) throw std::invalid_argument("expansion_coefficients: Mq must be >= M");
    const Vec<double> g = jackson_kernel(M);
    Vec<double> acc(M, 0.0), T(M);
    for (int i = 0; i < Mq; i++) {
        const double x = std::cos(Pi * (i + 0.5) / Mq);
        const double fi = f(es.unscale(x));
        chebyshev_fill_array(x, T);
        for (int m = 0; m < M; m++) acc[m] += fi * T[m];
    }
    Vec<double> c(M);
    for (int m = 0; m < M; m++) c[m] = (m == 0 ? 1.0 : 2.0) * g[m] * acc[m] / Mq;
    return c;
}
double moment_product(Vec<double> const& c, Vec<double> const& mu) {
    double r = 0;
    for (size_t i = 0; i < c.size(); i++) r += c[i] * mu[i];
    return r;
}
cx_double moment_product(Vec<Vec<cx_double>> const& c, Vec<Vec<cx_double>> const& mu) {
    cx_double r(0.0, 0.0);
    for (size_t a = 0; a < c.size(); a++)
        for (size_t b = 0; b < c[a].size(); b++) r += c[a][b] * mu[a][b];
    return r;
}
// Kubo-Bastin coefficients of the conductivity, src/fastkpm.cpp:80-233 (the direct-sum branch
// without FFTW): static (omega = 0) and optical (0 < omega < 2 mag) forms on the Chebyshev
// nodes, points within `cutoff` of the band edges skipped, scaled by the kernel and 2 pi.
Vec<Vec<cx_double>> electrical_conductivity_coefficients(int M, int Mq, double kT, double mu, double omega,
                                                         EnergyScale es, Vec<double> const& kernel) {
    if ((int)kernel.size() != M) throw std::invalid_argument("electrical_conductivity_coefficients: kernel size != M");
    if (Mq < 2 * M) throw std::invalid_argument("electrical_conductivity_coefficients: need Mq >= 2 M");
    if (omega < 0.0) throw std::invalid_argument("electrical_conductivity_coefficients: omega must be >= 0");
    const double cutoff = 1e-4;
    const double ws = omega / es.mag();
    Vec<Vec<cx_double>> ret(M, Vec<cx_double>(M, cx_double(0.0, 0.0)));
    if (ws >= 2.0) return ret;
    Vec<double> Ta(M), Tb(M);
    if (ws < 1.0e-10) {
        for (int i = 0; i < Mq; i++) {
            const double x = std::cos(Pi * (i + 0.5) / Mq);
            const double one_m = 1.0 - x * x;
            if (one_m < cutoff) continue;
            chebyshev_fill_array(x, Ta);            // T_m(x) = cos(m theta)
            chebyshev_fill_array(x, Tb, 2);         // U_m(x); sin(m theta) = sqrt(1-x^2) U_{m-1}(x)
            const double sq = std::sqrt(one_m);
            for (int m = M - 1; m > 0; m--) Tb[m] = Tb[m - 1] * sq;
            Tb[0] = 0.0;
            const double f = fermi_density(es.unscale(x), kT, mu) / std::pow(one_m, 1.5);
            for (int m1 = 0; m1 < M; m1++)
                for (int m2 = 0; m2 < M; m2++)
                    ret[m1][m2] += (Ta[m1] * cx_double(Ta[m2], -Tb[m2]) * cx_double(x, m2 * sq) +
                                    Ta[m2] * cx_double(Ta[m1], Tb[m1]) * cx_double(x, -m1 * sq)) * f;
        }
    } else {
        const int i_start = (int)std::ceil(std::acos(1.0 - ws) / Pi * Mq - 0.5);
        if (Mq - i_start < 20) throw std::invalid_argument("electrical_conductivity_coefficients: omega too large for Mq");
        for (int i = i_start; i < Mq; i++) {
            const double x = std::cos(Pi * (i + 0.5) / Mq);
            const double xw = x + ws;
            if (x < -1.0 + cutoff || xw > 1.0 - cutoff) continue;
            chebyshev_fill_array(xw, Ta);
            chebyshev_fill_array(x, Tb);
            const double E = es.unscale(x);
            const double f = (fermi_density(E, kT, mu) - fermi_density(E + omega, kT, mu)) / (ws * std::sqrt(1.0 - xw * xw));
            for (int m1 = 0; m1 < M; m1++)
                for (int m2 = 0; m2 < M; m2++) ret[m1][m2] += Ta[m1] * Tb[m2] * f;
        }
    }
    for (int m1 = 0; m1 < M; m1++) {
        const double p1 = 2.0 * Pi * (m1 == 0 ? 1.0 : 2.0) * kernel[m1] / (Mq * es.mag() * es.mag());
        for (int m2 = 0; m2 < M; m2++) ret[m1][m2] *= p1 * (m2 == 0 ? 1.0 : 2.0) * kernel[m2];
    }
    return ret;
}

// Two-dimensional moment_transform (src/fastkpm.cpp:258-289): gamma[i][j] =
// sum_{m1,m2} T_m1(x_i) T_m2(x_j) mup[m1][m2], mup = (m1?2:1)(m2?2:1) g_m1 g_m2 mu[m1][m2],
// evaluated as two matrix products (T^T mup, then by T) instead of the reference's fourfold loop.
Vec<Vec<cx_double>> moment_transform(Vec<Vec<cx_double>> const& moments, int Mq, Vec<double> const& kernel) {
    const int M = (int)moments.size();
    Vec<double> T((size_t)Mq * M), row(M);
    for (int i = 0; i < Mq; i++) {
        chebyshev_fill_array(std::cos(Pi * (i + 0.5) / Mq), row);
        std::copy(row.begin(), row.end(), T.begin() + (size_t)i * M);
    }
    std::vector<cx_double> mup((size_t)M * M), half((size_t)Mq * M, cx_double(0.0, 0.0));
    for (int a = 0; a < M; a++)
        for (int b = 0; b < M; b++)
            mup[(size_t)a * M + b] = ((a == 0 ? 1.0 : 2.0) * (b == 0 ? 1.0 : 2.0) * kernel[a] * kernel[b]) * moments[a][b];
    for (int i = 0; i < Mq; i++)        // half[i][m2] = sum_m1 T_m1(x_i) mup[m1][m2]
        for (int a = 0; a < M; a++) {
            const double t = T[(size_t)i * M + a];
            for (int b = 0; b < M; b++) half[(size_t)i * M + b] += t * mup[(size_t)a * M + b];
        }
    Vec<Vec<cx_double>> gamma(Mq, Vec<cx_double>(Mq, cx_double(0.0, 0.0)));
    for (int i = 0; i < Mq; i++)
        for (int j = 0; j < Mq; j++) {
            cx_double acc(0.0, 0.0);
            for (int b = 0; b < M; b++) acc += T[(size_t)j * M + b] * half[(size_t)i * M + b];
            gamma[i][j] = acc;
        }
    return gamma;
}

// Two-dimensional density_function (src/fastkpm.cpp:335-361)
void density_function(Vec<Vec<cx_double>> const& gamma, EnergyScale es, Vec<double>& x, Vec<double>& y,
                      Vec<Vec<cx_double>>& rho) {
    const int Mq1 = (int)gamma.size(), Mq2 = Mq1 ? (int)gamma[0].size() : 0;
    x.assign(Mq1, 0.0);
    y.assign(Mq2, 0.0);
    rho.assign(Mq1, Vec<cx_double>(Mq2, cx_double(0.0, 0.0)));
    for (int i2 = 0; i2 < Mq2; i2++) y[Mq2 - 1 - i2] = es.unscale(std::cos(Pi * (i2 + 0.5) / Mq2));
    for (int i1 = 0; i1 < Mq1; i1++) {
        const double x1 = std::cos(Pi * (i1 + 0.5) / Mq1);
        x[Mq1 - 1 - i1] = es.unscale(x1);
        for (int i2 = 0; i2 < Mq2; i2++) {
            const double x2 = std::cos(Pi * (i2 + 0.5) / Mq2);
            rho[Mq1 - 1 - i1][Mq2 - 1 - i2] =
                gamma[i1][i2] / (Pi * std::sqrt(1.0 - x1 * x1) * Pi * std::sqrt(1.0 - x2 * x2) * es.mag() * es.mag());
        }
    }
}

Vec<double> moment_transform(Vec<double> const& moments, int Mq) {
    const int M = (int)moments.size();
    const Vec<double> g = jackson_kernel(M);
    Vec<double> T(M), gamma(Mq, 0.0);
    for (int i = 0; i < Mq; i++) {
        chebyshev_fill_array(std::cos(Pi * (i + 0.5) / Mq), T);
        for (int m = 0; m < M; m++) gamma[i] += (m == 0 ? 1 : 2) * moments[m] * g[m] * T[m];
    }
    return gamma;
}
double density_product(Vec<double> const& gamma, std::function<double(double)> f, EnergyScale es) {
    const int Mq = (int)gamma.size();
    double r = 0.0;
    for (int i = 0; i < Mq; i++) r += gamma[i] * f(es.unscale(std::cos(Pi * (i + 0.5) / Mq)));
    return r / Mq;
}
void density_function(Vec<double> const& gamma, EnergyScale es, Vec<double>& x, Vec<double>& rho) {
    const int Mq = (int)gamma.size();
    x.resize(Mq);
    rho.resize(Mq);
    for (int i = Mq - 1; i >= 0; i--) {
        const double xi = std::cos(Pi * (i + 0.5) / Mq);
        x[Mq - 1 - i] = es.unscale(xi);
        rho[Mq - 1 - i] = gamma[i] / (Pi * std::sqrt(1 - xi * xi) * es.mag());
    }
}
void integrated_density_function(Vec<double> const& gamma, EnergyScale es, Vec<double>& x, Vec<double>& irho) {
    const int Mq = (int)gamma.size();
    x.resize(Mq);
    irho.resize(Mq);
    double acc = 0.0;
    for (int i = Mq - 1; i >= 0; i--) {
        x[Mq - 1 - i] = es.unscale(std::cos(Pi * (i + 0.5) / Mq));
        irho[Mq - 1 - i] = (acc + 0.5 * gamma[i]) / Mq;
        acc += gamma[i];
    }
}
double fermi_energy(double x, double kT, double mu) {
    const double a = (x - mu) / std::fabs(kT);
    if (kT < 1e-15 || std::fabs(a) > 20) return (x < mu) ? (x - mu) : 0.0;
    return -kT * std::log(1 + std::exp(-a));
}
double fermi_density(double x, double kT, double mu) {
    const double a = (x - mu) / std::fabs(kT);
    if (kT < 1e-15 || std::fabs(a) > 20) return (x < mu) ? 1.0 : 0.0;
    return 1.0 / (std::exp(a) + 1.0);
}
double mu_to_filling(Vec<double> const& gamma, EnergyScale const& es, double kT, double mu) {
    const double occ = density_product(gamma, [&](double x) { return fermi_density(x, kT, mu); }, es);
    const double tot = density_product(gamma, [](double) { return 1.0; }, es);
    return occ / tot;
}
// Chemical potential for a filling (src/fastkpm.cpp:418-432): thermal smearing
// kT' = max(kT, 0.1 mag / Mq), bracket [lo - max(c, 0), hi + max(-c, 0)] with
// c = kT' log(1/filling - 1), root of mu_to_filling(gamma, es, kT', mu) = filling
// (two roots at filling +- delta_filling, averaged, when delta_filling != 0). The
// reference solves with Boost's toms748 to 30 bits; this bisects to 1e-14, so the
// two agree to the reference's tolerance.
double filling_to_mu(Vec<double> const& gamma, EnergyScale const& es, double kT, double filling, double delta_filling) {
    const double kTs = std::max(kT, 0.1 * es.mag() / (double)gamma.size());
    const double c = kTs * std::log(1.0 / filling - 1.0);
    const double a0 = es.lo - std::max(c, 0.0), b0 = es.hi + std::max(-c, 0.0);
    auto root = [&](double target) {
        double a = a0, b = b0;
        for (int it = 0; it < 200; it++) {
            const double mid = 0.5 * (a + b);
            if (mu_to_filling(gamma, es, kTs, mid) - target < 0) a = mid;
            else b = mid;
            if (b - a <= 1e-14 * std::max(1.0, std::fabs(mid))) break;
        }
        return 0.5 * (a + b);
    };
    if (delta_filling == 0) return root(filling);
    return 0.5 * (root(filling + delta_filling) + root(filling - delta_filling));
}
double electronic_grand_energy(Vec<double> const& gamma, EnergyScale const& es, double kT, double mu) {
    return density_product(gamma, [&](double x) { return fermi_energy(x, kT, mu); }, es);
}
double electronic_energy(Vec<double> const& gamma, EnergyScale const& es, double kT, double filling, double mu) {
    const double n_tot = density_product(gamma, [](double) { return 1.0; }, es);
    return electronic_grand_energy(gamma, es, kT, mu) + mu * n_tot * filling;
}

// ================================== probes ==================================
// Reference src/engine.cpp:7-116. R must be bit-identical to the reference's for
// the same std::mt19937 state, so the same <random> distributions are used.

template <typename T> T random_phase(RNG& rng);
template <> double random_phase(RNG& rng) {
    std::uniform_int_distribution<int> two(0, 1);
    return 2 * two(rng) - 1;
}
template <> float random_phase(RNG& rng) { return float(random_phase<double>(rng)); }
template <> cx_double random_phase(RNG& rng) {
    std::uniform_int_distribution<int> four(0, 3);
    static const cx_double ph[4] = {{+1, 0}, {0, +1}, {-1, 0}, {0, -1}};
    return ph[four(rng)];
}
template <> cx_float random_phase(RNG& rng) { return cx_float(random_phase<cx_double>(rng)); }

template <typename T>
void Engine<T>::set_R_identity(int n, int j_start, int j_end) {
    if (!(0 <= j_start && j_start <= j_end && j_end <= n)) throw std::invalid_argument("set_R_identity: bad column range");
    R.set_size(n, j_end - j_start);
    for (int j = j_start; j < j_end; j++) R(j, j - j_start) = T(1.0);
    R2 = R;
    transfer_R();
}
template <typename T>
void Engine<T>::set_R_identity(int n) { set_R_identity(n, 0, n); }

template <typename T>
void Engine<T>::set_R_uncorrelated(int n, int s, RNG& rng, int j_start, int j_end) {
    if (!(0 <= j_start && j_start <= j_end && j_end <= s)) throw std::invalid_argument("set_R_uncorrelated: bad column range");
    R.set_size(n, j_end - j_start);
    const T x = T(1.0 / std::sqrt(s));
    for (int j = j_start; j < j_end; j++) {
        RNG rng_j(rng());   // each column draws its own generator seed from the master
        for (int i = 0; i < n; i++) R(i, j - j_start) = random_phase<T>(rng_j) * x;
    }
    R2 = R;
    transfer_R();
}
template <typename T>
void Engine<T>::set_R_uncorrelated(int n, int s, RNG& rng) { set_R_uncorrelated(n, s, rng, 0, s); }

template <typename T>
void Engine<T>::set_R_correlated(Vec<int> const& groups, RNG& rng, int j_start, int j_end) {
    const int n = (int)groups.size();
    if (!(0 <= j_start && j_start <= j_end && j_end <= n)) throw std::invalid_argument("set_R_correlated: bad column range");
    R.set_size(n, j_end - j_start);
    // bucket rows by group once instead of scanning all rows for every column
    std::vector<int> start(j_end - j_start + 1, 0), rows;
    for (int i = 0; i < n; i++) if (groups[i] >= j_start && groups[i] < j_end) start[groups[i] - j_start + 1]++;
    for (size_t q = 1; q < start.size(); q++) start[q] += start[q - 1];
    rows.resize(start.back());
    std::vector<int> fillp(start.begin(), start.end() - 1);
    for (int i = 0; i < n; i++) if (groups[i] >= j_start && groups[i] < j_end) rows[fillp[groups[i] - j_start]++] = i;
    for (int j = j_start; j < j_end; j++) {
        RNG rng_j(rng());
        for (int q = start[j - j_start]; q < start[j - j_start + 1]; q++) R(rows[q], j - j_start) = random_phase<T>(rng_j);
    }
    R2 = R;
    transfer_R();
}
template <typename T>
void Engine<T>::set_R_correlated(Vec<int> const& groups, RNG& rng) {
    if (groups.empty()) throw std::invalid_argument("set_R_correlated: empty groups");
    auto mm = std::minmax_element(groups.begin(), groups.end());
    if (*mm.first != 0) throw std::invalid_argument("set_R_correlated: groups must start at 0");
    const int n = (int)groups.size(), s = *mm.second + 1;
    if (s < n) set_R_correlated(groups, rng, 0, s);
    else set_R_identity(n, 0, n);
}

template class Engine<float>;
template class Engine<double>;
template class Engine<cx_float>;
template class Engine<cx_double>;

// ================================ GB300 engine ================================

namespace {
template <typename T> constexpr bool is_cx() { return std::is_same<T, cx_float>::value || std::is_same<T, cx_double>::value; }

[[noreturn]] void raise(fk_engine* e, int rc, const char* what) {
    std::string msg = std::string("fkpm: ") + what + ": " + fk_status_string(rc);
    if (e) { msg += " ("; msg += fk_engine_last_error(e); msg += ")"; }
    throw std::runtime_error(msg);
}

// values of T as interleaved doubles
template <typename T>
void to_doubles(const T* src, size_t n, std::vector<double>& dst) {
    if constexpr (is_cx<T>()) {
        dst.resize(2 * n);
        for (size_t q = 0; q < n; q++) { dst[2 * q] = double(src[q].real()); dst[2 * q + 1] = double(src[q].imag()); }
    } else {
        dst.resize(n);
        for (size_t q = 0; q < n; q++) dst[q] = double(src[q]);
    }
}
template <typename T>
void from_doubles(const double* src, size_t n, T* dst) {
    for (size_t q = 0; q < n; q++) {
        if constexpr (is_cx<T>()) dst[q] = T(src[2 * q], src[2 * q + 1]);
        else dst[q] = T(src[q]);
    }
}

Precision default_precision(bool single) {
    if (const char* p = std::getenv("FKPM_PRECISION")) {
        std::string s(p);
        if (s == "fp64") return Precision::FP64;
        if (s == "fp32") return Precision::FP32;
        if (s == "ds") return Precision::DS;
    }
    return single ? Precision::FP32 : Precision::FP64;
}
}  // namespace

template <typename T>
class Engine_GB300 : public Engine<T> {
    fk_engine* e_ = nullptr;
    EnergyScale es_{0, 0};
    int b_len_ = 0, n_rows_ = 0;
    std::vector<double> buf_;

    void check(int rc, const char* what) { if (rc != FK_OK) raise(e_, rc, what); }

public:
    Engine_GB300(int device, Precision p) {
        const int rc = fk_engine_create(device, is_cx<T>() ? FK_COMPLEX : FK_REAL, int(p), &e_);
        if (rc != FK_OK) raise(nullptr, rc, "engine creation");
    }
    ~Engine_GB300() override { fk_engine_destroy(e_); }
    fk_engine* handle() { return e_; }

    EnergyScale energy_scale(SpMatBsr<T> const& H, double extend, int iters) override {
        if (H.n_rows != H.n_cols) throw std::invalid_argument("energy_scale: H must be square");
        to_doubles(H.val.data(), H.val.size(), buf_);
        double lo = 0, hi = 0;
        check(fk_engine_energy_scale(e_, H.n_rows, H.b_len, H.n_blocks(), H.row_ptr.data(), H.col_idx.data(),
                                     buf_.data(), extend, iters, nullptr, &lo, &hi), "energy_scale");
        return {lo, hi};
    }

    void transfer_R() override {
        if (this->R.n_cols == 0) throw std::invalid_argument("transfer_R: cannot handle an empty R matrix");
        const double* src;
        if constexpr (std::is_same<T, double>::value || std::is_same<T, cx_double>::value) {
            src = reinterpret_cast<const double*>(this->R.memptr());   // std::complex<double> is (re, im)
        } else {
            to_doubles(this->R.memptr(), this->R.size(), buf_);
            src = buf_.data();
        }
        check(fk_engine_set_R(e_, this->R.n_rows, this->R.n_cols, src), "transfer_R");
    }

    void set_H(SpMatBsr<T> const& H, EnergyScale const& es) override {
        if (H.n_rows != H.n_cols) throw std::invalid_argument("set_H: H must be square");
        es_ = es;
        b_len_ = H.b_len;
        n_rows_ = H.n_rows;
        to_doubles(H.val.data(), H.val.size(), buf_);
        check(fk_engine_set_H(e_, H.n_rows, H.b_len, H.n_blocks(), H.row_ptr.data(), H.col_idx.data(), buf_.data(),
                              es.lo, es.hi), "set_H");
    }

    Vec<double> moments(int M) override {
        Vec<double> mu(M);
        check(fk_engine_moments(e_, M, mu.data()), "moments");
        return mu;
    }

    Vec<Vec<cx_double>> moments2_v1(int M, SpMatBsr<T> const& j1op, SpMatBsr<T> const& j2op, int a_chunk_ncols,
                                    int R_chunk_ncols) override {
        for (auto* j : {&j1op, &j2op})
            if (j->n_rows != n_rows_ || j->n_cols != n_rows_ || j->b_len != b_len_)
                throw std::invalid_argument("moments2_v1: j1 and j2 must have H's shape and block size");
        std::vector<double> v1, v2, out(2 * (size_t)M * M);
        to_doubles(j1op.val.data(), j1op.val.size(), v1);
        to_doubles(j2op.val.data(), j2op.val.size(), v2);
        check(fk_engine_moments2_v1(e_, M, j1op.n_blocks(), j1op.row_ptr.data(), j1op.col_idx.data(), v1.data(),
                                    j2op.n_blocks(), j2op.row_ptr.data(), j2op.col_idx.data(), v2.data(),
                                    a_chunk_ncols, R_chunk_ncols, out.data()),
              "moments2_v1");
        Vec<Vec<cx_double>> mu(M, Vec<cx_double>(M));
        for (int m1 = 0; m1 < M; m1++)
            for (int m2 = 0; m2 < M; m2++) {
                const size_t q = (size_t)m1 * M + m2;
                mu[m1][m2] = cx_double(out[2 * q], out[2 * q + 1]);
            }
        return mu;
    }
    // R2 must have R's shape (the reference asserts it, src/engine_cpu.cpp:174); an empty R2
    // means R2 = R. The chunk arguments are unused, as in the reference.
    Vec<Vec<cx_double>> moments2_v2(int M, SpMatBsr<T> const& j1op, SpMatBsr<T> const& j2op, int, int) override {
        for (auto* j : {&j1op, &j2op})
            if (j->n_rows != n_rows_ || j->n_cols != n_rows_ || j->b_len != b_len_)
                throw std::invalid_argument("moments2_v2: j1 and j2 must have H's shape and block size");
        const bool own_r2 = this->R2.size() != 0;
        if (own_r2 && (this->R2.n_rows != this->R.n_rows || this->R2.n_cols != this->R.n_cols))
            throw std::invalid_argument("moments2_v2: R2 must have R's shape");
        std::vector<double> v1, v2, r2, out(2 * (size_t)M * M);
        to_doubles(j1op.val.data(), j1op.val.size(), v1);
        to_doubles(j2op.val.data(), j2op.val.size(), v2);
        if (own_r2) to_doubles(this->R2.memptr(), this->R2.size(), r2);
        check(fk_engine_moments2_v2(e_, M, j1op.n_blocks(), j1op.row_ptr.data(), j1op.col_idx.data(), v1.data(),
                                    j2op.n_blocks(), j2op.row_ptr.data(), j2op.col_idx.data(), v2.data(),
                                    own_r2 ? r2.data() : nullptr, out.data()),
              "moments2_v2");
        Vec<Vec<cx_double>> mu(M, Vec<cx_double>(M));
        for (int m1 = 0; m1 < M; m1++)
            for (int m2 = 0; m2 < M; m2++) {
                const size_t q = (size_t)m1 * M + m2;
                mu[m1][m2] = cx_double(out[2 * q], out[2 * q + 1]);
            }
        return mu;
    }

    void stoch_matrix(Vec<double> const& c, SpMatBsr<T>& D) override {
        if (D.n_rows != n_rows_ || D.n_cols != n_rows_ || D.b_len != b_len_)
            throw std::invalid_argument("stoch_matrix: D's shape must match H");
        std::vector<double> out(D.val.size() * (is_cx<T>() ? 2 : 1));
        check(fk_engine_stoch_matrix(e_, (int)c.size(), c.data(), D.n_rows, D.n_blocks(), D.row_ptr.data(),
                                     D.col_idx.data(), out.data()), "stoch_matrix");
        from_doubles(out.data(), D.val.size(), D.val.data());
    }

    void autodiff_matrix(Vec<double> const& c, SpMatBsr<T>& D) override {
        if (D.n_rows != n_rows_ || D.n_cols != n_rows_ || D.b_len != b_len_)
            throw std::invalid_argument("autodiff_matrix: D's shape must match H");
        std::vector<double> out(D.val.size() * (is_cx<T>() ? 2 : 1));
        check(fk_engine_autodiff_matrix(e_, (int)c.size(), c.data(), D.n_rows, D.n_blocks(), D.row_ptr.data(),
                                        D.col_idx.data(), out.data()), "autodiff_matrix");
        from_doubles(out.data(), D.val.size(), D.val.data());
    }
};

// Probe columns split over several devices (the reference's Engine_Threaded,
// src/engine_cusparse.cpp:1043-1168): every worker engine holds H and a contiguous slice of
// R's columns; moments and D are sums over probe columns, so the workers' results are added
// on the host in worker order (deterministic). set_R_* fill this engine's R exactly as one
// engine would (one draw of the master generator per column, the same columns the
// reference's per-worker generators produce), and transfer_R hands each worker its slice.
// Solves are enqueued on every worker's stream first and collected afterwards, so the
// devices run concurrently without a host thread per device; set_H, whose host preparation
// is the heavy part, runs one thread per worker. moments2_v2 couples all probe columns
// (traces over s x s products) and is not split: more than one worker throws.
template <typename T>
class Engine_Split : public Engine<T> {
    std::vector<std::shared_ptr<Engine_GB300<T>>> w_;
    std::vector<int> active_;   // workers that hold at least one probe column
    std::vector<double> buf_;

    static void check(fk_engine* e, int rc, const char* what) { if (rc != FK_OK) raise(e, rc, what); }
    template <class F>
    void parallel(F&& fn) {
        std::vector<std::thread> ts;
        std::vector<std::exception_ptr> errs(w_.size());
        for (size_t t = 0; t < w_.size(); t++)
            ts.emplace_back([&, t] { try { fn(t); } catch (...) { errs[t] = std::current_exception(); } });
        for (auto& th : ts) th.join();
        for (auto& e : errs) if (e) std::rethrow_exception(e);
    }
    template <class Enqueue>
    void d_sum(SpMatBsr<T>& D, Enqueue&& enqueue, const char* what) {
        if (active_.empty()) throw std::logic_error(std::string(what) + ": no probe block (call set_R_* first)");
        for (int t : active_) enqueue(w_[t]->handle());
        const size_t nv = D.val.size() * (is_cx<T>() ? 2 : 1);
        std::vector<double> acc(nv, 0.0), part(nv);
        for (int t : active_) {
            check(w_[t]->handle(), fk_engine_fetch_D(w_[t]->handle(), part.data()), what);
            for (size_t q = 0; q < nv; q++) acc[q] += part[q];
        }
        from_doubles(acc.data(), D.val.size(), D.val.data());
    }

public:
    Engine_Split(const Vec<int>& devices, Precision p) {
        for (int d : devices) w_.push_back(std::make_shared<Engine_GB300<T>>(d, p));
    }
    int workers() const { return (int)w_.size(); }

    EnergyScale energy_scale(SpMatBsr<T> const& H, double extend, int iters) override {
        return w_[0]->energy_scale(H, extend, iters);
    }
    void transfer_R() override {
        if (this->R.n_cols == 0) throw std::invalid_argument("transfer_R: cannot handle an empty R matrix");
        const int s = this->R.n_cols, n = this->R.n_rows, nw = (int)w_.size();
        active_.clear();
        for (int t = 0; t < nw; t++) {
            const int j1 = t * s / nw, j2 = (t + 1) * s / nw;   // the reference's contiguous column ranges
            if (j2 == j1) continue;
            Mat<T>& Rt = w_[t]->R;
            Rt.set_size(n, j2 - j1);
            std::copy(this->R.colptr(j1), this->R.colptr(j1) + (size_t)n * (j2 - j1), Rt.memptr());
            w_[t]->transfer_R();
            active_.push_back(t);
        }
    }
    void set_H(SpMatBsr<T> const& H, EnergyScale const& es) override {
        parallel([&](size_t t) { w_[t]->set_H(H, es); });
    }
    Vec<double> moments(int M) override {
        if (active_.empty()) throw std::logic_error("moments: no probe block (call set_R_* first)");
        for (int t : active_) check(w_[t]->handle(), fk_engine_moments_async(w_[t]->handle(), M), "moments");
        Vec<double> mu(M, 0.0), part(M);
        for (int t : active_) {
            check(w_[t]->handle(), fk_engine_fetch_moments(w_[t]->handle(), part.data()), "moments");
            for (int m = 0; m < M; m++) mu[m] += part[m];
        }
        return mu;
    }
    Vec<Vec<cx_double>> moments2_v1(int M, SpMatBsr<T> const& j1op, SpMatBsr<T> const& j2op, int a_chunk_ncols,
                                    int R_chunk_ncols) override {
        Vec<Vec<cx_double>> mu(M, Vec<cx_double>(M, cx_double(0.0, 0.0)));
        for (int t : active_) {
            auto part = w_[t]->moments2_v1(M, j1op, j2op, a_chunk_ncols, R_chunk_ncols);
            for (int m1 = 0; m1 < M; m1++)
                for (int m2 = 0; m2 < M; m2++) mu[m1][m2] += part[m1][m2];
        }
        return mu;
    }
    Vec<Vec<cx_double>> moments2_v2(int M, SpMatBsr<T> const& j1op, SpMatBsr<T> const& j2op, int a, int r) override {
        if (w_.size() > 1)
            throw std::logic_error("moments2_v2 couples all probe columns and is not split over devices: use one device");
        w_[0]->R2 = this->R2;
        return w_[0]->moments2_v2(M, j1op, j2op, a, r);
    }
    void stoch_matrix(Vec<double> const& c, SpMatBsr<T>& D) override {
        d_sum(D, [&](fk_engine* e) {
            check(e, fk_engine_stoch_matrix_async(e, (int)c.size(), c.data(), D.n_rows, D.n_blocks(), D.row_ptr.data(),
                                                  D.col_idx.data()), "stoch_matrix");
        }, "stoch_matrix");
    }
    void autodiff_matrix(Vec<double> const& c, SpMatBsr<T>& D) override {
        d_sum(D, [&](fk_engine* e) {
            check(e, fk_engine_autodiff_matrix_async(e, (int)c.size(), c.data(), D.n_rows, D.n_blocks(),
                                                     D.row_ptr.data(), D.col_idx.data()), "autodiff_matrix");
        }, "autodiff_matrix");
    }
};

template <typename T>
std::shared_ptr<Engine<T>> mk_engine_gb300(int device, Precision precision) {
    return std::make_shared<Engine_GB300<T>>(device, precision);
}
template <typename T>
std::shared_ptr<Engine<T>> mk_engine_cuSPARSE(Vec<int> devices) {
    const bool single = std::is_same<T, float>::value || std::is_same<T, cx_float>::value;
    if (devices.size() > 1) return std::make_shared<Engine_Split<T>>(devices, default_precision(single));
    return mk_engine_gb300<T>(devices.empty() ? 0 : devices[0], default_precision(single));
}
template <typename T>
std::shared_ptr<Engine<T>> mk_engine() {
    int count = 0;
    if (fk_device_count(&count) != FK_OK || count == 0)
        throw std::runtime_error("fkpm: no CUDA device available for the GB300 engine");
    return mk_engine_cuSPARSE<T>({});
}
template <typename T>
std::shared_ptr<Engine<T>> mk_engine_cpu() {
    throw std::runtime_error("fkpm: the CPU engine is not part of the GB300 build");
}
template <typename T>
std::shared_ptr<Engine<T>> mk_engine_mpi() {
    throw std::runtime_error("fkpm: the MPI engine is not part of the GB300 build (one GPU per process)");
}

#define FK_INST(T)                                                                          \
    template std::shared_ptr<Engine<T>> mk_engine_gb300<T>(int, Precision);                 \
    template std::shared_ptr<Engine<T>> mk_engine_cuSPARSE<T>(Vec<int>);                    \
    template std::shared_ptr<Engine<T>> mk_engine<T>();                                     \
    template std::shared_ptr<Engine<T>> mk_engine_cpu<T>();                                 \
    template std::shared_ptr<Engine<T>> mk_engine_mpi<T>();
FK_INST(float)
FK_INST(double)
FK_INST(cx_float)
FK_INST(cx_double)
#undef FK_INST

// ================================== timer ==================================
Timer::Timer() { reset(); }
void Timer::reset() { t0 = std::chrono::steady_clock::now(); }
double Timer::measure() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
Timer timer[10];

}  // namespace fkpm

// ============================ host-helper C ABI ============================
namespace {
template <typename T>
int bsr_build_c(int n_rows, int b, int ne, const int* ri, const int* ci, const double* v, int* orp, int* ori, int* oci,
                double* ov, int* nnzb) {
    fkpm::SpMatElems<T> el(n_rows, n_rows, b);
    const int cw = std::is_same<T, fkpm::cx_double>::value ? 2 : 1;
    for (int k = 0; k < ne; k++) {
        if (ri[k] < 0 || ri[k] >= n_rows || ci[k] < 0 || ci[k] >= n_rows) return FK_ERR_PATTERN;
        el.add(ri[k], ci[k], reinterpret_cast<const T*>(v + (size_t)k * b * b * cw));
    }
    fkpm::SpMatBsr<T> H(el);
    std::copy(H.row_ptr.begin(), H.row_ptr.end(), orp);
    std::copy(H.row_idx.begin(), H.row_idx.end(), ori);
    std::copy(H.col_idx.begin(), H.col_idx.end(), oci);
    std::memcpy(ov, H.val.data(), sizeof(T) * H.val.size());
    *nnzb = H.n_blocks();
    return FK_OK;
}
template <typename T>
int bsr_sym_c(int n_rows, int b, int nnzb, const int* rp, const int* ri, const int* ci, double* v) {
    fkpm::SpMatBsr<T> D;
    D.n_rows = D.n_cols = n_rows;
    D.b_len = b;
    D.row_ptr.assign(rp, rp + n_rows + 1);
    D.row_idx.assign(ri, ri + nnzb);
    D.col_idx.assign(ci, ci + nnzb);
    T* tv = reinterpret_cast<T*>(v);
    D.val.assign(tv, tv + (size_t)nnzb * b * b);
    try { D.symmetrize(); } catch (const std::out_of_range&) { return FK_ERR_PATTERN; }
    std::copy(D.val.begin(), D.val.end(), tv);
    return FK_OK;
}
// Probe generation through Engine<T>'s own set_R_* (transfer_R is a no-op here).
template <typename T>
struct ProbeOnly : fkpm::Engine<T> {
    fkpm::EnergyScale energy_scale(fkpm::SpMatBsr<T> const&, double, int) override { return {0, 0}; }
    void set_H(fkpm::SpMatBsr<T> const&, fkpm::EnergyScale const&) override {}
    fkpm::Vec<double> moments(int) override { return {}; }
    fkpm::Vec<fkpm::Vec<fkpm::cx_double>> moments2_v1(int, fkpm::SpMatBsr<T> const&, fkpm::SpMatBsr<T> const&, int, int) override { return {}; }
    fkpm::Vec<fkpm::Vec<fkpm::cx_double>> moments2_v2(int, fkpm::SpMatBsr<T> const&, fkpm::SpMatBsr<T> const&, int, int) override { return {}; }
    void stoch_matrix(fkpm::Vec<double> const&, fkpm::SpMatBsr<T>&) override {}
    void autodiff_matrix(fkpm::Vec<double> const&, fkpm::SpMatBsr<T>&) override {}
};
template <typename T>
void copy_R(const fkpm::Mat<T>& R, double* out) {
    std::memcpy(out, R.memptr(), sizeof(T) * R.size());
}
}  // namespace

extern "C" {

int fk_bsr_build(int kind, int n_rows, int b, int n_elems, const int* ri, const int* ci, const double* v, int* orp,
                 int* ori, int* oci, double* ov, int* nnzb) {
    if (n_rows <= 0 || b <= 0 || n_elems < 0 || !orp || !nnzb) return FK_ERR_ARG;
    return kind == FK_COMPLEX ? bsr_build_c<fkpm::cx_double>(n_rows, b, n_elems, ri, ci, v, orp, ori, oci, ov, nnzb)
                              : bsr_build_c<double>(n_rows, b, n_elems, ri, ci, v, orp, ori, oci, ov, nnzb);
}

int fk_bsr_symmetrize(int kind, int n_rows, int b, int nnzb, const int* rp, const int* ri, const int* ci, double* v) {
    if (n_rows <= 0 || b <= 0 || nnzb < 0 || !rp) return FK_ERR_ARG;
    return kind == FK_COMPLEX ? bsr_sym_c<fkpm::cx_double>(n_rows, b, nnzb, rp, ri, ci, v)
                              : bsr_sym_c<double>(n_rows, b, nnzb, rp, ri, ci, v);
}

int fk_probe_identity(int kind, int n, int j0, int j1, double* R) {
    if (!R || !(0 <= j0 && j0 <= j1 && j1 <= n)) return FK_ERR_ARG;
    if (kind == FK_COMPLEX) { ProbeOnly<fkpm::cx_double> p; p.set_R_identity(n, j0, j1); copy_R(p.R, R); }
    else { ProbeOnly<double> p; p.set_R_identity(n, j0, j1); copy_R(p.R, R); }
    return FK_OK;
}

int fk_probe_uncorrelated(int kind, int n, int s, uint32_t seed, unsigned long long discard, int j0, int j1, double* R) {
    if (!R || !(0 <= j0 && j0 <= j1 && j1 <= s) || n <= 0) return FK_ERR_ARG;
    fkpm::RNG rng(seed);
    rng.discard(discard);
    if (kind == FK_COMPLEX) { ProbeOnly<fkpm::cx_double> p; p.set_R_uncorrelated(n, s, rng, j0, j1); copy_R(p.R, R); }
    else { ProbeOnly<double> p; p.set_R_uncorrelated(n, s, rng, j0, j1); copy_R(p.R, R); }
    return FK_OK;
}

int fk_probe_correlated(int kind, int n, const int* groups, uint32_t seed, unsigned long long discard, int j0, int j1,
                        double* R) {
    if (!R || !groups || !(0 <= j0 && j0 <= j1 && j1 <= n)) return FK_ERR_ARG;
    fkpm::RNG rng(seed);
    rng.discard(discard);
    fkpm::Vec<int> g(groups, groups + n);
    if (kind == FK_COMPLEX) { ProbeOnly<fkpm::cx_double> p; p.set_R_correlated(g, rng, j0, j1); copy_R(p.R, R); }
    else { ProbeOnly<double> p; p.set_R_correlated(g, rng, j0, j1); copy_R(p.R, R); }
    return FK_OK;
}

int fk_jackson_kernel(int M, double* out) {
    if (M < 0 || (!out && M > 0)) return FK_ERR_ARG;
    const auto g = fkpm::jackson_kernel(M);
    std::copy(g.begin(), g.end(), out);
    return FK_OK;
}

int fk_expansion_coefficients(int M, int Mq, int f_kind, double kT, double mu, double lo, double hi, double* out) {
    if (M < 1 || Mq < M || !out || (f_kind != 0 && f_kind != 1) || !(hi > lo)) return FK_ERR_ARG;
    fkpm::EnergyScale es{lo, hi};
    auto f = [&](double x) { return f_kind == 0 ? fkpm::fermi_density(x, kT, mu) : fkpm::fermi_energy(x, kT, mu); };
    const auto c = fkpm::expansion_coefficients(M, Mq, f, es);
    std::copy(c.begin(), c.end(), out);
    return FK_OK;
}

}  // extern "C"
