// kpm_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle); see kpm_oracle.h.
//
// CPU restatement of the reference's CPU engine (src/engine_cpu.cpp), probe
// generation (src/engine.cpp), BSR handling (src/spmat.cpp) and KPM helpers
// (src/fastkpm.cpp). Every function cites the reference lines it follows.
// Armadillo's SpMat x Mat product becomes an explicit BSR x (row-major n x s)
// loop, arma::cdot(A, B) becomes sum(conj(A) .* B) over all elements, and
// arma::eig_sym on the Lanczos tridiagonal becomes Sturm bisection.
// PARITY UNPINNED against the reference itself (no reference tests or golden
// vectors exist, and the reference does not build here); the tests pin this
// oracle against analytic known answers instead.
#include "kpm_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <random>
#include <thread>
#include <type_traits>
#include <vector>
#include <sched.h>

namespace {

using cx = std::complex<double>;
constexpr double kPi = 3.141592653589793238463;   // src/fastkpm.h:28

inline double conj_(double x) { return x; }
inline cx conj_(cx x) { return std::conj(x); }
inline double re_(double x) { return x; }
inline double re_(cx x) { return x.real(); }

int usable_cores() {
    cpu_set_t set;
    CPU_ZERO(&set);
    if (sched_getaffinity(0, sizeof(set), &set) == 0) {
        int n = CPU_COUNT(&set);
        if (n > 0) return n;
    }
    unsigned n = std::thread::hardware_concurrency();
    return n ? int(n) : 1;
}

// Static partition of [0, n) into nthreads contiguous ranges, one std::thread each.
void parallel_ranges(int nthreads, long n, const std::function<void(int, long, long)>& fn) {
    if (nthreads <= 1 || n < 2 * nthreads) { fn(0, 0, n); return; }
    std::vector<std::thread> ts;
    for (int t = 0; t < nthreads; t++) {
        long a = n * t / nthreads, b = n * (t + 1) / nthreads;
        ts.emplace_back(fn, t, a, b);
    }
    for (auto& th : ts) th.join();
}

// random_phase<T> (src/engine.cpp:7-32): {+1,-1} for real, {+1,+i,-1,-i} for complex.
template <typename T> T random_phase(std::mt19937& rng);
template <> double random_phase<double>(std::mt19937& rng) {
    std::uniform_int_distribution<int> dist2(0, 1);
    return 2 * dist2(rng) - 1;
}
template <> cx random_phase<cx>(std::mt19937& rng) {
    std::uniform_int_distribution<int> dist4(0, 3);
    switch (dist4(rng)) {
        case 0: return {+1, 0};
        case 1: return {0, +1};
        case 2: return {-1, 0};
        default: return {0, -1};
    }
}

// Host BSR matrix, blocks column-major b x b (src/fastkpm.h:64-65).
template <typename T>
struct Bsr {
    int n_b = 0, b = 0;
    std::vector<int> row_ptr, col_idx;
    std::vector<T> val;
    int nnzb() const { return int(col_idx.size()); }
};

template <typename T>
struct Engine {
    int nthreads = 1;
    double es_lo = 0, es_hi = 0;
    Bsr<T> Hs;
    int n = 0, s = 0;              // R is n x s
    std::vector<T> R;              // row-major n x s (row i = scalar row i)
    std::vector<T> a0, a1, a2;     // recursion state, row-major n x s
    bool have_moment_state = false;

    double avg() const { return (es_hi + es_lo) / 2.0; }   // EnergyScale::avg (fastkpm.h:115)
    double mag() const { return (es_hi - es_lo) / 2.0; }   // EnergyScale::mag (fastkpm.h:116)

    // y = alpha * Hs * x + beta * z  (row-major n x s); Armadillo's SpMat*Mat in
    // src/engine_cpu.cpp:71,76,236,240,286,290, with the scalar row sum taken in
    // ascending column order.
    void spmm(double alpha, const Bsr<T>& H, const std::vector<T>& x, double beta,
              const std::vector<T>* z, std::vector<T>& y) const {
        const int b = H.b, S = s;
        y.resize(size_t(n) * S);
        parallel_ranges(nthreads, H.n_b, [&](int, long i0, long i1) {
            std::vector<T> acc(size_t(b) * S);
            for (long i = i0; i < i1; i++) {
                std::fill(acc.begin(), acc.end(), T(0));
                for (int k = H.row_ptr[i]; k < H.row_ptr[i + 1]; k++) {
                    const int j = H.col_idx[k];
                    const T* blk = &H.val[size_t(b) * b * k];
                    for (int bj = 0; bj < b; bj++) {
                        const T* xr = &x[size_t(b * j + bj) * S];
                        for (int bi = 0; bi < b; bi++) {
                            const T h = blk[b * bj + bi];   // column-major block
                            T* ar = &acc[size_t(bi) * S];
                            for (int c = 0; c < S; c++) ar[c] += h * xr[c];
                        }
                    }
                }
                for (int bi = 0; bi < b; bi++) {
                    T* yr = &y[size_t(b * i + bi) * S];
                    const T* ar = &acc[size_t(bi) * S];
                    if (z) {
                        const T* zr = &(*z)[size_t(b * i + bi) * S];
                        for (int c = 0; c < S; c++) yr[c] = alpha * ar[c] + beta * zr[c];
                    } else {
                        for (int c = 0; c < S; c++) yr[c] = alpha * ar[c];
                    }
                }
            }
        });
    }

    // arma::cdot(A, B) = sum conj(A) .* B over all elements; per-thread partials
    // combined in thread order.
    T cdot(const std::vector<T>& A, const std::vector<T>& B) const {
        std::vector<T> part(std::max(nthreads, 1), T(0));
        parallel_ranges(nthreads, long(A.size()), [&](int t, long i0, long i1) {
            T acc = 0;
            for (long i = i0; i < i1; i++) acc += conj_(A[i]) * B[i];
            part[t] = acc;
        });
        T r = 0;
        for (auto& p : part) r += p;
        return r;
    }

    // outer_product (src/engine_cpu.cpp:212-226):
    // D_k(bi, bj) += alpha * cdot(B.row(b j + bj), A.row(b i + bi)) for k = (i, j)
    void outer_product(T alpha, const std::vector<T>& A, const std::vector<T>& B, int nnzb,
                       const int* rows, const int* cols, int b, T* D) const {
        const int S = s;
        parallel_ranges(nthreads, nnzb, [&](int, long k0, long k1) {
            for (long k = k0; k < k1; k++) {
                const int i = rows[k], j = cols[k];
                T* v = &D[size_t(b) * b * k];
                for (int bj = 0; bj < b; bj++) {
                    for (int bi = 0; bi < b; bi++) {
                        const T* ar = &A[size_t(b * i + bi) * S];
                        const T* br = &B[size_t(b * j + bj) * S];
                        T acc = 0;
                        for (int c = 0; c < S; c++) acc += conj_(br[c]) * ar[c];
                        v[b * bj + bi] += alpha * acc;
                    }
                }
            }
        });
    }
};

// SpMatBsr::build (src/spmat.cpp:46-129): stable per-row sort by column, duplicates summed.
template <typename T>
int bsr_build(int n_rows, int b, int n_elems, const int* ri, const int* ci, const T* v,
              int* out_row_ptr, int* out_row_idx, int* out_col_idx, T* out_val) {
    const int bb = b * b;
    bool sorted = true;
    for (int k = 0; k + 1 < n_elems; k++) {
        if (ri[k] > ri[k + 1] || (ri[k] == ri[k + 1] && ci[k] > ci[k + 1])) { sorted = false; break; }
    }
    std::vector<int> order(n_elems);
    if (!sorted) {
        std::vector<std::vector<int>> bins(n_rows);
        for (int p = 0; p < n_elems; p++) bins[ri[p]].push_back(p);
        order.clear();
        for (int i = 0; i < n_rows; i++) {
            std::sort(bins[i].begin(), bins[i].end(), [&](int p1, int p2) { return ci[p1] < ci[p2]; });
            order.insert(order.end(), bins[i].begin(), bins[i].end());
        }
    } else {
        for (int p = 0; p < n_elems; p++) order[p] = p;
    }
    int max_row = -1, cnt = 0;
    for (int p : order) {
        const int i = ri[p], j = ci[p];
        if (cnt > 0 && out_row_idx[cnt - 1] == i && out_col_idx[cnt - 1] == j) {
            for (int q = 0; q < bb; q++) out_val[size_t(bb) * (cnt - 1) + q] += v[size_t(bb) * p + q];
        } else {
            out_row_idx[cnt] = i;
            out_col_idx[cnt] = j;
            std::copy_n(v + size_t(bb) * p, bb, out_val + size_t(bb) * cnt);
            while (max_row < i) out_row_ptr[++max_row] = cnt;
            cnt++;
        }
    }
    while (max_row < n_rows) out_row_ptr[++max_row] = cnt;
    return cnt;
}

// SpMatBsr::find_index (src/spmat.cpp:145-154)
int find_index(const int* row_ptr, const int* col_idx, int i, int j) {
    for (int p = row_ptr[i]; p < row_ptr[i + 1]; p++)
        if (col_idx[p] == j) return p;
    return -1;
}

// SpMatBsr::symmetrize (src/spmat.cpp:171-190): D_ij <- (D_ij + D_ji^dagger)/2 blockwise.
template <typename T>
int bsr_symmetrize(int b, int nnzb, const int* row_ptr, const int* row_idx, const int* col_idx, T* val) {
    for (int k = 0; k < nnzb; k++) {
        const int i = row_idx[k], j = col_idx[k];
        if (i >= j) {
            const int kt = find_index(row_ptr, col_idx, j, i);
            if (kt < 0) return -1;   // reference aborts (spmat.cpp:151-152)
            T* v1b = &val[size_t(b) * b * k];
            T* v2b = &val[size_t(b) * b * kt];
            for (int bj = 0; bj < b; bj++) {
                for (int bi = 0; bi < b; bi++) {
                    T* v1 = &v1b[bj * b + bi];
                    T* v2 = &v2b[bi * b + bj];
                    T sym = (*v1 + conj_(*v2)) / T(2);
                    *v1 = sym;
                    *v2 = conj_(sym);
                }
            }
        }
    }
    return 0;
}

template <typename T>
int set_H(Engine<T>& e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
          const T* val, double lo, double hi) {
    if (n_b <= 0 || b <= 0 || nnzb < 0) return 1;
    e.es_lo = lo; e.es_hi = hi;
    // Hs = (H - avg I)/mag (src/engine_cpu.cpp:53-61). A row without a stored
    // diagonal block receives one (Armadillo inserts the element on Hs(i,i) -= avg).
    Bsr<T>& H = e.Hs;
    H.n_b = n_b; H.b = b;
    H.row_ptr.assign(n_b + 1, 0);
    H.col_idx.clear(); H.val.clear();
    const int bb = b * b;
    const double avg = e.avg(), mag = e.mag();
    for (int i = 0; i < n_b; i++) {
        bool have_diag = false;
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) have_diag |= (col_idx[k] == i);
        bool inserted = have_diag;
        for (int k = row_ptr[i]; k <= row_ptr[i + 1]; k++) {
            const bool end = (k == row_ptr[i + 1]);
            const int j = end ? n_b : col_idx[k];
            if (!inserted && j > i) {
                H.col_idx.push_back(i);
                for (int q = 0; q < bb; q++) H.val.push_back(T(0));
                inserted = true;
            }
            if (end) break;
            H.col_idx.push_back(j);
            for (int q = 0; q < bb; q++) H.val.push_back(val[size_t(bb) * k + q]);
        }
        H.row_ptr[i + 1] = int(H.col_idx.size());
    }
    for (int i = 0; i < n_b; i++) {
        for (int k = H.row_ptr[i]; k < H.row_ptr[i + 1]; k++) {
            T* blk = &H.val[size_t(bb) * k];
            if (H.col_idx[k] == i)
                for (int q = 0; q < b; q++) blk[q * b + q] -= avg;
            for (int q = 0; q < bb; q++) blk[q] /= mag;
        }
    }
    e.have_moment_state = false;
    return 0;
}

template <typename T>
int moments(Engine<T>& e, int M, double* mu) {
    const int n = e.n;
    if (M < 2 || M % 2 != 0) return 1;                      // assert(M % 2 == 0)
    if (e.Hs.b * e.Hs.n_b != n || n == 0) return 6;
    e.a0 = e.R;                                              // alpha_0
    e.spmm(1.0, e.Hs, e.R, 0.0, nullptr, e.a1);              // alpha_1 = Hs R
    mu[0] = re_(e.cdot(e.a0, e.a0));
    mu[1] = re_(e.cdot(e.a1, e.a0));
    for (int m = 1; m < M / 2; m++) {
        e.spmm(2.0, e.Hs, e.a1, -1.0, &e.a0, e.a2);          // a2 = 2 Hs a1 - a0
        std::swap(e.a0, e.a1);                               // a0 = alpha_m
        std::swap(e.a1, e.a2);                               // a1 = alpha_{m+1}
        mu[2 * m] = 2 * re_(e.cdot(e.a0, e.a0)) - mu[0];
        mu[2 * m + 1] = 2 * re_(e.cdot(e.a1, e.a0)) - mu[1];
    }
    e.have_moment_state = true;
    return 0;
}

template <typename T>
int stoch_matrix(Engine<T>& e, int M, const double* c, int nnzb, const int* rows,
                 const int* cols, T* D) {
    if (M < 2 || e.n == 0) return 1;
    const int b = e.Hs.b;
    e.a0 = e.R;
    e.spmm(1.0, e.Hs, e.R, 0.0, nullptr, e.a1);
    std::vector<T> xi(e.a0.size());
    for (size_t q = 0; q < xi.size(); q++) xi[q] = c[0] * e.a0[q] + c[1] * e.a1[q];
    for (int m = 2; m < M; m++) {
        e.spmm(2.0, e.Hs, e.a1, -1.0, &e.a0, e.a2);
        for (size_t q = 0; q < xi.size(); q++) xi[q] += c[m] * e.a2[q];
        std::swap(e.a0, e.a1);
        std::swap(e.a1, e.a2);
    }
    std::fill(D, D + size_t(b) * b * nnzb, T(0));
    e.outer_product(T(0.5), e.R, xi, nnzb, rows, cols, b, D);
    e.outer_product(T(0.5), xi, e.R, nnzb, rows, cols, b, D);
    e.have_moment_state = false;                             // a0, a1 cleared (:249-251)
    return 0;
}

template <typename T>
int autodiff_matrix(Engine<T>& e, int M, const double* c, int nnzb, const int* row_ptr,
                    const int* rows, const int* cols, T* D) {
    if (!e.have_moment_state) return 6;                      // REQUIREMENT: moments() first
    const int b = e.Hs.b;
    const size_t sz = e.R.size();
    double diag = c[1];
    for (int m = 1; m < M / 2; m++) diag -= c[2 * m + 1];
    std::fill(D, D + size_t(b) * b * nnzb, T(0));
    e.outer_product(T(diag), e.R, e.R, nnzb, rows, cols, b, D);
    std::vector<T> b2(sz), b1(sz, T(0)), b0(sz, T(0));
    if (M > 2)
        for (size_t q = 0; q < sz; q++) b0[q] = 2 * c[M - 1] * e.a0[q];
    for (int m = M / 2 - 1; m >= 1; m--) {
        e.outer_product(T(2), e.a0, b0, nnzb, rows, cols, b, D);   // D += 2 alpha_m beta_{m+1}^dag
        std::swap(e.a2, e.a1);                                       // a2 = a1
        e.a1 = e.a0;                                                 // a1 = a0
        e.spmm(2.0, e.Hs, e.a1, -1.0, &e.a2, e.a0);                  // a0 = 2 Hs a1 - a2
        std::swap(b2, b1);
        b1 = b0;
        e.spmm(2.0, e.Hs, b1, -1.0, &b2, b0);                        // 2 Hs b1 - b2
        for (size_t q = 0; q < sz; q++) {
            b0[q] += 4 * c[2 * m] * e.a1[q] + 2 * c[2 * m + 1] * e.a2[q];
            if (m > 1) b0[q] += 2 * c[2 * m - 1] * e.a0[q];
        }
    }
    e.outer_product(T(1), e.a0, b0, nnzb, rows, cols, b, D);        // D += alpha_0 beta_1^dag
    if (bsr_symmetrize(b, nnzb, row_ptr, rows, cols, D) != 0) return 3;
    const double inv = 1.0 / e.mag();
    for (size_t q = 0; q < size_t(b) * b * nnzb; q++) D[q] *= inv;
    e.have_moment_state = false;
    return 0;
}

// Lanczos (src/engine_cpu.cpp:14-51) with caller-given start vector.
template <typename T>
int energy_scale(Engine<T>& e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
                 const T* val, double extend, int iters, const T* v_start, double* lo, double* hi) {
    if (iters < 1) return 1;
    Bsr<T> H;
    H.n_b = n_b; H.b = b;
    H.row_ptr.assign(row_ptr, row_ptr + n_b + 1);
    H.col_idx.assign(col_idx, col_idx + nnzb);
    H.val.assign(val, val + size_t(b) * b * nnzb);
    const int n = n_b * b;
    Engine<T> tmp;
    tmp.nthreads = e.nthreads;
    tmp.n = n; tmp.s = 1;
    std::vector<T> v0(n, T(0)), v1(v_start, v_start + n), w;
    double nrm = std::sqrt(re_(tmp.cdot(v1, v1)));
    for (auto& x : v1) x /= nrm;
    std::vector<double> alpha(iters), beta(iters);
    beta[0] = 0;
    for (int j = 1; j < iters; j++) {
        tmp.spmm(1.0, H, v1, 0.0, nullptr, w);
        alpha[j - 1] = re_(tmp.cdot(w, v1));
        for (int q = 0; q < n; q++) w[q] = w[q] - alpha[j - 1] * v1[q] - beta[j - 1] * v0[q];
        beta[j] = std::sqrt(re_(tmp.cdot(w, w)));
        v0 = v1;
        for (int q = 0; q < n; q++) v1[q] = w[q] / beta[j];
    }
    tmp.spmm(1.0, H, v1, 0.0, nullptr, w);
    alpha[iters - 1] = re_(tmp.cdot(w, v1));
    double emin, emax;
    orc_tridiag_extremes(iters, alpha.data(), beta.data(), &emin, &emax);
    const double slack = extend * (emax - emin);
    *lo = emin - slack;
    *hi = emax + slack;
    return 0;
}

// Number of eigenvalues of the tridiagonal (alpha, beta) below x (Sturm count).
int sturm_count(int n, const double* a, const double* bt, double x) {
    int cnt = 0;
    double q = a[0] - x;
    if (q < 0) cnt++;
    for (int j = 1; j < n; j++) {
        const double d = (q == 0) ? 1e-300 : q;
        q = a[j] - x - bt[j] * bt[j] / d;
        if (q < 0) cnt++;
    }
    return cnt;
}

template <typename T>
void fill_R_identity(int n, int j0, int j1, T* R) {
    const int cols = j1 - j0;
    std::fill(R, R + size_t(n) * cols, T(0));
    for (int j = j0; j < j1; j++) R[size_t(j - j0) * n + j] = T(1.0);
}

// y = A x for one vector (BSR A, no scaling)
template <typename T>
void bsr_spmv(const int n_b, const int b, const int* row_ptr, const int* col_idx, const T* val, const T* x, T* y) {
    for (int i = 0; i < n_b; i++) {
        for (int bi = 0; bi < b; bi++) y[b * i + bi] = T(0);
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
            const T* blk = val + size_t(b) * b * k;
            for (int bj = 0; bj < b; bj++)
                for (int bi = 0; bi < b; bi++) y[b * i + bi] += blk[b * bj + bi] * x[b * col_idx[k] + bj];
        }
    }
}

// moments2_v1 (src/engine_cpu.cpp:86-160): mu[m1][m2] = sum_k cdot(alpha_m1, j2 atild_m2) with
// alpha_m = T_m(Hs) r_k, atild_m = T_m(Hs) j1 r_k over the probe columns r_k. The reference walks
// the orders in chunks of a_chunk_ncols, recomputing the recursions; the chunking changes no sum,
// so this keeps every order of one column at once. Columns run in parallel; the per-column
// contributions are added in column order.
template <typename T>
int moments2_v1(Engine<T>& e, int M, int n_b, int b, const int* rp1, const int* ci1, const T* v1, const int* rp2,
                const int* ci2, const T* v2, cx* mu) {
    const int n = e.n, s = e.s;
    if (M < 2 || M % 2 != 0 || n == 0 || n_b * b != n || e.Hs.n_b != n_b || e.Hs.b != b) return 1;
    std::vector<std::vector<cx>> part(s, std::vector<cx>(size_t(M) * M, cx(0)));
    const Bsr<T>& H = e.Hs;
    auto hs = [&](const T* x, T* y) {
        bsr_spmv(n_b, b, H.row_ptr.data(), H.col_idx.data(), H.val.data(), x, y);
    };
    parallel_ranges(e.nthreads, s, [&](int, long k0, long k1) {
        std::vector<T> A(size_t(M) * n), Bt(size_t(M) * n), t(n), r(n);
        for (long k = k0; k < k1; k++) {
            for (int i = 0; i < n; i++) r[i] = e.R[size_t(i) * s + k];
            auto recurse = [&](const T* v0, T* out) {   // out[m] = T_m(Hs) v0
                std::copy_n(v0, n, out);
                if (M > 1) hs(out, out + n);
                for (int m = 2; m < M; m++) {
                    hs(out + size_t(m - 1) * n, out + size_t(m) * n);
                    for (int i = 0; i < n; i++)
                        out[size_t(m) * n + i] = T(2) * out[size_t(m) * n + i] - out[size_t(m - 2) * n + i];
                }
            };
            recurse(r.data(), A.data());
            bsr_spmv(n_b, b, rp1, ci1, v1, r.data(), t.data());   // j1 r_k
            recurse(t.data(), Bt.data());
            for (int m2 = 0; m2 < M; m2++) {
                bsr_spmv(n_b, b, rp2, ci2, v2, Bt.data() + size_t(m2) * n, t.data());   // j2 atild_m2
                for (int m1 = 0; m1 < M; m1++) {
                    cx acc = 0;
                    const T* a = A.data() + size_t(m1) * n;
                    for (int i = 0; i < n; i++) acc += cx(conj_(a[i]) * t[i]);
                    part[k][size_t(m1) * M + m2] = acc;
                }
            }
        }
    });
    for (size_t q = 0; q < size_t(M) * M; q++) {
        cx acc = 0;
        for (int k = 0; k < s; k++) acc += part[k][q];
        mu[q] = acc;
    }
    return 0;
}

// moments2_v2 (src/engine_cpu.cpp:162-209): A_i = R^dag T_i(Hs) j2 R2, B_i = R2^dag T_i(Hs) j1 R
// (s x s each, arma::trans is the conjugate transpose), mu[m1][m2] = sum_k A_m1.row(k) . B_m2.col(k)
// (arma::dot, no conjugation) = tr(A_m1 B_m2). R2: n x s row-major like R.
template <typename T>
int moments2_v2(Engine<T>& e, int M, int n_b, int b, const int* rp1, const int* ci1, const T* v1, const int* rp2,
                const int* ci2, const T* v2, const std::vector<T>& R2, cx* mu) {
    const int n = e.n, s = e.s;
    if (M < 2 || M % 2 != 0 || n == 0 || n_b * b != n || e.Hs.n_b != n_b || e.Hs.b != b) return 1;
    const Bsr<T>& H = e.Hs;
    // projected s x s matrices, row-major [k][l]
    std::vector<cx> Ap(size_t(M) * s * s), Bp(size_t(M) * s * s);
    auto run = [&](const std::vector<T>& start, const int* rp, const int* ci, const T* v, const std::vector<T>& proj,
                   std::vector<cx>& out) {
        std::vector<T> X0(size_t(n) * s), X1(size_t(n) * s), X2(size_t(n) * s), col(n), y(n);
        for (int k = 0; k < s; k++) {   // X0 = j start, column by column
            for (int i = 0; i < n; i++) col[i] = start[size_t(i) * s + k];
            bsr_spmv(n_b, b, rp, ci, v, col.data(), y.data());
            for (int i = 0; i < n; i++) X0[size_t(i) * s + k] = y[i];
        }
        auto project = [&](const std::vector<T>& X, int m) {   // out[m] = proj^dag X
            parallel_ranges(e.nthreads, s, [&](int, long k0, long k1) {
                for (long k = k0; k < k1; k++)
                    for (int l = 0; l < s; l++) {
                        cx acc = 0;
                        for (int i = 0; i < n; i++) acc += cx(conj_(proj[size_t(i) * s + k]) * X[size_t(i) * s + l]);
                        out[(size_t(m) * s + k) * s + l] = acc;
                    }
            });
        };
        project(X0, 0);
        e.spmm(1.0, H, X0, 0.0, nullptr, X1);
        if (M > 1) project(X1, 1);
        for (int m = 2; m < M; m++) {
            e.spmm(2.0, H, X1, -1.0, &X0, X2);
            project(X2, m);
            std::swap(X0, X1);
            std::swap(X1, X2);
        }
    };
    run(R2, rp2, ci2, v2, e.R, Ap);   // A_i = R^dag T_i j2 R2
    run(e.R, rp1, ci1, v1, R2, Bp);   // B_i = R2^dag T_i j1 R
    for (int m1 = 0; m1 < M; m1++)
        for (int m2 = 0; m2 < M; m2++) {
            cx acc = 0;
            for (int k = 0; k < s; k++)
                for (int l = 0; l < s; l++) acc += Ap[(size_t(m1) * s + k) * s + l] * Bp[(size_t(m2) * s + l) * s + k];
            mu[size_t(m1) * M + m2] = acc;
        }
    return 0;
}

}  // namespace

struct orc_engine {
    int cplx;
    Engine<double> er;
    Engine<cx> ec;
};

extern "C" {

orc_engine* orc_engine_create(int cplx, int nthreads) {
    auto* e = new orc_engine();
    e->cplx = cplx ? 1 : 0;
    const int nt = nthreads > 0 ? nthreads : usable_cores();
    e->er.nthreads = nt;
    e->ec.nthreads = nt;
    return e;
}
void orc_engine_destroy(orc_engine* e) { delete e; }
int orc_engine_threads(const orc_engine* e) { return e->er.nthreads; }

int orc_set_H(orc_engine* e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
              const double* val, double lo, double hi) {
    if (e->cplx) return set_H(e->ec, n_b, b, nnzb, row_ptr, col_idx, reinterpret_cast<const cx*>(val), lo, hi);
    return set_H(e->er, n_b, b, nnzb, row_ptr, col_idx, val, lo, hi);
}

int orc_set_R(orc_engine* e, int n, int s, const double* R) {
    if (n <= 0 || s <= 0) return 1;
    auto load = [&](auto& eng, const auto* src) {
        eng.n = n; eng.s = s;
        eng.R.resize(size_t(n) * s);
        for (int j = 0; j < s; j++)
            for (int i = 0; i < n; i++) eng.R[size_t(i) * s + j] = src[size_t(j) * n + i];
        eng.have_moment_state = false;
    };
    if (e->cplx) load(e->ec, reinterpret_cast<const cx*>(R));
    else load(e->er, R);
    return 0;
}

int orc_moments(orc_engine* e, int M, double* mu) {
    return e->cplx ? moments(e->ec, M, mu) : moments(e->er, M, mu);
}

int orc_stoch_matrix(orc_engine* e, int M, const double* c, int nnzb, const int* rows,
                     const int* cols, double* D) {
    if (e->cplx) return stoch_matrix(e->ec, M, c, nnzb, rows, cols, reinterpret_cast<cx*>(D));
    return stoch_matrix(e->er, M, c, nnzb, rows, cols, D);
}

int orc_autodiff_matrix(orc_engine* e, int M, const double* c, int n_b, int nnzb, const int* row_ptr,
                        const int* rows, const int* cols, double* D) {
    (void)n_b;
    if (e->cplx) return autodiff_matrix(e->ec, M, c, nnzb, row_ptr, rows, cols, reinterpret_cast<cx*>(D));
    return autodiff_matrix(e->er, M, c, nnzb, row_ptr, rows, cols, D);
}

int orc_moments2_v1(orc_engine* e, int M, int n_b, int b, const int* rp1, const int* ci1, const double* v1,
                    const int* rp2, const int* ci2, const double* v2, double* mu) {
    cx* out = reinterpret_cast<cx*>(mu);
    if (e->cplx)
        return moments2_v1(e->ec, M, n_b, b, rp1, ci1, reinterpret_cast<const cx*>(v1), rp2, ci2,
                           reinterpret_cast<const cx*>(v2), out);
    return moments2_v1(e->er, M, n_b, b, rp1, ci1, v1, rp2, ci2, v2, out);
}

int orc_moments2_v2(orc_engine* e, int M, int n_b, int b, const int* rp1, const int* ci1, const double* v1,
                    const int* rp2, const int* ci2, const double* v2, const double* R2, double* mu) {
    cx* out = reinterpret_cast<cx*>(mu);
    auto load = [&](auto& eng, const auto* src) {   // column-major n x s -> row-major, or R itself
        using TT = typename std::decay<decltype(eng.R)>::type::value_type;
        std::vector<TT> r2(eng.R.size());
        if (!src) return eng.R;
        for (int j = 0; j < eng.s; j++)
            for (int i = 0; i < eng.n; i++) r2[size_t(i) * eng.s + j] = src[size_t(j) * eng.n + i];
        return r2;
    };
    if (e->cplx) {
        const auto r2 = load(e->ec, reinterpret_cast<const cx*>(R2));
        return moments2_v2(e->ec, M, n_b, b, rp1, ci1, reinterpret_cast<const cx*>(v1), rp2, ci2,
                           reinterpret_cast<const cx*>(v2), r2, out);
    }
    const auto r2 = load(e->er, R2);
    return moments2_v2(e->er, M, n_b, b, rp1, ci1, v1, rp2, ci2, v2, r2, out);
}

int orc_energy_scale(orc_engine* e, int n_b, int b, int nnzb, const int* row_ptr, const int* col_idx,
                     const double* val, double extend, int iters, const double* v_start,
                     double* lo, double* hi) {
    if (e->cplx)
        return energy_scale(e->ec, n_b, b, nnzb, row_ptr, col_idx, reinterpret_cast<const cx*>(val),
                            extend, iters, reinterpret_cast<const cx*>(v_start), lo, hi);
    return energy_scale(e->er, n_b, b, nnzb, row_ptr, col_idx, val, extend, iters, v_start, lo, hi);
}

void orc_tridiag_extremes(int n, const double* a, const double* bt, double* emin, double* emax) {
    // Gershgorin bounds, then bisection on the Sturm count for the smallest and largest eigenvalue.
    double glo = 1e300, ghi = -1e300;
    for (int j = 0; j < n; j++) {
        double r = (j > 0 ? std::fabs(bt[j]) : 0.0) + (j + 1 < n ? std::fabs(bt[j + 1]) : 0.0);
        glo = std::min(glo, a[j] - r);
        ghi = std::max(ghi, a[j] + r);
    }
    auto kth = [&](int k) {   // k-th smallest eigenvalue (0-based)
        double l = glo, h = ghi;
        for (int it = 0; it < 200 && h - l > 1e-15 * std::max(1.0, std::fabs(l) + std::fabs(h)); it++) {
            const double mid = 0.5 * (l + h);
            if (sturm_count(n, a, bt, mid) > k) h = mid; else l = mid;
        }
        return 0.5 * (l + h);
    };
    *emin = kth(0);
    *emax = kth(n - 1);
}

int orc_R_identity(int cplx, int n, int j0, int j1, double* R) {
    if (!(0 <= j0 && j0 <= j1 && j1 <= n)) return 1;
    if (cplx) fill_R_identity(n, j0, j1, reinterpret_cast<cx*>(R));
    else fill_R_identity(n, j0, j1, R);
    return 0;
}

// set_R_uncorrelated (src/engine.cpp:50-70): column j draws its own mt19937 seed
// from the master generator, and entries are random_phase(rng_j) / sqrt(s).
int orc_R_uncorrelated(int cplx, int n, int s, uint32_t seed, unsigned long long discard,
                       int j0, int j1, double* R) {
    if (!(0 <= j0 && j0 <= j1 && j1 <= s)) return 1;
    std::mt19937 rng(seed);
    rng.discard(discard);
    auto fill = [&](auto* out, auto tag) {
        using T = decltype(tag);
        const T x = 1.0 / std::sqrt(double(s));
        for (int j = j0; j < j1; j++) {
            std::mt19937 rng_j(rng());
            for (int i = 0; i < n; i++) out[size_t(j - j0) * n + i] = random_phase<T>(rng_j) * x;
        }
    };
    if (cplx) fill(reinterpret_cast<cx*>(R), cx());
    else fill(R, double());
    return 0;
}

// set_R_correlated (src/engine.cpp:76-102): row i is nonzero only in column groups[i].
int orc_R_correlated(int cplx, int n, const int* groups, uint32_t seed, unsigned long long discard,
                     int j0, int j1, double* R) {
    if (!(0 <= j0 && j0 <= j1 && j1 <= n)) return 1;
    std::mt19937 rng(seed);
    rng.discard(discard);
    auto fill = [&](auto* out, auto tag) {
        using T = decltype(tag);
        std::fill(out, out + size_t(n) * (j1 - j0), T(0));
        for (int j = j0; j < j1; j++) {
            std::mt19937 rng_j(rng());
            for (int i = 0; i < n; i++)
                if (groups[i] == j) out[size_t(j - j0) * n + i] = random_phase<T>(rng_j);
        }
    };
    if (cplx) fill(reinterpret_cast<cx*>(R), cx());
    else fill(R, double());
    return 0;
}

int orc_bsr_build(int cplx, int n_rows, int b, int n_elems, const int* ri, const int* ci,
                  const double* v, int* orp, int* ori, int* oci, double* ov) {
    if (cplx)
        return bsr_build(n_rows, b, n_elems, ri, ci, reinterpret_cast<const cx*>(v), orp, ori, oci,
                         reinterpret_cast<cx*>(ov));
    return bsr_build(n_rows, b, n_elems, ri, ci, v, orp, ori, oci, ov);
}

int orc_bsr_symmetrize(int cplx, int n_rows, int b, int nnzb, const int* row_ptr, const int* ri,
                       const int* ci, double* val) {
    (void)n_rows;
    if (cplx) return bsr_symmetrize(b, nnzb, row_ptr, ri, ci, reinterpret_cast<cx*>(val));
    return bsr_symmetrize(b, nnzb, row_ptr, ri, ci, val);
}

// jackson_kernel (src/fastkpm.cpp:13-20)
void orc_jackson_kernel(int M, double* out) {
    const double Mp = M + 1.0;
    for (int m = 0; m < M; m++)
        out[m] = (1.0 / Mp) * ((Mp - m) * std::cos(kPi * m / Mp) + std::sin(kPi * m / Mp) / std::tan(kPi / Mp));
}

// chebyshev_fill_array (src/fastkpm.cpp:30-39)
void orc_chebyshev_fill_array(double x, int M, int kind, double* out) {
    if (M > 0) out[0] = 1.0;
    if (M > 1) out[1] = kind * x;
    for (int m = 2; m < M; m++) out[m] = 2 * x * out[m - 1] - out[m - 2];
}

// fermi_density / fermi_energy (src/fastkpm.cpp:375-393)
double orc_fermi_density(double x, double kT, double mu) {
    const double alpha = (x - mu) / std::fabs(kT);
    if (kT < 1e-15 || std::fabs(alpha) > 20) return (x < mu) ? 1.0 : 0.0;
    return 1.0 / (std::exp(alpha) + 1.0);
}
double orc_fermi_energy(double x, double kT, double mu) {
    const double alpha = (x - mu) / std::fabs(kT);
    if (kT < 1e-15 || std::fabs(alpha) > 20) return (x < mu) ? (x - mu) : 0.0;
    return -kT * std::log(1 + std::exp(-alpha));
}

// expansion_coefficients, direct-sum branch (src/fastkpm.cpp:41-78, :62-75)
void orc_expansion_coefficients(int M, int Mq, int kind, double kT, double mu, double lo, double hi,
                                double* out) {
    std::vector<double> kernel(M), fp(M, 0.0), T(M);
    orc_jackson_kernel(M, kernel.data());
    const double avg = (hi + lo) / 2.0, mag = (hi - lo) / 2.0;
    for (int i = 0; i < Mq; i++) {
        const double x_i = std::cos(kPi * (i + 0.5) / Mq);
        const double E = x_i * mag + avg;                      // EnergyScale::unscale
        const double f_i = kind == 0 ? orc_fermi_density(E, kT, mu) : orc_fermi_energy(E, kT, mu);
        orc_chebyshev_fill_array(x_i, M, 1, T.data());
        for (int m = 0; m < M; m++) fp[m] += f_i * T[m];
    }
    for (int m = 0; m < M; m++) out[m] = (m == 0 ? 1.0 : 2.0) * kernel[m] * fp[m] / Mq;
}

// moment_product (src/fastkpm.cpp:291-298)
double orc_moment_product(int M, const double* c, const double* mu) {
    double r = 0;
    for (int i = 0; i < M; i++) r += c[i] * mu[i];
    return r;
}

// electrical_conductivity_coefficients, direct-sum branch (src/fastkpm.cpp:80-233 without FFTW):
// out[2*(m1*M + m2) + {0,1}]; returns 1 on the reference's assertion failures
int orc_electrical_conductivity_coefficients(int M, int Mq, double kT, double mu, double omega, double lo, double hi,
                                             const double* kernel, double* out) {
    if (Mq < 2 * M || omega < 0.0) return 1;
    const double mag = (hi - lo) / 2.0, avg = (hi + lo) / 2.0, cutoff = 1e-4, ws = omega / mag;
    std::vector<cx> ret(size_t(M) * M, cx(0.0, 0.0));
    std::vector<double> Ti(M), Tj(M);
    if (ws < 2.0 && ws < 1.0e-10) {
        for (int i = 0; i < Mq; i++) {
            const double x = std::cos(kPi * (i + 0.5) / Mq);
            if (1.0 - x * x < cutoff) continue;
            orc_chebyshev_fill_array(x, M, 1, Ti.data());
            orc_chebyshev_fill_array(x, M, 2, Tj.data());
            const double s1 = std::sqrt(1.0 - x * x);
            for (int m = M - 1; m > 0; m--) Tj[m] = Tj[m - 1] * s1;
            Tj[0] = 0.0;
            const double f = orc_fermi_density(x * mag + avg, kT, mu) / std::pow(1.0 - x * x, 1.5);
            for (int a = 0; a < M; a++)
                for (int b = 0; b < M; b++)
                    ret[size_t(a) * M + b] += (Ti[a] * cx(Ti[b], -Tj[b]) * cx(x, b * s1) +
                                               Ti[b] * cx(Ti[a], Tj[a]) * cx(x, -a * s1)) * f;
        }
    } else if (ws < 2.0) {
        const int i_start = int(std::ceil(std::acos(1.0 - ws) / kPi * Mq - 0.5));
        if (Mq - i_start < 20) return 1;
        for (int i = i_start; i < Mq; i++) {
            const double x = std::cos(kPi * (i + 0.5) / Mq), xw = x + ws;
            if (x < -1.0 + cutoff || xw > 1.0 - cutoff) continue;
            orc_chebyshev_fill_array(xw, M, 1, Ti.data());
            orc_chebyshev_fill_array(x, M, 1, Tj.data());
            const double E = x * mag + avg;
            const double f = (orc_fermi_density(E, kT, mu) - orc_fermi_density(E + omega, kT, mu)) /
                             (ws * std::sqrt(1.0 - xw * xw));
            for (int a = 0; a < M; a++)
                for (int b = 0; b < M; b++) ret[size_t(a) * M + b] += Ti[a] * Tj[b] * f;
        }
    }
    for (int a = 0; a < M; a++)
        for (int b = 0; b < M; b++) {
            const double pref = 2.0 * kPi * (a == 0 ? 1.0 : 2.0) * kernel[a] / (Mq * mag * mag) * (b == 0 ? 1.0 : 2.0) *
                                kernel[b];
            const cx v = ret[size_t(a) * M + b] * pref;
            out[2 * (size_t(a) * M + b)] = v.real();
            out[2 * (size_t(a) * M + b) + 1] = v.imag();
        }
    return 0;
}

// moment_transform (src/fastkpm.cpp:236-256): Jackson-damped density on the Mq Chebyshev nodes
void orc_moment_transform(int M, const double* mu, int Mq, double* gamma) {
    std::vector<double> kernel(M), T(M), mup(M);
    orc_jackson_kernel(M, kernel.data());
    for (int m = 0; m < M; m++) mup[m] = mu[m] * kernel[m];
    for (int i = 0; i < Mq; i++) {
        gamma[i] = 0.0;
        orc_chebyshev_fill_array(std::cos(kPi * (i + 0.5) / Mq), M, 1, T.data());
        for (int m = 0; m < M; m++) gamma[i] += (m == 0 ? 1 : 2) * mup[m] * T[m];
    }
}

// density_product (src/fastkpm.cpp:314-322) with f = 1 (kind -1), fermi_density (0), fermi_energy (1)
static double density_product(int Mq, const double* gamma, int kind, double kT, double mu, double lo, double hi) {
    const double avg = (hi + lo) / 2.0, mag = (hi - lo) / 2.0;
    double r = 0.0;
    for (int i = 0; i < Mq; i++) {
        const double E = std::cos(kPi * (i + 0.5) / Mq) * mag + avg;
        const double f = kind < 0 ? 1.0 : (kind == 0 ? orc_fermi_density(E, kT, mu) : orc_fermi_energy(E, kT, mu));
        r += gamma[i] * f;
    }
    return r / Mq;
}

// mu_to_filling (src/fastkpm.cpp:395-400)
double orc_mu_to_filling(int Mq, const double* gamma, double lo, double hi, double kT, double mu) {
    return density_product(Mq, gamma, 0, kT, mu, lo, hi) / density_product(Mq, gamma, -1, kT, mu, lo, hi);
}

// filling_to_mu (src/fastkpm.cpp:418-432): smearing kT' = max(kT, 0.1 mag / Mq), bracket
// [lo - max(c, 0), hi + max(-c, 0)] with c = kT' log(1/filling - 1); the reference's toms748
// root (30-bit tolerance, src/fastkpm.cpp:410-416) is replaced by bisection to 1e-14, so the
// two agree to the reference's tolerance; two roots at filling +- delta are averaged.
double orc_filling_to_mu(int Mq, const double* gamma, double lo, double hi, double kT, double filling,
                         double delta_filling) {
    const double kTs = std::max(kT, 0.1 * ((hi - lo) / 2.0) / Mq);
    const double c = kTs * std::log(1.0 / filling - 1.0);
    const double a0 = lo - std::max(c, 0.0), b0 = hi + std::max(-c, 0.0);
    auto root = [&](double target) {
        double a = a0, b = b0;
        for (int it = 0; it < 200; it++) {
            const double mid = 0.5 * (a + b);
            if (orc_mu_to_filling(Mq, gamma, lo, hi, kTs, mid) - target < 0) a = mid;
            else b = mid;
            if (b - a <= 1e-14 * std::max(1.0, std::fabs(mid))) break;
        }
        return 0.5 * (a + b);
    };
    if (delta_filling == 0) return root(filling);
    return 0.5 * (root(filling + delta_filling) + root(filling - delta_filling));
}

// electronic_energy (src/fastkpm.cpp:452-456) = electronic_grand_energy (:440-443) + mu n_occ
double orc_electronic_energy(int Mq, const double* gamma, double lo, double hi, double kT, double filling, double mu) {
    const double n_tot = density_product(Mq, gamma, -1, kT, mu, lo, hi);
    return density_product(Mq, gamma, 1, kT, mu, lo, hi) + mu * filling * n_tot;
}

}  // extern "C"
