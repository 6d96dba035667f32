// fastkpm.h -- drop-in C++ interface of the GB300 KPM engine.
//
// Same namespace, types and Engine<T> members as the reference header
// (reference src/fastkpm.h:16-263), so code written against FastKPM's
// fkpm::Engine<T> compiles and links against libfastkpm_gb300.so unchanged,
// with these documented differences:
//   * No Armadillo. Engine<T>::R and R2 are fkpm::Mat<T>, a column-major
//     matrix exposing the arma::Mat subset the engine API uses (n_rows, n_cols,
//     set_size, fill, zeros, size, memptr, colptr, operator()). SpMatBsr has no
//     to_arma / to_arma_dense, and the arma::vec overloads of mu_to_filling,
//     filling_to_mu, electronic_grand_energy and electronic_energy are absent.
//   * mk_engine<T>() returns the GB300 engine and throws std::runtime_error when
//     no CUDA device is usable; it never falls back to a CPU engine.
//     mk_engine_cpu<T>() and mk_engine_mpi<T>() throw: neither is part of this
//     build. mk_engine_cuSPARSE<T>(devices) returns the GB300 engine on
//     devices[0] (device 0 when empty); with two or more entries it splits the
//     probe columns over one engine per listed device, like the reference's
//     threaded engine, and sums moments and D on the host in device order
//     (moments2_v2 is not split: it throws with more than one device).
//   * moments2_v1 and moments2_v2 run on the GPU (the reference's GPU engine exits
//     in moments2_v2); moments2_v2 takes R2 = R when R2 is empty.
//   * Errors throw std::runtime_error instead of assert/abort/exit.
//   * set_H(H) (one argument) is added; it takes the energy scale from
//     energy_scale(H, 0.01).
#ifndef __fastkpm__
#define __fastkpm__

#include <chrono>
#include <complex>
#include <functional>
#include <memory>
#include <ostream>
#include <random>
#include <string>
#include <vector>

namespace fkpm {
    typedef std::mt19937 RNG;

    template <typename T>
    using Vec = std::vector<T>;

    template <typename S, typename T>
    void copy_vec(Vec<S> const& src_vec, Vec<T>& dst_vec) {
        dst_vec.resize(src_vec.size());
        for (size_t i = 0; i < src_vec.size(); i++) dst_vec[i] = T(src_vec[i]);
    }

    constexpr double Pi = 3.141592653589793238463;

    typedef std::complex<float>  cx_float;
    typedef std::complex<double> cx_double;

    // conj() for every element type: the identity on float and double, std::conj on complex
    inline float     conj(float x)     { return x; }
    inline double    conj(double x)    { return x; }
    inline cx_float  conj(cx_float x)  { return std::conj(x); }
    inline cx_double conj(cx_double x) { return std::conj(x); }

    inline void parallel_for(size_t start, size_t end, std::function<void(size_t)> fn) {
        for (size_t i = start; i < end; i++) fn(i);
    }

    // Column-major dense matrix (stand-in for the arma::Mat<T> members R and R2).
    template <typename T>
    class Mat {
    public:
        int n_rows = 0, n_cols = 0;
        Mat() = default;
        Mat(int r, int c) { set_size(r, c); }
        void set_size(int r, int c) { n_rows = r; n_cols = c; data_.assign(size_t(r) * c, T(0)); }
        void fill(T v) { std::fill(data_.begin(), data_.end(), v); }
        void zeros() { fill(T(0)); }
        size_t size() const { return data_.size(); }
        T* memptr() { return data_.data(); }
        T const* memptr() const { return data_.data(); }
        T* colptr(int j) { return data_.data() + size_t(j) * n_rows; }
        T const* colptr(int j) const { return data_.data() + size_t(j) * n_rows; }
        T& operator()(int i, int j) { return data_[size_t(j) * n_rows + i]; }
        T const& operator()(int i, int j) const { return data_[size_t(j) * n_rows + i]; }
        void reset() { n_rows = n_cols = 0; data_.clear(); }
    private:
        std::vector<T> data_;
    };

    // -- spmat ------------------------------------------------------------------

    // Coordinate list of b x b blocks (row, column, b*b values each), any order; build() sorts it
    template <typename T>
    class SpMatElems {
    public:
        int n_rows, n_cols, b_len;
        Vec<int> row_idx, col_idx;
        Vec<T> val;
        SpMatElems(int n_rows, int n_cols, int b_len);
        int n_blocks() const;
        void clear();
        void add(int i, int j, T const* v);
    };

    // Sparse matrix in block compressed sparse row (BSR) format. Each dense block is
    // stored in column-major order.
    template <typename T>
    class SpMatBsr {
    public:
        int n_rows = 0, n_cols = 0, b_len = 0;
        Vec<int> row_idx, col_idx, row_ptr;
        Vec<T> val;
        SpMatBsr();
        SpMatBsr(SpMatElems<T> const& elems);
        void build(SpMatElems<T> const& elems);
        int n_blocks() const;
        void clear();
        int find_index(int i, int j) const;
        T* operator()(int i, int j);
        T const* operator()(int i, int j) const;
        void zeros();
        void symmetrize();
        void scale(T alpha);

        template <typename S>
        SpMatBsr(SpMatBsr<S> const& that) : SpMatBsr() { *this = that; }
        template <typename S>
        SpMatBsr<T>& operator=(SpMatBsr<S> const& that) {
            if ((void*)this != (void*)&that) {
                n_rows = that.n_rows;
                n_cols = that.n_cols;
                b_len = that.b_len;
                copy_vec(that.row_idx, row_idx);
                copy_vec(that.col_idx, col_idx);
                copy_vec(that.row_ptr, row_ptr);
                copy_vec(that.val, val);
            }
            return *this;
        }
    };

    // -- KPM host math ------------------------------------------------------------

    // Affine map of the spectrum [lo, hi] onto [-1, +1] and back
    class EnergyScale {
    public:
        double lo, hi;
        double avg() const { return (hi + lo) / 2.0; }
        double mag() const { return (hi - lo) / 2.0; }
        double scale(double x) const { return (x - avg()) / mag(); }
        double unscale(double x) const { return x * mag() + avg(); }
        friend std::ostream& operator<<(std::ostream& stream, EnergyScale const& es) {
            return stream << "< lo = " << es.lo << " hi = " << es.hi << " >\n";
        }
    };

    Vec<double> jackson_kernel(int M);
    Vec<double> lorentz_kernel(int M, double lambda);
    void chebyshev_fill_array(double x, Vec<double>& ret, int kind = 1);
    // Coefficients c_m with f(x) = sum_m T_m(x) c_m, Jackson-damped
    Vec<double> expansion_coefficients(int M, int Mq, std::function<double(double)> f, EnergyScale es);
    double moment_product(Vec<double> const& c, Vec<double> const& mu);
    cx_double moment_product(Vec<Vec<cx_double>> const& c, Vec<Vec<cx_double>> const& mu);
    Vec<double> moment_transform(Vec<double> const& moments, int Mq);
    // conductivity: Kubo-Bastin coefficients (direct-sum form) and the 2D transforms
    Vec<Vec<cx_double>> electrical_conductivity_coefficients(int M, int Mq, double kT, double mu, double omega,
                                                             EnergyScale es, Vec<double> const& kernel);
    Vec<Vec<cx_double>> moment_transform(Vec<Vec<cx_double>> const& moments, int Mq, Vec<double> const& kernel);
    void density_function(Vec<Vec<cx_double>> const& gamma, EnergyScale es, Vec<double>& x, Vec<double>& y,
                          Vec<Vec<cx_double>>& rho);
    double density_product(Vec<double> const& gamma, std::function<double(double)> f, EnergyScale es);
    void density_function(Vec<double> const& gamma, EnergyScale es, Vec<double>& x, Vec<double>& rho);
    void integrated_density_function(Vec<double> const& gamma, EnergyScale es, Vec<double>& x, Vec<double>& irho);
    double fermi_energy(double x, double kT, double mu);
    double fermi_density(double x, double kT, double mu);
    double mu_to_filling(Vec<double> const& gamma, EnergyScale const& es, double kT, double mu);
    double filling_to_mu(Vec<double> const& gamma, EnergyScale const& es, double kT, double filling, double delta_filling);
    double electronic_grand_energy(Vec<double> const& gamma, EnergyScale const& es, double kT, double mu);
    double electronic_energy(Vec<double> const& gamma, EnergyScale const& es, double kT, double filling, double mu);

    // -- engine -------------------------------------------------------------------

    template <typename T>
    class Engine {
    public:
        Mat<T> R;    // Random vectors
        Mat<T> R2;   // Copy kept for the reference's second moments interface

        virtual ~Engine() {}

        // Lanczos approximation to eigenvalue span
        virtual EnergyScale energy_scale(SpMatBsr<T> const& H, double extend, int iters = 128) = 0;

        virtual void set_R_identity(int n, int j_start, int j_end);
        virtual void set_R_identity(int n);
        virtual void set_R_uncorrelated(int n, int s, RNG& rng, int j_start, int j_end);
        virtual void set_R_uncorrelated(int n, int s, RNG& rng);
        virtual void set_R_correlated(Vec<int> const& groups, RNG& rng, int j_start, int j_end);
        virtual void set_R_correlated(Vec<int> const& groups, RNG& rng);

        // Upload the host probe block R to the engine's device copy; every set_R_* calls it
        virtual void transfer_R() {}

        // Upload H, scaled to Hs = (H - avg) / mag by the given energy scale
        virtual void set_H(SpMatBsr<T> const& H, EnergyScale const& es) = 0;
        void set_H(SpMatBsr<T> const& H) { set_H(H, energy_scale(H, 0.01)); }

        // Chebyshev moments: mu_m = tr T_m(Hs) ~ tr R^dagger T_m(Hs) R
        virtual Vec<double> moments(int M) = 0;

        // Conductivity moments: mu_{m1,m2} = tr(j1 T_m1(Hs) j2 T_m2(Hs)) (both run on the GPU)
        virtual Vec<Vec<cx_double>> moments2_v1(int M, SpMatBsr<T> const& j1op, SpMatBsr<T> const& j2op,
                                                int a_chunk_ncols = 0, int R_chunk_ncols = 0) = 0;
        virtual Vec<Vec<cx_double>> moments2_v2(int M, SpMatBsr<T> const& j1op, SpMatBsr<T> const& j2op,
                                                int a_chunk_ncols = 0, int R_chunk_ncols = 0) = 0;

        // D ~ (xi R^dagger + R xi^dagger)/2 with xi = (sum_m c_m T_m(Hs)) R
        virtual void stoch_matrix(Vec<double> const& c, SpMatBsr<T>& D) = 0;

        // D ~ (d/dH^T) tr g, g = sum_m c_m T_m(Hs); D's sparsity structure is an input.
        // REQUIREMENT: moments(M) with M = c.size() must have been called previously.
        virtual void autodiff_matrix(Vec<double> const& c, SpMatBsr<T>& D) = 0;
    };

    // Recursion precision of a GB300 engine
    enum class Precision { FP64 = 0, FP32 = 1, DS = 2 };

    template <typename T>
    std::shared_ptr<Engine<T>> mk_engine_cpu();
    template <typename T>
    std::shared_ptr<Engine<T>> mk_engine_cuSPARSE(Vec<int> devices = {});
    template <typename T>
    std::shared_ptr<Engine<T>> mk_engine();
    template <typename T>
    std::shared_ptr<Engine<T>> mk_engine_mpi();
    // GB300 engine on one device with a chosen recursion precision
    template <typename T>
    std::shared_ptr<Engine<T>> mk_engine_gb300(int device, Precision precision);

    // -- timer --------------------------------------------------------------------
    class Timer {
    public:
        std::chrono::time_point<std::chrono::steady_clock> t0;
        Timer();
        void reset();
        double measure();   // elapsed time in seconds
    };
    extern Timer timer[10];
}

#endif /* defined(__fastkpm__) */
