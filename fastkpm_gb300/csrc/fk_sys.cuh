// fk_sys.cuh -- number systems for the Chebyshev kernels (sm_103a).
//
// A "system" fixes how one vector element, one H block entry and the running
// sums are stored and combined. Three precisions x {real, complex}:
//
//   F64  native IEEE double storage and DFMA arithmetic.
//   F32  float storage and arithmetic; per-row partial sums in float, accumulated
//        in FP64 (SysF32RA / SysF32CA, the engine default) or in float-float
//        pairs (SysF32R / SysF32C), the moment sums and the D accumulator alike;
//        D finished in FP64.
//   DS   "double-single": every real number is an unevaluated sum hi + lo of
//        two floats (about 48 significant bits), stored in 8 bytes like a
//        double, and all arithmetic runs on the FP32 pipe with error-free
//        transformations (Knuth's TwoSum, FMA-based TwoProduct; Dekker 1971,
//        "A floating-point technique for extending the available precision").
//        On this GPU the FP64 pipe issues ~1/58 of the FP32 rate, so DS is
//        the fast path for FP64-accurate results.
//
// Vectors are read and written in 16-byte packets; EPP = elements per packet.
// H entries of a block whose class is "real" are read through hreal().
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fk {

// ---- error-free float transformations (explicit _rn intrinsics: never contracted) ----
__device__ __forceinline__ float2 two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return make_float2(s, e);
}
// acc(hi, lo; unnormalised) += a * b, a and b double-single values
__device__ __forceinline__ void ds_mac(float2& acc, float2 a, float2 b) {
    float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    float2 s = two_sum(acc.x, p);
    acc.x = s.x;
    acc.y = __fadd_rn(acc.y, __fadd_rn(s.y, e));
}
// a * b as an unevaluated hi + lo pair: what ds_mac gives from a zero accumulator, without the
// error-free addition to zero (4 instead of 12 FP32 instructions)
__device__ __forceinline__ float2 ds_mul(float2 a, float2 b) {
    float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return make_float2(p, e);
}
// acc -= a * b
__device__ __forceinline__ void ds_msub(float2& acc, float2 a, float2 b) {
    ds_mac(acc, make_float2(-a.x, -a.y), b);
}
// acc += a (both double-single)
__device__ __forceinline__ void ds_add(float2& acc, float2 a) {
    float2 s = two_sum(acc.x, a.x);
    acc.x = s.x;
    acc.y = __fadd_rn(acc.y, __fadd_rn(s.y, a.y));
}
__device__ __forceinline__ float2 ds_norm(float2 a) {
    float2 s = two_sum(a.x, a.y);
    return s;
}
__device__ __forceinline__ float2 ds_from_double(double d) {
    float hi = __double2float_rn(d);
    float lo = __double2float_rn(d - (double)hi);
    return make_float2(hi, lo);
}
__device__ __forceinline__ double ds_to_double(float2 a) { return (double)a.x + (double)a.y; }

// ---- systems ----
struct SysF64R {
    typedef double E; typedef double H; typedef double Hr; typedef double Acc;
    typedef double Coef; typedef double RowDot; typedef double Dot; typedef double OAcc;
    static constexpr bool CPLX = false; static constexpr int EPP = 2; static constexpr int PREC = 0;   // 0 FP64, 1 FP32, 2 float-float
    __device__ static Coef coef(double c) { return c; }
    __device__ static Acc zero() { return 0.0; }
    __device__ static Hr hreal(H h) { return h; }
    __device__ static void mac(Acc& a, H h, E x) { a = fma(h, x, a); }
    __device__ static void mac_re(Acc& a, Hr h, E x) { a = fma(h, x, a); }
    // y = alpha * acc + beta * z, alpha in {1, 2}, beta in {0, -1}
    // 2 a - z as one fma: 2 a is exact, so fma(2, a, -z) = round(2 a - z), the same value as
    // (2 a) - z with one FP64-pipe instruction instead of two (the flags are kernel arguments)
    __device__ static E fin(Acc a, bool two, bool has_z, E z) {
        if (two && has_z) return fma(2.0, a, -z);
        double v = two ? 2.0 * a : a;
        return has_z ? v - z : v;
    }
    __device__ static void axpy(Acc& a, Coef c, E x) { a = fma(c, x, a); }     // a += c x
    __device__ static Acc from(E x) { return x; }
    __device__ static E to(Acc a) { return a; }
    __device__ static E scale(Coef c, E x) { return c * x; }
    __device__ static void rd_nrm(RowDot& d, E x) { d = fma(x, x, d); }
    __device__ static void rd_re(RowDot& d, E y, E x) { d = fma(y, x, d); }
    __device__ static RowDot rd_zero() { return 0.0; }
    __device__ static Dot dot_zero() { return 0.0; }
    __device__ static void dot_add(Dot& d, RowDot r) { d += r; }
    __device__ static Dot dot_shfl_add(Dot d, int off) { return d + __shfl_xor_sync(0xffffffffu, d, off); }
    __device__ static double dot_get(Dot d) { return d; }
    __device__ static OAcc oa_zero() { return 0.0; }
    __device__ static void oa_mac(OAcc& o, E a, E b) { o = fma(a, b, o); }          // o += a conj(b)
    __device__ static OAcc oa_first(E a, E b) { return a * b; }                        // a conj(b)
    __device__ static OAcc oa_shfl_add(OAcc o, int off) { return o + __shfl_xor_sync(0xffffffffu, o, off); }
    static constexpr bool DACC_DS = false;   // D accumulated in FP64
    __device__ static float2 oa_ds(OAcc, int) { return make_float2(0.f, 0.f); }
    __device__ static double2 oa_get(OAcc o) { return make_double2(o, 0.0); }
    __device__ static OAcc oa_add(OAcc a, OAcc b) { return a + b; }
    __device__ static OAcc oa_shfl(OAcc o, int off) { return __shfl_xor_sync(0xffffffffu, o, off); }
    __device__ static E from_double2(double2 v) { return v.x; }
    __device__ static double2 to_double2(E x) { return make_double2(x, 0.0); }
};

struct SysF64C {
    typedef double2 E; typedef double2 H; typedef double Hr; typedef double2 Acc;
    typedef double Coef; typedef double RowDot; typedef double Dot; typedef double2 OAcc;
    static constexpr bool CPLX = true; static constexpr int EPP = 1; static constexpr int PREC = 0;   // 0 FP64, 1 FP32, 2 float-float
    __device__ static Coef coef(double c) { return c; }
    __device__ static Acc zero() { return make_double2(0.0, 0.0); }
    __device__ static Hr hreal(H h) { return h.x; }
    __device__ static void mac(Acc& a, H h, E x) {
        a.x = fma(h.x, x.x, a.x); a.x = fma(-h.y, x.y, a.x);
        a.y = fma(h.x, x.y, a.y); a.y = fma(h.y, x.x, a.y);
    }
    __device__ static void mac_re(Acc& a, Hr h, E x) { a.x = fma(h, x.x, a.x); a.y = fma(h, x.y, a.y); }
    __device__ static E fin(Acc a, bool two, bool has_z, E z) {
        if (two && has_z) return make_double2(fma(2.0, a.x, -z.x), fma(2.0, a.y, -z.y));   // exact as above
        double vr = two ? 2.0 * a.x : a.x, vi = two ? 2.0 * a.y : a.y;
        return has_z ? make_double2(vr - z.x, vi - z.y) : make_double2(vr, vi);
    }
    __device__ static void axpy(Acc& a, Coef c, E x) { a.x = fma(c, x.x, a.x); a.y = fma(c, x.y, a.y); }
    __device__ static Acc from(E x) { return x; }
    __device__ static E to(Acc a) { return a; }
    __device__ static E scale(Coef c, E x) { return make_double2(c * x.x, c * x.y); }
    __device__ static void rd_nrm(RowDot& d, E x) { d = fma(x.x, x.x, d); d = fma(x.y, x.y, d); }
    __device__ static void rd_re(RowDot& d, E y, E x) { d = fma(y.x, x.x, d); d = fma(y.y, x.y, d); }
    __device__ static RowDot rd_zero() { return 0.0; }
    __device__ static Dot dot_zero() { return 0.0; }
    __device__ static void dot_add(Dot& d, RowDot r) { d += r; }
    __device__ static Dot dot_shfl_add(Dot d, int off) { return d + __shfl_xor_sync(0xffffffffu, d, off); }
    __device__ static double dot_get(Dot d) { return d; }
    __device__ static OAcc oa_zero() { return make_double2(0.0, 0.0); }
    __device__ static void oa_mac(OAcc& o, E a, E b) {   // o += a * conj(b)
        o.x = fma(a.x, b.x, o.x); o.x = fma(a.y, b.y, o.x);
        o.y = fma(a.y, b.x, o.y); o.y = fma(-a.x, b.y, o.y);
    }
    __device__ static OAcc oa_first(E a, E b) {          // a * conj(b), the same roundings as oa_mac from zero
        return make_double2(fma(a.y, b.y, a.x * b.x), fma(-a.x, b.y, a.y * b.x));
    }
    __device__ static OAcc oa_shfl_add(OAcc o, int off) {
        return make_double2(o.x + __shfl_xor_sync(0xffffffffu, o.x, off),
                            o.y + __shfl_xor_sync(0xffffffffu, o.y, off));
    }
    static constexpr bool DACC_DS = false;
    __device__ static float2 oa_ds(OAcc, int) { return make_float2(0.f, 0.f); }
    __device__ static double2 oa_get(OAcc o) { return o; }
    __device__ static OAcc oa_add(OAcc a, OAcc b) { return make_double2(a.x + b.x, a.y + b.y); }
    __device__ static OAcc oa_shfl(OAcc o, int off) {
        return make_double2(__shfl_xor_sync(0xffffffffu, o.x, off), __shfl_xor_sync(0xffffffffu, o.y, off));
    }
    __device__ static E from_double2(double2 v) { return v; }
    __device__ static double2 to_double2(E x) { return x; }
};

struct SysF32R {
    typedef float E; typedef float H; typedef float Hr; typedef float Acc;
    typedef float Coef; typedef float RowDot; typedef float2 Dot; typedef float OAcc;
    static constexpr bool CPLX = false; static constexpr int EPP = 4; static constexpr int PREC = 1;   // 0 FP64, 1 FP32, 2 float-float
    __device__ static Coef coef(double c) { return __double2float_rn(c); }
    __device__ static Acc zero() { return 0.f; }
    __device__ static Hr hreal(H h) { return h; }
    __device__ static void mac(Acc& a, H h, E x) { a = fmaf(h, x, a); }
    __device__ static void mac_re(Acc& a, Hr h, E x) { a = fmaf(h, x, a); }
    __device__ static E fin(Acc a, bool two, bool has_z, E z) {
        if (two && has_z) return fmaf(2.f, a, -z);   // 2 a exact: the same value as (2 a) - z
        float v = two ? 2.f * a : a;
        return has_z ? v - z : v;
    }
    __device__ static void axpy(Acc& a, Coef c, E x) { a = fmaf(c, x, a); }
    __device__ static Acc from(E x) { return x; }
    __device__ static E to(Acc a) { return a; }
    __device__ static E scale(Coef c, E x) { return c * x; }
    __device__ static void rd_nrm(RowDot& d, E x) { d = fmaf(x, x, d); }
    __device__ static void rd_re(RowDot& d, E y, E x) { d = fmaf(y, x, d); }
    __device__ static RowDot rd_zero() { return 0.f; }
    __device__ static Dot dot_zero() { return make_float2(0.f, 0.f); }
    __device__ static void dot_add(Dot& d, RowDot r) { ds_add(d, make_float2(r, 0.f)); }
    __device__ static Dot dot_shfl_add(Dot d, int off) {
        float2 o = make_float2(__shfl_xor_sync(0xffffffffu, d.x, off), __shfl_xor_sync(0xffffffffu, d.y, off));
        ds_add(d, o);
        return d;
    }
    __device__ static double dot_get(Dot d) { return ds_to_double(d); }
    __device__ static OAcc oa_zero() { return 0.f; }
    __device__ static void oa_mac(OAcc& o, E a, E b) { o = fmaf(a, b, o); }
    __device__ static OAcc oa_first(E a, E b) { return a * b; }
    __device__ static OAcc oa_shfl_add(OAcc o, int off) { return o + __shfl_xor_sync(0xffffffffu, o, off); }
    // D accumulated as float-float on the FP32 pipe (the FP64 pipe is ~1/58 of it)
    static constexpr bool DACC_DS = true;
    __device__ static float2 oa_ds(OAcc o, int) { return make_float2(o, 0.f); }
    __device__ static double2 oa_get(OAcc o) { return make_double2((double)o, 0.0); }
    __device__ static OAcc oa_add(OAcc a, OAcc b) { return a + b; }
    __device__ static OAcc oa_shfl(OAcc o, int off) { return __shfl_xor_sync(0xffffffffu, o, off); }
    __device__ static E from_double2(double2 v) { return __double2float_rn(v.x); }
    __device__ static double2 to_double2(E x) { return make_double2((double)x, 0.0); }
};

struct SysF32C {
    typedef float2 E; typedef float2 H; typedef float Hr; typedef float2 Acc;
    typedef float Coef; typedef float RowDot; typedef float2 Dot; typedef float2 OAcc;
    static constexpr bool CPLX = true; static constexpr int EPP = 2; static constexpr int PREC = 1;   // 0 FP64, 1 FP32, 2 float-float
    __device__ static Coef coef(double c) { return __double2float_rn(c); }
    __device__ static Acc zero() { return make_float2(0.f, 0.f); }
    __device__ static Hr hreal(H h) { return h.x; }
    __device__ static void mac(Acc& a, H h, E x) {
        a.x = fmaf(h.x, x.x, a.x); a.x = fmaf(-h.y, x.y, a.x);
        a.y = fmaf(h.x, x.y, a.y); a.y = fmaf(h.y, x.x, a.y);
    }
    __device__ static void mac_re(Acc& a, Hr h, E x) { a.x = fmaf(h, x.x, a.x); a.y = fmaf(h, x.y, a.y); }
    __device__ static E fin(Acc a, bool two, bool has_z, E z) {
        if (two && has_z) return make_float2(fmaf(2.f, a.x, -z.x), fmaf(2.f, a.y, -z.y));   // exact as above
        float vr = two ? 2.f * a.x : a.x, vi = two ? 2.f * a.y : a.y;
        return has_z ? make_float2(vr - z.x, vi - z.y) : make_float2(vr, vi);
    }
    __device__ static void axpy(Acc& a, Coef c, E x) { a.x = fmaf(c, x.x, a.x); a.y = fmaf(c, x.y, a.y); }
    __device__ static Acc from(E x) { return x; }
    __device__ static E to(Acc a) { return a; }
    __device__ static E scale(Coef c, E x) { return make_float2(c * x.x, c * x.y); }
    __device__ static void rd_nrm(RowDot& d, E x) { d = fmaf(x.x, x.x, d); d = fmaf(x.y, x.y, d); }
    __device__ static void rd_re(RowDot& d, E y, E x) { d = fmaf(y.x, x.x, d); d = fmaf(y.y, x.y, d); }
    __device__ static RowDot rd_zero() { return 0.f; }
    __device__ static Dot dot_zero() { return make_float2(0.f, 0.f); }
    __device__ static void dot_add(Dot& d, RowDot r) { ds_add(d, make_float2(r, 0.f)); }
    __device__ static Dot dot_shfl_add(Dot d, int off) {
        float2 o = make_float2(__shfl_xor_sync(0xffffffffu, d.x, off), __shfl_xor_sync(0xffffffffu, d.y, off));
        ds_add(d, o);
        return d;
    }
    __device__ static double dot_get(Dot d) { return ds_to_double(d); }
    __device__ static OAcc oa_zero() { return make_float2(0.f, 0.f); }
    __device__ static void oa_mac(OAcc& o, E a, E b) {
        o.x = fmaf(a.x, b.x, o.x); o.x = fmaf(a.y, b.y, o.x);
        o.y = fmaf(a.y, b.x, o.y); o.y = fmaf(-a.x, b.y, o.y);
    }
    __device__ static OAcc oa_first(E a, E b) {
        return make_float2(fmaf(a.y, b.y, a.x * b.x), fmaf(-a.x, b.y, a.y * b.x));
    }
    __device__ static OAcc oa_shfl_add(OAcc o, int off) {
        return make_float2(o.x + __shfl_xor_sync(0xffffffffu, o.x, off),
                           o.y + __shfl_xor_sync(0xffffffffu, o.y, off));
    }
    static constexpr bool DACC_DS = true;
    __device__ static float2 oa_ds(OAcc o, int comp) { return make_float2(comp ? o.y : o.x, 0.f); }
    __device__ static double2 oa_get(OAcc o) { return make_double2((double)o.x, (double)o.y); }
    __device__ static OAcc oa_add(OAcc a, OAcc b) { return make_float2(a.x + b.x, a.y + b.y); }
    __device__ static OAcc oa_shfl(OAcc o, int off) {
        return make_float2(__shfl_xor_sync(0xffffffffu, o.x, off), __shfl_xor_sync(0xffffffffu, o.y, off));
    }
    __device__ static E from_double2(double2 v) { return make_float2(__double2float_rn(v.x), __double2float_rn(v.y)); }
    __device__ static double2 to_double2(E x) { return make_double2((double)x.x, (double)x.y); }
};

// FP32 storage and arithmetic with FP64 accumulators: each thread's moment sums are doubles
// (one DADD per column chunk), and the D accumulator holds one double per real, updated by a
// DFMA from the chunk's FP32 lane reduction. Everything else is the FP32 system's.
struct SysF32RA : SysF32R {
    typedef double Dot;
    __device__ static Dot dot_zero() { return 0.0; }
    __device__ static void dot_add(Dot& d, RowDot r) { d += (double)r; }
    __device__ static Dot dot_shfl_add(Dot d, int off) { return d + __shfl_xor_sync(0xffffffffu, d, off); }
    __device__ static double dot_get(Dot d) { return d; }
    static constexpr bool DACC_DS = false;
};
struct SysF32CA : SysF32C {
    typedef double Dot;
    __device__ static Dot dot_zero() { return 0.0; }
    __device__ static void dot_add(Dot& d, RowDot r) { d += (double)r; }
    __device__ static Dot dot_shfl_add(Dot d, int off) { return d + __shfl_xor_sync(0xffffffffu, d, off); }
    __device__ static double dot_get(Dot d) { return d; }
    static constexpr bool DACC_DS = false;
};

// Double-single real: E = (hi, lo)
struct SysDSR {
    typedef float2 E; typedef float2 H; typedef float2 Hr; typedef float2 Acc;
    typedef float2 Coef; typedef float2 RowDot; typedef float2 Dot; typedef float2 OAcc;
    static constexpr bool CPLX = false; static constexpr int EPP = 2; static constexpr int PREC = 2;   // 0 FP64, 1 FP32, 2 float-float
    __device__ static Coef coef(double c) { return ds_from_double(c); }
    __device__ static Acc zero() { return make_float2(0.f, 0.f); }
    __device__ static Hr hreal(H h) { return h; }
    __device__ static void mac(Acc& a, H h, E x) { ds_mac(a, h, x); }
    __device__ static void mac_re(Acc& a, Hr h, E x) { ds_mac(a, h, x); }
    // a += x and a = h a: a row's identity blocks of one value h summed first, scaled once
    __device__ static void acc_add(Acc& a, E x) { ds_add(a, x); }
    __device__ static void acc_scale(Acc& a, Hr h) { a = ds_mul(h, a); }
    __device__ static E fin(Acc a, bool two, bool has_z, E z) {
        float2 v = ds_norm(a);
        if (two) { v.x *= 2.f; v.y *= 2.f; }
        if (has_z) { ds_add(v, make_float2(-z.x, -z.y)); v = fast_two_sum(v.x, v.y); }
        return v;
    }
    __device__ static void axpy(Acc& a, Coef c, E x) { ds_mac(a, c, x); }
    __device__ static Acc from(E x) { return x; }
    __device__ static E to(Acc a) { return ds_norm(a); }
    __device__ static E scale(Coef c, E x) { float2 a = make_float2(0.f, 0.f); ds_mac(a, c, x); return ds_norm(a); }
    __device__ static void rd_nrm(RowDot& d, E x) { ds_mac(d, x, x); }
    __device__ static void rd_re(RowDot& d, E y, E x) { ds_mac(d, y, x); }
    __device__ static RowDot rd_zero() { return make_float2(0.f, 0.f); }
    __device__ static Dot dot_zero() { return make_float2(0.f, 0.f); }
    __device__ static void dot_add(Dot& d, RowDot r) { ds_add(d, r); }
    __device__ static Dot dot_shfl_add(Dot d, int off) {
        float2 o = make_float2(__shfl_xor_sync(0xffffffffu, d.x, off), __shfl_xor_sync(0xffffffffu, d.y, off));
        ds_add(d, o);
        return d;
    }
    __device__ static double dot_get(Dot d) { return ds_to_double(d); }
    __device__ static OAcc oa_zero() { return make_float2(0.f, 0.f); }
    __device__ static void oa_mac(OAcc& o, E a, E b) { ds_mac(o, a, b); }
    __device__ static OAcc oa_first(E a, E b) { return ds_mul(a, b); }
    __device__ static OAcc oa_shfl_add(OAcc o, int off) {
        float2 t = make_float2(__shfl_xor_sync(0xffffffffu, o.x, off), __shfl_xor_sync(0xffffffffu, o.y, off));
        ds_add(o, t);
        return ds_norm(o);
    }
    static constexpr bool DACC_DS = true;
    __device__ static float2 oa_ds(OAcc o, int) { return o; }
    __device__ static double2 oa_get(OAcc o) { return make_double2(ds_to_double(o), 0.0); }
    __device__ static OAcc oa_add(OAcc a, OAcc b) { ds_add(a, b); return a; }
    __device__ static OAcc oa_shfl(OAcc o, int off) {
        return make_float2(__shfl_xor_sync(0xffffffffu, o.x, off), __shfl_xor_sync(0xffffffffu, o.y, off));
    }
    __device__ static E from_double2(double2 v) { return ds_from_double(v.x); }
    __device__ static double2 to_double2(E x) { return make_double2(ds_to_double(x), 0.0); }
};

// Double-single complex: E = (re.hi, re.lo, im.hi, im.lo)
struct SysDSC {
    typedef float4 E; typedef float4 H; typedef float2 Hr; typedef float4 Acc;
    typedef float2 Coef; typedef float2 RowDot; typedef float2 Dot; typedef float4 OAcc;
    static constexpr bool CPLX = true; static constexpr int EPP = 1; static constexpr int PREC = 2;   // 0 FP64, 1 FP32, 2 float-float
    __device__ static float2 re(float4 v) { return make_float2(v.x, v.y); }
    __device__ static float2 im(float4 v) { return make_float2(v.z, v.w); }
    __device__ static float4 pack(float2 r, float2 i) { return make_float4(r.x, r.y, i.x, i.y); }
    __device__ static Coef coef(double c) { return ds_from_double(c); }
    __device__ static Acc zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static Hr hreal(H h) { return re(h); }
    __device__ static void mac(Acc& a, H h, E x) {
        float2 ar = re(a), ai = im(a);
        ds_mac(ar, re(h), re(x)); ds_msub(ar, im(h), im(x));
        ds_mac(ai, re(h), im(x)); ds_mac(ai, im(h), re(x));
        a = pack(ar, ai);
    }
    __device__ static void mac_re(Acc& a, Hr h, E x) {
        float2 ar = re(a), ai = im(a);
        ds_mac(ar, h, re(x)); ds_mac(ai, h, im(x));
        a = pack(ar, ai);
    }
    __device__ static void acc_add(Acc& a, E x) {   // a += x
        float2 ar = re(a), ai = im(a);
        ds_add(ar, re(x)); ds_add(ai, im(x));
        a = pack(ar, ai);
    }
    __device__ static void acc_scale(Acc& a, Hr h) { a = pack(ds_mul(h, re(a)), ds_mul(h, im(a))); }   // a = h a
    __device__ static E fin(Acc a, bool two, bool has_z, E z) {
        float2 vr = SysDSR::fin(re(a), two, has_z, re(z));
        float2 vi = SysDSR::fin(im(a), two, has_z, im(z));
        return pack(vr, vi);
    }
    __device__ static void axpy(Acc& a, Coef c, E x) {
        float2 ar = re(a), ai = im(a);
        ds_mac(ar, c, re(x)); ds_mac(ai, c, im(x));
        a = pack(ar, ai);
    }
    __device__ static Acc from(E x) { return x; }
    __device__ static E to(Acc a) { return pack(ds_norm(re(a)), ds_norm(im(a))); }
    __device__ static E scale(Coef c, E x) { return pack(SysDSR::scale(c, re(x)), SysDSR::scale(c, im(x))); }
    __device__ static void rd_nrm(RowDot& d, E x) { ds_mac(d, re(x), re(x)); ds_mac(d, im(x), im(x)); }
    __device__ static void rd_re(RowDot& d, E y, E x) { ds_mac(d, re(y), re(x)); ds_mac(d, im(y), im(x)); }
    __device__ static RowDot rd_zero() { return make_float2(0.f, 0.f); }
    __device__ static Dot dot_zero() { return make_float2(0.f, 0.f); }
    __device__ static void dot_add(Dot& d, RowDot r) { ds_add(d, r); }
    __device__ static Dot dot_shfl_add(Dot d, int off) {
        float2 o = make_float2(__shfl_xor_sync(0xffffffffu, d.x, off), __shfl_xor_sync(0xffffffffu, d.y, off));
        ds_add(d, o);
        return d;
    }
    __device__ static double dot_get(Dot d) { return ds_to_double(d); }
    __device__ static OAcc oa_zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static void oa_mac(OAcc& o, E a, E b) {   // o += a * conj(b)
        float2 orr = re(o), oi = im(o);
        ds_mac(orr, re(a), re(b)); ds_mac(orr, im(a), im(b));
        ds_mac(oi, im(a), re(b)); ds_msub(oi, re(a), im(b));
        o = pack(orr, oi);
    }
    __device__ static OAcc oa_first(E a, E b) {          // a * conj(b): oa_mac from zero, first products exact
        float2 orr = ds_mul(re(a), re(b)), oi = ds_mul(im(a), re(b));
        ds_mac(orr, im(a), im(b));
        ds_msub(oi, re(a), im(b));
        return pack(orr, oi);
    }
    __device__ static OAcc oa_shfl_add(OAcc o, int off) {
        return pack(SysDSR::oa_shfl_add(re(o), off), SysDSR::oa_shfl_add(im(o), off));
    }
    static constexpr bool DACC_DS = true;
    __device__ static float2 oa_ds(OAcc o, int comp) { return comp ? im(o) : re(o); }
    __device__ static double2 oa_get(OAcc o) { return make_double2(ds_to_double(re(o)), ds_to_double(im(o))); }
    __device__ static OAcc oa_add(OAcc a, OAcc b) {
        float2 r = re(a), i = im(a);
        ds_add(r, re(b));
        ds_add(i, im(b));
        return pack(r, i);
    }
    __device__ static OAcc oa_shfl(OAcc o, int off) {
        return make_float4(__shfl_xor_sync(0xffffffffu, o.x, off), __shfl_xor_sync(0xffffffffu, o.y, off),
                           __shfl_xor_sync(0xffffffffu, o.z, off), __shfl_xor_sync(0xffffffffu, o.w, off));
    }
    __device__ static E from_double2(double2 v) { return pack(ds_from_double(v.x), ds_from_double(v.y)); }
    __device__ static double2 to_double2(E x) { return make_double2(ds_to_double(re(x)), ds_to_double(im(x))); }
};

}  // namespace fk
