"""ctypes loader of the oracle (TEST INFRASTRUCTURE ONLY).

CPU restatement of the reference's CPU engine; used only by tests/, the smoke
test and bench.py's CPU-baseline leg, to check results. PARITY UNPINNED against the
reference itself (no reference tests or golden vectors; the reference needs
Armadillo/Boost and does not build here); pinned against analytic known
answers in tests/.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_p = C.c_void_p
_i = C.c_int
_d = C.c_double
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

_SIG = {
    "orc_engine_create": (_p, [_i, _i]),
    "orc_engine_destroy": (None, [_p]),
    "orc_engine_threads": (_i, [_p]),
    "orc_set_H": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _d, _d]),
    "orc_set_R": (_i, [_p, _i, _i, _dp]),
    "orc_moments": (_i, [_p, _i, _dp]),
    "orc_stoch_matrix": (_i, [_p, _i, _dp, _i, _ip, _ip, _dp]),
    "orc_autodiff_matrix": (_i, [_p, _i, _dp, _i, _i, _ip, _ip, _ip, _dp]),
    "orc_energy_scale": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _d, _i, _dp, _dp, _dp]),
    "orc_tridiag_extremes": (None, [_i, _dp, _dp, _dp, _dp]),
    "orc_R_identity": (_i, [_i, _i, _i, _i, _dp]),
    "orc_R_uncorrelated": (_i, [_i, _i, _i, C.c_uint32, C.c_ulonglong, _i, _i, _dp]),
    "orc_R_correlated": (_i, [_i, _i, _ip, C.c_uint32, C.c_ulonglong, _i, _i, _dp]),
    "orc_bsr_build": (_i, [_i, _i, _i, _i, _ip, _ip, _dp, _ip, _ip, _ip, _dp]),
    "orc_bsr_symmetrize": (_i, [_i, _i, _i, _i, _ip, _ip, _ip, _dp]),
    "orc_jackson_kernel": (None, [_i, _dp]),
    "orc_chebyshev_fill_array": (None, [_d, _i, _i, _dp]),
    "orc_fermi_density": (_d, [_d, _d, _d]),
    "orc_fermi_energy": (_d, [_d, _d, _d]),
    "orc_expansion_coefficients": (None, [_i, _i, _i, _d, _d, _d, _d, _dp]),
    "orc_moment_product": (_d, [_i, _dp, _dp]),
    "orc_moment_transform": (None, [_i, _dp, _i, _dp]),
    "orc_moments2_v1": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _ip, _ip, _dp, _dp]),
    "orc_moments2_v2": (_i, [_p, _i, _i, _i, _ip, _ip, _dp, _ip, _ip, _dp, _dp, _dp]),
    "orc_electrical_conductivity_coefficients": (_i, [_i, _i, _d, _d, _d, _d, _d, _dp, _dp]),
    "orc_mu_to_filling": (_d, [_i, _dp, _d, _d, _d, _d]),
    "orc_filling_to_mu": (_d, [_i, _dp, _d, _d, _d, _d, _d]),
    "orc_electronic_energy": (_d, [_i, _dp, _d, _d, _d, _d, _d]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _ip_(a):
    return a.ctypes.data_as(_ip)


def _dp_(a):
    return a.ctypes.data_as(_dp)


def _dbl(a):
    a = np.asarray(a)
    if np.iscomplexobj(a):
        return np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleEngine:
    """Engine_CPU<T> restated (reference src/engine_cpu.cpp)."""

    def __init__(self, complex_values=False, nthreads=0):
        self.L = lib()
        self.cplx = bool(complex_values)
        self.h = self.L.orc_engine_create(int(self.cplx), int(nthreads))
        self.threads = self.L.orc_engine_threads(self.h)
        self.es = None

    def __del__(self):
        try:
            self.L.orc_engine_destroy(self.h)
        except Exception:
            pass

    def set_H(self, H, es):
        self.es = es
        self._H = H
        v = _dbl(H.val)
        st = self.L.orc_set_H(self.h, H.n_rows, H.b_len, H.n_blocks(), _ip_(H.row_ptr), _ip_(H.col_idx), _dp_(v),
                              es.lo, es.hi)
        assert st == 0, st

    def set_R(self, R):
        dt = np.complex128 if self.cplx else np.float64
        n, s = R.shape
        flat = np.ascontiguousarray(np.asarray(R, dt).reshape(-1, order="F"))
        st = self.L.orc_set_R(self.h, n, s, _dp_(_dbl(flat)))
        assert st == 0, st

    def moments(self, M):
        mu = np.zeros(M)
        st = self.L.orc_moments(self.h, M, _dp_(mu))
        assert st == 0, st
        return mu

    def stoch_matrix(self, c, D):
        dt = np.complex128 if self.cplx else np.float64
        out = np.zeros(D.n_blocks() * D.b_len ** 2, dt)
        c = np.ascontiguousarray(c, np.float64)
        st = self.L.orc_stoch_matrix(self.h, len(c), _dp_(c), D.n_blocks(), _ip_(D.row_idx), _ip_(D.col_idx),
                                     _dp_(_dbl(out)))
        assert st == 0, st
        return out

    def autodiff_matrix(self, c, D):
        dt = np.complex128 if self.cplx else np.float64
        out = np.zeros(D.n_blocks() * D.b_len ** 2, dt)
        c = np.ascontiguousarray(c, np.float64)
        st = self.L.orc_autodiff_matrix(self.h, len(c), _dp_(c), D.n_rows, D.n_blocks(), _ip_(D.row_ptr),
                                        _ip_(D.row_idx), _ip_(D.col_idx), _dp_(_dbl(out)))
        assert st == 0, st
        return out

    def moments2_v1(self, M, j1, j2):
        """mu[m1, m2] = sum_k <T_m1 r_k, j2 T_m2 j1 r_k> (src/engine_cpu.cpp:86-160), (M, M) complex."""
        out = np.zeros(2 * M * M)
        v1 = _dbl(j1.val)
        v2 = _dbl(j2.val)
        st = lib().orc_moments2_v1(self.h, M, j1.n_rows, j1.b_len, _ip_(j1.row_ptr), _ip_(j1.col_idx), _dp_(v1),
                                   _ip_(j2.row_ptr), _ip_(j2.col_idx), _dp_(v2), _dp_(out))
        if st:
            raise RuntimeError("orc_moments2_v1: status %d" % st)
        return out.view(np.complex128).reshape(M, M)

    def moments2_v2(self, M, j1, j2, R2=None):
        """mu[m1, m2] = tr(A_m1 B_m2), A_i = R^dag T_i j2 R2, B_i = R2^dag T_i j1 R
        (src/engine_cpu.cpp:162-209), (M, M) complex; R2 = R when None."""
        out = np.zeros(2 * M * M)
        v1 = _dbl(j1.val)
        v2 = _dbl(j2.val)
        r2 = None
        if R2 is not None:
            dt = np.complex128 if self.cplx else np.float64
            r2 = _dbl(np.ascontiguousarray(np.asarray(R2, dt).reshape(-1, order="F")))
        st = lib().orc_moments2_v2(self.h, M, j1.n_rows, j1.b_len, _ip_(j1.row_ptr), _ip_(j1.col_idx), _dp_(v1),
                                   _ip_(j2.row_ptr), _ip_(j2.col_idx), _dp_(v2),
                                   _dp_(r2) if r2 is not None else None, _dp_(out))
        if st:
            raise RuntimeError("orc_moments2_v2: status %d" % st)
        return out.view(np.complex128).reshape(M, M)

    def energy_scale(self, H, extend, iters, v0):
        lo, hi = C.c_double(), C.c_double()
        st = self.L.orc_energy_scale(self.h, H.n_rows, H.b_len, H.n_blocks(), _ip_(H.row_ptr), _ip_(H.col_idx),
                                     _dp_(_dbl(H.val)), extend, iters, _dp_(_dbl(v0)), C.byref(lo), C.byref(hi))
        assert st == 0, st
        return lo.value, hi.value


def R_uncorrelated(n, s, seed, discard=0, j_start=0, j_end=None, complex_values=False):
    j_end = s if j_end is None else j_end
    dt = np.complex128 if complex_values else np.float64
    flat = np.zeros(n * (j_end - j_start), dt)
    st = lib().orc_R_uncorrelated(int(complex_values), n, s, seed, discard, j_start, j_end, _dp_(_dbl(flat)))
    assert st == 0
    return flat.reshape((n, j_end - j_start), order="F")


def R_correlated(groups, seed, discard=0, j_start=0, j_end=None, complex_values=False):
    g = np.ascontiguousarray(groups, np.int32)
    n = len(g)
    j_end = int(g.max()) + 1 if j_end is None else j_end
    dt = np.complex128 if complex_values else np.float64
    flat = np.zeros(n * (j_end - j_start), dt)
    st = lib().orc_R_correlated(int(complex_values), n, _ip_(g), seed, discard, j_start, j_end, _dp_(_dbl(flat)))
    assert st == 0
    return flat.reshape((n, j_end - j_start), order="F")


def R_identity(n, j_start=0, j_end=None, complex_values=False):
    j_end = n if j_end is None else j_end
    dt = np.complex128 if complex_values else np.float64
    flat = np.zeros(n * (j_end - j_start), dt)
    st = lib().orc_R_identity(int(complex_values), n, j_start, j_end, _dp_(_dbl(flat)))
    assert st == 0
    return flat.reshape((n, j_end - j_start), order="F")


def bsr_build(n_rows, b, row_idx, col_idx, blocks, complex_values):
    dt = np.complex128 if complex_values else np.float64
    ne = len(row_idx)
    v = np.ascontiguousarray(blocks, dt).reshape(-1)
    rp = np.zeros(n_rows + 1, np.int32)
    ri = np.zeros(max(ne, 1), np.int32)
    ci = np.zeros(max(ne, 1), np.int32)
    vo = np.zeros(max(ne, 1) * b * b, dt)
    k = lib().orc_bsr_build(int(complex_values), n_rows, b, ne, _ip_(np.ascontiguousarray(row_idx, np.int32)),
                            _ip_(np.ascontiguousarray(col_idx, np.int32)), _dp_(_dbl(v)), _ip_(rp), _ip_(ri),
                            _ip_(ci), _dp_(_dbl(vo)))
    return rp, ri[:k], ci[:k], vo[:k * b * b]


def jackson_kernel(M):
    out = np.zeros(M)
    lib().orc_jackson_kernel(M, _dp_(out))
    return out


def expansion_coefficients(M, Mq, kind, kT, mu, lo, hi):
    out = np.zeros(M)
    lib().orc_expansion_coefficients(M, Mq, {"fermi_density": 0, "fermi_energy": 1}[kind], kT, mu, lo, hi, _dp_(out))
    return out


def tridiag_extremes(alpha, beta):
    a = np.ascontiguousarray(alpha, np.float64)
    b = np.ascontiguousarray(beta, np.float64)
    lo, hi = C.c_double(), C.c_double()
    lib().orc_tridiag_extremes(len(a), _dp_(a), _dp_(b), C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def moment_transform(mu, Mq):
    mu = np.ascontiguousarray(mu, np.float64)
    gamma = np.zeros(Mq)
    lib().orc_moment_transform(len(mu), _dp_(mu), Mq, _dp_(gamma))
    return gamma


def mu_to_filling(gamma, lo, hi, kT, mu):
    g = np.ascontiguousarray(gamma, np.float64)
    return lib().orc_mu_to_filling(len(g), _dp_(g), lo, hi, kT, mu)


def filling_to_mu(gamma, lo, hi, kT, filling, delta_filling=0.0):
    g = np.ascontiguousarray(gamma, np.float64)
    return lib().orc_filling_to_mu(len(g), _dp_(g), lo, hi, kT, filling, delta_filling)


def electronic_energy(gamma, lo, hi, kT, filling, mu):
    g = np.ascontiguousarray(gamma, np.float64)
    return lib().orc_electronic_energy(len(g), _dp_(g), lo, hi, kT, filling, mu)


def electrical_conductivity_coefficients(M, Mq, kT, mu, omega, lo, hi, kernel):
    k = np.ascontiguousarray(kernel, np.float64)
    out = np.zeros(2 * M * M)
    st = lib().orc_electrical_conductivity_coefficients(M, Mq, kT, mu, omega, lo, hi, _dp_(k), _dp_(out))
    if st:
        raise ValueError("electrical_conductivity_coefficients: reference assertion")
    return out.view(np.complex128).reshape(M, M)
