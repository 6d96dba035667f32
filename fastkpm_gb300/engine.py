"""Python mirror of the reference's fkpm interface (reference src/fastkpm.h:16-250),
calling the GB300 engine through the C ABI.

    eng = mk_engine(complex_values=False)          # mk_engine<double>()
    eng.set_H(H, EnergyScale(-4.5, 4.5))
    eng.set_R_uncorrelated(n, s, RNG(seed))
    mu = eng.moments(M)
    c = expansion_coefficients(M, 2 * M, "fermi_density", 0.0, 0.0, es)
    eng.stoch_matrix(c, D)                          # D.val overwritten on D's pattern

Values follow the reference layouts: R is column-major n x s (a Fortran-ordered
numpy array), SpMatBsr.val holds nnzb blocks of b*b column-major entries.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _as_doubles(a):
    """Contiguous float64 view of a real or complex128 array (interleaved re, im)."""
    a = np.asarray(a)
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        return a.view(np.float64)
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class EnergyScale:
    """Spectral bounds (reference src/fastkpm.h:112-122)."""

    def __init__(self, lo, hi):
        self.lo = float(lo)
        self.hi = float(hi)

    def avg(self):
        return (self.hi + self.lo) / 2.0

    def mag(self):
        return (self.hi - self.lo) / 2.0

    def scale(self, x):
        return (x - self.avg()) / self.mag()

    def unscale(self, x):
        return x * self.mag() + self.avg()

    def __repr__(self):
        return "EnergyScale(lo=%r, hi=%r)" % (self.lo, self.hi)


class RNG:
    """State of a std::mt19937 master generator: its seed and the draws taken so far.

    Probe generation consumes exactly j_end - j_start draws, like the reference's
    set_R_* (src/engine.cpp:56, src/engine_cusparse.cpp:1085)."""

    def __init__(self, seed=5489, discard=0):
        self.seed = int(seed) & 0xFFFFFFFF
        self.drawn = int(discard)

    def discard(self, k):
        self.drawn += int(k)


class SpMatBsr:
    """Block-sparse matrix (reference src/fastkpm.h:66-106), numpy storage."""

    def __init__(self, n_rows=0, b_len=1, row_ptr=None, col_idx=None, val=None, complex_values=False):
        self.n_rows = self.n_cols = int(n_rows)
        self.b_len = int(b_len)
        self.row_ptr = _i32(row_ptr if row_ptr is not None else np.zeros(n_rows + 1, np.int32))
        self.col_idx = _i32(col_idx if col_idx is not None else np.zeros(0, np.int32))
        self.row_idx = np.repeat(np.arange(self.n_rows, dtype=np.int32), np.diff(self.row_ptr)).astype(np.int32)
        dt = np.complex128 if complex_values else np.float64
        if val is None:
            val = np.zeros(len(self.col_idx) * self.b_len ** 2, dt)
        self.val = np.ascontiguousarray(val, dtype=dt).reshape(-1)

    @property
    def is_complex(self):
        return np.iscomplexobj(self.val)

    def n_blocks(self):
        return len(self.col_idx)

    @classmethod
    def build(cls, n_rows, b_len, row_idx, col_idx, blocks, complex_values=None):
        """SpMatBsr(SpMatElems) (reference src/spmat.cpp:46-129): sort by (row, col), sum duplicates.
        blocks: (n_elems, b*b) column-major entries."""
        lib = L.load()
        blocks = np.asarray(blocks)
        cplx = np.iscomplexobj(blocks) if complex_values is None else complex_values
        ne = len(row_idx)
        dt = np.complex128 if cplx else np.float64
        vin = np.ascontiguousarray(blocks, dtype=dt).reshape(-1)
        rp = np.zeros(n_rows + 1, np.int32)
        ri = np.zeros(max(ne, 1), np.int32)
        ci = np.zeros(max(ne, 1), np.int32)
        vout = np.zeros(max(ne, 1) * b_len * b_len, dt)
        nnzb = C.c_int(0)
        rri, rci = _i32(row_idx), _i32(col_idx)
        st = lib.fk_bsr_build(L.FK_COMPLEX if cplx else L.FK_REAL, n_rows, b_len, ne, _ip(rri), _ip(rci),
                              _dp(_as_doubles(vin)), _ip(rp), _ip(ri), _ip(ci), _dp(vout.view(np.float64)),
                              C.byref(nnzb))
        if st != L.FK_OK:
            raise L.FkError(st, "SpMatBsr.build")
        k = nnzb.value
        return cls(n_rows, b_len, rp, ci[:k], vout[:k * b_len * b_len], complex_values=cplx)

    def copy(self):
        return SpMatBsr(self.n_rows, self.b_len, self.row_ptr.copy(), self.col_idx.copy(), self.val.copy(),
                        complex_values=self.is_complex)

    def with_values(self, val):
        """A matrix on this pattern whose values are `val` (no copy); the pattern arrays are shared."""
        m = object.__new__(SpMatBsr)
        m.n_rows = m.n_cols = self.n_rows
        m.b_len = self.b_len
        m.row_ptr, m.col_idx, m.row_idx = self.row_ptr, self.col_idx, self.row_idx
        m.val = val.reshape(-1)
        return m

    def pattern_like(self, complex_values=None):
        """Same pattern, zero values (the D argument of stoch/autodiff)."""
        cplx = self.is_complex if complex_values is None else complex_values
        return SpMatBsr(self.n_rows, self.b_len, self.row_ptr.copy(), self.col_idx.copy(), None, complex_values=cplx)

    def zeros(self):
        self.val[:] = 0

    def find_index(self, i, j):
        lo, hi = self.row_ptr[i], self.row_ptr[i + 1]
        k = lo + np.searchsorted(self.col_idx[lo:hi], j)
        if k >= hi or self.col_idx[k] != j:
            raise KeyError("block (%d, %d) not stored" % (i, j))
        return int(k)

    def block(self, i, j):
        b = self.b_len
        k = self.find_index(i, j)
        return self.val[k * b * b:(k + 1) * b * b].reshape(b, b, order="F")

    def symmetrize(self):
        lib = L.load()
        st = lib.fk_bsr_symmetrize(L.FK_COMPLEX if self.is_complex else L.FK_REAL, self.n_rows, self.b_len,
                                   self.n_blocks(), _ip(self.row_ptr), _ip(self.row_idx), _ip(self.col_idx),
                                   _dp(self.val.view(np.float64)))
        if st != L.FK_OK:
            raise L.FkError(st, "SpMatBsr.symmetrize")

    def scale(self, alpha):
        self.val *= alpha

    def to_dense(self):
        b, n = self.b_len, self.n_rows
        A = np.zeros((n * b, n * b), self.val.dtype)
        for k in range(self.n_blocks()):
            i, j = self.row_idx[k], self.col_idx[k]
            A[b * i:b * i + b, b * j:b * j + b] = self.val[k * b * b:(k + 1) * b * b].reshape(b, b, order="F")
        return A


def jackson_kernel(M):
    out = np.zeros(M)
    st = L.load().fk_jackson_kernel(M, _dp(out))
    if st != L.FK_OK:
        raise L.FkError(st, "jackson_kernel")
    return out


def expansion_coefficients(M, Mq, f, kT, mu, es):
    """c_m for f = 'fermi_density' or 'fermi_energy' at (kT, mu) on es (reference src/fastkpm.cpp:41-78)."""
    kind = {"fermi_density": 0, "fermi_energy": 1}[f]
    out = np.zeros(M)
    st = L.load().fk_expansion_coefficients(M, Mq, kind, kT, mu, es.lo, es.hi, _dp(out))
    if st != L.FK_OK:
        raise L.FkError(st, "expansion_coefficients")
    return out


def moment_product(c, mu):
    return float(np.dot(np.asarray(c, float), np.asarray(mu, float)))


def probe_identity(n, j_start=0, j_end=None, complex_values=False):
    j_end = n if j_end is None else j_end
    dt = np.complex128 if complex_values else np.float64
    R = np.zeros((n, j_end - j_start), dt, order="F")
    st = L.load().fk_probe_identity(L.FK_COMPLEX if complex_values else L.FK_REAL, n, j_start, j_end,
                                    _dp(R.reshape(-1, order="F").view(np.float64)))
    if st != L.FK_OK:
        raise L.FkError(st, "probe_identity")
    return R


def probe_uncorrelated(n, s, rng, j_start=0, j_end=None, complex_values=False):
    """set_R_uncorrelated's R (reference src/engine.cpp:50-70); advances rng by j_end - j_start draws."""
    j_end = s if j_end is None else j_end
    dt = np.complex128 if complex_values else np.float64
    flat = np.zeros(n * (j_end - j_start), dt)
    st = L.load().fk_probe_uncorrelated(L.FK_COMPLEX if complex_values else L.FK_REAL, n, s, rng.seed, rng.drawn,
                                        j_start, j_end, _dp(flat.view(np.float64)))
    if st != L.FK_OK:
        raise L.FkError(st, "probe_uncorrelated")
    rng.discard(j_end - j_start)
    return flat.reshape((n, j_end - j_start), order="F")


def probe_correlated(groups, rng, j_start=0, j_end=None, complex_values=False):
    """set_R_correlated's R (reference src/engine.cpp:76-116), identity fallback when s >= n."""
    g = _i32(groups)
    n = len(g)
    if j_end is None:
        s = int(g.max()) + 1
        if int(g.min()) != 0:
            raise ValueError("groups must start at 0")
        if s >= n:
            return probe_identity(n, 0, n, complex_values)
        j_start, j_end = 0, s
    dt = np.complex128 if complex_values else np.float64
    flat = np.zeros(n * (j_end - j_start), dt)
    st = L.load().fk_probe_correlated(L.FK_COMPLEX if complex_values else L.FK_REAL, n, _ip(g), rng.seed, rng.drawn,
                                      j_start, j_end, _dp(flat.view(np.float64)))
    if st != L.FK_OK:
        raise L.FkError(st, "probe_correlated")
    rng.discard(j_end - j_start)
    return flat.reshape((n, j_end - j_start), order="F")


def device_count():
    n = C.c_int(0)
    st = L.load().fk_device_count(C.byref(n))
    return n.value if st == L.FK_OK else 0


class Engine:
    """GB300 engine with the reference's Engine<T> members (reference src/fastkpm.h:185-234)."""

    def __init__(self, complex_values=False, precision="fp64", device=0):
        self.lib = L.load()
        self.complex_values = bool(complex_values)
        self.precision = precision
        h = C.c_void_p()
        st = self.lib.fk_engine_create(device, L.FK_COMPLEX if complex_values else L.FK_REAL,
                                       L.PRECISIONS[precision], C.byref(h))
        if st != L.FK_OK:
            raise L.FkError(st, "mk_engine")
        self.h = h
        self.R = None
        self.R2 = None
        self._r_shape = None
        self.es = None
        self._H = None

    # -- plumbing --
    def _check(self, st, where):
        if st != L.FK_OK:
            raise L.FkError(st, where, self.lib.fk_engine_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fk_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, opt, value):
        self._check(self.lib.fk_engine_set_option(self.h, opt, int(value)), "set_option")

    def get_option(self, opt):
        v = C.c_int(0)
        self._check(self.lib.fk_engine_get_option(self.h, opt, C.byref(v)), "get_option")
        return v.value

    def synchronize(self):
        self._check(self.lib.fk_engine_synchronize(self.h), "synchronize")

    def set_profiling(self, on):
        self._check(self.lib.fk_engine_set_profiling(self.h, int(on)), "set_profiling")

    def profile(self, kind):
        n = C.c_longlong(0)
        ms = C.c_double(0)
        self._check(self.lib.fk_engine_profile_read(self.h, kind, C.byref(n), C.byref(ms)), "profile_read")
        return n.value, ms.value

    def profile_reset(self):
        self._check(self.lib.fk_engine_profile_reset(self.h), "profile_reset")

    def timer_start(self):
        self._check(self.lib.fk_engine_timer_start(self.h), "timer_start")

    def timer_stop(self):
        ms = C.c_double(0)
        self._check(self.lib.fk_engine_timer_stop(self.h, C.byref(ms)), "timer_stop")
        return ms.value

    def memory(self):
        b = C.c_size_t(0)
        self._check(self.lib.fk_engine_memory(self.h, C.byref(b)), "memory")
        return b.value

    # -- Engine<T> --
    def energy_scale(self, H, extend, iters=128, v0=None):
        lo, hi = C.c_double(0), C.c_double(0)
        v = None if v0 is None else _as_doubles(v0)
        self._check(self.lib.fk_engine_energy_scale(self.h, H.n_rows, H.b_len, H.n_blocks(), _ip(H.row_ptr),
                                                    _ip(H.col_idx), _dp(_as_doubles(H.val)), float(extend), int(iters),
                                                    None if v is None else _dp(v), C.byref(lo), C.byref(hi)),
                    "energy_scale")
        return EnergyScale(lo.value, hi.value)

    def set_H(self, H, es):
        self.es = es
        self._H = H
        self._check(self.lib.fk_engine_set_H(self.h, H.n_rows, H.b_len, H.n_blocks(), _ip(H.row_ptr), _ip(H.col_idx),
                                             _dp(_as_doubles(H.val)), es.lo, es.hi), "set_H")

    def transfer_R(self):
        R = np.asarray(self.R)
        n, s = R.shape
        flat = _as_doubles(R.reshape(-1, order="F")) if not np.iscomplexobj(R) else \
            np.ascontiguousarray(R.reshape(-1, order="F"), dtype=np.complex128).view(np.float64)
        self._check(self.lib.fk_engine_set_R(self.h, n, s, _dp(flat)), "transfer_R")
        self._r_shape = (n, s)

    def set_R_sparse(self, n, s, cols, vals):
        """Upload the probe block from its nonzeros, k per row: R[i, cols[i, q]] += vals[i, q]
        (cols, vals of shape (n, k)); every other entry is zero. The public R is not kept."""
        dt = np.complex128 if self.complex_values else np.float64
        cols = np.ascontiguousarray(cols, dtype=np.int32).reshape(n, -1)
        vals = np.ascontiguousarray(vals, dtype=dt).reshape(cols.shape)
        self._check(self.lib.fk_engine_set_R_sparse(self.h, n, s, cols.shape[1], _ip(cols),
                                                    _dp(vals.view(np.float64))), "set_R_sparse")
        self.R = self.R2 = None
        self._r_shape = (n, s)

    def get_R(self):
        n, s = self._r_shape
        dt = np.complex128 if self.complex_values else np.float64
        flat = np.zeros(n * s, dt)
        self._check(self.lib.fk_engine_get_R(self.h, _dp(flat.view(np.float64))), "get_R")
        return flat.reshape((n, s), order="F")

    def set_R(self, R):
        """Write the public R (column-major n x s) and transfer it."""
        dt = np.complex128 if self.complex_values else np.float64
        self.R = np.asfortranarray(R, dtype=dt)
        self.R2 = self.R
        self.transfer_R()

    def set_R_identity(self, n, j_start=0, j_end=None):
        self.set_R(probe_identity(n, j_start, j_end, self.complex_values))

    def set_R_uncorrelated(self, n, s, rng, j_start=0, j_end=None):
        self.set_R(probe_uncorrelated(n, s, rng, j_start, j_end, self.complex_values))

    def set_R_correlated(self, groups, rng, j_start=0, j_end=None):
        self.set_R(probe_correlated(groups, rng, j_start, j_end, self.complex_values))

    def moments(self, M):
        mu = np.zeros(M)
        self._check(self.lib.fk_engine_moments(self.h, M, _dp(mu)), "moments")
        return mu

    def moments_async(self, M):
        self._check(self.lib.fk_engine_moments_async(self.h, M), "moments_async")

    def fetch_moments(self, M):
        mu = np.zeros(M)
        self._check(self.lib.fk_engine_fetch_moments(self.h, _dp(mu)), "fetch_moments")
        return mu

    def _D_call(self, fn, c, D, where):
        c = np.ascontiguousarray(c, dtype=np.float64)
        dt = np.complex128 if self.complex_values else np.float64
        out = np.zeros(D.n_blocks() * D.b_len ** 2, dt)
        self._check(fn(self.h, len(c), _dp(c), D.n_rows, D.n_blocks(), _ip(D.row_ptr), _ip(D.col_idx),
                       _dp(out.view(np.float64))), where)
        D.val = out

    def stoch_matrix(self, c, D):
        self._D_call(self.lib.fk_engine_stoch_matrix, c, D, "stoch_matrix")

    def autodiff_matrix(self, c, D):
        self._D_call(self.lib.fk_engine_autodiff_matrix, c, D, "autodiff_matrix")

    def stoch_matrix_async(self, c, D):
        c = np.ascontiguousarray(c, dtype=np.float64)
        self._check(self.lib.fk_engine_stoch_matrix_async(self.h, len(c), _dp(c), D.n_rows, D.n_blocks(),
                                                          _ip(D.row_ptr), _ip(D.col_idx)), "stoch_matrix_async")

    def autodiff_matrix_async(self, c, D):
        c = np.ascontiguousarray(c, dtype=np.float64)
        self._check(self.lib.fk_engine_autodiff_matrix_async(self.h, len(c), _dp(c), D.n_rows, D.n_blocks(),
                                                             _ip(D.row_ptr), _ip(D.col_idx)), "autodiff_matrix_async")

    def fetch_D(self, D):
        dt = np.complex128 if self.complex_values else np.float64
        out = np.zeros(D.n_blocks() * D.b_len ** 2, dt)
        self._check(self.lib.fk_engine_fetch_D(self.h, _dp(out.view(np.float64))), "fetch_D")
        D.val = out

    def expansion_coefficients(self, M, Mq, f, kT, mu, es):
        """Jackson-damped Fermi expansion computed in FP64 on this engine's device."""
        kind = {"fermi_density": 0, "fermi_energy": 1}[f]
        out = np.zeros(M)
        self._check(self.lib.fk_engine_expansion_coefficients(self.h, M, Mq, kind, kT, mu, es.lo, es.hi, _dp(out)),
                    "expansion_coefficients")
        return out

    def kpm_filling(self, Mq, kT, filling, delta_filling=0.0):
        """Post-process the last moments(M) on the device: returns (mu_F, energy, n_tot, gamma) with
        gamma = moment_transform(mu, Mq), mu_F = filling_to_mu(gamma, es, kT, filling, delta_filling),
        energy = electronic_energy(gamma, es, kT, filling, mu_F) (src/fastkpm.cpp:236-476)."""
        res = np.zeros(3)
        gamma = np.zeros(Mq)
        self._check(self.lib.fk_engine_kpm_filling(self.h, Mq, kT, filling, delta_filling, _dp(res), _dp(gamma)),
                    "kpm_filling")
        return res[0], res[1], res[2], gamma

    def solve_filling(self, M, Mq, kT, filling, D, delta_filling=0.0):
        """moments(M) -> mu_F, energy at the filling -> fermi_energy coefficients at mu_F ->
        autodiff_matrix(c, D), every stage on the device. Fills D.val; returns (mu_F, energy, gamma)."""
        res = np.zeros(3)
        gamma = np.zeros(Mq)
        dt = np.complex128 if self.complex_values else np.float64
        out = np.zeros(D.n_blocks() * D.b_len ** 2, dt)
        self._check(self.lib.fk_engine_solve_filling(self.h, M, Mq, kT, filling, delta_filling, D.n_rows, D.n_blocks(),
                                                     _ip(D.row_ptr), _ip(D.col_idx), _dp(out.view(np.float64)),
                                                     _dp(res), _dp(gamma)), "solve_filling")
        D.val = out
        return res[0], res[1], gamma

    def moments2_v1(self, M, j1, j2, a_chunk_ncols=0, R_chunk_ncols=0):
        """Second-order moments mu[m1, m2] = sum_k <T_m1 r_k, j2 T_m2 j1 r_k> ((M, M) complex;
        src/engine_cusparse.cpp:793-902). j1, j2: SpMatBsr with H's block rows, unscaled."""
        dt = np.complex128 if self.complex_values else np.float64
        v1 = np.ascontiguousarray(j1.val, dtype=dt)
        v2 = np.ascontiguousarray(j2.val, dtype=dt)
        out = np.zeros(2 * M * M)
        self._check(self.lib.fk_engine_moments2_v1(self.h, M, j1.n_blocks(), _ip(j1.row_ptr), _ip(j1.col_idx),
                                                   _dp(v1.view(np.float64)), j2.n_blocks(), _ip(j2.row_ptr),
                                                   _ip(j2.col_idx), _dp(v2.view(np.float64)), a_chunk_ncols,
                                                   R_chunk_ncols, _dp(out)), "moments2_v1")
        return out.view(np.complex128).reshape(M, M)

    def moments2_v2(self, M, j1, j2, a_chunk_ncols=0, R_chunk_ncols=0):
        """mu[m1, m2] = tr(A_m1 B_m2), A_i = R^dag T_i j2 R2, B_i = R2^dag T_i j1 R ((M, M) complex;
        src/engine_cpu.cpp:162-209). R2 is the public attribute (R itself unless replaced); the
        chunk arguments are accepted for the reference's signature and unused, as there."""
        dt = np.complex128 if self.complex_values else np.float64
        v1 = np.ascontiguousarray(j1.val, dtype=dt)
        v2 = np.ascontiguousarray(j2.val, dtype=dt)
        r2p = None
        if self.R2 is not None and self.R2 is not self.R:
            r2 = np.asarray(self.R2, dtype=dt)
            if r2.shape != self.R.shape:
                raise ValueError("R2 must have R's shape")
            r2f = np.ascontiguousarray(r2.reshape(-1, order="F"))
            r2p = _dp(r2f.view(np.float64))
        out = np.zeros(2 * M * M)
        self._check(self.lib.fk_engine_moments2_v2(self.h, M, j1.n_blocks(), _ip(j1.row_ptr), _ip(j1.col_idx),
                                                   _dp(v1.view(np.float64)), j2.n_blocks(), _ip(j2.row_ptr),
                                                   _ip(j2.col_idx), _dp(v2.view(np.float64)), r2p, _dp(out)),
                    "moments2_v2")
        return out.view(np.complex128).reshape(M, M)


class Batch:
    """Many Hamiltonians of uneven size and probe count (same block size b) solved together: one
    launch per Chebyshev step covers every system; moments for all systems at once."""

    def __init__(self, complex_values=False, precision="fp32", device=0):
        self.lib = L.load()
        self.complex_values = bool(complex_values)
        h = C.c_void_p()
        st = self.lib.fk_batch_create(device, L.FK_COMPLEX if complex_values else L.FK_REAL,
                                      L.PRECISIONS[precision], C.byref(h))
        if st != L.FK_OK:
            raise L.FkError(st, "batch_create")
        self.h = h
        self.n = 0
        self.patterns = []   # per system: its H pattern as added (values left empty)

    def _check(self, st, where):
        if st != L.FK_OK:
            raise L.FkError(st, where, self.lib.fk_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fk_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, H, es, R):
        dt = np.complex128 if self.complex_values else np.float64
        R = np.asarray(R, dtype=dt)
        n, s = R.shape
        if n != H.n_rows * H.b_len:
            raise ValueError("R has %d rows; H has %d scalar rows" % (n, H.n_rows * H.b_len))
        flat = np.ascontiguousarray(R.reshape(-1, order="F"))
        idx = C.c_int(0)
        self._check(self.lib.fk_batch_add(self.h, H.n_rows, H.b_len, H.n_blocks(), _ip(H.row_ptr), _ip(H.col_idx),
                                          _dp(_as_doubles(H.val)), es.lo, es.hi, s, _dp(_as_doubles(flat)),
                                          C.byref(idx)), "batch_add")
        self.n += 1
        self.patterns.append(SpMatBsr(H.n_rows, H.b_len, H.row_ptr.copy(), H.col_idx.copy(), np.zeros(0)))
        return idx.value

    def commit(self):
        self._check(self.lib.fk_batch_commit(self.h), "batch_commit")

    def moments(self, M):
        mu = np.zeros(self.n * M)
        self._check(self.lib.fk_batch_moments(self.h, M, _dp(mu)), "batch_moments")
        return mu.reshape(self.n, M)

    def autodiff_matrix(self, M, c, out=None):
        """Engine.autodiff_matrix for every system after moments(M): c is (systems, M), one row of
        coefficients per system; returns one SpMatBsr per system on its own H pattern. `out` (optional):
        a contiguous array of all systems' block values, reused across calls (pinned with
        fk_host_register it is filled at copy-engine speed); the returned matrices are views of it."""
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(self.n, M)
        dt = np.complex128 if self.complex_values else np.float64
        total = sum(P.n_blocks() * P.b_len ** 2 for P in self.patterns)
        if out is None:
            out = np.zeros(total, dt)
        elif out.dtype != dt or out.size != total or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous %s array of %d values" % (np.dtype(dt).name, total))
        self._check(self.lib.fk_batch_autodiff_matrix(self.h, M, _dp(c), _dp(out.view(np.float64))),
                    "batch_autodiff_matrix")
        Ds, off = [], 0
        for P in self.patterns:
            k = P.n_blocks() * P.b_len ** 2
            Ds.append(P.with_values(out[off:off + k]))
            off += k
        return Ds

    def set_option(self, opt, value):
        self._check(self.lib.fk_batch_set_option(self.h, opt, int(value)), "batch_set_option")

    def get_option(self, opt):
        v = C.c_int(0)
        self._check(self.lib.fk_batch_get_option(self.h, opt, C.byref(v)), "batch_get_option")
        return v.value

    def autotune(self, trial_steps=8):
        g, npk, cap, st = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        ms = C.c_double()
        self._check(self.lib.fk_batch_autotune(self.h, trial_steps, C.byref(g), C.byref(npk), C.byref(cap),
                                               C.byref(st), C.byref(ms)), "batch_autotune")
        return dict(lanes_per_row=g.value, packets_per_lane=npk.value, ctas_per_sm=cap.value, stage_h=st.value,
                    ms_per_step=ms.value)

    def profile_moments(self, M):
        """moments(M) once with direct launches, each step launch timed by CUDA events on the batch's
        stream: (sum of the launch times in ms, number of launches)."""
        ms, n = C.c_double(0), C.c_int(0)
        self._check(self.lib.fk_batch_profile_moments(self.h, M, C.byref(ms), C.byref(n)), "batch_profile_moments")
        return ms.value, n.value

    def timer_start(self):
        self._check(self.lib.fk_batch_timer_start(self.h), "batch_timer_start")

    def timer_stop(self):
        ms = C.c_double(0)
        self._check(self.lib.fk_batch_timer_stop(self.h, C.byref(ms)), "batch_timer_stop")
        return ms.value

    def info(self):
        n, rows, b = C.c_int(), C.c_longlong(), C.c_size_t()
        self._check(self.lib.fk_batch_info(self.h, C.byref(n), C.byref(rows), C.byref(b)), "batch_info")
        return dict(n_systems=n.value, total_rows=rows.value, device_bytes=b.value)


def mk_engine(complex_values=False, precision="fp64", device=0):
    """mk_engine<T>() (reference src/engine.cpp:124-131): the GB300 engine, never a CPU fallback."""
    if device_count() == 0:
        raise RuntimeError("fastkpm_gb300: no CUDA device available")
    return Engine(complex_values, precision, device)
