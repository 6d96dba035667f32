"""Pins of the oracle against analytic known answers (CPU only).

The reference ships no tests or golden vectors, so these known answers are what
pin the oracle: exact traces with identity probes, closed-form lattice moments,
dense eigendecomposition and finite differences of the moment sum.
"""
import numpy as np
import pytest

from oracle import oracle as O
from fastkpm_gb300 import workloads as W
from fastkpm_gb300.engine import EnergyScale, SpMatBsr
from tests.conftest import cheb_T


def dense_Hs(H, es):
    A = H.to_dense()
    A = (A - es.avg() * np.eye(A.shape[0])) / es.mag()
    return A


def test_identity_probes_give_exact_traces_real():
    H, _ = W.square_lattice(8, -1.0, 1.0, seed=3)
    es = EnergyScale(-4.5, 4.5)
    lam = np.linalg.eigvalsh(dense_Hs(H, es))
    e = O.OracleEngine(False, nthreads=2)
    e.set_H(H, es)
    e.set_R(O.R_identity(64))
    M = 40
    mu = e.moments(M)
    ref = np.array([cheb_T(m, lam).sum() for m in range(M)])
    assert np.max(np.abs(mu - ref)) / 64 < 1e-12


def test_identity_probes_give_exact_traces_complex_spin_blocks():
    H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, seed=5)
    A = dense_Hs(H, es)
    assert np.allclose(A, A.conj().T)
    lam = np.linalg.eigvalsh(A)
    n = A.shape[0]
    e = O.OracleEngine(True, nthreads=3)
    e.set_H(H, es)
    e.set_R(O.R_identity(n, complex_values=True))
    M = 30
    mu = e.moments(M)
    ref = np.array([cheb_T(m, lam).sum() for m in range(M)])
    assert np.max(np.abs(mu - ref)) / n < 1e-12


def test_clean_square_lattice_closed_form():
    L, t = 8, -1.0
    H, _ = W.square_lattice(L, t, 0.0, seed=0)
    es = EnergyScale(-4.5, 4.5)
    k = 2 * np.pi * np.arange(L) / L
    eps = (2 * t * (np.cos(k)[:, None] + np.cos(k)[None, :])).ravel() / 4.5
    e = O.OracleEngine(False, nthreads=1)
    e.set_H(H, es)
    e.set_R(O.R_identity(L * L))
    M = 50
    mu = e.moments(M)
    ref = np.array([cheb_T(m, eps).sum() for m in range(M)])
    assert np.max(np.abs(mu - ref)) / (L * L) < 1e-12


def test_stoch_matrix_identity_probes_is_matrix_function():
    H, _ = W.square_lattice(6, -1.0, 1.0, seed=7)
    es = EnergyScale(-4.5, 4.5)
    A = dense_Hs(H, es)
    lam, V = np.linalg.eigh(A)
    M = 60
    c = O.expansion_coefficients(M, 2 * M, "fermi_density", 0.0, 0.1, es.lo, es.hi)
    g = sum(c[m] * cheb_T(m, lam) for m in range(M))
    F = (V * g) @ V.T
    e = O.OracleEngine(False, nthreads=2)
    e.set_H(H, es)
    e.set_R(O.R_identity(36))
    D = e.stoch_matrix(c, H)
    ref = F[H.row_idx, H.col_idx]
    assert np.max(np.abs(D - ref)) < 1e-12


def _chebU(m, x):
    th = np.arccos(np.clip(x, -1, 1))
    return np.sin((m + 1) * th) / np.sin(th)


@pytest.mark.parametrize("cplx", [False, True])
def test_autodiff_is_gradient_of_moment_sum(cplx):
    if cplx:
        H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, seed=11)
    else:
        H, _ = W.square_lattice(6, -1.0, 2.0, seed=9)
        es = EnergyScale(-5.5, 5.5)
    A = dense_Hs(H, es)
    lam, V = np.linalg.eigh(A)
    n = A.shape[0]
    M = 24
    c = O.expansion_coefficients(M, 2 * M, "fermi_energy", 0.0, 0.2, es.lo, es.hi)
    gp = sum(c[m] * m * _chebU(m - 1, lam) for m in range(1, M))   # g'(x) = sum c_m m U_{m-1}(x)
    Dref_dense = (V * gp) @ V.conj().T / es.mag()
    e = O.OracleEngine(cplx, nthreads=2)
    e.set_H(H, es)
    e.set_R(O.R_identity(n, complex_values=cplx))
    e.moments(M)
    D = e.autodiff_matrix(c, H)
    b = H.b_len
    ref = np.array([Dref_dense[b * H.row_idx[k] + bi, b * H.col_idx[k] + bj]
                    for k in range(H.n_blocks()) for bj in range(b) for bi in range(b)])
    assert np.max(np.abs(D - ref)) < 1e-10


def test_autodiff_matches_central_finite_differences():
    H, _ = W.square_lattice(5, -1.0, 2.0, seed=13)
    es = EnergyScale(-5.5, 5.5)
    M = 16
    c = O.expansion_coefficients(M, 2 * M, "fermi_energy", 0.0, 0.0, es.lo, es.hi)
    n = 25

    def G(Hm):
        e = O.OracleEngine(False, nthreads=1)
        e.set_H(Hm, es)
        e.set_R(O.R_identity(n))
        return float(np.dot(c, e.moments(M)))

    e = O.OracleEngine(False, nthreads=1)
    e.set_H(H, es)
    e.set_R(O.R_identity(n))
    e.moments(M)
    D = e.autodiff_matrix(c, H)
    h = 1e-5
    for (i, j) in [(0, 0), (0, 1), (7, 8), (12, 12)]:
        k1 = H.find_index(i, j)
        k2 = H.find_index(j, i)
        Hp, Hm = H.copy(), H.copy()
        Hp.val[k1] += h
        Hm.val[k1] -= h
        if k2 != k1:
            Hp.val[k2] += h
            Hm.val[k2] -= h
        dG = (G(Hp) - G(Hm)) / (2 * h)
        pred = D[k1] if k1 == k2 else D[k1] + D[k2]
        assert abs(dG - pred) < 1e-7 * max(1.0, abs(dG))


def test_lanczos_energy_scale_brackets_spectrum():
    H, _ = W.square_lattice(8, -1.0, 1.0, seed=2)
    lam = np.linalg.eigvalsh(H.to_dense())
    e = O.OracleEngine(False, nthreads=1)
    v0 = np.random.default_rng(0).standard_normal(64)
    lo, hi = e.energy_scale(H, 0.0, 64, v0)
    assert abs(lo - lam.min()) < 1e-8 and abs(hi - lam.max()) < 1e-8
    lo2, hi2 = e.energy_scale(H, 0.1, 64, v0)
    span = hi - lo
    assert abs(lo2 - (lo - 0.1 * span)) < 1e-8 and abs(hi2 - (hi + 0.1 * span)) < 1e-8


def test_tridiag_bisection():
    rng = np.random.default_rng(1)
    a = rng.standard_normal(30)
    b = np.concatenate([[0.0], rng.standard_normal(29)])
    T = np.diag(a) + np.diag(b[1:], 1) + np.diag(b[1:], -1)
    lam = np.linalg.eigvalsh(T)
    lo, hi = O.tridiag_extremes(a, b)
    assert abs(lo - lam[0]) < 1e-12 and abs(hi - lam[-1]) < 1e-12


def test_jackson_and_expansion_coefficients_closed_form():
    M, Mq = 64, 256
    g = O.jackson_kernel(M)
    m = np.arange(M)
    Mp = M + 1.0
    ref = ((Mp - m) * np.cos(np.pi * m / Mp) + np.sin(np.pi * m / Mp) / np.tan(np.pi / Mp)) / Mp
    assert np.max(np.abs(g - ref)) < 1e-14
    lo, hi = -3.0, 5.0
    c = O.expansion_coefficients(M, Mq, "fermi_density", 0.0, 0.5, lo, hi)
    x = np.cos(np.pi * (np.arange(Mq) + 0.5) / Mq)
    f = ((x * 4.0 + 1.0) < 0.5).astype(float)
    ref_c = np.array([(1 if k == 0 else 2) * g[k] * np.sum(f * np.cos(k * np.arccos(x))) / Mq for k in range(M)])
    assert np.max(np.abs(c - ref_c)) < 1e-12
    # the damped series reproduces the step away from the edge
    xs = np.array([-0.8, -0.5, 0.6, 0.9])
    series = sum(c[k] * cheb_T(k, xs) for k in range(M))
    assert np.allclose(series, [1, 1, 0, 0], atol=0.02)


def test_probe_semantics():
    n, s = 50, 12
    R = O.R_uncorrelated(n, s, seed=42)
    assert R.shape == (n, s)
    assert np.allclose(np.abs(R), 1 / np.sqrt(s))
    # Engine_Threaded splits columns: a master advanced by j0 draws gives columns j0..j1
    part = O.R_uncorrelated(n, s, seed=42, discard=5, j_start=5, j_end=9)
    assert np.array_equal(part, R[:, 5:9])
    Rc = O.R_uncorrelated(n, s, seed=42, complex_values=True)
    assert np.allclose(np.abs(Rc), 1 / np.sqrt(s))
    assert set(np.round(Rc.ravel() * np.sqrt(s), 12)) <= {1, -1, 1j, -1j}
    groups = np.arange(n) % 7
    Rg = O.R_correlated(groups, seed=9)
    assert Rg.shape == (n, 7)
    for i in range(n):
        nz = np.nonzero(Rg[i])[0]
        assert list(nz) == [groups[i]] and abs(Rg[i, nz[0]]) == 1.0


def test_bsr_build_sorts_and_merges():
    rng = np.random.default_rng(0)
    n, b, ne = 20, 2, 200
    ri = rng.integers(0, n, ne)
    ci = rng.integers(0, n, ne)
    blocks = rng.standard_normal((ne, b * b))
    rp, r, c, v = O.bsr_build(n, b, ri, ci, blocks, False)
    dense = np.zeros((n * b, n * b))
    for k in range(ne):
        dense[b * ri[k]:b * ri[k] + b, b * ci[k]:b * ci[k] + b] += blocks[k].reshape(b, b, order="F")
    H = SpMatBsr(n, b, rp, c, v)
    assert np.allclose(H.to_dense(), dense)
    assert np.all(np.diff(r) >= 0)
    for i in range(n):
        assert np.all(np.diff(c[rp[i]:rp[i + 1]]) > 0)


def _exact_moments(lam, M):
    """mu_m = sum_k T_m(lam_k): the moments of identity probes on a matrix with spectrum lam."""
    return np.array([cheb_T(m, lam).sum() for m in range(M)])


def test_moment_transform_total_weight_is_mu0():
    # sum_i gamma_i / Mq = g_0 mu_0 = mu_0: the nodes' sum of T_m vanishes for 0 < m < 2 Mq
    rng = np.random.default_rng(0)
    lam = rng.uniform(-0.9, 0.9, 200)
    mu = _exact_moments(lam, 100)
    gamma = O.moment_transform(mu, 300)
    assert abs(gamma.sum() / 300 - 200) < 1e-10
    assert O.jackson_kernel(100)[0] == pytest.approx(1.0, abs=1e-15)


def test_filling_of_particle_hole_symmetric_spectrum():
    # a bipartite lattice has a symmetric spectrum: half filling puts mu at the band centre,
    # and the smeared filling of the returned mu is the requested one
    H, _ = W.square_lattice(16, -1.0, 0.0, seed=0)
    lam = np.linalg.eigvalsh(H.to_dense())
    es = EnergyScale(-4.5, 4.5)
    mu = _exact_moments(lam / es.mag(), 200)
    gamma = O.moment_transform(mu, 400)
    mu_f = O.filling_to_mu(gamma, es.lo, es.hi, 0.0, 0.5)
    assert abs(mu_f) < 1e-10
    kTs = 0.1 * es.mag() / 400
    for f in (0.2, 0.37, 0.8):
        m = O.filling_to_mu(gamma, es.lo, es.hi, 0.0, f)
        assert O.mu_to_filling(gamma, es.lo, es.hi, kTs, m) == pytest.approx(f, abs=1e-12)
    # delta_filling averages the roots at f +- delta
    a = O.filling_to_mu(gamma, es.lo, es.hi, 0.0, 0.3, 0.01)
    b = 0.5 * (O.filling_to_mu(gamma, es.lo, es.hi, 0.0, 0.31) + O.filling_to_mu(gamma, es.lo, es.hi, 0.0, 0.29))
    assert a == pytest.approx(b, abs=1e-13)


def test_electronic_energy_approaches_sum_of_occupied_levels():
    # at kT = 0 the KPM energy tends to the sum of the lowest filling*N eigenvalues as M grows
    rng = np.random.default_rng(1)
    H, _ = W.square_lattice(16, -1.0, 1.0, seed=2)
    lam = np.linalg.eigvalsh(H.to_dense())
    es = EnergyScale(-5.0, 5.0)
    exact = np.sort(lam)[:128].sum()
    errs = []
    for M in (100, 400):
        gamma = O.moment_transform(_exact_moments(lam / es.mag(), M), 2 * M)
        mu_f = O.filling_to_mu(gamma, es.lo, es.hi, 0.0, 0.5)
        errs.append(abs(O.electronic_energy(gamma, es.lo, es.hi, 0.0, 0.5, mu_f) - exact) / abs(exact))
    assert errs[1] < 5e-3 and errs[1] < errs[0]


def _dense_cheb(A, M):
    T = [np.eye(A.shape[0], dtype=A.dtype), A.copy()]
    for m in range(2, M):
        T.append(2 * A @ T[-1] - T[-2])
    return T[:M]


def test_moments2_v1_identity_probes_is_trace():
    # identity probes: mu[m1, m2] = tr(j1 T_m1(Hs) j2 T_m2(Hs)) exactly
    H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, seed=4)
    n = H.n_rows * H.b_len                      # scalar rows (n_rows counts block rows)
    A = dense_Hs(H, es)
    rng = np.random.default_rng(5)
    rows, cols = H.row_idx, H.col_idx

    def rand_op():
        return SpMatBsr.build(H.n_rows, 2, rows, cols,
                              rng.standard_normal((len(rows), 4)) + 1j * rng.standard_normal((len(rows), 4)))
    j1, j2 = rand_op(), rand_op()
    e = O.OracleEngine(True, nthreads=2)
    e.set_H(H, es)
    e.set_R(O.R_identity(n, complex_values=True))
    M = 8
    mu = e.moments2_v1(M, j1, j2)
    T = _dense_cheb(A, M)
    J1, J2 = j1.to_dense(), j2.to_dense()
    ref = np.array([[np.trace(J1 @ T[a] @ J2 @ T[b]) for b in range(M)] for a in range(M)])
    assert np.max(np.abs(mu - ref)) <= 1e-11 * np.max(np.abs(ref))


def test_moments2_v2_identity_probes_is_trace():
    # R = R2 = identity: A_i = T_i j2, B_i = T_i j1, tr(A_m1 B_m2) = tr(j1 T_m1 j2 T_m2)
    H, es, _ = W.cubic_spin_lattice(2, -1.0, 1.0, seed=7)
    n = H.n_rows * H.b_len
    A = dense_Hs(H, es)
    rng = np.random.default_rng(8)

    def rand_op():
        return SpMatBsr.build(H.n_rows, 2, H.row_idx, H.col_idx,
                              rng.standard_normal((len(H.row_idx), 4)) + 1j * rng.standard_normal((len(H.row_idx), 4)))
    j1, j2 = rand_op(), rand_op()
    e = O.OracleEngine(True, nthreads=2)
    e.set_H(H, es)
    e.set_R(O.R_identity(n, complex_values=True))
    M = 6
    T = _dense_cheb(A, M)
    J1, J2 = j1.to_dense(), j2.to_dense()
    ref = np.array([[np.trace(J1 @ T[a] @ J2 @ T[b]) for b in range(M)] for a in range(M)])
    assert np.max(np.abs(e.moments2_v2(M, j1, j2) - ref)) <= 1e-11 * np.max(np.abs(ref))
    # an explicit R2 equal to R gives the same
    assert np.max(np.abs(e.moments2_v2(M, j1, j2, O.R_identity(n, complex_values=True)) - ref)) <= 1e-11 * np.max(np.abs(ref))
