"""The benchmark Hamiltonian generators on the CPU: Hermiticity, neighbour structure, the
analytic energy bounds against dense eigenvalues, the colourings behind the probe blocks,
and the oracle on a small triangular spin lattice (the triangular L=512 precision
workload's generator at L=6) against exact traces and dense matrix functions.
Tolerances: exact traces and matrix functions to 1e-10 (relative to mu_0 / the norm).
"""
import numpy as np
import pytest

from fastkpm_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import cheb_T, rel_err


def dense_scaled(H, es):
    A = H.to_dense()
    return (A - es.avg() * np.eye(A.shape[0])) / es.mag()


@pytest.mark.parametrize("L_", [4, 6, 9])
def test_triangular_spin_lattice_structure_and_bound(L_):
    H, es, S = W.triangular_spin_lattice(L_, -1.0, 2.0, seed=L_)
    A = H.to_dense()
    assert np.allclose(A, A.conj().T)
    assert np.all(np.diff(H.row_ptr) == 7)                 # 6 neighbours + the on-site block
    assert np.allclose(np.linalg.norm(S, axis=1), 1.0)    # unit spins
    lam = np.linalg.eigvalsh(A)
    assert es.lo <= lam[0] and lam[-1] <= es.hi            # the 6|t| + |J| bound brackets the spectrum
    assert es.hi == pytest.approx(1.01 * (6 + 2))
    # the on-site block is J sigma.S: eigenvalues +-J
    k = H.find_index(0, 0)
    blk = H.val[4 * k:4 * k + 4].reshape(2, 2, order="F")
    assert np.allclose(np.linalg.eigvalsh(blk), [-2.0, 2.0])


@pytest.mark.parametrize("L_", [4, 6])
def test_cubic_spin_lattice_bound_brackets_spectrum(L_):
    H, es, _ = W.cubic_spin_lattice(L_, -1.0, 1.0, seed=L_)
    lam = np.linalg.eigvalsh(H.to_dense())
    assert es.lo <= lam[0] and lam[-1] <= es.hi
    assert np.all(np.diff(H.row_ptr) == 7)


def test_square_lattice_bound_brackets_spectrum():
    H, es = W.square_lattice(12, -1.0, 3.0, seed=2)
    lam = np.linalg.eigvalsh(H.to_dense())
    assert es.lo <= lam[0] and lam[-1] <= es.hi


def test_colourings_separate_neighbours():
    # a colour class never holds two neighbouring sites, so every correlated probe column is a
    # set of non-neighbouring sites (the gradient-based probing the configurations describe)
    for L_, (H, _, _), groups in [(16, W.triangular_spin_lattice(16, -1.0, 2.0, 1), W.square_colour_groups(16, 8, 8, True)),
                                  (8, W.cubic_spin_lattice(8, -1.0, 1.0, 1), W.cubic_colour_groups(8, 4))]:
        site_colour = groups[0::2] // 2
        assert np.array_equal(groups[1::2], groups[0::2] + 1)
        for i in range(H.n_rows):
            for k in range(H.row_ptr[i], H.row_ptr[i + 1]):
                j = H.col_idx[k]
                if j != i:
                    assert site_colour[i] != site_colour[j]
    assert len(np.unique(W.square_colour_groups(512, 8, 8, True))) == 128
    assert len(np.unique(W.cubic_colour_groups(64, 4))) == 128


def test_oracle_on_small_triangular_lattice_exact_traces_and_matrix_function():
    H, es, _ = W.triangular_spin_lattice(6, -1.0, 2.0, seed=3)
    n = H.n_rows * 2
    A = dense_scaled(H, es)
    lam, U = np.linalg.eigh(A)
    orc = O.OracleEngine(True, nthreads=2)
    orc.set_H(H, es)
    orc.set_R(O.R_identity(n, complex_values=True))
    M = 32
    mu = orc.moments(M)
    ref = np.array([cheb_T(m, lam).sum() for m in range(M)])
    assert np.max(np.abs(mu - ref)) / n < 1e-10
    # stoch_matrix with identity probes is sum_m c_m T_m(Hs) on H's pattern
    c = W.fermi_coefficients(M, es, "fermi_density", 0.0, 0.5)
    D = H.pattern_like(True)
    got = orc.stoch_matrix(c, D)
    F = (U * np.array([sum(c[m] * cheb_T(m, x) for m in range(M)) for x in lam])) @ U.conj().T
    want = np.concatenate([F[2 * i:2 * i + 2, 2 * j:2 * j + 2].reshape(-1, order="F")
                           for i, j in zip(D.row_idx, D.col_idx)])
    assert rel_err(got, want) < 1e-10


def test_phase_probe_entries_equal_dense_probes():
    groups = W.square_colour_groups(16, 8, 8, spin=True)
    R = W.phase_probes(groups, 2, seed=4)
    s, cols, vals = W.phase_probe_entries(groups, 2, seed=4)
    assert s == R.shape[1]
    Rd = np.zeros_like(R)
    for q in range(cols.shape[1]):
        Rd[np.arange(len(groups)), cols[:, q]] += vals[:, q]
    assert np.array_equal(Rd, R)
    assert np.allclose(np.abs(R[R != 0]), 1 / np.sqrt(2))
