"""Host logic of the product (no GPU): probe generation, BSR build / symmetrize,
KPM coefficients, all compared with the oracle. Probes must be bit-identical."""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import workloads as W
from oracle import oracle as O


@pytest.fixture(autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("cplx", [False, True])
def test_probe_uncorrelated_bit_identical(cplx):
    for n, s, seed in [(1024, 64, 1), (37, 5, 123), (200, 1, 7)]:
        rng = fk.RNG(seed)
        R = fk.probe_uncorrelated(n, s, rng, complex_values=cplx)
        assert rng.drawn == s
        assert np.array_equal(R, O.R_uncorrelated(n, s, seed, complex_values=cplx))


def test_probe_uncorrelated_column_split_matches_threaded_semantics():
    n, s = 64, 16
    full = fk.probe_uncorrelated(n, s, fk.RNG(99))
    rng = fk.RNG(99)
    a = fk.probe_uncorrelated(n, s, rng, 0, 6)
    b = fk.probe_uncorrelated(n, s, rng, 6, 16)
    assert np.array_equal(np.hstack([a, b]), full)


@pytest.mark.parametrize("cplx", [False, True])
def test_probe_correlated_bit_identical(cplx):
    groups = W.cubic_colour_groups(4, 2)
    rng = fk.RNG(5)
    R = fk.probe_correlated(groups, rng, complex_values=cplx)
    assert np.array_equal(R, O.R_correlated(groups, 5, complex_values=cplx))
    assert rng.drawn == groups.max() + 1


def test_probe_correlated_identity_fallback():
    groups = np.arange(10)
    R = fk.probe_correlated(groups, fk.RNG(1))
    assert np.array_equal(R, np.eye(10))


def test_probe_identity_range():
    R = fk.probe_identity(8, 2, 5)
    assert np.array_equal(R, O.R_identity(8, 2, 5))


@pytest.mark.parametrize("cplx", [False, True])
def test_bsr_build_matches_oracle(cplx):
    rng = np.random.default_rng(3)
    n, b, ne = 40, 2, 500
    ri = rng.integers(0, n, ne)
    ci = rng.integers(0, n, ne)
    blocks = rng.standard_normal((ne, b * b))
    if cplx:
        blocks = blocks + 1j * rng.standard_normal((ne, b * b))
    H = fk.SpMatBsr.build(n, b, ri, ci, blocks)
    rp, r, c, v = O.bsr_build(n, b, ri, ci, blocks, cplx)
    assert np.array_equal(H.row_ptr, rp) and np.array_equal(H.col_idx, c)
    assert np.allclose(H.val, v, rtol=0, atol=1e-13)


def test_workload_bsr_equals_build():
    H, _ = W.square_lattice(5, -1.0, 1.0, seed=1)
    n = H.n_rows
    H2 = fk.SpMatBsr.build(n, 1, H.row_idx, H.col_idx, H.val[:, None])
    assert np.array_equal(H.row_ptr, H2.row_ptr) and np.array_equal(H.col_idx, H2.col_idx)
    assert np.array_equal(H.val, H2.val)
    # L = 2: periodic neighbours coincide and must be summed
    H3, _ = W.square_lattice(2, -1.0, 0.0, seed=0)
    assert np.allclose(H3.to_dense(), np.array([[0, -2, -2, 0], [-2, 0, 0, -2], [-2, 0, 0, -2], [0, -2, -2, 0]]))


def test_symmetrize_matches_oracle():
    H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, seed=2)
    D = H.copy()
    rng = np.random.default_rng(0)
    D.val = rng.standard_normal(D.val.shape) + 1j * rng.standard_normal(D.val.shape)
    ref = D.val.copy()
    O.lib().orc_bsr_symmetrize(1, D.n_rows, 2, D.n_blocks(), O._ip_(D.row_ptr), O._ip_(D.row_idx),
                               O._ip_(D.col_idx), O._dp_(ref.view(np.float64)))
    D.symmetrize()
    assert np.allclose(D.val, ref, atol=1e-15)
    A = D.to_dense()
    assert np.allclose(A, A.conj().T)


def test_coefficients_match_oracle():
    es = fk.EnergyScale(-7.07, 7.07)
    for kind in ["fermi_density", "fermi_energy"]:
        for kT, mu in [(0.0, 0.0), (0.1, 0.3)]:
            c = fk.expansion_coefficients(200, 400, kind, kT, mu, es)
            ref = O.expansion_coefficients(200, 400, kind, kT, mu, es.lo, es.hi)
            assert np.max(np.abs(c - ref)) < 1e-14
    assert np.max(np.abs(fk.jackson_kernel(100) - O.jackson_kernel(100))) < 1e-15


def test_spmat_rejects_bad_pattern():
    with pytest.raises(fk._lib.FkError):
        fk.SpMatBsr.build(4, 1, [0, 5], [0, 1], np.ones((2, 1)))
