"""Batched engine: many uneven Hamiltonians per launch, CUDA-graph replay and the
autotuner, against the oracle per system (FP64: <= 1e-10, FP32: <= 1e-5 relative
to mu_0) and against single-system solves."""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu


def make_systems(n=6, S=32, seed=7, Ls=(5, 9, 16, 3, 12, 20)):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        L_ = Ls[k % len(Ls)]
        Wd = float(rng.uniform(0, 4))
        H, es = W.square_lattice(L_, -1.0, Wd, seed=seed * 100 + k)
        R = fk.probe_uncorrelated(H.n_rows, S, fk.RNG(seed * 100 + k))
        out.append((H, es, R))
    return out


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("ds", 1e-10), ("fp32", 1e-5)])
def test_batch_matches_oracle_per_system(gpu, prec, tol):
    systems = make_systems()
    M = 60
    bt = fk.Batch(False, prec)
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    mu = bt.moments(M)
    for k, (H, es, R) in enumerate(systems):
        o = O.OracleEngine(False, nthreads=2)
        o.set_H(H, es)
        o.set_R(R)
        ref = o.moments(M)
        assert np.max(np.abs(mu[k] - ref)) / ref[0] <= tol, k


def test_batch_graph_replay_and_alone_equal_mixed(gpu):
    systems = make_systems(5, 32, 11)
    M = 40
    bt = fk.Batch(False, "fp32")
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    a = bt.moments(M)
    bt.set_option(L.FK_OPT_GRAPHS, 1)
    b = bt.moments(M)
    c = bt.moments(M)
    assert np.array_equal(a, b) and np.array_equal(b, c)
    # each system alone in its own batch gives the same moments
    for k, (H, es, R) in enumerate(systems):
        one = fk.Batch(False, "fp32")
        one.add(H, es, R)
        one.commit()
        assert np.max(np.abs(one.moments(M)[0] - a[k])) / a[k][0] <= 1e-6


def test_batch_complex_spin_blocks(gpu):
    systems = []
    for k, L_ in enumerate([3, 4, 2]):
        H, es, _ = W.cubic_spin_lattice(L_, -1.0, 1.0, seed=k)
        R = W.phase_probes(np.arange(2 * H.n_rows) % 8, 1, seed=k)
        systems.append((H, es, R))
    M = 30
    bt = fk.Batch(True, "ds")
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    mu = bt.moments(M)
    for k, (H, es, R) in enumerate(systems):
        o = O.OracleEngine(True)
        o.set_H(H, es)
        o.set_R(R)
        ref = o.moments(M)
        assert np.max(np.abs(mu[k] - ref)) / ref[0] <= 1e-10


def test_autotune_keeps_results(gpu):
    systems = make_systems(4, 32, 3)
    M = 30
    bt = fk.Batch(False, "fp32")
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    before = bt.moments(M)
    best = bt.autotune(4)
    assert best["lanes_per_row"] in (1, 2, 4, 8, 16, 32) and best["packets_per_lane"] in (1, 2, 4)
    assert best["ms_per_step"] > 0
    after = bt.moments(M)
    assert np.max(np.abs(after - before) / before[:, :1]) <= 1e-5


def test_batch_rejects_mixed_shapes(gpu):
    # systems of one batch share the block size b (probe counts may differ)
    bt = fk.Batch(True, "fp32")
    H, es = W.square_lattice(4, -1.0, 1.0, 0)
    bt.add(H.with_values(H.val.astype(np.complex128)), es, fk.probe_uncorrelated(16, 8, fk.RNG(1), complex_values=True))
    Hs, ess, _ = W.cubic_spin_lattice(2, -1.0, 1.0, seed=1)
    with pytest.raises(L.FkError) as ei:
        bt.add(Hs, ess, fk.probe_uncorrelated(16, 8, fk.RNG(1), complex_values=True))
    assert ei.value.status == L.FK_ERR_ARG
    bt = fk.Batch(False, "fp32")
    bt.add(H, es, fk.probe_uncorrelated(16, 8, fk.RNG(1)))
    with pytest.raises(ValueError):
        bt.add(H, es, fk.probe_uncorrelated(15, 8, fk.RNG(1)))   # R rows must be b * n_b
    with pytest.raises(L.FkError) as ei:
        fk.Batch(False, "fp32").moments(10)
    assert ei.value.status == L.FK_ERR_STATE


def _spin_systems(Ls=(3, 4, 2, 5)):
    out = []
    for k, L_ in enumerate(Ls):
        H, es, _ = W.cubic_spin_lattice(L_, -1.0, 1.0, seed=40 + k)
        R = W.phase_probes(np.arange(2 * H.n_rows) % 8, 1, seed=40 + k)
        out.append((H, es, R))
    return out


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("ds", 1e-10), ("fp32", 1e-4)])
def test_batch_autodiff_matches_oracle_per_system(gpu, cplx, prec, tol):
    systems = _spin_systems() if cplx else make_systems(4, 16, 11, Ls=(6, 9, 4, 11))
    M = 24
    bt = fk.Batch(cplx, prec)
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    bt.moments(M)
    # a different Fermi level per system: the coefficient rows are the systems' own
    cs = np.stack([W.fermi_coefficients(M, es, "fermi_energy", mu=0.2 * k) for k, (_, es, _) in enumerate(systems)])
    Ds = bt.autodiff_matrix(M, cs)
    assert len(Ds) == len(systems)
    for k, (H, es, R) in enumerate(systems):
        o = O.OracleEngine(cplx)
        o.set_H(H, es)
        o.set_R(R)
        o.moments(M)
        ref = o.autodiff_matrix(cs[k], H.pattern_like(cplx))
        assert rel_err(Ds[k].val, ref) <= tol, k
    # the alpha state is consumed: a second call needs moments(M) again
    with pytest.raises(L.FkError) as ei:
        bt.autodiff_matrix(M, cs)
    assert ei.value.status == L.FK_ERR_STATE
    # a caller-provided output buffer: same values, returned matrices are views of it
    bt.moments(M)
    out = np.full(sum(D.val.size for D in Ds), np.nan, dtype=Ds[0].val.dtype)
    Ds2 = bt.autodiff_matrix(M, cs, out=out)
    assert all(np.array_equal(a.val, b_.val) for a, b_ in zip(Ds, Ds2))
    assert np.shares_memory(Ds2[-1].val, out)


def _without_diagonal(H):
    keep = H.col_idx != H.row_idx
    rp = np.concatenate([[0], np.cumsum(np.bincount(H.row_idx[keep], minlength=H.n_rows))]).astype(np.int32)
    bb = H.b_len * H.b_len
    val = H.val.reshape(-1, bb)[keep].reshape(-1)
    return fk.SpMatBsr(H.n_rows, H.b_len, rp, H.col_idx[keep], val)


def test_batch_autodiff_keeps_h_pattern_without_diagonal(gpu):
    H0, es0 = W.square_lattice(7, -1.0, 0.5, seed=3)
    H0 = _without_diagonal(H0)
    assert np.all(H0.col_idx != H0.row_idx)
    H1, es1 = W.square_lattice(5, -1.0, 2.0, seed=4)
    S, M = 8, 16
    R0 = fk.probe_uncorrelated(H0.n_rows, S, fk.RNG(5))
    R1 = fk.probe_uncorrelated(H1.n_rows, S, fk.RNG(6))
    bt = fk.Batch(False, "fp64")
    bt.add(H0, es0, R0)
    bt.add(H1, es1, R1)
    bt.commit()
    bt.moments(M)
    cs = np.stack([W.fermi_coefficients(M, es0, "fermi_energy"), W.fermi_coefficients(M, es1, "fermi_energy", mu=0.3)])
    Ds = bt.autodiff_matrix(M, cs)
    for k, (H, es, R) in enumerate([(H0, es0, R0), (H1, es1, R1)]):
        eng = fk.Engine(False, "fp64")
        eng.set_H(H, es)
        eng.set_R(R)
        eng.moments(M)
        D = H.pattern_like(False)
        eng.autodiff_matrix(cs[k], D)
        assert np.array_equal(Ds[k].col_idx, H.col_idx)
        assert np.max(np.abs(Ds[k].val - D.val)) <= 1e-12 * max(1.0, np.max(np.abs(D.val))), k


@pytest.mark.parametrize("acc64", [1, 0])
def test_batch_fp32_accumulator_forms(gpu, acc64):
    # FP64 (default) and float-float accumulators of the FP32 batch: moments and D against the oracle
    systems = make_systems(4, 32, 17)
    M = 40
    bt = fk.Batch(False, "fp32")
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    bt.set_option(L.FK_OPT_ACC64, acc64)
    assert bt.get_option(L.FK_OPT_ACC64) == acc64
    mu = bt.moments(M)
    cs = np.stack([W.fermi_coefficients(M, es, "fermi_energy") for _, es, _ in systems])
    Ds = bt.autodiff_matrix(M, cs)
    for k, (H, es, R) in enumerate(systems):
        o = O.OracleEngine(False, nthreads=2)
        o.set_H(H, es)
        o.set_R(R)
        ref = o.moments(M)
        assert np.max(np.abs(mu[k] - ref)) / ref[0] <= 1e-5, k
        D_ref = o.autodiff_matrix(cs[k], H.pattern_like(False))
        assert rel_err(Ds[k].val, D_ref) <= 1e-4, k


def test_batch_profile_moments(gpu):
    # the per-launch timing run gives the same moments as the plain and graph-replayed runs
    systems = make_systems(4, 32, 23)
    M = 30
    bt = fk.Batch(False, "fp32")
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    a = bt.moments(M)
    ms, n = bt.profile_moments(M)
    assert n == M // 2 and ms > 0
    bt.set_option(L.FK_OPT_GRAPHS, 1)
    b = bt.moments(M)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("prec,tol,dtol", [("fp64", 1e-10, 1e-10), ("ds", 1e-10, 1e-10), ("fp32", 1e-5, 1e-4)])
def test_batch_mixed_probe_counts(gpu, prec, tol, dtol):
    # Systems with different probe counts share one launch per step: the rows of all of them use the
    # widest system's stride and each system walks only its own packets (S = 8, 24, 32, 40, 64: whole
    # and ragged chunks). moments and autodiff_matrix per system against the oracle.
    Ss = [8, 24, 32, 40, 64]
    systems = []
    for k, S in enumerate(Ss):
        H, es = W.square_lattice([5, 9, 16, 3, 12][k], -1.0, 1.0 + k, seed=500 + k)
        systems.append((H, es, fk.probe_uncorrelated(H.n_rows, S, fk.RNG(500 + k))))
    M = 40
    bt = fk.Batch(False, prec)
    for H, es, R in systems:
        bt.add(H, es, R)
    bt.commit()
    mu = bt.moments(M)
    cs = np.stack([W.fermi_coefficients(M, es, "fermi_energy") for _, es, _ in systems])
    Ds = bt.autodiff_matrix(M, cs)
    for k, (H, es, R) in enumerate(systems):
        o = O.OracleEngine(False, nthreads=2)
        o.set_H(H, es)
        o.set_R(R)
        ref = o.moments(M)
        assert np.max(np.abs(mu[k] - ref)) / ref[0] <= tol, (k, Ss[k])
        D_ref = o.autodiff_matrix(cs[k], H.pattern_like(False))
        assert rel_err(Ds[k].val, D_ref) <= dtol, (k, Ss[k])
        # a system's lanes per row follow its own probe count, so alone in a batch it gives the same
        # bits (the packets per lane, two, are the same for every probe count here)
        one = fk.Batch(False, prec)
        one.add(H, es, R)
        one.commit()
        assert np.array_equal(one.moments(M)[0], mu[k]), (k, Ss[k])
        assert np.array_equal(one.autodiff_matrix(M, cs[k:k + 1])[0].val, Ds[k].val), (k, Ss[k])

