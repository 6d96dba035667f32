"""Batched engine: many uneven Hamiltonians per launch, CUDA-graph replay and the
autotuner, against the oracle per system (FP64: <= 1e-10, FP32: <= 1e-5 relative
to mu_0) and against single-system solves."""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W
from oracle import oracle as O

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
    bt = fk.Batch(False, "fp32")
    H, es = W.square_lattice(4, -1.0, 1.0, 0)
    bt.add(H, es, fk.probe_uncorrelated(16, 8, fk.RNG(1)))
    with pytest.raises(L.FkError) as ei:
        bt.add(H, es, fk.probe_uncorrelated(16, 4, fk.RNG(1)))
    assert ei.value.status == L.FK_ERR_ARG
    with pytest.raises(ValueError):
        bt.add(H, es, fk.probe_uncorrelated(15, 8, fk.RNG(1)))   # R rows must be b * n_b
    with pytest.raises(L.FkError) as ei:
        fk.Batch(False, "fp32").moments(10)
    assert ei.value.status == L.FK_ERR_STATE
