"""Serving loop: continuous batching of mixed-size KPM solves.

Each request's moments and D are the same whether it runs alone or in the mix
(tolerance 1e-12 relative; the kernels' reductions depend only on the request
itself, so in practice they are bit-identical), and match the oracle within
the FP32 tolerance (moments 1e-5 relative to mu_0, D 1e-4 Frobenius). Small
requests with the same pack key share batched launches; a packable request's
result alone is its result as a pack of one. Requests that cannot fit the
memory budget are rejected, not hung."""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W
from fastkpm_gb300.serve import DEFAULT_CTA_WAVES, Request, Server
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def mixed_requests(seed=3):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(8):
        if k % 2 == 0:
            L_ = int(rng.choice([6, 10, 16]))
            H, es = W.square_lattice(L_, -1.0, 1.0, seed + k)
            R = fk.probe_uncorrelated(H.n_rows, int(rng.choice([8, 16, 32])), fk.RNG(seed + k))
        else:
            L_ = int(rng.choice([2, 4]))
            H, es, _ = W.cubic_spin_lattice(L_, -1.0, 1.0, seed + k)
            R = W.phase_probes(W.cubic_colour_groups(L_, 2), 1, seed + k)
        M = int(rng.choice([20, 40]))
        c = W.fermi_coefficients(M, es, "fermi_energy")
        reqs.append((H, es, R, M, c))
    return reqs


def solo(H, es, R, M, c, precision, packable=False):
    """The request alone: on its own engine, or, if packable, as a pack of one."""
    cplx = np.iscomplexobj(R)
    if packable:
        bt = fk.Batch(cplx, precision)
        bt.add(H, es, R)
        bt.commit()
        mu = bt.moments(M)[0]
        D = bt.autodiff_matrix(M, np.asarray(c)[None, :])[0].val.copy()
        bt.close()
        return mu, D
    eng = fk.Engine(cplx, precision)
    eng.set_option(L.FK_OPT_CTA_WAVES, DEFAULT_CTA_WAVES)   # as the server's slot engines
    eng.set_H(H, es)
    eng.set_R(R)
    mu = eng.moments(M)
    D = H.pattern_like(cplx)
    eng.autodiff_matrix(c, D)
    eng.close()
    return mu, D.val


def test_results_same_alone_and_in_the_mix(gpu):
    reqs = mixed_requests()
    srv = Server(max_slots=4, memory_budget=8 << 30)
    tickets = [srv.submit(Request(H, es, R, M, c, "autodiff", "fp32")) for (H, es, R, M, c) in reqs]
    for t in tickets:
        srv.wait(t, timeout=300)
    st = srv.stats()
    srv.stop()
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["max_concurrent"] >= 2
    assert st["p99_s"] >= st["p50_s"] > 0
    for (H, es, R, M, c), t in zip(reqs, tickets):
        mu, D = solo(H, es, R, M, c, "fp32", t.pack_size > 1)
        assert np.max(np.abs(t.mu - mu)) / abs(mu[0]) <= 1e-12
        assert np.linalg.norm(t.D - D) <= 1e-12 * np.linalg.norm(D)
        o = O.OracleEngine(np.iscomplexobj(R), nthreads=2)
        o.set_H(H, es)
        o.set_R(R)
        mu_ref = o.moments(M)
        D_ref = o.autodiff_matrix(c, H.pattern_like(np.iscomplexobj(R)))
        assert np.max(np.abs(t.mu - mu_ref)) / abs(mu_ref[0]) <= 1e-5
        assert np.linalg.norm(t.D - D_ref) / np.linalg.norm(D_ref) <= 1e-4


def test_admission_by_memory(gpu):
    reqs = mixed_requests(9)
    small = Request(*reqs[0][:3], reqs[0][3], reqs[0][4], "autodiff", "fp32")
    budget = int(small.footprint() * 1.5)
    H, es = W.square_lattice(64, -1.0, 1.0, 1)
    big = Request(H, es, fk.probe_uncorrelated(H.n_rows, 64, fk.RNG(1)), 20,
                  W.fermi_coefficients(20, es, "fermi_energy"), "autodiff", "fp32")
    assert big.footprint() > budget
    srv = Server(max_slots=2, memory_budget=budget)
    t_big = srv.submit(big)
    t_small = srv.submit(small)
    with pytest.raises(L.FkError) as ei:
        srv.wait(t_big, timeout=60)
    assert ei.value.status == L.FK_ERR_OOM
    srv.wait(t_small, timeout=120)
    srv.stop()
    assert t_small.mu is not None and srv.stats()["rejected"] == 1


def test_small_requests_share_batched_launches(gpu):
    # six requests with one pack key and two with another, submitted together to a one-slot server:
    # while the first runs, the others queue and are solved as packs (one launch per Chebyshev step for
    # all requests of a pack); every result equals the same path's result alone (bit for bit), its own
    # engine's result and the oracle within the FP32 tolerances
    reqs = []
    for k in range(6):
        H, es = W.square_lattice(int([8, 12, 16][k % 3]), -1.0, 1.0, 40 + k)
        reqs.append((H, es, fk.probe_uncorrelated(H.n_rows, 16, fk.RNG(40 + k)), 30))
    for k in range(2):
        H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, 50 + k)
        reqs.append((H, es, W.phase_probes(W.cubic_colour_groups(4, 2), 1, 50 + k), 20))
    srv = Server(max_slots=1, memory_budget=8 << 30)
    tickets = []
    for H, es, R, M in reqs:
        c = W.fermi_coefficients(M, es, "fermi_energy")
        tickets.append(srv.submit(Request(H, es, R, M, c, "autodiff", "fp32")))
    for t in tickets:
        srv.wait(t, timeout=300)
    st = srv.stats()
    srv.stop()
    assert st["completed"] == len(reqs) and st["packs"] >= 1 and st["packed_requests"] >= 2
    for (H, es, R, M), t in zip(reqs, tickets):
        mu, D = solo(H, es, R, M, t.c, "fp32", t.pack_size > 1)   # the same path alone: bit-identical
        assert np.array_equal(t.mu, mu) and np.array_equal(t.D, D)
        mu_e, D_e = solo(H, es, R, M, t.c, "fp32")                # on its own engine: FP32 tolerance
        assert np.max(np.abs(t.mu - mu_e)) / abs(mu_e[0]) <= 1e-5
        assert np.linalg.norm(t.D - D_e) / np.linalg.norm(D_e) <= 1e-4
        o = O.OracleEngine(np.iscomplexobj(R), nthreads=2)
        o.set_H(H, es)
        o.set_R(R)
        mu_ref = o.moments(M)
        D_ref = o.autodiff_matrix(t.c, H.pattern_like(np.iscomplexobj(R)))
        assert np.max(np.abs(t.mu - mu_ref)) / abs(mu_ref[0]) <= 1e-5
        assert np.linalg.norm(t.D - D_ref) / np.linalg.norm(D_ref) <= 1e-4
