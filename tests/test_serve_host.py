"""Host-side bookkeeping of the serving loop (no GPU): busy time as the union of the
solves' service intervals, and each request's algorithmic byte count."""
import numpy as np

import fastkpm_gb300 as fk
from fastkpm_gb300 import workloads as W
from fastkpm_gb300.serve import Request, Server


def _req(L_, M, S, admitted, finished, kind="autodiff"):
    H, es = W.square_lattice(L_, -1.0, 1.0, seed=L_)
    R = np.ones((H.n_rows, S))
    r = Request(H, es, R, M, np.zeros(M), kind, "fp32", arrival=admitted - 0.5)
    r.admitted, r.finished = admitted, finished
    return r


def test_busy_time_is_union_of_service_intervals():
    srv = Server(max_slots=2, memory_budget=1 << 30)
    try:
        srv.completed = [_req(4, 10, 8, 0.0, 2.0), _req(4, 10, 8, 1.0, 3.0), _req(4, 10, 8, 5.0, 6.0),
                         _req(4, 10, 8, 5.5, 5.8)]
        st = srv.stats()
        assert abs(st["busy_s"] - 4.0) < 1e-12
        assert abs(st["algorithmic_bytes"] - sum(r.algorithmic_bytes() for r in srv.completed)) < 1e-6
    finally:
        srv.stop()


def test_algorithmic_bytes_formula():
    H, es = W.square_lattice(6, -1.0, 1.0, seed=1)
    n, S, M = H.n_rows, 16, 20
    r = Request(H, es, np.ones((n, S)), M, np.zeros(M), "autodiff", "fp32")
    h = H.n_blocks() * (4 + 4) + 4 * (H.n_rows + 1)
    fwd = (M // 2) * (3 * n * S * 4 + h)
    rev = (M // 2 - 1) * (6 * n * S * 4 + h + 2 * H.n_blocks() * 8)
    assert r.algorithmic_bytes() == fwd + rev
    r2 = Request(H, es, np.ones((n, S)), M, np.zeros(M), "stoch", "fp32")
    assert r2.algorithmic_bytes() == fwd


def test_phase_probe_entries_expand_to_phase_probes():
    groups = W.cubic_colour_groups(4, 2)
    for cplx in (True, False):
        for real in (1, 2):
            R = W.phase_probes(groups, realisations=real, seed=5, complex_values=cplx)
            s, cols, vals = W.phase_probe_entries(groups, realisations=real, seed=5, complex_values=cplx)
            D = np.zeros((len(groups), s), vals.dtype)
            for q in range(cols.shape[1]):
                np.add.at(D, (np.arange(len(groups)), cols[:, q]), vals[:, q])
            assert D.shape == R.shape and np.array_equal(D, R)


def test_request_with_probe_entries():
    H, es = W.square_lattice(5, -1.0, 1.0, seed=2)
    s, cols, vals = W.phase_probe_entries(np.arange(H.n_rows) % 4, 1, seed=3, complex_values=False)
    r = Request(H, es, None, 10, np.zeros(10), "autodiff", "fp32", R_entries=(s, cols, vals))
    assert (r.n_rows, r.s) == (H.n_rows, 4) and r.probe_steps() == H.n_rows * 10 * 4
    import pytest
    with pytest.raises(ValueError):
        Request(H, es, np.ones((H.n_rows, 4)), 10, np.zeros(10), R_entries=(s, cols, vals))


def test_pack_group_takes_same_key_requests_in_order():
    from fastkpm_gb300.serve import pack_group
    H8, es8 = W.square_lattice(8, -1.0, 1.0, seed=1)
    H6, es6 = W.square_lattice(6, -1.0, 1.0, seed=2)

    def req(H, es, S=8, M=10, kind="autodiff"):
        return Request(H, es, np.ones((H.n_rows, S)), M, np.zeros(M), kind, "fp32")
    a, b, c, d, e = req(H8, es8), req(H6, es6), req(H8, es8, S=512), req(H8, es8, M=12), req(H6, es6, kind="stoch")
    f, g, h = req(H6, es6), req(H8, es8), req(H6, es6, S=24)
    queue = [a, b, c, d, e, f, g, h]
    # same kind, b, M, precision and packets per lane: probe counts 8 and 24 (2 and 6 packets) share
    # packs, 512 (128 packets: four per lane) does not
    assert pack_group(a, queue, 1 << 30, 16) == [a, b, f, g, h]
    assert pack_group(a, queue, 1 << 30, 3) == [a, b, f]            # at most pack_max
    assert pack_group(e, queue, 1 << 30, 16) == [e]                 # stoch solves are not packed
    assert pack_group(a, queue, a.footprint() - 1, 16) == [a]       # above the footprint bound: alone
    assert a.pack_key(1 << 30) != c.pack_key(1 << 30) != d.pack_key(1 << 30)
    assert a.pack_key(1 << 30) == h.pack_key(1 << 30)


def test_batch_packets_per_lane_rule():
    from fastkpm_gb300.serve import batch_packets_per_lane as np_of
    # FP32 complex (8-byte elements, 2 per packet): S = 8..128 -> 4..64 packets -> two per lane
    assert {np_of(s, "fp32", True) for s in (8, 32, 64, 128)} == {2}
    assert np_of(256, "fp32", True) == 4 and np_of(2, "fp32", False) == 1
    assert np_of(256, "ds", True) == 4 and np_of(64, "fp64", False) == 2
