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
