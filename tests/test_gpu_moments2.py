"""moments2_v1 (second-order moments for conductivity) on the GPU against the oracle's
restatement of the reference CPU engine (src/engine_cpu.cpp:86-160) and against exact traces.

Tolerances: max |mu - mu_ref| / max |mu_ref| <= 1e-10 for FP64 and DS engines, <= 1e-5 for FP32
(FP32 Chebyshev vectors; the reduction is FP64 in every precision)."""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "ds": 1e-10, "fp32": 1e-5}


def _ops(H, cplx, seed):
    rng = np.random.default_rng(seed)
    b = H.b_len
    nb = len(H.row_idx)

    def one():
        v = rng.standard_normal((nb, b * b))
        if cplx:
            v = v + 1j * rng.standard_normal((nb, b * b))
        return fk.SpMatBsr.build(H.n_rows, b, H.row_idx, H.col_idx, v)
    return one(), one()


def _case(cplx):
    if cplx:
        H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, 2)
        R = W.phase_probes(W.cubic_colour_groups(4, 2), realisations=1, seed=9)[:, :12]
    else:
        H, es = W.square_lattice(10, -1.0, 1.0, 3)
        R = fk.probe_uncorrelated(H.n_rows, 7, fk.RNG(2))
    return H, es, np.asfortranarray(R)


def _err(mu, ref):
    return float(np.max(np.abs(mu - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
@pytest.mark.parametrize("cplx", [False, True])
def test_moments2_v1_matches_oracle(gpu, prec, cplx):
    H, es, R = _case(cplx)
    j1, j2 = _ops(H, cplx, 7)
    M = 16
    eng = fk.Engine(cplx, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    mu = eng.moments2_v1(M, j1, j2)
    orc = O.OracleEngine(cplx)
    orc.set_H(H, es)
    orc.set_R(R)
    ref = orc.moments2_v1(M, j1, j2)
    assert _err(mu, ref) <= TOL[prec]
    eng.close()


def test_moments2_v1_chunking_does_not_change_results(gpu):
    H, es, R = _case(True)
    j1, j2 = _ops(H, True, 8)
    M = 12
    eng = fk.Engine(True, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    full = eng.moments2_v1(M, j1, j2)
    for a_chunk, r_chunk in [(3, 0), (5, 5), (12, 1), (4, 7)]:
        part = eng.moments2_v1(M, j1, j2, a_chunk, r_chunk)
        assert _err(part, full) <= 1e-13
    eng.close()


def test_moments2_v1_identity_probes_give_traces(gpu):
    H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, 6)
    n = H.n_rows * H.b_len
    j1, j2 = _ops(H, True, 9)
    A = (H.to_dense() - es.avg() * np.eye(n)) / es.mag()
    M = 10
    T = [np.eye(n, dtype=complex), A.astype(complex)]
    for m in range(2, M):
        T.append(2 * A @ T[-1] - T[-2])
    J1, J2 = j1.to_dense(), j2.to_dense()
    ref = np.array([[np.trace(J1 @ T[a] @ J2 @ T[b]) for b in range(M)] for a in range(M)])
    eng = fk.Engine(True, "fp64")
    eng.set_H(H, es)
    eng.set_R_identity(n)
    assert _err(eng.moments2_v1(M, j1, j2), ref) <= 1e-11
    eng.close()


def test_moments2_v1_consumes_the_autodiff_state(gpu):
    H, es, R = _case(False)
    j1, j2 = _ops(H, False, 1)
    eng = fk.Engine(False, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    M = 10
    eng.moments(M)
    eng.moments2_v1(M, j1, j2)
    c = W.fermi_coefficients(M, es, "fermi_energy")
    with pytest.raises(L.FkError) as ei:
        eng.autodiff_matrix(c, H.pattern_like())
    assert ei.value.status == L.FK_ERR_STATE
    with pytest.raises(L.FkError) as ei:
        eng.moments2_v1(7, j1, j2)
    assert ei.value.status == L.FK_ERR_ARG
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
@pytest.mark.parametrize("cplx", [False, True])
def test_moments2_v2_matches_oracle(gpu, prec, cplx):
    """moments2_v2 (the reference's CPU-only variant, src/engine_cpu.cpp:162-209) with R2 = R and
    with an independent R2, against the oracle."""
    H, es, R = _case(cplx)
    j1, j2 = _ops(H, cplx, 11)
    M = 12
    eng = fk.Engine(cplx, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    orc = O.OracleEngine(cplx)
    orc.set_H(H, es)
    orc.set_R(R)
    assert _err(eng.moments2_v2(M, j1, j2), orc.moments2_v2(M, j1, j2)) <= TOL[prec]
    R2 = fk.probe_uncorrelated(R.shape[0], R.shape[1], fk.RNG(5), complex_values=cplx)
    eng.R2 = R2
    assert _err(eng.moments2_v2(M, j1, j2), orc.moments2_v2(M, j1, j2, R2)) <= TOL[prec]
    eng.close()


def test_moments2_v2_identity_probes_give_traces(gpu):
    H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, 6)
    n = H.n_rows * H.b_len
    j1, j2 = _ops(H, True, 12)
    A = (H.to_dense() - es.avg() * np.eye(n)) / es.mag()
    M = 8
    T = [np.eye(n, dtype=complex), A.astype(complex)]
    for m in range(2, M):
        T.append(2 * A @ T[-1] - T[-2])
    J1, J2 = j1.to_dense(), j2.to_dense()
    ref = np.array([[np.trace(J1 @ T[a] @ J2 @ T[b]) for b in range(M)] for a in range(M)])
    eng = fk.Engine(True, "fp64")
    eng.set_H(H, es)
    eng.set_R_identity(n)
    assert _err(eng.moments2_v2(M, j1, j2), ref) <= 1e-11
    eng.close()
