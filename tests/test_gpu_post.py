"""Device KPM post-processing (moment_transform, filling_to_mu, electronic_energy) and the
fixed-filling solve against the oracle's restatement of the same functions.

Tolerances: gamma <= 1e-12 relative to max|gamma|; the chemical potential <= 1e-10 absolute
(both sides bisect to 1e-14 on the same bracket); the energy <= 1e-10 relative; D of the
fixed-filling solve <= 1e-10 (FP64, DS) / 1e-4 (FP32) Frobenius, as for autodiff_matrix.
"""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu


def _case(cplx):
    if cplx:
        H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, 11)
        R = W.phase_probes(W.cubic_colour_groups(4, 2), realisations=2, seed=4)
    else:
        H, es = W.square_lattice(12, -1.0, 1.0, 12)
        R = fk.probe_uncorrelated(H.n_rows, 24, fk.RNG(3))
    return H, es, R


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("kT,filling,delta", [(0.0, 0.5, 0.0), (0.05, 0.3, 0.0), (0.0, 0.42, 0.01)])
def test_kpm_filling_matches_oracle(gpu, cplx, kT, filling, delta):
    H, es, R = _case(cplx)
    M, Mq = 60, 150
    eng = fk.Engine(cplx, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    mu = eng.moments(M)
    mu_f, energy, n_tot, gamma = eng.kpm_filling(Mq, kT, filling, delta)
    g_ref = O.moment_transform(mu, Mq)
    assert np.max(np.abs(gamma - g_ref)) <= 1e-12 * np.max(np.abs(g_ref))
    mu_ref = O.filling_to_mu(g_ref, es.lo, es.hi, kT, filling, delta)
    assert abs(mu_f - mu_ref) <= 1e-10
    e_ref = O.electronic_energy(g_ref, es.lo, es.hi, kT, filling, mu_ref)
    assert abs(energy - e_ref) <= 1e-10 * abs(e_ref)
    assert n_tot == pytest.approx(g_ref.sum() / Mq, rel=1e-12)
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_solve_filling_equals_the_stages_run_separately(gpu, prec):
    H, es, R = _case(True)
    M, Mq, kT, filling = 40, 100, 0.02, 0.45
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    D = H.pattern_like(True)
    mu_f, energy, gamma = eng.solve_filling(M, Mq, kT, filling, D)
    # the same stages through the oracle: moments, filling, coefficients at mu_F, autodiff
    orc = O.OracleEngine(True)
    orc.set_H(H, es)
    orc.set_R(R)
    mu_ref = orc.moments(M)
    g_ref = O.moment_transform(mu_ref, Mq)
    muf_ref = O.filling_to_mu(g_ref, es.lo, es.hi, kT, filling)
    tol_mu = 1e-10 if prec != "fp32" else 1e-5
    assert abs(mu_f - muf_ref) <= tol_mu
    c = O.expansion_coefficients(M, Mq, "fermi_energy", kT, mu_f, es.lo, es.hi)
    D_ref = orc.autodiff_matrix(c, H.pattern_like(True))
    assert rel_err(D.val, D_ref) <= (1e-10 if prec != "fp32" else 1e-4)
    e_ref = O.electronic_energy(g_ref, es.lo, es.hi, kT, filling, muf_ref)
    assert abs(energy - e_ref) <= (1e-10 if prec != "fp32" else 1e-5) * abs(e_ref)
    # moments of the solve are still fetchable (the device sums were left in place)
    assert np.max(np.abs(eng.fetch_moments(M) - mu_ref)) / abs(mu_ref[0]) <= (1e-10 if prec != "fp32" else 1e-5)
    eng.close()


def test_post_processing_errors(gpu):
    H, es, R = _case(False)
    eng = fk.Engine(False, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    with pytest.raises(L.FkError) as ei:
        eng.kpm_filling(100, 0.0, 0.5)
    assert ei.value.status == L.FK_ERR_STATE
    eng.moments(40)
    for bad in [dict(Mq=20, filling=0.5), dict(Mq=100, filling=1.0), dict(Mq=100, filling=0.0)]:
        with pytest.raises(L.FkError) as ei:
            eng.kpm_filling(bad["Mq"], 0.0, bad["filling"])
        assert ei.value.status == L.FK_ERR_ARG
    with pytest.raises(L.FkError) as ei:
        eng.kpm_filling(100, 0.0, 0.5, 0.6)
    assert ei.value.status == L.FK_ERR_ARG
    eng.close()
