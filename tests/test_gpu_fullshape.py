"""GPU parity at the benchmark workloads' full shapes against the oracle, at a small order M.

  * cubic L=64 Kondo-lattice spin blocks (N = 524,288 scalar rows, b = 2 complex,
    nnzb = 1,835,008), S = 256 colour probes (two phase realisations of 128 colours);
  * triangular L=512 spin lattice, J = 2 (N = 524,288, nnzb = 1,835,008), S = 128 colour
    probes (x%8, y%8) x spin;
  * a small triangular spin lattice (L=12) at M = 40, stoch_matrix and autodiff_matrix.

The oracle solves each full-shape case once (moments(M) + autodiff_matrix(c, D), all host
threads); each engine precision is compared with it on the same seeded H and R:
  FP64, DS: moments max_m |mu_m - mu_m^ref| / |mu_0^ref| <= 1e-10, D ||D - D_ref||_F / ||D_ref||_F <= 1e-10;
  FP32:     moments <= 1e-5, D <= 1e-4.
"""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu

TOL_MU = {"fp64": 1e-10, "ds": 1e-10, "fp32": 1e-5}
TOL_D = {"fp64": 1e-10, "ds": 1e-10, "fp32": 1e-4}
M_FULL = 8


def mu_err(mu, ref):
    return float(np.max(np.abs(np.asarray(mu) - ref)) / abs(ref[0]))


def oracle_solve(H, es, R, M, c):
    orc = O.OracleEngine(True, nthreads=0)
    orc.set_H(H, es)
    orc.set_R(R)
    mu = orc.moments(M)
    D = orc.autodiff_matrix(c, H.pattern_like(True))
    return mu, D


def engine_solve(H, es, R, M, c, prec):
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    mu = eng.moments(M)
    D = H.pattern_like(True)
    eng.autodiff_matrix(c, D)
    eng.close()
    return mu, D.val


@pytest.fixture(scope="module")
def cubic64():
    cfg = W.config2()
    H, es = cfg["H"], cfg["es"]
    R = W.phase_probes(cfg["groups"], cfg["realisations"], cfg["probe_seed"])
    assert H.n_rows == 64 ** 3 and R.shape == (2 * 64 ** 3, 256) and H.n_blocks() == 1835008
    c = W.fermi_coefficients(M_FULL, es, "fermi_energy")
    return H, es, R, c, oracle_solve(H, es, R, M_FULL, c)


@pytest.fixture(scope="module")
def triangular512():
    cfg = W.config3()
    H, es = cfg["H"], cfg["es"]
    R = W.phase_probes(cfg["groups"], cfg["realisations"], cfg["probe_seed"])
    assert H.n_rows == 512 ** 2 and R.shape == (2 * 512 ** 2, 128) and H.n_blocks() == 1835008
    c = W.fermi_coefficients(M_FULL, es, "fermi_energy")
    return H, es, R, c, oracle_solve(H, es, R, M_FULL, c)


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_cubic_l64_s256_against_oracle(gpu, cubic64, prec):
    H, es, R, c, (mu_ref, D_ref) = cubic64
    mu, D = engine_solve(H, es, R, M_FULL, c, prec)
    assert mu_err(mu, mu_ref) <= TOL_MU[prec]
    assert rel_err(D, D_ref) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_triangular_l512_s128_against_oracle(gpu, triangular512, prec):
    H, es, R, c, (mu_ref, D_ref) = triangular512
    mu, D = engine_solve(H, es, R, M_FULL, c, prec)
    assert mu_err(mu, mu_ref) <= TOL_MU[prec]
    assert rel_err(D, D_ref) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
@pytest.mark.parametrize("kind", ["autodiff", "stoch"])
def test_small_triangular_lattice_against_oracle(gpu, prec, kind):
    H, es, _ = W.triangular_spin_lattice(12, -1.0, 2.0, seed=12)
    R = W.phase_probes(W.square_colour_groups(12, 4, 4, spin=True), realisations=1, seed=12)
    M = 40
    c = W.fermi_coefficients(M, es, "fermi_energy" if kind == "autodiff" else "fermi_density", 0.0, 0.4)
    orc = O.OracleEngine(True, nthreads=2)
    orc.set_H(H, es)
    orc.set_R(R)
    mu_ref = orc.moments(M)
    D = H.pattern_like(True)
    D_ref = orc.autodiff_matrix(c, D) if kind == "autodiff" else orc.stoch_matrix(c, D)
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    mu = eng.moments(M)
    if kind == "autodiff":
        eng.autodiff_matrix(c, D)
    else:
        eng.stoch_matrix(c, D)
    eng.close()
    assert mu_err(mu, mu_ref) <= TOL_MU[prec]
    assert rel_err(D.val, D_ref) <= TOL_D[prec]
