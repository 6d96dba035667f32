"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the product's probe generator reproduces the fixture's R bit for bit
(SHA-256), and the oracle reproduces the stored moments and D exactly up to
floating-point re-association (<= 1e-12). GPU: the engine matches the stored
oracle outputs within the FP64 tolerance (1e-10 relative).
"""
import hashlib
import os

import numpy as np
import pytest

import fastkpm_gb300 as fk
from oracle import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["cfg1_square32", "spin_cubic4"]


def load(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    cplx = np.iscomplexobj(z["val"])
    n_b = len(z["row_ptr"]) - 1
    H = fk.SpMatBsr(n_b, int(z["b"]), z["row_ptr"], z["col_idx"], z["val"], complex_values=cplx)
    es = fk.EnergyScale(*z["es"])
    n = n_b * int(z["b"])
    if str(z["probe"]) == "uncorrelated":
        R = fk.probe_uncorrelated(n, int(z["S"]), fk.RNG(int(z["seed"])), complex_values=cplx)
    else:
        R = fk.probe_correlated(z["groups"], fk.RNG(int(z["seed"])), complex_values=cplx)
    return z, H, es, R, cplx


@pytest.mark.parametrize("name", CASES)
def test_fixture_probes_regenerate_bit_identically(built_lib, name):
    z, H, es, R, cplx = load(name)
    assert hashlib.sha256(np.ascontiguousarray(R).tobytes(order="F")).hexdigest() == str(z["R_sha256"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_fixture(built_lib, name):
    z, H, es, R, cplx = load(name)
    o = O.OracleEngine(cplx, nthreads=2)
    o.set_H(H, es)
    o.set_R(R)
    M = int(z["M"])
    mu = o.moments(M)
    assert np.max(np.abs(mu - z["mu"])) / abs(z["mu"][0]) <= 1e-12
    D = o.autodiff_matrix(z["c_en"], H)
    assert np.linalg.norm(D - z["D_auto"]) <= 1e-12 * np.linalg.norm(z["D_auto"])
    D = o.stoch_matrix(z["c_den"], H)
    assert np.linalg.norm(D - z["D_stoch"]) <= 1e-12 * np.linalg.norm(z["D_stoch"])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "ds"])
@pytest.mark.parametrize("name", CASES)
def test_engine_matches_fixture(gpu, name, prec):
    z, H, es, R, cplx = load(name)
    eng = fk.Engine(cplx, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    M = int(z["M"])
    mu = eng.moments(M)
    assert np.max(np.abs(mu - z["mu"])) / abs(z["mu"][0]) <= 1e-10
    D = H.pattern_like(cplx)
    eng.autodiff_matrix(z["c_en"], D)
    assert np.linalg.norm(D.val - z["D_auto"]) <= 1e-10 * np.linalg.norm(z["D_auto"])
    eng.stoch_matrix(z["c_den"], D)
    assert np.linalg.norm(D.val - z["D_stoch"]) <= 1e-10 * np.linalg.norm(z["D_stoch"])
