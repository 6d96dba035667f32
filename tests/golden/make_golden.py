"""Generate the golden fixtures in tests/golden/ (run from the repository root):

    python tests/golden/make_golden.py

Each fixture holds a seeded Hamiltonian (BSR arrays), its energy scale, the
probe-generation recipe and the SHA-256 of the resulting R, the expansion
coefficients, and the oracle's moments, stoch_matrix D and autodiff_matrix D.
The oracle is the CPU restatement of the reference engine (oracle/); these
files pin its outputs so later changes to either side are caught without
re-running it. They are oracle outputs, not outputs of the reference itself
(which ships no fixtures and does not build here).
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import fastkpm_gb300 as fk  # noqa: E402
from fastkpm_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def r_hash(R):
    return hashlib.sha256(np.ascontiguousarray(R).tobytes(order="F")).hexdigest()


def cfg1_case():
    cfg = W.config1()
    H, es, M, S = cfg["H"], cfg["es"], cfg["M"], cfg["S"]
    R = O.R_uncorrelated(H.n_rows, S, cfg["probe_seed"])
    c_den = O.expansion_coefficients(M, 2 * M, "fermi_density", 0.0, 0.0, es.lo, es.hi)
    c_en = O.expansion_coefficients(M, 2 * M, "fermi_energy", 0.0, 0.0, es.lo, es.hi)
    return dict(name="cfg1_square32", H=H, es=es, M=M, R=R, cplx=False, probe="uncorrelated", seed=cfg["probe_seed"],
                S=S, c_den=c_den, c_en=c_en)


def spin_case():
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=7)
    groups = W.cubic_colour_groups(4, 2)
    R = O.R_correlated(groups, 11, complex_values=True)
    M = 40
    c_den = O.expansion_coefficients(M, 2 * M, "fermi_density", 0.0, 0.2, es.lo, es.hi)
    c_en = O.expansion_coefficients(M, 2 * M, "fermi_energy", 0.0, 0.2, es.lo, es.hi)
    return dict(name="spin_cubic4", H=H, es=es, M=M, R=R, cplx=True, probe="correlated", seed=11, S=R.shape[1],
                c_den=c_den, c_en=c_en, groups=groups)


def main():
    for case in (cfg1_case(), spin_case()):
        H, es, R, M = case["H"], case["es"], case["R"], case["M"]
        o = O.OracleEngine(case["cplx"], nthreads=1)
        o.set_H(H, es)
        o.set_R(R)
        mu = o.moments(M)
        D_auto = o.autodiff_matrix(case["c_en"], H)
        D_stoch = o.stoch_matrix(case["c_den"], H)
        out = dict(row_ptr=H.row_ptr, col_idx=H.col_idx, val=H.val, b=H.b_len, es=np.array([es.lo, es.hi]), M=M,
                   probe=case["probe"], seed=case["seed"], S=case["S"], R_sha256=r_hash(R), c_den=case["c_den"],
                   c_en=case["c_en"], mu=mu, D_auto=D_auto, D_stoch=D_stoch)
        if "groups" in case:
            out["groups"] = case["groups"]
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("wrote", case["name"], "mu0=%.6g" % mu[0])


if __name__ == "__main__":
    main()
