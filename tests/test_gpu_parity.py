"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same
seeded H and R, plus analytic answers, edge cases and error behaviour.

Tolerances (stated with every check):
  FP64 and DS engines: moments max_m |mu_m - mu_m^ref| / |mu_0^ref| <= 1e-10,
                       D ||D - D_ref||_F / ||D_ref||_F <= 1e-10.
  FP32 engine:         moments <= 1e-5 (relative to mu_0), D <= 1e-4 (Frobenius).
"""
import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import cheb_T, rel_err

pytestmark = pytest.mark.gpu

TOL_MU = {"fp64": 1e-10, "ds": 1e-10, "fp32": 1e-5}
TOL_D = {"fp64": 1e-10, "ds": 1e-10, "fp32": 1e-4}


def mu_err(mu, ref):
    return float(np.max(np.abs(np.asarray(mu) - ref)) / abs(ref[0]))


def small_complex_case(L_=4, S=16, seed=21):
    H, es, _ = W.cubic_spin_lattice(L_, -1.0, 1.0, seed)
    R = W.phase_probes(W.cubic_colour_groups(L_, 2), realisations=max(1, S // 16), seed=seed)
    return H, es, R


def small_real_case(L_=12, S=24, seed=31):
    H, es = W.square_lattice(L_, -1.0, 1.0, seed)
    R = fk.probe_uncorrelated(H.n_rows, S, fk.RNG(seed))
    return H, es, R


def run_pair(H, es, R, cplx, prec, M, c, kind, options=None):
    eng = fk.Engine(cplx, prec)
    for k, v in (options or {}).items():
        eng.set_option(k, v)
    eng.set_H(H, es)
    eng.set_R(R)
    orc = O.OracleEngine(cplx)
    orc.set_H(H, es)
    orc.set_R(R)
    mu = eng.moments(M)
    mu_ref = orc.moments(M)
    D = H.pattern_like(cplx)
    if kind == "autodiff":
        eng.autodiff_matrix(c, D)
        D_ref = orc.autodiff_matrix(c, D)
    else:
        eng.stoch_matrix(c, D)
        D_ref = orc.stoch_matrix(c, D)
    return mu, mu_ref, D.val, D_ref


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_config1_moments_and_stoch(gpu, prec):
    cfg = W.config1()
    H, es = cfg["H"], cfg["es"]
    R = fk.probe_uncorrelated(H.n_rows, cfg["S"], fk.RNG(cfg["probe_seed"]))
    c = W.fermi_coefficients(cfg["M"], es)
    mu, mu_ref, D, D_ref = run_pair(H, es, R, False, prec, cfg["M"], c, "stoch")
    assert mu_err(mu, mu_ref) <= TOL_MU[prec]
    assert rel_err(D, D_ref) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("kind", ["autodiff", "stoch"])
def test_small_cases(gpu, prec, cplx, kind):
    H, es, R = small_complex_case() if cplx else small_real_case()
    M = 40
    c = W.fermi_coefficients(M, es, "fermi_energy" if kind == "autodiff" else "fermi_density", 0.0, 0.3)
    mu, mu_ref, D, D_ref = run_pair(H, es, R, cplx, prec, M, c, kind)
    assert mu_err(mu, mu_ref) <= TOL_MU[prec]
    assert rel_err(D, D_ref) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp64", "ds"])
def test_identity_probes_exact_traces(gpu, prec):
    H, es, _ = W.cubic_spin_lattice(3, -1.0, 1.0, seed=5)
    A = (H.to_dense() - es.avg() * np.eye(54)) / es.mag()
    lam = np.linalg.eigvalsh(A)
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    eng.set_R_identity(54)
    M = 30
    mu = eng.moments(M)
    ref = np.array([cheb_T(m, lam).sum() for m in range(M)])
    assert np.max(np.abs(mu - ref)) / 54 < 1e-10


@pytest.mark.parametrize("opts", [
    {L.FK_OPT_TMA: 0},
    {L.FK_OPT_FUSE_D: 1},
    {L.FK_OPT_FUSE_D: 0},
    {L.FK_OPT_STAGE_H: 0},
    {L.FK_OPT_NP: 1},
    {L.FK_OPT_NP: 2},
    {L.FK_OPT_CTAS_PER_SM: 1},
    {L.FK_OPT_CTA_WAVES: 8},
])
def test_launch_options_do_not_change_results(gpu, opts):
    # S = 80 complex -> 80 packets per row: exercises column slices when NP is capped
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=3)
    R = W.phase_probes(W.cubic_colour_groups(4, 2), realisations=5, seed=3)
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    mu, mu_ref, D, D_ref = run_pair(H, es, R, True, "fp64", M, c, "autodiff", opts)
    assert mu_err(mu, mu_ref) <= 1e-10
    assert rel_err(D, D_ref) <= 1e-10


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
@pytest.mark.parametrize("S", [32, 40])
@pytest.mark.parametrize("fuse", [0, 1])
def test_whole_and_ragged_column_chunks(gpu, prec, S, fuse):
    # S = 32 complex: every kernel's rows split into whole chunks (the unmasked instances);
    # S = 40: the last chunk is ragged (the masked instances). Both against the oracle.
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=9)
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, S, fk.RNG(9), complex_values=True)
    M = 16
    c = W.fermi_coefficients(M, es, "fermi_energy")
    for kind in ("autodiff", "stoch"):
        mu, mu_ref, D, D_ref = run_pair(H, es, R, True, prec, M, c, kind, {L.FK_OPT_FUSE_D: fuse})
        assert mu_err(mu, mu_ref) <= TOL_MU[prec]
        assert rel_err(D, D_ref) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_sparse_probe_upload_equals_dense(gpu, prec):
    # set_R_sparse (nonzeros, k per row) builds the same device R as set_R of the dense block
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=4)
    groups = W.cubic_colour_groups(4, 2)
    R = W.phase_probes(groups, realisations=2, seed=6)
    s, cols, vals = W.phase_probe_entries(groups, realisations=2, seed=6)
    M = 16
    c = W.fermi_coefficients(M, es, "fermi_energy")
    out = []
    for sparse in (False, True):
        eng = fk.Engine(True, prec)
        eng.set_H(H, es)
        if sparse:
            eng.set_R_sparse(R.shape[0], s, cols, vals)
        else:
            eng.set_R(R)
        assert np.array_equal(eng.get_R(), R.astype(np.complex128)) or prec != "fp64"
        mu = eng.moments(M)
        D = H.pattern_like(True)
        eng.autodiff_matrix(c, D)
        out.append((mu, D.val))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    # repeated columns of a row add up; a column outside [0, s) is refused
    eng = fk.Engine(False, prec)
    eng.set_H(*W.square_lattice(4, -1.0, 1.0, 1))
    eng.set_R_sparse(16, 3, np.tile([[1, 1]], (16, 1)), np.full((16, 2), 0.5))
    Rr = eng.get_R()
    assert np.allclose(Rr[:, 1], 1.0) and np.allclose(Rr[:, [0, 2]], 0.0)
    with pytest.raises(L.FkError) as ei:
        eng.set_R_sparse(16, 3, np.full((16, 1), 3), np.ones((16, 1)))
    assert ei.value.status == L.FK_ERR_ARG


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
@pytest.mark.parametrize("S", [32, 40])
def test_two_pass_adjoint_equals_one_pass(gpu, prec, S):
    # k_adjoint_split does the same arithmetic in the same order as k_adjoint_step (the warp-per-row
    # kernels, which rows of 32 lanes would otherwise take, have their own test)
    H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=12)
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, S, fk.RNG(12), complex_values=True)
    M = 16
    c = W.fermi_coefficients(M, es, "fermi_energy")
    one = run_pair(H, es, R, True, prec, M, c, "autodiff", {L.FK_OPT_ADJ_SPLIT: 0, L.FK_OPT_WARP_ROWS: 0})
    two = run_pair(H, es, R, True, prec, M, c, "autodiff", {L.FK_OPT_ADJ_SPLIT: 1, L.FK_OPT_WARP_ROWS: 0})
    assert np.array_equal(one[0], two[0]) and np.array_equal(one[2], two[2])
    assert rel_err(two[2], two[3]) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp32", "ds"])
@pytest.mark.parametrize("cplx", [True, False])
@pytest.mark.parametrize("S", [32, 40])
def test_pipelined_step_equals_plain(gpu, prec, cplx, S):
    # k_cheb_step_pipe and k_adjoint_pipe (gathers double-buffered through shared memory) do the
    # plain kernels' arithmetic in the same order: identical moments and D, whole and ragged chunks
    # (the warp-per-row reverse step, which rows of 32 lanes would otherwise take, has its own test)
    if cplx:
        H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=13)
        R = fk.probe_uncorrelated(H.n_rows * H.b_len, S, fk.RNG(13), complex_values=True)
    else:
        H, es, R = small_real_case(10, S, 13)
    M = 16
    c = W.fermi_coefficients(M, es, "fermi_energy")
    for kind in ("autodiff", "stoch"):
        plain = run_pair(H, es, R, cplx, prec, M, c, kind, {L.FK_OPT_PIPE: 0})
        piped = run_pair(H, es, R, cplx, prec, M, c, kind, {L.FK_OPT_PIPE: 1, L.FK_OPT_WARP_ROWS: 0})
        assert np.array_equal(plain[0], piped[0]) and np.array_equal(plain[2], piped[2])
        assert mu_err(piped[0], piped[1]) <= TOL_MU[prec]


def test_stream_priority_option(gpu):
    # the engine's own stream can be recreated with a CUDA priority (clamped to the device's
    # range); results do not depend on it
    H, es, R = small_real_case(8, 16, 5)
    M = 20
    c = W.fermi_coefficients(M, es, "fermi_energy")
    base = run_pair(H, es, R, False, "fp32", M, c, "autodiff")
    urgent = run_pair(H, es, R, False, "fp32", M, c, "autodiff", {L.FK_OPT_PRIORITY: -100})
    assert np.array_equal(base[0], urgent[0]) and np.array_equal(base[2], urgent[2])
    eng = fk.Engine(False, "fp32")
    eng.set_option(L.FK_OPT_PRIORITY, -100)
    assert eng.get_option(L.FK_OPT_PRIORITY) <= 0
    eng.set_option(L.FK_OPT_PRIORITY, 5)
    assert eng.get_option(L.FK_OPT_PRIORITY) == 0


@pytest.mark.parametrize("M", [2, 4, 6])
def test_autodiff_small_orders(gpu, M):
    H, es, R = small_real_case(6, 8, 2)
    c = W.fermi_coefficients(M, es, "fermi_energy", 0.0, 0.1, Mq=2 * M)
    mu, mu_ref, D, D_ref = run_pair(H, es, R, False, "fp64", M, c, "autodiff")
    assert mu_err(mu, mu_ref) <= 1e-12
    assert rel_err(D, D_ref) <= 1e-12


@pytest.mark.parametrize("prec,S", [("fp64", 1), ("fp32", 3), ("ds", 5), ("fp32", 1)])
def test_odd_and_single_probe_columns(gpu, prec, S):
    H, es, R = small_real_case(7, S, 4)
    M = 20
    c = W.fermi_coefficients(M, es)
    mu, mu_ref, D, D_ref = run_pair(H, es, R, False, prec, M, c, "stoch")
    assert mu_err(mu, mu_ref) <= TOL_MU[prec]
    assert rel_err(D, D_ref) <= TOL_D[prec] * 10


def test_D_pattern_wider_than_H(gpu):
    # D on second-neighbour pattern (not H's): exercises the standalone outer-product kernel
    H, es, R = small_complex_case(4, 16, 8)
    H2 = W.cubic_spin_lattice(4, -1.0, 1.0, seed=8)[0]
    A = (np.abs(H2.to_dense()) > 0).astype(float)
    P = ((A @ A) > 0)
    b = 2
    Pb = P[::b, ::b]
    rows, cols = np.nonzero(Pb)
    D = fk.SpMatBsr.build(Pb.shape[0], b, rows, cols, np.zeros((len(rows), 4), complex))
    M = 20
    c = W.fermi_coefficients(M, es, "fermi_energy")
    eng = fk.Engine(True, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    orc = O.OracleEngine(True)
    orc.set_H(H, es)
    orc.set_R(R)
    eng.moments(M)
    orc.moments(M)
    eng.autodiff_matrix(c, D)
    assert rel_err(D.val, orc.autodiff_matrix(c, D)) <= 1e-10
    eng.stoch_matrix(c, D)
    assert rel_err(D.val, orc.stoch_matrix(c, D)) <= 1e-10


def test_missing_diagonal_blocks_are_inserted(gpu):
    H, _ = W.square_lattice(6, -1.0, 0.0, seed=0)
    keep = H.row_idx != H.col_idx
    H0 = fk.SpMatBsr.build(H.n_rows, 1, H.row_idx[keep], H.col_idx[keep], H.val[keep][:, None])
    es = fk.EnergyScale(-3.0, 5.0)   # avg != 0: the diagonal shift needs the inserted blocks
    R = fk.probe_uncorrelated(36, 8, fk.RNG(1))
    M = 20
    c = W.fermi_coefficients(M, es)
    mu, mu_ref, D, D_ref = run_pair(H0, es, R, False, "fp64", M, c, "stoch")
    assert mu_err(mu, mu_ref) <= 1e-12
    assert rel_err(D, D_ref) <= 1e-12


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_staged_and_plain_step_agree(gpu, prec):
    """The staged step kernels (TMA bulk copies, cp.async) and the per-thread-gather kernel compute
    the same rows in the same order: FP64/DS moments agree to rounding of the CTA sums (1e-13).
    FP32 complex products may be contracted into FMAs differently in the two compiled kernels,
    so FP32 moments agree to FP32 rounding (1e-6, measured 9e-9)."""
    H, es, R = small_complex_case(6, 32, 4)
    M = 30
    mus = []
    for tma in (1, 2, 0):   # TMA bulk copies, cp.async copies, per-thread gathers
        eng = fk.Engine(True, prec)
        eng.set_option(L.FK_OPT_TMA, tma)
        eng.set_H(H, es)
        eng.set_R(R)
        assert eng.get_option(L.FK_OPT_TMA) == tma
        mus.append(eng.moments(M))
        eng.close()
    for mu in mus[:2]:
        assert np.max(np.abs(mu - mus[2])) / abs(mus[2][0]) <= (1e-6 if prec == "fp32" else 1e-13)


def test_device_expansion_coefficients(gpu):
    """FP64 coefficients on the device match the host restatement (<= 1e-13 absolute)."""
    eng = fk.Engine(False, "fp64")
    for kind in ["fermi_density", "fermi_energy"]:
        for (M, Mq, kT, mu, lo, hi) in [(200, 400, 0.0, 0.0, -4.5, 4.5), (1000, 2000, 0.05, 0.3, -7.07, 7.07)]:
            c = eng.expansion_coefficients(M, Mq, kind, kT, mu, fk.EnergyScale(lo, hi))
            ref = O.expansion_coefficients(M, Mq, kind, kT, mu, lo, hi)
            assert np.max(np.abs(c - ref)) <= 1e-13


@pytest.mark.parametrize("prec", ["fp64", "ds", "fp32"])
def test_graph_replay_matches_direct_launches(gpu, prec):
    """FK_OPT_GRAPHS: captured sequences give bit-identical results to direct launches, replays
    see new coefficients and new R values, and a reallocated R (more columns) is recaptured."""
    H, es, _ = small_complex_case(4, 16, 6)
    M = 24
    probes = [W.phase_probes(W.cubic_colour_groups(4, 2), realisations=r, seed=s) for r, s in [(1, 1), (1, 2), (3, 3)]]
    coefs = [W.fermi_coefficients(M, es, "fermi_energy", 0.0, mu) for mu in (0.0, 0.4)]

    def run(graphs):
        eng = fk.Engine(True, prec)
        eng.set_option(L.FK_OPT_GRAPHS, graphs)
        eng.set_H(H, es)
        out = []
        for R in probes:
            eng.set_R(R)
            for c in coefs:
                D = H.pattern_like(True)
                out.append(eng.moments(M))
                eng.autodiff_matrix(c, D)
                out.append(D.val.copy())
                eng.stoch_matrix(c, D)
                out.append(D.val.copy())
        eng.close()
        return out

    direct, replayed = run(0), run(1)
    for a, b in zip(direct, replayed):
        assert np.array_equal(a, b)
    # the replayed results are the right ones, not only repeatable
    orc = O.OracleEngine(True)
    orc.set_H(H, es)
    orc.set_R(probes[2])
    mu_ref = orc.moments(M)
    D_ref = orc.autodiff_matrix(coefs[1], H.pattern_like(True))
    assert mu_err(replayed[-3], mu_ref) <= TOL_MU[prec]
    assert rel_err(replayed[-2], D_ref) <= TOL_D[prec]


@pytest.mark.parametrize("prec", ["fp64", "ds"])
def test_permutation_invariance(gpu, prec):
    """Moments and D do not depend on the order of the probe columns, nor on the labelling of
    the sites (H, R and D permuted together): equal to rounding (1e-12)."""
    H, es, R = small_complex_case(4, 16, 13)
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    mu0 = eng.moments(M)
    D0 = H.pattern_like(True)
    eng.autodiff_matrix(c, D0)
    # probe columns reversed
    eng.set_R(np.asfortranarray(R[:, ::-1]))
    mu1 = eng.moments(M)
    D1 = H.pattern_like(True)
    eng.autodiff_matrix(c, D1)
    assert mu_err(mu1, mu0) <= 1e-12
    assert rel_err(D1.val, D0.val) <= 1e-12
    # sites relabelled by a seeded permutation p: block row i of H' is block row p[i] of H
    b = H.b_len
    p = np.random.default_rng(3).permutation(H.n_rows)
    inv = np.argsort(p)
    blocks = H.val.reshape(-1, b * b)
    Hp = fk.SpMatBsr.build(H.n_rows, b, inv[H.row_idx], inv[H.col_idx], blocks)
    rows = (b * p[:, None] + np.arange(b)).reshape(-1)   # scalar row r' of R' is row rows[r'] of R
    eng.set_H(Hp, es)
    eng.set_R(np.asfortranarray(R[rows]))
    mu2 = eng.moments(M)
    D2 = Hp.pattern_like(True)
    eng.autodiff_matrix(c, D2)
    assert mu_err(mu2, mu0) <= 1e-12
    for k in range(0, H.n_blocks(), 7):
        i, j = H.row_idx[k], H.col_idx[k]
        ref = D0.val[k * b * b:(k + 1) * b * b]
        kp = Hp.find_index(inv[i], inv[j])
        assert np.max(np.abs(D2.val[kp * b * b:(kp + 1) * b * b] - ref)) <= 1e-12 * np.max(np.abs(D0.val))
    eng.close()


@pytest.mark.parametrize("cplx", [False, True])
def test_upload_paths_agree(gpu, cplx):
    """set_R through staging copies (FK_OPT_UPLOAD 1) and read in place (0, from ordinary and
    from page-locked host memory) give the same device R, bit for bit."""
    H, es, R = small_complex_case(4, 16, 17) if cplx else small_real_case(9, 37, 17)
    lib = L.load()
    outs = []
    for upload, pin in [(1, False), (0, False), (0, True)]:
        eng = fk.Engine(cplx, "fp64")
        eng.set_option(L.FK_OPT_UPLOAD, upload)
        assert eng.get_option(L.FK_OPT_UPLOAD) == upload
        eng.set_H(H, es)
        Rh = np.asfortranarray(R.copy())
        if pin:
            assert lib.fk_host_register(Rh.ctypes.data, Rh.nbytes) == L.FK_OK
        eng.set_R(Rh)
        outs.append((eng.get_R(), eng.moments(20)))
        if pin:
            lib.fk_host_unregister(Rh.ctypes.data)
        eng.close()
    for Rg, mu in outs:
        assert np.array_equal(Rg, R)
        assert np.array_equal(mu, outs[0][1])


def test_results_are_deterministic(gpu):
    H, es, R = small_complex_case(6, 32, 2)
    eng = fk.Engine(True, "ds")
    eng.set_H(H, es)
    eng.set_R(R)
    M = 50
    a = eng.moments(M)
    b = eng.moments(M)
    assert np.array_equal(a, b)


def test_error_behaviour(gpu):
    H, es, R = small_real_case(6, 8, 1)
    eng = fk.Engine(False, "fp64")
    with pytest.raises(L.FkError) as ei:
        eng.moments(10)
    assert ei.value.status == L.FK_ERR_STATE
    eng.set_H(H, es)
    eng.set_R(R)
    with pytest.raises(L.FkError) as ei:
        eng.moments(7)
    assert ei.value.status == L.FK_ERR_ARG
    D = H.pattern_like()
    c = W.fermi_coefficients(10, es)
    with pytest.raises(L.FkError) as ei:
        eng.autodiff_matrix(c, D)   # no moments(10) first
    assert ei.value.status == L.FK_ERR_STATE
    eng.moments(10)
    # an asymmetric D pattern cannot be symmetrized
    Dbad = fk.SpMatBsr(H.n_rows, 1, np.r_[0, np.ones(H.n_rows, np.int32)].cumsum().astype(np.int32),
                       np.r_[1, np.arange(1, H.n_rows)].astype(np.int32))
    with pytest.raises(L.FkError) as ei:
        eng.autodiff_matrix(c, Dbad)
    assert ei.value.status == L.FK_ERR_PATTERN
    with pytest.raises(L.FkError) as ei:
        eng.set_R(np.ones((H.n_rows + 1, 2)))
        eng.moments(10)
    assert ei.value.status == L.FK_ERR_ARG
    with pytest.raises(L.FkError) as ei:
        eng.set_R(np.ones((H.n_rows, 0)))
    assert ei.value.status == L.FK_ERR_ARG
    bad = H.copy()
    bad.col_idx = bad.col_idx.copy()
    bad.col_idx[0], bad.col_idx[1] = bad.col_idx[1], bad.col_idx[0]
    with pytest.raises(L.FkError) as ei:
        eng.set_H(bad, es)
    assert ei.value.status == L.FK_ERR_PATTERN


def test_energy_scale_lanczos(gpu):
    H, _ = W.square_lattice(10, -1.0, 2.0, seed=4)
    lam = np.linalg.eigvalsh(H.to_dense())
    eng = fk.Engine(False, "fp64")
    v0 = np.random.default_rng(0).standard_normal(100)
    es = eng.energy_scale(H, 0.0, 100, v0=v0)
    assert abs(es.lo - lam.min()) < 1e-8 and abs(es.hi - lam.max()) < 1e-8
    lo, hi = O.OracleEngine(False).energy_scale(H, 0.05, 40, v0)
    es2 = eng.energy_scale(H, 0.05, 40, v0=v0)
    assert abs(es2.lo - lo) < 1e-9 and abs(es2.hi - hi) < 1e-9
    es3 = eng.energy_scale(H, 0.01)   # seeded start vector
    assert es3.lo <= lam.min() + 1e-6 and es3.hi >= lam.max() - 1e-6
    # a start vector that is an eigenvector ends the recursion at beta_1 = 0 (exactly)
    d = np.arange(1.0, 9.0)
    Hd = fk.SpMatBsr.build(8, 1, np.arange(8), np.arange(8), d[:, None])
    e0 = np.zeros(8)
    e0[2] = 1.0
    es4 = eng.energy_scale(Hd, 0.0, 6, v0=e0)
    assert es4.lo == 3.0 and es4.hi == 3.0


def test_complex_energy_scale(gpu):
    H, _, _ = W.cubic_spin_lattice(3, -1.0, 1.0, seed=1)
    lam = np.linalg.eigvalsh(H.to_dense())
    es = fk.Engine(True, "fp64").energy_scale(H, 0.0, 54)
    assert abs(es.lo - lam.min()) < 1e-7 and abs(es.hi - lam.max()) < 1e-7


@pytest.mark.parametrize("prec", ["fp64", "ds"])
def test_probe_split_additivity_full_size(gpu, prec):
    """Size-independent property at the full cubic L=64, S=256 shape: moments and D are sums
    over probe columns, so the two halves of R must add up to the whole; mu_0 = ||R||^2."""
    cfg = W.config2()
    H, es = cfg["H"], cfg["es"]
    R = W.phase_probes(cfg["groups"], cfg["realisations"], cfg["probe_seed"])
    M = 8
    c = W.fermi_coefficients(M, es, "fermi_energy")
    D = H.pattern_like(True)
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    parts_mu, parts_D = [], []
    for cols in [slice(0, 256), slice(0, 128), slice(128, 256)]:
        eng.set_R(R[:, cols])
        parts_mu.append(eng.moments(M))
        eng.autodiff_matrix(c, D)
        parts_D.append(D.val.copy())
    assert abs(parts_mu[0][0] - np.vdot(R, R).real) / parts_mu[0][0] < 1e-12
    assert mu_err(parts_mu[1] + parts_mu[2], parts_mu[0]) < 1e-12
    assert rel_err(parts_D[1] + parts_D[2], parts_D[0]) < 1e-11


@pytest.mark.parametrize("acc64", [1, 0])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("kind", ["autodiff", "stoch"])
def test_fp32_accumulator_forms_against_oracle(gpu, acc64, cplx, kind):
    # FP32 recursion with FP64 moment sums and D accumulator (FK_OPT_ACC64 = 1, the default) and
    # with float-float ones (0): both within the FP32 tolerances of the oracle
    H, es, R = small_complex_case(4, 32, 41) if cplx else small_real_case(12, 32, 41)
    M = 60
    c = W.fermi_coefficients(M, es, "fermi_energy" if kind == "autodiff" else "fermi_density", 0.0, 0.2)
    mu, mu_ref, D, D_ref = run_pair(H, es, R, cplx, "fp32", M, c, kind, {L.FK_OPT_ACC64: acc64})
    assert mu_err(mu, mu_ref) <= TOL_MU["fp32"]
    assert rel_err(D, D_ref) <= TOL_D["fp32"]


def test_acc64_option_reads_back(gpu):
    for prec, want in [("fp64", 1), ("ds", 0), ("fp32", 1)]:
        eng = fk.Engine(True, prec)
        assert eng.get_option(L.FK_OPT_ACC64) == want
        eng.close()
    eng = fk.Engine(False, "fp32")
    eng.set_option(L.FK_OPT_ACC64, 0)
    assert eng.get_option(L.FK_OPT_ACC64) == 0
    with pytest.raises(L.FkError):
        eng.set_option(L.FK_OPT_ACC64, 2)
    eng.close()


@pytest.mark.parametrize("prec,opts", [("fp32", {L.FK_OPT_ACC64: 1}), ("fp32", {L.FK_OPT_ACC64: 0}),
                                       ("fp32", {L.FK_OPT_FUSE_D: 0}), ("fp32", {L.FK_OPT_CTAS_PER_SM: 1}),
                                       ("fp64", {}), ("fp64", {L.FK_OPT_CTAS_PER_SM: 1}),
                                       ("ds", {}), ("ds", {L.FK_OPT_CTAS_PER_SM: 1})])
def test_warp_row_adjoint_against_general(gpu, prec, opts):
    # b=2 complex rows with S=256 columns are served by a whole warp (32 lanes, whole chunks):
    # the reverse step runs k_adjoint_warp (FP32, float-float) / k_adjoint_step_warp (FP64) by default
    # (FK_OPT_WARP_ROWS 1) and k_adjoint_pipe / k_adjoint_step with the option off. Same moments (the
    # forward step is shared); D within the engine's tolerance of the oracle, and within rounding of
    # the general kernel (FP32 1e-5, FP64 and float-float 1e-12, Frobenius).
    # L=16: 4,096 rows in 512 tiles, more than the CTAs of one wave (and 152 CTAs with one per SM),
    # so warps walk several rows and the unit stream continues across rows
    H, es, _ = W.cubic_spin_lattice(16, -1.0, 1.0, seed=17)
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, 256, fk.RNG(17), complex_values=True)
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    warp = run_pair(H, es, R, True, prec, M, c, "autodiff", dict(opts))
    general = run_pair(H, es, R, True, prec, M, c, "autodiff", {**opts, L.FK_OPT_WARP_ROWS: 0})
    assert np.array_equal(warp[0], general[0])
    assert mu_err(warp[0], warp[1]) <= TOL_MU[prec]
    assert rel_err(warp[2], warp[3]) <= TOL_D[prec]
    assert rel_err(warp[2], general[2]) <= (1e-5 if prec == "fp32" else 1e-12)
    for p, want in [("fp32", 1), ("ds", 1), ("fp64", 1)]:
        eng = fk.Engine(True, p)
        eng.set_H(H, es)
        eng.set_R(R)
        assert eng.get_option(L.FK_OPT_WARP_ROWS) == want
        eng.set_option(L.FK_OPT_WARP_ROWS, 0)
        assert eng.get_option(L.FK_OPT_WARP_ROWS) == 0
        eng.close()


@pytest.mark.parametrize("prec,opts", [("fp32", {L.FK_OPT_ACC64: 1}), ("fp32", {L.FK_OPT_ACC64: 0}), ("ds", {})])
def test_adjoint_column_sweeps_same_bits(gpu, prec, opts):
    # FK_OPT_ADJ_SWEEP 1: the warp-per-row reverse step runs as one launch per column chunk (S=256
    # complex columns: FP32 2 chunks, float-float 4). Every D entry adds its chunks in the same order
    # as in one launch over whole rows, so D is the same to the bit; the moments come from the shared
    # forward step. D against the oracle within the engine's tolerance.
    H, es, _ = W.cubic_spin_lattice(16, -1.0, 1.0, seed=31)
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, 256, fk.RNG(31), complex_values=True)
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    swept = run_pair(H, es, R, True, prec, M, c, "autodiff", {**opts, L.FK_OPT_ADJ_SWEEP: 1})
    whole = run_pair(H, es, R, True, prec, M, c, "autodiff", {**opts, L.FK_OPT_ADJ_SWEEP: 0})
    assert np.array_equal(swept[0], whole[0])
    assert np.array_equal(swept[2], whole[2])
    assert mu_err(swept[0], swept[1]) <= TOL_MU[prec]
    assert rel_err(swept[2], swept[3]) <= TOL_D[prec]
    eng = fk.Engine(True, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    assert eng.get_option(L.FK_OPT_ADJ_SWEEP) == 0   # 16^3: two planes of rows fit L2 many times over
    eng.set_option(L.FK_OPT_ADJ_SWEEP, 1)
    assert eng.get_option(L.FK_OPT_ADJ_SWEEP) == 1
    eng.close()


def test_adjoint_column_sweeps_by_size(gpu):
    # Float-float engines sweep by default when the six vectors' rows moved between a row's first
    # and last gathers (twice the block-column distance 90% of H's blocks keep within: L^2 sites on
    # the periodic cubic lattice) exceed half of L2: cubic L=32 with S=256 complex columns moves
    # 2 x 1024 sites x 2 rows x 6 x 4 KB = 101 MB (sweeps on a GPU whose L2 is below 201 MB).
    # FP32 engines run one launch by default.
    import torch
    l2 = getattr(torch.cuda.get_device_properties(0), "L2_cache_size", None)
    if not l2:
        pytest.skip("torch does not report the L2 size")
    H, es, _ = W.cubic_spin_lattice(32, -1.0, 1.0, seed=37)
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, 256, fk.RNG(37), complex_values=True)
    for prec, want in [("ds", 1 if 2 * 1024 * 2 * 6 * 256 * 16 > l2 / 2 else 0), ("fp32", 0)]:
        eng = fk.Engine(True, prec)
        eng.set_H(H, es)
        eng.set_R(R)
        assert eng.get_option(L.FK_OPT_ADJ_SWEEP) == want
        eng.close()


@pytest.mark.parametrize("prec", ["ds", "fp32"])
def test_warp_row_adjoint_nonuniform_hopping(gpu, prec):
    # Rows whose identity (hopping) blocks do not all share one value: every third bond of the 16^3
    # spin lattice hops with 1.5 t (bond (i, j) and (j, i) alike, so H stays Hermitian). Float-float
    # rows with one hopping value sum their identity blocks' rows first and scale once; the others
    # (and every FP32 row) multiply-add block by block. Against the oracle and the general kernel.
    H, es0, _ = W.cubic_spin_lattice(16, -1.0, 1.0, seed=23)
    rows = np.repeat(np.arange(H.n_rows), np.diff(H.row_ptr))
    cols = H.col_idx
    b2 = H.b_len * H.b_len
    pick = (rows != cols) & ((rows + cols) % 3 == 0)
    val = H.val.reshape(-1, b2).copy()
    val[pick] *= 1.5
    H = H.with_values(val.ravel())
    es = fk.EnergyScale(1.6 * es0.lo, 1.6 * es0.hi)
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, 256, fk.RNG(23), complex_values=True)
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    warp = run_pair(H, es, R, True, prec, M, c, "autodiff")
    general = run_pair(H, es, R, True, prec, M, c, "autodiff", {L.FK_OPT_WARP_ROWS: 0})
    assert mu_err(warp[0], warp[1]) <= TOL_MU[prec]
    assert rel_err(warp[2], warp[3]) <= TOL_D[prec]
    assert rel_err(warp[2], general[2]) <= (1e-5 if prec == "fp32" else 1e-12)


@pytest.mark.parametrize("prec", ["ds", "fp32", "fp64"])
def test_warp_row_adjoint_real_b2(gpu, prec):
    # Real 2x2 blocks with S=256 probe columns (the real part of the cubic spin lattice: symmetric,
    # hopping blocks t I2 and real exchange blocks): rows served by a whole warp take the warp-per-row
    # reverse step (FP32 and float-float: real block entries, D entries 8 bytes each) in FP32 and
    # float-float; FP64 keeps k_adjoint_step (its warp form is for complex blocks). Against the
    # oracle and the general kernel.
    Hc, es, _ = W.cubic_spin_lattice(16, -1.0, 1.0, seed=29)
    H = Hc.with_values(np.ascontiguousarray(Hc.val.real))
    R = fk.probe_uncorrelated(H.n_rows * H.b_len, 256, fk.RNG(29))
    M = 24
    c = W.fermi_coefficients(M, es, "fermi_energy")
    warp = run_pair(H, es, R, False, prec, M, c, "autodiff")
    general = run_pair(H, es, R, False, prec, M, c, "autodiff", {L.FK_OPT_WARP_ROWS: 0})
    assert mu_err(warp[0], warp[1]) <= TOL_MU[prec]
    assert rel_err(warp[2], warp[3]) <= TOL_D[prec]
    assert rel_err(warp[2], general[2]) <= (1e-5 if prec == "fp32" else 1e-12)
    eng = fk.Engine(False, prec)
    eng.set_H(H, es)
    eng.set_R(R)
    assert eng.get_option(L.FK_OPT_WARP_ROWS) == (0 if prec == "fp64" else 1)
    eng.close()
