"""fk_moments_noalloc -- moments for callers that cannot allocate device memory --
against the engine's fk_engine_moments, both through the C ABI.

Such callers hold all their device memory through another allocator (a host
application's pool, or a fixed reservation made at start-up), or must not
trigger cudaFree's device-wide synchronisation while their other streams run;
they pass every buffer themselves. Here torch plays that caller and owns the
buffers. Tolerance: max_m |mu_m - mu_m^ref| / |mu_0^ref| <= 1e-10 (the FP64
tolerance of the other GPU tests), checked on two calls in a row, since every
call reuses the library's static scratch array.
"""
import ctypes as C

import numpy as np
import pytest

import fastkpm_gb300 as fk
from fastkpm_gb300 import _lib as L
from fastkpm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-10


def scaled_values(H, es):
    """Hs = (H - avg I)/mag on H's pattern (every row of these lattices stores its diagonal block)."""
    b = H.b_len
    v = H.val.copy().reshape(-1, b * b)
    diag = np.nonzero(H.row_idx == H.col_idx)[0]
    assert len(diag) == H.n_rows
    for q in range(b):
        v[diag, q * b + q] -= es.avg()
    return (v / es.mag()).reshape(-1)


def two_orbital_square(L_, seed):
    """Real b=2 Hamiltonian: L x L periodic square lattice with two orbitals per site, hopping
    -I2 to the 4 neighbours and a random real symmetric 2x2 on-site block; es from the dense
    spectrum widened by 1%."""
    rng = np.random.default_rng(seed)
    n = L_ * L_
    idx = np.arange(n)
    x, y = idx % L_, idx // L_
    nbrs = [((x + 1) % L_) + L_ * y, ((x - 1) % L_) + L_ * y, x + L_ * ((y + 1) % L_), x + L_ * ((y - 1) % L_)]
    hop = np.tile(np.array([-1.0, 0.0, 0.0, -1.0]), (n, 1))
    e = rng.uniform(-1.0, 1.0, (n, 3))
    onsite = np.stack([e[:, 0], e[:, 2], e[:, 2], e[:, 1]], axis=1)   # column-major [[e0, v], [v, e1]]
    H = W._bsr_from_coo(n, 2, np.concatenate([idx] * 5), np.concatenate(nbrs + [idx]),
                        np.concatenate([hop] * 4 + [onsite]), False)
    lam = np.linalg.eigvalsh(H.to_dense())
    w = 0.01 * (lam[-1] - lam[0])
    return H, fk.EnergyScale(lam[0] - w, lam[-1] + w)


def run_noalloc(lib, torch, H, es, R, M, cplx, stream=None):
    dev = torch.device("cuda:0")
    n, s = R.shape
    epp = 1 if cplx else 2
    ld = (s + epp - 1) // epp * epp
    Rr = np.zeros((n, ld), np.complex128 if cplx else np.float64)
    Rr[:, :s] = R
    hv = scaled_values(H, es)
    as_f64 = (lambda a: np.ascontiguousarray(a).view(np.float64)) if cplx else (lambda a: np.ascontiguousarray(a, np.float64))
    d_rp = torch.from_numpy(H.row_ptr.copy()).to(dev)
    d_ci = torch.from_numpy(H.col_idx.copy()).to(dev)
    d_hv = torch.from_numpy(as_f64(hv).copy()).to(dev)
    d_R = torch.from_numpy(as_f64(Rr).reshape(-1).copy()).to(dev)
    d_work = torch.zeros(2 * n * ld * (2 if cplx else 1), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    outs = []
    for _ in range(2):   # two calls in a row on the shared scratch
        mu = np.zeros(M)
        st = lib.fk_moments_noalloc(L.FK_COMPLEX if cplx else L.FK_REAL, H.n_rows, H.b_len, d_rp.data_ptr(),
                                    d_ci.data_ptr(), d_hv.data_ptr(), ld, s, d_R.data_ptr(), d_work.data_ptr(), M,
                                    mu.ctypes.data_as(C.POINTER(C.c_double)), stream)
        assert st == L.FK_OK, st
        outs.append(mu)
    return outs, (d_rp, d_ci, d_hv, d_R, d_work, ld)


def case(kind):
    if kind == "complex b=2":
        H, es, _ = W.cubic_spin_lattice(4, -1.0, 1.0, seed=5)
        return H, es, W.phase_probes(W.cubic_colour_groups(4, 2), realisations=1, seed=5), True
    if kind == "real b=2":
        H, es = two_orbital_square(8, seed=7)
        return H, es, fk.probe_uncorrelated(2 * H.n_rows, 24, fk.RNG(7)), False
    H, es = W.square_lattice(16, -1.0, 1.0, seed=3)
    return H, es, fk.probe_uncorrelated(H.n_rows, 32, fk.RNG(3)), False


def engine_moments(H, es, R, cplx, M):
    eng = fk.Engine(cplx, "fp64")
    eng.set_H(H, es)
    eng.set_R(R)
    ref = eng.moments(M)
    eng.close()
    return ref


@pytest.mark.parametrize("kind", ["real b=1", "real b=2", "complex b=2"])
def test_noalloc_moments_match_engine(gpu, kind):
    torch = pytest.importorskip("torch")
    lib = L.load()
    H, es, R, cplx = case(kind)
    M = 60
    ref = engine_moments(H, es, R, cplx, M)
    outs, _ = run_noalloc(lib, torch, H, es, R, M, cplx)
    for mu in outs:
        assert np.max(np.abs(mu - ref)) / abs(ref[0]) <= TOL


def test_noalloc_on_a_non_blocking_caller_stream(gpu):
    # a torch side stream (created non-blocking): the launch tables are written on that stream,
    # ordered before the first step without any legacy-stream operation
    torch = pytest.importorskip("torch")
    lib = L.load()
    H, es, R, cplx = case("complex b=2")
    M = 40
    ref = engine_moments(H, es, R, cplx, M)
    side = torch.cuda.Stream()
    outs, _ = run_noalloc(lib, torch, H, es, R, M, cplx, stream=side.cuda_stream)
    for mu in outs:
        assert np.max(np.abs(mu - ref)) / abs(ref[0]) <= TOL


def test_noalloc_rejects_a_misaligned_value_buffer(gpu):
    # complex H values are read as 16-byte elements: a buffer 8 bytes off is refused before any launch
    torch = pytest.importorskip("torch")
    lib = L.load()
    H, es, R, cplx = case("complex b=2")
    _, (d_rp, d_ci, d_hv, d_R, d_work, ld) = run_noalloc(lib, torch, H, es, R, 10, cplx)
    mu = np.zeros(10)
    st = lib.fk_moments_noalloc(L.FK_COMPLEX, H.n_rows, 2, d_rp.data_ptr(), d_ci.data_ptr(), d_hv.data_ptr() + 8, ld,
                                R.shape[1], d_R.data_ptr(), d_work.data_ptr(), 10,
                                mu.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert st == L.FK_ERR_ARG


def test_noalloc_rejects_sizes_beyond_its_limits(gpu):
    torch = pytest.importorskip("torch")
    lib = L.load()
    H, es = W.square_lattice(6, -1.0, 1.0, seed=1)
    R = fk.probe_uncorrelated(H.n_rows, 8, fk.RNG(1))
    _, (d_rp, d_ci, d_hv, d_R, d_work, ld) = run_noalloc(lib, torch, H, es, R, 10, False)
    mu = np.zeros(32770)
    args = lambda M: (L.FK_REAL, H.n_rows, 1, d_rp.data_ptr(), d_ci.data_ptr(), d_hv.data_ptr(), ld, 8,
                      d_R.data_ptr(), d_work.data_ptr(), M, mu.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert lib.fk_moments_noalloc(*args(32770)) == L.FK_ERR_UNSUPPORTED   # beyond the static scratch
    assert lib.fk_moments_noalloc(*args(7)) == L.FK_ERR_ARG               # odd M
    assert lib.fk_moments_noalloc(*args(32768)) == L.FK_OK                # the largest M it holds
