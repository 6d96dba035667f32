"""Seeded synthetic Hamiltonians and probe blocks with the benchmark configs' shapes.

All generators are deterministic for a given numpy seed. Block layouts follow
the reference (BSR, column-major b x b blocks). Energy scales are analytic
bounds on the spectrum widened by 1%:
  square lattice, hopping t, disorder in [-W/2, W/2]:  |E| <= 4|t| + W/2
  cubic lattice with spin blocks, exchange J:           |E| <= 6|t| + |J|
  triangular lattice with spin blocks, exchange J:      |E| <= 6|t| + |J|
"""
import numpy as np

from .engine import EnergyScale, SpMatBsr, expansion_coefficients


def _bsr_from_coo(n_b, b, rows, cols, blocks, complex_values):
    """Sorted BSR with duplicates summed (numpy; same result as SpMatBsr.build)."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    key = rows * n_b + cols
    order = np.argsort(key, kind="stable")
    key = key[order]
    blocks = np.asarray(blocks)[order]
    uniq, first = np.unique(key, return_index=True)
    summed = np.add.reduceat(blocks, first, axis=0) if len(key) else blocks
    r = (uniq // n_b).astype(np.int32)
    c = (uniq % n_b).astype(np.int32)
    row_ptr = np.zeros(n_b + 1, np.int32)
    np.add.at(row_ptr, r + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    dt = np.complex128 if complex_values else np.float64
    return SpMatBsr(n_b, b, row_ptr, c, np.ascontiguousarray(summed, dtype=dt).reshape(-1), complex_values)


def square_lattice(L, t=-1.0, W=1.0, seed=0):
    """L x L periodic square lattice, b = 1 real, nearest-neighbour hopping t and
    on-site disorder uniform in [-W/2, W/2]. Returns (H, es)."""
    rng = np.random.default_rng(seed)
    n = L * L
    idx = np.arange(n)
    x, y = idx % L, idx // L
    nbrs = [((x + 1) % L) + L * y, ((x - 1) % L) + L * y, x + L * ((y + 1) % L), x + L * ((y - 1) % L)]
    rows = np.concatenate([idx] * 5)
    cols = np.concatenate(nbrs + [idx])
    vals = np.concatenate([np.full(n, t)] * 4 + [rng.uniform(-W / 2, W / 2, n)])
    H = _bsr_from_coo(n, 1, rows, cols, vals[:, None], False)
    bound = 4 * abs(t) + W / 2
    return H, EnergyScale(-1.01 * bound, 1.01 * bound)


def _unit_spins(rng, n):
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def _exchange_blocks(J, S):
    """J sigma . S as column-major 2x2 complex blocks: [[Sz, Sx - iSy], [Sx + iSy, -Sz]]."""
    sx, sy, sz = S[:, 0], S[:, 1], S[:, 2]
    blk = np.zeros((len(S), 4), np.complex128)
    blk[:, 0] = J * sz                 # (0,0)
    blk[:, 1] = J * (sx + 1j * sy)     # (1,0)
    blk[:, 2] = J * (sx - 1j * sy)     # (0,1)
    blk[:, 3] = -J * sz                # (1,1)
    return blk


def _spin_lattice(n, nbr_list, t, J, seed):
    rng = np.random.default_rng(seed)
    S = _unit_spins(rng, n)
    idx = np.arange(n)
    hop = np.zeros((n, 4), np.complex128)
    hop[:, 0] = t
    hop[:, 3] = t
    rows = np.concatenate([idx] * (len(nbr_list) + 1))
    cols = np.concatenate(list(nbr_list) + [idx])
    blocks = np.concatenate([hop] * len(nbr_list) + [_exchange_blocks(J, S)])
    H = _bsr_from_coo(n, 2, rows, cols, blocks, True)
    return H, S


def cubic_spin_lattice(L, t=-1.0, J=1.0, seed=0):
    """L^3 periodic cubic Kondo-lattice-style Hamiltonian: 2x2 spin blocks, hopping t I2
    to 6 neighbours, on-site J sigma . S_i with seeded unit spins. Returns (H, es, spins)."""
    n = L ** 3
    idx = np.arange(n)
    x, y, z = idx % L, (idx // L) % L, idx // (L * L)
    site = lambda a, b_, c: (a % L) + L * ((b_ % L) + L * (c % L))
    nbrs = [site(x + 1, y, z), site(x - 1, y, z), site(x, y + 1, z), site(x, y - 1, z), site(x, y, z + 1),
            site(x, y, z - 1)]
    H, S = _spin_lattice(n, nbrs, t, J, seed)
    bound = 6 * abs(t) + abs(J)
    return H, EnergyScale(-1.01 * bound, 1.01 * bound), S


def triangular_spin_lattice(L, t=-1.0, J=2.0, seed=0):
    """L x L periodic triangular lattice (6 neighbours: +-a1, +-a2, +-(a1 - a2)) with 2x2 spin
    blocks, hopping t I2 and exchange J sigma . S_i. Returns (H, es, spins)."""
    n = L * L
    idx = np.arange(n)
    x, y = idx % L, idx // L
    site = lambda a, b_: (a % L) + L * (b_ % L)
    nbrs = [site(x + 1, y), site(x - 1, y), site(x, y + 1), site(x, y - 1), site(x + 1, y - 1), site(x - 1, y + 1)]
    H, S = _spin_lattice(n, nbrs, t, J, seed)
    bound = 6 * abs(t) + abs(J)
    return H, EnergyScale(-1.01 * bound, 1.01 * bound), S


def cubic_colour_groups(L, period=4):
    """Colour of each scalar row of a cubic spin lattice: (x % p, y % p, z % p) x spin."""
    n = L ** 3
    idx = np.arange(n)
    x, y, z = idx % L, (idx // L) % L, idx // (L * L)
    colour = (x % period) + period * ((y % period) + period * (z % period))
    return np.stack([2 * colour, 2 * colour + 1], axis=1).reshape(-1).astype(np.int32)


def square_colour_groups(L, px, py, spin=False):
    """Colour of each scalar row of a square/triangular lattice: (x % px, y % py) [x spin]."""
    n = L * L
    idx = np.arange(n)
    colour = (idx % L % px) + px * (idx // L % py)
    if spin:
        return np.stack([2 * colour, 2 * colour + 1], axis=1).reshape(-1).astype(np.int32)
    return colour.astype(np.int32)


def phase_probes(groups, realisations=1, seed=0, complex_values=True):
    """Correlated probes with seeded uniform unit phases: column r * G + g is nonzero on the
    rows of group g with phase exp(i theta), scaled by 1/sqrt(realisations). Returns a
    Fortran-ordered n x (realisations * G) array."""
    rng = np.random.default_rng(seed)
    groups = np.asarray(groups)
    n = len(groups)
    G = int(groups.max()) + 1
    dt = np.complex128 if complex_values else np.float64
    R = np.zeros((n, realisations * G), dt, order="F")
    rows = np.arange(n)
    for r in range(realisations):
        if complex_values:
            ph = np.exp(2j * np.pi * rng.random(n))
        else:
            ph = rng.choice([-1.0, 1.0], n)
        R[rows, r * G + groups] = ph / np.sqrt(realisations)
    return R


def phase_probe_entries(groups, realisations=1, seed=0, complex_values=True):
    """phase_probes as its nonzeros: (s, cols, vals) with cols, vals of shape (n, realisations), the
    same seeded phases, so that R[i, cols[i, r]] = vals[i, r] is phase_probes(groups, ...)."""
    rng = np.random.default_rng(seed)
    groups = np.asarray(groups)
    n = len(groups)
    G = int(groups.max()) + 1
    cols = np.empty((n, realisations), np.int32)
    vals = np.empty((n, realisations), np.complex128 if complex_values else np.float64)
    for r in range(realisations):
        if complex_values:
            ph = np.exp(2j * np.pi * rng.random(n))
        else:
            ph = rng.choice([-1.0, 1.0], n)
        cols[:, r] = r * G + groups
        vals[:, r] = ph / np.sqrt(realisations)
    return realisations * G, cols, vals


def fermi_coefficients(M, es, kind="fermi_density", kT=0.0, mu=0.0, Mq=None):
    """Jackson-damped zero-temperature Fermi expansion (Mq = 2M unless given)."""
    return expansion_coefficients(M, Mq or 2 * M, kind, kT, mu, es)


# ---------------------------------------------------------------------------
# The five configurations
# ---------------------------------------------------------------------------

def config1(seed=1):
    """2D square lattice L=32, t=-1, disorder U[-0.5, 0.5], b=1 real, es = +-4.5, M=200,
    S=64 uncorrelated +-1 probes (set_R_uncorrelated), zero-T Fermi at mu=0, Mq = 2M."""
    H, _ = square_lattice(32, -1.0, 1.0, seed)
    es = EnergyScale(-4.5, 4.5)
    return dict(H=H, es=es, M=200, S=64, probe_seed=seed, complex_values=False)


def config2(L=64, seed=2, S=256):
    """Cubic L^3 spin lattice, t=-1 I2, J=1 seeded unit spins, b=2 complex, M=1000, S=256:
    colours (x%4, y%4, z%4) x spin = 128 groups, two seeded phase realisations each scaled
    1/sqrt(2). Outputs: moments + autodiff_matrix D on H's pattern."""
    H, es, _ = cubic_spin_lattice(L, -1.0, 1.0, seed)
    groups = cubic_colour_groups(L, 4)
    real = max(1, S // 128)
    return dict(H=H, es=es, M=1000, S=S, groups=groups, realisations=real, probe_seed=seed, complex_values=True)


def config3(L=512, seed=3):
    """Triangular L x L spin lattice, t=-1, J=2, b=2 complex, M=2000, S=128 probes coloured by
    (x%8, y%8) x spin, one phase realisation. FP32 recursion vs the FP64 answer."""
    H, es, _ = triangular_spin_lattice(L, -1.0, 2.0, seed)
    groups = square_colour_groups(L, 8, 8, spin=True)
    return dict(H=H, es=es, M=2000, S=128, groups=groups, realisations=1, probe_seed=seed, complex_values=True)


def config4(n_systems=64, seed=4, M=500, S=32, Lmin=32, Lmax=256):
    """64 square lattices, L ~ U{32..256}, W ~ U[0, 4], t=-1, b=1 real, M=500, S=32 +-1 probes."""
    rng = np.random.default_rng(seed)
    systems = []
    for k in range(n_systems):
        L = int(rng.integers(Lmin, Lmax + 1))
        W = float(rng.uniform(0.0, 4.0))
        H, es = square_lattice(L, -1.0, W, seed * 1000 + k)
        systems.append(dict(H=H, es=es, L=L, W=W, M=M, S=S, probe_seed=seed * 1000 + k))
    return systems
