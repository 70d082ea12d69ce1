"""Seeded synthetic point sets for the five measured configurations.

Generator: splitmix64 (state_k = seed + k * 0x9E3779B97F4A7C15, mixed), and a
uniform f64 in [0, 1) is (x >> 11) * 2^-53.  Seeds are 0xD1A00000 + config
number.  No public dataset exists for this path; these stand in with the
shapes, sizes and distributions the configurations name.

  C1  2D, N = 10,000 uniform in [0,1)^2
  C2  3D, N = 1,000,000 uniform in [0,1)^3
  C3  3D, N = 262,144: half on a 64^3 lattice (i/64, distinct sites) with
      uniform jitter of +-1e-12 per coordinate, half from 64 isotropic
      Gaussians (centres uniform in the cube, sigma = 0.01, not clipped)
  C4  4,096 independent 3D sets, sizes floor(exp(U(ln 32, ln 65536)))
  C5  20,000 requests, 2D/3D at 50/50, sizes log-uniform in [100, 200000]
"""
import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
C1 = np.uint64(0xBF58476D1CE4E5B9)
C2 = np.uint64(0x94D049BB133111EB)
SEED_BASE = 0xD1A00000


def splitmix64(seed, n, offset=0):
    """n consecutive outputs of splitmix64 starting after `offset` draws."""
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * GOLDEN
        z = (z ^ (z >> np.uint64(30))) * C1
        z = (z ^ (z >> np.uint64(27))) * C2
        return z ^ (z >> np.uint64(31))


def uniform01(seed, n, offset=0):
    return (splitmix64(seed, n, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def uniform_points(n, dim, seed):
    return uniform01(seed, n * dim).reshape(n, dim)


def config_seed(k):
    return SEED_BASE + k


def c1_points():
    return uniform_points(10_000, 2, config_seed(1))


def c2_points(n=1_000_000):
    return uniform_points(n, 3, config_seed(2))


def c3_points(n=262_144, seed=None):
    """Near-degenerate mix: jittered lattice sites + tight Gaussian clusters."""
    seed = config_seed(3) if seed is None else seed
    half = n // 2
    side = 64
    sites = side ** 3
    # distinct lattice sites: the `half` smallest random keys
    keys = splitmix64(seed, sites)
    pick = np.argsort(keys, kind="stable")[:half]
    ijk = np.stack([pick // (side * side), (pick // side) % side, pick % side], axis=1)
    jit = (uniform01(seed, half * 3, offset=sites) * 2.0 - 1.0) * 1e-12
    lattice = ijk.astype(np.float64) / side + jit.reshape(half, 3)
    off = sites + half * 3
    centres = uniform01(seed, 64 * 3, offset=off).reshape(64, 3)
    off += 64 * 3
    m = n - half
    comp = (splitmix64(seed, m, offset=off) % np.uint64(64)).astype(np.int64)
    off += m
    u1 = uniform01(seed, m * 3, offset=off)
    off += m * 3
    u2 = uniform01(seed, m * 3, offset=off)
    u1 = np.maximum(u1, 2.0 ** -53)
    g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)  # Box-Muller
    gauss = centres[comp] + 0.01 * g.reshape(m, 3)
    return np.concatenate([lattice, gauss], axis=0)


def c4_sizes(nsets=4096, lo=32, hi=65536, seed=None):
    seed = config_seed(4) if seed is None else seed
    u = uniform01(seed, nsets)
    return np.floor(np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))).astype(np.int64)


def c4_sets(nsets=4096, seed=None):
    seed = config_seed(4) if seed is None else seed
    sizes = c4_sizes(nsets, seed=seed)
    offsets = np.concatenate([[0], np.cumsum(sizes)])
    pts = uniform01(seed, int(offsets[-1]) * 3, offset=nsets).reshape(-1, 3)
    return pts, offsets


def lattice_points(side, dim, jitter=0.0, seed=7):
    """Exact integer lattice (all sites), optionally jittered: a degenerate stress case."""
    axes = [np.arange(side, dtype=np.float64)] * dim
    g = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, dim)
    if jitter:
        g = g + (uniform01(seed, g.size).reshape(g.shape) * 2 - 1) * jitter
    return g


def c5_requests(nreq=20_000, lo=100, hi=200_000, seed=None):
    """Serving stream: per request (dim, n, point seed); dims 2/3 at 50/50,
    sizes floor(exp(U(ln lo, ln hi)))."""
    seed = config_seed(5) if seed is None else seed
    u = uniform01(seed, 2 * nreq).reshape(nreq, 2)
    dims = np.where(u[:, 0] < 0.5, 2, 3)
    sizes = np.floor(np.exp(np.log(lo) + u[:, 1] * (np.log(hi) - np.log(lo)))).astype(np.int64)
    return [(int(d), int(n), seed * 1_000_003 + i) for i, (d, n) in enumerate(zip(dims, sizes))]


def c5_points(req):
    dim, n, s = req
    return uniform_points(n, dim, s)
