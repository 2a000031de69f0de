"""Seeded synthetic trajectories with the shapes of the all-pairs RMSD workloads.

No public dataset is named for this path, so these generators stand in for
real trajectories.  A reference chain is a 3-D random walk with 3.8 Angstrom
steps (Gaussian direction, normalised).  Each frame is the chain plus i.i.d.
Gaussian displacement, then a uniformly random rotation (normalised Gaussian
quaternion) and a translation drawn from U[-20, 20]^3.
"""
from __future__ import annotations

import numpy as np

#: Element masses and their probabilities used for mass-weighted workloads
#: (H, C, N, O, S).
MASS_VALUES = np.array([1.008, 12.011, 14.007, 15.999, 32.06])
MASS_PROBS = np.array([0.50, 0.32, 0.09, 0.08, 0.01])


def random_walk(rng: np.random.Generator, n_atom: int, step: float = 3.8) -> np.ndarray:
    """Return an (n_atom, 3) random-walk chain with fixed step length."""
    d = rng.standard_normal((n_atom, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[0] = 0.0
    return np.cumsum(d * step, axis=0)


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from normalised Gaussian quaternions."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    a, b, c, d = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = a * a + b * b - c * c - d * d
    R[:, 0, 1] = 2 * (b * c - a * d)
    R[:, 0, 2] = 2 * (b * d + a * c)
    R[:, 1, 0] = 2 * (b * c + a * d)
    R[:, 1, 1] = a * a - b * b + c * c - d * d
    R[:, 1, 2] = 2 * (c * d - a * b)
    R[:, 2, 0] = 2 * (b * d - a * c)
    R[:, 2, 1] = 2 * (c * d + a * b)
    R[:, 2, 2] = a * a - b * b - c * c + d * d
    return R


def perturb_frames(rng, chains, labels, sigma):
    """chains[labels[f]] + N(0, sigma[f]^2), rotated and translated."""
    n_frame = len(labels)
    n_atom = chains.shape[1]
    X = chains[labels] + rng.standard_normal((n_frame, n_atom, 3)) * sigma[:, None, None]
    R = random_rotations(rng, n_frame)
    X = np.einsum("fij,faj->fai", R, X)
    X += rng.uniform(-20.0, 20.0, (n_frame, 1, 3))
    return X


def masses(rng: np.random.Generator, n_atom: int) -> np.ndarray:
    return rng.choice(MASS_VALUES, size=n_atom, p=MASS_PROBS)


def trajectory(seed: int, n_frame: int, n_atom: int, sigma_lo: float, sigma_hi: float,
               dtype=np.float32, weighted: bool = False):
    """One chain, per-frame sigma ~ U(sigma_lo, sigma_hi).

    Returns (coords[n_frame, n_atom, 3] of ``dtype``, masses[n_atom] float64 or None).
    """
    rng = np.random.default_rng(seed)
    chain = random_walk(rng, n_atom)[None]
    sigma = rng.uniform(sigma_lo, sigma_hi, n_frame)
    X = perturb_frames(rng, chain, np.zeros(n_frame, dtype=np.int64), sigma)
    m = masses(rng, n_atom) if weighted else None
    return np.ascontiguousarray(X.astype(dtype)), m


def clustered(seed: int, n_frame: int, n_atom: int, n_centroid: int = 20, sigma: float = 0.8,
              dtype=np.float32):
    """Frames drawn around ``n_centroid`` random-walk centroids.

    Returns (coords, labels) where labels[f] is the centroid index of frame f.
    """
    rng = np.random.default_rng(seed)
    chains = np.stack([random_walk(rng, n_atom) for _ in range(n_centroid)])
    labels = rng.integers(0, n_centroid, n_frame)
    X = perturb_frames(rng, chains, labels, np.full(n_frame, sigma))
    return np.ascontiguousarray(X.astype(dtype)), labels


def md_like(seed: int, n_frame: int, n_atom: int, amp: float = 1.0, tau: float = 50.0,
            dtype=np.float32, weighted: bool = False):
    """Time-correlated trajectory: chain + an Ornstein-Uhlenbeck displacement
    field (stationary amplitude ``amp`` per coordinate, correlation time
    ``tau`` frames), each frame rotated and translated.  Consecutive frames
    are near-duplicates, the hard case for cancellation in E0 - lambda."""
    rng = np.random.default_rng(seed)
    chain = random_walk(rng, n_atom)
    a = np.exp(-1.0 / tau)
    u = rng.standard_normal((n_atom, 3)) * amp
    X = np.empty((n_frame, n_atom, 3))
    for f in range(n_frame):
        u = a * u + np.sqrt(1 - a * a) * amp * rng.standard_normal((n_atom, 3))
        X[f] = chain + u
    R = random_rotations(rng, n_frame)
    X = np.einsum("fij,faj->fai", R, X) + rng.uniform(-20.0, 20.0, (n_frame, 1, 3))
    m = masses(rng, n_atom) if weighted else None
    return np.ascontiguousarray(X.astype(dtype)), m


def near_duplicates(seed: int, n_centroid: int, n_base: int, n_copy: int, n_atom: int, resid: float = 3.0,
                    dup: float = 0.01, dtype=np.float32, weighted: bool = True):
    """Stress case for the per-pair error bound: groups of near-identical
    frames far from any pre-alignment reference.  ``n_centroid`` random-walk
    centroids; around each, ``n_base`` base structures displaced from it by
    an RMS of ``resid`` Angstrom; each base repeated ``n_copy`` times with a
    further RMS displacement of ``dup`` Angstrom (copies of one base are
    ~dup*sqrt(2) apart).  Every frame is randomly rotated and translated and
    the frame order is shuffled.  Returns (coords, masses or None, base index
    per frame)."""
    rng = np.random.default_rng(seed)
    chains = np.stack([random_walk(rng, n_atom) for _ in range(n_centroid)])
    n_b = n_centroid * n_base
    base = chains[np.repeat(np.arange(n_centroid), n_base)]
    base = base + rng.standard_normal((n_b, n_atom, 3)) * (resid / np.sqrt(3.0))
    bidx = np.repeat(np.arange(n_b), n_copy)
    X = base[bidx] + rng.standard_normal((n_b * n_copy, n_atom, 3)) * (dup / np.sqrt(3.0))
    R = random_rotations(rng, len(X))
    X = np.einsum("fij,faj->fai", R, X) + rng.uniform(-20.0, 20.0, (len(X), 1, 3))
    perm = rng.permutation(len(X))
    m = masses(rng, n_atom) if weighted else None
    return np.ascontiguousarray(X[perm].astype(dtype)), m, bidx[perm]


# Named workloads ---------------------------------------------------------------------------

def workload_c0(seed: int = 0, n_frame: int = 500, n_atom: int = 304):
    """rms2d fit, 500 frames x 304 atoms, FP64, unweighted, sigma ~ U(0.5, 2.0)."""
    X, _ = trajectory(seed, n_frame, n_atom, 0.5, 2.0, dtype=np.float64, weighted=False)
    return X, None


def workload_c1(seed: int = 1, n_frame: int = 10000, n_atom: int = 2000):
    """10,000 frames x 2,000 atoms, FP32, mass-weighted, sigma ~ U(0.1, 3.0)."""
    return trajectory(seed, n_frame, n_atom, 0.1, 3.0, dtype=np.float32, weighted=True)


def workload_c2(seed: int = 2, n_frame: int = 50000, n_atom: int = 500):
    """Clustering cache: 50,000 frames x 500 atoms around 20 centroids, sigma 0.8."""
    return clustered(seed, n_frame, n_atom, 20, 0.8, dtype=np.float32)


def trajectory_f32(seed: int, n_frame: int, n_atom: int, sigma_lo: float, sigma_hi: float,
                   weighted: bool = True):
    """The frames of ``trajectory`` generated in float32 throughout (same
    distributions, different draws): about 20x faster for multi-GB batches.
    Returns (coords float32 [n_frame, n_atom, 3], masses or None)."""
    rng = np.random.default_rng(seed)
    chain = random_walk(rng, n_atom).astype(np.float32)
    sigma = rng.uniform(sigma_lo, sigma_hi, n_frame).astype(np.float32)
    X = rng.standard_normal((n_frame, n_atom, 3), dtype=np.float32)
    X *= sigma[:, None, None]
    X += chain[None]
    R = random_rotations(rng, n_frame).astype(np.float32)
    X = np.matmul(X, R.transpose(0, 2, 1))
    X += rng.uniform(-20.0, 20.0, (n_frame, 1, 3)).astype(np.float32)
    m = masses(rng, n_atom) if weighted else None
    return np.ascontiguousarray(X), m


def workload_c3(seed: int = 3, n_traj: int = 256, f_range=(100, 4000), n_range=(50, 3000), threads: int = 8):
    """Batch of independent trajectories with random frame/atom counts,
    mass-weighted (about 9.4 GB of FP32 frames at the default sizes, generated
    in float32 on ``threads`` host threads, one seed per trajectory)."""
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.default_rng(seed)
    specs = []
    for t in range(n_traj):
        nf = int(rng.integers(f_range[0], f_range[1] + 1))
        na = int(rng.integers(n_range[0], n_range[1] + 1))
        specs.append((seed * 100003 + t, nf, na))
    with ThreadPoolExecutor(max(1, threads)) as ex:
        return list(ex.map(lambda s: trajectory_f32(s[0], s[1], s[2], 0.1, 3.0, True), specs))


def workload_c4(seed: int = 4, n_frame: int = 4096, n_atom: int = 1000):
    """Differentiation workload: 4,096 frames x 1,000 atoms, sigma 1.0, unweighted."""
    X, _ = trajectory(seed, n_frame, n_atom, 1.0, 1.0, dtype=np.float32, weighted=False)
    return X, None
