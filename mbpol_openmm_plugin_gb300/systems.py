"""Seeded synthetic water systems (no dataset is used anywhere).

Monomers: O-H 0.9572 A and H-O-H 104.52 deg, each bond jittered by
N(0, 0.01 A) and the angle by N(0, 2 deg), uniformly random orientation; the
M site is placed with the MB-pol weights (python/mbpol.xml:14).
Particles are laid out per water as O, H1, H2, M (nm).

Workloads (sizes as used by the tests and the benchmark):
  cluster14   14 waters, O inside a 4.5 A sphere, min O-O 2.6 A, non-periodic
  box256      256 waters, cubic box 19.73 A, jittered 7x7x6 lattice (first 256 sites)
  clusters    4096 clusters, n ~ U[2, 64], radius 2.0*n^(1/3) A
  box4096     4096 waters, cubic box 49.67 A, jittered 16^3 lattice
  box32768    32768 waters, cubic box 99.34 A, jittered 32^3 lattice
Lattice jitter: uniform +-0.3 A per coordinate, minimum O-O 2.5 A (redrawn).
"""
from dataclasses import dataclass, field
import numpy as np

M_WEIGHTS = (0.573293118, 0.213353441, 0.213353441)  # python/mbpol.xml:14
ROH, THETA = 0.9572, np.deg2rad(104.52)


@dataclass
class WaterSystem:
    positions: np.ndarray          # (4*nw, 3) nm, O,H1,H2,M per water
    box: np.ndarray | None         # (3,) nm or None
    seed: int
    name: str
    cluster_of_water: np.ndarray | None = None  # (nw,) cluster id, for batched clusters
    meta: dict = field(default_factory=dict)

    @property
    def num_waters(self):
        return self.positions.shape[0] // 4

    def water_indices(self):
        """(nw, 3) particle indices O, H1, H2."""
        base = 4 * np.arange(self.num_waters)
        return np.stack([base, base + 1, base + 2], axis=1).astype(np.int32)


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def monomer(rng, center_A):
    r1 = ROH + rng.normal(0, 0.01)
    r2 = ROH + rng.normal(0, 0.01)
    th = THETA + np.deg2rad(rng.normal(0, 2.0))
    h1 = np.array([r1 * np.sin(th / 2), 0.0, r1 * np.cos(th / 2)])
    h2 = np.array([-r2 * np.sin(th / 2), 0.0, r2 * np.cos(th / 2)])
    R = _random_rotation(rng)
    o = np.asarray(center_A, dtype=float)
    h1 = o + R @ h1
    h2 = o + R @ h2
    m = M_WEIGHTS[0] * o + M_WEIGHTS[1] * h1 + M_WEIGHTS[2] * h2
    return np.stack([o, h1, h2, m]) * 0.1  # nm


def _min_image(d, L):
    return d - L * np.round(d / L)


def sphere_oxygens(rng, n, radius, dmin):
    pts = []
    tries = 0
    while len(pts) < n:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place %d oxygens in r=%.2f" % (n, radius))
        p = rng.uniform(-radius, radius, 3)
        if p @ p > radius * radius:
            continue
        if pts and np.min(np.linalg.norm(np.asarray(pts) - p, axis=1)) < dmin:
            continue
        pts.append(p)
    return np.asarray(pts)


def cluster(n, seed=0, radius=None, dmin=2.6):
    rng = np.random.default_rng(seed)
    radius = 4.5 if radius is None else radius
    oxy = sphere_oxygens(rng, n, radius, dmin)
    pos = np.concatenate([monomer(rng, o) for o in oxy])
    return WaterSystem(pos, None, seed, "cluster%d" % n)


def lattice_box(nx, ny, nz, L_A, n, seed=0, jitter=0.3, dmin=2.5):
    rng = np.random.default_rng(seed)
    sp = np.array([L_A / nx, L_A / ny, L_A / nz])
    sites = np.array([[i, j, k] for i in range(nx) for j in range(ny) for k in range(nz)], float)[:n]
    sites = (sites + 0.5) * sp
    oxy = sites.copy()
    L = np.array([L_A] * 3)
    for i in range(n):
        for _ in range(1000):
            cand = sites[i] + rng.uniform(-jitter, jitter, 3)
            if i == 0:
                break
            d = _min_image(oxy[:i] - cand, L)
            if np.min(np.sqrt((d * d).sum(1))) >= dmin:
                break
        oxy[i] = cand
    pos = np.concatenate([monomer(rng, o) for o in oxy])
    return WaterSystem(pos, L * 0.1, seed, "box%d" % n)


def batched_clusters(nclusters=4096, nmin=2, nmax=64, seed=0):
    """Independent clusters with n ~ U[nmin, nmax] and radius 2.0*n^(1/3) A,
    each centred 100 nm apart along x (they never interact)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=nclusters)
    pos, cid = [], []
    for c, n in enumerate(sizes):
        sub = cluster(int(n), seed=int(rng.integers(1 << 31)), radius=2.0 * n ** (1.0 / 3.0), dmin=2.5)
        p = sub.positions.copy()
        p[:, 0] += 100.0 * c
        pos.append(p)
        cid += [c] * int(n)
    return WaterSystem(np.concatenate(pos), None, seed, "clusters%d" % nclusters,
                       cluster_of_water=np.asarray(cid, np.int32), meta={"sizes": sizes})


def workload(name, seed=0):
    if name == "cluster14":
        return cluster(14, seed)
    if name == "box256":
        return lattice_box(7, 7, 6, 19.73, 256, seed)
    if name == "box4096":
        return lattice_box(16, 16, 16, 49.67, 4096, seed)
    if name == "box32768":
        return lattice_box(32, 32, 32, 99.34, 32768, seed)
    if name == "clusters":
        return batched_clusters(seed=seed)
    raise KeyError(name)
