"""Seeded synthetic microstructures for the benchmark and parity workloads.

* grains: periodic Voronoi tessellation -- seed points uniform in the cell box,
  every cell centre takes the material of its nearest seed under periodic
  distance (the construction of DAMASK's seeds.from_random + Grid.from_Voronoi_tessellation,
  reference python/damask/seeds.py:14-47, _grid.py:534-571);
* orientations: uniformly random unit quaternions (w, x, y, z) by Shoemake's
  subgroup algorithm (K. Shoemake, Graphics Gems III, 1992), sign-standardised
  to w >= 0 (reference python/damask/_rotation.py:1111-1139 uses the same method).
The random stream is numpy's PCG64 seeded with the given integer.
"""
import numpy as np


def voronoi(cells, size, n_grains, seed):
    cells = np.asarray(cells, dtype=int)
    size = np.asarray(size, dtype=float)
    rng = np.random.default_rng(seed)
    seeds = rng.random((n_grains, 3)) * size
    grid = [(np.arange(c) + 0.5) * s / c for c, s in zip(cells, size)]
    X, Y, Z = np.meshgrid(*grid, indexing="ij")
    pts = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    try:
        from scipy.spatial import cKDTree
        tree = cKDTree(seeds, boxsize=size)
        _, idx = tree.query(pts)
    except ImportError:  # pragma: no cover - scipy is present on both machines
        best = np.full(len(pts), np.inf); idx = np.zeros(len(pts), dtype=int)
        for g in range(n_grains):
            d = np.abs(pts - seeds[g]); d = np.minimum(d, size - d)
            d2 = (d * d).sum(1)
            m = d2 < best; best[m] = d2[m]; idx[m] = g
    # (x, y, z) -> cell index x fastest
    return np.ascontiguousarray(idx.reshape(cells[0], cells[1], cells[2]).transpose(2, 1, 0).ravel()).astype(np.int32)


def random_quaternions(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.random((n, 3))
    a, b = np.sqrt(1.0 - u[:, 0]), np.sqrt(u[:, 0])
    q = np.stack([np.cos(2 * np.pi * u[:, 2]) * b, np.sin(2 * np.pi * u[:, 1]) * a,
                  np.cos(2 * np.pi * u[:, 1]) * a, np.sin(2 * np.pi * u[:, 2]) * b], axis=1)
    q[q[:, 0] < 0] *= -1.0
    return q


def microstructure(cells, n_grains, seed, size=(1.0, 1.0, 1.0)):
    """(material_at, orientations) for a seeded periodic Voronoi RVE."""
    mat = voronoi(cells, size, n_grains, seed)
    q = random_quaternions(n_grains, seed + 7919)
    return mat, q


# the batched configuration: grids uniform in {8,16,32,48}^3, 8-200 grains, load case
# uniform in tension x / y / z and shear xy (1e-3/s), per-RVE seeds 1000 + k
BATCH_SIZES = (8, 16, 32, 48)
BATCH_KINDS = ("tensionX", "tensionY", "tensionZ", "shearXY")


def batch_member(k, seed=1000):
    """Member k of the batched population: (cells, grains, load kind, material_at, orientations)."""
    rng = np.random.default_rng(seed + k)
    c = int(BATCH_SIZES[rng.integers(len(BATCH_SIZES))])
    ng = int(rng.integers(8, 201))
    kind = BATCH_KINDS[rng.integers(len(BATCH_KINDS))]
    mat, q = microstructure((c, c, c), ng, seed + k)
    return (c, c, c), ng, kind, mat, q


def batch_population(count, seed=1000):
    return [batch_member(k, seed) for k in range(count)]


def batch_member_sizes(count, seed=1000):
    """Grid edge of each member without building the microstructures."""
    return [int(BATCH_SIZES[np.random.default_rng(seed + k).integers(len(BATCH_SIZES))]) for k in range(count)]
