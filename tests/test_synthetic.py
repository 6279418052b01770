"""The seeded synthetic inputs of the benchmark workloads (CPU only): the periodic
Voronoi tessellation equals a brute-force nearest-seed search under periodic distance
with the cell index x fastest; the orientations are unit quaternions with w >= 0 whose
rotation matrices are orthonormal; the batched population draws its grids, grain
counts and load cases from the sets the benchmark names."""
import numpy as np


def test_voronoi_is_the_periodic_nearest_seed():
    from solver_cpp_gb300.synthetic import voronoi
    cells, size, ng, seed = (5, 4, 3), np.array([1.0, 0.8, 0.6]), 7, 3
    mat = voronoi(cells, size, ng, seed)
    seeds = np.random.default_rng(seed).random((ng, 3)) * size
    for z in range(cells[2]):
        for y in range(cells[1]):
            for x in range(cells[0]):
                p = (np.array([x, y, z]) + 0.5) * size / np.array(cells)
                d = np.abs(seeds - p)
                d = np.minimum(d, size - d)
                assert mat[x + cells[0] * (y + cells[1] * z)] == np.argmin((d * d).sum(1))


def test_orientations_are_unit_quaternions_with_nonnegative_w():
    from solver_cpp_gb300.synthetic import random_quaternions
    from oracle import dgo
    q = random_quaternions(500, 11)
    assert np.allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-15) and np.all(q[:, 0] >= 0.0)
    for k in range(0, 500, 50):
        R = dgo.qu2om(q[k]).reshape(3, 3, order="F")
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-14) and abs(np.linalg.det(R) - 1.0) < 1e-14


def test_batched_population_draws_from_the_benchmark_sets():
    from solver_cpp_gb300.synthetic import batch_population
    pop = batch_population(64)
    assert {c[0] for c, *_ in pop} <= {8, 16, 32, 48}
    assert all(8 <= ng <= 200 for _, ng, *_ in pop)
    assert {kind for _, _, kind, *_ in pop} <= {"tensionX", "tensionY", "tensionZ", "shearXY"}
    for cells, ng, kind, mat, q in pop[:8]:
        assert mat.size == int(np.prod(cells)) and mat.max() < ng and q.shape == (ng, 4)
    assert batch_population(3)[2][3].tolist() == pop[2][3].tolist()      # seeded: reproducible
