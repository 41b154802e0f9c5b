"""g6x_knn (the neighbour lists of ph4's get_densities_on_gpu,
src/amuse_ph4/src/gpu.cc:568-866, reduced as save_neighbors does,
gpu.cc:534-558) against the oracle's restatement: exact ids and squared
distances, ties to the smaller slot."""
import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from amuse_gb300 import ic

pytestmark = pytest.mark.gpu


def _check(ids, d2, ref_j, ref_d):
    ref_ids = np.where(ref_j >= 0, ref_j + 1, -1)
    assert np.array_equal(ids, ref_ids)
    assert np.array_equal(d2, ref_d)


def test_knn_all_particles_plummer(g6):
    rng = np.random.RandomState(5)
    m, x, v = ic.plummer(4096, rng=rng)
    g6.load_particles(m, x, v)
    ids, d2 = g6.knn(4096, k=12)
    _check(ids, d2, *oracle.knn(x, 12))


def test_knn_subset_large_n_k32(g6):
    rng = np.random.RandomState(6)
    m, x, v = ic.plummer(65536, rng=rng)
    g6.load_particles(m, x, v)
    slots = rng.choice(65536, 384, replace=False)
    ids, d2 = g6.knn(65536, k=32, slots=slots)
    _check(ids, d2, *oracle.knn(x, 32, slots))


def test_knn_lattice_ties_far_from_origin(g6):
    """Exact ties everywhere and coordinates near 1000 (the FP32 filter's
    slack grows with the largest coordinate)."""
    g = np.arange(16) * 0.0625
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) + 1000.0
    n = len(x)
    g6.load_particles(np.full(n, 1.0 / n), x, np.zeros_like(x))
    ids, d2 = g6.knn(n, k=26)
    _check(ids, d2, *oracle.knn(x, 26))


def test_knn_predicted_positions(g6):
    """Particles at different times, neighbours at t = 0.01 from ph4's
    predictor."""
    rng = np.random.RandomState(7)
    n = 2048
    m, x, v = ic.plummer(n, rng=rng)
    a = rng.normal(size=(n, 3))
    j = rng.normal(size=(n, 3))
    t = rng.randint(0, 4, n) * 2.0 ** -10
    g6.load_particles(m, x, v, acc=a, jerk=j, t=t, dt=np.full(n, 2.0 ** -10))
    ids, d2 = g6.knn(n, k=12, t=0.01)
    pp, _ = oracle.predict(0.01, t, x, v, a, j)
    _check(ids, d2, *oracle.knn(pp, 12))


def test_knn_edges(g6):
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 2.0, 0], [0, 0, 3.0], [4.0, 0, 0]])
    g6.load_particles(np.full(5, 0.2), x, np.zeros_like(x))
    ids, d2 = g6.knn(5, k=12)
    assert ids[0, :4].tolist() == [2, 3, 4, 5] and np.all(ids[:, 4:] == -1)
    assert np.all(np.isinf(d2[:, 4:])) and d2[0, 0] == 1.0
    for k in (0, 33):
        with pytest.raises(ag.G6Error):
            g6.knn(5, k=k)
    with pytest.raises(ag.G6Error):
        g6.knn(5, k=2, slots=[7])
