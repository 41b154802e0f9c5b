"""The oracle's k-nearest-neighbour restatement (save_neighbors,
src/amuse_ph4/src/gpu.cc:534-558, applied to all other particles) against an
independent numpy sort.  The reference's own caller, get_densities_on_gpu,
needs sapporo's GPU neighbour lists and is never called by ph4
(jdata.cc:1063-1065), so it cannot be run here."""
import numpy as np

import oracle
from amuse_gb300 import ic


def _numpy_knn(pos, k, slots):
    out_j, out_d = [], []
    for i in slots:
        d = pos[i] - pos
        r = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        idx = np.arange(len(pos))
        keep = idx != i
        order = np.lexsort((idx[keep], r[keep]))[:k]
        j = idx[keep][order]
        dd = r[keep][order]
        pad = k - len(j)
        out_j.append(np.concatenate([j, -np.ones(pad, int)]))
        out_d.append(np.concatenate([dd, np.full(pad, np.inf)]))
    return np.array(out_j), np.array(out_d)


def test_knn_plummer_matches_numpy():
    rng = np.random.RandomState(3)
    _, x, _ = ic.plummer(1500, rng=rng)
    slots = rng.choice(1500, 200, replace=False)
    j, d = oracle.knn(x, 12, slots)
    nj, nd = _numpy_knn(x, 12, slots)
    assert np.array_equal(j, nj) and np.array_equal(d, nd)


def test_knn_lattice_ties_to_smaller_index():
    g = np.arange(6) * 0.25
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) + 100.0
    j, d = oracle.knn(x, 20)
    nj, nd = _numpy_knn(x, 20, np.arange(len(x)))
    assert np.array_equal(j, nj) and np.array_equal(d, nd)
    assert d[0, 0] == 0.0625 and d[0, 1] == 0.0625     # exact ties on the lattice


def test_knn_fewer_particles_than_k():
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 2.0, 0]])
    j, d = oracle.knn(x, 4)
    assert j[0].tolist() == [1, 2, -1, -1] and d[0, 2] == np.inf
