"""Batched few-body systems (config 4 shape: n ~ U[3, 64], Plummer with
virial radius 1e-3, eps = 0) in one persistent kernel, against smallN's
integrator restated in the oracle (itself bit-identical to smallN built from
the reference sources with dt_crit = 0, tests/test_batch_oracle.py)."""
import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from amuse_gb300 import ic

pytestmark = pytest.mark.gpu


def _systems(nsys, nmin, nmax, seed):
    ns, m, x, v, tcr = ic.encounter_batch(nsys, nmin, nmax, seed=seed)
    return ns, m, x, v, tcr


def test_exact_mode_is_bit_identical_to_smalln(g6):
    ns, m, x, v, tcr = _systems(24, 3, 40, seed=5)
    t_end = np.full(len(ns), 1.0 * tcr)
    r = g6.batch_run(ns, t_end, m, x, v, eta=0.14, exact=True)
    off = np.concatenate([[0], np.cumsum(ns)])
    for s in range(len(ns)):
        a, b = off[s], off[s + 1]
        px, pv, tf, st = oracle.smalln(m[a:b], x[a:b], v[a:b], 0.14, t_end[s])
        assert r["status"][s] == 0
        assert r["steps"][s] == st, s
        assert r["t_final"][s] == tf, s
        assert np.array_equal(r["pos"][a:b], px), s
        assert np.array_equal(r["vel"][a:b], pv), s


def test_exact_mode_matches_reference_smalln_fixtures(g6):
    """Against smallN built from the reference sources (tests/golden/
    smalln_systems.npz): n = 3 ... 64, two crossing times, bit for bit."""
    from conftest import golden
    g = golden("smalln_systems.npz")
    k = int(g["nsys"])
    ns = np.array([len(g[f"s{i}_mass"]) for i in range(k)], np.int32)
    cat = lambda key: np.concatenate([g[f"s{i}_{key}"] for i in range(k)])
    t_end = np.full(k, float(g["t_end"]))
    r = g6.batch_run(ns, t_end, cat("mass"), cat("pos0"), cat("vel0"), eta=float(g["eta"]),
                     exact=True)
    assert np.array_equal(r["pos"], cat("pos")) and np.array_equal(r["vel"], cat("vel"))
    assert np.array_equal(r["t_final"], np.array([float(g[f"s{i}_t"]) for i in range(k)]))


def _energy(m, x, v):
    k = 0.5 * np.sum(m * np.sum(v * v, 1))
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt(np.sum(d * d, -1))
    iu = np.triu_indices(len(m), 1)
    return k - np.sum(m[iu[0]] * m[iu[1]] / r[iu])


def test_fast_mode_conserves_energy_like_exact(g6):
    ns, m, x, v, tcr = _systems(64, 3, 64, seed=6)
    t_end = np.full(len(ns), 2.0 * tcr)
    fast = g6.batch_run(ns, t_end, m, x, v, exact=False)
    exact = g6.batch_run(ns, t_end, m, x, v, exact=True)
    off = np.concatenate([[0], np.cumsum(ns)])
    de_f, de_e = [], []
    for s in range(len(ns)):
        a, b = off[s], off[s + 1]
        e0 = _energy(m[a:b], x[a:b], v[a:b])
        de_f.append(abs((_energy(m[a:b], fast["pos"][a:b], fast["vel"][a:b]) - e0) / e0))
        de_e.append(abs((_energy(m[a:b], exact["pos"][a:b], exact["vel"][a:b]) - e0) / e0))
    print(f"median |dE/E| fast {np.median(de_f):.2e} exact {np.median(de_e):.2e}; "
          f"max fast {max(de_f):.2e} exact {max(de_e):.2e}")
    assert np.all(fast["status"] == 0) and np.all(fast["t_final"] >= t_end)
    # the scheme's own truncation error dominates: both modes agree on it
    assert np.median(de_f) < 2 * np.median(de_e) + 1e-12
    assert max(de_f) < 3 * max(de_e) + 1e-12


def test_split_mode_energy_and_short_time_agreement(g6):
    """Split mode (FP32 pair terms from double-single positions): over two
    crossing times its energy error stays at the scheme's truncation level
    (within 10x of exact mode, or 1e-7), and over a short time, before the
    systems' chaos amplifies rounding, it tracks the exact mode closely."""
    ns, m, x, v, tcr = _systems(64, 3, 64, seed=6)
    t_end = np.full(len(ns), 2.0 * tcr)
    split = g6.batch_run(ns, t_end, m, x, v, mode="split")
    exact = g6.batch_run(ns, t_end, m, x, v, mode="exact")
    off = np.concatenate([[0], np.cumsum(ns)])
    de_s, de_e = [], []
    for s in range(len(ns)):
        a, b = off[s], off[s + 1]
        e0 = _energy(m[a:b], x[a:b], v[a:b])
        de_s.append(abs((_energy(m[a:b], split["pos"][a:b], split["vel"][a:b]) - e0) / e0))
        de_e.append(abs((_energy(m[a:b], exact["pos"][a:b], exact["vel"][a:b]) - e0) / e0))
    print(f"median |dE/E| split {np.median(de_s):.2e} exact {np.median(de_e):.2e}; "
          f"max split {max(de_s):.2e} exact {max(de_e):.2e}")
    assert np.all(split["status"] == 0) and np.all(split["t_final"] >= t_end)
    assert np.median(de_s) < 10 * np.median(de_e) + 1e-7
    short = np.full(len(ns), 0.02 * tcr)
    rs = g6.batch_run(ns, short, m, x, v, mode="split")
    re = g6.batch_run(ns, short, m, x, v, mode="exact")
    scale = np.abs(re["pos"]).max()
    assert np.abs(rs["pos"] - re["pos"]).max() <= 1e-5 * scale


def test_step_budget_and_queue(g6):
    ns, m, x, v, tcr = _systems(500, 3, 64, seed=7)
    r = g6.batch_run(ns, 5 * tcr, m, x, v, max_steps=10)
    assert np.all(r["steps"] == 10) and np.all(r["status"] == 1)
    r = g6.batch_run(ns, 0.05 * tcr, m, x, v)
    assert np.all(r["status"] == 0) and np.all(r["t_final"] >= 0.05 * tcr)
    assert np.all(r["wall_ms"] > 0)


def test_autotuner(g6):
    ns, m, x, v, tcr = _systems(300, 3, 64, seed=8)
    best = g6.batch_tune(ns, tcr, m, x, v, frac=0.02)
    assert best["warps_per_cta"] >= 1 and best["ctas_per_sm"] >= 1 and best["ms"] > 0
    r = g6.batch_run(ns, 0.05 * tcr, m, x, v)
    assert np.all(r["status"] == 0)


# --- smallN's unperturbed binaries --------------------------------------------

def _unpert_fixture():
    from conftest import golden
    g = golden("smalln_unpert.npz")
    k = int(g["nsys"])
    ns = np.array([len(g[f"s{i}_mass"]) for i in range(k)], np.int32)
    cat = lambda key: np.concatenate([g[f"s{i}_{key}"] for i in range(k)])
    t_end = np.array([float(g[f"s{i}_t_end"]) for i in range(k)])
    return g, k, ns, cat, t_end


@pytest.mark.parametrize("mode", ["fast", "split"])
def test_unperturbed_binaries_follow_oracle_and_smalln(g6, mode):
    """Hierarchical systems with hard binaries (tests/golden/smalln_unpert.npz,
    written by the unmodified smallN with its unperturbed binaries): the batch
    kernel with the same treatment ends where the oracle's restatement
    (orc_smalln_unpert) and smallN end, to 1e-4 of the system size (fast:
    FP64 pair terms; split: FP32 pair terms), having made binaries, in far
    fewer steps than without them."""
    g, k, ns, cat, t_end = _unpert_fixture()
    g6.batch_unperturbed(True)
    try:
        r = g6.batch_run(ns, t_end, cat("mass"), cat("pos0"), cat("vel0"), eta=0.14, mode=mode)
        nbin = g6.batch_binaries(k)
    finally:
        g6.batch_unperturbed(False)
    plain = g6.batch_run(ns, t_end, cat("mass"), cat("pos0"), cat("vel0"), eta=0.14, mode=mode)
    off = np.concatenate([[0], np.cumsum(ns)])
    for s in range(k):
        a, b = off[s], off[s + 1]
        m, x0, v0 = g[f"s{s}_mass"], g[f"s{s}_pos0"], g[f"s{s}_vel0"]
        po, vo, to, so, nbo = oracle.smalln_unpert(m, x0, v0, 0.14, t_end[s])
        scale = np.abs(x0).max()
        d_or = np.abs(r["pos"][a:b] - po).max() / scale
        d_ref = np.abs(r["pos"][a:b] - g[f"s{s}_pos"]).max() / scale
        print(f"system {s} ({mode}): steps {r['steps'][s]} (plain {plain['steps'][s]}, oracle "
              f"{so}), binaries {nbin[s]} (oracle {nbo}), |dx| vs oracle {d_or:.1e}, "
              f"vs smallN {d_ref:.1e}")
        assert r["status"][s] == 0
        assert nbin[s] >= 1
        assert d_or <= 1e-4 and d_ref <= 1e-4
        assert r["steps"][s] < plain["steps"][s]


def test_unperturbed_refused_in_exact_mode(g6):
    g, k, ns, cat, t_end = _unpert_fixture()
    g6.batch_unperturbed(True)
    try:
        with pytest.raises(ag.G6Error, match="exact"):
            g6.batch_run(ns, t_end, cat("mass"), cat("pos0"), cat("vel0"), mode="exact")
    finally:
        g6.batch_unperturbed(False)


def test_unperturbed_batching_workload_completes(g6):
    """The batching configuration's systems (n ~ U[3, 64], Plummer r_vir =
    1e-3, eps = 0) to 10 crossing times with the unperturbed treatment: no
    system reaches the step budget, and the per-system energy error stays at
    the level of the scheme's truncation error."""
    ns, m, x, v, tcr = _systems(256, 3, 64, seed=9)
    t_end = np.full(len(ns), 10.0 * tcr)
    g6.batch_unperturbed(True)
    try:
        r = g6.batch_run(ns, t_end, m, x, v, mode="split", max_steps=2_000_000)
        nbin = g6.batch_binaries(len(ns))
    finally:
        g6.batch_unperturbed(False)
    off = np.concatenate([[0], np.cumsum(ns)])
    de = []
    for s in range(len(ns)):
        a, b = off[s], off[s + 1]
        e0 = _energy(m[a:b], x[a:b], v[a:b])
        de.append(abs((_energy(m[a:b], r["pos"][a:b], r["vel"][a:b]) - e0) / e0))
    de = np.array(de)
    print(f"binaries made: {nbin.sum()} in {np.sum(nbin > 0)} systems; |dE/E| median "
          f"{np.median(de):.2e} p99 {np.percentile(de, 99):.2e} max {de.max():.2e}; steps max "
          f"{r['steps'].max()}")
    assert np.all(r["status"] == 0) and np.all(r["t_final"] >= t_end)
    assert np.all(np.isfinite(de)) and np.median(de) < 1e-3
