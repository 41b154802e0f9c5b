"""The encounter check on the CPU: the oracle's restatement of ph4's
idata::check_encounters (idata.cc:620-700) and of the COLLISION_DETECTION
stopping condition (jdata.cc:797-850) against block-step runs of the
unmodified ph4 objects (tests/golden/encounter_runs.npz, made by
tests/golden/make_golden.py --only encounters)."""
import numpy as np
import pytest

import oracle
from conftest import golden


def _cases():
    g = golden("encounter_runs.npz")
    return g, int(g["ncase"])


@pytest.mark.parametrize("k", range(5))
def test_oracle_encounter_runs_match_ph4(k):
    """Same final state bit for bit, same stop time and block count, same
    pair.  ph4 orders the pair by its scheduler's list, the oracle by slot,
    so the pair is compared as a set."""
    g, n = _cases()
    assert k < n
    c = {key[len(f"c{k}_"):]: g[key] for key in g if key.startswith(f"c{k}_")}
    r = oracle.run_enc(c["mass"], c["radius"], c["pos0"], c["vel0"], float(g["eps2"]),
                       float(g["eta"]), float(c["t_end"]), mode=int(c["mode"]))
    assert r["t"] == float(c["t"]) and r["blocks"] == int(c["blocks"])
    assert np.array_equal(r["pos"], c["pos"]) and np.array_equal(r["vel"], c["vel"])
    pair = r["stop_pair"] if int(c["mode"]) & oracle.ENC_STOP_COLL else r["close"]
    assert sorted(pair) == sorted(int(p) for p in c["pair"])
    assert r["rmin"] == float(c["rmin"]) == 2.0 / len(c["mass"])
    assert r["stopped"] == (1 if int(c["mode"]) & oracle.ENC_STOP_COLL else 2)


def test_oracle_check_without_stop_runs_to_the_end():
    """CHECK alone reports the last block's pairs and never stops the run."""
    g, _ = _cases()
    c = {key[3:]: g[key] for key in g if key.startswith("c3_")}
    r = oracle.run_enc(c["mass"], c["radius"], c["pos0"], c["vel0"], float(g["eps2"]),
                       float(g["eta"]), float(c["t"]), mode=oracle.ENC_CHECK)
    assert r["stopped"] == 0 and r["t"] == float(c["t"]) and r["blocks"] == int(c["blocks"])
    assert sorted(r["close"]) == sorted(int(p) for p in c["pair"])
    assert r["rmax_close"] >= 1.0


def test_oracle_collision_needs_approach():
    """Two particles inside each other's radius but receding on an unbound
    orbit (relative speed 100, escape speed 10): the collision pair is
    reported every block, the stop waits for vr < 0.001 r v, which they
    never meet; approaching, they stop after the first block."""
    m = np.array([0.5, 0.5])
    x = np.array([[-0.01, 0.0, 0.0], [0.01, 0.0, 0.0]])
    v = np.array([[-50.0, 0.0, 0.0], [50.0, 0.0, 0.0]])
    r = oracle.run_enc(m, np.full(2, 10.0), x, v, 1e-4, 0.14, 0.05)
    assert r["stopped"] == 0 and r["coll"] is not None and r["t"] >= 0.05
    v2 = -v
    r2 = oracle.run_enc(m, np.full(2, 10.0), x, v2, 1e-4, 0.14, 0.05)
    assert r2["stopped"] == 1 and r2["blocks"] == 1 and sorted(r2["stop_pair"]) == [1, 2]


def test_oracle_encounter_off_is_plain_run():
    """mode 0 is exactly the plain block-step run."""
    g, _ = _cases()
    c = {key[3:]: g[key] for key in g if key.startswith("c0_")}
    a = oracle.run_enc(c["mass"], c["radius"], c["pos0"], c["vel0"], 1e-4, 0.14, 0.25, mode=0)
    b = oracle.run(c["mass"], c["pos0"], c["vel0"], 1e-4, 0.14, 0.25)
    assert np.array_equal(a["pos"], b["pos"]) and a["blocks"] == b["blocks"]
    assert a["stopped"] == 0 and a["close"] is None and a["coll"] is None


def test_oracle_massless_pairs_are_not_encounters():
    """ph4 skips a pair whose members are both massless (idata.cc:648);
    one massive member is enough (and a CPU-mode force never picks a
    massless neighbour, idata.cc:193)."""
    m = np.array([1.0, 0.0, 0.0])
    x = np.array([[0.0, 0.0, 0.0], [5.0, 0.0, 0.0], [5.001, 0.0, 0.0]])
    v = np.array([[0.0, 0.0, 0.0], [0.0, 0.45, 0.0], [0.0, 0.45, 0.0]])
    r = oracle.run_enc(m, np.full(3, 0.01), x, v, 0.0, 0.14, 0.01,
                       mode=oracle.ENC_CHECK, rmin=0.1)
    # the two test particles are 0.001 apart but massless: no pair; their
    # nearest massive neighbour (the central mass) is far away
    assert r["close"] is None and r["coll"] is None


def test_oracle_explicit_rmin():
    """rmin given explicitly replaces ph4's 2/n."""
    m = np.array([0.5, 0.5])
    x = np.array([[-0.05, 0.0, 0.0], [0.05, 0.0, 0.0]])
    v = np.array([[0.0, -1.0, 0.0], [0.0, 1.0, 0.0]])
    r = oracle.run_enc(m, np.zeros(2), x, v, 0.0, 0.14, 1e-3, mode=oracle.ENC_CHECK, rmin=0.2)
    assert r["rmin"] == 0.2 and r["close"] is not None and r["rmax_close"] >= 1.0
    r2 = oracle.run_enc(m, np.zeros(2), x, v, 0.0, 0.14, 1e-3, mode=oracle.ENC_CHECK, rmin=0.05)
    assert r2["rmin"] == 0.05 and r2["close"] is None
