"""The encounter check of the device block-step driver (g6x_set_encounters,
g6x_set_radius, g6x_run, g6x_encounter) against block-step runs of the
unmodified ph4 objects with the COLLISION_DETECTION stopping condition
(idata.cc:620-700, jdata.cc:797-850; tests/golden/encounter_runs.npz) and
against the oracle's restatement, which breaks ties by slot as the library
does."""
import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from conftest import golden

pytestmark = pytest.mark.gpu


def _case(k):
    g = golden("encounter_runs.npz")
    c = {key[len(f"c{k}_"):]: g[key] for key in g if key.startswith(f"c{k}_")}
    return float(g["eps2"]), float(g["eta"]), c


def _run(g6, prec, c, mode, eps2, eta, t_end, max_blocks=0):
    g6.set_precision(prec)
    try:
        g6.load_particles(c["mass"], c["pos0"], c["vel0"])
        g6.set_radius(c["radius"])
        g6.set_encounters(mode)
        g6.run_init(eps2, eta)
        nb, _ = g6.run(t_end, max_blocks)
        enc = g6.encounter()
        st = g6.read_particles(len(c["mass"]))
        st["t"] = g6.system_time()
    finally:
        g6.set_encounters(0)
        g6.set_precision(ag.SPLIT)
    return nb, enc, st


@pytest.mark.parametrize("k", range(5))
def test_fp64_encounter_stop_matches_ph4(g6, k):
    """FP64 forces: the run stops after the same block at the same time as
    ph4, on the same pair (ordered as the oracle orders ties)."""
    eps2, eta, c = _case(k)
    mode = int(c["mode"])
    nb, enc, st = _run(g6, ag.FP64, c, mode, eps2, eta, float(c["t_end"]))
    port = oracle.run_enc(c["mass"], c["radius"], c["pos0"], c["vel0"], eps2, eta,
                          float(c["t_end"]), mode=mode)
    coll = bool(mode & ag.ENC_STOP_COLLISION)
    pair = enc["coll"] if coll else enc["close"]
    print(f"case {k}: blocks {nb} (ph4 {int(c['blocks'])}) t {st['t']} (ph4 {float(c['t'])}) "
          f"pair {pair} (ph4 {tuple(c['pair'])}) rmax {enc['rmax_close']:.4f} {enc['rmax_coll']:.4f}")
    assert nb == int(c["blocks"]) and st["t"] == float(c["t"]) and enc["t"] == st["t"]
    assert enc["stopped"] == (1 if coll else 2)
    assert sorted(pair) == sorted(int(p) for p in c["pair"])
    assert pair == (port["stop_pair"] if coll else port["close"])
    np.testing.assert_allclose(st["pos"], c["pos"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("k", range(3))
def test_split_collision_stop(g6, k):
    """Split-precision forces: the same pair collides; the stop comes at
    the block where the approaching pair first overlaps, and there the two
    particles are within about the sum of their radii."""
    eps2, eta, c = _case(k)
    nb, enc, st = _run(g6, ag.SPLIT, c, int(c["mode"]), eps2, eta, float(c["t_end"]))
    print(f"case {k} split: blocks {nb} (ph4 {int(c['blocks'])}) t {st['t']} "
          f"(ph4 {float(c['t'])}) pair {enc['coll']}")
    assert enc["stopped"] == 1 and st["t"] < float(c["t_end"])
    assert sorted(enc["coll"]) == sorted(int(p) for p in c["pair"])
    a, b = (p - 1 for p in enc["coll"])
    d = np.linalg.norm(st["pos"][a] - st["pos"][b])
    assert d <= 1.5 * (c["radius"][a] + c["radius"][b])
    assert abs(st["t"] - float(c["t"])) <= 0.02


def test_check_only_reports_without_stopping(g6):
    """ENC_CHECK alone: after the block in which ph4 first sees the close
    pair the library reports the same pair, stopped = 0, and the run goes
    on."""
    eps2, eta, c = _case(3)
    nb, enc, st = _run(g6, ag.FP64, c, ag.ENC_CHECK, eps2, eta, 10.0, int(c["blocks"]))
    assert nb == int(c["blocks"]) and st["t"] == float(c["t"])
    assert enc["stopped"] == 0 and sorted(enc["close"]) == sorted(int(p) for p in c["pair"])
    assert enc["rmax_close"] >= 1.0


def test_encounter_arguments(g6):
    with pytest.raises(ag.G6Error):
        g6.set_encounters(8)
    with pytest.raises(ag.G6Error):
        g6.set_encounters(ag.ENC_CHECK, -1.0)
    g6.set_encounters(0)
    r = g6.encounter()
    assert r["stopped"] in (0, 1, 2)
