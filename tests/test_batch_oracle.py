"""smallN's integrator restated in the oracle, pinned bit-for-bit against
smallN compiled from the reference sources (dt_crit = 0: no unperturbed
binary tree): directly where the reference build exists (oracle/_ref), and
everywhere through the fixtures it wrote (tests/golden/smalln_systems.npz)."""
import numpy as np
import pytest

import oracle
from amuse_gb300 import ic


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build absent")
@pytest.mark.parametrize("n,seed", [(3, 1), (5, 2), (16, 3), (40, 4)])
def test_smalln_restatement_bitexact(n, seed):
    np.random.seed(seed)
    m, x, v = ic.plummer(n, do_scale=True)
    x, v = x * 1e-3, v * np.sqrt(1e3)
    tcr = 2 * np.sqrt(2) * 1e-3 ** 1.5
    pr, vr, tr, _ = oracle.smalln(m, x, v, 0.14, 2 * tcr, lib="ref")
    pp, vp, tp, st = oracle.smalln(m, x, v, 0.14, 2 * tcr)
    assert np.array_equal(pr, pp) and np.array_equal(vr, vp) and tr == tp
    assert st > 0


def test_smalln_restatement_matches_fixtures():
    from conftest import golden
    g = golden("smalln_systems.npz")
    for i in range(int(g["nsys"])):
        p, v, t, st = oracle.smalln(g[f"s{i}_mass"], g[f"s{i}_pos0"], g[f"s{i}_vel0"],
                                    float(g["eta"]), float(g["t_end"]))
        assert np.array_equal(p, g[f"s{i}_pos"]) and np.array_equal(v, g[f"s{i}_vel"])
        assert t == float(g[f"s{i}_t"]) and st > 0


def _energy(m, x, v):
    k = 0.5 * np.sum(m * np.sum(v * v, 1))
    u = 0.0
    for i in range(len(m)):
        d = np.linalg.norm(x[i + 1:] - x[i], axis=1)
        u -= m[i] * np.sum(m[i + 1:] / d)
    return k + u


def test_smalln_unperturbed_restatement_matches_fixtures():
    """smallN WITH unperturbed binaries (the worker's defaults), restated in
    the oracle (orc_smalln_unpert), against the unmodified smallN on systems
    with hard binaries (tests/golden/smalln_unpert.npz): over 90-360 binary
    segments the restatement's Kepler propagator and its energy correction
    (the relative velocity rescaled for the tidal-potential change) follow
    smallN's to |dx| <= 5e-5 of the system size, the same final time to
    1e-5, and the same energy error to 10%."""
    from conftest import golden
    g = golden("smalln_unpert.npz")
    for i in range(int(g["nsys"])):
        m, x0, v0 = g[f"s{i}_mass"], g[f"s{i}_pos0"], g[f"s{i}_vel0"]
        p, v, t, st, nb = oracle.smalln_unpert(m, x0, v0, float(g["eta"]),
                                               float(g[f"s{i}_t_end"]))
        scale = np.abs(x0).max()
        assert np.abs(p - g[f"s{i}_pos"]).max() <= 5e-5 * scale, i
        assert abs(t - float(g[f"s{i}_t"])) <= 1e-5, i
        e0 = _energy(m, x0, v0)
        de_ref = abs(_energy(m, g[f"s{i}_pos"], g[f"s{i}_vel"]) - e0)
        de = abs(_energy(m, p, v) - e0)
        assert abs(de - de_ref) <= 0.1 * de_ref + 1e-12 * abs(e0), i
        assert nb >= 1 and st > 0


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build absent")
def test_smalln_unperturbed_one_segment_vs_reference():
    """One binary, one fully unperturbed segment: the restatement and smallN
    agree to 1e-9 in position and 1e-10 in the final time (the Kepler
    solvers differ at the 1e-11 level; nothing chaotic in between)."""
    import importlib.util, os
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    m, x, v = mg.hierarchical("field", 5)
    pr, vr, tr, _ = oracle.smalln(m, x, v, 0.14, 0.5, lib="ref", dt_crit=1e-3)
    p, vv, t, st, nb = oracle.smalln_unpert(m, x, v, 0.14, 0.5)
    assert nb == 1 and abs(t - tr) <= 1e-10
    assert np.abs(p - pr).max() <= 1e-9 * np.abs(x).max()
