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
