"""The oracle (C restatement of ph4's FP64 CPU path) pinned against fixtures
made by the unmodified ph4 objects (tests/golden/make_golden.py), plus the
known-answer tests of src/amuse_ph4/tests/test_ph4.py restated as direct
calls.  CPU only."""
import numpy as np
import pytest

import oracle
from conftest import golden


@pytest.fixture(scope="module", autouse=True)
def _port():
    oracle.build_port()


@pytest.mark.parametrize("name,ikey", [
    ("force_plummer1024_eps1e-4.npz", None),
    ("force_salpeter4096_eps1e-6.npz", "ipos"),
    ("force_plummer128_eps0.npz", None),
])
def test_force_bitexact(name, ikey):
    g = golden(name)
    ipos = g["pos"] if ikey is None else g["ipos"]
    ivel = g["vel"] if ikey is None else g["ivel"]
    out = oracle.force(g["mass"], g["pos"], g["vel"], float(g["eps2"]), ipos, ivel)
    for k in ("acc", "jerk", "pot", "nn", "dnn"):
        assert np.array_equal(out[k], g[k]), k


def test_force_threads_identical():
    g = golden("force_plummer1024_eps1e-4.npz")
    a = oracle.force(g["mass"], g["pos"], g["vel"], 1e-4, g["pos"], g["vel"], threads=1)
    b = oracle.force(g["mass"], g["pos"], g["vel"], 1e-4, g["pos"], g["vel"], threads=5)
    for k in a:
        assert np.array_equal(a[k], b[k])


def test_correct_bitexact():
    g = golden("correct512.npz")
    c = oracle.correct(float(g["tnext"]), float(g["eta"]), g["itime"], g["istep"], g["ipos"],
                       g["ivel"], g["old_acc"], g["old_jerk"], g["iacc"], g["ijerk"])
    assert np.array_equal(c["pos"], g["out_pos"])
    assert np.array_equal(c["vel"], g["out_vel"])
    assert np.array_equal(c["time"], g["out_time"])
    assert np.array_equal(c["timestep"], g["out_step"])


def test_run_short_bitexact():
    g = golden("run_plummer256_eps1e-6.npz")
    r = oracle.run(g["mass"], g["pos0"], g["vel0"], float(g["eps2"]), float(g["eta"]),
                   float(g["t_end"]), threads=4)
    for k in ("pos", "vel", "acc", "jerk", "time", "timestep"):
        assert np.array_equal(r[k], g[k]), k
    assert r["E0"] == g["E0"] and r["E1"] == g["E1"]
    assert r["blocks"] == g["blocks"]


@pytest.mark.slow
def test_run_c1_bitexact():
    """Config 1: N=1024 Plummer, eps2=1e-4, eta=0.01, to t=1 (33k block steps)."""
    g = golden("run_plummer1024_t1.npz")
    r = oracle.run(g["mass"], g["pos0"], g["vel0"], 1e-4, 0.01, 1.0, threads=8)
    assert r["blocks"] == g["blocks"]
    for k in ("pos", "vel", "time", "timestep"):
        assert np.array_equal(r[k], g[k]), k
    assert abs((r["E1"] - r["E0"]) / r["E0"]) < 1e-6


def test_predict_matches_formula():
    rng = np.random.RandomState(0)
    n = 64
    t = rng.uniform(0, 0.1, n)
    t[:5] = 0.25
    x, v, a, j = (rng.normal(size=(n, 3)) for _ in range(4))
    pp, pv = oracle.predict(0.25, t, x, v, a, j)
    dt = (0.25 - t)[:, None]
    assert np.allclose(pp, x + dt * (v + 0.5 * dt * (a + dt * j / 3)), rtol=1e-15, atol=1e-15)
    assert np.array_equal(pp[:5], x[:5]) and np.array_equal(pv[:5], v[:5])


def test_initial_step_power_of_two():
    g = golden("force_plummer1024_eps1e-4.npz")
    ts = oracle.initial_step(g["acc"], g["jerk"], 0.01)
    assert np.all(ts > 0) and np.all(ts <= 0.03125)
    m, e = np.frexp(ts)
    assert np.all(m == 0.5)


# --- known answers, src/amuse_ph4/tests/test_ph4.py restated -------------

def _two(m1, m2, x2, eps2):
    mass = np.array([m1, m2])
    pos = np.array([[0.0, 0, 0], [x2, 0, 0]])
    vel = np.zeros((2, 3))
    return oracle.force(mass, pos, vel, eps2, pos, vel)


def test_kat_test7_softened_pair():
    # test_ph4.py:34-54: pot(id1) = -10 / sqrt(2^2 + 0.1^2)
    f = _two(10.0, 10.0, 2.0, 0.01)
    assert f["pot"][0] == pytest.approx(-10.0 / np.sqrt(4.0 + 0.01), rel=1e-8)


def test_kat_test8_unsoftened_pair():
    # test_ph4.py:56-77
    f = _two(10.0, 1.0, 2.0, 0.0)
    assert f["pot"][0] == pytest.approx(-0.5, rel=1e-8)
    assert f["pot"][1] == pytest.approx(-5.0, rel=1e-8)


def test_kat_test20_field_points():
    # test_ph4.py:786-822: two unit masses at x=0 and x=2, eps2=1e-5; the
    # potential and force at points on the axis.
    mass = np.array([1.0, 1.0])
    pos = np.array([[0.0, 0, 0], [2.0, 0, 0]])
    vel = np.zeros((2, 3))
    pots = [-4.57110767688, -2.66662518639, -2.13331892165]
    for x, pref in zip((0.25, 0.5, 0.75), pots):
        pts = np.array([[x, 0, 0], [2.0 - x, 0, 0]])
        f = oracle.force(mass, pos, vel, 1e-5, pts, np.zeros((2, 3)))
        assert f["pot"][0] == pytest.approx(pref, rel=1e-5)
        assert f["pot"][1] == pytest.approx(f["pot"][0], rel=1e-5)
        fx = -1.0 / x ** 2 + 1.0 / (2.0 - x) ** 2
        assert f["acc"][0, 0] == pytest.approx(fx, rel=1e-2)
        assert f["acc"][0, 0] == pytest.approx(-f["acc"][1, 0], rel=1e-5)


def test_kat_test26_exact():
    # test_ph4.py:948-968: m=[1,2] at x=-1,1: pot of particle 0 = -2/2 exactly
    mass = np.array([1.0, 2.0])
    pos = np.array([[-1.0, 0, 0], [1.0, 0, 0]])
    vel = np.array([[-1.0, -1, -1], [1, 1, 1]])
    f = oracle.force(mass, pos, vel, 0.0, pos, vel)
    assert f["pot"][0] == pytest.approx(-1.0, rel=1e-15)
