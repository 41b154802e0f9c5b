"""GPU edge cases: empty and minimal inputs, sizes at the limits, rejected
arguments -- each through the public entry points, with the expected result
stated (the reference either returns zeros or exits; this library returns
zeros or a negative code and stays usable)."""
import numpy as np
import pytest
import torch

import amuse_gb300 as ag
import oracle
from amuse_gb300 import ic

pytestmark = pytest.mark.gpu


def test_empty_i_block(g6):
    """ni = 0: firsthalf/lasthalf do nothing and succeed (ph4 can issue an
    empty chunk); the outputs are untouched."""
    np.random.seed(21)
    m, x, v = ic.plummer(32)
    ids = np.arange(1, 33)
    ag.drive_load(m, x, v, ids=ids)
    out = ag.drive_force(32, 0.0, 1e-4, np.zeros(0, np.int32), np.zeros((0, 3)),
                         np.zeros((0, 3)))
    assert out["acc"].shape == (0, 3)


def test_single_j_particle(g6):
    """nj = 1 and the i-particle is that particle: no pairs, zero force."""
    m, x, v = np.array([1.0]), np.array([[0.1, 0.2, 0.3]]), np.array([[0.0, 0.1, 0.0]])
    ag.drive_load(m, x, v, ids=np.array([7]))
    out = ag.drive_force(1, 0.0, 1e-4, np.array([7]), x, v)
    assert np.all(out["acc"] == 0) and np.all(out["jerk"] == 0) and np.all(out["pot"] == 0)


def test_two_body_exact_field(g6):
    """Two bodies: the force on each is the analytic softened pair force."""
    m = np.array([0.3, 0.7])
    x = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])
    v = np.zeros((2, 3))
    ag.drive_load(m, x, v, ids=np.array([1, 2]))
    out = ag.drive_force(2, 0.0, 1e-4, np.array([1, 2]), x, v)
    r2 = 0.25 + 1e-4
    np.testing.assert_allclose(out["acc"][0, 0], 0.7 * 0.5 / r2 ** 1.5, rtol=1e-6)
    np.testing.assert_allclose(out["acc"][1, 0], -0.3 * 0.5 / r2 ** 1.5, rtol=1e-6)
    np.testing.assert_allclose(out["pot"], [-0.7 / r2 ** 0.5, -0.3 / r2 ** 0.5], rtol=1e-6)


def test_j_count_not_multiple_of_tile(g6):
    """nj = 257 and 511 (one past / one short of the 256-record tile)."""
    for n in (257, 511):
        np.random.seed(n)
        m, x, v = ic.plummer(n)
        g6.load_particles(m, x, v)
        out = g6.force(0.0, 1e-4, n, x, v, self_slot=np.arange(n))
        ref = oracle.force(m, x, v, 1e-4, x, v)
        e = np.linalg.norm(out["acc"] - ref["acc"], axis=1) / np.linalg.norm(ref["acc"], axis=1)
        assert np.percentile(e, 99) <= 1e-6 and e.max() <= 1e-5


def test_batch_size_limits(g6):
    """n = 2 (smallest) and n = 64 (largest) systems run; n = 1 and n = 65
    are refused by the host before any launch; the context stays usable."""
    rng = np.random.RandomState(4)
    for n in (2, 64):
        m, x, v = ic.plummer(n, do_scale=True, rng=rng)
        x, v = x * 1e-3, v / np.sqrt(1e-3)
        r = g6.batch_run([n], 1e-5, m, x, v, exact=True)
        px, pv, _, _ = oracle.smalln(m, x, v, 0.14, 1e-5)
        assert np.array_equal(r["pos"], px) and np.array_equal(r["vel"], pv)
    for n in (1, 65):
        m = np.full(n, 1.0 / n)
        with pytest.raises(ag.G6Error):
            g6.batch_run([n], 1e-5, m, np.zeros((n, 3)), np.zeros((n, 3)))
    m, x, v = ic.plummer(8, do_scale=True, rng=rng)
    r = g6.batch_run([8], 1e-5, m, x * 1e-3, v / np.sqrt(1e-3))
    assert r["status"][0] == 0


def test_batch_rejects_bad_mode(g6):
    """A mode other than fast/exact/split is refused by the C entry point."""
    import ctypes
    m, x, v = ic.plummer(4, do_scale=True, rng=np.random.RandomState(1))
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    n = np.array([4], np.int32)
    rc = g6.lib.g6x_batch_run(1, n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                              P(np.array([1e-5])), P(np.ascontiguousarray(m)),
                              P(np.ascontiguousarray(x)), P(np.ascontiguousarray(v)),
                              0.14, 2, 0, 7, None, None, None, None, None)
    assert rc == -2  # G6_ERR_ARG


def test_fixed_step_two_bodies_and_single_body(g6):
    """The fixed-step path at n = 2 (against the oracle's hermite step) and
    n = 1 (no pairs: straight-line motion, zero gradient w.r.t. mass)."""
    from amuse_gb300.adjoint import hermite_fixed
    m = np.array([0.5, 0.5])
    x = np.array([[0.5, 0.0, 0.0], [-0.5, 0.0, 0.0]])
    v = np.array([[0.0, 0.5, 0.0], [0.0, -0.5, 0.0]])
    t = [torch.tensor(a, device="cuda") for a in (x, v, m)]
    xf, vf = hermite_fixed(t[0], t[1], t[2], eps2=0.0, dt=1 / 64, nsteps=32, precision="fp64")
    p, vv, _, _ = oracle.hermite_fixed(m, x, v, 0.0, 1 / 64, 32)
    np.testing.assert_allclose(xf.cpu().numpy(), p, rtol=0, atol=1e-13)
    f64 = dict(device="cuda", dtype=torch.float64, requires_grad=True)
    x1 = torch.tensor([[0.1, 0.2, 0.3]], **f64)
    v1 = torch.tensor([[1.0, 0.0, 0.0]], **f64)
    m1 = torch.tensor([1.0], **f64)
    xf1, _ = hermite_fixed(x1, v1, m1, eps2=1e-4, dt=0.25, nsteps=4)
    np.testing.assert_allclose(xf1.detach().cpu().numpy(), [[1.1, 0.2, 0.3]], rtol=0,
                               atol=1e-15)
    xf1.sum().backward()
    assert float(m1.grad.abs().max()) == 0.0


def test_fixed_step_rejects_bad_inputs(g6):
    from amuse_gb300.adjoint import hermite_fixed
    x = torch.zeros((4, 3), device="cuda", dtype=torch.float32)
    with pytest.raises(TypeError):
        hermite_fixed(x, x, torch.ones(4, device="cuda"), eps2=0.0, dt=0.1, nsteps=1)
    xd = torch.zeros((4, 3), device="cuda", dtype=torch.float64)
    with pytest.raises(ValueError):
        hermite_fixed(xd, xd, torch.ones(3, device="cuda", dtype=torch.float64), eps2=0.0,
                      dt=0.1, nsteps=1)
    with pytest.raises(ValueError):
        hermite_fixed(xd, xd, torch.ones(4, device="cuda", dtype=torch.float64), eps2=0.0,
                      dt=0.1, nsteps=0)


def test_close_and_reopen(g6):
    """g6_close_ releases every buffer (j-store, batch, fixed-step,
    neighbour lists); a new g6_open_ gives a working context again."""
    from amuse_gb300.adjoint import hermite_fixed
    rng = np.random.RandomState(31)
    m, x, v = ic.plummer(64, do_scale=True, rng=rng)
    ids = np.arange(1, 65)
    ag.drive_load(m, x, v, ids=ids)
    before = ag.drive_force(64, 0.0, 1e-4, ids, x, v)
    g6.close()
    ag.G6X(0)  # g6_open_ again
    ag.drive_load(m, x, v, ids=ids)
    after = ag.drive_force(64, 0.0, 1e-4, ids, x, v)
    np.testing.assert_array_equal(before["acc"], after["acc"])
    r = g6.batch_run([5], 1e-5, m[:5], x[:5] * 1e-3, v[:5] / np.sqrt(1e-3), exact=True)
    assert r["status"][0] == 0
    t = [torch.tensor(a, device="cuda") for a in (x, v, m)]
    xf, _ = hermite_fixed(t[0], t[1], t[2], eps2=1e-4, dt=1 / 256, nsteps=2)
    assert torch.isfinite(xf).all()


def test_bounded_wait_expiry(g6):
    """The force kernel's waits are bounded: with the test hook, the first
    CTA waits on a barrier that nothing arrives on; after 20 ms the wait
    gives up, the CTA drains its copies and sets the error word, and the call
    returns G6_ERR_KERNEL.  The next call runs normally and is correct."""
    np.random.seed(41)
    n = 4096
    m, x, v = ic.plummer(n)
    g6.load_particles(m, x, v)
    sel = np.arange(0, n, 8)
    g6.test_wait_expiry(True)
    with pytest.raises(ag.G6Error) as ei:
        g6.force(0.0, 1e-4, n, x[sel], v[sel], self_slot=sel)
    assert "error word" in str(ei.value)
    out = g6.force(0.0, 1e-4, n, x[sel], v[sel], self_slot=sel)
    ref = oracle.force(m, x, v, 1e-4, x[sel], v[sel])
    e = np.linalg.norm(out["acc"] - ref["acc"], axis=1) / np.linalg.norm(ref["acc"], axis=1)
    assert e.max() <= 1e-6
