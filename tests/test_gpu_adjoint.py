"""GPU: fixed-step Hermite forward and its hand-written adjoint.

* forward (FP64 force) against the torch FP64 restatement (both jerk forms)
  and against the oracle's restatement of the hermite code;
* adjoint (FP64) against torch autograd of the restatement (reference
  gradient), against central finite differences of the GPU forward
  (h = 1e-6, relative error <= 1e-4), and independent of the checkpoint
  interval (bit for bit);
* split-precision adjoint against the FP64 adjoint.
"""
import numpy as np
import pytest
import torch

import hermite_torch as ht

pytestmark = pytest.mark.gpu


def _system(n, seed, eps_mass=True):
    from amuse_gb300 import ic
    rng = np.random.RandomState(seed)
    m, x, v = ic.plummer(n, do_scale=True, rng=rng)
    if eps_mass:
        m = m * rng.uniform(0.5, 1.5, n)
    w = rng.uniform(0.5, 1.5, n)
    return m, x, v, w


def _cuda(*arrays):
    return [torch.tensor(a, dtype=torch.float64, device="cuda") for a in arrays]


def _grad(m, x, v, w, eps2, dt, nsteps, checkpoint, precision, jerk="hermite"):
    from amuse_gb300.adjoint import hermite_fixed
    tm, tx, tv, tw = _cuda(m, x, v, w)
    for t in (tm, tx, tv):
        t.requires_grad_(True)
    xf, vf = hermite_fixed(tx, tv, tm, eps2=eps2, dt=dt, nsteps=nsteps, checkpoint=checkpoint,
                           precision=precision, jerk=jerk)
    loss = ht.loss(xf, tw)
    loss.backward()
    return (loss.item(), tx.grad.cpu().numpy(), tv.grad.cpu().numpy(), tm.grad.cpu().numpy(),
            xf.detach().cpu().numpy(), vf.detach().cpu().numpy())


@pytest.mark.parametrize("jerk", ["hermite", "softened"])
def test_forward_fp64_matches_torch(g6, jerk):
    from amuse_gb300.adjoint import hermite_fixed
    m, x, v, _ = _system(96, 1)
    tm, tx, tv = _cuda(m, x, v)
    xf, vf = hermite_fixed(tx, tv, tm, eps2=1e-4, dt=1 / 256, nsteps=24, precision="fp64",
                           jerk=jerk)
    rx, rv = ht.run(torch.tensor(x), torch.tensor(v), torch.tensor(m), 1e-4, 1 / 256, 24, jerk)
    np.testing.assert_allclose(xf.cpu().numpy(), rx.numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(vf.cpu().numpy(), rv.numpy(), rtol=0, atol=1e-11)


@pytest.mark.parametrize("eps2", [0.0, 1e-4])
def test_forward_fp64_matches_hermite_oracle(g6, eps2):
    import oracle
    m, x, v, _ = _system(300, 2, eps_mass=False)
    tm, tx, tv = _cuda(m, x, v)
    from amuse_gb300.adjoint import hermite_fixed
    xf, vf = hermite_fixed(tx, tv, tm, eps2=eps2, dt=1 / 1024, nsteps=16, precision="fp64")
    p, vv, _, _ = oracle.hermite_fixed(m, x, v, eps2, 1 / 1024, 16)
    np.testing.assert_allclose(xf.cpu().numpy(), p, rtol=0, atol=1e-11)
    np.testing.assert_allclose(vf.cpu().numpy(), vv, rtol=0, atol=1e-9)


@pytest.mark.parametrize("jerk", ["hermite", "softened"])
def test_adjoint_fp64_matches_autograd(g6, jerk):
    m, x, v, w = _system(64, 3)
    eps2, dt, nsteps = 1e-4, 1 / 256, 12
    _, gx, gv, gm, _, _ = _grad(m, x, v, w, eps2, dt, nsteps, 5, "fp64", jerk)
    tx = torch.tensor(x, requires_grad=True)
    tv = torch.tensor(v, requires_grad=True)
    tm = torch.tensor(m, requires_grad=True)
    xf, _ = ht.run(tx, tv, tm, eps2, dt, nsteps, jerk)
    ht.loss(xf, torch.tensor(w)).backward()
    for g, r in ((gx, tx.grad), (gv, tv.grad), (gm, tm.grad)):
        r = r.numpy()
        assert np.abs(g - r).max() <= 1e-9 * np.abs(r).max()


def test_adjoint_checkpoint_invariant(g6):
    m, x, v, w = _system(200, 4)
    ref = _grad(m, x, v, w, 1e-4, 1 / 256, 10, 10, "fp64")
    for k in (1, 3, 16):
        out = _grad(m, x, v, w, 1e-4, 1 / 256, 10, k, "fp64")
        for a, b in zip(ref[1:4], out[1:4]):
            np.testing.assert_array_equal(a, b)


def _loss_fp64(m, x, v, w, eps2, dt, nsteps, precision="fp64"):
    from amuse_gb300.adjoint import hermite_fixed
    tm, tx, tv, tw = _cuda(m, x, v, w)
    with torch.no_grad():
        xf, _ = hermite_fixed(tx, tv, tm, eps2=eps2, dt=dt, nsteps=nsteps, precision=precision)
        return float(ht.loss(xf, tw))


def test_adjoint_fp64_matches_finite_differences(g6):
    m, x, v, w = _system(512, 5)
    eps2, dt, nsteps, h = 1e-4, 1 / 256, 16, 1e-6
    _, gx, gv, gm, _, _ = _grad(m, x, v, w, eps2, dt, nsteps, 4, "fp64")
    rng = np.random.RandomState(9)
    for _ in range(12):
        kind = rng.randint(3)
        i = rng.randint(len(m))
        c = rng.randint(3)
        args = [m.copy(), x.copy(), v.copy()]
        if kind == 0:
            target, g = (1, (i, c)), gx[i, c]
        elif kind == 1:
            target, g = (2, (i, c)), gv[i, c]
        else:
            target, g = (0, (i,)), gm[i]
        lp = [a.copy() for a in args]
        lm_ = [a.copy() for a in args]
        lp[target[0]][target[1]] += h
        lm_[target[0]][target[1]] -= h
        fd = (_loss_fp64(*lp, w, eps2, dt, nsteps) - _loss_fp64(*lm_, w, eps2, dt, nsteps)) / (2 * h)
        assert abs(fd - g) <= 1e-4 * max(abs(g), 1e-2 * np.abs(gx).max()), (kind, i, c, fd, g)


def test_adjoint_split_close_to_fp64(g6):
    m, x, v, w = _system(2048, 6)
    ref = _grad(m, x, v, w, 1e-4, 1 / 256, 16, 4, "fp64")
    out = _grad(m, x, v, w, 1e-4, 1 / 256, 16, 4, "split")
    assert abs(out[0] - ref[0]) <= 1e-9 * abs(ref[0])
    for a, b in zip(out[1:4], ref[1:4]):
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel <= 1e-4, rel


def test_force_vjp_rejects_empty(g6):
    with pytest.raises(Exception):
        g6.force_vjp(0, 0.0, 0, 0, 0, 0, 0, 0, 0, 0)


@pytest.mark.parametrize("precision", ["split", "fp64"])
def test_fixed_force_matches_torch(g6, precision):
    """The force alone, hermite jerk form, against the torch restatement."""
    from amuse_gb300.adjoint import final_forces
    m, x, v, _ = _system(1000, 8)
    tm, tx, tv = _cuda(m, x, v)
    a, j = final_forces(tx, tv, tm, eps2=1e-4, precision=precision)
    ra, rj = ht.forces(torch.tensor(x), torch.tensor(v), torch.tensor(m), 1e-4)
    for g, r, tol_split in ((a, ra, 1e-6), (j, rj, 1e-5)):
        err = ((g.cpu() - r).norm(dim=1) / r.norm(dim=1)).numpy()
        if precision == "fp64":
            assert err.max() <= 1e-10, err.max()
        else:
            assert np.quantile(err, 0.99) <= tol_split, np.quantile(err, 0.99)
