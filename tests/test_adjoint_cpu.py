"""CPU checks for the fixed-step Hermite path and its adjoint.

* the oracle's restatement of the hermite code (orc_hermite_fixed) against
  the reference test's known answer (src/amuse_hermite/tests/
  test_hermite.py:86-113: an equal-mass circular binary returns to its
  mirror position after half a period and to its start after a period, to
  3 decimals) and against the torch restatement;
* the adjoint equations the kernels implement (the header of
  amuse_gb300/csrc/kern_fixed.cu), restated in numpy, against torch autograd
  of the forward map.
"""
import math

import numpy as np
import pytest
import torch

import hermite_torch as ht


def test_oracle_hermite_binary_known_answer(lib_built):
    import oracle
    m = np.array([0.5, 0.5])
    x = np.array([[0.5, 0, 0], [-0.5, 0, 0]], float)
    v = np.array([[0, 0.5, 0], [0, -0.5, 0]], float)
    dt = math.pi / 2048
    p1, v1, _, _ = oracle.hermite_fixed(m, x, v, 0.0, dt, 2048)
    np.testing.assert_allclose(p1, [[-0.5, 0, 0], [0.5, 0, 0]], atol=5e-4)
    p2, _, _, _ = oracle.hermite_fixed(m, p1, v1, 0.0, dt, 2048)
    np.testing.assert_allclose(p2, [[0.5, 0, 0], [-0.5, 0, 0]], atol=5e-4)


def test_oracle_hermite_force_matches_ph4_force_unsoftened(lib_built):
    """At eps2 = 0 the hermite code's pair force (symmetric j > i loop) equals
    ph4's (idata.cc:147-237, pinned bit-exact against the reference build)
    up to summation order."""
    import oracle
    from amuse_gb300 import ic
    rng = np.random.RandomState(8)
    m, x, v = ic.plummer(200, do_scale=True, rng=rng)
    _, _, a, j = oracle.hermite_fixed(m, x, v, 0.0, 1 / 256, 0)
    ref = oracle.force(m, x, v, 0.0, x, v)
    for got, want in ((a, ref["acc"]), (j, ref["jerk"])):
        err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
        assert err.max() <= 1e-12, err.max()


@pytest.mark.parametrize("eps2", [0.0, 1e-4])
def test_oracle_hermite_matches_torch(lib_built, eps2):
    """The oracle's hermite step and the torch restatement (hermite jerk)."""
    import oracle
    from amuse_gb300 import ic
    rng = np.random.RandomState(5)
    m, x, v = ic.plummer(48, do_scale=True, rng=rng)
    p, vv, a, j = oracle.hermite_fixed(m, x, v, eps2, 1 / 512, 32)
    tx, tv = ht.run(torch.tensor(x), torch.tensor(v), torch.tensor(m), eps2, 1 / 512, 32)
    np.testing.assert_allclose(p, tx.numpy(), rtol=0, atol=1e-11)
    np.testing.assert_allclose(vv, tv.numpy(), rtol=0, atol=1e-10)


# ---- numpy restatement of the kernels' adjoint arithmetic ----

def _forces(x, v, m, eps2, jerk):
    a, j = ht.forces(torch.tensor(x), torch.tensor(v), torch.tensor(m), eps2, jerk)
    return a.numpy(), j.numpy()


def _force_vjp(x, v, m, eps2, la, lj, jerk):
    n = len(m)
    gx = np.zeros((n, 3)); gv = np.zeros((n, 3)); gm = np.zeros(n)
    e2 = eps2 + ht.TINY
    for k in range(n):
        for jj in range(n):
            if jj == k:
                continue
            r = x[jj] - x[k]; w = v[jj] - v[k]
            s = r @ r + e2
            s3, s5, s7 = s ** -1.5, s ** -2.5, s ** -3.5
            if jerk == "hermite":
                qi = 1.0 / (r @ r)
                qs, c7 = qi * s3, 3 * (2 * qi * qi * s3 + 3 * qi * s5)
            else:
                qs, c7 = s5, 15 * s7
            lam = m[k] * la[jj] - m[jj] * la[k]
            mu = m[k] * lj[jj] - m[jj] * lj[k]
            rv, rm, rl, vm = r @ w, r @ mu, r @ lam, w @ mu
            gx[k] += (lam * s3 - 3 * rl * r * s5 - 3 * vm * r * s5
                      - 3 * (rm * w + rv * mu) * qs + c7 * rv * rm * r)
            gv[k] += mu * s3 - 3 * rm * r * qs
            gm[k] -= la[jj] @ r * s3 + lj[jj] @ (w * s3 - 3 * rv * r * qs)
    return gx, gv, gm


def _adjoint(x0, v0, m, eps2, h, nsteps, lx, lv, jerk):
    # forward, keeping the predicted states
    x, v = x0.copy(), v0.copy()
    a, j = _forces(x, v, m, eps2, jerk)
    preds = []
    for _ in range(nsteps):
        xp = x + (v * h + a * h * h / 2 + j * h ** 3 / 6)
        vp = v + (a * h + j * h * h / 2)
        preds.append((xp, vp))
        a1, j1 = _forces(xp, vp, m, eps2, jerk)
        vn = v + (a + a1) * h / 2 + (j - j1) * h * h / 12
        x = x + (v + vn) * h / 2 + (a - a1) * h * h / 12
        v, a, j = vn, a1, j1
    la = np.zeros_like(x0); lj = np.zeros_like(x0); lm = np.zeros_like(m)
    for xp, vp in reversed(preds):
        lvt = lv + lx * h / 2
        la1 = la - lx * h * h / 12 + lvt * h / 2
        lj1 = lj - lvt * h * h / 12
        lx, lv, la, lj = (lx, lx * h / 2 + lvt, lx * h * h / 12 + lvt * h / 2,
                          lvt * h * h / 12)
        gx, gv, gm = _force_vjp(xp, vp, m, eps2, la1, lj1, jerk)
        lx = lx + gx
        lv = lv + gx * h + gv
        la = la + gx * h * h / 2 + gv * h
        lj = lj + gx * h ** 3 / 6 + gv * h * h / 2
        lm = lm + gm
    gx, gv, gm = _force_vjp(x0, v0, m, eps2, la, lj, jerk)
    return lx + gx, lv + gv, lm + gm


@pytest.mark.parametrize("jerk", ["hermite", "softened"])
@pytest.mark.parametrize("eps2", [0.0, 1e-2])
def test_adjoint_equations_match_autograd(eps2, jerk):
    from amuse_gb300 import ic
    rng = np.random.RandomState(11)
    m, x, v = ic.plummer(12, do_scale=True, rng=rng)
    m = m * rng.uniform(0.5, 1.5, len(m))
    w = rng.uniform(0.5, 1.5, len(m))
    h, nsteps = 1 / 128, 6
    tx = torch.tensor(x, requires_grad=True)
    tv = torch.tensor(v, requires_grad=True)
    tm = torch.tensor(m, requires_grad=True)
    xf, vf = ht.run(tx, tv, tm, eps2, h, nsteps, jerk)
    loss = ht.loss(xf, torch.tensor(w)) + (vf * vf).sum()
    loss.backward()
    lx = 2 * w[:, None] * xf.detach().numpy()
    lv = 2 * vf.detach().numpy()
    gx, gv, gm = _adjoint(x, v, m, eps2, h, nsteps, lx, lv, jerk)
    np.testing.assert_allclose(gx, tx.grad.numpy(), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(gv, tv.grad.numpy(), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(gm, tm.grad.numpy(), rtol=1e-10, atol=1e-12)


def test_jerk_forms_differ_only_when_softened():
    from amuse_gb300 import ic
    rng = np.random.RandomState(6)
    m, x, v = (torch.tensor(a) for a in ic.plummer(32, do_scale=True, rng=rng))
    a0, j0 = ht.forces(x, v, m, 0.0, "hermite")
    a1, j1 = ht.forces(x, v, m, 0.0, "softened")
    assert torch.equal(a0, a1)
    # they differ only through the 2^-52 softening term
    assert (j0 - j1).abs().max() <= 1e-12 * j1.abs().max()
    _, j2 = ht.forces(x, v, m, 1e-2, "hermite")
    _, j3 = ht.forces(x, v, m, 1e-2, "softened")
    assert (j2 - j3).abs().max() > 1e-3 * j3.abs().max()
