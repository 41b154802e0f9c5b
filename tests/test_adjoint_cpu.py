"""CPU checks for the fixed-step Hermite path and its adjoint.

* the oracle's restatement of the hermite code (orc_hermite_fixed) against
  the reference test's known answer (src/amuse_hermite/tests/
  test_hermite.py:86-113: an equal-mass circular binary returns to its
  mirror position after half a period and to its start after a period, to
  3 decimals) and against the torch restatement at eps2 = 0;
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


def test_oracle_hermite_matches_torch_unsoftened(lib_built):
    """With eps2 = 0 the hermite jerk equals the library's (ph4) jerk."""
    import oracle
    from amuse_gb300 import ic
    rng = np.random.RandomState(5)
    m, x, v = ic.plummer(48, do_scale=True, rng=rng)
    p, vv, a, j = oracle.hermite_fixed(m, x, v, 0.0, 1 / 512, 32)
    tx, tv = ht.run(torch.tensor(x), torch.tensor(v), torch.tensor(m), 0.0, 1 / 512, 32)
    np.testing.assert_allclose(p, tx.numpy(), rtol=0, atol=1e-11)
    np.testing.assert_allclose(vv, tv.numpy(), rtol=0, atol=1e-10)


# ---- numpy restatement of the kernels' adjoint arithmetic ----

def _forces(x, v, m, eps2):
    a, j = ht.forces(torch.tensor(x), torch.tensor(v), torch.tensor(m), eps2)
    return a.numpy(), j.numpy()


def _force_vjp(x, v, m, eps2, la, lj):
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
            lam = m[k] * la[jj] - m[jj] * la[k]
            mu = m[k] * lj[jj] - m[jj] * lj[k]
            rv, rm, rl, vm = r @ w, r @ mu, r @ lam, w @ mu
            gx[k] += (lam * s3 - 3 * rl * r * s5
                      - 3 * (vm * r + rm * w + rv * mu) * s5 + 15 * rv * rm * r * s7)
            gv[k] += mu * s3 - 3 * rm * r * s5
            gm[k] -= la[jj] @ r * s3 + lj[jj] @ (w * s3 - 3 * rv * r * s5)
    return gx, gv, gm


def _adjoint(x0, v0, m, eps2, h, nsteps, lx, lv):
    # forward, keeping the predicted states
    x, v = x0.copy(), v0.copy()
    a, j = _forces(x, v, m, eps2)
    a0, j0 = a, j
    preds = []
    for _ in range(nsteps):
        xp = x + (v * h + a * h * h / 2 + j * h ** 3 / 6)
        vp = v + (a * h + j * h * h / 2)
        preds.append((xp, vp))
        a1, j1 = _forces(xp, vp, m, eps2)
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
        gx, gv, gm = _force_vjp(xp, vp, m, eps2, la1, lj1)
        lx = lx + gx
        lv = lv + gx * h + gv
        la = la + gx * h * h / 2 + gv * h
        lj = lj + gx * h ** 3 / 6 + gv * h * h / 2
        lm = lm + gm
    gx, gv, gm = _force_vjp(x0, v0, m, eps2, la, lj)
    return lx + gx, lv + gv, lm + gm


@pytest.mark.parametrize("eps2", [0.0, 1e-2])
def test_adjoint_equations_match_autograd(eps2):
    from amuse_gb300 import ic
    rng = np.random.RandomState(11)
    m, x, v = ic.plummer(12, do_scale=True, rng=rng)
    m = m * rng.uniform(0.5, 1.5, len(m))
    w = rng.uniform(0.5, 1.5, len(m))
    h, nsteps = 1 / 128, 6
    tx = torch.tensor(x, requires_grad=True)
    tv = torch.tensor(v, requires_grad=True)
    tm = torch.tensor(m, requires_grad=True)
    xf, vf = ht.run(tx, tv, tm, eps2, h, nsteps)
    loss = ht.loss(xf, torch.tensor(w)) + (vf * vf).sum()
    loss.backward()
    lx = 2 * w[:, None] * xf.detach().numpy()
    lv = 2 * vf.detach().numpy()
    gx, gv, gm = _adjoint(x, v, m, eps2, h, nsteps, lx, lv)
    np.testing.assert_allclose(gx, tx.grad.numpy(), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(gv, tv.grad.numpy(), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(gm, tm.grad.numpy(), rtol=1e-10, atol=1e-12)
