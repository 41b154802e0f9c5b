"""Plain-torch FP64 restatement of the fixed-step Hermite map (test helper).

The scheme is the hermite code's (src/amuse_hermite/interface.cc:
predict_step :266-281, correct_step :536-552, evolve_step :558-616) with
either jerk form: "hermite" (interface.cc:440-449,486: the (r.v) factor
divided by the unsoftened r^2) or "softened" (ph4's, src/amuse_ph4/src/
idata.cc:147-237: 3 (r.v)/(r^2 + eps^2)); softening eps^2 + 2^-52 as the GPU
force.  Written with differentiable torch ops so that autograd gives an
independent FP64 reference gradient for the hand-written adjoint kernels;
CPU, small n only.
"""
import torch

TINY = 2.0 ** -52


def forces(x, v, m, eps2, jerk="hermite"):
    r = x[None, :, :] - x[:, None, :]          # r[i, j] = x_j - x_i
    w = v[None, :, :] - v[:, None, :]
    n = x.shape[0]
    s = (r * r).sum(-1) + (eps2 + TINY)
    eye = torch.eye(n, dtype=torch.bool, device=x.device)
    s = torch.where(eye, torch.ones_like(s), s)
    s3 = s ** -1.5
    rv = (r * w).sum(-1)
    q = (r * r).sum(-1) if jerk == "hermite" else s
    q = torch.where(eye, torch.ones_like(q), q)
    mj = torch.where(eye, torch.zeros_like(s), m[None, :].expand(n, n))
    a = (mj[..., None] * r * s3[..., None]).sum(1)
    j = (mj[..., None] * (w - 3.0 * (rv / q)[..., None] * r) * s3[..., None]).sum(1)
    return a, j


def run(x0, v0, m, eps2, dt, nsteps, jerk="hermite"):
    x, v = x0, v0
    a, j = forces(x, v, m, eps2, jerk)
    for _ in range(nsteps):
        xp = x + (v * dt + a * dt * dt / 2 + j * dt * dt * dt / 6)
        vp = v + (a * dt + j * dt * dt / 2)
        a1, j1 = forces(xp, vp, m, eps2, jerk)
        vn = v + (a + a1) * dt / 2 + (j - j1) * dt * dt / 12
        x = x + (v + vn) * dt / 2 + (a - a1) * dt * dt / 12
        v, a, j = vn, a1, j1
    return x, v


def loss(x, w):
    """Sum of squared final positions weighted by w."""
    return (w * (x * x).sum(1)).sum()
