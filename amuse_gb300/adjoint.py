"""Differentiable fixed-step Hermite integration (reverse mode).

The forward map is the hermite code's shared fixed-step scheme
(src/amuse_hermite/interface.cc: ``predict_step`` :266-281, ``evolve_step``
:558-616, ``correct_step`` :536-552, with ``test_mode`` making the step the
constant ``dt_param``, :618-637), evaluated with this library's pair force
(split precision or FP64).  The reverse pass is the exact discrete adjoint of
that map, run by hand-written kernels (``g6x_fixed_step_adjoint`` and
``g6x_force_vjp``); nothing here is traced or differentiated by torch.

Memory: the state (x, v, a, j) is checkpointed every ``checkpoint`` steps on
the forward pass.  The backward pass walks the segments last to first,
recomputes each segment from its checkpoint keeping the predicted states
(xp, vp) the forces were evaluated at, and runs the step adjoints through it.
Peak extra memory is (nsteps / checkpoint) * 12n + checkpoint * 6n doubles.

Usage::

    x, v = hermite_fixed(x0, v0, m, eps2=1e-4, dt=1/256, nsteps=256)
    loss = (w * (x * x).sum(1)).sum()
    loss.backward()              # x0.grad, v0.grad, m.grad

x0, v0 are (n, 3) and m is (n,) float64 CUDA tensors.
"""
from __future__ import annotations

import torch

from . import FP64, G6X, JERK_HERMITE, JERK_SOFTENED, SPLIT

_ctx = {}


def context(device=0):
    """The library context of ``device`` (opened once per process)."""
    if device not in _ctx:
        _ctx[device] = G6X(device)
    return _ctx[device]


def _p(t):
    return t.data_ptr()


class _Run:
    """Fixed-step runner bound to one library context and precision."""

    def __init__(self, g6, n, eps2, dt, precision, jerk):
        self.g6, self.n, self.eps2, self.dt = g6, n, float(eps2), float(dt)
        self.prec = FP64 if precision == "fp64" else SPLIT
        self.jerk = JERK_SOFTENED if jerk == "softened" else JERK_HERMITE

    def __enter__(self):
        self.old = self.g6.get_precision()
        self.g6.set_precision(self.prec)
        self.g6.set_fixed_jerk(self.jerk)
        return self

    def __exit__(self, *exc):
        self.g6.set_precision(self.old)

    def force(self, x, v, m):
        a = torch.empty_like(x)
        j = torch.empty_like(x)
        self.g6.fixed_force(self.n, self.eps2, _p(x), _p(v), _p(m), _p(a), _p(j))
        return a, j

    def run(self, x, v, a, j, m, nsteps, xps=None, vps=None):
        """nsteps steps in place; xps/vps ([nsteps, n, 3]) keep the predicted states."""
        self.g6.fixed_run(self.n, self.dt, self.eps2, nsteps, _p(x), _p(v), _p(a), _p(j), _p(m),
                          None if xps is None else _p(xps), None if vps is None else _p(vps))

    def adjoint_run(self, xps, vps, m, lx, lv, la, lj, lm, work):
        self.g6.fixed_adjoint_run(self.n, self.dt, self.eps2, xps.shape[0], _p(xps), _p(vps),
                                  _p(m), _p(lx), _p(lv), _p(la), _p(lj), _p(lm), _p(work))


def _check_inputs(x0, v0, m):
    for t, shape in ((x0, (-1, 3)), (v0, (-1, 3)), (m, (-1,))):
        if not t.is_cuda or t.dtype != torch.float64:
            raise TypeError("hermite_fixed wants float64 CUDA tensors")
        if t.dim() != len(shape) or (len(shape) == 2 and t.shape[1] != 3):
            raise ValueError("x0, v0 must be (n, 3) and m (n,)")
    if not (x0.shape[0] == v0.shape[0] == m.shape[0]):
        raise ValueError("x0, v0, m disagree on n")


class HermiteFixedFunction(torch.autograd.Function):
    """(x0, v0, m) -> (x, v) after ``nsteps`` fixed Hermite steps."""

    @staticmethod
    def forward(ctx, x0, v0, m, eps2, dt, nsteps, checkpoint, precision, jerk, device):
        _check_inputs(x0, v0, m)
        g6 = context(device)
        n = x0.shape[0]
        stream = torch.cuda.ExternalStream(g6.stream(), device=x0.device)
        stream.wait_stream(torch.cuda.current_stream(x0.device))
        with torch.cuda.stream(stream), _Run(g6, n, eps2, dt, precision, jerk) as r:
            x, v, mm = x0.detach().clone(), v0.detach().clone(), m.detach().contiguous()
            a, j = r.force(x, v, mm)
            ckpt = []
            for s0 in range(0, nsteps, checkpoint):
                ckpt.append(torch.stack((x, v, a, j)))
                r.run(x, v, a, j, mm, min(checkpoint, nsteps - s0))
        torch.cuda.current_stream(x0.device).wait_stream(stream)
        ctx.save_for_backward(x0, v0, mm, *ckpt)
        ctx.cfg = (eps2, dt, nsteps, checkpoint, precision, jerk, device)
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        x0, v0, m, *ckpt = ctx.saved_tensors
        eps2, dt, nsteps, checkpoint, precision, jerk, device = ctx.cfg
        g6 = context(device)
        n = x0.shape[0]
        stream = torch.cuda.ExternalStream(g6.stream(), device=x0.device)
        stream.wait_stream(torch.cuda.current_stream(x0.device))
        with torch.cuda.stream(stream), _Run(g6, n, eps2, dt, precision, jerk) as r:
            lx = gx.clone() if gx is not None else torch.zeros_like(x0)
            lv = gv.clone() if gv is not None else torch.zeros_like(x0)
            la, lj = torch.zeros_like(x0), torch.zeros_like(x0)
            lm = torch.zeros_like(m)
            work = torch.empty(7 * n, dtype=torch.float64, device=x0.device)
            for c in range(len(ckpt) - 1, -1, -1):
                s0 = c * checkpoint
                k = min(checkpoint, nsteps - s0)
                x, v, a, j = (t.clone() for t in ckpt[c])
                xps = torch.empty((k, n, 3), dtype=torch.float64, device=x0.device)
                vps = torch.empty_like(xps)
                r.run(x, v, a, j, m, k, xps, vps)
                r.adjoint_run(xps, vps, m, lx, lv, la, lj, lm, work)
            # initial forces (a0, j0) = F(x0, v0, m)
            gx0, gv0 = torch.empty_like(x0), torch.empty_like(x0)
            gm0 = torch.empty_like(m)
            g6.force_vjp(n, float(eps2), _p(x0.contiguous()), _p(v0.contiguous()), _p(m), _p(la),
                         _p(lj), _p(gx0), _p(gv0), _p(gm0))
            lx += gx0
            lv += gv0
            lm += gm0
        torch.cuda.current_stream(x0.device).wait_stream(stream)
        return lx, lv, lm, None, None, None, None, None, None, None


def hermite_fixed(x0, v0, m, *, eps2, dt, nsteps, checkpoint=16, precision="split",
                  jerk="hermite", device=0):
    """Integrate ``nsteps`` fixed Hermite steps of size dt; differentiable in
    (x0, v0, m) through the hand-written adjoint.  precision: "split"
    (double-single positions, FP32 pair arithmetic) or "fp64".  jerk:
    "hermite" (the hermite code's form, whose (r.v) factor uses the
    unsoftened r^2) or "softened" (the exact derivative of the softened
    acceleration, as ph4 and the g6 force); equal when eps2 = 0."""
    if precision not in ("split", "fp64"):
        raise ValueError("precision must be 'split' or 'fp64'")
    if jerk not in ("hermite", "softened"):
        raise ValueError("jerk must be 'hermite' or 'softened'")
    if nsteps < 1 or checkpoint < 1:
        raise ValueError("nsteps and checkpoint must be positive")
    return HermiteFixedFunction.apply(x0, v0, m, float(eps2), float(dt), int(nsteps),
                                      int(checkpoint), precision, jerk, device)


def final_forces(x, v, m, *, eps2, precision="split", jerk="hermite", device=0):
    """(acc, jerk) of the state (x, v) (no gradient)."""
    g6 = context(device)
    stream = torch.cuda.ExternalStream(g6.stream(), device=x.device)
    stream.wait_stream(torch.cuda.current_stream(x.device))
    with torch.cuda.stream(stream), _Run(g6, x.shape[0], eps2, 0.0, precision, jerk) as r:
        a, j = r.force(x.detach().contiguous(), v.detach().contiguous(), m.detach().contiguous())
    torch.cuda.current_stream(x.device).wait_stream(stream)
    return a, j
