"""Batched multiples hand-off: many close encounters resolved at once.

AMUSE's multiples module resolves one encounter at a time: it hands the
encounter's particles to a smallN worker and advances it in increments until
smallN's structure analysis calls the interaction over
(`Multiples.resolve_collision`, src/amuse/couple/multiples.py:1722-1880).
`resolve_encounters` takes a list of such encounters and advances all of them
together on the GPU batch kernel (g6x_batch_run, smallN's scheme, one warp
per system), checking each system's structure on the host after every
increment (g6x_check_structure_batch: smallN's check_structure restated,
on the host's cores) and retiring the systems whose interaction is over; the others continue in the
next launch.

Kept from resolve_collision's loop: increments of `delta_t` (its
"initial_delta_t": it checks is_over after every such substep, whatever its
outer step has grown to), the end time, the break scale (a top-level node
farther than `break_scale` from the origin of the system's frame ends the
encounter with over = 3, as smallN's is_over(rlimit)).  Not kept: the
retries with perturbed initial conditions when an encounter does not end by
`end_time` (those are returned with over = 0 for the caller to decide), and
the quasi-stable termination (over = 2), which smallN takes from a history
of repeated states.  Each increment restarts the integrator from the
returned state: unperturbed binaries are resolved at the end of an increment
and found again in the next.
"""
import time

import numpy as np

import amuse_gb300 as ag


def resolve_encounters(g6, systems, end_time, delta_t, break_scale=np.inf, mode="split",
                       unperturbed=True, eta=0.14, max_steps=2_000_000, timing=None):
    """Advance every encounter until its interaction is over or end_time.

    systems: list of (mass[n], pos[n][3], vel[n][3]), n <= 64, each in its
    own frame (G = 1).  end_time, delta_t, break_scale: scalars or one per
    system.  Returns a list of dicts, one per system: pos, vel, time (the
    integrated time), over (0 not over by end_time, 1 over, 3 beyond the
    break scale), summary (the structure as g6x_check_structure writes it),
    top_of, checks (how many increments it took), steps, energy (initial and
    final total energy).  timing (a dict, optional) receives launches,
    batch_s (wall time of the batch calls, copies included), check_s (the
    structure checks) and the active systems per launch."""
    ns = len(systems)
    end_time = np.broadcast_to(np.asarray(end_time, float), (ns,))
    delta_t = np.broadcast_to(np.asarray(delta_t, float), (ns,))
    rlim2 = np.broadcast_to(np.asarray(break_scale, float) ** 2, (ns,))
    # all bodies in flat arrays; system s owns bodies off[s] .. off[s+1]-1
    nper = np.array([len(m) for m, _, _ in systems], np.int32)
    if ns and (nper.min() < 2 or nper.max() > 64):
        raise ValueError("encounters of 2 to 64 bodies")
    off = np.concatenate([[0], np.cumsum(nper)]).astype(np.int64)
    M = np.concatenate([np.asarray(m, float) for m, _, _ in systems]) if ns else np.zeros(0)
    X = np.concatenate([np.asarray(x, float).reshape(-1, 3) for _, x, _ in systems]) \
        if ns else np.zeros((0, 3))
    V = np.concatenate([np.asarray(v, float).reshape(-1, 3) for _, _, v in systems]) \
        if ns else np.zeros((0, 3))
    TOP = np.zeros(len(M), np.int32)
    t = np.zeros(ns)
    steps = np.zeros(ns, np.int64)
    checks = np.zeros(ns, np.int64)
    over = np.zeros(ns, np.int32)
    summary = [""] * ns
    e0 = [_energy(M[off[k]:off[k + 1]], X[off[k]:off[k + 1]], V[off[k]:off[k + 1]])
          for k in range(ns)]
    active = np.arange(ns)
    t_batch = t_check = 0.0
    per_launch = []
    if unperturbed:
        g6.batch_unperturbed(True)
    try:
        while len(active):
            # one batch launch per increment for every system still running
            na = nper[active]
            bodies = np.repeat(off[active] - np.concatenate([[0], np.cumsum(na)[:-1]]), na) \
                + np.arange(int(na.sum()))
            dts = np.minimum(delta_t[active], end_time[active] - t[active])
            per_launch.append(len(active))
            t0 = time.perf_counter()
            r = g6.batch_run(na, dts, M[bodies], X[bodies], V[bodies], eta=eta,
                             max_steps=max_steps, mode=mode)
            t1 = time.perf_counter()
            t_batch += t1 - t0
            # every system's structure at once, on the host's cores
            c = ag.check_structure_batch(na, M[bodies], r["pos"], r["vel"])
            X[bodies], V[bodies], TOP[bodies] = r["pos"], r["vel"], c["top_of"]
            t[active] += r["t_final"]
            steps[active] += r["steps"]
            checks[active] += 1
            for q in np.flatnonzero(c["over"]):
                over[active[q]] = 1
            if np.isfinite(rlim2[active]).any():
                for q, s in enumerate(active):
                    if not c["over"][q] and np.isfinite(rlim2[s]) and _beyond(
                            M[off[s]:off[s + 1]], X[off[s]:off[s + 1]],
                            TOP[off[s]:off[s + 1]], rlim2[s]):
                        over[s] = 3
            go = (over[active] == 0) & (t[active] < end_time[active] * (1 - 1e-12)) \
                & (r["status"] == 0)
            for q, s in enumerate(active):
                summary[s] = c["summary"][q]
            active = active[go]
            t_check += time.perf_counter() - t1
    finally:
        if unperturbed:
            g6.batch_unperturbed(False)
    if timing is not None:
        timing.update(launches=len(per_launch), batch_s=t_batch, check_s=t_check,
                      active_per_launch=per_launch)
    out = []
    for k in range(ns):
        a, b = off[k], off[k + 1]
        out.append(dict(pos=X[a:b].copy(), vel=V[a:b].copy(), time=float(t[k]),
                        over=int(over[k]), summary=summary[k], top_of=TOP[a:b].copy(),
                        checks=int(checks[k]), steps=int(steps[k]),
                        energy=(e0[k], _energy(M[a:b], X[a:b], V[a:b]))))
    return out


def _beyond(m_all, x_all, top_of, rlim2):
    """A top-level node (its centre of mass) farther than the break scale
    from the origin of the system's frame."""
    for t in np.unique(top_of):
        sel = top_of == t
        m = m_all[sel]
        cm = (m[:, None] * x_all[sel]).sum(0) / m.sum()
        if cm @ cm > rlim2:
            return True
    return False


def _energy(m, x, v):
    k = 0.5 * np.sum(m * np.sum(v * v, 1))
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt(np.sum(d * d, -1))
    iu = np.triu_indices(len(m), 1)
    return k - np.sum(m[iu[0]] * m[iu[1]] / r[iu])
