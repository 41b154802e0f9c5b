"""Batched multiples hand-off: many close encounters resolved at once.

AMUSE's multiples module resolves one encounter at a time: it hands the
encounter's particles to a smallN worker and advances it in increments until
smallN's structure analysis calls the interaction over
(`Multiples.resolve_collision`, src/amuse/couple/multiples.py:1722-1880).
`resolve_encounters` takes a list of such encounters and advances all of them
together on the GPU batch kernel (g6x_batch_run, smallN's scheme, one warp
per system), checking each system's structure on the host after every
increment (g6x_check_structure, smallN's check_structure restated) and
retiring the systems whose interaction is over; the others continue in the
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
    state = []
    for m, x, v in systems:
        m = np.asarray(m, float)
        if not 2 <= len(m) <= 64:
            raise ValueError("encounters of 2 to 64 bodies")
        state.append(dict(m=m, x=np.array(x, float).reshape(-1, 3),
                          v=np.array(v, float).reshape(-1, 3), t=0.0, steps=0, checks=0,
                          over=0, summary="", top_of=None))
    e0 = [_energy(s["m"], s["x"], s["v"]) for s in state]
    active = list(range(ns))
    t_batch = t_check = 0.0
    per_launch = []
    if unperturbed:
        g6.batch_unperturbed(True)
    try:
        while active:
            # one batch launch per increment for every system still running
            dts = np.array([min(delta_t[s], end_time[s] - state[s]["t"]) for s in active])
            nper = np.array([len(state[s]["m"]) for s in active], np.int32)
            per_launch.append(len(active))
            t0 = time.perf_counter()
            r = g6.batch_run(nper, dts, np.concatenate([state[s]["m"] for s in active]),
                             np.concatenate([state[s]["x"] for s in active]),
                             np.concatenate([state[s]["v"] for s in active]), eta=eta,
                             max_steps=max_steps, mode=mode)
            t1 = time.perf_counter()
            t_batch += t1 - t0
            off = np.concatenate([[0], np.cumsum(nper)])
            still = []
            for q, s in enumerate(active):
                st = state[s]
                st["x"] = r["pos"][off[q]:off[q + 1]].copy()
                st["v"] = r["vel"][off[q]:off[q + 1]].copy()
                st["t"] += float(r["t_final"][q])
                st["steps"] += int(r["steps"][q])
                st["checks"] += 1
                c = ag.check_structure(st["m"], st["x"], st["v"])
                st["summary"], st["top_of"] = c["summary"], c["top_of"]
                if c["over"]:
                    st["over"] = 1
                elif np.isfinite(rlim2[s]) and _beyond(st, c["top_of"], rlim2[s]):
                    st["over"] = 3
                elif st["t"] < end_time[s] * (1 - 1e-12) and r["status"][q] == 0:
                    still.append(s)
            active = still
            t_check += time.perf_counter() - t1
    finally:
        if unperturbed:
            g6.batch_unperturbed(False)
    if timing is not None:
        timing.update(launches=len(per_launch), batch_s=t_batch, check_s=t_check,
                      active_per_launch=per_launch)
    return [dict(pos=st["x"], vel=st["v"], time=st["t"], over=st["over"],
                 summary=st["summary"], top_of=st["top_of"], checks=st["checks"],
                 steps=st["steps"], energy=(e0[k], _energy(st["m"], st["x"], st["v"])))
            for k, st in enumerate(state)]


def _beyond(st, top_of, rlim2):
    """A top-level node (its centre of mass) farther than the break scale
    from the origin of the system's frame."""
    for t in np.unique(top_of):
        sel = top_of == t
        m = st["m"][sel]
        cm = (m[:, None] * st["x"][sel]).sum(0) / m.sum()
        if cm @ cm > rlim2:
            return True
    return False


def _energy(m, x, v):
    k = 0.5 * np.sum(m * np.sum(v * v, 1))
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt(np.sum(d * d, -1))
    iu = np.triu_indices(len(m), 1)
    return k - np.sum(m[iu[0]] * m[iu[1]] / r[iu])
