"""Batched multiples hand-off: many close encounters resolved at once.

AMUSE's multiples module resolves one encounter at a time: it hands the
encounter's particles to a smallN worker and advances it in increments until
smallN's structure analysis calls the interaction over
(`Multiples.resolve_collision`, src/amuse/couple/multiples.py:1722-1880).
`resolve_encounters` takes a list of such encounters and advances all of them
together on the GPU batch kernel (g6x_batch_run, smallN's scheme, one warp
per system), checking each system's structure on the host after every
increment (g6x_check_structure_batch: smallN's check_structure restated,
on the host's cores) and retiring the systems whose interaction is over;
the others continue in the next launch.  `resolve_serial` is the same loop
for one encounter around any host integrator.

Kept from resolve_collision's loop: increments of `delta_t` (its
"initial_delta_t": it checks is_over after every such substep, whatever its
outer step has grown to), the end time, smallN's quasi-stable ending and the
break scale.  Quasi-stable (over = 2, analyze.cc:909-990, 1031-1039): every
top-level node escapes but not all are stable, and the top-level grouping
has been the same at more than 15 consecutive checks.  smallN keeps that
history in file statics shared by all the encounters its worker resolves;
here each encounter has its own, starting empty.  Break scale (over = 3,
analyze.cc:1050-1059): after an increment that did not end the encounter,
a top-level body farther than `break_scale` from the origin of the system's
frame (between increments every body is top-level in the integrator's
tree).  smallN itself also stops inside an increment once a top-level
body passes the break scale (every NCHECK steps, smallN.cc:1008-1017); here
the break-scale ending comes at the end of that increment.

Retries (`min_break_scale`, resolve_collision's loop over loop_count,
multiples.py:1763-2090): an encounter that has not ended by `end_time` is
run again from its initial conditions, up to 10 passes in all, with the
break scale multiplied by (min_break_scale / break_scale)^(2/10) at each
pass.  Under Python 3 resolve_collision never takes its other branch (the
end-time extension: `2*(loop_count/2) != loop_count` is never true with true
division), so a pass differs from the one before only in its break scale.
The integration is deterministic, so a pass replays the same checks: the
over and quasi-stable decisions fire at the same checks as in the first
pass (none, by the end time), and only the break scale can end it.  Each
pass is therefore decided from the first pass's recorded checks (the
largest body distance and the state at each), without integrating again.
An encounter that no pass ends comes back with over = 0, where
resolve_collision raises DidNotFinishException.  Each increment restarts
the integrator from the returned state: unperturbed binaries are resolved
at the end of an increment and found again in the next.
"""
import time

import numpy as np

import amuse_gb300 as ag


def resolve_encounters(g6, systems, end_time, delta_t, break_scale=np.inf, mode="split",
                       unperturbed=True, eta=0.14, max_steps=2_000_000, timing=None,
                       min_break_scale=None):
    """Advance every encounter until its interaction is over or end_time.

    systems: list of (mass[n], pos[n][3], vel[n][3]), n <= 64, each in its
    own frame (G = 1).  end_time, delta_t, break_scale: scalars or one per
    system.  Returns a list of dicts, one per system: pos, vel, time (the
    integrated time), over (0 not over by end_time, 1 over, 2 quasi-stable,
    3 beyond the break scale), summary (the structure as
    g6x_check_structure writes it), top_of, checks (how many increments it
    took, in the pass that ended it), passes (1, or the retry that ended
    it), steps, status (the batch status of its last increment: 0, or 1 if
    it stopped at max_steps), energy (initial and final total energy).
    min_break_scale (scalar or one per system, with a finite break_scale):
    the retries of resolve_collision.  unperturbed: smallN's unperturbed
    binaries on for these launches (switched off again on return).  timing
    (a dict, optional) receives launches, batch_s (wall time of the batch
    calls, copies included), check_s (the structure checks) and the active
    systems per launch."""
    ns = len(systems)
    end_time = np.broadcast_to(np.asarray(end_time, float), (ns,))
    delta_t = np.broadcast_to(np.asarray(delta_t, float), (ns,))
    rlim2 = np.broadcast_to(np.asarray(break_scale, float) ** 2, (ns,))
    retry = min_break_scale is not None
    if retry:
        if not np.isfinite(rlim2).all():
            raise ValueError("retries need a finite break_scale")
        # the squared break scale shrinks by this factor from one pass to the next
        fac2 = (np.broadcast_to(np.asarray(min_break_scale, float), (ns,)) ** 2 / rlim2) \
            ** (2.0 / LOOP_MAX)
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
    # smallN's state at the last check: per body the rank of its top-level
    # node (equal ranks over a system: the same grouping in the same order)
    RANK = np.full(len(M), -1, np.int32)
    state_count = np.zeros(ns, np.int64)
    passes = np.ones(ns, np.int32)
    status = np.zeros(ns, np.int32)
    record = [[] for _ in range(ns)] if retry else None  # the first pass's checks
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
            status[active] = r["status"]
            starts = np.concatenate([[0], np.cumsum(na)[:-1]])
            same = np.logical_and.reduceat(c["top_rank"] == RANK[bodies], starts)
            state_count[active] = np.where(same, state_count[active] + 1, 0)
            RANK[bodies] = c["top_rank"]
            over[active[c["over"]]] = 1
            over[active[~c["over"] & c["escaping"] & (state_count[active] > QSTABLE_COUNT)]] = 2
            if np.isfinite(rlim2[active]).any():
                r2 = np.einsum("ij,ij->i", r["pos"], r["pos"])
                far = np.maximum.reduceat(r2, starts)
                hit = (over[active] == 0) & (far > rlim2[active])
                over[active[hit]] = 3
                if retry:
                    for q, s in enumerate(active):
                        a, b = off[s], off[s + 1]
                        record[s].append((far[q], t[s], steps[s], X[a:b].copy(), V[a:b].copy(),
                                          TOP[a:b].copy(), c["summary"][q]))
            go = (over[active] == 0) & (t[active] < end_time[active] * (1 - 1e-12)) \
                & (r["status"] == 0)
            for q, s in enumerate(active):
                summary[s] = c["summary"][q]
            if retry:
                for q in np.flatnonzero(~go & (over[active] == 0) & (r["status"] == 0)):
                    s = active[q]
                    p, k = _retry_pass(record[s], rlim2[s], fac2[s])
                    if p:
                        _, t[s], steps[s], x_k, v_k, top_k, summary[s] = record[s][k]
                        a, b = off[s], off[s + 1]
                        X[a:b], V[a:b], TOP[a:b] = x_k, v_k, top_k
                        over[s], passes[s], checks[s] = 3, p, k + 1
                    record[s] = []
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
                        checks=int(checks[k]), passes=int(passes[k]), steps=int(steps[k]),
                        status=int(status[k]),
                        energy=(e0[k], _energy(M[a:b], X[a:b], V[a:b]))))
    return out


def resolve_serial(integrate, m, x, v, end_time, delta_t, break_scale=np.inf):
    """One encounter the way resolve_collision runs it, with any host
    integrator: integrate(m, x, v, dt) -> (x, v, dt_done) advances the
    system by one increment.  The same decisions as resolve_encounters
    (structure check, smallN's quasi-stable history, break scale; no
    retries).  Returns (over, summary, checks, time, x, v)."""
    m = np.asarray(m, float)
    x = np.array(x, float).reshape(-1, 3)
    v = np.array(v, float).reshape(-1, 3)
    t, checks, last, count, summary = 0.0, 0, None, 0, ""
    while t < end_time * (1 - 1e-12):
        x, v, dt = integrate(m, x, v, min(delta_t, end_time - t))
        t += dt
        checks += 1
        c = ag.check_structure(m, x, v)
        summary = c["summary"]
        g = grouping(summary)
        count = count + 1 if g == last else 0
        last = g
        if c["over"]:
            return 1, summary, checks, t, x, v
        if c["escaping"] and count > QSTABLE_COUNT:
            return 2, summary, checks, t, x, v
        if np.isfinite(break_scale) and (x * x).sum(1).max() > break_scale ** 2:
            return 3, summary, checks, t, x, v
    return 0, summary, checks, t, x, v


# resolve_collision's loop_max: passes over one encounter in all
LOOP_MAX = 10


def _retry_pass(rec, rlim2, fac2):
    """The first retry pass (2 .. LOOP_MAX) whose break scale one of the
    recorded checks passes, and that check; (0, -1) if none."""
    far = np.array([e[0] for e in rec])
    for p in range(2, LOOP_MAX + 1):
        hit = np.flatnonzero(far > rlim2 * fac2 ** (p - 1))
        if len(hit):
            return p, int(hit[0])
    return 0, -1


# smallN's min_qstable_count: quasi-stable once the grouping has been
# unchanged at more than this many consecutive checks (analyze.cc:909-950)
QSTABLE_COUNT = 15


def grouping(summary):
    """The top-level grouping of a structure summary, in the order of the
    top-level nodes: smallN's state string (analyze.cc:771-821) holds the
    same information (each node's leaves, not its inner structure)."""
    out = []
    for tok in summary.split():
        ids = tok.replace("(", " ").replace(")", " ").replace(",", " ").split()
        out.append(tuple(sorted(int(i) for i in ids)))
    return tuple(out)


def _energy(m, x, v):
    k = 0.5 * np.sum(m * np.sum(v * v, 1))
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt(np.sum(d * d, -1))
    iu = np.triu_indices(len(m), 1)
    return k - np.sum(m[iu[0]] * m[iu[1]] / r[iu])
