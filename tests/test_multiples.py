"""The batched multiples hand-off (amuse_gb300.multiples.resolve_encounters):
its loop logic on the host against a direct restatement of
resolve_collision's loop (smallN, then smallN's own check_structure where
the reference build exists), and on the GPU batch kernel."""
import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from amuse_gb300 import multiples, workloads


def scattering(seed, v_inf=0.6, b_max=1.5, d0=15.0):
    return workloads.binary_single(seed, v_inf, b_max, d0)


class HostBatch:
    """Stands in for the GPU batch: the oracle's smallN restatement (no
    binary tree), which is bit-identical to smallN."""

    def batch_unperturbed(self, on=True):
        pass

    def batch_run(self, nper, t_end, mass, pos, vel, eta=0.14, max_steps=0, mode=None):
        off = np.concatenate([[0], np.cumsum(nper)])
        pos, vel = pos.copy(), vel.copy()
        tf = np.zeros(len(nper))
        steps = np.zeros(len(nper), np.int64)
        status = np.zeros(len(nper), np.int32)
        for s in range(len(nper)):
            a, b = off[s], off[s + 1]
            p, v, t, st = oracle.smalln(mass[a:b], pos[a:b], vel[a:b], eta, t_end[s],
                                        max_steps=max_steps)
            pos[a:b], vel[a:b], tf[s], steps[s] = p, v, t, st
            status[s] = 1 if max_steps and st >= max_steps and t < t_end[s] else 0
        return dict(pos=pos, vel=vel, t_final=tf, steps=steps, status=status)


def direct_loop(m, x, v, end_time, delta_t, structure):
    """resolve_collision's loop for one encounter, check after every
    delta_t substep; structure(m, x, v) -> (over, tree, hierarchy_tested)."""
    t = 0.0
    checks = 0
    hier = False
    while t < end_time * (1 - 1e-12):
        x, v, tf, _ = oracle.smalln(m, x, v, 0.14, min(delta_t, end_time - t))
        t += tf
        checks += 1
        over, tree, h = structure(m, x, v)
        hier |= h
        if over:
            return over, tree, checks, t, hier
    return 0, tree, checks, t, hier


def product_check():
    """The library's stateless check plus smallN's quasi-stable history,
    restated here from the top-level grouping in top_of: quasi-stable once
    every top-level node escapes without all being stable and the grouping
    has not changed for more than 15 consecutive checks."""
    hist = {"last": None, "count": 0}

    def f(m, x, v):
        c = ag.check_structure(m, x, v)
        top = c["top_of"]
        g = frozenset(tuple(np.flatnonzero(top == t)) for t in np.unique(top))
        hist["count"] = hist["count"] + 1 if g == hist["last"] else 0
        hist["last"] = g
        over = 1 if c["over"] else (2 if c["escaping"] and hist["count"] > 15 else 0)
        return over, c["summary"], c["hierarchy_tested"]
    return f


def smalln_check():
    """smallN's own check_structure (the reference build).  Its history is
    a file static shared by every call: one check of a two-body system
    first makes the next encounter's first grouping count as a change, so
    each encounter starts afresh, as in the library."""
    xb = np.array([[-0.5, 0, 0], [0.5, 0, 0]])
    vb = np.array([[0, -0.5, 0], [0, 0.5, 0]])
    oracle.check_structure_ref(np.array([0.5, 0.5]), xb, vb)
    return lambda m, x, v: oracle.check_structure_ref(m, x, v) + (False,)


def test_resolve_loop_matches_a_direct_loop():
    systems = [scattering(s) for s in range(12)]
    res = multiples.resolve_encounters(HostBatch(), systems, end_time=400.0, delta_t=10.0)
    n_over = 0
    for (m, x, v), r in zip(systems, res):
        over, tree, checks, t, _ = direct_loop(m, x, v, 400.0, 10.0, product_check())
        assert (r["over"], r["summary"], r["checks"]) == (over, tree, checks)
        assert r["time"] == t
        n_over += r["over"] in (1, 2)
    assert n_over >= 8  # most scatterings end well within the end time


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build absent")
def test_resolve_decisions_against_smalln():
    """The same loop with smallN's own check_structure, quasi-stable ending
    included: the outcomes agree, except where a multiple above a binary
    was judged (smallN: Mardling's nstab; here Mardling & Aarseth).  On the
    first 200 of these encounters all 200 agree, 41 of them quasi-stable."""
    systems = [scattering(s) for s in range(64)]
    res = multiples.resolve_encounters(HostBatch(), systems, end_time=400.0, delta_t=10.0)
    differ = quasi = 0
    for (m, x, v), r in zip(systems, res):
        ref = direct_loop(m, x, v, 400.0, 10.0, smalln_check())
        mine = direct_loop(m, x, v, 400.0, 10.0, product_check())
        quasi += ref[0] == 2
        if (ref[0], ref[1], ref[2]) == (r["over"], r["summary"], r["checks"]):
            continue
        differ += 1
        assert mine[4], (ref, mine)   # only where the hierarchy test ran
    print(f"{differ} of 64 differ; smallN ended {quasi} as quasi-stable")
    assert quasi >= 5 and differ <= 2


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build absent")
def test_binary_binary_decisions_against_smalln():
    """Binary-binary scatterings, where triples and quadruples form and the
    hierarchy test decides often: the loop's decisions equal those around
    smallN's own check_structure except where Mardling-Aarseth and nstab
    judge a multiple differently (on these 100 encounters: 98 identical,
    84 with a hierarchy test; the two others are triples nstab calls
    stable and Mardling-Aarseth does not)."""
    systems = [workloads.binary_binary(s) for s in range(100)]
    res = multiples.resolve_encounters(HostBatch(), systems, end_time=600.0, delta_t=10.0)
    differ = 0
    for (m, x, v), r in zip(systems, res):
        ref = direct_loop(m, x, v, 600.0, 10.0, smalln_check())
        if (ref[0], ref[1], ref[2]) == (r["over"], r["summary"], r["checks"]):
            continue
        differ += 1
        mine = direct_loop(m, x, v, 600.0, 10.0, product_check())
        assert mine[4], (ref, mine)
    assert differ <= 2


def retry_loop(m, x0, v0, end_time, delta_t, scale, min_scale, loop_max=10):
    """resolve_collision's retries as it runs them: every pass integrates
    again from the initial conditions, with the break scale multiplied by
    (min_scale / scale)^(2 / loop_max) from one pass to the next."""
    fac = (min_scale / scale) ** (2.0 / loop_max)
    for p in range(1, loop_max + 1):
        check = product_check()
        x, v, t, checks = x0, v0, 0.0, 0
        while t < end_time * (1 - 1e-12):
            x, v, tf, _ = oracle.smalln(m, x, v, 0.14, min(delta_t, end_time - t))
            t += tf
            checks += 1
            over, tree, _ = check(m, x, v)
            if not over and (x * x).sum(1).max() > scale ** 2:
                over = 3
            if over:
                return over, tree, checks, t, p, x
        scale *= fac
    return 0, tree, checks, t, loop_max, x


def test_retries_match_rerunning_each_pass():
    """Encounters stopped long before they can end (end time 40): the
    retries shrink the break scale until it ends them; the replay of the
    first pass's checks decides each as integrating every pass again does."""
    systems = [scattering(s) for s in range(10)]
    res = multiples.resolve_encounters(HostBatch(), systems, end_time=40.0, delta_t=10.0,
                                       break_scale=100.0, min_break_scale=4.0)
    seen = []
    for (m, x, v), r in zip(systems, res):
        over, tree, checks, t, p, xe = retry_loop(m, x, v, 40.0, 10.0, 100.0, 4.0)
        assert (r["over"], r["summary"], r["checks"], r["passes"]) == (over, tree, checks, p)
        assert r["time"] == t and np.array_equal(r["pos"], xe)
        seen.append(p)
    print("passes", seen)
    assert len(set(seen)) >= 2 and max(seen) > 1


def test_retries_need_a_finite_break_scale():
    with pytest.raises(ValueError):
        multiples.resolve_encounters(HostBatch(), [scattering(0)], end_time=10.0, delta_t=10.0,
                                     min_break_scale=1.0)


def test_serial_loop_decides_as_the_batched_one():
    """resolve_serial (one encounter at a time, the loop the host-core
    baseline runs) and resolve_encounters make the same decisions on the
    same integrator."""
    def integrate(m, x, v, dt):
        x, v, tf, _ = oracle.smalln(m, x, v, 0.14, dt)
        return x, v, tf
    systems = [scattering(s) for s in range(16)] + [workloads.binary_binary(s) for s in range(8)]
    res = multiples.resolve_encounters(HostBatch(), systems, end_time=400.0, delta_t=10.0,
                                       break_scale=40.0)
    kinds = set()
    for (m, x, v), r in zip(systems, res):
        over, summ, checks, t, xe, _ = multiples.resolve_serial(integrate, m, x, v, 400.0, 10.0,
                                                                break_scale=40.0)
        assert (r["over"], r["summary"], r["checks"], r["time"]) == (over, summ, checks, t)
        assert np.array_equal(r["pos"], xe)
        kinds.add(over)
    assert {1, 2, 3} <= kinds


def test_step_cap_retires_an_encounter():
    """A system stopped by the step cap leaves the loop with over = 0 and
    its status, after that increment."""
    r = multiples.resolve_encounters(HostBatch(), [scattering(1), scattering(2)], end_time=400.0,
                                     delta_t=10.0, max_steps=50)
    for x in r:
        assert x["status"] == 1 and x["over"] == 0 and x["checks"] == 1 and x["time"] < 10.0


def test_break_scale_ends_an_encounter():
    m, x, v = scattering(3, v_inf=2.0)
    r = multiples.resolve_encounters(HostBatch(), [(m, x, v)], end_time=1e4, delta_t=5.0,
                                     break_scale=3.0)[0]
    assert r["over"] in (1, 3) and r["time"] < 1e4


@pytest.mark.gpu
def test_resolve_encounters_on_the_gpu(g6):
    """64 binary-single scatterings advanced together on the batch kernel
    (split mode, unperturbed binaries): about as many end within the end time
    as on the host path (smallN itself; 52 of 64 — the trajectories are
    chaotic, so the two resolve different encounters), with the structure
    analysis agreeing on the final states and the energy kept at the
    integrator's level (smallN's own drift here is up to 7e-4)."""
    systems = [scattering(s) for s in range(64)]
    res = multiples.resolve_encounters(g6, systems, end_time=800.0, delta_t=10.0)
    host = multiples.resolve_encounters(HostBatch(), systems, end_time=800.0, delta_t=10.0)
    over = [r for r in res if r["over"] == 1]
    n_host = sum(r["over"] == 1 for r in host)
    print(f"{len(over)} of 64 over (host {n_host}); "
          f"checks {np.median([r['checks'] for r in res]):.0f} median")
    assert abs(len(over) - n_host) <= 8 and len(over) >= 44
    for (m, x, v), r in zip(systems, res):
        e0, e1 = r["energy"]
        assert abs((e1 - e0) / e0) < 5e-3
        if r["over"] == 1:
            assert ag.check_structure(m, r["pos"], r["vel"])["over"]
    # the outcome keeps the bodies: every final tree names each body once
    for r in over:
        ids = sorted(int(t) for t in r["summary"].replace("(", " ").replace(")", " ")
                     .replace(",", " ").split())
        assert ids == [0, 1, 2]


def test_scattering_outcomes():
    f = workloads.scattering_outcome
    assert f("(0,1) 2", 1) == "flyby"
    assert f("(1,2) 0", 1) == f("(0,2) 1", 1) == "exchange"
    assert f("0 1 2", 1) == "ionization"
    assert f("((0,1),2)", 1) == "bound"
    assert f("(0,1) 2", 0) == "unresolved"
    assert f("(0,1) 2", 2) == "quasi-stable"
    assert f("(0,1) 2", 3) == "break-scale"
