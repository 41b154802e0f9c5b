"""Generate the golden fixtures in this directory.

Runs in the development container only (it needs the reference checkout):
  * AMUSE's own IC generators (src/amuse/ic/plummer.py, salpeter.py),
    imported from the reference tree, give the inputs;
  * the unmodified ph4 CPU objects, compiled by ``make -C oracle ref`` into
    oracle/_ref/libph4ref.so, give the outputs (force: idata.cc:147-237,
    corrector: idata.cc:399-514, full block-step run: interface.cc:317-711,
    smallN few-body runs: smallN.cc:906-1117 with dt_crit = 0, block-step
    runs with the encounter check: idata.cc:620-700, jdata.cc:797-850).

Usage:  AMUSE_REF=<checkout> python tests/golden/make_golden.py [--ref <checkout>]
                                          [--only smalln|encounters]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def amuse_plummer(n, do_scale):
    from amuse.ic.plummer import new_plummer_model
    from amuse.units import nbody_system as nb
    p = new_plummer_model(n, do_scale=do_scale)
    pos = np.stack([p.x.value_in(nb.length), p.y.value_in(nb.length), p.z.value_in(nb.length)], 1)
    vel = np.stack([p.vx.value_in(nb.speed), p.vy.value_in(nb.speed), p.vz.value_in(nb.speed)], 1)
    return p.mass.value_in(nb.mass), pos, vel


def amuse_salpeter(n, mmin, mmax):
    from amuse.ic.salpeter import new_powerlaw_mass_distribution_nbody
    from amuse.units import nbody_system as nb
    m = new_powerlaw_mass_distribution_nbody(n, alpha=-2.35, mass_min=mmin | nb.mass,
                                             mass_max=mmax | nb.mass)
    return m.value_in(nb.mass)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", name, os.path.getsize(path), "bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("AMUSE_REF"))
    ap.add_argument("--only", default=None,
                    choices=[None, "smalln", "encounters", "unpert", "structure"])
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set AMUSE_REF to the AMUSE checkout")
    sys.path.insert(0, os.path.join(args.ref, "src"))
    import oracle
    oracle.build_ref(args.ref)
    if args.only == "smalln":
        return smalln_fixtures(oracle)
    if args.only == "encounters":
        return encounter_fixtures(oracle)
    if args.only == "unpert":
        return smalln_unpert_fixtures(oracle)
    if args.only == "structure":
        return structure_fixtures(oracle)

    # 1. IC generators (pins amuse_gb300/ic.py).
    np.random.seed(1)
    m0, x0, v0 = amuse_plummer(256, False)
    np.random.seed(1)
    m1, x1, v1 = amuse_plummer(256, True)
    np.random.seed(3)
    ms = amuse_salpeter(512, 0.1, 100.0)
    save("ic_amuse.npz", plummer_mass=m0, plummer_pos=x0, plummer_vel=v0,
         scaled_mass=m1, scaled_pos=x1, scaled_vel=v1, salpeter_mass=ms)

    # 2. Force on all i, C1 shape: N=1024 scaled Plummer, eps2=1e-4.
    np.random.seed(1)
    m, x, v = amuse_plummer(1024, True)
    f = oracle.force(m, x, v, 1e-4, x, v, lib="ref")
    save("force_plummer1024_eps1e-4.npz", mass=m, pos=x, vel=v, eps2=1e-4, **f)

    # 3. Force, C2 shape at reduced N: Salpeter masses 0.1..100, re-scaled,
    #    eps2=1e-6; a random i-subset whose positions are offset from the
    #    j-set (as after an i-prediction), plus zero-offset members.
    np.random.seed(2)
    m, x, v = amuse_plummer(4096, False)
    m = amuse_salpeter(4096, 0.1, 100.0)
    from amuse_gb300 import ic as myic
    myic.move_to_center(m, x, v)
    myic.scale_to_standard(m, x, v)
    rng = np.random.RandomState(7)
    isel = rng.choice(4096, 700, replace=False)
    ipos = x[isel].copy()
    ivel = v[isel].copy()
    ipos[:350] += rng.normal(scale=1e-7, size=(350, 3))
    f = oracle.force(m, x, v, 1e-6, ipos, ivel, lib="ref")
    save("force_salpeter4096_eps1e-6.npz", mass=m, pos=x, vel=v, eps2=1e-6, isel=isel,
         ipos=ipos, ivel=ivel, **f)

    # 4. Unsoftened force (eps2 = 0), N=128, plus a zero-mass j and a
    #    duplicated position (excluded from pot/nn by the r2 > 2^-52 rule).
    np.random.seed(4)
    m, x, v = amuse_plummer(128, True)
    m = m.copy()
    m[5] = 0.0
    f = oracle.force(m, x, v, 0.0, x, v, lib="ref")
    save("force_plummer128_eps0.npz", mass=m, pos=x, vel=v, eps2=0.0, **f)

    # 5. Corrector + Aarseth step on states from a short run.
    np.random.seed(5)
    m, x, v = amuse_plummer(512, True)
    r = oracle.run(m, x, v, 1e-4, 0.01, 0.0625, lib="ref")
    rng = np.random.RandomState(11)
    old_acc = r["acc"]
    old_jerk = r["jerk"]
    ts = r["timestep"]
    tnext = r["t"] + np.min(ts)
    new_acc = old_acc + rng.normal(scale=1e-3, size=old_acc.shape) * np.abs(old_acc)
    new_jerk = old_jerk + rng.normal(scale=1e-2, size=old_jerk.shape) * np.abs(old_jerk)
    itime = np.full(512, tnext) - ts
    c = oracle.correct(tnext, 0.01, itime, ts, r["pos"], r["vel"], old_acc, old_jerk,
                       new_acc, new_jerk, lib="ref")
    save("correct512.npz", tnext=tnext, eta=0.01, itime=itime, istep=ts, ipos=r["pos"],
         ivel=r["vel"], old_acc=old_acc, old_jerk=old_jerk, iacc=new_acc, ijerk=new_jerk,
         out_time=c["time"], out_step=c["timestep"], out_pos=c["pos"], out_vel=c["vel"])

    # 6. Full block-step runs through the unmodified ph4 loop.
    #    a) C1: N=1024 scaled Plummer, eps2=1e-4, eta=0.01, to t=1 (seed 1).
    np.random.seed(1)
    m, x, v = amuse_plummer(1024, True)
    r = oracle.run(m, x, v, 1e-4, 0.01, 1.0, lib="ref")
    save("run_plummer1024_t1.npz", mass=m, pos0=x, vel0=v, eps2=1e-4, eta=0.01, t_end=1.0,
         **{k: np.asarray(r[k]) for k in r})
    #    b) a short unsoftened-ish run (eps2=1e-6), N=256, to t=0.125.
    np.random.seed(6)
    m, x, v = amuse_plummer(256, True)
    r = oracle.run(m, x, v, 1e-6, 0.01, 0.125, lib="ref")
    save("run_plummer256_eps1e-6.npz", mass=m, pos0=x, vel0=v, eps2=1e-6, eta=0.01,
         t_end=0.125, **{k: np.asarray(r[k]) for k in r})
    smalln_fixtures(oracle)
    encounter_fixtures(oracle)
    smalln_unpert_fixtures(oracle)
    structure_fixtures(oracle)


def smalln_fixtures(oracle):
    """7. smallN on few-body systems like the batching configuration's
    (equal-mass Plummer, virial radius 1e-3, eps = 0, eta = 0.14) to two
    crossing times, through the unmodified smallN objects."""
    from amuse_gb300 import ic
    out = {}
    tcr = 2 * np.sqrt(2) * 1e-3 ** 1.5
    for k, (n, seed) in enumerate([(3, 11), (4, 12), (9, 13), (24, 14), (64, 15)]):
        rng = np.random.RandomState(seed)
        m, x, v = ic.plummer(n, do_scale=True, rng=rng)
        x, v = x * 1e-3, v / np.sqrt(1e-3)
        p, vv, t, _ = oracle.smalln(m, x, v, 0.14, 2 * tcr, lib="ref")
        out.update({f"s{k}_mass": m, f"s{k}_pos0": x, f"s{k}_vel0": v, f"s{k}_pos": p,
                    f"s{k}_vel": vv, f"s{k}_t": t})
    save("smalln_systems.npz", nsys=len(out) // 6, eta=0.14, t_end=2 * tcr, **out)


def hierarchical(kind, seed):
    """Few-body systems with hard binaries, in the CM frame: "triple" (an
    eccentric inner binary and a third body on a bound outer orbit), "quad"
    (two binaries on a bound orbit), "field" (a binary among 6 single
    stars).  Used for smallN's unperturbed-binary treatment."""
    rng = np.random.RandomState(seed)

    def binary(m1, m2, a, e):
        r = a * (1 + e)
        vrel = np.sqrt((m1 + m2) * (1 - e) / r)
        x = np.array([[-m2 / (m1 + m2) * r, 0, 0], [m1 / (m1 + m2) * r, 0, 0]])
        v = np.array([[0, -m2 / (m1 + m2) * vrel, 0], [0, m1 / (m1 + m2) * vrel, 0]])
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))  # random orientation
        return x @ q.T, v @ q.T

    if kind == "triple":
        m = np.array([0.4, 0.4, 0.2]) * rng.uniform(0.8, 1.2, 3)
        xb, vb = binary(m[0], m[1], 0.01, rng.uniform(0.1, 0.8))
        d = rng.uniform(0.8, 1.2)
        x = np.vstack([xb, [[0, d, 0]]])
        v = np.vstack([vb, [[0.8 * np.sqrt(m.sum() / d), 0, 0]]])
    elif kind == "quad":
        m = np.full(4, 0.25) * rng.uniform(0.8, 1.2, 4)
        x1, v1 = binary(m[0], m[1], 0.01, rng.uniform(0.1, 0.7))
        x2, v2 = binary(m[2], m[3], 0.015, rng.uniform(0.1, 0.7))
        x = np.vstack([x1 + [-0.6, 0, 0], x2 + [0.6, 0, 0]])
        vo = 0.5 * np.sqrt(m.sum() / 1.2)
        v = np.vstack([v1 + [0, -vo, 0], v2 + [0, vo, 0]])
    else:
        m = np.concatenate([[0.3, 0.3], np.full(6, 0.4 / 6)])
        xb, vb = binary(m[0], m[1], 0.005, rng.uniform(0.2, 0.9))
        xf = rng.normal(0, 1.0, (6, 3))
        vf = rng.normal(0, 0.3, (6, 3))
        x, v = np.vstack([xb, xf]), np.vstack([vb, vf])
    cm = (m[:, None] * x).sum(0) / m.sum()
    cv = (m[:, None] * v).sum(0) / m.sum()
    return m, x - cm, v - cv


SMALLN_UNPERT_CASES = [("triple", 1, 2.0), ("triple", 2, 2.0), ("triple", 3, 4.0),
                       ("quad", 4, 2.0), ("field", 5, 1.0), ("field", 6, 1.0)]


def smalln_unpert_fixtures(oracle):
    """9. smallN WITH its unperturbed binaries (the worker's defaults:
    dt_crit 1e-3, r2_crit 1e-2, gamma 1e-6, full unperturbed motion allowed)
    on systems with hard binaries, through the unmodified smallN objects
    (the leaves of binary nodes left at the end reported in absolute
    coordinates)."""
    out = {}
    for k, (kind, seed, t_end) in enumerate(SMALLN_UNPERT_CASES):
        m, x, v = hierarchical(kind, seed)
        p, vv, t, _ = oracle.smalln(m, x, v, 0.14, t_end, lib="ref", dt_crit=1e-3)
        out.update({f"s{k}_mass": m, f"s{k}_pos0": x, f"s{k}_vel0": v, f"s{k}_pos": p,
                    f"s{k}_vel": vv, f"s{k}_t": t, f"s{k}_t_end": t_end})
    save("smalln_unpert.npz", nsys=len(SMALLN_UNPERT_CASES), eta=0.14, **out)


# (n, seed, radius, mode): collision stops (radius R for all particles) and
# close-pair stops (radius 0, ph4's rmin = 2/n).
ENCOUNTER_CASES = [(64, 1, 0.02, "coll"), (128, 3, 0.01, "coll"), (256, 4, 0.005, "coll"),
                   (64, 5, 0.0, "close"), (256, 4, 0.0, "close")]


def encounter_fixtures(oracle):
    """8. ph4 block-step runs with the encounter check: AMUSE's Plummer
    spheres (eps2 = 1e-4, eta = 0.14, to t = 1 or 2) run through the
    unmodified ph4 objects with the COLLISION_DETECTION stopping condition
    enabled (idata.cc:620-700, jdata.cc:797-850), or until the first block
    that reports a close pair.  Ids are slot + 1."""
    from amuse_gb300 import ic
    out = {}
    for k, (n, seed, rad, kind) in enumerate(ENCOUNTER_CASES):
        np.random.seed(seed)
        m, x, v = ic.plummer(n)
        radius = np.full(n, rad)
        mode = oracle.ENC_CHECK | (oracle.ENC_STOP_COLL if kind == "coll"
                                   else oracle.ENC_STOP_CLOSE)
        t_end = 1.0 if kind == "coll" else 2.0
        r = oracle.run_enc(m, radius, x, v, 1e-4, 0.14, t_end, mode=mode, lib="ref")
        pair = r["stop_pair"] if kind == "coll" else r["close"]
        assert pair is not None, (n, seed, kind)
        out.update({f"c{k}_mass": m, f"c{k}_pos0": x, f"c{k}_vel0": v, f"c{k}_radius": radius,
                    f"c{k}_mode": mode, f"c{k}_t_end": t_end, f"c{k}_t": r["t"],
                    f"c{k}_blocks": r["blocks"], f"c{k}_pair": np.array(pair),
                    f"c{k}_pos": r["pos"], f"c{k}_vel": r["vel"], f"c{k}_rmin": r["rmin"]})
    save("encounter_runs.npz", ncase=len(ENCOUNTER_CASES), eps2=1e-4, eta=0.14, **out)


def structure_fixtures(oracle):
    """10. smallN's structure analysis (analyze.cc check_structure, get_tree)
    on few-body states: the batching configuration's kind of system
    (n = 3 ... 12, Plummer r_vir = 1e-3, eps = 0) evolved by the unmodified
    smallN (no binary tree) to 0.5, 2, 6 and 20 crossing times; per state the
    reference's over flag and its tree as text ("(first,second)" of 0-based
    body indices, top-level nodes separated by spaces)."""
    from amuse_gb300 import ic
    ns, m, x, v, tcr = ic.encounter_batch(60, 3, 12, seed=11)
    off = np.concatenate([[0], np.cumsum(ns)])
    out, k = {}, 0
    for s in range(len(ns)):
        a, b = off[s], off[s + 1]
        for f in (0.5, 2.0, 6.0, 20.0):
            p, vv, t, _ = oracle.smalln(m[a:b], x[a:b], v[a:b], 0.14, f * tcr, lib="ref")
            over, tree = oracle.check_structure_ref(m[a:b], p, vv)
            out.update({f"s{k}_mass": m[a:b], f"s{k}_pos": p, f"s{k}_vel": vv,
                        f"s{k}_over": over, f"s{k}_tree": np.array(tree)})
            k += 1
    save("structure_states.npz", nstate=k, **out)


if __name__ == "__main__":
    main()
