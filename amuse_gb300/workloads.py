"""Workload runners for the benchmark configurations other than the headline
one (which is bench.py).  Each prints one JSON line.

  python -m amuse_gb300.workloads batch   [--nsys 4096]
      nsys few-body systems, n ~ U[3, 64], Plummer with virial radius 1e-3,
      eps = 0, to 10 crossing times, smallN's scheme (g6x_batch_run) after
      the autotuner; systems/s and p50/p99 per-system GPU time.
      (bench.py --workload batch adds the host-core baseline.)
  python -m amuse_gb300.workloads precision [--n 1048576]
      Split vs FP64 per-particle force errors on all N and the energy drift
      over 64 block steps.
  python -m amuse_gb300.workloads salpeter [--n 65536] [--t-end 0.25] [--encounters]
      Salpeter-IMF Plummer block-step run on the device, then split vs FP64
      forces at ni = 1 ... N; --encounters repeats the run with ph4's
      encounter check and reports its cost.
  python -m amuse_gb300.workloads knn [--n 1048576] [--k 12]
      The k nearest neighbours of every particle (g6x_knn), timed.
  python -m amuse_gb300.workloads multiples [--nsys 4096]
      nsys binary-single scatterings resolved together by the multiples
      hand-off (amuse_gb300.multiples.resolve_encounters: batch launches of
      delta_t = 10 with smallN's unperturbed binaries, the structure check
      after each); encounters/s, outcomes, increments, energy.
      (bench.py --workload multiples adds the host-core baseline.)
  python -m amuse_gb300.workloads adjoint [--n 16384] [--nsteps 256]
      Differentiable fixed-step Hermite: timing of forward and backward in
      split precision and FP64, split vs FP64 gradients, and finite
      differences of the forward against the adjoint.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _few_body_energy(m, x, v):
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt(np.sum(d * d, -1))
    iu = np.triu_indices(len(m), 1)
    return 0.5 * np.sum(m * np.sum(v * v, 1)) - np.sum(m[iu[0]] * m[iu[1]] / r[iu])


def run_batch(args):
    """Config 4 on the GPU: autotune, the full batch, and a sample of systems
    (returned for a host-core comparison by the caller)."""
    import amuse_gb300 as ag
    from amuse_gb300 import ic
    ns, m, x, v, tcr = ic.encounter_batch(args.nsys, 3, 64, r_vir=1e-3, seed=args.seed)
    t_end = 10 * tcr
    off = np.concatenate([[0], np.cumsum(ns)])
    g6 = ag.G6X(0)
    mode = getattr(args, "batch_mode", "split")
    # smallN's unperturbed binaries (its default; not in the exact mode)
    unpert = mode != "exact" and not getattr(args, "no_unpert", False)
    g6.batch_unperturbed(unpert)
    out = {"workload": f"{args.nsys} few-body systems, n~U[3,64], Plummer r_vir=1e-3, eps=0, "
                       f"t_end=10 t_cross={t_end:.4g}, eta={args.eta}, smallN scheme "
                       f"(n_iter=2, Kepler criterion"
                       f"{', unperturbed binaries' if unpert else ''}), FP64 state, step cap "
                       f"{args.max_steps}/system", "mode": mode, "unperturbed_binaries": unpert}

    # 1. autotune on 512 systems for 0.5% of the end time
    kt = min(args.nsys, 512)
    tune = g6.batch_tune(ns[:kt], t_end, m[:off[kt]], x[:off[kt]], v[:off[kt]], eta=args.eta,
                         frac=0.005, mode=mode)
    out["autotune"] = tune
    print(json.dumps(out), flush=True)

    # 2. the sample the caller times on the host cores (same step cap)
    kc = min(args.cpu_sample, args.nsys)
    sc = slice(0, off[kc])
    rg = g6.batch_run(ns[:kc], t_end, m[sc], x[sc], v[sc], eta=args.eta,
                      max_steps=args.max_steps, mode=mode)
    out["sample"] = {"systems": kc, "gpu_systems_per_s": kc / (rg["elapsed_ms"] / 1e3),
                     "gpu_mode": mode}

    # 3. the full batch
    t0 = time.perf_counter()
    r = g6.batch_run(ns, t_end, m, x, v, eta=args.eta, max_steps=args.max_steps, mode=mode)
    wall = time.perf_counter() - t0
    nbin = g6.batch_binaries(args.nsys) if unpert else np.zeros(args.nsys, np.int32)
    g6.batch_unperturbed(False)
    done = r["status"] == 0
    de, bad = [], []
    for s_ in range(args.nsys):
        a, b = off[s_], off[s_ + 1]
        e0 = _few_body_energy(m[a:b], x[a:b], v[a:b])
        e1 = _few_body_energy(m[a:b], r["pos"][a:b], r["vel"][a:b])
        if np.isfinite(e1):
            de.append(abs((e1 - e0) / e0))
        else:
            bad.append(s_)
    out["dE_over_E"] = {"p50": float(np.percentile(de, 50)), "p90": float(np.percentile(de, 90)),
                        "p99": float(np.percentile(de, 99)), "max": float(np.max(de)),
                        "systems": len(de), "nonfinite_systems": bad[:20],
                        "n_nonfinite": len(bad)}
    out.update({
        "systems_per_s": args.nsys / (r["elapsed_ms"] / 1e3),
        "completed_systems_per_s": int(done.sum()) / (r["elapsed_ms"] / 1e3),
        "elapsed_ms_gpu": r["elapsed_ms"], "wall_s_incl_copies": wall,
        "per_system_ms": {"p50": float(np.percentile(r["wall_ms"], 50)),
                          "p99": float(np.percentile(r["wall_ms"], 99)),
                          "max": float(r["wall_ms"].max())},
        "steps": {"total": int(r["steps"].sum()), "p50": float(np.percentile(r["steps"], 50)),
                  "p90": float(np.percentile(r["steps"], 90)),
                  "p99": float(np.percentile(r["steps"], 99)), "max": int(r["steps"].max())},
        "completed": int(done.sum()), "capped": int((r["status"] == 1).sum()),
        "binaries": {"made": int(nbin.sum()), "systems_with_binaries": int((nbin > 0).sum())},
    })
    print(json.dumps(out), flush=True)
    sample = dict(ns=ns[:kc], mass=m[sc], pos=x[sc], vel=v[sc], t_end=t_end, off=off[:kc + 1],
                  unpert=unpert)
    return out, sample


def binary_single(seed, v_inf=0.6, b_max=1.5, d0=15.0):
    """One binary-single scattering: a binary of 0.5 + 0.5 (a = 1, e uniform
    in [0, 0.7], random orientation and phase) and a single of 0.5 coming in
    from d0 with speed v_inf (0.6 is 0.69 of the critical speed, so most
    encounters are resonant) and impact parameter up to b_max;
    centre-of-mass frame, G = 1.  numpy RandomState(seed)."""
    rng = np.random.RandomState(seed)
    m = np.array([0.5, 0.5, 0.5])
    a, e = 1.0, rng.uniform(0, 0.7)
    E = rng.uniform(0, 2 * np.pi)
    r = a * (1 - e * np.cos(E))
    xr = np.array([a * (np.cos(E) - e), a * np.sqrt(1 - e * e) * np.sin(E), 0.0])
    s = np.sqrt(1.0 * a) / r
    vr = np.array([-s * np.sin(E), s * np.sqrt(1 - e * e) * np.cos(E), 0.0])
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    xr, vr = q @ xr, q @ vr
    b = b_max * np.sqrt(rng.uniform())
    x = np.array([-0.5 * xr, 0.5 * xr, [-d0, b, 0.0]])
    v = np.array([-0.5 * vr, 0.5 * vr, [v_inf, 0.0, 0.0]])
    cm = (m[:, None] * x).sum(0) / m.sum()
    cv = (m[:, None] * v).sum(0) / m.sum()
    return m, x - cm, v - cv


def _kepler_binary(rng, m1, m2, a):
    """Two bodies on a Kepler orbit of semi-major axis a, e uniform in
    [0, 0.7], random phase and orientation, in their centre-of-mass frame."""
    e = rng.uniform(0, 0.7)
    E = rng.uniform(0, 2 * np.pi)
    M = m1 + m2
    r = a * (1 - e * np.cos(E))
    xr = np.array([a * (np.cos(E) - e), a * np.sqrt(1 - e * e) * np.sin(E), 0.0])
    s = np.sqrt(M * a) / r
    vr = np.array([-s * np.sin(E), s * np.sqrt(1 - e * e) * np.cos(E), 0.0])
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    xr, vr = q @ xr, q @ vr
    return np.array([-m2 / M * xr, m1 / M * xr]), np.array([-m2 / M * vr, m1 / M * vr])


def binary_binary(seed, v_inf=0.5, b_max=2.0, d0=20.0):
    """One binary-binary scattering: two binaries of 0.25 + 0.25 (a = 1 and
    a uniform in [0.5, 1.5]) approaching at relative speed v_inf from d0
    apart with impact parameter up to b_max; centre-of-mass frame, G = 1.
    numpy RandomState(seed)."""
    rng = np.random.RandomState(seed)
    m = np.full(4, 0.25)
    x1, v1 = _kepler_binary(rng, 0.25, 0.25, 1.0)
    x2, v2 = _kepler_binary(rng, 0.25, 0.25, rng.uniform(0.5, 1.5))
    b = b_max * np.sqrt(rng.uniform())
    x = np.vstack([x1 + [d0 / 2, 0, 0], x2 + [-d0 / 2, b, 0]])
    v = np.vstack([v1 + [-v_inf / 2, 0, 0], v2 + [v_inf / 2, 0, 0]])
    cm = (m[:, None] * x).sum(0) / m.sum()
    cv = (m[:, None] * v).sum(0) / m.sum()
    return m, x - cm, v - cv


def scattering_outcome(summary, over):
    """flyby (the binary (0,1) survives), exchange (the single is in the
    final binary), ionization (three singles), bound (a stable triple),
    quasi-stable (smallN's ending for a repeating unstable grouping),
    break-scale or unresolved."""
    if not over:
        return "unresolved"
    if over == 2:
        return "quasi-stable"
    if over == 3:
        return "break-scale"
    if summary.count("(") > 1:
        return "bound"
    if summary == "(0,1) 2":
        return "flyby"
    if summary in ("(0,2) 1", "(1,2) 0"):
        return "exchange"
    if summary == "0 1 2":
        return "ionization"
    return "bound"


def run_multiples(args):
    """The multiples hand-off on the GPU: args.nsys binary-single scatterings
    resolved together (end time args.end_time, increments args.delta_t).
    Returns the JSON dict and the systems (all of them: the host loop over
    the same encounters takes ~4 ms of one core each)."""
    import amuse_gb300 as ag
    from amuse_gb300 import multiples
    systems = [binary_single(args.seed * 1_000_003 + k) for k in range(args.nsys)]
    g6 = ag.G6X(0)
    kw = dict(end_time=args.end_time, delta_t=args.delta_t, eta=args.eta,
              max_steps=args.max_steps)
    multiples.resolve_encounters(g6, systems[:64], **kw)  # warm (context, graphs, buffers)
    tm = {}
    t0 = time.perf_counter()
    res = multiples.resolve_encounters(g6, systems, timing=tm, **kw)
    wall = time.perf_counter() - t0
    outc = {}
    for r in res:
        k = scattering_outcome(r["summary"], r["over"])
        outc[k] = outc.get(k, 0) + 1
    de = np.array([abs((r["energy"][1] - r["energy"][0]) / r["energy"][0]) for r in res])
    checks = np.array([r["checks"] for r in res])
    steps = np.array([r["steps"] for r in res])
    resolved = int(sum(r["over"] != 0 for r in res))
    out = {
        "metric": "encounters/s (multiples hand-off to batched smallN)",
        "value": args.nsys / wall, "unit": "encounters/s",
        "workload": f"{args.nsys} binary-single scatterings (0.5+0.5, a=1, e~U[0,0.7]; "
                    f"single 0.5 from d=15, v_inf=0.6, b<=1.5), end_time={args.end_time}, "
                    f"delta_t={args.delta_t}, eta={args.eta}, smallN scheme with unperturbed "
                    f"binaries (split mode), structure check after every increment",
        "resolved": resolved, "resolved_per_s": resolved / wall, "outcomes": outc,
        "wall_s": wall, "launches": tm["launches"], "batch_s": tm["batch_s"],
        "check_s": tm["check_s"],
        "active_per_launch": {"first": tm["active_per_launch"][0],
                              "p50": float(np.median(tm["active_per_launch"]))},
        "increments": {"p50": float(np.median(checks)), "p99": float(np.percentile(checks, 99)),
                       "max": int(checks.max())},
        "steps": {"total": int(steps.sum()), "p50": float(np.median(steps)),
                  "max": int(steps.max())},
        "dE_over_E": {"p50": float(np.median(de)), "p99": float(np.percentile(de, 99)),
                      "max": float(de.max())},
    }
    print(json.dumps(out), flush=True)
    return out, systems


def run_adjoint(args):
    """Config 5: Plummer n equal-mass bodies, eps2 = 1e-4, fixed dt = 1/256
    for 256 steps, loss = sum w_i |x_i|^2 (seeded w); gradient w.r.t. x0, v0,
    m through the adjoint with a checkpoint every 16 steps, in split
    precision and in FP64; central finite differences (h = 1e-6) on seeded
    coordinates of the split forward and, on fewer, of the FP64 forward."""
    import torch
    from amuse_gb300 import ic
    from amuse_gb300.adjoint import hermite_fixed
    n, eps2, dt, nsteps, ck = args.n, 1e-4, 1.0 / 256, args.nsteps, 16
    rng = np.random.RandomState(args.seed)
    m, x, v = ic.plummer(n, do_scale=True, rng=rng)
    w = rng.uniform(0.5, 1.5, n)
    dev = torch.device("cuda", 0)
    base = [torch.tensor(a, dtype=torch.float64, device=dev) for a in (x, v, m)]
    tw = torch.tensor(w, dtype=torch.float64, device=dev)
    out = {"workload": f"Plummer n={n} equal mass, eps2={eps2}, dt=1/256, {nsteps} steps, "
                       f"checkpoint every {ck}, loss=sum w|x|^2"}

    def grad(prec):
        xs = [t.clone().requires_grad_(True) for t in base]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xf, _ = hermite_fixed(xs[0], xs[1], xs[2], eps2=eps2, dt=dt, nsteps=nsteps,
                              checkpoint=ck, precision=prec)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss = (tw * (xf * xf).sum(1)).sum()
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return float(loss), [t.grad.cpu().numpy() for t in xs], t1 - t0, t2 - t1

    def loss_at(which, idx, delta, prec):
        xs = [t.clone() for t in base]
        xs[which][idx] += delta
        with torch.no_grad():
            xf, _ = hermite_fixed(xs[0], xs[1], xs[2], eps2=eps2, dt=dt, nsteps=nsteps,
                                  checkpoint=nsteps, precision=prec)
            return float((tw * (xf * xf).sum(1)).sum())

    # warm-up: first forward and backward (library buffers, autograd's device
    # threads), outside the timed calls
    for prec in ("split", "fp64"):
        w0 = [t[:256].clone().requires_grad_(True) for t in base]
        xw, _ = hermite_fixed(w0[0], w0[1], w0[2], eps2=eps2, dt=dt, nsteps=2, checkpoint=1,
                              precision=prec)
        (xw * xw).sum().backward()
    torch.cuda.synchronize()
    ls, gs, fs, bs = grad("split")
    pairs_fwd = (nsteps + 1) * n * (n - 1)
    out["split"] = {"loss": ls, "forward_s": fs, "backward_s": bs,
                    "forward_pairs_per_s": pairs_fwd / fs}
    print(json.dumps(out), flush=True)
    ld, gd, fd_, bd = grad("fp64")
    out["fp64"] = {"loss": ld, "forward_s": fd_, "backward_s": bd}
    names = ["x0", "v0", "m"]
    out["split_vs_fp64_gradient"] = {
        names[k]: float(np.linalg.norm(gs[k] - gd[k]) / np.linalg.norm(gd[k])) for k in range(3)}
    out["split_vs_fp64_loss_rel"] = abs(ls - ld) / abs(ld)
    print(json.dumps(out), flush=True)

    h = 1e-6
    crng = np.random.RandomState(args.seed + 1)
    coords = []
    for _ in range(args.fd_coords):
        k = crng.randint(3)
        i = crng.randint(n)
        coords.append((k, (i,) if k == 2 else (i, crng.randint(3))))

    def fd_errors(prec, cs):
        rel = []
        for k, idx in cs:
            fd = (loss_at(k, idx, h, prec) - loss_at(k, idx, -h, prec)) / (2 * h)
            g_ad = (gs if prec == "split" else gd)[k][idx]
            scale = max(abs(g_ad), 1e-2 * np.abs((gs if prec == "split" else gd)[k]).max())
            rel.append(abs(fd - g_ad) / scale)
        return rel

    if coords:
        t0 = time.perf_counter()
        rs = fd_errors("split", coords)
        out["fd_split"] = {"coords": len(coords), "h": h, "max_rel": float(max(rs)),
                           "median_rel": float(np.median(rs)),
                           "n_above_1e-4": int(sum(r > 1e-4 for r in rs)),
                           "seconds": time.perf_counter() - t0}
        print(json.dumps(out), flush=True)
    if args.fd64_coords > 0 and coords:
        t0 = time.perf_counter()
        rd = fd_errors("fp64", coords[: args.fd64_coords])
        out["fd_fp64"] = {"coords": len(rd), "h": h, "max_rel": float(max(rd)),
                          "median_rel": float(np.median(rd)),
                          "seconds": time.perf_counter() - t0}
        print(json.dumps(out), flush=True)
    return out


def _stats(err):
    err = np.asarray(err)
    return {"min": float(err.min()), "p50": float(np.percentile(err, 50)),
            "p99": float(np.percentile(err, 99)), "max": float(err.max()),
            "frac_le_1e-6": float(np.mean(err <= 1e-6))}


def _slot_forces(g6, torch, prec, n, ni, eps2, ilist):
    """acc, jerk, pot of slots [0, ni) against slots [0, n) (device run)."""
    g6.set_precision(prec)
    dev = ilist.device
    acc = torch.empty((ni, 3), dtype=torch.float64, device=dev)
    jerk = torch.empty_like(acc)
    pot = torch.empty(ni, dtype=torch.float64, device=dev)
    t0 = time.perf_counter()
    g6.force_slots(g6.system_time(), eps2, n, ilist.data_ptr(), ni, acc.data_ptr(),
                   jerk.data_ptr(), pot.data_ptr(), None)
    dt = time.perf_counter() - t0
    return acc.cpu().numpy(), jerk.cpu().numpy(), pot.cpu().numpy(), dt


def _errors(s, d):
    a, j, p = s[:3]
    ad, jd, pd = d[:3]
    return {"acc": _stats(np.linalg.norm(a - ad, axis=1) / np.linalg.norm(ad, axis=1)),
            "jerk": _stats(np.linalg.norm(j - jd, axis=1) / np.linalg.norm(jd, axis=1)),
            "pot": _stats(np.abs(p - pd) / np.abs(pd))}


def run_precision(args):
    """Config 3: Plummer N = 2^20 equal mass, eps2 = 1e-6 (the benchmark's
    particles).  Per-particle relative acc/jerk/pot errors of the split
    kernel against the plain FP64 kernel on all N (min/p50/p99/max), and the
    energy drift of the device block-step driver over 64 block steps."""
    import torch
    import amuse_gb300 as ag
    from amuse_gb300 import ic
    n, eps2 = args.n, 1e-6
    np.random.seed(1)
    m, x, v = ic.plummer(n, do_scale=False)
    g6 = ag.G6X(0)
    g6.load_particles(m, x, v)
    ilist = torch.arange(n, dtype=torch.int32, device="cuda")
    out = {"workload": f"plummer N={n} equal mass eps2={eps2} (numpy seed 1)"}
    if not args.skip_fp64:
        sp = _slot_forces(g6, torch, ag.SPLIT, n, n, eps2, ilist)
        dp = _slot_forces(g6, torch, ag.FP64, n, n, eps2, ilist)
        out["split_vs_fp64"] = _errors(sp, dp)
        out["force_seconds"] = {"split": sp[3], "fp64": dp[3],
                                "split_pairs_per_s": n * (n - 1) / sp[3],
                                "fp64_pairs_per_s": n * (n - 1) / dp[3]}
        print(json.dumps(out), flush=True)
    g6.set_precision(ag.SPLIT)
    g6.run_init(eps2, args.eta)
    k0, p0 = g6.energy()
    t0 = time.perf_counter()
    e0 = k0 + p0
    if args.t_end:
        # to a system time (e.g. one N-body time unit) in 8 segments, with the
        # energy printed after each, so that partial results survive a time limit
        nb = ns = 0
        for seg in range(1, 9):
            b, st = g6.run(args.t_end * seg / 8)
            nb += b
            ns += st
            ks, ps = g6.energy()
            print(json.dumps({"segment": seg, "t": g6.system_time(), "blocks": nb,
                              "particle_steps": ns, "seconds": time.perf_counter() - t0,
                              "dE_over_E": abs(ks + ps - e0) / abs(e0)}), flush=True)
    else:
        nb, ns = g6.run(1e30, max_blocks=64)
    wall = time.perf_counter() - t0
    k1, p1 = g6.energy()
    e1 = k1 + p1
    out["block_steps"] = {"eta": args.eta, "precision": "split", "blocks": nb,
                          "particle_steps": ns, "t_reached": g6.system_time(),
                          "seconds": wall, "pairs_per_s": ns * (n - 1) / wall,
                          "E0": e0, "E1": e1, "dE_over_E": abs(e1 - e0) / abs(e0)}
    print(json.dumps(out), flush=True)
    return out


def run_blocks(args):
    """Config 2's system at fixed block sizes: for ni random slots of the
    Salpeter N = 65536 system at t = 0, the GPU time of the force kernel (with
    its split merge) and of the refinement pass (CUDA events), the refinement
    queue and the launch shape; the median of the repeats after two warm-up
    calls."""
    import torch
    import amuse_gb300 as ag
    from amuse_gb300 import ic
    n, eps2 = args.n, 1e-6
    g6 = ag.G6X(0)
    ilist = torch.arange(n, dtype=torch.int32, device="cuda")

    def gpu_potential(mass, pos):
        g6.load_particles(mass, pos, np.zeros_like(pos))
        _, _, pot, _ = _slot_forces(g6, torch, ag.FP64, len(mass), len(mass), 0.0, ilist)
        return 0.5 * float(np.sum(mass * pot))

    rng = np.random.RandomState(args.seed)
    m, x, v = ic.plummer_salpeter(n, mass_min=0.1, mass_max=100.0, rng=rng,
                                  potential_energy=gpu_potential)
    g6.load_particles(m, x, v)
    g6.set_precision(ag.SPLIT)
    rows = []
    for ni in args.ni:
        sel = np.sort(np.random.RandomState(ni).choice(n, ni, replace=False)).astype(np.int32)
        il = torch.tensor(sel, device="cuda")
        a = torch.empty((ni, 3), dtype=torch.float64, device="cuda")
        j = torch.empty_like(a)
        p = torch.empty(ni, dtype=torch.float64, device="cuda")
        g6.timing(True)
        ks, rs = [], []
        for r in range(2 + args.reps):
            g6.force_slots(0.0, eps2, n, il.data_ptr(), ni, a.data_ptr(), j.data_ptr(),
                           p.data_ptr(), None)
            st = g6.stats()
            if r >= 2:
                ks.append(st["kernel_ms"] * 1e3)
                rs.append(st["refine_ms"] * 1e3)
        g6.timing(False)
        rows.append({"ni": ni, "force_us": float(np.median(ks)), "refine_us": float(np.median(rs)),
                     "refine": g6.refine_stats(), "jl": int(st["jl"]),
                     "nsplit": int(st["nsplit"])})
    print(json.dumps({"workload": f"plummer N={n} Salpeter IMF (-2.35, 0.1-100) eps2={eps2}, "
                                  f"seed {args.seed}, t = 0: force calls on ni random slots",
                      "blocks": rows}), flush=True)


def run_salpeter(args):
    """Config 2: Plummer N = 65536 with a Salpeter IMF (slope -2.35, mass
    range 0.1-100, total mass 1, re-scaled to virial after the masses),
    eps2 = 1e-6, block steps to t = 0.25 on the device; then split vs FP64
    forces on blocks of ni = 1 ... N slots."""
    import torch
    import amuse_gb300 as ag
    from amuse_gb300 import ic
    n, eps2 = args.n, 1e-6
    g6 = ag.G6X(0)
    ilist = torch.arange(n, dtype=torch.int32, device="cuda")

    def gpu_potential(mass, pos):
        g6.load_particles(mass, pos, np.zeros_like(pos))
        _, _, pot, _ = _slot_forces(g6, torch, ag.FP64, len(mass), len(mass), 0.0, ilist)
        return 0.5 * float(np.sum(mass * pot))

    rng = np.random.RandomState(args.seed)
    m, x, v = ic.plummer_salpeter(n, mass_min=0.1, mass_max=100.0, rng=rng,
                                  potential_energy=gpu_potential)
    g6.load_particles(m, x, v)
    out = {"workload": f"plummer N={n} Salpeter IMF (-2.35, 0.1-100) eps2={eps2}, "
                       f"block steps to t={args.t_end}, eta={args.eta}, seed {args.seed}"}
    prec = ag.FP64 if args.fp64 else ag.SPLIT
    g6.set_precision(prec)
    g6.run_init(eps2, args.eta)
    k0, p0 = g6.energy()
    t0 = time.perf_counter()
    nb, ns = g6.run(args.t_end)
    wall = time.perf_counter() - t0
    k1, p1 = g6.energy()
    e0, e1 = k0 + p0, k1 + p1
    rs = g6.run_stats()
    out["run"] = {"precision": "fp64" if args.fp64 else "split", "blocks": nb,
                  "host_wall_ms": rs["wall_ms"], "host_sync_wait_ms": rs["sync_ms"],
                  "particle_steps": ns, "mean_ni": ns / max(nb, 1), "seconds": wall,
                  "pairs_per_s": ns * (n - 1) / wall, "E0": e0, "E1": e1,
                  "dE_over_E": abs(e1 - e0) / abs(e0)}
    print(json.dumps(out), flush=True)
    if args.encounters:
        # The same run with ph4's encounter check after every block (nearest
        # neighbours in the force, the criteria before and the stopping test
        # after the corrector; radius 0, so nothing stops).  The forces are
        # the same arithmetic with or without the neighbour search, so the
        # block sequence must repeat exactly.
        g6.load_particles(m, x, v)
        g6.set_encounters(ag.ENC_CHECK)
        g6.run_init(eps2, args.eta)
        t0 = time.perf_counter()
        nb2, ns2 = g6.run(args.t_end)
        wall2 = time.perf_counter() - t0
        enc = g6.encounter()
        g6.set_encounters(0)
        k2, p2 = g6.energy()
        out["run_with_encounter_check"] = {
            "blocks": nb2, "seconds": wall2, "overhead": wall2 / wall - 1.0,
            "same_blocks": nb2 == nb and ns2 == ns, "same_energy": (k2 + p2) == e1,
            "rmin": 2.0 / n, "last_block": enc}
        print(json.dumps(out), flush=True)
    checks = {}
    for ni in (1, 2, 3, 7, 31, 100, 1000, 4096, 10000, n):
        ni = min(ni, n)
        sp = _slot_forces(g6, torch, ag.SPLIT, n, ni, eps2, ilist)
        dp = _slot_forces(g6, torch, ag.FP64, n, ni, eps2, ilist)
        e = _errors(sp, dp)
        checks[str(ni)] = {k: {"p99": e[k]["p99"], "max": e[k]["max"]} for k in e}
    out["split_vs_fp64_by_ni"] = checks
    g6.set_precision(ag.SPLIT)
    print(json.dumps(out), flush=True)
    return out


def run_knn(args):
    """The k nearest neighbours of every particle (the lists ph4's
    get_densities_on_gpu builds, gpu.cc:568-866) for a Plummer sphere of N
    particles: one g6x_knn call over all N, timed after a warm-up call; and
    the same for a 1024-particle subset."""
    import amuse_gb300 as ag
    from amuse_gb300 import ic
    n, k = args.n, args.k
    g6 = ag.G6X(0)
    rng = np.random.RandomState(args.seed)
    m, x, v = ic.plummer(n, rng=rng)
    g6.load_particles(m, x, v)
    out = {"workload": f"plummer N={n}, k={k} nearest neighbours of every particle, seed {args.seed}"}
    for label, slots in (("all", None), ("subset1024", rng.choice(n, min(1024, n), replace=False))):
        g6.knn(n, k=k, slots=slots)                   # warm-up (allocation, attributes)
        t0 = time.perf_counter()
        ids, d2 = g6.knn(n, k=k, slots=slots)
        sec = time.perf_counter() - t0
        ni = n if slots is None else len(slots)
        out[label] = {"ni": ni, "seconds": sec, "pair_distances_per_s": ni * (n - 1) / sec,
                      "median_kth_distance": float(np.sqrt(np.median(d2[:, k - 1])))}
        print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    b = sub.add_parser("batch")
    b.add_argument("--nsys", type=int, default=4096)
    b.add_argument("--seed", type=int, default=1)
    b.add_argument("--eta", type=float, default=0.14)
    b.add_argument("--max-steps", type=int, default=2_000_000)
    b.add_argument("--cpu-sample", type=int, default=64)
    b.add_argument("--batch-mode", default="split", choices=["fast", "exact", "split"])
    b.add_argument("--no-unpert", action="store_true")
    d = sub.add_parser("adjoint")
    d.add_argument("--n", type=int, default=16384)
    d.add_argument("--nsteps", type=int, default=256)
    d.add_argument("--seed", type=int, default=7)
    d.add_argument("--fd-coords", type=int, default=32)
    d.add_argument("--fd64-coords", type=int, default=4)
    pr = sub.add_parser("precision")
    pr.add_argument("--n", type=int, default=1 << 20)
    pr.add_argument("--eta", type=float, default=0.14)
    pr.add_argument("--t-end", type=float, default=None,
                    help="block steps to this system time instead of 64 blocks")
    pr.add_argument("--skip-fp64", action="store_true",
                    help="skip the all-N FP64 force comparison")
    sa = sub.add_parser("salpeter")
    sa.add_argument("--n", type=int, default=65536)
    sa.add_argument("--eta", type=float, default=0.14)
    sa.add_argument("--t-end", type=float, default=0.25)
    sa.add_argument("--seed", type=int, default=1)
    sa.add_argument("--fp64", action="store_true")
    sa.add_argument("--encounters", action="store_true",
                    help="repeat the run with the encounter check on and report its cost")
    bl = sub.add_parser("blocks")
    bl.add_argument("--n", type=int, default=65536)
    bl.add_argument("--seed", type=int, default=1)
    bl.add_argument("--reps", type=int, default=5)
    bl.add_argument("--ni", type=int, nargs="+", default=[1, 16, 128, 722, 4096, 65536])
    mu = sub.add_parser("multiples")
    mu.add_argument("--nsys", type=int, default=4096)
    mu.add_argument("--seed", type=int, default=1)
    mu.add_argument("--eta", type=float, default=0.14)
    mu.add_argument("--end-time", type=float, default=1000.0)
    mu.add_argument("--delta-t", type=float, default=10.0)
    mu.add_argument("--max-steps", type=int, default=2_000_000)
    kn = sub.add_parser("knn")
    kn.add_argument("--n", type=int, default=1 << 20)
    kn.add_argument("--k", type=int, default=12)
    kn.add_argument("--seed", type=int, default=3)
    a = ap.parse_args()
    if a.cmd == "batch":
        run_batch(a)
    elif a.cmd == "adjoint":
        run_adjoint(a)
    elif a.cmd == "precision":
        run_precision(a)
    elif a.cmd == "salpeter":
        run_salpeter(a)
    elif a.cmd == "knn":
        run_knn(a)
    elif a.cmd == "blocks":
        run_blocks(a)
    elif a.cmd == "multiples":
        run_multiples(a)


if __name__ == "__main__":
    main()
