"""Benchmark: Hermite pair-interactions/s of the split-precision force path.

Workload (the precision configuration): Plummer sphere N = 2^20, equal mass,
eps2 = 1e-6, FP64 state, seeded synthetic input (numpy seed 1, AMUSE's
generator restated in amuse_gb300.ic).  One step = one shared Hermite step of
all N particles on the device: FP64 j-prediction, split-precision force
(acc, jerk, pot) on all N i-particles (N*(N-1) pair interactions), FP64
corrector.  As in ph4's step (gpu.cc:394-407 calls g6calc_lasthalf unless a
particle's step is below dtmin) the nearest-neighbour search is off in the
step; its cost is reported separately ("with_nn").  Inputs are
resident in HBM; L2 is flushed (256 MB write) between timed steps.

Reported next to it:
  e2e          the same metric through the GRAPE-6 C ABI with host buffers
               (g6_set_j_particle for all N, g6_set_ti, g6calc_firsthalf /
               lasthalf chunked by npipes, as ph4's gpu.cc calls it);
  predictor    the FP64 j-predictor's time, HBM GB/s and FP64-pipe fraction
               (on GB300 its FP64 arithmetic, not HBM, bounds it);
  fp64         the plain FP64 GPU kernel's pairs/s and the split kernel's,
               both on the same 16384-particle i-subset (the 2048 nearest
               the centre among them) against all N j, nn off in both;
  errors       per-particle relative acc/jerk/pot errors of the split
               results against the FP64 kernel's on that subset;
  roofline     the force kernel against the FP32 peak, 60 flop/pair (ph4's
               convention, src/amuse_ph4/src/jdata.cc:1038);
  cpu_baseline the oracle port of ph4's CPU force loop on the host cores
               (bounded i-sample against all N j), all cores, and one core
               in cpu_baseline.single_core.

--impl reference times the reference's CPU force path (ph4's
idata::get_partial_acc_and_jerk restated in oracle/, all host threads).

Secondary workloads (one JSON line each; not the headline metric):
  --workload batch    4096 few-body systems through g6x_batch_run
                      (amuse_gb300.workloads.run_batch) with the oracle's
                      smallN restatement timed on the host cores on the
                      same sample of systems as cpu_baseline;
  --workload multiples  4096 binary-single scatterings resolved by the
                      multiples hand-off (amuse_gb300.workloads.run_multiples)
                      with the same loop on the host cores (the oracle's
                      smallN with unperturbed binaries, then the structure
                      check) on a sample of the encounters as cpu_baseline;
  --workload adjoint  the differentiable fixed-step Hermite at n = 16384
                      (amuse_gb300.workloads.run_adjoint) with the oracle's
                      restatement of the hermite code's step timed on the
                      host cores as cpu_baseline.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# The metric as the benchmark specification names it; both arms print it.
METRIC = "Hermite pair-interactions/s, split-prec vs plain FP64 GPU, at |\u0394E/E|\u22641e-6"
FLOP_PER_PAIR = 60.0
PRED_FP64_OPS = 36  # FP64-pipe operations per j of the split-record predictor
# DRAM bytes (read + write) of one force launch at the default N = 2^20, from
# one ncu capture of this benchmark (profiles/force_kernel_dram_n1048576.md).
FORCE_TRAFFIC_N = 1 << 20
FORCE_TRAFFIC_BYTES = 81806592 + 89248256
N_DEFAULT = 1 << 20
EPS2 = 1e-6
ETA = 0.01
DT_STEP = 2.0 ** -12


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="force", choices=["force", "batch", "multiples", "adjoint"])
    # batch workload
    ap.add_argument("--nsys", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--eta", type=float, default=0.14)
    ap.add_argument("--max-steps", type=int, default=2_000_000)
    ap.add_argument("--cpu-sample", type=int, default=64)
    ap.add_argument("--batch-mode", default="split", choices=["fast", "exact", "split"])
    ap.add_argument("--no-unpert", action="store_true",
                    help="batch without smallN's unperturbed binaries")
    # multiples workload
    ap.add_argument("--end-time", type=float, default=1000.0)
    ap.add_argument("--delta-t", type=float, default=10.0)
    # adjoint workload
    ap.add_argument("--nsteps", type=int, default=256)
    ap.add_argument("--fd-coords", type=int, default=32)
    ap.add_argument("--fd64-coords", type=int, default=4)
    return ap.parse_args()




def workload(n):
    from amuse_gb300 import ic
    np.random.seed(1)
    return ic.plummer(n, do_scale=False)


def config(n):
    """The workload both arms measure (identical dict in both JSON lines)."""
    return {"workload": f"plummer N={n} equal mass eps2={EPS2} (numpy seed 1); per step the "
                        f"Hermite force (acc, jerk, pot) on all N i-particles against all N j",
            "n": n, "eps2": EPS2,
            "l2": "GPU arm: flushed by a 256 MB write between timed steps; CPU arm: n/a"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [q.strip() for q in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
                power.append(float(p[3]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_baseline(mass, pos, vel, seconds, threads):
    """ph4 CPU force loop (oracle port) on a bounded i-sample against all j."""
    import oracle
    oracle.build_port()
    n = len(mass)
    probe = max(threads, 8)
    t0 = time.perf_counter()
    oracle.force(mass, pos, vel, EPS2, pos[:probe], vel[:probe], threads=threads)
    dt = time.perf_counter() - t0
    rate = probe * (n - 1) / max(dt, 1e-9)
    ni = int(max(threads, min(n, rate * seconds / (n - 1))))
    t0 = time.perf_counter()
    oracle.force(mass, pos, vel, EPS2, pos[:ni], vel[:ni], threads=threads)
    dt = time.perf_counter() - t0
    return {"value": ni * (n - 1) / dt, "unit": "pair-interactions/s", "cores": threads,
            "kind": "port",
            "sample": f"{ni} i-particles x {n} j (ph4 idata::get_partial_acc_and_jerk "
                      f"restated in oracle/g6_oracle.c, {threads} threads, {dt:.1f} s)"}


def single_core_baseline(mass, pos, vel, cpu_seconds):
    """The same loop on one core (a short sample: a fifth of the all-core
    budget, at most 3 s)."""
    one = cpu_baseline(mass, pos, vel, min(3.0, cpu_seconds / 5), 1)
    return {"value": one["value"], "unit": one["unit"], "cores": 1, "sample": one["sample"]}


def run_reference(args):
    from amuse_gb300 import replicas
    rank, world, _ = replicas.env()
    if rank != 0:
        return 0
    mass, pos, vel = workload(args.n)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(mass, pos, vel, max(1.0, args.cpu_seconds / 4), threads)
    for _ in range(args.steps):
        vals.append(cpu_baseline(mass, pos, vel, args.cpu_seconds / 2, threads))
    v = statistics.median([c["value"] for c in vals])
    line = {
        "impl": "reference", "metric": METRIC,
        "value": v, "unit": "pair-interactions/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Plummer, AMUSE generator restated)",
        "config": config(args.n),
        "path": "ph4's CPU force loop idata::get_partial_acc_and_jerk (FP64; it always "
                "finds the nearest neighbour too), restated in oracle/g6_oracle.c, all host "
                "threads, on a bounded i-sample against all N j",
        "cpu_baseline": {"value": v, "unit": "pair-interactions/s", "cores": threads,
                         "kind": "port", "sample": vals[-1]["sample"]},
        "e2e": {"value": v, "unit": "pair-interactions/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch

    import amuse_gb300 as ag
    from amuse_gb300 import build as b

    from amuse_gb300 import replicas
    rank, world, local = replicas.env()
    replicas.init("nccl")
    torch.cuda.set_device(local)
    if local == 0:
        b.build()  # one builder per node; the other ranks wait for it
    replicas.barrier()
    n = args.n
    mass, pos, vel = workload(n)
    g6 = ag.G6X(local)
    g6.set_precision(ag.SPLIT)
    g6.load_particles(mass, pos, vel)
    g6.run_init(EPS2, ETA)
    k0, u0 = g6.energy()
    e0 = k0 + u0
    stream = torch.cuda.ExternalStream(g6.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    t = 0.0

    def one_step():
        nonlocal t
        t += DT_STEP
        g6.step_all(t)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    replicas.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    g6.timing(True)
    times, fms, kms, rms, pms, launches = [], [], [], [], [], 0
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e_a = torch.cuda.Event(enable_timing=True)
        e_b = torch.cuda.Event(enable_timing=True)
        e_a.record(stream)
        one_step()
        e_b.record(stream)
        e_b.synchronize()
        times.append(e_a.elapsed_time(e_b) / 1e3)
        st = g6.stats()
        fms.append(st["force_ms"])
        kms.append(st["kernel_ms"])
        rms.append(st["refine_ms"])
        pms.append(st["predict_ms"])
        launches += 4  # predict, force (split merge inside), refinement pass, correct
    torch.cuda.synchronize()
    g6.timing(False)
    refine_all = g6.refine_stats()  # the last timed step's refinement pass
    clocks = sampler.stop()
    total = replicas.max_over_ranks(sum(times), device=f"cuda:{local}")
    k1, u1 = g6.energy()
    e1 = k1 + u1
    pairs_step = n * (n - 1)
    value = replicas.whole_job_rate(args.steps * pairs_step, world, total)
    # the roofline is the force kernel's own (CUDA events around it alone);
    # the refinement pass that follows it is timed apart
    force_s = statistics.mean(kms) / 1e3
    achieved = FLOP_PER_PAIR * pairs_step / force_s / 1e12
    pk = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = nsm * 128 * 2 * sm_max * 1e6 / 1e12
    pred_gbs = (n * (15 * 8 + 4 + 48)) / (statistics.mean(pms) / 1e3) / 1e9 if pms[0] > 0 else None

    # plain FP64 GPU kernel and the split kernel on the same i-subset (nn off
    # in both, as in the timed step): the like-for-like speed-up, and the
    # split results' per-particle errors against FP64.  The subset holds the
    # 2048 particles nearest the centre (the worst-conditioned sums) and the
    # first 14336 of the others.
    nsub = min(n, 16384)
    r = np.linalg.norm(pos, axis=1)
    core = np.argsort(r)[: min(2048, nsub // 8)]
    rest = np.setdiff1d(np.arange(n), core)[: nsub - len(core)]
    sub = np.sort(np.concatenate([core, rest])).astype(np.int32)
    d_il = torch.tensor(sub, dtype=torch.int32, device=f"cuda:{local}")

    def subset_forces(prec):
        g6.set_precision(prec)
        acc = torch.empty(nsub * 3, dtype=torch.float64, device=f"cuda:{local}")
        jerk = torch.empty_like(acc)
        pot = torch.empty(nsub, dtype=torch.float64, device=f"cuda:{local}")
        g6.timing(True)
        ms = []
        for rep in range(3):
            g6.force_slots(t, EPS2, n, d_il.data_ptr(), nsub, acc.data_ptr(), jerk.data_ptr(),
                           pot.data_ptr(), None, sync=True)
            if rep:
                ms.append(g6.stats()["force_ms"])
        g6.timing(False)
        res = (acc.view(nsub, 3).cpu().numpy(), jerk.view(nsub, 3).cpu().numpy(),
               pot.cpu().numpy())
        return statistics.mean(ms), res

    fp64_ms, d64 = subset_forces(ag.FP64)
    sub_ms, d32 = subset_forces(ag.SPLIT)
    refine_sub = g6.refine_stats()
    fp64_rate = nsub * (n - 1) / (fp64_ms / 1e3)
    sub_rate = nsub * (n - 1) / (sub_ms / 1e3)
    split_rate = pairs_step / force_s

    def qstats(e):
        return {"p50": float(np.percentile(e, 50)), "p99": float(np.percentile(e, 99)),
                "max": float(e.max()), "frac_le_1e-6": float(np.mean(e <= 1e-6))}

    errors = {
        "against": "plain FP64 GPU kernel, same particles and j-set",
        "sample": f"{nsub} i-particles ({len(core)} nearest the centre) x {n} j",
        "acc": qstats(np.linalg.norm(d32[0] - d64[0], axis=1) / np.linalg.norm(d64[0], axis=1)),
        "jerk": qstats(np.linalg.norm(d32[1] - d64[1], axis=1) / np.linalg.norm(d64[1], axis=1)),
        "pot": qstats(np.abs(d32[2] - d64[2]) / np.abs(d64[2])),
        "refined": {"condition_fp64": refine_sub["kappa"],
                    "dominant_term": refine_sub["dominant"]}}

    # the same split kernel with the nearest-neighbour search on (what
    # g6calc_lasthalf2 asks for), on a 65536-particle i-subset
    nsub2 = min(n, 65536)
    d_il2 = torch.arange(nsub2, dtype=torch.int32, device=f"cuda:{local}")
    d_a2 = torch.empty(nsub2 * 3, dtype=torch.float64, device=f"cuda:{local}")
    d_j2 = torch.empty_like(d_a2)
    d_p2 = torch.empty(nsub2, dtype=torch.float64, device=f"cuda:{local}")
    d_n2 = torch.empty(nsub2, dtype=torch.int32, device=f"cuda:{local}")
    g6.timing(True)
    nn_ms, nn_kms, nn_rms = [], [], []
    for r in range(3):
        g6.force_slots(t, EPS2, n, d_il2.data_ptr(), nsub2, d_a2.data_ptr(), d_j2.data_ptr(),
                       d_p2.data_ptr(), d_n2.data_ptr(), sync=True)
        if r:
            st2 = g6.stats()
            nn_ms.append(st2["force_ms"])
            nn_kms.append(st2["kernel_ms"])
            nn_rms.append(st2["refine_ms"])
    g6.timing(False)
    nn_refine = g6.refine_stats()
    nn_rate = nsub2 * (n - 1) / (statistics.mean(nn_ms) / 1e3)
    # the kernel's own rate (force kernel + split-j merge, CUDA events
    # around them), the basis of the headline roofline too
    nn_kernel_rate = nsub2 * (n - 1) / (statistics.mean(nn_kms) / 1e3)

    # end to end through the GRAPE-6 ABI with host buffers
    e2e = None
    if not args.no_e2e:
        x, v = pos.copy(), vel.copy()
        ids = np.arange(1, n + 1, dtype=np.int32)
        out = dict(acc=np.zeros((n, 3)), jerk=np.zeros((n, 3)), pot=np.zeros(n),
                   nn=np.zeros(n, np.int32))
        # warm (pinned buffers, capacities)
        # ph4's common path: g6calc_lasthalf (no neighbour), as in the timed step
        ag.drive_load(mass, x, v, ids=ids)
        ag.drive_force(n, 0.0, EPS2, ids, x, v, want_nn=False, out=out)
        e2e_t = []
        for _ in range(max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ag.drive_load(mass, x, v, ids=ids)          # j updates for all N (ph4 update_gpu)
            ag.drive_force(n, 0.0, EPS2, ids, x, v, want_nn=False, out=out)
            e2e_t.append(time.perf_counter() - t0)
        e2e = {"value": pairs_step / statistics.median(e2e_t), "unit": "pair-interactions/s",
               "h2d_bytes_per_step": n * (128 + 6 * 8 + 8 + 4),
               "d2h_bytes_per_step": n * 7 * 8 + 16 * ((n + 16383) // 16384),
               "path": "g6_set_j_particle x N + g6_set_ti + g6calc_firsthalf/lasthalf "
                       "chunks of g6_npipes()=16384 (libg6drive.so, ph4 gpu.cc order)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(mass, pos, vel, args.cpu_seconds, os.cpu_count() or 1)
        cpu["single_core"] = single_core_baseline(mass, pos, vel, args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "pair-interactions/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Plummer, AMUSE generator restated)",
            "config": config(n),
            "step": "one shared Hermite step dt=2^-12 of all N on the device: FP64 predict, "
                    "split force (nn off, as g6calc_lasthalf) with its refinement pass, FP64 "
                    "correct",
            "parallelism": f"replicas x{world}",
            "energy": {"dE_over_E": (e1 - e0) / abs(e0), "steps": args.warmup + args.steps,
                       "E0": e0, "E1": e1},
            "fp64": {"value": fp64_rate, "unit": "pair-interactions/s",
                     "sample": f"{nsub} i x {n} j, nn off",
                     "split_same_sample": sub_rate,
                     "split_over_fp64": split_rate / fp64_rate,
                     "split_over_fp64_same_sample": sub_rate / fp64_rate},
            "errors": errors,
            "with_nn": {"value": nn_rate, "unit": "pair-interactions/s",
                        "sample": f"{nsub2} i x {n} j, nearest neighbour on (g6calc_lasthalf2)",
                        "frac_fp32": FLOP_PER_PAIR * nn_kernel_rate / 1e12 / fp32_peak,
                        "frac_basis": "force kernel + split-j merge alone, as roofline.frac",
                        "call_frac_fp32": FLOP_PER_PAIR * nn_rate / 1e12 / fp32_peak,
                        "kernel_ms": statistics.mean(nn_kms),
                        "refine_ms": statistics.mean(nn_rms),
                        "refined": nn_refine},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                         "traffic": FORCE_TRAFFIC_BYTES if n == FORCE_TRAFFIC_N else None,
                         "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + "
                                         "dram__bytes_write.sum, one capture at N = 2^20)",
                         "kernel": "force_kernel<SplitP,1,false> (packed f32x2)",
                         "peak_source": f"{nsm} SMs x 128 FP32 lanes x 2 flop x {sm_max:.0f} MHz "
                                        "(sm_max_mhz, MEASURED_PEAKS.json; it holds no FP32 figure)",
                         "flop_per_pair": FLOP_PER_PAIR, "force_ms": 1e3 * force_s},
            "refine": {"ms": statistics.mean(rms), "particles": refine_all["queued"],
                       "of_which_condition": refine_all["kappa"],
                       "of_which_dominant_term": refine_all["dominant"],
                       "share_of_step": statistics.mean(rms) / (1e3 * total / args.steps),
                       "what": "refine_kernel after the force kernel: acc and pot redone in "
                               "FP64 where the FP32 sum is ill-conditioned (kappa > 48), with "
                               "compensated FP32 sums and the large terms in FP64 where one "
                               "term exceeds |a|"},
            "predictor": {"ms": statistics.mean(pms), "GB_s": pred_gbs,
                          "bytes_per_j": 15 * 8 + 4 + 48,
                          "hbm_peak_gbs": pk.get("hbm_gbs"),
                          # ph4's FP64 expression: ~20 FP64 ops per j for x and v,
                          # plus ~16 conversions for the double-single record
                          "bound": "fp64",
                          "fp64_ops_per_j": PRED_FP64_OPS,
                          "fp64_frac": (PRED_FP64_OPS * n / (statistics.mean(pms) / 1e3)
                                        / (nsm * 2 * sm_max * 1e6)) if pms[0] > 0 else None,
                          "fp64_peak_source": f"{nsm} SMs x 2 FP64 lanes x {sm_max:.0f} MHz "
                                              "(GB300 FP64 = 1/64 of FP32)"},
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    replicas.finalize()
    return 0


def run_secondary(args):
    """The batch / multiples / adjoint workloads with their host-core
    baselines."""
    from amuse_gb300 import workloads
    import oracle
    oracle.build_port()
    threads = os.cpu_count() or 1
    if args.workload == "batch":
        args.seed = 1 if args.seed is None else args.seed
        out, smp = workloads.run_batch(args)
        off = smp["off"]

        def one(s):
            a, b = off[s], off[s + 1]
            if smp["unpert"]:
                return oracle.smalln_unpert(smp["mass"][a:b], smp["pos"][a:b], smp["vel"][a:b],
                                            args.eta, smp["t_end"], max_steps=args.max_steps)
            return oracle.smalln(smp["mass"][a:b], smp["pos"][a:b], smp["vel"][a:b], args.eta,
                                 smp["t_end"], max_steps=args.max_steps)

        import concurrent.futures as cf
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, range(len(off) - 1)))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": (len(off) - 1) / dt, "unit": "systems/s", "cores": threads, "kind": "port",
            "sample": f"the first {len(off) - 1} systems (smallN"
                      f"{' with unperturbed binaries' if smp['unpert'] else ''} restated in "
                      f"oracle/g6_oracle.c, same step cap), {dt:.1f} s"}
    elif args.workload == "multiples":
        args.seed = 1 if args.seed is None else args.seed
        out, sample = workloads.run_multiples(args)

        from amuse_gb300 import multiples

        def smalln_host(m, x, v, dt):
            x, v, tf, _, _ = oracle.smalln_unpert(m, x, v, args.eta, dt,
                                                  max_steps=args.max_steps)
            return x, v, tf

        def one(sys_):
            # resolve_collision's loop on the host (the decisions of
            # resolve_encounters) around the oracle's smallN
            multiples.resolve_serial(smalln_host, *sys_, args.end_time, args.delta_t)

        import concurrent.futures as cf
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, sample))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": len(sample) / dt, "unit": "encounters/s", "cores": threads, "kind": "port",
            "sample": f"all {len(sample)} encounters through the same loop (smallN with "
                      f"unperturbed binaries restated in oracle/g6_oracle.c, FP64, then the "
                      f"structure check), {dt:.1f} s"}
    else:
        args.seed = 7 if args.seed is None else args.seed
        args.n = 16384 if args.n == N_DEFAULT else args.n
        out = workloads.run_adjoint(args)
        from amuse_gb300 import ic
        rng = np.random.RandomState(args.seed)
        m, x, v = ic.plummer(args.n, do_scale=True, rng=rng)
        t0 = time.perf_counter()
        oracle.hermite_fixed(m, x, v, 1e-4, 1.0 / 256, 1)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": 2 * args.n * (args.n - 1) / dt, "unit": "pair-interactions/s (forward)",
            "cores": 1, "kind": "port",
            "sample": f"one fixed step (2 force evaluations) of the hermite code's scheme "
                      f"restated in oracle/g6_oracle.c at n={args.n}, {dt:.1f} s"}
    print(json.dumps(out), flush=True)
    return 0


def main():
    args = parse()
    if args.workload != "force":
        return run_secondary(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
