"""The config-2 workload at its own size: Plummer N = 65536 with a Salpeter
IMF (slope -2.35, masses 0.1-100, total mass 1, re-scaled to virial after the
masses), eps2 = 1e-6, evolved by the device block-step driver.  At the
blocks the scheduler produces (ph4's scheduler: all particles whose
t + dt equals the smallest one), the split force on the block's slots is
checked against the oracle's ph4 force loop on the same predicted state,
with the tolerances of test_gpu_force (acc and pot <= 1e-6 for every
particle, nn equal to ph4's except at exact distance ties)."""
import os

import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from amuse_gb300 import ic
from test_gpu_force import check_force

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

N = 65536
EPS2 = 1e-6


def _salpeter_system(g6, torch):
    ilist = torch.arange(N, dtype=torch.int32, device="cuda")

    def gpu_potential(mass, pos):
        g6.set_precision(ag.FP64)
        g6.load_particles(mass, pos, np.zeros_like(pos))
        pot = torch.empty(N, dtype=torch.float64, device="cuda")
        acc = torch.empty((N, 3), dtype=torch.float64, device="cuda")
        jerk = torch.empty_like(acc)
        g6.force_slots(0.0, 0.0, N, ilist.data_ptr(), N, acc.data_ptr(), jerk.data_ptr(),
                       pot.data_ptr(), None)
        return 0.5 * float(np.sum(mass * pot.cpu().numpy()))

    rng = np.random.RandomState(1)
    m, x, v = ic.plummer_salpeter(N, mass_min=0.1, mass_max=100.0, rng=rng,
                                  potential_energy=gpu_potential)
    g6.set_precision(ag.SPLIT)
    return m, x, v


def _block_force(g6, torch, m, st, threads):
    """The next scheduler block of the state st: GPU split force on its slots
    at the block time vs the oracle on the oracle-predicted state."""
    tend = st["time"] + st["timestep"]
    tnext = tend.min()
    blk = np.nonzero(tend == tnext)[0].astype(np.int32)
    pp, pv = oracle.predict(tnext, st["time"], st["pos"], st["vel"], st["acc"], st["jerk"])
    ref = oracle.force(m, pp, pv, EPS2, pp[blk], pv[blk], threads=threads)
    ni = len(blk)
    il = torch.tensor(blk, device="cuda")
    acc = torch.empty((ni, 3), dtype=torch.float64, device="cuda")
    jerk = torch.empty_like(acc)
    pot = torch.empty(ni, dtype=torch.float64, device="cuda")
    nn = torch.empty(ni, dtype=torch.int32, device="cuda")
    g6.force_slots(tnext, EPS2, N, il.data_ptr(), ni, acc.data_ptr(), jerk.data_ptr(),
                   pot.data_ptr(), nn.data_ptr())
    out = dict(acc=acc.cpu().numpy(), jerk=jerk.cpu().numpy(), pot=pot.cpu().numpy(),
               nn=nn.cpu().numpy())
    return blk, out, ref, pp


def test_c2_force_at_scheduler_blocks(g6):
    torch = pytest.importorskip("torch")
    threads = os.cpu_count() or 1
    m, x, v = _salpeter_system(g6, torch)
    g6.load_particles(m, x, v)

    # t = 0: every particle (ni = N)
    blk = np.arange(N, dtype=np.int32)
    ref = oracle.force(m, x, v, EPS2, x, v, threads=threads)
    out = g6.force(0.0, EPS2, N, x, v, self_slot=blk)
    check_force(out, ref, ag.SPLIT, x, x, label=f"C2 t=0 ni={N}")

    g6.run_init(EPS2, 0.14)
    sizes = []
    for hop in (1, 2, 5, 10, 30, 100, 300, 1000):
        g6.run(1e30, max_blocks=hop)
        st = g6.read_particles(N)
        blk, out, ref, pp = _block_force(g6, torch, m, st, threads)
        sizes.append(len(blk))
        check_force(out, ref, ag.SPLIT, pp, pp[blk],
                    label=f"C2 t={g6.system_time():.6f} ni={len(blk)}")
    print("block sizes checked:", [N] + sizes)
    assert max(sizes) > 1  # blocks of more than one particle were among them
