"""The device-resident ph4-style integration (extension API): initial steps,
block-step loop with the FP64 corrector and Aarseth step, energy, against
the golden run of the unmodified ph4 loop (config 1: N=1024 Plummer,
eps2=1e-4, eta=0.01, t=1)."""
import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from amuse_gb300 import ic
from conftest import golden

pytestmark = pytest.mark.gpu


def _run(g6, prec, mass, pos, vel, eps2, eta, t_end):
    g6.set_precision(prec)
    try:
        g6.load_particles(mass, pos, vel)
        g6.run_init(eps2, eta)
        k0, u0 = g6.energy()
        nb, ns = g6.run(t_end)
        k1, u1 = g6.energy()
        st = g6.read_particles(len(mass))
    finally:
        g6.set_precision(ag.SPLIT)
    st.update(E0=k0 + u0, E1=k1 + u1, blocks=nb, steps=ns)
    return st


def test_block_run_c1_fp64(g6):
    """Config 1 (eta = 0.01) with FP64 forces vs the golden ph4 run."""
    g = golden("run_plummer1024_t1.npz")
    r = _run(g6, ag.FP64, g["mass"], g["pos0"], g["vel0"], 1e-4, 0.01, 1.0)
    de = (r["E1"] - r["E0"]) / abs(r["E0"])
    print(f"fp64 blocks={r['blocks']} (ph4 {int(g['blocks'])}) steps={r['steps']:.0f} "
          f"(ph4 {float(g['total_steps']):.0f}) E0={r['E0']:.15f} (ph4 {float(g['E0']):.15f}) "
          f"dE/E={de:.2e} (ph4 {(float(g['E1']) - float(g['E0'])) / abs(float(g['E0'])):.2e})")
    assert abs(r["E0"] - float(g["E0"])) <= 1e-12 * abs(float(g["E0"]))
    assert abs(de) <= 1e-6
    assert abs(r["blocks"] - float(g["blocks"])) <= 0.02 * float(g["blocks"])
    assert np.all(r["time"] + r["timestep"] > 1.0 - 1e-12)
    assert np.max(np.abs(r["pos"] - g["pos"])) < 1e-5


def test_block_run_split_default_eta(g6):
    """Split-precision forces at ph4's default eta = 0.14 reproduce the FP64
    scheme: same block structure, same energy to |dE/E| <= 1e-6.  (At
    eta <= 0.03 FP32-level force noise dominates the Aarseth criterion's
    third differences and the steps shrink; that regime needs FP64 forces.)"""
    np.random.seed(1)
    m, x, v = ic.plummer(1024, do_scale=True)
    ref = oracle.run(m, x, v, 1e-4, 0.14, 1.0, threads=8)
    r = _run(g6, ag.SPLIT, m, x, v, 1e-4, 0.14, 1.0)
    de = (r["E1"] - r["E0"]) / abs(r["E0"])
    de_ref = (ref["E1"] - ref["E0"]) / abs(ref["E0"])
    print(f"split eta=0.14 blocks={r['blocks']} (ph4 {ref['blocks']}) dE/E={de:.2e} (ph4 {de_ref:.2e})")
    assert abs(r["E0"] - ref["E0"]) <= 1e-6 * abs(ref["E0"])
    assert abs(de) <= 1e-6
    assert abs(r["blocks"] - ref["blocks"]) <= 0.02 * ref["blocks"]


def test_step_all_energy(g6):
    np.random.seed(21)
    n = 4096
    m, x, v = ic.plummer(n)
    g6.load_particles(m, x, v)
    g6.run_init(1e-4, 0.01)
    k0, u0 = g6.energy()
    t = 0.0
    for _ in range(8):
        t += 2.0 ** -10
        g6.step_all(t)
    k1, u1 = g6.energy()
    de = ((k1 + u1) - (k0 + u0)) / abs(k0 + u0)
    print(f"step_all dE/E={de:.2e}")
    assert abs(de) < 1e-7
    assert g6.system_time() == t


def test_force_dev_without_nn(g6):
    """Device-pointer entry with no nearest-neighbour outputs requested."""
    torch = pytest.importorskip("torch")
    np.random.seed(22)
    n = 3000
    m, x, v = ic.plummer(n)
    g6.load_particles(m, x, v)
    sel = np.arange(0, n, 3)
    dx = torch.tensor(x[sel], device="cuda").contiguous()
    dv = torch.tensor(v[sel], device="cuda").contiguous()
    ds = torch.tensor(sel, dtype=torch.int32, device="cuda")
    da = torch.empty((len(sel), 3), dtype=torch.float64, device="cuda")
    dj = torch.empty_like(da)
    dp = torch.empty(len(sel), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    g6.force_dev(0.0, 1e-4, n, len(sel), dx.data_ptr(), dv.data_ptr(), ds.data_ptr(),
                 da.data_ptr(), dj.data_ptr(), dp.data_ptr(), None, None, sync=True)
    ref = oracle.force(m, x, v, 1e-4, x[sel], v[sel])
    ea = np.linalg.norm(da.cpu().numpy() - ref["acc"], axis=1) / np.linalg.norm(ref["acc"], axis=1)
    assert np.percentile(ea, 99) < 1e-6
    assert np.allclose(dp.cpu().numpy(), ref["pot"], rtol=1e-6)


@pytest.mark.parametrize("prec", [ag.SPLIT, ag.FP64], ids=["split", "fp64"])
def test_initial_step_bitexact(g6, prec):
    """g6x_run_init's initial time steps (initial_step_kernel + the median
    limit, jdata.cc:503-580 with force_initial_timestep(0.0625, 0.03125, 8),
    interface.cc:29-31) equal the oracle's set_initial_timestep bit for bit,
    on the config-1 particles, from the accelerations and jerks the device
    stored at t = 0."""
    g = golden("run_plummer1024_t1.npz")
    n = len(g["mass"])
    g6.set_precision(prec)
    try:
        g6.load_particles(g["mass"], g["pos0"], g["vel0"])
        g6.run_init(float(g["eps2"]), float(g["eta"]))
        st = g6.read_particles(n)
    finally:
        g6.set_precision(ag.SPLIT)
    ref = oracle.initial_step(st["acc"], st["jerk"], float(g["eta"]), fac=0.0625,
                              limit=0.03125, limitm=8.0)
    assert np.array_equal(st["timestep"], ref)
    assert np.all(st["time"] == 0.0)
