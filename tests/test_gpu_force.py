"""GPU parity of the force path through the C ABI, against the oracle.

Tolerances (per-particle relative errors against ph4's FP64 CPU loop):
  split precision (FP32 pair terms on double-single positions, with the
  refinement pass: ill-conditioned sums redone in FP64):
    acc  : |da|/|a| <= 1e-6 for every particle
    pot  : |dp|/|p| <= 1e-6 for every particle
    jerk : |dj|/|j| <= JERK_P99_SPLIT at p99, <= JERK_MAX_SPLIT for every
           particle (the jerk sum cancels more than the acceleration; its
           error is stated, not bounded by the condition-number pass; at
           N = 2^20 its p99 is 0.9e-6, on a few hundred particles of a small
           system the p99 is the third-worst value)
  FP64: acc/pot <= 1e-12, jerk <= 1e-12 at p99 and 1e-10 for every particle.
  nn (both): the oracle's index (ph4: smallest FP64 r^2, first j on equal
  values), except where the two indices' FP64 r^2 are equal.
"""
import numpy as np
import pytest

import amuse_gb300 as ag
import oracle
from amuse_gb300 import ic
from conftest import golden

pytestmark = pytest.mark.gpu

JERK_P99_SPLIT = 1.5e-6
JERK_MAX_SPLIT = 1e-4
TOL = {ag.SPLIT: dict(accmax=1e-6, pot=1e-6, jerk99=JERK_P99_SPLIT, jerkmax=JERK_MAX_SPLIT),
       ag.FP64: dict(accmax=1e-12, pot=1e-12, jerk99=1e-12, jerkmax=1e-10)}


def vrel(a, b):
    return np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), 1e-300)


def ph4_r2(xj, xi):
    """ph4's squared distance (idata.cc:200-205): dx = x_j - x_i, summed in
    component order with IEEE operations (numpy does not contract)."""
    d = xj - xi
    return (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]


def check_nn(got, want, jpos, ipos, label=""):
    """nn equal to the oracle's except at exact FP64 distance ties."""
    bad = np.nonzero(got != want)[0]
    ties = 0
    for i in bad:
        assert got[i] >= 0, (label, i, got[i], want[i])
        d_got = ph4_r2(jpos[got[i]], ipos[i])
        d_want = ph4_r2(jpos[want[i]], ipos[i])
        assert d_got == d_want, (label, i, got[i], want[i], d_got, d_want)
        ties += 1
    return ties


def check_force(out, ref, prec, jpos=None, ipos=None, nn_is_id=False, label=""):
    t = TOL[prec]
    ea = vrel(out["acc"], ref["acc"])
    ej = vrel(out["jerk"], ref["jerk"])
    ep = np.abs(out["pot"] - ref["pot"]) / np.abs(ref["pot"])
    print(f"{label} prec={prec} acc p50={np.median(ea):.2e} p99={np.percentile(ea, 99):.2e} "
          f"max={ea.max():.2e} | jerk p99={np.percentile(ej, 99):.2e} max={ej.max():.2e} | "
          f"pot max={ep.max():.2e}")
    assert ea.max() <= t["accmax"]
    assert ep.max() <= t["pot"]
    assert np.percentile(ej, 99) <= t["jerk99"]
    assert ej.max() <= t["jerkmax"]
    if "nn" in out and jpos is not None:
        got = out["nn"] - (1 if nn_is_id else 0)
        return check_nn(got, ref["nn"], jpos, ipos, label)
    return 0


@pytest.fixture(params=[ag.SPLIT, ag.FP64], ids=["split", "fp64"])
def prec(request, g6):
    g6.set_precision(request.param)
    yield request.param
    g6.set_precision(ag.SPLIT)


def test_force_c1_golden_via_g6_api(g6, prec):
    """Config-1 inputs through g6_set_j_particle + chunked g6calc calls."""
    g = golden("force_plummer1024_eps1e-4.npz")
    n = len(g["mass"])
    ids = np.arange(1, n + 1)
    ag.drive_load(g["mass"], g["pos"], g["vel"], ids=ids)
    out = ag.drive_force(n, 0.0, 1e-4, ids, g["pos"], g["vel"], want_nn=True)
    check_force(out, g, prec, g["pos"], g["pos"], nn_is_id=True, label="C1")


def test_force_salpeter_offsets(g6, prec):
    """Config-2 shape (Salpeter masses, eps2=1e-6); half the i-particles are
    displaced by ~1e-7 (not their j copy: ids outside the j-set)."""
    g = golden("force_salpeter4096_eps1e-6.npz")
    n = len(g["mass"])
    ids = np.arange(1, n + 1)
    ag.drive_load(g["mass"], g["pos"], g["vel"], ids=ids)
    iids = g["isel"] + 1
    iids[:350] = -1 - np.arange(350)
    out = ag.drive_force(n, 0.0, 1e-6, iids, g["ipos"], g["ivel"], want_nn=True)
    check_force(out, g, prec, g["pos"], g["ipos"], nn_is_id=True, label="salpeter")


def test_force_eps0_zero_mass(g6, prec):
    g = golden("force_plummer128_eps0.npz")
    n = len(g["mass"])
    ids = np.arange(1, n + 1)
    ag.drive_load(g["mass"], g["pos"], g["vel"], ids=ids)
    out = ag.drive_force(n, 0.0, 0.0, ids, g["pos"], g["vel"], want_nn=True)
    # GRAPE semantics: a massless j may be a neighbour (the CPU skips it).
    keep = (out["nn"] - 1) != 5
    ref = {k: (g[k][keep] if k != "nn" else g[k][keep]) for k in ("acc", "jerk", "pot", "nn")}
    got = {k: out[k][keep] for k in ("acc", "jerk", "pot", "nn")}
    check_force(got, ref, prec, g["pos"], g["pos"][keep], nn_is_id=True, label="eps0")


@pytest.mark.parametrize("ni", [1, 2, 3, 7, 32, 100, 255, 256, 511, 512, 1000, 4096])
def test_force_block_sizes(g6, prec, ni):
    """Every launch shape (j-lanes 1..128, split-j across CTAs) vs the oracle."""
    np.random.seed(11)
    m, x, v = ic.plummer(4096)
    rng = np.random.RandomState(ni)
    sel = np.sort(rng.choice(4096, ni, replace=False))
    g6.load_particles(m, x, v)
    out = g6.force(0.0, 1e-4, 4096, x[sel], v[sel], self_slot=sel)
    ref = oracle.force(m, x, v, 1e-4, x[sel], v[sel])
    check_force(out, ref, prec, x, x[sel], label=f"ni={ni}")


def test_force_1m_subset_vs_oracle(g6, prec):
    """The precision configuration's particles (Plummer N = 2^20, eps2 = 1e-6):
    a 1024-particle i-subset against all N j, GPU vs the oracle's ph4 loop
    on the host cores.  This is the cross-check that makes the FP64 GPU kernel
    the oracle for the all-N error distribution."""
    import os
    n = 1 << 20
    np.random.seed(1)
    m, x, v = ic.plummer(n)
    sel = np.sort(np.random.RandomState(3).choice(n, 1024, replace=False))
    g6.load_particles(m, x, v)
    out = g6.force(0.0, 1e-6, n, x[sel], v[sel], self_slot=sel)
    ref = oracle.force(m, x, v, 1e-6, x[sel], v[sel], threads=os.cpu_count() or 1)
    check_force(out, ref, prec, x, x[sel], label="N=2^20")


def test_chunking_by_npipes(g6):
    np.random.seed(12)
    m, x, v = ic.plummer(2048)
    ids = np.arange(1, 2049)
    ag.drive_load(m, x, v, ids=ids)
    full = ag.drive_force(2048, 0.0, 1e-4, ids, x, v)
    g6.set_npipes(300)
    try:
        part = ag.drive_force(2048, 0.0, 1e-4, ids, x, v)
    finally:
        g6.set_npipes(16384)
    # different i-chunks may pick different launch shapes: equal to rounding
    d = vrel(part["acc"], full["acc"])
    assert np.percentile(d, 99) <= 1e-6 and d.max() <= 1e-5
    assert np.mean(part["nn"] == full["nn"]) > 0.999


def test_predictor_and_time_offsets(g6, prec):
    """j-particles at different times with acc/jerk, predicted on the GPU."""
    np.random.seed(13)
    n = 3000
    m, x, v = ic.plummer(n)
    base = oracle.force(m, x, v, 1e-4, x, v)
    rng = np.random.RandomState(5)
    t = rng.choice([0.0, 1 / 64, 1 / 32, 3 / 64], n)
    ti = 1 / 16
    ids = np.arange(1, n + 1)
    ag.drive_load(m, x, v, acc=base["acc"], jerk=base["jerk"], t=t, dt=np.full(n, 1 / 64),
                  ids=ids)
    pp, pv = oracle.predict(ti, t, x, v, base["acc"], base["jerk"])
    out = ag.drive_force(n, ti, 1e-4, ids, pp, pv)
    ref = oracle.force(m, pp, pv, 1e-4, pp, pv)
    check_force(out, ref, prec, pp, pp, nn_is_id=True, label="predict")


def test_corrector_bitexact(g6):
    """Device FP64 corrector + Aarseth step == oracle (predict + correct)."""
    np.random.seed(14)
    n = 1024
    m, x, v = ic.plummer(n)
    f0 = oracle.force(m, x, v, 1e-4, x, v)
    rng = np.random.RandomState(3)
    dt = 2.0 ** -rng.randint(6, 12, n)
    tnext = 1.0 / 64
    t = tnext - dt
    g6.load_particles(m, x, v, acc=f0["acc"], jerk=f0["jerk"], t=t, dt=dt)
    pp, pv = oracle.predict(tnext, t, x, v, f0["acc"], f0["jerk"])
    f1 = oracle.force(m, pp, pv, 1e-4, pp, pv)
    slots = np.arange(n)
    g6.correct(slots, tnext, 0.01, f1["acc"], f1["jerk"])
    got = g6.read_particles(n)
    ref = oracle.correct(tnext, 0.01, t, dt, pp, pv, f0["acc"], f0["jerk"], f1["acc"], f1["jerk"])
    assert np.array_equal(got["timestep"], ref["timestep"])
    assert np.array_equal(got["time"], ref["time"])
    assert np.array_equal(got["pos"], ref["pos"])
    assert np.array_equal(got["vel"], ref["vel"])


def test_deterministic(g6):
    np.random.seed(15)
    m, x, v = ic.plummer(5000)
    g6.load_particles(m, x, v)
    sel = np.arange(0, 5000, 7)
    a = g6.force(0.0, 1e-6, 5000, x[sel], v[sel], self_slot=sel)
    b = g6.force(0.0, 1e-6, 5000, x[sel], v[sel], self_slot=sel)
    for k in a:
        assert np.array_equal(a[k], b[k])


# --- known answers (src/amuse_ph4/tests/test_ph4.py) through the GPU ------

def _pair(g6, m1, m2, x2, eps2, pts=None):
    mass = np.array([m1, m2])
    pos = np.array([[0.0, 0, 0], [x2, 0, 0]])
    g6.load_particles(mass, pos, np.zeros((2, 3)))
    if pts is None:
        return g6.force(0.0, eps2, 2, pos, np.zeros((2, 3)), self_slot=[0, 1])
    return g6.force(0.0, eps2, 2, pts, np.zeros_like(pts))


def test_kat_pairs(g6, prec):
    tol = 1e-7 if prec == ag.SPLIT else 1e-14
    f = _pair(g6, 10.0, 10.0, 2.0, 0.01)
    assert f["pot"][0] == pytest.approx(-10.0 / np.sqrt(4.01), rel=tol)
    f = _pair(g6, 10.0, 1.0, 2.0, 0.0)
    assert f["pot"][0] == pytest.approx(-0.5, rel=tol)
    assert f["pot"][1] == pytest.approx(-5.0, rel=tol)
    assert f["nn"][0] == 1 and f["nn"][1] == 0


def test_kat_field_points(g6, prec):
    pots = [-4.57110767688, -2.66662518639, -2.13331892165]
    for x, pref in zip((0.25, 0.5, 0.75), pots):
        pts = np.array([[x, 0, 0], [2.0 - x, 0, 0]])
        f = _pair(g6, 1.0, 1.0, 2.0, 1e-5, pts)
        assert f["pot"][0] == pytest.approx(pref, rel=1e-5)
        assert f["pot"][1] == pytest.approx(f["pot"][0], rel=1e-5)
        fx = -1.0 / x ** 2 + 1.0 / (2.0 - x) ** 2
        assert f["acc"][0, 0] == pytest.approx(fx, rel=1e-2)
        assert f["acc"][0, 0] == pytest.approx(-f["acc"][1, 0], rel=1e-5)


def test_neighbour_lists(g6, prec):
    np.random.seed(16)
    n = 2000
    m, x, v = ic.plummer(n)
    ids = np.arange(1, n + 1)
    ag.drive_load(m, x, v, ids=ids)
    sel = np.arange(0, n, 13)
    h2 = np.full(len(sel), 0.01)
    h2[::2] = 0.05
    g6.set_ti(0.0)
    g6.calc(n, ids[sel], x[sel], v[sel], 1e-4, h2=h2)
    over = g6.read_neighbour_list()
    d2 = np.sum((x[None, :, :] - x[sel, None, :]) ** 2, axis=-1)
    any_over = False
    for q, i in enumerate(sel):
        want = np.sort(ids[(d2[q] <= h2[q]) & (np.arange(n) != i)])
        got, rc = g6.get_neighbour_list(q)
        if len(want) > ag.NGB_MAX:
            any_over = True
            assert rc == 1
            continue
        assert np.array_equal(got, want), q
    assert over == (1 if any_over else 0)


def test_error_codes(g6):
    np.random.seed(17)
    m, x, v = ic.plummer(64)
    ids = np.arange(1, 65)
    ag.drive_load(m, x, v, ids=ids)
    g6.set_npipes(16)
    try:
        with pytest.raises(ag.G6Error):
            g6.calc(64, ids, x, v, 1e-4)  # ni > npipes
    finally:
        g6.set_npipes(16384)
    with pytest.raises(ag.G6Error):
        g6.set_j_particle(-1, 1, 0.0, 0.0, 1.0, np.zeros(3), np.zeros(3), np.zeros(3),
                          np.zeros(3), np.zeros(3))
    # a normal call still works afterwards
    acc, jerk, pot, nn = g6.calc(64, ids, x, v, 1e-4)
    assert np.all(np.isfinite(acc))


# --- nearest neighbour: ties and near-ties, and the FP64 redo ------------

def test_nn_lattice_ties(g6, prec):
    """A cubic lattice with a power-of-two spacing: every particle has up to
    six neighbours at exactly the same FP64 distance, and ph4 takes the first
    (strict <).  The FP32 keys tie too, so the split path must rank the
    candidates in FP64 and take the smallest slot."""
    k = 8
    g = np.arange(k) * 0.125
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) - 0.4375
    n = len(x)
    m = np.full(n, 1.0 / n)
    v = np.random.RandomState(4).normal(0, 0.1, (n, 3))
    g6.load_particles(m, x, v)
    out = g6.force(0.0, 1e-4, n, x, v, self_slot=np.arange(n))
    ref = oracle.force(m, x, v, 1e-4, x, v)
    assert np.array_equal(out["nn"], ref["nn"])
    if prec == ag.SPLIT:
        st = g6.refine_stats()
        assert st["queued"] >= n // 2 and st["overflow"] == 0, st


def test_nn_near_ties(g6, prec):
    """Pairs of candidates whose distances differ by ~1e-9 relative (below
    FP32 resolution): the FP32 keys cannot order them, the FP64 ranking must."""
    rng = np.random.RandomState(21)
    n = 3000
    x = rng.uniform(-1, 1, (n, 3))
    # for the first 200 particles, two companions at nearly equal distance
    ncase = 200
    d = 1e-3
    u = rng.normal(size=(ncase, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    w = np.cross(u, rng.normal(size=(ncase, 3)))
    w /= np.linalg.norm(w, axis=1)[:, None]
    eps = rng.choice([-1, 1], ncase) * rng.uniform(1e-10, 1e-8, ncase)
    x[n - 2 * ncase: n - ncase] = x[:ncase] + d * u
    x[n - ncase:] = x[:ncase] + d * (1 + eps)[:, None] * w
    m = np.full(n, 1.0 / n)
    v = rng.normal(0, 0.3, (n, 3))
    g6.load_particles(m, x, v)
    sel = np.arange(ncase)
    out = g6.force(0.0, 1e-6, n, x[sel], v[sel], self_slot=sel)
    ref = oracle.force(m, x, v, 1e-6, x[sel], v[sel])
    assert check_nn(out["nn"], ref["nn"], x, x[sel], "near-ties") == 0
    assert np.array_equal(out["nn"], ref["nn"])


def test_refine_ill_conditioned(g6):
    """A particle near the centre of a shell of opposite pairs, one of them
    displaced by 2%: the pulls cancel to ~1e-5 of their sum (condition number
    ~1e5), so FP32 pair terms alone miss 1e-6 by orders of magnitude; the
    FP64 redo must recover it."""
    g6.set_precision(ag.SPLIT)
    rng = np.random.RandomState(22)
    nshell = 4000
    u = rng.normal(size=(nshell // 2, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    shell = np.concatenate([u, -u]) * 0.5
    shell[0] *= 1.02  # break the symmetry a little
    centre = np.array([[1e-7, -2e-7, 3e-7]])
    x = np.concatenate([centre, shell])
    n = len(x)
    m = np.full(n, 1.0 / n)
    v = rng.normal(0, 0.1, (n, 3))
    g6.load_particles(m, x, v)
    sel = np.arange(16)
    ref = oracle.force(m, x, v, 1e-6, x[sel], v[sel])
    try:
        g6.set_refine(0.0)
        plain = g6.force(0.0, 1e-6, n, x[sel], v[sel], self_slot=sel)
        g6.set_refine(48.0)
        out = g6.force(0.0, 1e-6, n, x[sel], v[sel], self_slot=sel)
        st = g6.refine_stats()
    finally:
        g6.set_refine(48.0)
    e_plain = vrel(plain["acc"][:1], ref["acc"][:1])[0]
    e = vrel(out["acc"], ref["acc"])
    print(f"centre particle: acc rel err {e_plain:.2e} without, {e[0]:.2e} with the FP64 redo "
          f"({st})")
    assert e_plain > 1e-5  # the case does exercise the pass
    assert st["kappa"] >= 1
    assert e.max() <= 1e-6
    assert np.max(np.abs(out["pot"] - ref["pot"]) / np.abs(ref["pot"])) <= 1e-6


def test_refine_dominant_term(g6):
    """i-particles between a cluster's centre and a massive star that pulls
    against the cluster: one term is ~4 |a| while the condition number stays
    below its limit, so the dominant-term pass (FP32 terms, compensated sums,
    the large terms in FP64) must take them to acc <= 1e-6."""
    g6.set_precision(ag.SPLIT)
    rng = np.random.RandomState(23)
    nc = 4000
    r = rng.uniform(0, 1, nc) ** (1 / 3)
    u = rng.normal(size=(nc, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    cluster = r[:, None] * u
    star = np.array([[0.3, 0.0, 0.0]])
    d, ni = 0.05, 256
    th = rng.uniform(0, 0.35, ni)
    ph = rng.uniform(0, 2 * np.pi, ni)
    dirs = np.stack([np.cos(th), np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph)], 1)
    xi = star - d * dirs
    x = np.concatenate([xi, star, cluster])
    n = len(x)
    m = np.concatenate([np.full(ni, 1e-12), [1e-3], np.full(nc, 1.0 / nc)])
    v = rng.normal(0, 0.1, (n, 3))
    g6.load_particles(m, x, v)
    sel = np.arange(ni)
    ref = oracle.force(m, x, v, 1e-6, x[sel], v[sel])
    try:
        g6.set_refine(0.0)
        plain = g6.force(0.0, 1e-6, n, x[sel], v[sel], self_slot=sel)
        g6.set_refine(48.0)
        out = g6.force(0.0, 1e-6, n, x[sel], v[sel], self_slot=sel)
        st = g6.refine_stats()
    finally:
        g6.set_refine(48.0)
    e_plain = vrel(plain["acc"], ref["acc"])
    e = vrel(out["acc"], ref["acc"])
    print(f"acc rel err: max {e_plain.max():.2e} without, {e.max():.2e} with the refinement ({st})")
    assert st["dominant"] >= ni // 2 and st["overflow"] == 0, st
    assert e.max() <= 1e-6
    assert np.max(np.abs(out["pot"] - ref["pot"]) / np.abs(ref["pot"])) <= 1e-6


def _slot_force(g6, torch, n, sel, want_nn):
    il = torch.tensor(np.asarray(sel, np.int32), device="cuda")
    ni = len(sel)
    acc = torch.empty((ni, 3), dtype=torch.float64, device="cuda")
    jerk = torch.empty_like(acc)
    pot = torch.empty(ni, dtype=torch.float64, device="cuda")
    nn = torch.empty(ni, dtype=torch.int32, device="cuda") if want_nn else None
    g6.force_slots(0.0, 1e-6, n, il.data_ptr(), ni, acc.data_ptr(), jerk.data_ptr(),
                   pot.data_ptr(), nn.data_ptr() if want_nn else None)
    return dict(acc=acc.cpu().numpy(), jerk=jerk.cpu().numpy(), pot=pot.cpu().numpy(),
                nn=nn.cpu().numpy() if want_nn else None)


@pytest.mark.parametrize("want_nn", [False, True])
def test_refine_dominant_term_slots(g6, want_nn):
    """The dominant-term case through g6x_force_slots (the block-step path),
    with the nearest neighbour off (the pass's vectorised loop over record
    pairs) and on (the general loop, which also ranks the neighbour)."""
    torch = pytest.importorskip("torch")
    g6.set_precision(ag.SPLIT)
    rng = np.random.RandomState(29)
    nc = 6000
    r = rng.uniform(0, 1, nc) ** (1 / 3)
    u = rng.normal(size=(nc, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    star = np.array([[0.3, 0.0, 0.0]])
    ni = 200
    th = rng.uniform(0, 0.35, ni)
    ph = rng.uniform(0, 2 * np.pi, ni)
    dirs = np.stack([np.cos(th), np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph)], 1)
    x = np.concatenate([star - 0.05 * dirs, star, r[:, None] * u])
    n = len(x)
    m = np.concatenate([np.full(ni, 1e-12), [1e-3], np.full(nc, 1.0 / nc)])
    v = rng.normal(0, 0.1, (n, 3))
    g6.load_particles(m, x, v)
    sel = np.arange(ni)
    ref = oracle.force(m, x, v, 1e-6, x[sel], v[sel])
    out = _slot_force(g6, torch, n, sel, want_nn)
    st = g6.refine_stats()
    e = vrel(out["acc"], ref["acc"])
    print(f"nn={want_nn}: acc rel err max {e.max():.2e} ({st})")
    assert st["dominant"] >= ni // 2 and st["overflow"] == 0, st
    assert e.max() <= 1e-6
    assert np.max(np.abs(out["pot"] - ref["pot"]) / np.abs(ref["pot"])) <= 1e-6
    if want_nn:
        assert check_nn(out["nn"], ref["nn"], x, x[sel], "dominant") == 0


def test_results_do_not_depend_on_the_launch_shape(g6):
    """g6x_set_shape: the same block under forced shapes (j-lanes, j-splits)
    gives the same nearest neighbours and forces within the contract."""
    torch = pytest.importorskip("torch")
    g6.set_precision(ag.SPLIT)
    np.random.seed(31)
    n = 20000
    m, x, v = ic.plummer(n, do_scale=False)
    g6.load_particles(m, x, v)
    sel = np.arange(0, n, 7)[:2048]
    ref = oracle.force(m, x, v, 1e-6, x[sel], v[sel])
    outs = []
    try:
        for jl, ns in [(0, 0), (1, 1), (1, 13), (4, 5), (32, 40)]:
            g6.set_shape(jl, ns)
            out = _slot_force(g6, torch, n, sel, True)
            st = g6.stats()
            # the split count is normalised to whole tiles per split
            assert jl == 0 or (st["jl"] == jl and abs(st["nsplit"] - ns) <= 2), (jl, ns, st)
            assert vrel(out["acc"], ref["acc"]).max() <= 1e-6, (jl, ns)
            assert check_nn(out["nn"], ref["nn"], x, x[sel], f"shape {jl}x{ns}") == 0
            outs.append(out)
    finally:
        g6.set_shape(0, 0)
    for o in outs[1:]:
        assert np.array_equal(o["nn"], outs[0]["nn"])
