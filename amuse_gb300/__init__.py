"""amuse_gb300 -- GB300-native GRAPE-6 Hermite library for AMUSE's ph4/phiGRAPE path.

The product is ``lib/libsapporo.so`` (C host + sm_103a CUDA kernels) with the
C ABI declared in ``include/g6.h``.  This module loads it with ctypes and
mirrors its interface for Python callers and tests:

* :class:`G6`      -- the GRAPE-6 calls (g6_open, g6_set_ti,
  g6_set_j_particle, g6calc_firsthalf/lasthalf(2), neighbour lists) with the
  reference's argument meaning (lib/sapporo_light/g6lib.h:5-51);
* :class:`G6X`     -- the extension API (device-resident state, the FP64
  corrector / block-step driver with ph4's encounter check, k nearest
  neighbours, batched few-body systems, the fixed-step path, precision
  selection, statistics);
* :func:`driver`   -- ``libg6drive.so``, the C caller that chunks a force
  call by npipes the way ph4's gpu.cc does.

There is no CPU fallback: if the shared library is missing, or no CUDA
device is present, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libsapporo.so")
DRV_PATH = os.path.join(LIB_DIR, "libg6drive.so")

G6_OK = 0
G6_ERR = {
    -1: "not open", -2: "bad argument", -3: "CUDA error", -4: "out of memory",
    -5: "no such device", -6: "kernel error word set", -7: "call out of order",
}
SPLIT, FP64 = 0, 1
JERK_HERMITE, JERK_SOFTENED = 0, 1
NGB_MAX = 256

# Every symbol include/g6.h declares.
ABI_SYMBOLS = [
    "g6_open_", "g6_close_", "g6_npipes_", "g6_set_tunit_", "g6_set_xunit_", "g6_set_ti_",
    "g6_set_j_particle_", "g6calc_firsthalf_", "g6calc_lasthalf_", "g6calc_lasthalf2_",
    "g6_initialize_jp_buffer_", "g6_flush_jp_buffer_", "g6_reset_", "g6_reset_fofpga_",
    "g6_read_neighbour_list_", "g6_get_neighbour_list_",
]
BYVALUE_SYMBOLS = [s[:-1] for s in ABI_SYMBOLS]
EXT_SYMBOLS = [
    "g6x_set_precision", "g6x_get_precision", "g6x_set_refine", "g6x_refine_stats",
    "g6x_test_wait_expiry", "g6x_batch_unperturbed", "g6x_batch_binaries", "g6x_set_npipes", "g6x_last_error", "g6x_load",
    "g6x_read", "g6x_force", "g6x_force_dev", "g6x_force_dev_noalloc", "g6x_force_slots", "g6x_run_init", "g6x_run",
    "g6x_energy", "g6x_run_stats", "g6x_step_all", "g6x_correct", "g6x_batch_run", "g6x_batch_config",
    "g6x_batch_tune", "g6x_system_time", "g6x_timing", "g6x_stats", "g6x_stats_n", "g6x_set_shape", "g6x_check_structure",
    "g6x_check_structure_batch",
    "g6x_stream",
    "g6x_set_fixed_jerk", "g6x_fixed_force", "g6x_fixed_step", "g6x_force_vjp",
    "g6x_fixed_step_adjoint", "g6x_fixed_run", "g6x_fixed_adjoint_run",
    "g6x_set_encounters", "g6x_set_radius", "g6x_encounter", "g6x_knn",
]

# Encounter-check modes of g6x_set_encounters (bits).
ENC_CHECK, ENC_STOP_COLLISION, ENC_STOP_CLOSE = 1, 2, 4

_lib = None
_drv = None

_pi = ctypes.POINTER(ctypes.c_int)
_pd = ctypes.POINTER(ctypes.c_double)
_pf = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p


class G6Error(RuntimeError):
    pass


def _ptr(a, ct):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ct))


def load():
    """Load libsapporo.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise G6Error(f"{LIB_PATH} is missing: run amuse_gb300.build.build() (needs nvcc)")
    lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    I, D = ctypes.c_int, ctypes.c_double
    lib.g6_open_.argtypes = [_pi]
    lib.g6_close_.argtypes = [_pi]
    lib.g6_npipes_.argtypes = []
    lib.g6_set_ti_.argtypes = [_pi, _pd]
    lib.g6_set_j_particle_.argtypes = [_pi, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    lib.g6calc_firsthalf_.argtypes = [_pi, _pi, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    lib.g6calc_firsthalf_.restype = None
    lib.g6calc_lasthalf_.argtypes = [_pi, _pi, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    lib.g6calc_lasthalf2_.argtypes = [_pi, _pi, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd, _pi]
    lib.g6_read_neighbour_list_.argtypes = [_pi]
    lib.g6_get_neighbour_list_.argtypes = [_pi, _pi, _pi, _pi, _pi]
    lib.g6x_set_precision.argtypes = [I]
    lib.g6x_set_refine.argtypes = [D]
    lib.g6x_refine_stats.argtypes = [_pi]
    lib.g6x_test_wait_expiry.argtypes = [I]
    lib.g6x_set_npipes.argtypes = [I]
    lib.g6x_last_error.restype = ctypes.c_char_p
    lib.g6x_load.argtypes = [I, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    lib.g6x_read.argtypes = [I, _pd, _pd, _pd, _pd, _pd, _pd, _pd, _pi]
    lib.g6x_force.argtypes = [D, D, I, I, _pd, _pd, _pi, _pd, _pd, _pd, _pi, _pf]
    lib.g6x_force_dev.argtypes = [D, D, I, I, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, I]
    lib.g6x_force_slots.argtypes = [D, D, I, I, _vp, _vp, _vp, _vp, _vp, I]
    lib.g6x_force_dev_noalloc.argtypes = [D, D, I, I, _vp, _vp, _vp, _vp, _vp, _vp, _vp, I]
    lib.g6x_run_init.argtypes = [D, D]
    lib.g6x_run.argtypes = [D, ctypes.POINTER(ctypes.c_longlong), _pd]
    lib.g6x_energy.argtypes = [_pd, _pd]
    lib.g6x_run_stats.argtypes = [_pd]
    lib.g6x_set_encounters.argtypes = [I, D]
    lib.g6x_set_radius.argtypes = [I, _pd]
    lib.g6x_encounter.argtypes = [_pi, _pd]
    lib.g6x_knn.argtypes = [I, I, D, I, _pi, _pi, _pd]
    lib.g6x_step_all.argtypes = [D]
    lib.g6x_correct.argtypes = [I, _pi, D, D, _pd, _pd]
    _pll = ctypes.POINTER(ctypes.c_longlong)
    lib.g6x_batch_run.argtypes = [I, _pi, _pd, _pd, _pd, _pd, D, I, ctypes.c_longlong, I, _pd,
                                  _pll, _pd, _pi, _pd]
    lib.g6x_batch_config.argtypes = [I, I]
    lib.g6x_batch_unperturbed.argtypes = [I, D, D, D, I]
    lib.g6x_batch_binaries.argtypes = [I, _pi]
    lib.g6x_batch_tune.argtypes = [I, _pi, _pd, _pd, _pd, _pd, D, I, I, D, _pd]
    lib.g6x_system_time.restype = D
    lib.g6x_timing.argtypes = [I]
    lib.g6x_stats.argtypes = [_pd]
    lib.g6x_stats_n.argtypes = [_pd, ctypes.c_int]
    lib.g6x_set_shape.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.g6x_check_structure.argtypes = [ctypes.c_int, _pd, _pd, _pd, _pi, ctypes.c_char_p,
                                        ctypes.c_int]
    lib.g6x_check_structure_batch.argtypes = [ctypes.c_int, _pi, _pd, _pd, _pd, _pi, _pi, _pi,
                                              ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    lib.g6x_stream.restype = _vp
    lib.g6x_set_fixed_jerk.argtypes = [I]
    lib.g6x_fixed_force.argtypes = [I, D] + [_vp] * 5
    lib.g6x_fixed_step.argtypes = [I, D, D] + [_vp] * 7
    lib.g6x_force_vjp.argtypes = [I, D] + [_vp] * 8
    lib.g6x_fixed_step_adjoint.argtypes = [I, D, D] + [_vp] * 9
    lib.g6x_fixed_run.argtypes = [I, D, D, I] + [_vp] * 7
    lib.g6x_fixed_adjoint_run.argtypes = [I, D, D, I] + [_vp] * 9
    _lib = lib
    return lib


def driver():
    """Load libg6drive.so (the ph4-style C caller of the ABI)."""
    global _drv
    if _drv is not None:
        return _drv
    load()
    if not os.path.exists(DRV_PATH):
        raise G6Error(f"{DRV_PATH} is missing: run amuse_gb300.build.build()")
    d = ctypes.CDLL(DRV_PATH)
    I, D = ctypes.c_int, ctypes.c_double
    d.drv_load.argtypes = [I, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    d.drv_update.argtypes = [I, _pi, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pd]
    d.drv_force.argtypes = [I, D, D, I, _pi, _pd, _pd, _pd, _pd, _pd, _pd, _pi, I]
    _drv = d
    return d


def _check(rc, what):
    if rc < 0:
        msg = load().g6x_last_error().decode(errors="replace")
        raise G6Error(f"{what}: {G6_ERR.get(rc, rc)} ({msg})")
    return rc


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


BATCH_MODES = {"fast": 0, "exact": 1, "split": 2}


def _batch_mode(mode, exact):
    if mode is None:
        return BATCH_MODES["exact" if exact else "fast"]
    return BATCH_MODES[mode]


class G6:
    """The GRAPE-6 API of the library (one context per process)."""

    def __init__(self, device=0):
        self.lib = load()
        self.cid = ctypes.c_int(device)
        _check(self.lib.g6_open_(ctypes.byref(self.cid)), "g6_open")

    def close(self):
        self.lib.g6_close_(ctypes.byref(self.cid))

    def npipes(self):
        return self.lib.g6_npipes_()

    def set_ti(self, ti):
        _check(self.lib.g6_set_ti_(ctypes.byref(self.cid), ctypes.byref(ctypes.c_double(ti))),
               "g6_set_ti")

    def set_j_particle(self, address, index, tj, dtj, mass, k18, j6, a2, v, x):
        c = [_f64(a, (3,)) for a in (k18, j6, a2, v, x)]
        _check(self.lib.g6_set_j_particle_(
            ctypes.byref(self.cid), ctypes.byref(ctypes.c_int(address)),
            ctypes.byref(ctypes.c_int(index)), ctypes.byref(ctypes.c_double(tj)),
            ctypes.byref(ctypes.c_double(dtj)), ctypes.byref(ctypes.c_double(mass)),
            *[_ptr(a, ctypes.c_double) for a in c]), "g6_set_j_particle")

    def calc(self, nj, index, xi, vi, eps2, h2=None, want_nn=True):
        """firsthalf + lasthalf(2): returns acc, jerk, pot (, nn ids)."""
        index = _i32(index)
        ni = len(index)
        xi, vi = _f64(xi, (ni, 3)), _f64(vi, (ni, 3))
        h2 = _f64(np.full(ni, eps2) if h2 is None else h2)
        zero3 = np.zeros((max(ni, 1), 3))
        phi = np.zeros(max(ni, 1))
        acc = np.zeros((ni, 3)); jerk = np.zeros((ni, 3)); pot = np.zeros(ni)
        nn = np.zeros(ni, np.int32)
        cnj, cni, ce = ctypes.c_int(nj), ctypes.c_int(ni), ctypes.c_double(eps2)
        P = lambda a: _ptr(a, ctypes.c_double)
        self.lib.g6calc_firsthalf_(ctypes.byref(self.cid), ctypes.byref(cnj), ctypes.byref(cni),
                                   _ptr(index, ctypes.c_int), P(xi), P(vi), P(zero3), P(zero3),
                                   P(phi), ctypes.byref(ce), P(h2))
        if want_nn:
            rc = self.lib.g6calc_lasthalf2_(ctypes.byref(self.cid), ctypes.byref(cnj),
                                            ctypes.byref(cni), _ptr(index, ctypes.c_int), P(xi),
                                            P(vi), ctypes.byref(ce), P(h2), P(acc), P(jerk),
                                            P(pot), _ptr(nn, ctypes.c_int))
            _check(rc, "g6calc_lasthalf2")
            return acc, jerk, pot, nn
        rc = self.lib.g6calc_lasthalf_(ctypes.byref(self.cid), ctypes.byref(cnj),
                                       ctypes.byref(cni), _ptr(index, ctypes.c_int), P(xi), P(vi),
                                       ctypes.byref(ce), P(h2), P(acc), P(jerk), P(pot))
        _check(rc, "g6calc_lasthalf")
        return acc, jerk, pot

    def read_neighbour_list(self):
        return _check(self.lib.g6_read_neighbour_list_(ctypes.byref(self.cid)),
                      "g6_read_neighbour_list")

    def get_neighbour_list(self, ipipe, maxlength=NGB_MAX):
        out = np.zeros(maxlength, np.int32)
        n = ctypes.c_int(0)
        rc = _check(self.lib.g6_get_neighbour_list_(
            ctypes.byref(self.cid), ctypes.byref(ctypes.c_int(ipipe)),
            ctypes.byref(ctypes.c_int(maxlength)), ctypes.byref(n), _ptr(out, ctypes.c_int)),
            "g6_get_neighbour_list")
        return out[: n.value].copy(), rc


class G6X(G6):
    """Extension API (device-resident state and driver)."""

    def set_precision(self, prec):
        _check(self.lib.g6x_set_precision(prec), "g6x_set_precision")

    def get_precision(self):
        return self.lib.g6x_get_precision()

    def set_refine(self, kappa):
        """Condition-number limit of the split refinement pass (0: no FP64 redo)."""
        _check(self.lib.g6x_set_refine(float(kappa)), "g6x_set_refine")

    def refine_stats(self):
        """Last call's refinement queue: queued, queued for kappa, overflow,
        queued for a dominant term."""
        out = np.zeros(4, np.int32)
        _check(self.lib.g6x_refine_stats(_ptr(out, ctypes.c_int)), "g6x_refine_stats")
        return dict(queued=int(out[0]), kappa=int(out[1]), overflow=int(out[2]),
                    dominant=int(out[3]))

    def test_wait_expiry(self, on=True):
        """Test hook: the next force call's bounded wait expires (20 ms)."""
        _check(self.lib.g6x_test_wait_expiry(1 if on else 0), "g6x_test_wait_expiry")

    def set_npipes(self, n):
        _check(self.lib.g6x_set_npipes(n), "g6x_set_npipes")

    def load_particles(self, mass, pos, vel, acc=None, jerk=None, t=None, dt=None, ids=None):
        n = len(mass)
        ids = _i32(np.arange(1, n + 1) if ids is None else ids)
        arrs = [_f64(mass), _f64(pos, (n, 3)), _f64(vel, (n, 3)),
                None if acc is None else _f64(acc, (n, 3)),
                None if jerk is None else _f64(jerk, (n, 3)),
                None if t is None else _f64(t), None if dt is None else _f64(dt)]
        _check(self.lib.g6x_load(n, _ptr(ids, ctypes.c_int),
                                 *[_ptr(a, ctypes.c_double) for a in arrs]), "g6x_load")

    def read_particles(self, n):
        x = np.zeros((n, 3)); v = np.zeros((n, 3)); a = np.zeros((n, 3)); j = np.zeros((n, 3))
        pot = np.zeros(n); t = np.zeros(n); dt = np.zeros(n); nn = np.zeros(n, np.int32)
        _check(self.lib.g6x_read(n, *[_ptr(q, ctypes.c_double) for q in (x, v, a, j, pot, t, dt)],
                                 _ptr(nn, ctypes.c_int)), "g6x_read")
        return dict(pos=x, vel=v, acc=a, jerk=j, pot=pot, time=t, timestep=dt, nn=nn)

    def force(self, ti, eps2, nj, xi, vi, self_slot=None):
        """Blocking force on explicit i (any ni): acc, jerk, pot, nn slot, nn r2."""
        xi = _f64(xi).reshape(-1, 3)
        ni = len(xi)
        vi = _f64(vi, (ni, 3))
        ss = None if self_slot is None else _i32(self_slot)
        acc = np.zeros((ni, 3)); jerk = np.zeros((ni, 3)); pot = np.zeros(ni)
        nn = np.zeros(ni, np.int32); r2 = np.zeros(ni, np.float32)
        _check(self.lib.g6x_force(ti, eps2, nj, ni, _ptr(xi, ctypes.c_double),
                                  _ptr(vi, ctypes.c_double), _ptr(ss, ctypes.c_int),
                                  _ptr(acc, ctypes.c_double), _ptr(jerk, ctypes.c_double),
                                  _ptr(pot, ctypes.c_double), _ptr(nn, ctypes.c_int),
                                  _ptr(r2, ctypes.c_float)), "g6x_force")
        return dict(acc=acc, jerk=jerk, pot=pot, nn=nn, nn_r2=r2)

    def force_slots(self, ti, eps2, nj, d_ilist, ni, d_acc, d_jerk, d_pot, d_nn, sync=True):
        _check(self.lib.g6x_force_slots(ti, eps2, nj, ni, d_ilist, d_acc, d_jerk, d_pot, d_nn,
                                        1 if sync else 0), "g6x_force_slots")

    def force_dev(self, ti, eps2, nj, ni, d_xi, d_vi, d_self, d_acc, d_jerk, d_pot, d_nn,
                  d_nnr2=None, sync=True):
        _check(self.lib.g6x_force_dev(ti, eps2, nj, ni, d_xi, d_vi, d_self, d_acc, d_jerk, d_pot,
                                      d_nn, d_nnr2, 1 if sync else 0), "g6x_force_dev")

    def force_dev_noalloc(self, ti, eps2, nj, ni, d_xi, d_vi, d_self, d_acc, d_jerk, d_pot,
                          d_nn=None, sync=True):
        """g6x_force_dev without any device allocation (fixed 16 MiB scratch)."""
        _check(self.lib.g6x_force_dev_noalloc(ti, eps2, nj, ni, d_xi, d_vi, d_self, d_acc,
                                              d_jerk, d_pot, d_nn, 1 if sync else 0),
               "g6x_force_dev_noalloc")

    # ---- fixed-step Hermite and its adjoint (device pointers, [n][3]) ----
    def set_fixed_jerk(self, form):
        """JERK_HERMITE (the hermite code's form) or JERK_SOFTENED."""
        _check(self.lib.g6x_set_fixed_jerk(form), "g6x_set_fixed_jerk")

    def fixed_force(self, n, eps2, d_x, d_v, d_m, d_a, d_j):
        _check(self.lib.g6x_fixed_force(n, eps2, d_x, d_v, d_m, d_a, d_j), "g6x_fixed_force")

    def fixed_step(self, n, h, eps2, d_x, d_v, d_a, d_j, d_m, d_xp, d_vp):
        _check(self.lib.g6x_fixed_step(n, h, eps2, d_x, d_v, d_a, d_j, d_m, d_xp, d_vp),
               "g6x_fixed_step")

    def force_vjp(self, n, eps2, d_x, d_v, d_m, d_la, d_lj, d_gx, d_gv, d_gm):
        _check(self.lib.g6x_force_vjp(n, eps2, d_x, d_v, d_m, d_la, d_lj, d_gx, d_gv, d_gm),
               "g6x_force_vjp")

    def fixed_step_adjoint(self, n, h, eps2, d_xp, d_vp, d_m, d_lx, d_lv, d_la, d_lj, d_lm,
                           d_work):
        _check(self.lib.g6x_fixed_step_adjoint(n, h, eps2, d_xp, d_vp, d_m, d_lx, d_lv, d_la,
                                               d_lj, d_lm, d_work), "g6x_fixed_step_adjoint")

    def fixed_run(self, n, h, eps2, nsteps, d_x, d_v, d_a, d_j, d_m, d_xp_all=None,
                  d_vp_all=None):
        _check(self.lib.g6x_fixed_run(n, h, eps2, nsteps, d_x, d_v, d_a, d_j, d_m, d_xp_all,
                                      d_vp_all), "g6x_fixed_run")

    def fixed_adjoint_run(self, n, h, eps2, nsteps, d_xp_all, d_vp_all, d_m, d_lx, d_lv, d_la,
                          d_lj, d_lm, d_work):
        _check(self.lib.g6x_fixed_adjoint_run(n, h, eps2, nsteps, d_xp_all, d_vp_all, d_m, d_lx,
                                              d_lv, d_la, d_lj, d_lm, d_work),
               "g6x_fixed_adjoint_run")

    def run_init(self, eps2, eta):
        _check(self.lib.g6x_run_init(eps2, eta), "g6x_run_init")

    def run(self, t_end, max_blocks=0):
        """Block steps to t_end (or max_blocks of them); -> (blocks, particle steps)."""
        nb = ctypes.c_longlong(max_blocks)
        ns = ctypes.c_double(0)
        _check(self.lib.g6x_run(t_end, ctypes.byref(nb), ctypes.byref(ns)), "g6x_run")
        return nb.value, ns.value

    def run_stats(self):
        """Host-side account of the last run(): blocks, wall_ms, sync_ms, steps."""
        out = np.zeros(4)
        _check(self.lib.g6x_run_stats(_ptr(out, ctypes.c_double)), "g6x_run_stats")
        return dict(blocks=out[0], wall_ms=out[1], sync_ms=out[2], particle_steps=out[3])

    def set_encounters(self, mode, rmin=0.0):
        """Encounter check in run(): ENC_CHECK, ENC_STOP_COLLISION and
        ENC_STOP_CLOSE bits (0 turns it off); rmin <= 0 is ph4's 2/n."""
        _check(self.lib.g6x_set_encounters(int(mode), float(rmin)), "g6x_set_encounters")

    def set_radius(self, radius):
        """Particle radii by slot (the collision criterion's R)."""
        radius = _f64(radius)
        _check(self.lib.g6x_set_radius(len(radius), _ptr(radius, ctypes.c_double)),
               "g6x_set_radius")

    def encounter(self):
        """The last checked block: close / coll (id pairs or None), stopped
        (1 collision, 2 close, 0 none), t, rmax_close, rmax_coll."""
        ids = np.zeros(4, np.int32)
        out = np.zeros(4)
        _check(self.lib.g6x_encounter(_ptr(ids, ctypes.c_int), _ptr(out, ctypes.c_double)),
               "g6x_encounter")
        pair = lambda a, b: None if a < 0 else (int(a), int(b))
        return dict(close=pair(ids[0], ids[1]), coll=pair(ids[2], ids[3]), stopped=int(out[0]),
                    t=float(out[1]), rmax_close=float(out[2]), rmax_coll=float(out[3]))

    def knn(self, nj, k=12, slots=None, t=0.0):
        """The k nearest neighbours of the listed slots (all nj by default)
        among slots [0, nj) at time t: (ids [ni, k] int32, -1 where fewer
        than k others exist; d2 [ni, k] squared distances, sorted)."""
        slots = _i32(np.arange(nj) if slots is None else slots)
        ni = len(slots)
        ids = np.empty((ni, k), np.int32)
        d2 = np.empty((ni, k))
        _check(self.lib.g6x_knn(int(k), int(nj), float(t), ni, _ptr(slots, ctypes.c_int),
                                _ptr(ids, ctypes.c_int), _ptr(d2, ctypes.c_double)), "g6x_knn")
        return ids, d2

    def correct(self, slots, tnext, eta, acc, jerk):
        slots = _i32(slots)
        n = len(slots)
        acc, jerk = _f64(acc, (n, 3)), _f64(jerk, (n, 3))
        _check(self.lib.g6x_correct(n, _ptr(slots, ctypes.c_int), tnext, eta,
                                    _ptr(acc, ctypes.c_double), _ptr(jerk, ctypes.c_double)),
               "g6x_correct")

    def batch_run(self, n_per_sys, t_end, mass, pos, vel, eta=0.14, n_iter=2, max_steps=0,
                  exact=False, mode=None):
        """Integrate many few-body systems (smallN's scheme); returns a dict
        with pos, vel (updated copies), t_final, steps, wall_ms, status, elapsed_ms.
        mode: "fast" (default), "exact" (bit-identical to smallN; also
        exact=True) or "split" (FP32 pair terms from double-single positions)."""
        n_per_sys = _i32(n_per_sys)
        nsys = len(n_per_sys)
        t_end = _f64(np.broadcast_to(np.asarray(t_end, dtype=np.float64), (nsys,)))
        nb = int(n_per_sys.sum())
        mass = _f64(mass)
        pos = _f64(pos, (nb, 3)).copy()
        vel = _f64(vel, (nb, 3)).copy()
        tf = np.zeros(nsys); st = np.zeros(nsys, np.int64); wall = np.zeros(nsys)
        status = np.zeros(nsys, np.int32); el = ctypes.c_double(0)
        P = lambda a: _ptr(a, ctypes.c_double)
        _check(self.lib.g6x_batch_run(nsys, _ptr(n_per_sys, ctypes.c_int), P(t_end), P(mass),
                                      P(pos), P(vel), eta, n_iter, int(max_steps),
                                      _batch_mode(mode, exact), P(tf),
                                      st.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                      P(wall), _ptr(status, ctypes.c_int), ctypes.byref(el)),
               "g6x_batch_run")
        return dict(pos=pos, vel=vel, t_final=tf, steps=st, wall_ms=wall, status=status,
                    elapsed_ms=el.value)

    def batch_config(self, warps_per_cta, ctas_per_sm):
        _check(self.lib.g6x_batch_config(warps_per_cta, ctas_per_sm), "g6x_batch_config")

    def batch_unperturbed(self, on=True, dt_crit=1e-3, r2_crit=1e-2, gamma=1e-6,
                          allow_full=True):
        """smallN's unperturbed binaries in the fast and split batch modes
        (defaults: the smallN worker's)."""
        _check(self.lib.g6x_batch_unperturbed(1 if on else 0, dt_crit, r2_crit, gamma,
                                              1 if allow_full else 0), "g6x_batch_unperturbed")

    def batch_binaries(self, nsys):
        """Binaries made per system in the last batch run."""
        out = np.zeros(nsys, np.int32)
        _check(self.lib.g6x_batch_binaries(nsys, _ptr(out, ctypes.c_int)), "g6x_batch_binaries")
        return out

    def batch_tune(self, n_per_sys, t_end, mass, pos, vel, eta=0.14, n_iter=2, exact=False,
                   frac=0.1, mode=None):
        n_per_sys = _i32(n_per_sys)
        nsys = len(n_per_sys)
        t_end = _f64(np.broadcast_to(np.asarray(t_end, dtype=np.float64), (nsys,)))
        out = np.zeros(3)
        P = lambda a: _ptr(a, ctypes.c_double)
        _check(self.lib.g6x_batch_tune(nsys, _ptr(n_per_sys, ctypes.c_int), P(t_end),
                                       P(_f64(mass)), P(_f64(pos)), P(_f64(vel)), eta, n_iter,
                                       _batch_mode(mode, exact), frac, P(out)),
               "g6x_batch_tune")
        return dict(warps_per_cta=int(out[0]), ctas_per_sm=int(out[1]), ms=out[2])

    def step_all(self, tnext):
        _check(self.lib.g6x_step_all(tnext), "g6x_step_all")

    def energy(self):
        k = ctypes.c_double(0)
        p = ctypes.c_double(0)
        _check(self.lib.g6x_energy(ctypes.byref(k), ctypes.byref(p)), "g6x_energy")
        return k.value, p.value

    def system_time(self):
        return self.lib.g6x_system_time()

    def timing(self, on=True):
        self.lib.g6x_timing(1 if on else 0)

    def stats(self):
        out = np.zeros(10)
        self.lib.g6x_stats_n(_ptr(out, ctypes.c_double), 10)
        keys = ["predict_ms", "force_ms", "pairs", "jl", "nsplit", "grid_x", "predict_bytes", "nj",
                "kernel_ms", "refine_ms"]
        return dict(zip(keys, out.tolist()))

    def stream(self):
        return self.lib.g6x_stream()

    def set_shape(self, jl=0, nsplit=0):
        """Launch shape override (0: the cost model's choice)."""
        _check(self.lib.g6x_set_shape(int(jl), int(nsplit)), "g6x_set_shape")


def check_structure(mass, pos, vel):
    """Structure of one few-body system (g6x_check_structure, host code):
    returns dict(over, hierarchy_tested, escaping, top_of, summary).  over:
    every top-level node escaping and stable (smallN's check_structure);
    hierarchy_tested: a multiple above a binary was judged by the published
    Mardling-Aarseth criterion where smallN uses Mardling's nstab; escaping:
    every top-level node escaping, stable or not; top_of:
    per body, the smallest body index of its top-level node; summary: the
    tree, a binary as "(first,second)" of body indices."""
    lib = load()
    m = _f64(mass)
    n = len(m)
    x, v = _f64(pos, (n, 3)), _f64(vel, (n, 3))
    top = np.zeros(n, np.int32)
    buf = ctypes.create_string_buffer(4096)
    rc = lib.g6x_check_structure(n, _ptr(m, ctypes.c_double), _ptr(x, ctypes.c_double),
                                 _ptr(v, ctypes.c_double), _ptr(top, ctypes.c_int), buf, 4096)
    _check(rc if rc < 0 else 0, "g6x_check_structure")
    return dict(over=bool(rc & 1), hierarchy_tested=bool(rc & 2), escaping=bool(rc & 4),
                top_of=top, summary=buf.value.decode())


def check_structure_batch(n_per_sys, mass, pos, vel, nthreads=0, summary_cap=512):
    """g6x_check_structure over many systems stored back to back, on the
    host's cores (g6x_check_structure_batch; summary_cap 512 holds the
    longest tree of 64 bodies).  Returns dict(over, hierarchy_tested,
    escaping, top_of, top_rank, summary): per-system arrays, per-body arrays
    (top_of: local indices; top_rank: the position of the body's top-level
    node in the tree's order) and a list of summaries."""
    lib = load()
    nper = _i32(n_per_sys)
    ns = len(nper)
    nb = int(nper.sum())
    m = _f64(mass)
    x, v = _f64(pos, (nb, 3)), _f64(vel, (nb, 3))
    if len(m) != nb:
        raise G6Error("g6x_check_structure_batch: mass has the wrong length")
    flags = np.zeros(ns, np.int32)
    top = np.zeros(nb, np.int32)
    rank = np.zeros(nb, np.int32)
    buf = ctypes.create_string_buffer(max(1, ns * summary_cap))
    rc = lib.g6x_check_structure_batch(ns, _ptr(nper, ctypes.c_int), _ptr(m, ctypes.c_double),
                                       _ptr(x, ctypes.c_double), _ptr(v, ctypes.c_double),
                                       _ptr(flags, ctypes.c_int), _ptr(top, ctypes.c_int),
                                       _ptr(rank, ctypes.c_int), buf, summary_cap, int(nthreads))
    _check(rc, "g6x_check_structure_batch")
    raw = buf.raw
    summ = [raw[k * summary_cap:(k + 1) * summary_cap].split(b"\0", 1)[0].decode()
            for k in range(ns)]
    return dict(over=(flags & 1).astype(bool), hierarchy_tested=(flags & 2).astype(bool),
                escaping=(flags & 4).astype(bool), top_of=top, top_rank=rank, summary=summ)


def drive_load(mass, pos, vel, acc=None, jerk=None, t=None, dt=None, ids=None):
    """ph4 jdata::initialize_gpu: one g6_set_j_particle per particle (C loop)."""
    n = len(mass)
    ids = _i32(np.arange(1, n + 1) if ids is None else ids)
    arrs = [None if t is None else _f64(t), None if dt is None else _f64(dt), _f64(mass),
            _f64(pos, (n, 3)), _f64(vel, (n, 3)),
            None if acc is None else _f64(acc, (n, 3)), None if jerk is None else _f64(jerk, (n, 3))]
    _check(driver().drv_load(n, _ptr(ids, ctypes.c_int),
                             *[_ptr(a, ctypes.c_double) for a in arrs]), "drv_load")


def drive_force(nj, ti, eps2, ids, ipos, ivel, want_nn=True, h2=None, out=None):
    """ph4 get_partial_acc_and_jerk_on_gpu: chunked g6calc calls (C loop)."""
    ids = _i32(ids)
    ni = len(ids)
    ipos, ivel = _f64(ipos, (ni, 3)), _f64(ivel, (ni, 3))
    if out is None:
        out = dict(acc=np.zeros((ni, 3)), jerk=np.zeros((ni, 3)), pot=np.zeros(ni),
                   nn=np.zeros(ni, np.int32))
    h2 = None if h2 is None else _f64(h2)
    _check(driver().drv_force(nj, ti, eps2, ni, _ptr(ids, ctypes.c_int),
                              _ptr(ipos, ctypes.c_double), _ptr(ivel, ctypes.c_double),
                              _ptr(h2, ctypes.c_double), _ptr(out["acc"], ctypes.c_double),
                              _ptr(out["jerk"], ctypes.c_double), _ptr(out["pot"], ctypes.c_double),
                              _ptr(out["nn"], ctypes.c_int), 1 if want_nn else 0), "drv_force")
    return out
