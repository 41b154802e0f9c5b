"""Oracle package -- TEST INFRASTRUCTURE ONLY.

ctypes bindings for
  * ``liborc.so``   -- the C restatement of ph4's FP64 CPU path (g6_oracle.c),
  * ``_ref/libph4ref.so`` -- the unmodified ph4 objects built from the
    reference sources (present only where the reference checkout exists).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package, and only as the checker / the timed CPU baseline.
The shipped library never loads either .so.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_PORT = os.path.join(HERE, "liborc.so")
_REF = os.path.join(HERE, "_ref", "libph4ref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_c_int, _c_dbl, _c_long = ctypes.c_int, ctypes.c_double, ctypes.c_long

_port_lib = None
_ref_lib = None


def build_port():
    subprocess.check_call(["make", "-s", "-C", HERE, "port"])


def ref_root():
    """The AMUSE checkout named by the AMUSE_REF environment variable, or None."""
    r = os.environ.get("AMUSE_REF")
    return r if r and os.path.isdir(os.path.join(r, "src", "amuse_ph4", "src")) else None


def build_ref(root=None):
    """Compile the unmodified ph4 CPU objects (needs the reference sources,
    at ``root`` or $AMUSE_REF)."""
    root = root or ref_root()
    if root is None:
        raise RuntimeError("set AMUSE_REF to the AMUSE checkout to build oracle/_ref")
    subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={root}", "-j8"])


def port():
    global _port_lib
    if _port_lib is None:
        if not os.path.exists(_PORT):
            build_port()
        lib = ctypes.CDLL(_PORT)
        lib.orc_force.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_int, _dp, _dp,
                                  _dp, _dp, _dp, _ip, _dp]
        lib.orc_force.restype = None
        lib.orc_force_mt.argtypes = [_c_int, _c_int, _dp, _dp, _dp, _c_dbl, _c_int,
                                     _dp, _dp, _dp, _dp, _dp, _ip, _dp]
        lib.orc_force_mt.restype = _c_int
        lib.orc_predict.argtypes = [_c_int, _c_dbl, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        lib.orc_predict.restype = None
        lib.orc_correct.argtypes = [_c_int, _c_dbl, _c_dbl, _dp, _dp, _dp, _dp, _dp,
                                    _dp, _dp, _dp]
        lib.orc_correct.restype = None
        lib.orc_initial_step.argtypes = [_c_int, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl,
                                         _dp, _dp, _dp]
        lib.orc_initial_step.restype = None
        lib.orc_run.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_dbl, _c_dbl, _c_int,
                                _dp, _dp, _dp, _dp, _dp, _dp, _c_long]
        lib.orc_run.restype = _c_long
        lib.orc_run_enc.argtypes = [_c_int, _dp, _dp, _dp, _dp, _c_dbl, _c_dbl, _c_dbl,
                                    _c_int, _dp, _dp, _dp, _dp, _dp, _dp, _c_long, _c_int,
                                    _c_dbl, _dp]
        lib.orc_run_enc.restype = _c_long
        lib.orc_knn.argtypes = [_c_int, _dp, _c_int, _c_int, _ip, _ip, _dp]
        lib.orc_knn.restype = None
        lib.orc_smalln.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_int, _c_dbl, _dp, _c_long]
        lib.orc_smalln.restype = _c_long
        lib.orc_smalln_unpert.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_int, _c_dbl,
                                          _c_dbl, _c_dbl, _c_dbl, _c_int, _dp, _c_long, _ip]
        lib.orc_smalln_unpert.restype = _c_long
        lib.orc_kepler.argtypes = [_c_dbl, _dp, _dp, _c_dbl, _dp, _dp]
        lib.orc_kepler.restype = None
        lib.orc_hermite_fixed.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_dbl, _c_int, _dp,
                                          _dp]
        lib.orc_hermite_fixed.restype = None
        _port_lib = lib
    return _port_lib


def ref_available():
    return os.path.exists(_REF)


def ref():
    global _ref_lib
    if _ref_lib is None:
        lib = ctypes.CDLL(_REF)
        lib.ph4ref_force.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_int, _dp, _dp,
                                     _dp, _dp, _dp, _ip, _dp]
        lib.ph4ref_correct.argtypes = [_c_int, _c_dbl, _c_dbl, _dp, _dp, _dp, _dp, _dp,
                                       _dp, _dp, _dp]
        lib.ph4ref_run.argtypes = [_c_int, _dp, _ip, _dp, _dp, _c_dbl, _c_dbl, _c_dbl,
                                   _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        lib.ph4ref_smalln.argtypes = [_c_int, _dp, _dp, _dp, _c_dbl, _c_dbl, _c_dbl, _dp]
        lib.ph4ref_check_structure.argtypes = [_c_int, _dp, _dp, _dp, ctypes.c_char_p, _c_int]
        lib.ph4ref_check_structure.restype = _c_int
        lib.ph4ref_run_coll.argtypes = [_c_int, _dp, _dp, _ip, _dp, _dp, _c_dbl, _c_dbl,
                                        _c_dbl, _c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        _ref_lib = lib
    return _ref_lib


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


def force(mass, jpos, jvel, eps2, ipos, ivel, threads=1, lib=None):
    """FP64 ph4 force (idata.cc:147-237) -> dict(acc, jerk, pot, nn, dnn).

    nn is a j index (-1 when no neighbour)."""
    mass, jpos, jvel, ipos, ivel = map(_c, (mass, jpos, jvel, ipos, ivel))
    nj, ni = len(mass), len(ipos)
    acc = np.zeros((ni, 3)); jerk = np.zeros((ni, 3)); pot = np.zeros(ni)
    nn = np.zeros(ni, np.int32); dnn = np.zeros(ni)
    if lib == "ref":
        ref().ph4ref_force(nj, mass, jpos, jvel, eps2, ni, ipos, ivel, acc, jerk, pot, nn, dnn)
    elif threads == 1:
        port().orc_force(nj, mass, jpos, jvel, eps2, ni, ipos, ivel, acc, jerk, pot, nn, dnn)
    else:
        port().orc_force_mt(threads, nj, mass, jpos, jvel, eps2, ni, ipos, ivel, acc, jerk,
                            pot, nn, dnn)
    return dict(acc=acc, jerk=jerk, pot=pot, nn=nn, dnn=dnn)


def predict(t, time, pos, vel, acc, jerk):
    time, pos, vel, acc, jerk = map(_c, (time, pos, vel, acc, jerk))
    pp = np.zeros_like(pos); pv = np.zeros_like(vel)
    port().orc_predict(len(time), t, time, pos, vel, acc, jerk, pp, pv)
    return pp, pv


def correct(tnext, eta, itime, istep, ipos, ivel, old_acc, old_jerk, iacc, ijerk, lib=None):
    """ph4 corrector + Aarseth step (idata.cc:399-514); returns new arrays."""
    itime, istep, ipos, ivel = (_c(a).copy() for a in (itime, istep, ipos, ivel))
    old_acc, old_jerk, iacc, ijerk = map(_c, (old_acc, old_jerk, iacc, ijerk))
    f = ref().ph4ref_correct if lib == "ref" else port().orc_correct
    f(len(itime), tnext, eta, itime, istep, ipos, ivel, old_acc, old_jerk, iacc, ijerk)
    return dict(time=itime, timestep=istep, pos=ipos, vel=ivel)


def initial_step(acc, jerk, eta, system_time=0.0, fac=0.0625, limit=0.03125, limitm=8.0):
    acc, jerk = _c(acc), _c(jerk)
    ts = np.zeros(len(acc))
    port().orc_initial_step(len(acc), system_time, eta, fac, limit, limitm, acc, jerk, ts)
    return ts


def run(mass, pos, vel, eps2, eta, t_end, threads=1, lib=None, ids=None, max_blocks=0):
    """Block-step ph4 run, CPU mode.  Returns final state + E0/E1."""
    mass, pos, vel = _c(mass), _c(pos).copy(), _c(vel).copy()
    n = len(mass)
    acc = np.zeros((n, 3)); jerk = np.zeros((n, 3)); pot = np.zeros(n)
    time = np.zeros(n); step = np.zeros(n)
    if lib == "ref":
        ids = _c(np.arange(1, n + 1) if ids is None else ids, np.int32)
        stats = np.zeros(5)
        pos_o = np.zeros_like(pos); vel_o = np.zeros_like(vel)
        ref().ph4ref_run(n, mass, ids, pos, vel, eps2, eta, t_end, pos_o, vel_o, acc, jerk,
                         pot, time, step, stats)
        return dict(pos=pos_o, vel=vel_o, acc=acc, jerk=jerk, pot=pot, time=time,
                    timestep=step, E0=stats[0], E1=stats[1], total_steps=stats[2],
                    t=stats[3], blocks=stats[4])
    stats = np.zeros(4)
    blocks = port().orc_run(n, mass, pos, vel, eps2, eta, t_end, threads, acc, jerk, pot,
                            time, step, stats, max_blocks)
    return dict(pos=pos, vel=vel, acc=acc, jerk=jerk, pot=pot, time=time, timestep=step,
                E0=stats[0], E1=stats[1], total_steps=stats[2], t=stats[3], blocks=blocks)


def knn(pos, k, slots=None):
    """save_neighbors (gpu.cc:534-558) over all other particles: the k
    nearest (indices, squared distances), ties to the smaller index;
    -1 / inf past the last."""
    pos = _c(pos)
    n = len(pos)
    slots = _c(np.arange(n) if slots is None else slots, np.int32)
    ni = len(slots)
    out_j = np.empty((ni, k), np.int32)
    out_d2 = np.empty((ni, k))
    port().orc_knn(n, pos, k, ni, slots, out_j, out_d2)
    return out_j, out_d2


ENC_CHECK, ENC_STOP_COLL, ENC_STOP_CLOSE = 1, 2, 4


def run_enc(mass, radius, pos, vel, eps2, eta, t_end, mode=ENC_CHECK | ENC_STOP_COLL, rmin=0.0,
            threads=1, lib=None, max_blocks=0):
    """Block-step ph4 run with idata::check_encounters after every block
    (idata.cc:620-700) and the COLLISION_DETECTION stopping condition
    (jdata.cc:797-850).  Particle ids are 1..n (slot + 1).  Returns the
    final state plus: close / coll (id pairs of the last block, None if
    none), stopped (0 none, 1 collision, 2 close), t, blocks, rmin.  The
    reference build supports only mode = CHECK | STOP_COLL with the default
    rmin; its pair order follows ph4's scheduler list, the port's slot
    order.  With lib="ref", mode CHECK | STOP_CLOSE ends the harness loop
    after the first block with a close pair (the pair ph4 would hand to
    resolve_encounter)."""
    mass, radius = _c(mass), _c(radius)
    pos, vel = _c(pos).copy(), _c(vel).copy()
    n = len(mass)
    time = np.zeros(n); step = np.zeros(n)
    enc = np.zeros(8)

    def pair(a, b):
        return None if a < 0 else (int(a), int(b))

    if lib == "ref":
        if mode not in (ENC_CHECK | ENC_STOP_COLL, ENC_CHECK | ENC_STOP_CLOSE,
                        ENC_CHECK | ENC_STOP_COLL | ENC_STOP_CLOSE) or rmin > 0:
            raise ValueError("the reference harness needs CHECK and the default rmin")
        ids = _c(np.arange(1, n + 1), np.int32)
        stats = np.zeros(5)
        pos_o = np.zeros_like(pos); vel_o = np.zeros_like(vel)
        ref().ph4ref_run_coll(n, mass, radius, ids, pos, vel, eps2, eta, t_end,
                              1 if mode & ENC_STOP_CLOSE else 0, pos_o, vel_o, time, step, stats,
                              enc)
        stop_pair = pair(enc[5], enc[6]) if enc[4] else None
        return dict(pos=pos_o, vel=vel_o, time=time, timestep=step, E0=stats[0], E1=stats[1],
                    total_steps=stats[2], t=stats[3], blocks=int(stats[4]),
                    close=pair(enc[0], enc[1]), coll=pair(enc[2], enc[3]),
                    stopped=int(enc[4]), stop_pair=stop_pair, rmin=enc[7])
    acc = np.zeros((n, 3)); jerk = np.zeros((n, 3)); pot = np.zeros(n)
    stats = np.zeros(4)
    blocks = port().orc_run_enc(n, mass, radius, pos, vel, eps2, eta, t_end, threads, acc, jerk,
                                pot, time, step, stats, max_blocks, mode, rmin, enc)
    ids = lambda a, b: None if a < 0 else (int(a) + 1, int(b) + 1)
    stopped = int(enc[6])
    coll = ids(enc[2], enc[3])
    return dict(pos=pos, vel=vel, acc=acc, jerk=jerk, pot=pot, time=time, timestep=step,
                E0=stats[0], E1=stats[1], total_steps=stats[2], t=stats[3], blocks=int(blocks),
                close=ids(enc[0], enc[1]), coll=coll, rmax_close=enc[4], rmax_coll=enc[5],
                stopped=stopped, stop_pair=coll if stopped & 1 else None, rmin=enc[7])


def smalln(mass, pos, vel, eta, t_end, n_iter=2, lib=None, dt_crit=0.0, max_steps=0):
    """smallN's few-body integrator without unperturbed binaries (smallN.cc).
    Returns (pos, vel, t_final, steps); steps is None for the reference.
    lib="ref" runs the unmodified smallN with the given dt_crit (0 disables
    its unperturbed binaries); it raises if a binary node is left at the
    end with dt_crit = 0."""
    mass, pos, vel = _c(mass), _c(pos).copy(), _c(vel).copy()
    t = np.zeros(1)
    if lib == "ref":
        rc = ref().ph4ref_smalln(len(mass), mass, pos, vel, eta, t_end, dt_crit, t)
        if rc != 0 and dt_crit == 0.0:
            raise RuntimeError("smallN built a binary node")
        return pos, vel, float(t[0]), None
    steps = port().orc_smalln(len(mass), mass, pos, vel, eta, n_iter, t_end, t, max_steps)
    return pos, vel, float(t[0]), int(steps)


# smallN's unperturbed-binary defaults (src/amuse_ph4/src/hdyn.cc:10-14 and the
# smallN worker's gamma, src/amuse_smalln/interface.cc:72)
SMALLN_DT_CRIT, SMALLN_R2_CRIT, SMALLN_GAMMA = 1e-3, 1e-2, 1e-6


def smalln_unpert(mass, pos, vel, eta, t_end, n_iter=2, dt_crit=SMALLN_DT_CRIT,
                  r2_crit=SMALLN_R2_CRIT, gamma=SMALLN_GAMMA, allow_full=True, max_steps=0):
    """smallN with its unperturbed-binary treatment (restated in
    g6_oracle.c: orc_smalln_unpert).  Returns (pos, vel, t_final, steps,
    binaries formed)."""
    mass, pos, vel = _c(mass), _c(pos).copy(), _c(vel).copy()
    t = np.zeros(1)
    nb = np.zeros(1, np.int32)
    steps = port().orc_smalln_unpert(len(mass), mass, pos, vel, eta, n_iter, t_end, dt_crit,
                                     r2_crit, gamma, 1 if allow_full else 0, t, max_steps, nb)
    if steps < 0:
        raise ValueError("more than 64 bodies")
    return pos, vel, float(t[0]), int(steps), int(nb[0])


def check_structure_ref(mass, pos, vel):
    """smallN's check_structure and get_tree (the reference build): returns
    (over, tree text) with binaries as "(first,second)" of 0-based indices."""
    buf = ctypes.create_string_buffer(4096)
    over = ref().ph4ref_check_structure(len(mass), _c(mass), _c(pos), _c(vel), buf, 4096)
    return int(over), buf.value.decode()


def kepler(mu, r0, v0, dt):
    """The two-body propagator of orc_smalln_unpert: relative (r, v) after
    dt from (r0, v0), total mass mu."""
    r, v = np.zeros(3), np.zeros(3)
    port().orc_kepler(float(mu), _c(r0), _c(v0), float(dt), r, v)
    return r, v


def hermite_fixed(mass, pos, vel, eps2, dt, nsteps):
    """The hermite code's fixed-step shared Hermite (interface.cc:266-281,
    387-552, test_mode).  Returns (pos, vel, acc, jerk) after nsteps."""
    mass, pos, vel = _c(mass), _c(pos).copy(), _c(vel).copy()
    acc = np.zeros_like(pos); jerk = np.zeros_like(pos)
    port().orc_hermite_fixed(len(mass), mass, pos, vel, eps2, dt, nsteps, acc, jerk)
    return pos, vel, acc, jerk
