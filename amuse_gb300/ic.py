"""Synthetic initial conditions in N-body units (numpy).

Restates the two AMUSE generators every workload of this library draws from,
consuming numpy's global random stream in the same order so that a given
``numpy.random.seed`` gives the same particles as AMUSE itself (pinned by
tests/test_ic.py against fixtures made with the reference package):

* ``plummer``  -- ``MakePlummerModel.result`` (src/amuse/ic/plummer.py:20-194):
  radii from the truncated cumulative-mass inversion, isotropic angles,
  von Neumann rejection for the speed distribution g(q) = q^2 (1-q^2)^3.5,
  the 1/1.695 length scaling, ``move_to_center`` and, optionally,
  ``scale_to_standard`` (src/amuse/datamodel/particle_attributes.py:48-102).
* ``salpeter_masses`` -- ``new_powerlaw_mass_distribution_nbody``
  (src/amuse/ic/salpeter.py:17-75): inverse-CDF power law, total mass 1.
"""
from __future__ import annotations

import math

import numpy as np

_MASS_CUTOFF_DEFAULT = 0.999
_RADIUS_CUTOFF_DEFAULT = 22.8042468


def _mass_cutoff(radius_cutoff=_RADIUS_CUTOFF_DEFAULT, mass_cutoff=_MASS_CUTOFF_DEFAULT):
    # plummer.py:60-75
    if radius_cutoff > 99999:
        return min(mass_cutoff, 1.0)
    rfrac = radius_cutoff * 16.0 / (3.0 * math.pi)
    return min(mass_cutoff, rfrac ** 3 / pow(1.0 + rfrac ** 2, 1.5))


def _spherical(radius, theta, phi):
    return (radius * np.sin(theta) * np.cos(phi),
            radius * np.sin(theta) * np.sin(phi),
            radius * np.cos(theta))


def _speed_fractions(n, rng):
    # plummer.py:118-140: rejection sampling; note that the reference keeps
    # only the accepted x values.
    chosen = np.zeros(0)
    while len(chosen) < n:
        m = n - len(chosen)
        x = rng.uniform(0, 1.0, m)
        y = rng.uniform(0, 0.1, m)
        g = (x ** 2) * np.power(1.0 - x ** 2, 3.5)
        chosen = np.concatenate((chosen, x.compress(y <= g)))
    return np.atleast_2d(chosen).transpose()


def pair_potential_energy(mass, pos, eps2=0.0, chunk=2048):
    """-sum_{i<j} m_i m_j / sqrt(r_ij^2 + eps2) in FP64 (chunked numpy)."""
    n = len(mass)
    total = 0.0
    for i0 in range(0, n, chunk):
        i1 = min(n, i0 + chunk)
        d = pos[i0:i1, None, :] - pos[None, :, :]
        r2 = np.einsum("ijk,ijk->ij", d, d) + eps2
        idx_i = np.arange(i0, i1)[:, None]
        idx_j = np.arange(n)[None, :]
        mask = idx_j > idx_i
        with np.errstate(divide="ignore"):
            inv = np.where(mask, 1.0 / np.sqrt(np.where(mask, r2, 1.0)), 0.0)
        total -= float(np.sum(mass[i0:i1, None] * mass[None, :] * inv))
    return total


def move_to_center(mass, pos, vel):
    mtot = mass.sum()
    pos -= (mass[:, None] * pos).sum(axis=0) / mtot
    vel -= (mass[:, None] * vel).sum(axis=0) / mtot


def scale_to_standard(mass, pos, vel, potential_energy=None, virial_ratio=0.5):
    """particle_attributes.py:48-102 (unsoftened): M=1, U=-1/2, Q=virial_ratio.

    ``potential_energy(mass, pos)`` may be supplied (e.g. a GPU evaluation);
    the default is the FP64 numpy pair sum.
    """
    mass *= 1.0 / mass.sum()
    pe = (potential_energy or pair_potential_energy)(mass, pos)
    pos *= pe / -0.5
    pe = -0.5
    kin = 0.5 * float(np.sum(mass * np.sum(vel * vel, axis=1)))
    vel *= math.sqrt(abs(virial_ratio * pe) / kin)


def plummer(n, do_scale=False, rng=None, potential_energy=None):
    """Return (mass[n], pos[n,3], vel[n,3]) like ``new_plummer_model(n)``."""
    rng = np.random if rng is None else rng
    mcut = _mass_cutoff()
    mass = np.ones(n) / n
    radius = 1.0 / np.sqrt(np.power(rng.uniform(0, mcut, (n, 1)), -2.0 / 3.0) - 1.0)
    theta = np.arccos(rng.uniform(-1.0, 1.0, (n, 1)))
    phi = rng.uniform(0.0, 2 * math.pi, (n, 1))
    x, y, z = _spherical(radius, theta, phi)
    q = _speed_fractions(n, rng)
    speed = q * math.sqrt(2.0) * np.power(1.0 + radius * radius, -0.25)
    theta = np.arccos(rng.uniform(-1.0, 1.0, (n, 1)))
    phi = rng.uniform(0.0, 2 * math.pi, (n, 1))
    vx, vy, vz = _spherical(speed, theta, phi)
    pos = np.hstack([x, y, z]).reshape(n, 3) / 1.695
    vel = np.hstack([vx, vy, vz]).reshape(n, 3) / math.sqrt(1 / 1.695)
    move_to_center(mass, pos, vel)
    if do_scale:
        scale_to_standard(mass, pos, vel, potential_energy)
    return mass, pos, vel


def salpeter_masses(n, alpha=-2.35, mass_min=0.1, mass_max=125.0, rng=None):
    """``new_powerlaw_mass_distribution_nbody`` (total mass normalised to 1)."""
    rng = np.random if rng is None else rng
    a1 = alpha + 1
    factor = pow(mass_max / mass_min, a1) - 1.0
    m = mass_min * np.power(1.0 + factor * rng.random_sample(n), 1.0 / a1)
    return m / m.sum()


def plummer_salpeter(n, alpha=-2.35, mass_min=0.1, mass_max=100.0, rng=None,
                     potential_energy=None):
    """Plummer positions/velocities with a power-law IMF, re-scaled to
    standard units after the masses are assigned."""
    rng = np.random if rng is None else rng
    _, pos, vel = plummer(n, do_scale=False, rng=rng)
    mass = salpeter_masses(n, alpha, mass_min, mass_max, rng=rng)
    move_to_center(mass, pos, vel)
    scale_to_standard(mass, pos, vel, potential_energy)
    return mass, pos, vel


def encounter_batch(nsys=4096, nmin=3, nmax=64, r_vir=1e-3, seed=1):
    """Independent few-body systems: n ~ U[nmin, nmax] per system (seeded),
    each an equal-mass Plummer realisation in standard units (M = 1),
    re-scaled to virial radius r_vir (positions x r_vir, velocities
    x r_vir^-1/2, which keeps virial equilibrium with G = M = 1).
    Returns (n_per_sys, mass, pos, vel, t_cross) with bodies back to back and
    t_cross = 2 sqrt(2) r_vir^1.5 (G = M = 1)."""
    rng = np.random.RandomState(seed)
    ns = rng.randint(nmin, nmax + 1, size=nsys)
    ms, xs, vs = [], [], []
    for n in ns:
        m, x, v = plummer(int(n), do_scale=True, rng=rng)
        ms.append(m)
        xs.append(x * r_vir)
        vs.append(v / math.sqrt(r_vir))
    t_cross = 2 * math.sqrt(2) * r_vir ** 1.5
    return ns.astype(np.int32), np.concatenate(ms), np.concatenate(xs), np.concatenate(vs), t_cross
