"""The oracle's two-body propagator (the universal-variable solver that the
unperturbed-binary treatment advances binary components with), against
Kepler's equation solved independently here in the eccentric (hyperbolic)
anomaly by bisection: orbits from e = 0.5 to e = 1 - 1e-6 and hyperbolic
ones, across pericentre, as the binary segments take them (from a point
approaching pericentre to its mirror point), and over longer spans."""
import numpy as np
import pytest

import oracle

ROT = np.array([[0.36, 0.48, -0.8], [-0.8, 0.6, 0.0], [0.48, 0.64, 0.6]])  # orthonormal


def _bisect(f, lo, hi):
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if f(mid) < 0:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def _state(mu, a, e, anom):
    """Relative (r, v) at eccentric anomaly E (e < 1, a > 0) or hyperbolic
    anomaly F (e > 1, a > 0 its |semi-major axis|), rotated into 3-d."""
    if e < 1:
        E = anom
        r = a * (1 - e * np.cos(E))
        x = np.array([a * (np.cos(E) - e), a * np.sqrt(1 - e * e) * np.sin(E), 0.0])
        s = np.sqrt(mu * a) / r
        v = np.array([-s * np.sin(E), s * np.sqrt(1 - e * e) * np.cos(E), 0.0])
    else:
        F = anom
        r = a * (e * np.cosh(F) - 1)
        x = np.array([a * (e - np.cosh(F)), a * np.sqrt(e * e - 1) * np.sinh(F), 0.0])
        s = np.sqrt(mu * a) / r
        v = np.array([-s * np.sinh(F), s * np.sqrt(e * e - 1) * np.cosh(F), 0.0])
    return ROT @ x, ROT @ v


def _mean(e, anom):
    return anom - e * np.sin(anom) if e < 1 else e * np.sinh(anom) - anom


def _exact(mu, a, e, anom0, dt):
    n = np.sqrt(mu / a ** 3)
    M1 = _mean(e, anom0) + n * dt
    if e < 1:
        anom1 = _bisect(lambda E: _mean(e, E) - M1, M1 - 1.5, M1 + 1.5)
    else:
        w = np.arcsinh(abs(M1) / e) + 2 * abs(M1) + 10
        anom1 = _bisect(lambda F: _mean(e, F) - M1, -w, w)
    return _state(mu, a, e, anom1)


CASES = [
    # (e, starting anomaly, span as a multiple of the time to the mirror point)
    (0.5, -1.0, 1.0), (0.99, -0.3, 1.0), (0.9999, -0.05, 1.0), (1 - 1e-6, -0.01, 1.0),
    (0.99, -2.5, 1.7), (0.9999, -0.2, 0.37),
    (1.5, -1.2, 1.0), (1 + 1e-4, -0.5, 1.0), (3.0, -0.1, 5.0),
]


@pytest.mark.parametrize("e,anom0,span", CASES)
def test_kepler_propagator_against_keplers_equation(e, anom0, span):
    mu, a = 0.054, 3.8e-6  # a hard binary of the batch workload's systems
    n = np.sqrt(mu / a ** 3)
    dt = span * 2 * (-_mean(e, anom0)) / n
    r0, v0 = _state(mu, a, e, anom0)
    r, v = oracle.kepler(mu, r0, v0, dt)
    rx, vx = _exact(mu, a, e, anom0, dt)
    assert np.abs(r - rx).max() <= 1e-9 * a * max(1.0, abs(np.cosh(anom0)) if e > 1 else 1.0)
    assert np.abs(v - vx).max() <= 1e-9 * np.linalg.norm(vx) + 1e-9 * np.sqrt(mu / a)
    # energy and angular momentum of the relative orbit
    en = lambda r, v: 0.5 * v @ v - mu / np.linalg.norm(r)
    assert abs(en(r, v) - en(r0, v0)) <= 1e-9 * abs(en(r0, v0))
    assert np.abs(np.cross(r, v) - np.cross(r0, v0)).max() <= 1e-9 * np.linalg.norm(np.cross(r0, v0))


def test_kepler_propagator_backwards_and_zero():
    mu, a, e = 1.0, 1.0, 0.9
    r0, v0 = _state(mu, a, e, 0.7)
    r, v = oracle.kepler(mu, r0, v0, 0.0)
    assert np.array_equal(r, r0) and np.array_equal(v, v0)
    r, v = oracle.kepler(mu, r0, v0, -1.3)
    rx, vx = _exact(mu, a, e, 0.7, -1.3)
    assert np.abs(r - rx).max() <= 1e-12 and np.abs(v - vx).max() <= 1e-11
