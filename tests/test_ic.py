"""amuse_gb300.ic pinned against AMUSE's own generators (fixture made from
src/amuse/ic/plummer.py and salpeter.py by tests/golden/make_golden.py)."""
import numpy as np

from amuse_gb300 import ic
from conftest import golden


def test_plummer_matches_amuse():
    g = golden("ic_amuse.npz")
    np.random.seed(1)
    m, x, v = ic.plummer(256, do_scale=False)
    assert np.array_equal(m, g["plummer_mass"])
    assert np.allclose(x, g["plummer_pos"], rtol=0, atol=1e-14)
    assert np.allclose(v, g["plummer_vel"], rtol=0, atol=1e-14)


def test_plummer_scaled_matches_amuse():
    g = golden("ic_amuse.npz")
    np.random.seed(1)
    m, x, v = ic.plummer(256, do_scale=True)
    assert np.allclose(x, g["scaled_pos"], rtol=0, atol=1e-13)
    assert np.allclose(v, g["scaled_vel"], rtol=0, atol=1e-13)
    # standard units: U = -1/2, K = 1/4
    assert ic.pair_potential_energy(m, x) == np.float64(-0.5) or abs(
        ic.pair_potential_energy(m, x) + 0.5) < 1e-12
    assert abs(0.5 * np.sum(m * np.sum(v * v, 1)) - 0.25) < 1e-12


def test_salpeter_matches_amuse():
    g = golden("ic_amuse.npz")
    np.random.seed(3)
    m = ic.salpeter_masses(512, mass_max=100.0)
    assert np.allclose(m, g["salpeter_mass"], rtol=1e-14, atol=0)
    assert abs(m.sum() - 1) < 1e-12
