"""The seeded synthetic configurations (rismo2d_gb300/meshgen.py) on the CPU: sizes,
determinism and the properties the workloads rely on."""

import numpy as np

from rismo2d_gb300 import meshgen


def test_braided_window_shape_and_bed():
    """A small window of the braided river: P2 strip sizes, anabranch beds below the
    valley line, bars above it, a dry start on the bars and a wet one in the channels."""
    m = meshgen.braided(nx=40, ny=50, length=200.0, width=200.0)
    assert m.ne == 2 * 40 * 50
    assert m.np == (2 * 40 + 1) * (2 * 50 + 1)
    valley = 5.0e-4 * (200.0 - m.x)
    rel = m.z - valley
    assert rel.min() >= -3.0 - 0.3 - 1e-9          # channel bed with its roughness
    assert rel.max() <= 1.0 + 2.0 + 1e-9           # bar top
    wet = m.S0 - m.z > 0.0
    assert 0.0 < wet.mean() < 1.0
    assert np.all(m.S0 >= m.z - 1e-12)
    again = meshgen.braided(nx=40, ny=50, length=200.0, width=200.0)
    assert np.array_equal(again.z, m.z)
    other = meshgen.braided(nx=40, ny=50, length=200.0, width=200.0, seed=6)
    assert not np.array_equal(other.z, m.z)


def test_braided_hydrograph_rises_to_its_peak():
    h = meshgen.braided_hydrograph(S=10.0)
    t = np.array([r[0] for r in h])
    q = np.array([r[1] for r in h])
    assert q[0] == 500.0 and abs(q.max() - 3000.0) < 1e-6
    assert abs(t[np.argmax(q)] - 43200.0) < 600.0 + 1e-9   # peak at 12 h


def test_meander_bump_fields():
    """The learned configuration's beds: no bumps leaves the meander unchanged; a bump
    field is reproducible from its seed, differs between seeds and stays within the
    sum of the overlapping amplitudes."""
    base = meshgen.meander(nx=60, ny=10, length=600.0)
    same = meshgen.meander(nx=60, ny=10, length=600.0, bumps=0, bump_seed=10)
    assert np.array_equal(base.z, same.z)
    a = meshgen.meander(nx=60, ny=10, length=600.0, bumps=20, bump_seed=10, bump_amp=(0.05, 0.25))
    b = meshgen.meander(nx=60, ny=10, length=600.0, bumps=20, bump_seed=10, bump_amp=(0.05, 0.25))
    c = meshgen.meander(nx=60, ny=10, length=600.0, bumps=20, bump_seed=11, bump_amp=(0.05, 0.25))
    assert np.array_equal(a.z, b.z)
    assert not np.array_equal(a.z, c.z)
    d = a.z - base.z
    assert np.max(np.abs(d)) > 0.01
    assert np.max(np.abs(d)) <= 20 * 0.25
    assert np.all(a.S0 >= a.z - 1e-12)
    # the mesh itself is the meander's
    assert np.array_equal(a.elems, base.elems) and np.array_equal(a.x, base.x)
