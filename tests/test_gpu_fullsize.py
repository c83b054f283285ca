"""Size-independent properties at the full sizes of the 2D and 3D Weibel configurations
(the bench workloads), checked through device-side reductions so that no particle array
crosses to the host:

  * 2D, 2048 x 2048 cells, 64 ppc/species (536,870,912 particles): particle count conserved
    over the steps; the mixed path bitwise reproducible (two contexts, same plasma: identical
    fields and energies); mixed against FP64 from the same Philox plasma after 2 steps,
    every energy_history sum within 1e-4 relative;
  * 3D, 256^3 cells, 16 ppc/species (536,870,912 particles): the same count and
    mixed-against-FP64 checks after one step.
Contexts are released before the next one is made (the 2D FP64 state holds ~64 GB).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def weibel2d_full():
    from wumingpic_gb300.loader import Plasma2D
    return Plasma2D(nx=2048, ny=2048, ppc=64, drift=0.3, u_the=0.1, seed=20261206, np_slack=1.25)


def run2d(p, precision, steps):
    from wumingpic_gb300.pic2d import Pic2D
    g = Pic2D(p, precision=precision)
    g.load_weibel()
    n0 = g.num_particles()
    counts = []
    for _ in range(steps):
        g.step(1)
        counts.append(g.num_particles())
    e = g.energy()
    uf = g.get_fields() if precision == "mixed" else None
    g.close()
    return n0, counts, e, uf


def test_weibel2d_full_size(gpu_lib):
    p = weibel2d_full()
    n0, counts, em, ufm = run2d(p, "mixed", 2)
    assert n0 == p.n_particles and counts == [n0, n0]
    n1, counts1, em1, ufm1 = run2d(p, "mixed", 2)
    np.testing.assert_array_equal(em1, em)  # bitwise reproducible
    np.testing.assert_array_equal(ufm1, ufm)
    n2, counts2, ed, _ = run2d(p, "fp64", 2)
    assert counts2 == [n0, n0]
    np.testing.assert_allclose(em, ed, rtol=1e-4)


def test_weibel3d_full_size(gpu_lib):
    from wumingpic_gb300.loader import Plasma3D
    from wumingpic_gb300.pic3d import Pic3D
    p = Plasma3D(nx=256, ny=256, nz=256, ppc=16, mass_ratio=16.0, drift=0.5, drift_axis=0, u_the=0.05,
                 seed=20261207, np_slack=1.5)
    out = {}
    for precision in ("mixed", "fp64"):
        g = Pic3D(p, precision=precision)
        g.load_weibel()
        n0 = g.num_particles()
        g.step(1)
        assert n0 == p.n_particles and g.num_particles() == n0
        out[precision] = g.energy()
        g.close()
    np.testing.assert_allclose(out["mixed"], out["fp64"], rtol=1e-4)
