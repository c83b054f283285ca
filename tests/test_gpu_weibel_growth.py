"""Weibel growth rate of the mixed-precision path against the FP64 path (GPU).

The mixed path (integer cell + FP32 offset, FP32 push and deposition, FP64
fields and CG) must reproduce the physics of the FP64 path, with the Boris and
(2D) the Vay pusher: from the same
initial state, the exponential growth rate of the magnetic field energy in the
linear phase of the Weibel instability agrees within 1 %, and both runs reach
saturation (the nonlinear stage concentrates particles into current filaments,
several times the mean density per cell, which exercises the growth of the
mixed path's cell columns).  The energy history is the reference's
energy_history sums (2d/proj/weibel/app.f90:479-545).
"""
import numpy as np
import pytest

from wumingpic_gb300.diagnostics import energy_history, growth_rate
from wumingpic_gb300.loader import Plasma2D, load_weibel2d

pytestmark = pytest.mark.gpu

GROWTH_RATE_RTOL = 0.01


def _run(p, st, precision, nsteps, pusher="boris"):
    from wumingpic_gb300.pic2d import Pic2D
    g = Pic2D(p, precision=precision)
    g.set_pusher(pusher)
    g.put_state(st)
    t, e = energy_history(g.step, g.energy, nsteps, 10, p.delt)
    g.close()
    return t, e


@pytest.mark.parametrize("pusher", ["boris", "vay"])
def test_weibel_growth_rate_mixed_matches_fp64(gpu_lib, pusher):
    # counter-streaming electrons along z (+-0.5 c), filamentation in the x-y plane
    p = Plasma2D(nx=128, ny=128, ppc=16, drift=0.5, u_the=0.05, seed=424242, np_slack=5.0)
    st = load_weibel2d(p)
    nsteps = 1000
    t, e64 = _run(p, st, "fp64", nsteps, pusher)
    _, emx = _run(p, st, "mixed", nsteps, pusher)
    b64, bmx = e64[:, 3], emx[:, 3]
    # saturation reached: the magnetic energy grew by orders of magnitude in both runs
    assert b64.max() > 1e3 * b64[1] and bmx.max() > 1e3 * bmx[1]
    g64, win64, n64 = growth_rate(t, b64)
    gmx, winmx, nmx = growth_rate(t, bmx)
    assert n64 >= 5 and nmx >= 5
    assert abs(gmx / g64 - 1.0) <= GROWTH_RATE_RTOL, (gmx, g64, win64, winmx)
    # total energy of the two runs tracks within 1 % through saturation
    tot64, totmx = e64.sum(axis=1), emx.sum(axis=1)
    np.testing.assert_allclose(totmx, tot64, rtol=1e-2)


def test_weibel_growth_rate_mixed_matches_fp64_3d(gpu_lib):
    """The 3D configuration's physics (beams +-0.5c along x, u_th 0.05c, m_i/m_e 16) on
    32^3 cells: the mixed 3D path's magnetic growth rate within 1 % of the FP64 path's
    from the same initial state, both saturating, total energies within 1 %."""
    from wumingpic_gb300.loader import Plasma3D, load_weibel3d
    from wumingpic_gb300.pic3d import Pic3D
    p = Plasma3D(nx=32, ny=32, nz=32, ppc=16, mass_ratio=16.0, drift=0.5, drift_axis=0, u_the=0.05,
                 seed=434343, np_slack=16.0)
    st = load_weibel3d(p)
    runs = {}
    for precision in ("fp64", "mixed"):
        g = Pic3D(p, precision=precision)
        g.put_state(st)
        runs[precision] = energy_history(g.step, g.energy, 800, 10, p.delt)
        g.close()
    t, e64 = runs["fp64"]
    _, emx = runs["mixed"]
    b64, bmx = e64[:, 3], emx[:, 3]
    assert b64.max() > 1e2 * b64[1] and bmx.max() > 1e2 * bmx[1]
    g64, win64, n64 = growth_rate(t, b64)
    gmx, winmx, nmx = growth_rate(t, bmx)
    assert n64 >= 5 and nmx >= 5
    assert abs(gmx / g64 - 1.0) <= GROWTH_RATE_RTOL, (gmx, g64, win64, winmx)
    np.testing.assert_allclose(emx.sum(axis=1), e64.sum(axis=1), rtol=1e-2)
