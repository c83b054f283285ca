"""The reconnection configuration's Harris sheet (conducting walls in x, periodic y) on the
GPU: FP64 parity with the oracle and the mixed path against the FP64 path.

Tolerances (stated per test):
  * one fused step, exact build: particles, permutation, np2, cumcnt bit-exact; fields 1e-12;
  * eight steps, FP64 (FMA) build, oracle at the GPU's CG counts: 1e-10 relative;
  * mixed against FP64 over 40 steps: kinetic and field energies 1e-3 relative, total
    energy 1e-4; charge conservation of the FP32 deposit 1e-6 of |d rho / dt|;
  * every particle stays between the walls, none is lost.
"""
import numpy as np
import pytest

from tests.helpers import continuity_residual
from tests.test_gpu_mixed2d import _match_order
from tests.test_gpu_parity2d import assert_field, assert_particles, make_oracle
from wumingpic_gb300.loader import config_harris2d, load_harris2d
from wumingpic_gb300.pic2d import Pic2D

pytestmark = pytest.mark.gpu


def between_walls(st, p):
    for isp in range(p.nsp):
        for jj in range(p.ny):
            x = st.up[0, :st.np2[jj, isp], jj, isp]
            if len(x) and (x.min() < (p.nxgs + 1) * p.delx or x.max() >= (p.nxge - 1) * p.delx):
                return False
    return True


def test_harris_one_step_exact(gpu_lib):
    p = config_harris2d(seed=51)
    st = load_harris2d(p)
    g = Pic2D(p, precision="fp64_exact")
    g.put_state(st)
    g.step(1)
    o = make_oracle(p)
    o.cg_control(fixed=g.cg_iters())
    ref = st.copy()
    assert o.step(ref) == 0
    out = g.get_state()
    assert_particles(out.up, out.np2, ref.up, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_field(out.uf, ref.uf, 1e-12)
    g.close()


def test_harris_steps_fp64(gpu_lib):
    p = config_harris2d(seed=52)
    st = load_harris2d(p)
    g = Pic2D(p, precision="fp64")
    g.put_state(st)
    o = make_oracle(p)
    ref = st.copy()
    for _ in range(8):
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_particles(out.up, out.np2, ref.up, ref.np2, rel=1e-10)
    assert_field(out.uf, ref.uf, 1e-10)
    assert between_walls(out, p)
    g.close()


def test_harris_mixed_against_fp64(gpu_lib):
    p = config_harris2d(seed=53)
    st = load_harris2d(p)
    gm, gd = Pic2D(p, precision="mixed"), Pic2D(p, precision="fp64")
    gm.put_state(st)
    gd.put_state(st)
    q, _ = p.charges()
    before = gm.get_state()
    gm.step(1)
    after = gm.get_state()
    res, scale = continuity_residual(p, q, before.up, _match_order(before, after, p), before.np2, gm.get_uj())
    assert res <= 1e-6 * scale, (res, scale)
    gm.step(39)
    gd.step(40)
    em, ed = gm.energy(), gd.energy()
    np.testing.assert_allclose(em, ed, rtol=1e-3)
    assert abs(em.sum() - ed.sum()) <= 1e-4 * ed.sum()
    a = gm.get_state()
    assert a.np2.sum() == p.n_particles and between_walls(a, p)
    gm.close()
    gd.close()
