"""Edge cases of the state on the GPU: no particles at all, one species empty, particles on
cell faces, empty rows and cells on the mixed path and in 3D.

Tolerances (stated per test):
  * exact build against the oracle: after one step particles, permutation, np2, cumcnt
    bit-exact and fields 1e-12 (CG reductions); after the next step (pushed by those
    fields) particles 1e-12, integer bookkeeping still exact;
  * FMA build and mixed path without particles: fields 1e-12 of the oracle's;
  * mixed path with particles against the FP64 path: energies 1e-4 relative.
"""
import numpy as np
import pytest

from tests import test_gpu_parity3d as p3
from tests.helpers import small_case
from tests.test_gpu_parity2d import assert_field, assert_particles, make_oracle, perturbed_case
from wumingpic_gb300.pic2d import Pic2D
from wumingpic_gb300.pic3d import Pic3D

pytestmark = pytest.mark.gpu


def emptied(st, species):
    for isp in species:
        st.np2[..., isp] = 0
        st.cumcnt[..., isp] = 0
    return st


def run_against_oracle(p, st, precision, steps):
    g = Pic2D(p, precision=precision)
    g.put_state(st)
    o = make_oracle(p)
    ref = st.copy()
    for _ in range(steps):
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    e = g.energy()
    g.close()
    return out, ref, e, o


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "mixed"])
def test_no_particles(gpu_lib, precision):
    """A vacuum: the implicit field update alone, every kernel launched on empty columns."""
    p, st = perturbed_case(seed=61, nx=16, ny=16)
    emptied(st, range(p.nsp))
    out, ref, e, o = run_against_oracle(p, st, precision, 3)
    assert out.np2.sum() == 0
    assert_field(out.uf, ref.uf, 1e-12)
    assert e[0] == 0.0 and e[1] == 0.0


def exact_then_close(p, st):
    """one step bit-exact, then a second within 1e-12"""
    for steps, rel in ((1, 0.0), (2, 1e-12)):
        out, ref, e, o = run_against_oracle(p, st, "fp64_exact", steps)
        assert_particles(out.up, out.np2, ref.up, ref.np2, rel)
        np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
        assert_field(out.uf, ref.uf, 1e-12)


def test_one_species_empty(gpu_lib):
    p, st = perturbed_case(seed=62, nx=16, ny=12)
    exact_then_close(p, emptied(st, [0]))


def on_faces(p, st, rng):
    """Every third particle moved onto its cell's lower x face, every fifth onto its lower
    y face, every seventh to the largest double below its cell's upper x face: cell indices,
    and so cumcnt, unchanged."""
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            x = st.up[0, :n, jj, isp]
            y = st.up[1, :n, jj, isp]
            x[::3] = np.floor(x[::3])
            y[::5] = np.floor(y[::5])
            x[1::7] = np.nextafter(np.floor(x[1::7]) + 1.0, 0.0)
    return st


def test_particles_on_cell_faces(gpu_lib):
    p, st = perturbed_case(seed=63, nx=16, ny=16)
    st = on_faces(p, st, np.random.default_rng(63))
    exact_then_close(p, st)
    # the mixed path takes the same state (offsets 0 and just below 1 in FP32)
    gm, gd = Pic2D(p, precision="mixed"), Pic2D(p, precision="fp64")
    gm.put_state(st)
    gd.put_state(st)
    gm.step(3)
    gd.step(3)
    np.testing.assert_allclose(gm.energy(), gd.energy(), rtol=1e-4)
    assert gm.get_state().np2.sum() == st.np2.sum()
    gm.close()
    gd.close()


def test_mixed_empty_rows_and_cells(gpu_lib):
    p, st = small_case(nx=16, ny=16, ppc=4, seed=64)
    st.np2[3, :] = 0
    st.cumcnt[:, 3, :] = 0
    n = st.np2[0, 1]
    keep = st.up[0, :n, 0, 1] >= p.nxgs + 3  # the first three cells of row 0, species 1, emptied
    k = int(keep.sum())
    st.up[:, :k, 0, 1] = st.up[:, :n, 0, 1][:, keep]
    st.np2[0, 1] = k
    cnt = np.bincount(st.up[0, :k, 0, 1].astype(int) - p.nxgs, minlength=p.nx)
    st.cumcnt[:, 0, 1] = np.concatenate([[0], np.cumsum(cnt)])
    gm, gd = Pic2D(p, precision="mixed"), Pic2D(p, precision="fp64")
    gm.put_state(st)
    gd.put_state(st)
    gm.step(4)
    gd.step(4)
    np.testing.assert_allclose(gm.energy(), gd.energy(), rtol=1e-4)
    assert gm.get_state().np2.sum() == gd.get_state().np2.sum() == st.np2.sum()
    gm.close()
    gd.close()


def test_3d_empty_rows(gpu_lib):
    p, st = p3.perturbed_case(seed=65)
    st.np2[1, 2, :] = 0
    st.cumcnt[:, 1, 2, :] = 0
    st.np2[0, 0, 1] = 0
    st.cumcnt[:, 0, 0, 1] = 0
    for steps, rel in ((1, 0.0), (2, 1e-12)):
        g = Pic3D(p, precision="fp64_exact")
        g.put_state(st)
        o = p3.make_oracle(p)
        ref = st.copy()
        for _ in range(steps):
            g.step(1)
            o.cg_control(fixed=g.cg_iters())
            assert o.step(ref) == 0
        out = g.get_state()
        p3.assert_particles(out.up, out.np2, ref.up, ref.np2, rel)
        np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
        p3.assert_field(out.uf, ref.uf, 1e-12)
        g.close()
