"""GPU parity of the 2D FP64 path against the CPU oracle, stage by stage and
for whole steps, through the C ABI.

Tolerances (stated per test):
  * integer work (cell indices, np2, cumcnt, permutations, IDs): bit-exact;
  * FP64_EXACT build, push and deposit: bit-exact (same operations, same order);
  * FP64 (FMA) build: 1e-12 relative to the array's max magnitude;
  * fields after the CG solve: 1e-12 relative (reduction order differs), with
    the oracle run at the GPU's CG iteration counts (parity mode).
"""
import numpy as np
import pytest

from oracle.oracle import Oracle2D
from tests.helpers import continuity_residual, small_case, small_plasma
from wumingpic_gb300 import _lib
from wumingpic_gb300.loader import load_weibel2d

pytestmark = pytest.mark.gpu

REL = 1e-12


def make_oracle(p):
    q, r = p.charges()
    return Oracle2D(nx=p.nx, ny=p.ny, np_cap=p.np_cap, q=q, r=r, delt=p.delt, delx=p.delx, c=p.c, gfac=p.gfac,
                    bc=p.bc)


def make_gpu(p, precision, gpu_lib, **kw):
    from wumingpic_gb300.pic2d import Pic2D
    return Pic2D(p, precision=precision, **kw)


def valid(up, np2):
    """list of per-(row, species) valid slot arrays"""
    out = []
    for isp in range(up.shape[3]):
        for jj in range(up.shape[2]):
            out.append(up[:, :np2[jj, isp], jj, isp])
    return out


def assert_particles(a_up, a_np2, b_up, b_np2, rel=0.0):
    np.testing.assert_array_equal(a_np2, b_np2)
    for a, b in zip(valid(a_up, a_np2), valid(b_up, b_np2)):
        np.testing.assert_array_equal(a[5].view(np.int64), b[5].view(np.int64))  # ids: the permutation
        if rel == 0.0:
            np.testing.assert_array_equal(a[:5], b[:5])
        else:
            for k in range(5):
                scale = max(np.abs(b[k]).max(initial=0.0), 1e-300)
                np.testing.assert_allclose(a[k], b[k], rtol=0, atol=rel * scale)


def assert_field(a, b, rel):
    scale = max(np.abs(b).max(), 1e-300)
    if rel == 0.0:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=0, atol=rel * scale)


def perturbed_case(seed=7, nx=16, ny=12, ppc=6, **kw):
    """Small plasma with non-trivial fields so that every term of the push is exercised."""
    p, st = small_case(nx=nx, ny=ny, ppc=ppc, seed=seed, **kw)
    rng = np.random.default_rng(seed)
    st.uf[...] = 0.02 * rng.standard_normal(st.uf.shape)
    # keep the ghosts periodic copies, as the reference's state always is
    st.uf[:, :2, :] = st.uf[:, p.nx:p.nx + 2, :]
    st.uf[:, p.nx + 2:, :] = st.uf[:, 2:4, :]
    st.uf[:, :, :2] = st.uf[:, :, p.ny:p.ny + 2]
    st.uf[:, :, p.ny + 2:] = st.uf[:, :, 2:4]
    return p, st


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_push_parity(gpu_lib, precision, rel):
    p, st = perturbed_case()
    o = make_oracle(p)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    g.particle__solv()
    gp_gpu, np2, _ = g.get_particles(1)
    ref = st.copy()
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    assert_particles(gp_gpu, np2, ref.gp, ref.np2, rel)


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_push_vay_parity(gpu_lib, precision, rel):
    """particle__solv_vay (2d/common/particle.f90:182) against the oracle's Vay update."""
    p, st = perturbed_case(seed=8, u_the=0.3)
    st.uf[:3] *= 40.0  # magnetic rotation of a few tenths of a radian per step for electrons
    o = make_oracle(p)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    g.particle__solv_vay()
    gp_gpu, np2, _ = g.get_particles(1)
    ref = st.copy()
    assert o.particle_solv_vay(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    assert_particles(gp_gpu, np2, ref.gp, ref.np2, rel)


def test_one_step_vay_exact_is_bit_exact_on_particles(gpu_lib):
    """The fused step with the Vay push selected, exact build: particles bit-identical."""
    p, st = perturbed_case(seed=33, nx=16, ny=12, ppc=6)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.set_pusher("vay")
    g.put_state(st)
    g.step(1)
    o = make_oracle(p)
    o.cg_control(fixed=g.cg_iters())
    ref = st.copy()
    assert o.step(ref, pusher="vay") == 0
    out = g.get_state()
    assert_particles(out.up, out.np2, ref.up, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_field(out.uf, ref.uf, REL)


def test_vay_on_the_mixed_path_is_a_step_option(gpu_lib):
    """The mixed path runs Vay inside its fused step: wpic_set_pusher for wpic_step, or the
    staged particle__solv_vay, which requests a Vay push that the following field__fdtd_i runs
    (the two give the same state bit for bit)."""
    p, st = perturbed_case(seed=34, nx=16, ny=16)
    g = make_gpu(p, "mixed", gpu_lib)
    g.put_state(st)
    g.set_pusher("vay")
    g.step(1)
    h = make_gpu(p, "mixed", gpu_lib)
    h.put_state(st)
    h.particle__solv_vay()
    h.field__fdtd_i()
    a, b = g.get_state(), h.get_state()
    np.testing.assert_array_equal(a.np2, b.np2)
    np.testing.assert_array_equal(a.uf, b.uf)
    for isp in range(p.nsp):
        for j in range(p.ny):
            n = a.np2[j, isp]
            np.testing.assert_array_equal(a.up[:, :n, j, isp], b.up[:, :n, j, isp])


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_deposit_parity(gpu_lib, precision, rel):
    """ele_cur + bc__curre: the exact build reproduces the single-thread reduction order bit for bit."""
    p, st = perturbed_case(seed=12)
    o = make_oracle(p)
    ref = st.copy()
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    uj_ref = np.zeros((3, p.nx + 4, p.ny + 4), order="F")
    assert o.ele_cur(uj_ref, ref.up, ref.gp, ref.cumcnt) == 0
    assert o.bc_curre(uj_ref) == 0
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(ref, gp=True)
    g.ele_cur()
    assert_field(g.get_uj(), uj_ref, rel)


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64"])
def test_field_fdtd_i_parity(gpu_lib, precision):
    p, st = perturbed_case(seed=21)
    o = make_oracle(p)
    ref = st.copy()
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(ref, gp=True)
    g.field__fdtd_i()
    it_gpu = g.cg_iters()
    o2 = make_oracle(p)
    assert o2.field_fdtd_i(ref.uf, ref.up, ref.gp, ref.cumcnt) == 0
    it_ref = o2.cg_iters()
    # the reference stopping rule usually gives the same counts; parity is checked at equal counts
    assert np.abs(it_gpu - it_ref).max() <= 1
    ref2 = st.copy()
    o3 = make_oracle(p)
    o3.cg_control(fixed=it_gpu)
    assert o3.particle_solv(ref2.gp, ref2.up, ref2.uf, ref2.cumcnt) == 0
    assert o3.field_fdtd_i(ref2.uf, ref2.up, ref2.gp, ref2.cumcnt) == 0
    assert_field(g.get_fields(), ref2.uf, REL)
    assert_field(g.get_df(), o3.get_df(), REL)


def test_particle_boundaries_and_sort_are_bit_exact(gpu_lib):
    """bc__particle_x (round-down wraps), bc__particle_y (migration) and sort__bucket:
    integer bookkeeping and permutations identical to the oracle."""
    p, st = perturbed_case(seed=5, nx=12, ny=8, ppc=5)
    rng = np.random.default_rng(5)
    # large displacements (|dy| < 1 cell) so that many particles migrate and wrap
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            st.gp[:, :n, jj, isp] = st.up[:, :n, jj, isp]
            st.gp[0, :n, jj, isp] += rng.uniform(-0.9, 0.9, n)
            st.gp[1, :n, jj, isp] += rng.uniform(-0.9, 0.9, n)
    st.np2[2, 0] -= 7  # uneven rows: both b < h and b > h occur
    st.np2[5, 1] -= 3
    for isp in range(p.nsp):
        for jj in range(p.ny):
            cnt = np.bincount(st.up[0, :st.np2[jj, isp], jj, isp].astype(int) - p.nxgs, minlength=p.nx)
            st.cumcnt[:, jj, isp] = np.concatenate([[0], np.cumsum(cnt)])
    o = make_oracle(p)
    g = make_gpu(p, "fp64", gpu_lib)
    g.put_state(st, gp=True)
    ref = st.copy()
    g.bc__particle_x()
    assert o.bc_particle_x(ref.gp, ref.np2) == 0
    b_gp, b_np2, _ = g.get_particles(1)
    assert_particles(b_gp, b_np2, ref.gp, ref.np2)
    g.bc__particle_y()
    assert o.bc_particle_y(ref.gp, ref.np2) == 0
    b_gp, b_np2, _ = g.get_particles(1)
    assert_particles(b_gp, b_np2, ref.gp, ref.np2)
    g.sort__bucket()
    assert o.sort_bucket(ref.up, ref.gp, ref.cumcnt, ref.np2) == 0
    a_up, a_np2, a_cc = g.get_particles(0)
    assert_particles(a_up, a_np2, ref.up, ref.np2)
    np.testing.assert_array_equal(a_cc, ref.cumcnt)


@pytest.mark.parametrize("bc", ["periodic", "reconnection"])
def test_one_step_exact_is_bit_exact_on_particles(gpu_lib, bc):
    """One fused step in the exact build: particle state, permutation, np2 and cumcnt
    bit-identical to the oracle; fields within 1e-12."""
    p, st = perturbed_case(seed=31, nx=16, ny=12, ppc=6, bc=bc)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.step(1)
    it = g.cg_iters()
    o = make_oracle(p)
    o.cg_control(fixed=it)
    ref = st.copy()
    assert o.step(ref) == 0
    out = g.get_state()
    assert_particles(out.up, out.np2, ref.up, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_field(out.uf, ref.uf, REL)


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64"])
def test_multistep_parity(gpu_lib, precision):
    """Ten steps of a Weibel plasma: every step the oracle runs at the GPU's CG
    counts; state stays within 1e-10 relative and the integer bookkeeping agrees."""
    p, st = small_case(nx=16, ny=16, ppc=8, seed=41)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    o = make_oracle(p)
    ref = st.copy()
    for _ in range(10):
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_particles(out.up, out.np2, ref.up, ref.np2, rel=1e-10)
    assert_field(out.uf, ref.uf, 1e-10)
    np.testing.assert_allclose(g.energy(), o.energy(ref.up, ref.uf, ref.np2), rtol=1e-10)


def test_cg_iteration_counts_follow_reference_rule(gpu_lib):
    p, st = small_case(nx=16, ny=16, ppc=8, seed=43)
    g = make_gpu(p, "fp64", gpu_lib)
    g.put_state(st)
    o = make_oracle(p)
    ref = st.copy()
    agree = 0
    for _ in range(5):
        g.step(1)
        it_g = g.cg_iters()
        assert o.step(ref) == 0
        it_o = o.cg_iters()
        agree += int((it_g == it_o).all())
    assert agree >= 4


def test_energy_parity(gpu_lib):
    p, st = perturbed_case(seed=3)
    g = make_gpu(p, "fp64", gpu_lib)
    g.put_state(st)
    o = make_oracle(p)
    np.testing.assert_allclose(g.energy(), o.energy(st.up, st.uf, st.np2), rtol=1e-13)


def test_empty_rows_and_cells(gpu_lib):
    """Rows and cells without particles (edge of the bucket bookkeeping)."""
    p, st = small_case(nx=8, ny=6, ppc=3, seed=17)
    st.np2[2, :] = 0
    st.cumcnt[:, 2, :] = 0
    # empty the first two cells of row 0 of species 0
    n = st.np2[0, 0]
    keep = st.up[0, :n, 0, 0] >= p.nxgs + 2
    k = keep.sum()
    st.up[:, :k, 0, 0] = st.up[:, :n, 0, 0][:, keep]
    st.np2[0, 0] = k
    cnt = np.bincount(st.up[0, :k, 0, 0].astype(int) - p.nxgs, minlength=p.nx)
    st.cumcnt[:, 0, 0] = np.concatenate([[0], np.cumsum(cnt)])
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.step(2)
    o = make_oracle(p)
    ref = st.copy()
    o.cg_control(fixed=None)
    for _ in range(2):
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)


def test_status_codes_instead_of_stop(gpu_lib):
    """The reference stops the program; the library returns a status and stays usable."""
    from wumingpic_gb300._lib import WpicError
    p, st = small_case(nx=8, ny=6, ppc=4, seed=2)
    # capacity: device rows hold exactly the initial population; force arrivals
    g = make_gpu(p, "fp64", gpu_lib, device_cap=p.nx * p.ppc)
    g.put_state(st, gp=True)
    up, np2, _ = g.get_particles(1)
    for isp in range(p.nsp):
        up[1, :np2[1, isp] // 2, 1, isp] -= 1.0  # half of row 1 moves down into a full row 0
    g.put_particles(1, up, np2)
    with pytest.raises(WpicError) as e:
        g.bc__particle_y()
    assert e.value.status == _lib.CAPACITY
    # moved more than one row
    g2 = make_gpu(p, "fp64", gpu_lib)
    g2.put_state(st, gp=True)
    up, np2, _ = g2.get_particles(1)
    up[1, 0, 1, 0] += 2.0
    g2.put_particles(1, up, np2)
    with pytest.raises(WpicError) as e:
        g2.bc__particle_y()
    assert e.value.status == _lib.MOVED_TOO_FAR
    # CG not converged within ite_max
    g3 = make_gpu(p, "fp64", gpu_lib)
    g3.put_state(st)
    g3.cg_control(fixed=None, ite_max=1)
    with pytest.raises(WpicError) as e:
        g3.step(1)
    assert e.value.status == _lib.CG_NOT_CONVERGED
    # bad cumcnt is rejected at the boundary
    bad = st.copy()
    bad.cumcnt[-1, 0, 0] += 1  # last prefix sum no longer equals np2
    g4 = make_gpu(p, "fp64", gpu_lib)
    with pytest.raises(WpicError) as e:
        g4.put_state(bad)
    assert e.value.status == _lib.BAD_ARGUMENT
    # the context still works after an error
    g4.put_state(st)
    g4.step(1)


def test_device_loader_and_moderate_size_properties(gpu_lib):
    """A 128x128 plasma loaded on the device: particle count and ID set conserved,
    rows sorted by cell, cumcnt consistent, charge conserved to round-off."""
    from wumingpic_gb300.pic2d import Pic2D
    p = small_plasma(nx=128, ny=128, ppc=8, seed=99)
    g = Pic2D(p, precision="fp64")
    g.load_weibel()
    st0 = g.get_state()
    ids0 = np.sort(np.concatenate([a[5].view(np.int64) for a in valid(st0.up, st0.np2)]))
    assert len(ids0) == p.n_particles
    q, _ = p.charges()
    g.step(3)
    st = g.get_state()
    g.particle__solv()
    g.ele_cur()
    gp, _, _ = g.get_particles(1)
    res, scale = continuity_residual(p, q, st.up, gp, st.np2, g.get_uj())
    assert res <= 1e-12 * scale
    ids = np.sort(np.concatenate([a[5].view(np.int64) for a in valid(st.up, st.np2)]))
    np.testing.assert_array_equal(ids, ids0)
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            cell = st.up[0, :n, jj, isp].astype(int) - p.nxgs
            assert (np.diff(cell) >= 0).all()
            np.testing.assert_array_equal(st.cumcnt[:, jj, isp],
                                          np.concatenate([[0], np.cumsum(np.bincount(cell, minlength=p.nx))]))
            yj = np.floor(st.up[1, :n, jj, isp]).astype(int)
            assert (yj == p.nygs + jj).all()


def test_exact_step_matches_golden_fixture(gpu_lib):
    """One exact-build step from the golden fixture's initial state reproduces the
    fixture's particle state bit for bit (fields 1e-12, CG at the fixture's counts)."""
    import os
    from tests.golden.make_golden import CASE
    from wumingpic_gb300.loader import Plasma2D, State2D
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "weibel2d_small.npz"))
    p = Plasma2D(**CASE)
    st = State2D(up=np.asfortranarray(ref["up0"]), gp=np.asfortranarray(ref["up0"]).copy(order="F"),
                 uf=np.asfortranarray(ref["uf0"]), cumcnt=np.asfortranarray(ref["cumcnt0"]),
                 np2=np.asfortranarray(ref["np20"]))
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.cg_control(fixed=ref["cg1"])
    g.put_state(st)
    g.step(1)
    out = g.get_state()
    assert_particles(out.up, out.np2, ref["up1"], ref["np21"])
    np.testing.assert_array_equal(out.cumcnt, ref["cumcnt1"])
    assert_field(out.uf, ref["uf1"], REL)


# ---- moments: mom_calc__accl, mom_calc__nvt, bc__mom (2d/proj/weibel/app.f90:121-123) ----

def _valid_rows(a, np2, comps):
    for isp in range(a.shape[3]):
        for jj in range(a.shape[2]):
            yield a[comps, :np2[jj, isp], jj, isp]


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_mom_calc_accl_parity(gpu_lib, precision, rel):
    """The half-step push into gp: positions copied, momenta within the tolerance."""
    p, st = perturbed_case(seed=51, u_the=0.2)
    st.uf[:3] *= 40.0
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    g.mom_calc__accl()
    gp_gpu, np2, _ = g.get_particles(1)
    ref = st.copy()
    assert make_oracle(p).mom_calc_accl(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    np.testing.assert_array_equal(np2, ref.np2)
    for a, b in zip(_valid_rows(gp_gpu, np2, slice(0, 5)), _valid_rows(ref.gp, ref.np2, slice(0, 5))):
        if rel == 0.0:
            np.testing.assert_array_equal(a, b)
        else:
            np.testing.assert_allclose(a, b, rtol=0, atol=rel * max(np.abs(b).max(initial=0.0), 1e-300))


@pytest.mark.parametrize("bc", ["periodic", "reconnection"])
@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_moments_parity(gpu_lib, precision, rel, bc):
    """mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp) including the ghost nodes: bit-exact in the
    exact build (the node gather keeps the single-thread summation order), 1e-12 otherwise."""
    p, st = perturbed_case(seed=52, u_the=0.2, bc=bc)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    mom = g.moments()
    up_after, np2_after, _ = g.get_particles(0)
    rc, ref = make_oracle(p).moments(st.copy())
    assert rc == 0
    assert_field(mom, ref, rel)
    assert_particles(up_after, np2_after, st.up, st.np2)  # the state is not modified


def test_mom_calc_nvt_stages_and_source(gpu_lib):
    """The three stages called one by one, and mom_calc__nvt on up, match the oracle."""
    p, st = perturbed_case(seed=53, u_the=0.2)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    o = make_oracle(p)
    g.mom_calc__nvt(from_gp=False)
    a = g.get_mom()
    ref = np.zeros(o.mom_shape(), order="F")
    assert o.mom_calc_nvt(ref, st.up, st.np2) == 0
    np.testing.assert_array_equal(a, ref)
    g.bc__mom()
    assert o.bc_mom(ref) == 0
    np.testing.assert_array_equal(g.get_mom(), ref)


def test_mom_calc_nvt_on_pushed_and_displaced_particles(gpu_lib):
    """mom_calc__nvt only needs each particle's 2 x 2 node stencil to lie within the 3 x 3
    nodes around its bucket cell: gp straight after particle__solv (moved < 1/2 cell) gives
    the oracle's moments bit for bit; a particle displaced further is reported (out of
    range) instead of being dropped."""
    from wumingpic_gb300._lib import WpicError
    p, st = perturbed_case(seed=54, u_the=0.3)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.particle__solv()
    gp, np2, cc = g.get_particles(1)
    g.mom_calc__nvt(from_gp=True)
    o = make_oracle(p)
    ref = np.zeros(o.mom_shape(), order="F")
    assert o.mom_calc_nvt(ref, gp, np2) == 0
    np.testing.assert_array_equal(g.get_mom(), ref)
    k = cc[5, 1, 0]  # first particle of cell 5 in row 1
    gp[0, k, 1, 0] += 1.6
    g.put_particles(1, gp, np2)
    with pytest.raises(WpicError) as e:
        g.mom_calc__nvt(from_gp=True)
    assert e.value.status == _lib.OUT_OF_RANGE
    g.moments()  # the context stays usable


@pytest.mark.parametrize("bc", ["periodic", "reconnection"])
def test_moments_mixed_against_oracle(gpu_lib, bc):
    """Mixed path: FP32 half-step push and FP32 tile sums against the FP64 oracle run on the
    same (FP32-stored) particles: within 2e-5 of each moment's largest magnitude."""
    p, st = perturbed_case(seed=55, nx=32, ny=32, ppc=8, u_the=0.2, bc=bc)
    g = make_gpu(p, "mixed", gpu_lib)
    g.put_state(st)
    mom = g.moments()
    cur = g.get_state()
    cur.uf[...] = st.uf
    rc, ref = make_oracle(p).moments(cur)
    assert rc == 0
    for l in range(7):
        for isp in range(p.nsp):
            scale = np.abs(ref[l, :, :, isp]).max()
            np.testing.assert_allclose(mom[l, :, :, isp], ref[l, :, :, isp], rtol=0, atol=2e-5 * scale)
    after = g.get_state()
    np.testing.assert_array_equal(after.up, cur.up)


# ---- the shock boundary family (2d/proj/shock/boundary_shock.f90) on a window nxs..nxe ----

def shock_setup(seed, nx=24, ny=8, window=16, ppc=5, u0=0.3):
    p, st = small_case(nx=nx, ny=ny, ppc=ppc, seed=seed, bc="shock", window=window, u0=u0, u_the=0.1)
    rng = np.random.default_rng(seed)
    # small fields inside the window and its ghosts; the region beyond stays zero
    st.uf[:, :window + 4, :] = 0.02 * rng.standard_normal((6, window + 4, ny + 4))
    st.uf[:, :, :2] = st.uf[:, :, ny:ny + 2]
    st.uf[:, :, ny + 2:] = st.uf[:, :, 2:4]
    o = make_oracle(p)
    o.set_window(p.nxgs, p.nxe)
    o.u0 = p.u0
    return p, st, o


def assert_window_cumcnt(a, b, window):
    np.testing.assert_array_equal(a[:window + 1], b[:window + 1])


def test_shock_injection_parity(gpu_lib):
    p, st, o = shock_setup(91)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.particle__solv()
    g.bc__injection(p.u0)
    gp_gpu, np2, _ = g.get_particles(1)
    ref = st.copy()
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    assert o.bc_injection(ref.gp, ref.np2) == 0
    assert_particles(gp_gpu, np2, ref.gp, ref.np2)


def test_shock_one_step_exact(gpu_lib):
    """The shock driver's step (particle__solv, bc__injection, field__fdtd_i with the shock
    boundaries on the window, bc__particle_y, sort__bucket): particles bit-identical, cumcnt
    bit-identical inside the window, fields within 1e-12 at equal CG counts."""
    p, st, o = shock_setup(92)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.step(1)
    o.cg_control(fixed=g.cg_iters())
    ref = st.copy()
    assert o.step(ref) == 0
    out = g.get_state()
    assert_particles(out.up, out.np2, ref.up, ref.np2)
    assert_window_cumcnt(out.cumcnt, ref.cumcnt, p.window)
    assert_field(out.uf, ref.uf, REL)


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 1e-10), ("fp64", 1e-10)])
def test_shock_steps_with_expanding_window(gpu_lib, precision, rel):
    """Four steps, the window widened by one (empty) cell as relocate() does, three more
    steps.  relocate() keeps cumcnt of the new cell consistent (2d/proj/shock/app.f90:669);
    the oracle's copy is updated the same way, the library keeps it itself."""
    p, st, o = shock_setup(93)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    ref = st.copy()
    for k in range(7):
        if k == 4:
            g.set_window(p.nxgs, p.nxe + 1)
            o.set_window(p.nxgs, p.nxe + 1)
            ref.cumcnt[p.window + 1, :, :] = ref.cumcnt[p.window, :, :]
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    assert_window_cumcnt(out.cumcnt, ref.cumcnt, p.window + 1)
    assert_particles(out.up, out.np2, ref.up, ref.np2, rel=rel)
    assert_field(out.uf, ref.uf, rel)


def test_shock_rejected_where_unsupported(gpu_lib):
    from wumingpic_gb300._lib import WpicError
    p, st, o = shock_setup(94, nx=32, ny=16)
    g = make_gpu(p, "mixed", gpu_lib)  # the mixed path: only between a requested push and its field solve
    with pytest.raises(WpicError):
        g.bc__injection(p.u0)
    g.close()
    q, _ = small_case(nx=16, ny=12)
    g = make_gpu(q, "fp64", gpu_lib)
    with pytest.raises(WpicError):
        g.set_window(q.nxgs, q.nxge - 2)  # periodic: the window is the whole domain
    with pytest.raises(WpicError):
        g.bc__injection(0.1)


def test_shock_staged_calls_on_the_mixed_path(gpu_lib):
    """The shock driver's order (2d/proj/shock/app.f90:110-115) on a mixed context:
    particle__solv, boundary_shock__injection(u0), field__fdtd_i, particle_y, sort__bucket runs
    the fused mixed step with that u0, the same state bit for bit as wpic_set_injection(u0) and
    wpic_step."""
    p, st, o = shock_setup(95, nx=32, ny=16)
    g, h = make_gpu(p, "mixed", gpu_lib), make_gpu(p, "mixed", gpu_lib)
    for x in (g, h):
        x.put_state(st)
        x.set_injection(0.0)
    h.set_injection(p.u0)  # g receives p.u0 through its bc__injection calls only
    for _ in range(3):
        g.particle__solv()
        g.bc__injection(p.u0)
        g.field__fdtd_i()
        g.bc__particle_y()
        g.sort__bucket()
        h.step(1)
    a, b = g.get_state(), h.get_state()
    np.testing.assert_array_equal(a.np2, b.np2)
    np.testing.assert_array_equal(a.uf, b.uf)
    for isp in range(p.nsp):
        for j in range(p.ny):
            n = a.np2[j, isp]
            np.testing.assert_array_equal(a.up[:, :n, j, isp], b.up[:, :n, j, isp])
    g.close()
    h.close()
