"""GPU parity of the 3D FP64 path against the CPU oracle (oracle/oracle3d.cpp),
stage by stage and for whole steps, through the C ABI.

Tolerances (stated per test):
  * integer work (cell indices, np2, cumcnt, permutations, IDs): bit-exact;
  * FP64_EXACT build, push and deposit: bit-exact (same operations, same order);
  * FP64 (FMA) build: 1e-12 relative to the array's max magnitude;
  * fields after the CG solve: 1e-12 relative, with the oracle run at the GPU's CG
    iteration counts (reduction orders differ).
"""
import numpy as np
import pytest

from oracle.oracle import Oracle3D
from tests.helpers import small_case3d

pytestmark = pytest.mark.gpu

REL = 1e-12


def make_oracle(p):
    q, r = p.charges()
    return Oracle3D(nx=p.nx, ny=p.ny, nz=p.nz, np_cap=p.np_cap, q=q, r=r, delt=p.delt, delx=p.delx, c=p.c,
                    gfac=p.gfac, bc=getattr(p, "bc", "periodic"))


def make_gpu(p, precision, gpu_lib):
    from wumingpic_gb300.pic3d import Pic3D
    return Pic3D(p, precision=precision)


def rows(up, np2):
    for isp in range(up.shape[4]):
        for kk in range(up.shape[3]):
            for jj in range(up.shape[2]):
                yield up[:, :np2[jj, kk, isp], jj, kk, isp]


def assert_particles(a_up, a_np2, b_up, b_np2, rel=0.0):
    np.testing.assert_array_equal(a_np2, b_np2)
    for a, b in zip(rows(a_up, a_np2), rows(b_up, b_np2)):
        np.testing.assert_array_equal(a[6].view(np.int64), b[6].view(np.int64))
        if rel == 0.0:
            np.testing.assert_array_equal(a[:6], b[:6])
        else:
            for k in range(6):
                scale = max(np.abs(b[k]).max(initial=0.0), 1e-300)
                np.testing.assert_allclose(a[k], b[k], rtol=0, atol=rel * scale)


def assert_field(a, b, rel):
    scale = max(np.abs(b).max(), 1e-300)
    if rel == 0.0:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=0, atol=rel * scale)


def perturbed_case(seed=7, nx=8, ny=6, nz=5, ppc=4, **kw):
    kw.setdefault("u_the", 0.2)
    p, st = small_case3d(nx=nx, ny=ny, nz=nz, ppc=ppc, seed=seed, **kw)
    rng = np.random.default_rng(seed)
    core = 0.02 * rng.standard_normal((6, p.nx, p.ny, p.nz))
    st.uf[...] = np.pad(core, ((0, 0), (2, 2), (2, 2), (2, 2)), mode="wrap")
    return p, st


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_push_parity_3d(gpu_lib, precision, rel):
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
def test_push_vay_parity_3d(gpu_lib, precision, rel):
    """particle__solv_vay (3d/common/particle.f90:236) against the oracle's Vay update."""
    p, st = perturbed_case(seed=8, u_the=0.3)
    st.uf[:3] *= 40.0
    o = make_oracle(p)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    g.particle__solv_vay()
    gp_gpu, np2, _ = g.get_particles(1)
    ref = st.copy()
    assert o.particle_solv_vay(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    assert_particles(gp_gpu, np2, ref.gp, ref.np2, rel)


def test_one_step_vay_exact_is_bit_exact_on_particles_3d(gpu_lib):
    p, st = perturbed_case(seed=35, nx=8, ny=6, nz=5, ppc=4)
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


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_deposit_parity_3d(gpu_lib, precision, rel):
    """ele_cur + bc__curre: the exact build reproduces the single-thread reduction order bit for bit."""
    p, st = perturbed_case(seed=12)
    o = make_oracle(p)
    ref = st.copy()
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    uj_ref = np.zeros((3, p.nx + 4, p.ny + 4, p.nz + 4), order="F")
    assert o.ele_cur(uj_ref, ref.up, ref.gp, ref.cumcnt) == 0
    assert o.bc_curre(uj_ref) == 0
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(ref, gp=True)
    g.ele_cur()
    assert_field(g.get_uj(), uj_ref, rel)


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64"])
def test_field_fdtd_i_parity_3d(gpu_lib, precision):
    p, st = perturbed_case(seed=21)
    ref = st.copy()
    o = make_oracle(p)
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(ref, gp=True)
    g.field__fdtd_i()
    it_gpu = g.cg_iters()
    o2 = make_oracle(p)
    ref1 = ref.copy()
    assert o2.field_fdtd_i(ref1.uf, ref1.up, ref1.gp, ref1.cumcnt) == 0
    assert np.abs(it_gpu - o2.cg_iters()).max() <= 1
    o3 = make_oracle(p)
    o3.cg_control(fixed=it_gpu)
    ref2 = ref.copy()
    assert o3.field_fdtd_i(ref2.uf, ref2.up, ref2.gp, ref2.cumcnt) == 0
    assert_field(g.get_fields(), ref2.uf, REL)
    assert_field(g.get_df(), o3.get_df(), REL)


def test_particle_boundaries_and_sort_are_bit_exact_3d(gpu_lib):
    """bc__particle_x, bc__particle_yz (migration through the ghost-row buffers in the
    reference's order) and sort__bucket: permutations identical to the oracle."""
    p, st = perturbed_case(seed=5, nx=6, ny=5, nz=4, ppc=5)
    rng = np.random.default_rng(5)
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = st.np2[jj, kk, isp]
                st.gp[:, :n, jj, kk, isp] = st.up[:, :n, jj, kk, isp]
                for d in range(3):
                    st.gp[d, :n, jj, kk, isp] += rng.uniform(-0.9, 0.9, n)
    st.np2[2, 1, 0] -= 7  # uneven rows: both b < h and b > h occur
    st.np2[4, 3, 1] -= 3
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                cnt = np.bincount(st.up[0, :st.np2[jj, kk, isp], jj, kk, isp].astype(int) - p.nxgs, minlength=p.nx)
                st.cumcnt[:, jj, kk, isp] = np.concatenate([[0], np.cumsum(cnt)])
    o = make_oracle(p)
    g = make_gpu(p, "fp64", gpu_lib)
    g.put_state(st, gp=True)
    ref = st.copy()
    g.bc__particle_x()
    assert o.bc_particle_x(ref.gp, ref.np2) == 0
    b_gp, b_np2, _ = g.get_particles(1)
    assert_particles(b_gp, b_np2, ref.gp, ref.np2)
    g.bc__particle_yz()
    assert o.bc_particle_yz(ref.gp, ref.np2) == 0
    b_gp, b_np2, _ = g.get_particles(1)
    assert_particles(b_gp, b_np2, ref.gp, ref.np2)
    g.sort__bucket()
    assert o.sort_bucket(ref.up, ref.gp, ref.cumcnt, ref.np2) == 0
    a_up, a_np2, a_cc = g.get_particles(0)
    assert_particles(a_up, a_np2, ref.up, ref.np2)
    np.testing.assert_array_equal(a_cc, ref.cumcnt)


def test_one_step_exact_is_bit_exact_on_particles_3d(gpu_lib):
    p, st = perturbed_case(seed=31, nx=8, ny=6, nz=5, ppc=4)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.step(1)
    o = make_oracle(p)
    o.cg_control(fixed=g.cg_iters())
    ref = st.copy()
    assert o.step(ref) == 0
    out = g.get_state()
    assert_particles(out.up, out.np2, ref.up, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_field(out.uf, ref.uf, REL)


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64"])
def test_multistep_parity_3d(gpu_lib, precision):
    p, st = small_case3d(nx=8, ny=8, nz=6, ppc=4, seed=41, u_the=0.2, np_slack=3.0)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    o = make_oracle(p)
    ref = st.copy()
    for _ in range(6):
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_particles(out.up, out.np2, ref.up, ref.np2, rel=1e-10)
    assert_field(out.uf, ref.uf, 1e-10)
    np.testing.assert_allclose(g.energy(), o.energy(ref.up, ref.uf, ref.np2), rtol=1e-10)


def test_device_loader_3d(gpu_lib):
    """The device loader writes a sorted, in-cell, conserved plasma; a few steps conserve
    the particle count and keep the bookkeeping consistent."""
    from wumingpic_gb300.loader import Plasma3D
    p = Plasma3D(nx=16, ny=8, nz=8, ppc=6, drift=0.5, u_the=0.1, seed=99)
    g = make_gpu(p, "fp64", gpu_lib)
    g.load_weibel()
    assert g.num_particles() == p.n_particles
    st = g.get_state()
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = st.np2[jj, kk, isp]
                a = st.up[:, :n, jj, kk, isp]
                assert (np.floor(a[1]).astype(int) == p.nygs + jj).all()
                assert (np.floor(a[2]).astype(int) == p.nzgs + kk).all()
                cell = np.floor(a[0]).astype(int)
                assert (np.diff(cell) >= 0).all()
    g.step(3)
    assert g.num_particles() == p.n_particles
    e = g.energy()
    assert np.isfinite(e).all() and e[1] > 0


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_mom_calc_accl_parity_3d(gpu_lib, precision, rel):
    p, st = perturbed_case(seed=51, u_the=0.2)
    st.uf[:3] *= 40.0
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    g.mom_calc__accl()
    gp_gpu, np2, _ = g.get_particles(1)
    ref = st.copy()
    assert make_oracle(p).mom_calc_accl(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    np.testing.assert_array_equal(np2, ref.np2)
    for a, b in zip(rows(gp_gpu, np2), rows(ref.gp, ref.np2)):
        if rel == 0.0:
            np.testing.assert_array_equal(a[:6], b[:6])
        else:
            np.testing.assert_allclose(a[:6], b[:6], rtol=0, atol=rel * max(np.abs(b[:6]).max(initial=0.0), 1e-300))


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_moments_parity_3d(gpu_lib, precision, rel):
    p, st = perturbed_case(seed=52, u_the=0.2)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    mom = g.moments()
    rc, ref = make_oracle(p).moments(st.copy())
    assert rc == 0
    assert_field(mom, ref, rel)
    o = make_oracle(p)
    g.mom_calc__nvt(from_gp=False)
    g.bc__mom()
    ref2 = np.zeros(o.mom_shape(), order="F")
    assert o.mom_calc_nvt(ref2, st.up, st.np2) == 0 and o.bc_mom(ref2) == 0
    assert_field(g.get_mom(), ref2, rel)


# ---- conducting walls in x (3d/proj/reconnection/boundary_reconnection.f90) ----

def walls_case(seed, **kw):
    kw.setdefault("u_the", 0.3)
    return perturbed_case(seed=seed, nx=10, ny=6, nz=5, ppc=4, bc="reconnection", **kw)


def test_walls_steps_exact_3d(gpu_lib):
    """The reconnection driver's step in the exact build: one step bit-exact on particles
    (permutation, np2, cumcnt included), fields 1e-12; the next step 1e-12 (pushed by those
    fields); every particle between the walls."""
    p, st = walls_case(71)
    for steps, rel in ((1, 0.0), (2, 1e-12)):
        g = make_gpu(p, "fp64_exact", gpu_lib)
        g.put_state(st)
        o = make_oracle(p)
        ref = st.copy()
        for _ in range(steps):
            g.step(1)
            o.cg_control(fixed=g.cg_iters())
            assert o.step(ref) == 0
        out = g.get_state()
        assert_particles(out.up, out.np2, ref.up, ref.np2, rel)
        np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
        assert_field(out.uf, ref.uf, 1e-12)
        for a in rows(out.up, out.np2):
            assert a[0].min(initial=1e9) >= (p.nxgs + 1) * p.delx and a[0].max(initial=-1e9) < (p.nxge - 1) * p.delx
        g.close()


def test_walls_steps_fp64_3d(gpu_lib):
    p, st = walls_case(72)
    g = make_gpu(p, "fp64", gpu_lib)
    g.put_state(st)
    o = make_oracle(p)
    ref = st.copy()
    for _ in range(6):
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    assert_particles(out.up, out.np2, ref.up, ref.np2, rel=1e-10)
    assert_field(out.uf, ref.uf, 1e-10)
    g.close()


@pytest.mark.parametrize("precision,rel", [("fp64_exact", 0.0), ("fp64", REL)])
def test_walls_moments_3d(gpu_lib, precision, rel):
    p, st = walls_case(73)
    g = make_gpu(p, precision, gpu_lib)
    g.put_state(st)
    mom = g.moments()
    rc, ref = make_oracle(p).moments(st.copy())
    assert rc == 0
    assert_field(mom, ref, rel)
    g.close()



# ---- the shock boundary (3d/proj/shock/boundary_shock.f90) on a window nxs..nxe ----

def shock_case(seed, **kw):
    kw.setdefault("u_the", 0.1)
    p, st = perturbed_case(seed=seed, nx=12, ny=6, nz=5, ppc=4, bc="shock", window=9, u0=0.2, **kw)
    return p, st


def shock_oracle(p):
    o = make_oracle(p)
    o.set_window(p.nxgs, p.nxe)
    o.u0 = p.u0
    return o


def test_shock_injection_exact_3d(gpu_lib):
    """boundary_shock__injection on pushed particles: bit-exact against the oracle."""
    p, st = shock_case(81, u_the=0.4)
    g = make_gpu(p, "fp64_exact", gpu_lib)
    g.put_state(st)
    g.particle__solv()
    g.bc__injection(p.u0)
    gp, np2, _ = g.get_particles(1)
    o = shock_oracle(p)
    ref = st.copy()
    assert o.particle_solv(ref.gp, ref.up, ref.uf, ref.cumcnt) == 0
    assert o.bc_injection(ref.gp, ref.np2) == 0
    assert_particles(gp, np2, ref.gp, ref.np2)
    g.close()


def test_shock_steps_exact_3d(gpu_lib):
    p, st = shock_case(82)
    for steps, rel in ((1, 0.0), (2, 1e-12)):
        g = make_gpu(p, "fp64_exact", gpu_lib)
        g.put_state(st)
        o = shock_oracle(p)
        ref = st.copy()
        for _ in range(steps):
            g.step(1)
            o.cg_control(fixed=g.cg_iters())
            assert o.step(ref) == 0
        out = g.get_state()
        assert_particles(out.up, out.np2, ref.up, ref.np2, rel)
        # the reference's sort writes cumcnt(nxs:nxe+1) only; beyond the window its copy is stale
        np.testing.assert_array_equal(out.cumcnt[:p.window + 1], ref.cumcnt[:p.window + 1])
        assert_field(out.uf, ref.uf, 1e-12)
        g.close()


def test_shock_steps_with_expanding_window_3d(gpu_lib):
    """Three steps, the window widened by one (empty) cell as the driver's relocate() does
    (3d/proj/shock/app.f90:654), three more; the oracle's cumcnt of the new cell follows the
    row total as the driver keeps it."""
    p, st = shock_case(83)
    g = make_gpu(p, "fp64", gpu_lib)
    g.put_state(st)
    o = shock_oracle(p)
    ref = st.copy()
    for k in range(6):
        if k == 3:
            g.set_window(p.nxgs, p.nxe + 1)
            o.set_window(p.nxgs, p.nxe + 1)
            ref.cumcnt[p.window + 1, ...] = ref.cumcnt[p.window, ...]
        g.step(1)
        o.cg_control(fixed=g.cg_iters())
        assert o.step(ref) == 0
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, ref.np2)
    assert_particles(out.up, out.np2, ref.up, ref.np2, rel=1e-10)
    assert_field(out.uf, ref.uf, 1e-10)
    g.close()


def test_shock_injection_module_call_rejected_on_the_mixed_path_3d(gpu_lib):
    """The mixed path applies the shock boundary inside its fused step: bc__injection sets the
    step's u0 between a requested push and its field solve, and is refused anywhere else."""
    from wumingpic_gb300._lib import WpicError
    p, st = small_case3d(nx=16, ny=16, nz=8, ppc=2, seed=84, bc="shock", window=12, u0=0.1)
    g = make_gpu(p, "mixed", gpu_lib)
    with pytest.raises(WpicError):
        g.bc__injection(p.u0)
    g.close()
