"""The mixed-precision 3D path (FP32 push and deposit on split positions, FP64 fields and
bookkeeping) against the FP64 3D path as the oracle.

Tolerances (stated per test):
  * one step from the same state: positions within 1e-5 cell, momenta within 1e-5 of the
    largest |u|, current within 1e-5 of the largest |J| (FP32 arithmetic);
  * charge conservation |(rho1 - rho0) dx/dt + div J| <= 1e-6 of max |rho1 - rho0| dx/dt;
  * twenty steps of a Weibel plasma: total energy and field energy within 1e-3 relative,
    the particle bookkeeping (np2 totals) exact.
"""
import numpy as np
import pytest

from tests.helpers import rho3d, small_case3d

pytestmark = pytest.mark.gpu


def make(p, precision):
    from wumingpic_gb300.pic3d import Pic3D
    return Pic3D(p, precision=precision)


def by_id(st):
    """(species, id) -> (x, y, z, ux, uy, uz, id) over the valid slots.  The ids count within a
    species (ions and electrons share them), and the two paths order a row's particles
    differently (cell columns against the bucket sort), so rows are matched by species and id."""
    rows, sp = [], []
    for isp in range(st.np2.shape[2]):
        for k in range(st.np2.shape[1]):
            for j in range(st.np2.shape[0]):
                n = st.np2[j, k, isp]
                a = st.up[:, :n, j, k, isp]
                rows.append(np.vstack([a[:6], a[6].view(np.int64)[None, :].astype(np.float64)]))
                sp.append(np.full(n, isp))
    a = np.concatenate(rows, axis=1)
    order = np.lexsort((a[6], np.concatenate(sp)))
    return a[:, order]


def perturbed(seed, nx=16, ny=16, nz=8, ppc=6):
    p, st = small_case3d(nx=nx, ny=ny, nz=nz, ppc=ppc, seed=seed, u_the=0.2, np_slack=3.0)
    rng = np.random.default_rng(seed)
    core = 0.02 * rng.standard_normal((6, p.nx, p.ny, p.nz))
    st.uf[...] = np.pad(core, ((0, 0), (2, 2), (2, 2), (2, 2)), mode="wrap")
    return p, st


@pytest.mark.parametrize("pusher", ["boris", "vay"])
def test_mixed3d_one_step_against_fp64(gpu_lib, pusher):
    p, st = perturbed(71)
    m = make(p, "mixed")
    m.set_pusher(pusher)
    m.put_state(st)
    m.step(1)
    f = make(p, "fp64")
    f.set_pusher(pusher)
    f.put_state(st)
    f.step(1)
    sm, sf = m.get_state(), f.get_state()
    assert sm.np2.sum() == sf.np2.sum()
    a, b = by_id(sm), by_id(sf)
    np.testing.assert_array_equal(a[6], b[6])
    np.testing.assert_allclose(a[:3], b[:3], rtol=0, atol=1e-5 * p.delx)
    umax = np.abs(b[3:6]).max()
    np.testing.assert_allclose(a[3:6], b[3:6], rtol=0, atol=1e-5 * umax)
    jm, jf = m.get_uj(), f.get_uj()
    np.testing.assert_allclose(jm, jf, rtol=0, atol=1e-5 * np.abs(jf).max())


def test_mixed3d_charge_conservation(gpu_lib):
    """Second step (positions already split-representable): the FP32 Esirkepov current
    satisfies continuity against the FP64 charge density of the stored positions."""
    p, st = perturbed(72)
    q, _ = p.charges()
    m = make(p, "mixed")
    m.put_state(st)
    m.step(1)
    s0 = m.get_state()
    m.step(1)
    s1 = m.get_state()
    r0 = rho3d(p, s0.up, s0.np2, q)
    r1 = rho3d(p, s1.up, s1.np2, q)
    J = m.get_uj()[:, 2:-2, 2:-2, 2:-2]
    res = (r1 - r0) * p.delx / p.delt
    for d in range(3):
        res = res + (np.roll(J[d], -1, d) - J[d])
    scale = np.abs(r1 - r0).max() * p.delx / p.delt
    assert np.abs(res).max() <= 1e-6 * scale


def test_mixed3d_weibel_steps_track_fp64(gpu_lib):
    from wumingpic_gb300.loader import Plasma3D
    p = Plasma3D(nx=16, ny=16, nz=16, ppc=8, drift=0.5, u_the=0.05, seed=73, np_slack=2.0)
    m, f = make(p, "mixed"), make(p, "fp64")
    m.load_weibel()
    f.load_weibel()
    for _ in range(20):
        m.step(1)
        f.step(1)
    assert m.num_particles() == f.num_particles() == p.n_particles
    em, ef = m.energy(), f.energy()
    np.testing.assert_allclose(em.sum(), ef.sum(), rtol=1e-3)
    np.testing.assert_allclose(em[-2:], ef[-2:], rtol=1e-3, atol=1e-6 * ef.sum())


def walls_perturbed(seed):
    """The reconnection driver's walls in x (particles loaded between them), hot enough that
    particles reach the walls within a few steps, perturbed fields."""
    p, st = small_case3d(nx=16, ny=16, nz=8, ppc=6, seed=seed, u_the=0.3, np_slack=3.0, bc="reconnection")
    rng = np.random.default_rng(seed)
    core = 0.02 * rng.standard_normal((6, p.nx, p.ny, p.nz))
    st.uf[...] = np.pad(core, ((0, 0), (2, 2), (2, 2), (2, 2)), mode="wrap")
    return p, st


def between_walls(p, st):
    a = by_id(st)
    return a[0].min() >= (p.nxgs + 1) * p.delx and a[0].max() < (p.nxge - 1) * p.delx


def test_mixed3d_walls_one_step_against_fp64(gpu_lib):
    """Walls on the mixed 3D path: the reflection inside the fused push, before the deposit,
    as the reconnection driver orders particle_x; one step against the FP64 walls path."""
    p, st = walls_perturbed(76)
    m = make(p, "mixed")
    m.put_state(st)
    m.step(1)
    f = make(p, "fp64")
    f.put_state(st)
    f.step(1)
    sm, sf = m.get_state(), f.get_state()
    assert sm.np2.sum() == sf.np2.sum() == st.np2.sum()
    a, b = by_id(sm), by_id(sf)
    np.testing.assert_array_equal(a[6], b[6])
    np.testing.assert_allclose(a[:3], b[:3], rtol=0, atol=1e-5 * p.delx)
    umax = np.abs(b[3:6]).max()
    np.testing.assert_allclose(a[3:6], b[3:6], rtol=0, atol=1e-5 * umax)
    jm, jf = m.get_uj(), f.get_uj()
    np.testing.assert_allclose(jm, jf, rtol=0, atol=1e-5 * np.abs(jf).max())
    assert between_walls(p, sm)


def test_mixed3d_walls_steps_track_fp64(gpu_lib):
    p, st = walls_perturbed(77)
    m, f = make(p, "mixed"), make(p, "fp64")
    m.put_state(st)
    f.put_state(st)
    for _ in range(10):
        m.step(1)
        f.step(1)
    assert m.num_particles() == f.num_particles() == st.np2.sum()
    em, ef = m.energy(), f.energy()
    np.testing.assert_allclose(em.sum(), ef.sum(), rtol=1e-4)
    np.testing.assert_allclose(em, ef, rtol=1e-3, atol=1e-6 * ef.sum())
    assert between_walls(p, m.get_state())


def shock_perturbed(seed):
    """The shock driver's window (12 of 16 cells) with its injection boundary, u0 = 0.2."""
    p, st = small_case3d(nx=16, ny=8, nz=8, ppc=6, seed=seed, u_the=0.1, np_slack=3.0, bc="shock",
                         window=12, u0=0.2)
    rng = np.random.default_rng(seed)
    core = 0.02 * rng.standard_normal((6, p.nx, p.ny, p.nz))
    st.uf[...] = np.pad(core, ((0, 0), (2, 2), (2, 2), (2, 2)), mode="wrap")
    return p, st


@pytest.mark.parametrize("nsteps", [1, 6])
def test_mixed3d_shock_against_fp64(gpu_lib, nsteps):
    """The shock boundary on the mixed 3D path: the wall reflection and the injection
    boundary inside the fused push, before the deposit, as the shock driver orders them;
    particles within 1e-5 (one step) / 1e-4 (six steps) of the FP64 shock path."""
    p, st = shock_perturbed(78)
    m, f = make(p, "mixed"), make(p, "fp64")
    m.put_state(st)
    f.put_state(st)
    m.step(nsteps)
    f.step(nsteps)
    sm, sf = m.get_state(), f.get_state()
    assert sm.np2.sum() == sf.np2.sum() == st.np2.sum()
    a, b = by_id(sm), by_id(sf)
    np.testing.assert_array_equal(a[6], b[6])
    tol = 1e-5 if nsteps == 1 else 1e-4
    np.testing.assert_allclose(a[:3], b[:3], rtol=0, atol=tol * p.delx)
    umax = np.abs(b[3:6]).max()
    np.testing.assert_allclose(a[3:6], b[3:6], rtol=0, atol=tol * umax)
    assert a[0].min() >= (p.nxgs + 1) * p.delx and a[0].max() <= (p.nxgs + p.window) * p.delx + p.delx
    em, ef = m.energy(), f.energy()
    np.testing.assert_allclose(em, ef, rtol=1e-3, atol=1e-6 * ef.sum())


def test_mixed3d_rejects_out_of_order_staged_calls_and_odd_tiles(gpu_lib):
    """A field solve without its push, a second push, and particle_yz or sort__bucket between
    the push and the field solve are refused; so is a grid that is not a whole number of tiles."""
    from wumingpic_gb300._lib import WpicError
    p, st = perturbed(74)
    m = make(p, "mixed")
    m.put_state(st)
    with pytest.raises(WpicError):
        m.field__fdtd_i()
    m.particle__solv()
    for call in (m.particle__solv, m.bc__particle_yz, m.sort__bucket, lambda: m.step(1)):
        with pytest.raises(WpicError):
            call()
    m.field__fdtd_i()
    m.step(1)
    m.close()
    p2, _ = small_case3d(nx=12, ny=16, nz=8, ppc=2, seed=75)
    with pytest.raises(WpicError):
        make(p2, "mixed")


def test_mixed3d_moments_against_oracle(gpu_lib):
    """FP32 half-step push and FP32 node sums against the FP64 oracle on the same state:
    within 2e-5 of each moment's largest magnitude; the state is not modified."""
    from oracle.oracle import Oracle3D
    p, st = perturbed(76)
    m = make(p, "mixed")
    m.put_state(st)
    m.step(1)
    cur = m.get_state()
    mom = m.moments()
    q, r = p.charges()
    o = Oracle3D(nx=p.nx, ny=p.ny, nz=p.nz, np_cap=p.np_cap, q=q, r=r, delt=p.delt, delx=p.delx, c=p.c,
                 gfac=p.gfac)
    rc, ref = o.moments(cur.copy())
    assert rc == 0
    for l in range(7):
        for isp in range(p.nsp):
            scale = np.abs(ref[l, ..., isp]).max()
            np.testing.assert_allclose(mom[l, ..., isp], ref[l, ..., isp], rtol=0, atol=2e-5 * scale)
    after = m.get_state()
    np.testing.assert_array_equal(after.up, cur.up)


def test_mixed3d_shock_expanding_window_against_fp64(gpu_lib):
    """The window widened by one cell after three steps on a mixed 3D context, as the shock
    driver's relocate() does (3d/proj/shock/app.f90:654); six steps within 1e-4 of the FP64
    shock path with the same widening, energies within 1e-3."""
    p, st = shock_perturbed(80)
    m, f = make(p, "mixed"), make(p, "fp64")
    m.put_state(st)
    f.put_state(st)
    nxe = p.nxe
    for it in range(6):
        if it == 3:
            nxe += 1
            m.set_window(p.nxgs, nxe)
            f.set_window(p.nxgs, nxe)
        m.step(1)
        f.step(1)
    sm, sf = m.get_state(), f.get_state()
    assert sm.np2.sum() == sf.np2.sum() == st.np2.sum()
    a, b = by_id(sm), by_id(sf)
    np.testing.assert_array_equal(a[6], b[6])
    np.testing.assert_allclose(a[:3], b[:3], rtol=0, atol=1e-4 * p.delx)
    umax = np.abs(b[3:6]).max()
    np.testing.assert_allclose(a[3:6], b[3:6], rtol=0, atol=1e-4 * umax)
    assert a[0].min() >= (p.nxgs + 1) * p.delx and a[0].max() <= (nxe + 1) * p.delx
    em, ef = m.energy(), f.energy()
    np.testing.assert_allclose(em, ef, rtol=1e-3, atol=1e-6 * ef.sum())


def test_mixed3d_staged_calls_run_the_fused_step(gpu_lib):
    """The 3D Weibel driver's call order (3d/proj/weibel/app.f90:103-108) on a mixed context:
    particle__solv requests the push, field__fdtd_i runs the fused mixed step, particle_x,
    particle_yz and sort__bucket find their work done.  Three steps equal wpic3d_step bit for
    bit; the diagnostic block's calls give the mixed moments (1e-6 of each moment's largest
    value: FP32 shared-memory sums whose order varies)."""
    p, st = perturbed(74)
    g, h = make(p, "mixed"), make(p, "mixed")
    g.put_state(st)
    h.put_state(st)
    for _ in range(3):
        g.particle__solv()
        g.field__fdtd_i()
        g.bc__particle_x()
        g.bc__particle_yz()
        g.sort__bucket()
        h.step(1)
    a, b = g.get_state(), h.get_state()
    np.testing.assert_array_equal(a.np2, b.np2)
    np.testing.assert_array_equal(a.uf, b.uf)
    np.testing.assert_array_equal(by_id(a), by_id(b))
    g.mom_calc__accl()
    g.mom_calc__nvt()
    g.bc__mom()
    mg, mh = g.get_mom(), h.moments()
    for q in range(7):
        np.testing.assert_allclose(mg[q], mh[q], rtol=0, atol=1e-6 * np.abs(mh[q]).max())
    g.close()
    h.close()


def test_mixed3d_put_unsorted_rows_sorts_them(gpu_lib):
    """The 3D restart path on a mixed context: put with which = 1 takes rows in no particular
    order within the row, sorts them by x cell on the host and stores the sorted state: the same
    cumcnt, np2 and particles as a put of the sorted rows, and after two steps the same fields to
    1e-6 of their largest value (the order within a cell changes the FP32 register sums)."""
    p, st = perturbed(78)
    rng = np.random.default_rng(78)
    up = np.array(st.up, order="F", copy=True)
    for isp in range(st.np2.shape[2]):
        for k in range(st.np2.shape[1]):
            for j in range(st.np2.shape[0]):
                n = st.np2[j, k, isp]
                up[:, :n, j, k, isp] = up[:, rng.permutation(n), j, k, isp]
    a, b = make(p, "mixed"), make(p, "mixed")
    a.put_state(st)
    b.put_particles(1, up, st.np2)
    b.put_fields(st.uf)
    sa, sb = a.get_state(), b.get_state()
    np.testing.assert_array_equal(sb.np2, sa.np2)
    np.testing.assert_array_equal(sb.cumcnt, sa.cumcnt)
    np.testing.assert_array_equal(by_id(sb), by_id(sa))
    a.step(2)
    b.step(2)
    fa, fb = a.get_fields(), b.get_fields()
    np.testing.assert_allclose(fb, fa, rtol=0, atol=1e-6 * np.abs(fa).max())
    a.close()
    b.close()
