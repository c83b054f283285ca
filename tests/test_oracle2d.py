"""CPU tests of the 2D oracle against physical invariants and against an
independent restatement of the migration bookkeeping.  The reference ships no
golden vectors for this path, so these invariants are what pins the oracle."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle2D
from tests.helpers import (closed_form_plan, continuity_residual, literal_moments2d, literal_particle_y, small_case,
                           small_plasma)
from wumingpic_gb300.loader import load_weibel2d


def make_oracle(p, **kw):
    q, r = p.charges()
    return Oracle2D(nx=p.nx, ny=p.ny, np_cap=p.np_cap, q=q, r=r, delt=p.delt, delx=p.delx, c=p.c,
                    gfac=p.gfac, bc=p.bc, **kw)


def test_charge_conservation_multistep():
    """Esirkepov deposition: (rho1 - rho0)/dt + div J = 0 to round-off every step."""
    p, st = small_case(nx=16, ny=12, ppc=8, seed=11)
    q, _ = p.charges()
    o = make_oracle(p)
    for _ in range(6):
        up0 = st.up.copy(order="F")
        assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
        assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
        res, scale = continuity_residual(p, q, up0, st.gp, st.np2, o.get_uj())
        assert res <= 1e-12 * scale
        assert o.bc_particle_x(st.gp, st.np2) == 0
        assert o.bc_particle_y(st.gp, st.np2) == 0
        assert o.sort_bucket(st.up, st.gp, st.cumcnt, st.np2) == 0
    assert st.np2.sum() == p.n_particles


def test_free_streaming_push_is_exact():
    """With zero fields the push leaves u unchanged and moves x by u dt / gamma."""
    p, st = small_case(seed=5)
    st.uf[...] = 0.0
    o = make_oracle(p)
    assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            u = st.up[2:5, :n, jj, isp]
            np.testing.assert_array_equal(st.gp[2:5, :n, jj, isp], u)
            gam = 1.0 / np.sqrt(1.0 + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / (p.c * p.c))
            np.testing.assert_array_equal(st.gp[0, :n, jj, isp], st.up[0, :n, jj, isp] + u[0] * p.delt * gam)
            np.testing.assert_array_equal(st.gp[1, :n, jj, isp], st.up[1, :n, jj, isp] + u[1] * p.delt * gam)
            np.testing.assert_array_equal(st.gp[5, :n, jj, isp].view(np.int64), st.up[5, :n, jj, isp].view(np.int64))


def test_gyration_in_uniform_bz():
    """Uniform Bz, no E: |u| is conserved and u turns by 2 atan(q B dt / (2 m gamma c))."""
    p, st = small_case(seed=9, u_the=0.2, u_thi=0.1)
    q, r = p.charges()
    bz = 0.3
    st.uf[...] = 0.0
    st.uf[2] = bz
    o = make_oracle(p)
    assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        n = st.np2[0, isp]
        u0 = st.up[2:5, :n, 0, isp]
        u1 = st.gp[2:5, :n, 0, isp]
        np.testing.assert_allclose(np.linalg.norm(u1, axis=0), np.linalg.norm(u0, axis=0), rtol=1e-14)
        gc = np.sqrt(p.c ** 2 + (u0 ** 2).sum(0))
        theta = 2 * np.arctan(q[isp] / r[isp] * 0.5 * p.delt * bz / gc)
        ang = np.arctan2(u0[0] * u1[1] - u0[1] * u1[0], u0[0] * u1[0] + u0[1] * u1[1])
        np.testing.assert_allclose(ang, -theta, rtol=1e-10, atol=1e-14)
        np.testing.assert_allclose(u1[2], u0[2], rtol=1e-15)


def test_cg_solves_the_implicit_system():
    """After field__fdtd_i the B increment satisfies (f4 - N) dB = f5 gkl to the CG tolerance."""
    p, st = small_case(nx=16, ny=16, ppc=8, seed=21)
    q, _ = p.charges()
    o = make_oracle(p)
    uf0 = st.uf.copy(order="F")
    assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
    assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
    uj = o.get_uj()
    df = o.get_df()
    f1 = p.c * p.delt / p.delx
    f2 = p.gfac * f1 * f1
    f3 = 4 * math.pi * p.delx / p.c
    f5 = (p.delx / (p.c * p.delt * p.gfac)) ** 2
    f4 = 4 + f5
    U = uf0[:, 2:-2, 2:-2]
    J = uj[:, 2:-2, 2:-2]

    def lap(a):
        return np.roll(a, 1, 0) + np.roll(a, -1, 0) + np.roll(a, 1, 1) + np.roll(a, -1, 1) - 4 * a

    def sm(a, ax):  # a(i-1) along axis (x = 0, y = 1)
        return np.roll(a, 1, ax)
    gkl = np.zeros((3,) + U.shape[1:])
    gkl[0] = f2 * (lap(U[0]) + f3 * (-sm(J[2], 1) + J[2])) - f1 * (-sm(U[5], 1) + U[5])
    gkl[1] = f2 * (lap(U[1]) - f3 * (-sm(J[2], 0) + J[2])) + f1 * (-sm(U[5], 0) + U[5])
    gkl[2] = f2 * (lap(U[2]) + f3 * (-sm(J[1], 0) + J[1] + sm(J[0], 1) - J[0])) - f1 * (-sm(U[4], 0) + U[4] + sm(U[3], 1) - U[3])
    for l in range(3):
        b = f5 * gkl[l]
        x = df[l, 2:-2, 2:-2]
        res = b - (f4 * x - (lap(x) + 4 * x))
        assert np.linalg.norm(res) <= 2e-6 * np.linalg.norm(b) + 1e-300
    assert (o.cg_iters() > 0).all()


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_particle_y_matches_literal_restatement(seed):
    """The oracle's migration equals an independent line-by-line Python restatement,
    and the closed-form plan the GPU uses gives the same post-migration order."""
    rng = np.random.default_rng(seed)
    p = small_plasma(nx=8, ny=5, ppc=4, seed=seed)
    st = load_weibel2d(p)
    # strong y displacements so that many particles move up or down, with wraps
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            shift = rng.choice([-0.75, 0.0, 0.0, 0.75], size=n) * rng.random(n)
            st.up[1, :n, jj, isp] = np.floor((st.up[1, :n, jj, isp] + shift) * 64) / 64  # dyadic: wraps exact
    # unequal row populations (b < h and b > h)
    st.np2[1, 0] -= 5
    st.np2[3, 1] -= 9
    o = make_oracle(p)
    a_up, a_np2 = st.up.copy(order="F"), st.np2.copy(order="F")
    assert o.bc_particle_y(a_up, a_np2) == 0
    b_up, b_np2 = literal_particle_y(st.up.copy(order="F"), st.np2.copy(order="F"), p.nygs, p.nyge, p.nygs,
                                     p.nyge, p.delx, p.ndim, p.np_cap)
    np.testing.assert_array_equal(a_np2, b_np2)
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = a_np2[jj, isp]
            np.testing.assert_array_equal(a_up[:, :n, jj, isp], b_up[:, :n, jj, isp])
    # closed form
    for isp in range(p.nsp):
        dirs = []
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            jpos = np.floor(st.up[1, :n, jj, isp] / p.delx).astype(int)
            j = p.nygs + jj
            dirs.append(np.where(jpos == j, 0, np.where(jpos == j + 1, 1, 2)))
        plan = closed_form_plan(dirs, p.ny)
        for jj in range(p.ny):
            assert len(plan[jj]) == a_np2[jj, isp]
            for t, (sr, ss) in enumerate(plan[jj]):
                np.testing.assert_array_equal(a_up[[0, 2, 3, 4, 5], t, jj, isp],
                                              st.up[[0, 2, 3, 4, 5], ss, sr, isp])


def test_sort_is_stable_counting_sort():
    p, st = small_case(nx=8, ny=4, ppc=5, seed=8)
    rng = np.random.default_rng(0)
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            st.gp[:, :n, jj, isp] = st.up[:, rng.permutation(n), jj, isp]
    o = make_oracle(p)
    out = np.zeros_like(st.up, order="F")
    cc = np.zeros_like(st.cumcnt, order="F")
    assert o.sort_bucket(out, st.gp, cc, st.np2) == 0
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            cell = st.gp[0, :n, jj, isp].astype(int)
            order = np.argsort(cell, kind="stable")
            np.testing.assert_array_equal(out[:, :n, jj, isp], st.gp[:, order, jj, isp])
            counts = np.bincount(cell - p.nxgs, minlength=p.nx)
            np.testing.assert_array_equal(cc[:, jj, isp], np.concatenate([[0], np.cumsum(counts)]))


def test_energy_sums():
    p, st = small_case(seed=4)
    q, r = p.charges()
    st.uf[...] = np.random.default_rng(1).standard_normal(st.uf.shape)
    o = make_oracle(p)
    e = o.energy(st.up, st.uf, st.np2)
    for isp in range(p.nsp):
        u = st.up[2:5, :st.np2[0, isp], :, isp]
        g = np.sqrt(1 + (u ** 2).sum(0) / p.c ** 2)
        assert e[isp] == pytest.approx(r[isp] * (g - 1).sum(), rel=1e-13)
    U = st.uf[:, 2:-2, 2:-2]
    assert e[2] == pytest.approx((U[3:] ** 2).sum() / (8 * math.pi), rel=1e-13)
    assert e[3] == pytest.approx((U[:3] ** 2).sum() / (8 * math.pi), rel=1e-13)


def test_threads_do_not_change_push_and_fields():
    """Multi-threaded oracle (CPU baseline mode) keeps push bit-identical; fields agree to round-off."""
    p, st = small_case(nx=16, ny=16, ppc=6, seed=13)
    a, b = st.copy(), st.copy()
    o1, o4 = make_oracle(p, threads=1), make_oracle(p, threads=4)
    for o, s in ((o1, a), (o4, b)):
        assert o.step(s) == 0
    np.testing.assert_array_equal(a.np2, b.np2)
    np.testing.assert_allclose(a.uf, b.uf, rtol=0, atol=1e-12 * np.abs(a.uf).max())


def test_reconnection_walls_reflect():
    p = small_plasma(nx=12, ny=8, ppc=4, seed=2, bc="reconnection")
    st = load_weibel2d(p)
    o = make_oracle(p)
    # put a few particles beyond the walls
    st.gp[...] = st.up
    n = st.np2[0, 0]
    st.gp[0, 0, 0, 0] = p.nxgs + 0.25           # ipos = nxs < nxs+1 -> reflected about nxs+1
    st.gp[0, n - 1, 0, 0] = p.nxge + 0.5         # ipos = nxe >= nxe-1 -> reflected about nxe-1
    u0 = st.gp[2:5, [0, n - 1], 0, 0].copy()
    assert o.bc_particle_x(st.gp, st.np2) == 0
    assert st.gp[0, 0, 0, 0] == 2 * (p.nxgs + 1) - (p.nxgs + 0.25)
    assert st.gp[0, n - 1, 0, 0] == 2 * (p.nxge - 1) - (p.nxge + 0.5)
    np.testing.assert_array_equal(st.gp[2:5, [0, n - 1], 0, 0], -u0)


def _uniform_fields(uf, b, e):
    uf[...] = 0.0
    for k in range(3):
        uf[k] = b[k]
        uf[3 + k] = e[k]


def test_vay_conserves_momentum_magnitude_in_pure_b():
    """particle__solv_vay with E = 0: gamma' solves the quadratic exactly at gamma, so
    |u| is conserved for any direction of B (not only u perpendicular to B)."""
    p, st = small_case(seed=13, u_the=0.3, u_thi=0.2)
    _uniform_fields(st.uf, (0.2, -0.1, 0.35), (0.0, 0.0, 0.0))
    o = make_oracle(p)
    assert o.particle_solv_vay(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            u0 = st.up[2:5, :n, jj, isp]
            u1 = st.gp[2:5, :n, jj, isp]
            np.testing.assert_allclose(np.linalg.norm(u1, axis=0), np.linalg.norm(u0, axis=0), rtol=1e-13)
            np.testing.assert_array_equal(st.gp[5, :n, jj, isp].view(np.int64),
                                          st.up[5, :n, jj, isp].view(np.int64))


def test_vay_equals_boris_in_pure_e():
    """With B = 0 both pushes reduce to u += (q/m) dt E and x += u dt / gamma."""
    p, st = small_case(seed=17, u_the=0.3)
    _uniform_fields(st.uf, (0.0, 0.0, 0.0), (0.05, -0.02, 0.03))
    o = make_oracle(p)
    gb = st.gp.copy(order="F")
    assert o.particle_solv(gb, st.up, st.uf, st.cumcnt) == 0
    assert o.particle_solv_vay(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            np.testing.assert_allclose(st.gp[:5, :n, jj, isp], gb[:5, :n, jj, isp], rtol=1e-13, atol=1e-15)


def test_vay_keeps_relativistic_exb_drift_force_free():
    """E = -v x B / c for a particle at gamma ~ 5: the Lorentz force vanishes, and the Vay
    push leaves u unchanged to round-off; the Boris push does not (the defect the Vay
    scheme removes)."""
    p, st = small_case(seed=19)
    q, r = p.charges()
    ux = 5.0 * p.c
    bz = 0.2 / abs(q[1] / r[1] * 0.5 * p.delt)  # electrons turn by ~0.4 rad / gamma per step
    vx = ux / math.sqrt(1.0 + (ux / p.c) ** 2)
    _uniform_fields(st.uf, (0.0, 0.0, bz), (0.0, vx * bz / p.c, 0.0))
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            st.up[2, :n, jj, isp] = ux
            st.up[3:5, :n, jj, isp] = 0.0
    o = make_oracle(p)
    gb = st.gp.copy(order="F")
    assert o.particle_solv(gb, st.up, st.uf, st.cumcnt) == 0
    assert o.particle_solv_vay(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        n = st.np2[0, isp]
        np.testing.assert_allclose(st.gp[2, :n, 0, isp], ux, rtol=1e-12)
        np.testing.assert_allclose(st.gp[3:5, :n, 0, isp], 0.0, atol=1e-12 * ux)
    n = st.np2[0, 1]
    assert np.abs(gb[2:5, :n, 0, 1] - st.up[2:5, :n, 0, 1]).max() > 1e-5 * ux


@pytest.mark.parametrize("bc", ["periodic", "reconnection"])
def test_moments_match_numpy_restatement(bc):
    """mom_calc__accl -> mom_calc__nvt -> bc__mom (2d/proj/weibel/app.f90:121-123) against an
    independent numpy restatement of the deposit and the ghost folds."""
    p, st = small_case(seed=23, u_the=0.2, bc=bc)
    rng = np.random.default_rng(23)
    st.uf[...] = 0.02 * rng.standard_normal(st.uf.shape)
    o = make_oracle(p)
    rc, mom = o.moments(st)
    assert rc == 0
    ref = literal_moments2d(p, st.gp, st.np2, bc=bc)
    scale = np.abs(ref).max(axis=(1, 2, 3), keepdims=True)
    np.testing.assert_allclose(mom, ref, rtol=0, atol=1e-13 * scale.max())
    # particle number: the linear weights of each particle sum to one over the interior nodes
    for isp in range(p.nsp):
        n = mom[0, 1:p.nx + 1, 1:p.ny + 1, isp].sum()
        if bc == "periodic":
            np.testing.assert_allclose(n, st.np2[:, isp].sum(), rtol=1e-12)


def test_mom_calc_accl_is_a_half_step_in_pure_e():
    """With B = 0 the half-step push gives u + (q/m)(dt/2) E and leaves the positions."""
    p, st = small_case(seed=29, u_the=0.2)
    q, r = p.charges()
    e = (0.05, -0.02, 0.03)
    _uniform_fields(st.uf, (0.0, 0.0, 0.0), e)
    o = make_oracle(p)
    assert o.mom_calc_accl(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            np.testing.assert_array_equal(st.gp[0:2, :n, jj, isp], st.up[0:2, :n, jj, isp])
            for k in range(3):
                np.testing.assert_allclose(st.gp[2 + k, :n, jj, isp],
                                           st.up[2 + k, :n, jj, isp] + q[isp] / r[isp] * 0.5 * p.delt * e[k],
                                           rtol=1e-13, atol=1e-16)


def shock_oracle(p, window_cells):
    o = make_oracle(p)
    o.set_window(p.nxgs, p.nxgs + window_cells - 1)
    o.u0 = p.u0
    return o


def test_shock_injection_reflects_at_both_ends():
    """boundary_shock__injection: x below the wall (nxs+1) dx is mirrored with u reversed;
    x beyond xend = nxe dx + v0 dt is mirrored about xend with u_x -> 2 u0 - u_x."""
    p, st = small_case(nx=24, ny=8, ppc=4, seed=81, bc="shock", window=16, u0=0.3)
    o = shock_oracle(p, 16)
    nxs, nxe = p.nxgs, p.nxgs + 15
    xend = nxe * p.delx + p.u0 / math.sqrt(1 + p.u0 ** 2 / p.c ** 2) * p.delt
    gp = st.up.copy(order="F")
    n = st.np2[0, 1]
    gp[0, 0, 0, 1] = (nxs + 1) * p.delx - 0.25          # behind the wall
    gp[0, 1, 0, 1] = xend + 0.1                          # beyond the injection boundary
    u_before = gp[2:5, :n, 0, 1].copy()
    assert o.bc_injection(gp, st.np2) == 0
    assert gp[0, 0, 0, 1] == (nxs + 1) * p.delx + 0.25
    np.testing.assert_array_equal(gp[2:5, 0, 0, 1], -u_before[:, 0])
    np.testing.assert_allclose(gp[0, 1, 0, 1], xend - 0.1, rtol=0, atol=1e-12)
    assert gp[2, 1, 0, 1] == 2 * p.u0 - u_before[0, 1]
    np.testing.assert_array_equal(gp[3:5, 1, 0, 1], -u_before[1:, 1])
    np.testing.assert_array_equal(gp[:, 2:n, 0, 1], st.up[:, 2:n, 0, 1])


def test_shock_steps_stay_in_the_window():
    """Five steps of the shock boundary in a 16-cell window of a 24-cell domain: particles stay
    between the wall and the injection boundary, the count is conserved, the fields outside
    the window (and its two ghost columns) are untouched, and the CG converges."""
    p, st = small_case(nx=24, ny=8, ppc=4, seed=82, bc="shock", window=16, u0=0.3, u_the=0.1)
    o = shock_oracle(p, 16)
    uf0 = st.uf.copy()
    n_before = st.np2.sum()
    nxe = p.nxgs + 15
    for _ in range(5):
        assert o.step(st) == 0
    assert st.np2.sum() == n_before
    xend = nxe * p.delx + p.u0 / math.sqrt(1 + p.u0 ** 2 / p.c ** 2) * p.delt
    for isp in range(p.nsp):
        for j in range(p.ny):
            x = st.up[0, :st.np2[j, isp], j, isp]
            assert np.all(x >= (p.nxgs + 1) * p.delx) and np.all(x <= xend)
    # field columns beyond nxe+2 (array index nxe+2 - (nxgs-2) + 1 ...) are never written
    first_untouched = nxe + 3 - (p.nxgs - 2)
    np.testing.assert_array_equal(st.uf[:, first_untouched:, :], uf0[:, first_untouched:, :])
    assert np.abs(st.uf[:, :first_untouched, :]).max() > 0
    assert all(0 < k < 100 for k in o.cg_iters())
