"""CPU tests of the 3D oracle (oracle/oracle3d.cpp) against physical invariants and
against an independent restatement of the 3D migration.  The reference ships no
golden vectors for this path, so these invariants are what pins the oracle."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle3D
from tests.helpers import continuity_residual3d, literal_moments3d, literal_particle_yz, small_case3d


def make_oracle3d(p, **kw):
    q, r = p.charges()
    return Oracle3D(nx=p.nx, ny=p.ny, nz=p.nz, np_cap=p.np_cap, q=q, r=r, delt=p.delt, delx=p.delx, c=p.c,
                    gfac=p.gfac, **kw)


def test_charge_conservation_multistep_3d():
    """Esirkepov deposition in 3D: (rho1 - rho0)/dt + div J = 0 to round-off every step."""
    p, st = small_case3d(nx=6, ny=5, nz=4, ppc=4, seed=11, u_the=0.2)
    q, _ = p.charges()
    o = make_oracle3d(p)
    for _ in range(4):
        up0 = st.up.copy(order="F")
        assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
        assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
        res, scale = continuity_residual3d(p, q, up0, st.gp, st.np2, o.get_uj())
        assert res <= 1e-12 * scale, (res, scale)
        assert o.bc_particle_x(st.gp, st.np2) == 0
        assert o.bc_particle_yz(st.gp, st.np2) == 0
        assert o.sort_bucket(st.up, st.gp, st.cumcnt, st.np2) == 0
    assert st.np2.sum() == p.n_particles


def test_free_streaming_push_is_exact_3d():
    p, st = small_case3d(seed=5)
    st.uf[...] = 0.0
    o = make_oracle3d(p)
    assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
    n = st.np2[0, 0, 1]
    u = st.up[3:6, :n, 0, 0, 1]
    np.testing.assert_array_equal(st.gp[3:6, :n, 0, 0, 1], u)
    gam = 1.0 / np.sqrt(1.0 + (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / (p.c * p.c))
    for d in range(3):
        np.testing.assert_array_equal(st.gp[d, :n, 0, 0, 1], st.up[d, :n, 0, 0, 1] + u[d] * p.delt * gam)
    np.testing.assert_array_equal(st.gp[6].view(np.int64), st.up[6].view(np.int64))


def test_gyration_in_uniform_bx_3d():
    """Uniform Bx, no E: |u| conserved, rotation by 2 atan(q B dt / (2 m gamma c)) about x."""
    p, st = small_case3d(seed=9, u_the=0.2, u_thi=0.1)
    q, r = p.charges()
    bx = 0.3
    st.uf[...] = 0.0
    st.uf[0] = bx
    o = make_oracle3d(p)
    assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        n = st.np2[0, 0, isp]
        u0 = st.up[3:6, :n, 0, 0, isp]
        u1 = st.gp[3:6, :n, 0, 0, isp]
        np.testing.assert_allclose(np.linalg.norm(u1, axis=0), np.linalg.norm(u0, axis=0), rtol=1e-14)
        gc = np.sqrt(p.c ** 2 + (u0 ** 2).sum(0))
        theta = 2 * np.arctan(q[isp] / r[isp] * 0.5 * p.delt * bx / gc)
        ang = np.arctan2(u0[1] * u1[2] - u0[2] * u1[1], u0[1] * u1[1] + u0[2] * u1[2])
        np.testing.assert_allclose(ang, -theta, rtol=1e-10, atol=1e-14)
        np.testing.assert_allclose(u1[0], u0[0], rtol=1e-15)


def test_cg_solves_the_implicit_system_3d():
    """After field__fdtd_i the B increment satisfies (f4 - N) dB = f5 gkl to the CG tolerance."""
    p, st = small_case3d(nx=8, ny=8, nz=6, ppc=4, seed=21, u_the=0.2)
    o = make_oracle3d(p)
    uf0 = st.uf.copy(order="F")
    # a nonzero field so that every term of gkl contributes
    rng = np.random.default_rng(0)
    uf0[:, 2:-2, 2:-2, 2:-2] = 1e-3 * rng.standard_normal(uf0[:, 2:-2, 2:-2, 2:-2].shape)
    # periodic ghosts of the seeded field
    core = uf0[:, 2:-2, 2:-2, 2:-2]
    uf0[...] = np.pad(core, ((0, 0), (2, 2), (2, 2), (2, 2)), mode="wrap")
    st.uf[...] = uf0
    assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
    assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
    uj = o.get_uj()
    df = o.get_df()
    f1 = p.c * p.delt / p.delx
    f2 = p.gfac * f1 * f1
    f3 = 4 * math.pi * p.delx / p.c
    f5 = (p.delx / (p.c * p.delt * p.gfac)) ** 2
    f4 = 6 + f5
    U = uf0[:, 2:-2, 2:-2, 2:-2]
    J = uj[:, 2:-2, 2:-2, 2:-2]

    def lap(a):
        return sum(np.roll(a, s, ax) for ax in range(3) for s in (1, -1)) - 6 * a

    def sm(a, ax):  # a(i-1) along axis ax
        return np.roll(a, 1, ax)
    X, Y, Z = 0, 1, 2
    gkl = np.zeros((3,) + U.shape[1:])
    gkl[0] = f2 * (lap(U[0]) + f3 * (-sm(J[2], Y) + J[2] + sm(J[1], Z) - J[1])) - f1 * (-sm(U[5], Y) + U[5] + sm(U[4], Z) - U[4])
    gkl[1] = f2 * (lap(U[1]) + f3 * (-sm(J[0], Z) + J[0] + sm(J[2], X) - J[2])) - f1 * (-sm(U[3], Z) + U[3] + sm(U[5], X) - U[5])
    gkl[2] = f2 * (lap(U[2]) + f3 * (-sm(J[1], X) + J[1] + sm(J[0], Y) - J[0])) - f1 * (-sm(U[4], X) + U[4] + sm(U[3], Y) - U[3])
    for l in range(3):
        b = f5 * gkl[l]
        x = df[l, 2:-2, 2:-2, 2:-2]
        res = b - (f4 * x - (lap(x) + 6 * x))
        assert np.linalg.norm(res) <= 2e-6 * np.linalg.norm(b) + 1e-300
    assert (o.cg_iters() > 0).all()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_particle_yz_matches_literal_restatement(seed):
    """The oracle's 3D migration equals a literal pure-Python restatement, particle by particle."""
    p, st = small_case3d(nx=5, ny=4, nz=3, ppc=5, seed=seed, u_the=0.6, drift=0.0)
    o = make_oracle3d(p)
    # move particles by up to one cell in y and z (and across the periodic faces)
    rng = np.random.default_rng(seed)
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = st.np2[jj, kk, isp]
                st.up[1, :n, jj, kk, isp] += rng.uniform(-0.9, 0.9, n)
                st.up[2, :n, jj, kk, isp] += rng.uniform(-0.9, 0.9, n)
    a = st.up.copy(order="F")
    na = st.np2.copy(order="F")
    assert o.bc_particle_yz(a, na) == 0
    b = st.up.copy(order="F")
    nb = st.np2.copy(order="F")
    literal_particle_yz(b, nb, p)
    np.testing.assert_array_equal(na, nb)
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = na[jj, kk, isp]
                np.testing.assert_array_equal(a[:, :n, jj, kk, isp].view(np.int64), b[:, :n, jj, kk, isp].view(np.int64))
                # every particle now lies in its row
                assert (np.floor(a[1, :n, jj, kk, isp]).astype(int) == p.nygs + jj).all()
                assert (np.floor(a[2, :n, jj, kk, isp]).astype(int) == p.nzgs + kk).all()
    assert na.sum() == st.np2.sum()


def test_sort_and_bookkeeping_3d():
    p, st = small_case3d(nx=6, ny=4, nz=4, ppc=4, seed=7, u_the=0.3)
    o = make_oracle3d(p)
    ids0 = np.sort(np.concatenate([st.up[6, :st.np2[j, k, s], j, k, s].view(np.int64)
                                   for s in range(p.nsp) for k in range(p.nz) for j in range(p.ny)]))
    for _ in range(5):
        assert o.step(st) == 0
    ids = np.sort(np.concatenate([st.up[6, :st.np2[j, k, s], j, k, s].view(np.int64)
                                  for s in range(p.nsp) for k in range(p.nz) for j in range(p.ny)]))
    np.testing.assert_array_equal(ids, ids0)
    for s in range(p.nsp):
        for k in range(p.nz):
            for j in range(p.ny):
                n = st.np2[j, k, s]
                cell = np.floor(st.up[0, :n, j, k, s]).astype(int)
                assert (np.diff(cell) >= 0).all()
                cc = np.searchsorted(cell, np.arange(p.nxgs, p.nxge + 2), side="left")
                np.testing.assert_array_equal(st.cumcnt[:, j, k, s], cc)


def test_energy_sums_3d():
    p, st = small_case3d(seed=13)
    rng = np.random.default_rng(1)
    st.uf[...] = rng.standard_normal(st.uf.shape)
    o = make_oracle3d(p)
    e = o.energy(st.up, st.uf, st.np2)
    q, r = p.charges()
    for s in range(p.nsp):
        u = np.concatenate([st.up[3:6, :st.np2[j, k, s], j, k, s] for k in range(p.nz) for j in range(p.ny)], axis=1)
        ke = (r[s] * (np.sqrt(1 + (u ** 2).sum(0) / p.c ** 2) - 1)).sum()
        np.testing.assert_allclose(e[s], ke, rtol=1e-12)
    U = st.uf[:, 2:-2, 2:-2, 2:-2]
    np.testing.assert_allclose(e[p.nsp], (U[3:] ** 2).sum() / (8 * math.pi), rtol=1e-12)
    np.testing.assert_allclose(e[p.nsp + 1], (U[:3] ** 2).sum() / (8 * math.pi), rtol=1e-12)


def test_threads_do_not_change_push_and_fields_3d():
    p, st = small_case3d(nx=6, ny=6, nz=4, ppc=4, seed=17, u_the=0.2)
    s1 = st.copy()
    o1 = make_oracle3d(p, threads=1)
    o4 = make_oracle3d(p, threads=4)
    for _ in range(2):
        assert o1.step(st) == 0
        assert o4.step(s1) == 0
    np.testing.assert_allclose(s1.uf, st.uf, rtol=0, atol=1e-12 * np.abs(st.uf).max())
    np.testing.assert_array_equal(s1.np2, st.np2)


def _uniform_fields3d(uf, b, e):
    uf[...] = 0.0
    for k in range(3):
        uf[k] = b[k]
        uf[3 + k] = e[k]


def test_vay_conserves_momentum_magnitude_in_pure_b_3d():
    """particle__solv_vay (3d/common/particle.f90:236) with E = 0 conserves |u|."""
    p, st = small_case3d(seed=13, u_the=0.3)
    _uniform_fields3d(st.uf, (0.2, -0.1, 0.35), (0.0, 0.0, 0.0))
    o = make_oracle3d(p)
    assert o.particle_solv_vay(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = st.np2[jj, kk, isp]
                u0 = st.up[3:6, :n, jj, kk, isp]
                u1 = st.gp[3:6, :n, jj, kk, isp]
                np.testing.assert_allclose(np.linalg.norm(u1, axis=0), np.linalg.norm(u0, axis=0), rtol=1e-13)


def test_vay_equals_boris_in_pure_e_3d():
    p, st = small_case3d(seed=17, u_the=0.3)
    _uniform_fields3d(st.uf, (0.0, 0.0, 0.0), (0.05, -0.02, 0.03))
    o = make_oracle3d(p)
    gb = st.gp.copy(order="F")
    assert o.particle_solv(gb, st.up, st.uf, st.cumcnt) == 0
    assert o.particle_solv_vay(st.gp, st.up, st.uf, st.cumcnt) == 0
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = st.np2[jj, kk, isp]
                np.testing.assert_allclose(st.gp[:6, :n, jj, kk, isp], gb[:6, :n, jj, kk, isp],
                                           rtol=1e-13, atol=1e-15)


def test_moments_match_numpy_restatement_3d():
    p, st = small_case3d(seed=23, u_the=0.2)
    rng = np.random.default_rng(23)
    core = 0.02 * rng.standard_normal((6, p.nx, p.ny, p.nz))
    st.uf[...] = np.pad(core, ((0, 0), (2, 2), (2, 2), (2, 2)), mode="wrap")
    o = make_oracle3d(p)
    rc, mom = o.moments(st)
    assert rc == 0
    ref = literal_moments3d(p, st.gp, st.np2)
    np.testing.assert_allclose(mom, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    for isp in range(p.nsp):
        n = mom[0, 1:p.nx + 1, 1:p.ny + 1, 1:p.nz + 1, isp].sum()
        np.testing.assert_allclose(n, st.np2[:, :, isp].sum(), rtol=1e-12)


# ---- conducting walls in x (3d/proj/reconnection/boundary_reconnection.f90) ----

def walls_case(seed, **kw):
    kw.setdefault("u_the", 0.2)
    return small_case3d(nx=8, ny=5, nz=4, ppc=4, seed=seed, bc="reconnection", **kw)


def test_walls_steps_conserve_charge_3d():
    """The reconnection driver's order (3d/proj/reconnection/app.f90:103-108): push, reflection
    at the walls, field solve, y/z migration, sort.  Charge is conserved to round-off, no
    particle is lost and all stay between the walls."""
    p, st = walls_case(31, u_the=0.3)
    q, _ = p.charges()
    o = make_oracle3d(p, bc="reconnection")
    for _ in range(4):
        up0 = st.up.copy(order="F")
        assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
        assert o.bc_particle_x(st.gp, st.np2) == 0
        assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
        res, scale = continuity_residual3d(p, q, up0, st.gp, st.np2, o.get_uj())
        assert res <= 1e-12 * scale, (res, scale)
        assert o.bc_particle_yz(st.gp, st.np2) == 0
        assert o.sort_bucket(st.up, st.gp, st.cumcnt, st.np2) == 0
    assert st.np2.sum() == p.n_particles
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                x = st.up[0, :st.np2[jj, kk, isp], jj, kk, isp]
                assert x.min() >= (p.nxgs + 1) * p.delx and x.max() < (p.nxge - 1) * p.delx


def test_walls_reflection_3d():
    """boundary_reconnection__particle_x: x = 2 (nxs+1) dx - x below the left wall, 2 (nxe-1) dx - x
    from the right one, all three momenta reversed (numpy restatement)."""
    p, st = walls_case(32)
    o = make_oracle3d(p, bc="reconnection")
    rng = np.random.default_rng(32)
    gp = st.up.copy(order="F")
    n = st.np2[0, 0, 1]
    gp[0, :n, 0, 0, 1] = rng.uniform(p.nxgs + 0.5, p.nxge + 0.5, n) * p.delx
    ref = gp.copy(order="F")
    x = ref[0, :n, 0, 0, 1]
    cell = np.trunc(x / p.delx).astype(int)
    lo, hi = cell < p.nxgs + 1, cell >= p.nxge - 1
    x[lo] = 2.0 * (p.nxgs + 1) * p.delx - x[lo]
    x[hi] = 2.0 * (p.nxge - 1) * p.delx - x[hi]
    for d in (3, 4, 5):
        u = ref[d, :n, 0, 0, 1]
        u[lo | hi] = -u[lo | hi]
    assert lo.any() and hi.any()
    assert o.bc_particle_x(gp, st.np2) == 0
    np.testing.assert_array_equal(gp, ref)


def test_walls_dfield_rule_3d():
    """boundary_reconnection__dfield: periodic ghost copies in y and z, then at the walls Bx and
    (Ey, Ez) odd about nxs and nxe - 1/2, (By, Bz, Ex) even about nxs and nxe (numpy restatement)."""
    p, st = walls_case(33)
    o = make_oracle3d(p, bc="reconnection")
    rng = np.random.default_rng(33)
    df = np.asfortranarray(rng.standard_normal(st.uf.shape))
    ref = df.copy(order="F")
    o.bc_dfield(df)
    nx, ny, nz = p.nx, p.ny, p.nz
    # y then z ghost copies over the interior x columns (2..nx+1 in array indices)
    xs = slice(2, nx + 2)
    ref[:, xs, ny + 2, 2:nz + 2] = ref[:, xs, 2, 2:nz + 2]
    ref[:, xs, ny + 3, 2:nz + 2] = ref[:, xs, 3, 2:nz + 2]
    ref[:, xs, 0, 2:nz + 2] = ref[:, xs, ny, 2:nz + 2]
    ref[:, xs, 1, 2:nz + 2] = ref[:, xs, ny + 1, 2:nz + 2]
    ref[:, xs, :, nz + 2] = ref[:, xs, :, 2]
    ref[:, xs, :, nz + 3] = ref[:, xs, :, 3]
    ref[:, xs, :, 0] = ref[:, xs, :, nz]
    ref[:, xs, :, 1] = ref[:, xs, :, nz + 1]
    s, e = 2, nx + 1  # nxs, nxe
    ref[0, s - 1] = -ref[0, s]
    ref[1:4, s - 1] = ref[1:4, s + 1]
    ref[4:6, s - 1] = -ref[4:6, s]
    ref[0, e] = -ref[0, e - 1]
    ref[1:4, e + 1] = ref[1:4, e - 1]
    ref[4:6, e] = -ref[4:6, e - 1]
    np.testing.assert_array_equal(df, ref)


def test_walls_moments_3d():
    p, st = walls_case(34)
    o = make_oracle3d(p, bc="reconnection")
    rc, mom = o.moments(st)
    assert rc == 0
    ref = literal_moments3d(p, st.gp, st.np2, bc="reconnection")
    np.testing.assert_allclose(mom, ref, rtol=0, atol=1e-13 * np.abs(ref).max())


# ---- the shock boundary (3d/proj/shock/boundary_shock.f90): wall at nxs, open end at nxe ----

def shock_case(seed, **kw):
    kw.setdefault("u_the", 0.1)
    return small_case3d(nx=12, ny=5, nz=4, ppc=4, seed=seed, bc="shock", window=9, u0=0.2, **kw)


def shock_oracle(p):
    o = make_oracle3d(p, bc="shock")
    o.set_window(p.nxgs, p.nxe)
    o.u0 = p.u0
    return o


def test_shock_steps_conserve_charge_3d():
    """The shock driver's order (3d/proj/shock/app.f90:112-117): push, injection, field solve,
    y/z migration, sort, on the window; charge conserved to round-off, no particle lost, all
    between the wall and the injection boundary."""
    p, st = shock_case(41)
    q, _ = p.charges()
    o = shock_oracle(p)
    for _ in range(4):
        up0 = st.up.copy(order="F")
        assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
        assert o.bc_injection(st.gp, st.np2) == 0
        assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
        res, scale = continuity_residual3d(p, q, up0, st.gp, st.np2, o.get_uj())
        assert res <= 1e-12 * scale, (res, scale)
        assert o.bc_particle_yz(st.gp, st.np2) == 0
        assert o.sort_bucket(st.up, st.gp, st.cumcnt, st.np2) == 0
    assert st.np2.sum() == p.n_particles
    xend = p.nxe * p.delx + p.u0 / math.sqrt(1 + p.u0 ** 2 / p.c ** 2) * p.delt
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                x = st.up[0, :st.np2[jj, kk, isp], jj, kk, isp]
                assert x.min() >= (p.nxgs + 1) * p.delx and x.max() <= xend


def test_shock_injection_3d():
    """boundary_shock__injection: reflection at (nxs+1) dx with all momenta reversed, and at
    xend = nxe dx + v0 dt with u_x -> 2 u0 - u_x, u_y and u_z reversed (numpy restatement)."""
    p, st = shock_case(42)
    o = shock_oracle(p)
    rng = np.random.default_rng(42)
    gp = st.up.copy(order="F")
    n = st.np2[1, 2, 0]
    xend = p.nxe * p.delx + p.u0 / math.sqrt(1.0 + (p.u0 * p.u0) / (p.c * p.c)) * p.delt
    gp[0, :n, 1, 2, 0] = rng.uniform(p.nxgs + 0.05, xend + 0.9, n)
    ref = gp.copy(order="F")
    x, u = ref[0, :n, 1, 2, 0], ref[3:6, :n, 1, 2, 0]
    lo = np.trunc(x / p.delx).astype(int) < p.nxgs + 1
    hi = ~lo & (x > xend)
    x[lo] = 2.0 * (p.nxgs + 1) * p.delx - x[lo]
    u[:, lo] = -u[:, lo]
    x[hi] = 2.0 * xend - x[hi]
    u[0, hi] = 2.0 * p.u0 - u[0, hi]
    u[1:, hi] = -u[1:, hi]
    assert lo.any() and hi.any()
    assert o.bc_injection(gp, st.np2) == 0
    np.testing.assert_array_equal(gp, ref)


def test_shock_dfield_rule_3d():
    """boundary_shock__dfield: y and z copies over the window's columns, the wall rule at nxs,
    zero in column nxe+1; columns beyond are left as they are (numpy restatement)."""
    p, st = shock_case(43)
    o = shock_oracle(p)
    rng = np.random.default_rng(43)
    df = np.asfortranarray(rng.standard_normal(st.uf.shape))
    ref = df.copy(order="F")
    o.bc_dfield(df)
    ny, nz = p.ny, p.nz
    s, e = 2, p.nxe - p.nxgs + 2  # array columns of nxs and nxe
    xs = slice(s, e + 1)
    ref[:, xs, ny + 2, 2:nz + 2] = ref[:, xs, 2, 2:nz + 2]
    ref[:, xs, ny + 3, 2:nz + 2] = ref[:, xs, 3, 2:nz + 2]
    ref[:, xs, 0, 2:nz + 2] = ref[:, xs, ny, 2:nz + 2]
    ref[:, xs, 1, 2:nz + 2] = ref[:, xs, ny + 1, 2:nz + 2]
    ref[:, xs, :, nz + 2] = ref[:, xs, :, 2]
    ref[:, xs, :, nz + 3] = ref[:, xs, :, 3]
    ref[:, xs, :, 0] = ref[:, xs, :, nz]
    ref[:, xs, :, 1] = ref[:, xs, :, nz + 1]
    ref[0, s - 1] = -ref[0, s]
    ref[1:4, s - 1] = ref[1:4, s + 1]
    ref[4:6, s - 1] = -ref[4:6, s]
    ref[:, e + 1] = 0.0
    np.testing.assert_array_equal(df, ref)
