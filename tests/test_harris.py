"""The Harris-sheet loader of the reconnection configuration (walls in x, periodic y)."""
import math

import numpy as np

from oracle.oracle import Oracle2D
from tests.helpers import continuity_residual
from wumingpic_gb300.loader import Harris2D, config_harris2d, harris_fields, load_harris2d


def _current_profile(p, st):
    dv = p.derived()
    n = p.n_row
    J = np.zeros(p.nx)
    for isp in range(p.nsp):
        x = st.up[0, :n, :, isp].ravel()
        u = st.up[2:5, :n, :, isp].reshape(3, -1)
        cell = np.trunc(x).astype(int) - p.nxgs
        J += np.bincount(cell, weights=dv["q"][isp] * u[2], minlength=p.nx)
    return J / p.ny


def test_layout_and_walls():
    p = config_harris2d()
    st = load_harris2d(p)
    n = p.n_row
    assert (st.np2 == n).all()
    x = st.up[0, :n]
    assert x.min() >= (p.nxgs + 1) * p.delx and x.max() < (p.nxge - 1) * p.delx  # between the walls
    cell = np.trunc(x).astype(int) - p.nxgs
    assert (np.diff(cell, axis=0) >= 0).all()                                      # bucket-sorted rows
    for isp in range(p.nsp):
        for jj in range(p.ny):
            counts = np.bincount(cell[:, jj, isp], minlength=p.nx)
            np.testing.assert_array_equal(st.cumcnt[1:, jj, isp], np.cumsum(counts))
    y = st.up[1, :n]
    rows = np.arange(p.ny)[None, :, None] + p.nygs
    assert ((y >= rows) & (y < rows + 1)).all()
    ids = st.up[5, :n].view(np.int64)
    for isp in range(p.nsp):
        assert len(np.unique(ids[:, :, isp])) == n * p.ny
    np.testing.assert_array_equal(st.up[:2, :n, :, 0], st.up[:2, :n, :, 1])       # co-located species


def test_fields_and_temperatures():
    p = Harris2D(nx=64, ny=256, ppc=20, lcs=0.2, ncs=16, nbg=4, seed=5, e1=0.1)
    st = load_harris2d(p)
    dv = p.derived()
    i = np.arange(p.nxgs - 2, p.nxge + 3)[:, None]
    j = np.arange(p.nygs - 2, p.nyge + 3)[None, :]
    bx, by = harris_fields(p, i, j)
    np.testing.assert_array_equal(st.uf[0], bx)
    np.testing.assert_array_equal(st.uf[1], by)
    assert (st.uf[2:] == 0).all()
    # far from the X point the field is the Harris profile; the wall-side field is +-b0
    assert abs(st.uf[1, -3, 2] / dv["b0"] - 1) < 1e-3 and abs(st.uf[1, 2, 2] / dv["b0"] + 1) < 1e-3
    n = p.n_row
    for isp, vth in ((0, dv["vti"]), (1, dv["vte"])):
        ux = st.up[2, :n, :, isp]
        assert abs(ux.std() / (vth / math.sqrt(2)) - 1) < 0.02


def test_particle_current_carries_the_sheet():
    """sum q u_z per cell = jz (Ampere, c = 1) scaled by the loaded sheet count: each row
    holds nbg (nx-1) + int(2 ncs lcs) particles but only nbg (nx-3) in the background
    (2d/proj/reconnection/app.f90:307, 413), so the sheet carries 2 nbg more."""
    p = Harris2D(nx=64, ny=512, ppc=20, lcs=0.2, ncs=16, nbg=4, seed=3, e1=0.0)
    st = load_harris2d(p)
    dv = p.derived()
    J = _current_profile(p, st)
    xc = p.nxgs + np.arange(p.nx) + 0.5
    s2 = np.cosh((xc - dv["x0"]) / dv["lcs"]) ** -2
    jz = dv["b0"] / (4 * math.pi * dv["lcs"]) * s2
    L = 0.5 * (p.nxge - p.nxgs - 2) * p.delx
    ratio = (p.n_row - p.nbg * (p.nxge - p.nxgs - 2)) / (2 * p.ncs * dv["lcs"] * math.tanh(L / dv["lcs"]))
    expect = jz * (ratio * p.ncs * s2 + p.nbg) / (p.ncs * s2 + p.nbg)
    assert np.abs(J - expect)[2:-2].max() < 0.02 * jz.max()


def test_oracle_steps_conserve_charge_with_walls():
    """The reconnection driver's step order (2d/proj/reconnection/app.f90:101-106) on the
    Harris state in the oracle: the Esirkepov current conserves charge to round-off, walls
    included, and no particle is lost."""
    p = config_harris2d(seed=9)
    st = load_harris2d(p)
    q, r = p.charges()
    o = Oracle2D(nx=p.nx, ny=p.ny, np_cap=p.np_cap, q=q, r=r, delt=p.delt, delx=p.delx, c=p.c, gfac=p.gfac,
                 bc=p.bc)
    for _ in range(3):
        up0 = st.up.copy(order="F")
        assert o.particle_solv(st.gp, st.up, st.uf, st.cumcnt) == 0
        assert o.bc_particle_x(st.gp, st.np2) == 0
        assert o.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt) == 0
        res, scale = continuity_residual(p, q, up0, st.gp, st.np2, o.get_uj())
        assert res <= 1e-12 * scale, (res, scale)
        assert o.bc_particle_y(st.gp, st.np2) == 0
        assert o.sort_bucket(st.up, st.gp, st.cumcnt, st.np2) == 0
    assert st.np2.sum() == p.n_particles
    for isp in range(p.nsp):
        for jj in range(p.ny):
            x = st.up[0, :st.np2[jj, isp], jj, isp]
            assert x.min() >= (p.nxgs + 1) * p.delx and x.max() < (p.nxge - 1) * p.delx
