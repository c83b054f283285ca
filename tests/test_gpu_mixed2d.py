"""GPU tests of the mixed-precision 2D path (integer cell + FP32 offset,
FP32 push/gather/deposition, FP64 fields), through the C ABI.

Every result is stated as an error against the FP64 path:
  * one step from the same state (Boris and Vay pushers): momenta and positions within
    1e-5 relative to their scale, fields within 1e-4 of max|B, E|;
  * charge conservation |d rho/dt + div J| <= 1e-6 of max |d rho/dt|, rho computed in
    FP64 from the exact stored positions;
  * bookkeeping exact: particle count and the set of IDs conserved, every
    particle inside the cell its bin records.
"""
import numpy as np
import pytest

from tests.helpers import continuity_residual, small_case, small_plasma
from wumingpic_gb300.loader import load_weibel2d

pytestmark = pytest.mark.gpu


def make(p, precision, gpu_lib):
    from wumingpic_gb300.pic2d import Pic2D
    return Pic2D(p, precision=precision)


def by_id(st, p):
    """dict id -> (x, y, ux, uy, uz) over all valid particles, plus species index"""
    out = {}
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            a = st.up[:, :n, jj, isp]
            ids = a[5].view(np.int64)
            for k in range(n):
                out[(isp, int(ids[k]))] = a[:5, k]
    return out


def test_put_get_round_trip(gpu_lib):
    p, st = small_case(nx=32, ny=32, ppc=5, seed=4)
    g = make(p, "mixed", gpu_lib)
    g.put_state(st)
    out = g.get_state()
    np.testing.assert_array_equal(out.np2, st.np2)
    np.testing.assert_array_equal(out.cumcnt, st.cumcnt)
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            np.testing.assert_array_equal(out.up[5, :n, jj, isp].view(np.int64), st.up[5, :n, jj, isp].view(np.int64))
            np.testing.assert_allclose(out.up[0:2, :n, jj, isp], st.up[0:2, :n, jj, isp], rtol=0, atol=2 ** -22)
            np.testing.assert_allclose(out.up[2:5, :n, jj, isp], st.up[2:5, :n, jj, isp], rtol=2 ** -23, atol=1e-30)


@pytest.mark.parametrize("off16", [0, 8])
def test_put_get_in_place_through_registered_host_memory(gpu_lib, off16):
    """Host arrays page-locked with wpic_host_register are read and written in place by the
    conversion kernels (no staging copies): after two steps the same state as through ordinary
    host arrays, bit for bit.  The kernels move 16 bytes per access, so a particle array 8 bytes
    off a 16-byte boundary (a view into a registered buffer) takes the staged copies instead,
    with the same result."""
    from wumingpic_gb300 import _lib
    p, st = small_case(nx=32, ny=32, ppc=5, seed=24)
    a, b = make(p, "mixed", gpu_lib), make(p, "mixed", gpu_lib)
    a.put_state(st)
    reg = st.copy()
    buf = np.zeros(reg.up.size + 2)
    s0 = next(k for k in range(3) if (buf.ctypes.data + 8 * k) % 16 == off16)
    view = buf[s0:s0 + reg.up.size].reshape(reg.up.shape, order="F")
    view[...] = reg.up
    assert view.ctypes.data % 16 == off16 and view.flags.f_contiguous
    reg.up = view
    _lib.host_register(buf)
    try:
        b.put_state(reg)
        a.step(2)
        b.step(2)
        sa = a.get_state()
        sb = b.get_state(reg)  # into the registered array
        np.testing.assert_array_equal(sb.np2, sa.np2)
        np.testing.assert_array_equal(sb.cumcnt, sa.cumcnt)
        np.testing.assert_array_equal(sb.uf, sa.uf)
        for isp in range(p.nsp):
            for jj in range(p.ny):
                n = sa.np2[jj, isp]
                np.testing.assert_array_equal(sb.up[:, :n, jj, isp], sa.up[:, :n, jj, isp])
    finally:
        _lib.host_unregister(buf)
    a.close()
    b.close()


def test_put_unsorted_rows_sorts_them(gpu_lib):
    """The restart path on a mixed context: put with which = 1 (gp) takes rows whose particles
    are in no particular order within the row, sorts them by x cell on the host and stores the
    sorted state.  Against a put of the sorted rows: the same cumcnt and np2, the same particles
    (matched by id), and after two steps the same fields to 1e-6 of their largest value (the
    order within a cell changes the FP32 sums of the register current before each flush)."""
    p, st = small_case(nx=32, ny=32, ppc=5, seed=14)
    rng = np.random.default_rng(14)
    up = np.array(st.up, order="F", copy=True)
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = st.np2[jj, isp]
            up[:, :n, jj, isp] = up[:, rng.permutation(n), jj, isp]
    a, b = make(p, "mixed", gpu_lib), make(p, "mixed", gpu_lib)
    a.put_state(st)
    b.put_particles(1, up, st.np2)
    b.put_fields(st.uf)
    sa, sb = a.get_state(), b.get_state()
    np.testing.assert_array_equal(sb.np2, sa.np2)
    np.testing.assert_array_equal(sb.cumcnt, sa.cumcnt)
    ia, ib = by_id(sa, p), by_id(sb, p)
    assert ia.keys() == ib.keys()
    for key in ia:
        np.testing.assert_array_equal(ia[key], ib[key])
    a.step(2)
    b.step(2)
    fa, fb = a.get_fields(), b.get_fields()
    np.testing.assert_allclose(fb, fa, rtol=0, atol=1e-6 * np.abs(fa).max())
    a.close()
    b.close()


@pytest.mark.parametrize("pusher", ["boris", "vay"])
def test_one_step_against_fp64(gpu_lib, pusher):
    p, st = small_case(nx=32, ny=32, ppc=8, seed=6)
    rng = np.random.default_rng(6)
    st.uf[...] = 0.02 * rng.standard_normal(st.uf.shape)
    st.uf[:, :2, :] = st.uf[:, p.nx:p.nx + 2, :]
    st.uf[:, p.nx + 2:, :] = st.uf[:, 2:4, :]
    st.uf[:, :, :2] = st.uf[:, :, p.ny:p.ny + 2]
    st.uf[:, :, p.ny + 2:] = st.uf[:, :, 2:4]
    gm, gd = make(p, "mixed", gpu_lib), make(p, "fp64", gpu_lib)
    gm.set_pusher(pusher)
    gd.set_pusher(pusher)
    gm.put_state(st)
    gd.put_state(st)
    gm.step(1)
    gd.step(1)
    a, b = gm.get_state(), gd.get_state()
    assert a.np2.sum() == b.np2.sum() == p.n_particles
    pa, pb = by_id(a, p), by_id(b, p)
    assert pa.keys() == pb.keys()
    xa = np.array([pa[k] for k in sorted(pa)])
    xb = np.array([pb[k] for k in sorted(pb)])
    np.testing.assert_allclose(xa[:, :2], xb[:, :2], rtol=0, atol=1e-5)
    uscale = np.abs(xb[:, 2:]).max()
    np.testing.assert_allclose(xa[:, 2:], xb[:, 2:], rtol=0, atol=1e-5 * uscale)
    fscale = np.abs(b.uf).max()
    np.testing.assert_allclose(a.uf, b.uf, rtol=0, atol=1e-4 * fscale)


def test_charge_conservation_fp32_deposit(gpu_lib):
    p, st = small_case(nx=32, ny=32, ppc=16, seed=8)
    q, _ = p.charges()
    g = make(p, "mixed", gpu_lib)
    g.put_state(st)
    for _ in range(3):
        before = g.get_state()
        g.step(1)
        after = g.get_state()
        # positions after the step are the new positions (no x/y wrap issue: rho2d wraps periodically)
        res, scale = continuity_residual(p, q, before.up, _match_order(before, after, p), before.np2,
                                         g.get_uj())
        assert res <= 1e-6 * scale, (res, scale)


def _match_order(before, after, p):
    """after-step positions arranged in the before-step slot order (by id)"""
    m = by_id(after, p)
    out = np.array(before.up, order="F", copy=True)
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = before.np2[jj, isp]
            ids = before.up[5, :n, jj, isp].view(np.int64)
            for k in range(n):
                out[:5, k, jj, isp] = m[(isp, int(ids[k]))]
    # undo the periodic wrap so that positions are continuous with the old ones
    for dim, L in ((0, p.nx), (1, p.ny)):
        d = out[dim] - before.up[dim]
        out[dim] -= np.round(d / L) * L
    return out


def test_migration_bookkeeping_many_steps(gpu_lib):
    """Thirty steps of a hot plasma on a 64 x 48 grid (4 x 3 tiles): count and ID set
    conserved, every particle inside the cell its bucket says, cumcnt consistent."""
    p = small_plasma(nx=64, ny=48, ppc=6, seed=12, u_the=0.3, drift=0.5)
    g = make(p, "mixed", gpu_lib)
    st = load_weibel2d(p)
    g.put_state(st)
    ids0 = np.sort(np.concatenate([st.up[5, :st.np2[jj, s], jj, s].view(np.int64)
                                   for s in range(p.nsp) for jj in range(p.ny)]))
    g.step(30)
    out = g.get_state()
    ids = np.sort(np.concatenate([out.up[5, :out.np2[jj, s], jj, s].view(np.int64)
                                  for s in range(p.nsp) for jj in range(p.ny)]))
    np.testing.assert_array_equal(ids, ids0)
    for s in range(p.nsp):
        for jj in range(p.ny):
            n = out.np2[jj, s]
            x = out.up[0, :n, jj, s]
            y = out.up[1, :n, jj, s]
            cell = np.floor(x).astype(int) - p.nxgs
            assert (np.floor(y).astype(int) == p.nygs + jj).all()
            assert (np.diff(cell) >= 0).all()
            np.testing.assert_array_equal(out.cumcnt[:, jj, s],
                                          np.concatenate([[0], np.cumsum(np.bincount(cell, minlength=p.nx))]))


def test_device_loader_matches_fp64_loader(gpu_lib):
    """The mixed and FP64 device loaders draw the same plasma (same Philox counters)."""
    p = small_plasma(nx=32, ny=32, ppc=4, seed=77)
    gm, gd = make(p, "mixed", gpu_lib), make(p, "fp64", gpu_lib)
    gm.load_weibel()
    gd.load_weibel()
    a, b = gm.get_state(), gd.get_state()
    pa, pb = by_id(a, p), by_id(b, p)
    assert pa.keys() == pb.keys()
    xa = np.array([pa[k] for k in sorted(pa)])
    xb = np.array([pb[k] for k in sorted(pb)])
    np.testing.assert_allclose(xa, xb, rtol=2 ** -23, atol=2 ** -22)
    np.testing.assert_allclose(gm.energy(), gd.energy(), rtol=1e-6)


def test_reconnection_walls_mixed(gpu_lib):
    """Conducting walls in x: after 20 steps every particle is still between the walls."""
    p = small_plasma(nx=32, ny=32, ppc=6, seed=5, bc="reconnection", u_the=0.3)
    st = load_weibel2d(p)
    g = make(p, "mixed", gpu_lib)
    g.put_state(st)
    g.step(20)
    out = g.get_state()
    assert out.np2.sum() == st.np2.sum()
    for s in range(p.nsp):
        for jj in range(p.ny):
            x = out.up[0, :out.np2[jj, s], jj, s]
            assert (x >= p.nxgs + 1 - 1e-6).all() and (x <= p.nxge - 1 + 1e-6).all()


def test_mixed_path_is_bitwise_reproducible(gpu_lib):
    """Integer (fixed-point) current sums, deterministic reductions and deterministic
    migration: two runs from the same state agree bit for bit."""
    p, st = small_case(nx=32, ny=32, ppc=8, seed=23)
    outs = []
    for _ in range(2):
        g = make(p, "mixed", gpu_lib)
        g.put_state(st)
        g.step(5)
        outs.append((g.get_state(), g.energy()))
    (a, ea), (b, eb) = outs
    np.testing.assert_array_equal(a.np2, b.np2)
    np.testing.assert_array_equal(a.up.view(np.int64), b.up.view(np.int64))
    np.testing.assert_array_equal(a.uf.view(np.int64), b.uf.view(np.int64))
    np.testing.assert_array_equal(ea, eb)


@pytest.mark.parametrize("nsteps", [1, 6])
def test_shock_window_against_fp64(gpu_lib, nsteps):
    """The shock boundary on the mixed 2D path: the wall reflection at nxs + 1 and the
    injection boundary at xend inside the fused push, before the deposit (the shock driver
    calls bc__injection before field__fdtd_i); particles within 1e-5 (one step) / 1e-4 (six
    steps) of the FP64 shock path, energies within 1e-3."""
    p, st = small_case(nx=32, ny=16, ppc=8, seed=79, bc="shock", window=24, u0=0.2, u_the=0.1)
    rng = np.random.default_rng(79)
    st.uf[...] = np.pad(0.02 * rng.standard_normal((6, p.nx, p.ny)), ((0, 0), (2, 2), (2, 2)), mode="wrap")
    gm, gd = make(p, "mixed", gpu_lib), make(p, "fp64", gpu_lib)
    gm.put_state(st)
    gd.put_state(st)
    gm.step(nsteps)
    gd.step(nsteps)
    a, b = gm.get_state(), gd.get_state()
    assert a.np2.sum() == b.np2.sum() == st.np2.sum()
    pa, pb = by_id(a, p), by_id(b, p)
    assert pa.keys() == pb.keys()
    xa = np.array([pa[k] for k in sorted(pa)])
    xb = np.array([pb[k] for k in sorted(pb)])
    tol = 1e-5 if nsteps == 1 else 1e-4
    np.testing.assert_allclose(xa[:, :2], xb[:, :2], rtol=0, atol=tol * p.delx)
    uscale = np.abs(xb[:, 2:]).max()
    np.testing.assert_allclose(xa[:, 2:], xb[:, 2:], rtol=0, atol=tol * uscale)
    assert xa[:, 0].min() >= (p.nxgs + 1) * p.delx and xa[:, 0].max() <= (p.nxe + 1) * p.delx
    em, ed = gm.energy(), gd.energy()
    np.testing.assert_allclose(em, ed, rtol=1e-3, atol=1e-6 * ed.sum())



def _shock_pair(p, st, gpu_lib, steps, widen_at=None):
    gm, gd = make(p, "mixed", gpu_lib), make(p, "fp64", gpu_lib)
    gm.put_state(st)
    gd.put_state(st)
    nxe = p.nxe
    for it in range(steps):
        if widen_at is not None and it == widen_at:
            # the driver's relocate() widens the window by an empty cell (2d/proj/shock/app.f90:615-625)
            nxe += 1
            gm.set_window(p.nxgs, nxe)
            gd.set_window(p.nxgs, nxe)
        gm.step(1)
        gd.step(1)
    return gm, gd, nxe


def _compare_shock(p, st, gm, gd, tol, nxe):
    a, b = gm.get_state(), gd.get_state()
    assert a.np2.sum() == b.np2.sum() == st.np2.sum()
    pa, pb = by_id(a, p), by_id(b, p)
    assert pa.keys() == pb.keys()
    xa = np.array([pa[k] for k in sorted(pa)])
    xb = np.array([pb[k] for k in sorted(pb)])
    np.testing.assert_allclose(xa[:, :2], xb[:, :2], rtol=0, atol=tol * p.delx)
    uscale = np.abs(xb[:, 2:]).max()
    np.testing.assert_allclose(xa[:, 2:], xb[:, 2:], rtol=0, atol=tol * uscale)
    assert xa[:, 0].min() >= (p.nxgs + 1) * p.delx and xa[:, 0].max() <= (nxe + 1) * p.delx
    em, ed = gm.energy(), gd.energy()
    np.testing.assert_allclose(em, ed, rtol=1e-3, atol=1e-6 * ed.sum())


def test_shock_expanding_window_against_fp64(gpu_lib):
    """The window widened by one cell between steps on a mixed context, as the shock driver's
    relocate() does: xend and the wall follow the window; six steps within 1e-4 of the FP64
    shock path with the same widening."""
    p, st = small_case(nx=32, ny=16, ppc=8, seed=81, bc="shock", window=24, u0=0.2, u_the=0.1)
    rng = np.random.default_rng(81)
    st.uf[...] = np.pad(0.02 * rng.standard_normal((6, p.nx, p.ny)), ((0, 0), (2, 2), (2, 2)), mode="wrap")
    gm, gd, nxe = _shock_pair(p, st, gpu_lib, 6, widen_at=3)
    _compare_shock(p, st, gm, gd, 1e-4, nxe)


@pytest.mark.parametrize("nsteps", [1, 8])
def test_shock_far_window_against_fp64(gpu_lib, nsteps):
    """A window of 4100 cells with the plasma streaming hot towards the injection end (u0 < 0:
    drift +0.2c, u_th 0.3c): the particles reflected there, near x = 4100 cells, keep the split
    representation's precision (the mirror image is formed from the integer cells and the FP32
    offsets separately), within 1e-5 (one step) / 1e-4 (eight steps) of the FP64 path."""
    p, st = small_case(nx=4112, ny=16, ppc=2, seed=83, bc="shock", window=4100, u0=-0.2, u_the=0.3)
    gm, gd, nxe = _shock_pair(p, st, gpu_lib, nsteps)
    _compare_shock(p, st, gm, gd, 1e-5 if nsteps == 1 else 1e-4, nxe)
    if nsteps > 1:  # particles crossed the loaded plasma's edge into the cells before xend
        b = gd.get_state()
        far = sum(int((b.up[0, :b.np2[j, s], j, s] >= (p.nxgs + p.window - 2) * p.delx).sum())
                  for s in range(p.nsp) for j in range(p.ny))
        assert far > 0
