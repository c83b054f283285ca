"""The C ABI driven by a compiled C program in the 2D Weibel driver's call order.

wumingpic_gb300/driver/wpic_driver2d.c runs the main loop of 2d/proj/weibel/app.f90:99-126
through the header: particle__solv, field__fdtd_i, bc__particle_x, bc__particle_y and
sort__bucket every step; at every intvl_mom step it refreshes the host arrays (the sync point
of the Fortran shim, on entry to mom_calc__accl), runs mom_calc__accl, mom_calc__nvt and
bc__mom, and computes energy_history on the host from the refreshed arrays.  The host arrays it
writes at those steps must equal a ctypes run of the same calls, bit for bit, and the fused
wpic_step path; its host energy_history must equal the library's wpic_energy.
"""
import os
import subprocess

import numpy as np
import pytest

from wumingpic_gb300.loader import Plasma2D, load_weibel2d

pytestmark = pytest.mark.gpu

NSTEPS, INTVL = 6, 3


def _write_input(path, p, st):
    q, r = p.charges()
    with open(path, "wb") as f:
        np.asarray(q, np.float64).tofile(f)
        np.asarray(r, np.float64).tofile(f)
        st.up.ravel(order="F").tofile(f)
        st.uf.ravel(order="F").tofile(f)
        st.cumcnt.astype(np.int32).ravel(order="F").tofile(f)
        st.np2.astype(np.int32).ravel(order="F").tofile(f)


def _read_output(path, p):
    nup = 6 * p.np_cap * p.ny * 2
    nuf = 6 * (p.nx + 4) * (p.ny + 4)
    ncc, nnp, nmom = (p.nx + 1) * p.ny * 2, p.ny * 2, 7 * (p.nx + 2) * (p.ny + 2) * 2
    raw = open(path, "rb").read()
    recs, o = [], 0
    while o < len(raw):
        it = int(np.frombuffer(raw, np.int32, 1, o)[0]); o += 4
        up = np.frombuffer(raw, np.float64, nup, o).reshape((6, p.np_cap, p.ny, 2), order="F"); o += 8 * nup
        np2 = np.frombuffer(raw, np.int32, nnp, o).reshape((p.ny, 2), order="F"); o += 4 * nnp
        cc = np.frombuffer(raw, np.int32, ncc, o).reshape((p.nx + 1, p.ny, 2), order="F"); o += 4 * ncc
        uf = np.frombuffer(raw, np.float64, nuf, o).reshape((6, p.nx + 4, p.ny + 4), order="F"); o += 8 * nuf
        mom = np.frombuffer(raw, np.float64, nmom, o).reshape((7, p.nx + 2, p.ny + 2, 2), order="F"); o += 8 * nmom
        en = np.frombuffer(raw, np.float64, 4, o); o += 32
        recs.append((it, up, np2, cc, uf, mom, en))
    return recs


def _valid_equal(a_up, a_np2, b_up, b_np2):
    np.testing.assert_array_equal(a_np2, b_np2)
    for isp in range(a_np2.shape[1]):
        for j in range(a_np2.shape[0]):
            n = a_np2[j, isp]
            assert np.array_equal(a_up[:, :n, j, isp].view(np.int64), b_up[:, :n, j, isp].view(np.int64)), (j, isp)


def test_c_driver_in_app_order_matches_ctypes(gpu_lib, tmp_path):
    from wumingpic_gb300 import _build
    from wumingpic_gb300.pic2d import Pic2D
    exe = _build.build_driver()
    p = Plasma2D(nx=32, ny=24, ppc=8, drift=0.5, u_the=0.05, seed=31337, np_slack=3.0)
    st = load_weibel2d(p)
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(fin, p, st)
    r = subprocess.run([exe, fin, fout, str(p.nx), str(p.ny), str(p.np_cap), str(NSTEPS), str(INTVL)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    recs = _read_output(fout, p)
    assert [x[0] for x in recs] == list(range(INTVL, NSTEPS + 1, INTVL))

    # the same calls through ctypes
    g = Pic2D(p, precision="fp64")
    g.put_state(st)
    # the fused step from the same state
    h = Pic2D(p, precision="fp64")
    h.put_state(st)
    k = 0
    for it in range(1, NSTEPS + 1):
        g.particle__solv()
        g.field__fdtd_i()
        g.bc__particle_x()
        g.bc__particle_y()
        g.sort__bucket()
        h.step(1)
        if it % INTVL:
            continue
        cur = g.get_state()
        g.mom_calc__accl()
        g.mom_calc__nvt()
        g.bc__mom()
        mom = g.get_mom()
        en = g.energy()
        fused = h.get_state()
        _, up, np2, cc, uf, cmom, cen = recs[k]
        k += 1
        _valid_equal(up, np2, cur.up, cur.np2)
        np.testing.assert_array_equal(cc, cur.cumcnt)
        np.testing.assert_array_equal(uf, cur.uf)
        np.testing.assert_array_equal(cmom, mom)
        np.testing.assert_allclose(cen, en, rtol=1e-12)
        # the staged calls and the fused step give the same state
        _valid_equal(fused.up, fused.np2, cur.up, cur.np2)
        np.testing.assert_array_equal(fused.cumcnt, cur.cumcnt)
        np.testing.assert_array_equal(fused.uf, cur.uf)
    g.close()
    h.close()


def test_c_driver_mixed_precision_runs_the_fused_step(gpu_lib, tmp_path):
    """The same unchanged call sequence on a WPIC_MIXED context: particle__solv requests the
    push, field__fdtd_i runs the fused mixed step, particle_x, particle_y and sort__bucket find
    their work done, and the diagnostic block's calls give the mixed moments.  The host arrays
    at the diagnostic steps equal the fused wpic_step path's bit for bit; the moments (FP32
    shared-memory sums, whose order varies) agree to 1e-6 of each moment's largest value."""
    from wumingpic_gb300 import _build
    from wumingpic_gb300.pic2d import Pic2D
    exe = _build.build_driver()
    p = Plasma2D(nx=32, ny=32, ppc=8, drift=0.5, u_the=0.05, seed=4242, np_slack=3.0)
    st = load_weibel2d(p)
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(fin, p, st)
    r = subprocess.run([exe, fin, fout, str(p.nx), str(p.ny), str(p.np_cap), str(NSTEPS), str(INTVL), "2"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    recs = _read_output(fout, p)
    assert [x[0] for x in recs] == list(range(INTVL, NSTEPS + 1, INTVL))

    g = Pic2D(p, precision="mixed")  # the staged calls through ctypes
    g.put_state(st)
    h = Pic2D(p, precision="mixed")  # the fused step
    h.put_state(st)
    k = 0
    for it in range(1, NSTEPS + 1):
        g.particle__solv()
        g.field__fdtd_i()
        g.bc__particle_x()
        g.bc__particle_y()
        g.sort__bucket()
        h.step(1)
        if it % INTVL:
            continue
        cur = g.get_state()
        g.mom_calc__accl()
        g.mom_calc__nvt()
        g.bc__mom()
        mom = g.get_mom()
        fused = h.get_state()
        fmom = h.moments()
        _, up, np2, cc, uf, cmom, cen = recs[k]
        k += 1
        _valid_equal(up, np2, cur.up, cur.np2)
        np.testing.assert_array_equal(cc, cur.cumcnt)
        np.testing.assert_array_equal(uf, cur.uf)
        _valid_equal(fused.up, fused.np2, cur.up, cur.np2)
        np.testing.assert_array_equal(fused.uf, cur.uf)
        for a in (cmom, mom):
            for q in range(7):
                scale = np.abs(fmom[q]).max()
                np.testing.assert_allclose(a[q], fmom[q], rtol=0, atol=1e-6 * scale)
        np.testing.assert_allclose(cen, h.energy(), rtol=1e-10)
    g.close()
    h.close()


def test_staged_calls_on_mixed_context_reject_out_of_order_use(gpu_lib):
    """A field solve without its push, a second push, and particle_y or sort__bucket between the
    push and the field solve are refused with WPIC_BAD_ARGUMENT, which leaves the context usable."""
    from wumingpic_gb300._lib import WpicError
    from wumingpic_gb300.pic2d import Pic2D
    p = Plasma2D(nx=32, ny=32, ppc=4, drift=0.5, u_the=0.05, seed=5, np_slack=3.0)
    g = Pic2D(p, precision="mixed")
    g.put_state(load_weibel2d(p))
    with pytest.raises(WpicError):
        g.field__fdtd_i()
    g.particle__solv()
    for call in (g.particle__solv, g.bc__particle_y, g.sort__bucket, lambda: g.step(1)):
        with pytest.raises(WpicError):
            call()
    g.bc__particle_x()  # the reconnection driver's order: particle_x before the field solve
    g.field__fdtd_i()
    g.step(1)
    g.close()
