"""wpic_energy_noalloc against wpic_energy (collected last on purpose).

wpic_energy_noalloc serves callers that cannot allocate device memory: it reads the
caller's device arrays and keeps its scratch in a fixed __device__ array.  Two calls
in a row must both agree with the context-based entry point to 1e-12 relative (the
two reduce in different orders), and oversized grids are refused.  The test
allocates its own device arrays with torch; the entry point allocates nothing.
"""
import ctypes

import numpy as np
import pytest

from tests.helpers import small_case

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _bind(lib):
    f = lib.wpic_energy_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + \
                 [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_energy_noalloc_matches_energy(gpu_lib):
    import torch
    from wumingpic_gb300.pic2d import Pic2D

    p, st = small_case(nx=24, ny=20, ppc=6, seed=31, u_thi=0.02)
    rng = np.random.default_rng(31)
    st.uf[...] = 0.05 * rng.standard_normal(st.uf.shape)
    q, r = p.charges()
    g = Pic2D(p, precision="fp64")
    g.put_state(st)
    ref = g.energy()

    up_d = torch.from_numpy(np.ravel(st.up, order="F").copy()).cuda()
    np2_d = torch.from_numpy(np.ravel(st.np2, order="F").copy()).cuda()
    uf_d = torch.from_numpy(np.ravel(st.uf, order="F").copy()).cuda()
    out_d = torch.full((p.nsp + 2,), float("nan"), dtype=torch.float64, device="cuda")
    rr = np.ascontiguousarray(r, dtype=np.float64)
    f = _bind(gpu_lib)
    for _ in range(2):
        status = f(up_d.data_ptr(), np2_d.data_ptr(), uf_d.data_ptr(), p.ndim, p.np_cap, p.nx, p.ny, p.nsp,
                   rr.ctypes.data_as(ctypes.c_void_p), p.c, out_d.data_ptr(), None)
        assert status == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(out_d.cpu().numpy(), ref, rtol=RTOL)
        out_d.fill_(float("nan"))

    # a grid beyond the scratch size is refused before anything is launched
    status = f(up_d.data_ptr(), np2_d.data_ptr(), uf_d.data_ptr(), p.ndim, p.np_cap, p.nx, 8193, 1,
               rr.ctypes.data_as(ctypes.c_void_p), p.c, out_d.data_ptr(), None)
    assert status == 6  # WPIC_BAD_ARGUMENT
