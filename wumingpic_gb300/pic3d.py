"""Host-side mirror of WumingPIC's 3D module interface over the C ABI.

``Pic3D`` holds one device context of the 3D FP64 path (periodic in x, y and z)
and exposes the reference's procedure names (particle__solv, field__fdtd_i,
bc__particle_x, bc__particle_yz, sort__bucket) acting on device-resident state,
plus the reference-layout state exchange a Fortran driver needs.  Errors that
the reference reports with ``stop`` raise ``WpicError`` with the status code.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .loader import Plasma3D, State3D, empty_state3d


def _ptr(a, dtype):
    assert a.dtype == dtype and (a.flags.f_contiguous or a.ndim == 1), (a.dtype, a.flags)
    return a.ctypes.data_as(ctypes.c_void_p)


class Pic3D:
    def __init__(self, plasma: Plasma3D, precision="fp64", stream=None, device_cap=0):
        self.p = plasma
        q, r = plasma.charges()
        prm = _lib.WpicParams3D()
        prm.ndim, prm.np, prm.nsp = plasma.ndim, plasma.np_cap, plasma.nsp
        prm.nxgs, prm.nxge = plasma.nxgs, plasma.nxge
        prm.nygs, prm.nyge = plasma.nygs, plasma.nyge
        prm.nzgs, prm.nzge = plasma.nzgs, plasma.nzge
        prm.nys, prm.nye = plasma.nygs, plasma.nyge
        prm.nzs, prm.nze = plasma.nzgs, plasma.nzge
        prm.delx, prm.delt, prm.c, prm.gfac = plasma.delx, plasma.delt, plasma.c, plasma.gfac
        prm.q[0], prm.q[1] = q[0], q[1]
        prm.r[0], prm.r[1] = r[0], r[1]
        prm.precision = {"fp64": _lib.FP64, "fp64_exact": _lib.FP64_EXACT, "mixed": _lib.MIXED}[precision]
        prm.device_cap = int(device_cap)
        prm.bc_kind = {"periodic": _lib.BC_PERIODIC, "reconnection": _lib.BC_RECONNECTION,
                       "shock": _lib.BC_SHOCK}[getattr(plasma, "bc", "periodic")]
        self.precision = precision
        h = ctypes.c_void_p()
        check(lib().wpic3d_init(ctypes.byref(h), ctypes.byref(prm), ctypes.c_void_p(stream or 0)), "wpic3d_init")
        self._h = h
        if getattr(plasma, "bc", "periodic") == "shock":
            self.set_window(plasma.nxgs, plasma.nxe)
            self.set_injection(plasma.u0)

    def set_window(self, nxs, nxe):
        """the active x window nxs..nxe of a shock run (3d/proj/shock/app.f90:112-117, 654)"""
        check(lib().wpic3d_set_window(self._h, int(nxs), int(nxe)), "set_window")

    def set_injection(self, u0):
        """the injection boundary's upstream four-velocity for step()"""
        check(lib().wpic3d_set_injection(self._h, float(u0)), "set_injection")

    def bc__injection(self, u0):
        """boundary_shock__injection on gp (3d/proj/shock/boundary_shock.f90:424)"""
        check(lib().wpic3d_bc_injection(self._h, float(u0)), "bc__injection")

    def close(self):
        if getattr(self, "_h", None):
            lib().wpic3d_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def _fshape(self, ncomp):
        p = self.p
        return (ncomp, p.nx + 4, p.ny + 4, p.nz + 4)

    # ---- state exchange (reference layout) ----
    def put_state(self, st: State3D, gp=False):
        check(lib().wpic3d_put_particles(self._h, 0, _ptr(st.up, np.float64), _ptr(st.np2, np.int32),
                                         _ptr(st.cumcnt, np.int32)), "put up")
        if gp:
            check(lib().wpic3d_put_particles(self._h, 1, _ptr(st.gp, np.float64), _ptr(st.np2, np.int32), None),
                  "put gp")
        check(lib().wpic3d_put_fields(self._h, _ptr(st.uf, np.float64)), "put uf")

    def get_state(self, st: State3D = None) -> State3D:
        if st is None:
            st = empty_state3d(self.p)
        check(lib().wpic3d_get_particles(self._h, 0, _ptr(st.up, np.float64), _ptr(st.np2, np.int32),
                                         _ptr(st.cumcnt, np.int32)), "get up")
        if self.precision != "mixed":  # the mixed path keeps no gp
            check(lib().wpic3d_get_particles(self._h, 1, _ptr(st.gp, np.float64), None, None), "get gp")
        check(lib().wpic3d_get_fields(self._h, _ptr(st.uf, np.float64)), "get uf")
        return st

    def put_particles(self, which, up, np2, cumcnt=None):
        check(lib().wpic3d_put_particles(self._h, which, _ptr(up, np.float64), _ptr(np2, np.int32),
                                         None if cumcnt is None else _ptr(cumcnt, np.int32)), "put particles")

    def get_particles(self, which):
        p = self.p
        up = np.zeros((p.ndim, p.np_cap, p.ny, p.nz, p.nsp), order="F")
        np2 = np.zeros((p.ny, p.nz, p.nsp), np.int32, order="F")
        cc = np.zeros((p.nx + 1, p.ny, p.nz, p.nsp), np.int32, order="F")
        check(lib().wpic3d_get_particles(self._h, which, _ptr(up, np.float64), _ptr(np2, np.int32),
                                         _ptr(cc, np.int32)), "get particles")
        return up, np2, cc

    def put_fields(self, uf):
        check(lib().wpic3d_put_fields(self._h, _ptr(np.asfortranarray(uf), np.float64)), "put uf")

    def get_fields(self):
        uf = np.zeros(self._fshape(6), order="F")
        check(lib().wpic3d_get_fields(self._h, _ptr(uf, np.float64)), "get uf")
        return uf

    def get_df(self):
        df = np.zeros(self._fshape(6), order="F")
        check(lib().wpic3d_get_df(self._h, _ptr(df, np.float64)), "get df")
        return df

    def put_df(self, df):
        check(lib().wpic3d_put_df(self._h, _ptr(np.asfortranarray(df), np.float64)), "put df")

    def get_uj(self):
        uj = np.zeros(self._fshape(3), order="F")
        check(lib().wpic3d_get_uj(self._h, _ptr(uj, np.float64)), "get uj")
        return uj

    # ---- the module procedures ----
    def particle__solv(self):
        check(lib().wpic3d_particle_solv(self._h), "particle__solv")

    def particle__solv_vay(self):
        check(lib().wpic3d_particle_solv_vay(self._h), "particle__solv_vay")

    def set_pusher(self, name):
        """the push of the fused step: "boris" (particle__solv) or "vay" (particle__solv_vay)"""
        check(lib().wpic3d_set_pusher(self._h, {"boris": _lib.PUSH_BORIS, "vay": _lib.PUSH_VAY}[name]), "set_pusher")

    def field__fdtd_i(self):
        check(lib().wpic3d_field_fdtd_i(self._h), "field__fdtd_i")

    def ele_cur(self):
        """ele_cur + bc__curre (the deposit half of field__fdtd_i)."""
        check(lib().wpic3d_ele_cur(self._h), "ele_cur")

    def bc__particle_x(self):
        check(lib().wpic3d_bc_particle_x(self._h), "bc__particle_x")

    def bc__particle_yz(self):
        check(lib().wpic3d_bc_particle_yz(self._h), "bc__particle_yz")

    def sort__bucket(self):
        check(lib().wpic3d_sort_bucket(self._h), "sort__bucket")

    def step(self, nsteps=1):
        check(lib().wpic3d_step(self._h, int(nsteps)), "step")

    # ---- moments (mom_calc__accl, mom_calc__nvt, bc__mom) ----
    def mom_shape(self):
        """mom(7, nxgs-1:nxge+1, nys-1:nye+1[, nzs-1:nze+1], nsp)"""
        return (7, self.p.nx + 2, self.p.ny + 2, self.p.nz + 2, self.p.nsp)

    def mom_calc__accl(self):
        check(lib().wpic3d_mom_calc_accl(self._h), "mom_calc__accl")

    def mom_calc__nvt(self, from_gp=True):
        check(lib().wpic3d_mom_calc_nvt(self._h, 1 if from_gp else 0), "mom_calc__nvt")

    def bc__mom(self):
        check(lib().wpic3d_bc_mom(self._h), "bc__mom")

    def get_mom(self):
        out = np.zeros(self.mom_shape(), order="F")
        check(lib().wpic3d_get_mom(self._h, _ptr(out, np.float64)), "get_mom")
        return out

    def moments(self, to_host=True):
        """accl + nvt + bc__mom; returns the host copy (or None with to_host=False)"""
        if not to_host:
            check(lib().wpic3d_moments(self._h, None), "moments")
            return None
        out = np.zeros(self.mom_shape(), order="F")
        check(lib().wpic3d_moments(self._h, _ptr(out, np.float64)), "moments")
        return out

    def energy(self):
        out = np.zeros(self.p.nsp + 2)
        check(lib().wpic3d_energy(self._h, _ptr(out, np.float64)), "energy")
        return out

    def cg_control(self, fixed=None, ite_max=100):
        if fixed is None:
            check(lib().wpic3d_cg_control(self._h, None, ite_max))
        else:
            f = np.ascontiguousarray(fixed, dtype=np.int32)
            check(lib().wpic3d_cg_control(self._h, _ptr(f, np.int32), ite_max))

    def cg_iters(self):
        out = np.zeros(3, np.int32)
        check(lib().wpic3d_cg_iters(self._h, _ptr(out, np.int32)))
        return out

    def load_weibel(self, seed=None):
        p = self.p
        check(lib().wpic3d_load_weibel(self._h, p.ppc, p.seed if seed is None else seed, p.drift, p.drift_axis,
                                       p.u_thi, p.u_the), "load_weibel")

    def num_particles(self):
        return lib().wpic3d_num_particles(self._h)

    def synchronize(self):
        check(lib().wpic3d_synchronize(self._h), "synchronize")
