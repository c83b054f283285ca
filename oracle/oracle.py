"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, always as the checker.  It wraps oracle/oracle2d.cpp and
oracle/oracle3d.cpp, restatements of WumingPIC's Fortran time step in the
reference's own array layout.  Parity status: unpinned (the reference has no
golden vectors for this path and cannot be compiled in this image).

Arrays follow the reference layout exactly, as numpy arrays in Fortran order:
  2D: up/gp (ndim, np, ny, nsp) float64, uf (6, nx+4, ny+4), uj (3, nx+4, ny+4),
      cumcnt (nx+1, ny, nsp) int32, np2 (ny, nsp) int32
  3D: up/gp (ndim, np, ny, nz, nsp), uf (6, nx+4, ny+4, nz+4), cumcnt (nx+1, ny, nz, nsp),
      np2 (ny, nz, nsp)
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

OK, CG_NOT_CONVERGED, CAPACITY, OUT_OF_RANGE = 0, 1, 2, 3
BC_PERIODIC, BC_RECONNECTION, BC_SHOCK = 0, 1, 2

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"oracle library not built: {LIB_PATH} (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        vp, dp, ip, i, d = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc2d_create.restype = vp
        L.orc2d_create.argtypes = [i] * 9 + [d, d, d, dp, dp, d, i]
        L.orc2d_destroy.argtypes = [vp]
        L.orc2d_set_threads.argtypes = [vp, i]
        L.orc2d_cg_control.argtypes = [vp, ip, i]
        L.orc2d_cg_iters.argtypes = [vp, ip]
        for n in ("orc2d_get_df", "orc2d_set_df", "orc2d_get_uj"):
            getattr(L, n).argtypes = [vp, dp]
        L.orc2d_particle_solv.argtypes = [vp, dp, dp, dp, ip, i, i]
        L.orc2d_particle_solv_vay.argtypes = [vp, dp, dp, dp, ip, i, i]
        L.orc2d_mom_calc_accl.argtypes = [vp, dp, dp, dp, ip, i, i]
        L.orc2d_mom_calc_nvt.argtypes = [vp, dp, dp, ip]
        L.orc2d_bc_mom.argtypes = [vp, dp]
        L.orc2d_bc_injection.argtypes = [vp, dp, ip, i, i, d]
        L.orc2d_ele_cur.argtypes = [vp, dp, dp, dp, ip, i, i]
        L.orc2d_bc_curre.argtypes = [vp, dp, i, i]
        L.orc2d_bc_dfield.argtypes = [vp, dp, i, i]
        L.orc2d_bc_phi.argtypes = [vp, dp, i, i, i]
        L.orc2d_cgm.argtypes = [vp, dp, dp, i, i]
        L.orc2d_field_fdtd_i.argtypes = [vp, dp, dp, dp, ip, i, i]
        L.orc2d_bc_particle_x.argtypes = [vp, dp, ip, i, i]
        L.orc2d_bc_particle_y.argtypes = [vp, dp, ip]
        L.orc2d_sort_bucket.argtypes = [vp, dp, dp, ip, ip, i, i]
        L.orc2d_energy.argtypes = [vp, dp, dp, ip, dp]
        if hasattr(L, "orc3d_create"):
            L.orc3d_create.restype = vp
            L.orc3d_create.argtypes = [i] * 13 + [d, d, d, dp, dp, d]
            L.orc3d_destroy.argtypes = [vp]
            L.orc3d_set_threads.argtypes = [vp, i]
            L.orc3d_set_bc.argtypes = [vp, i]
            L.orc3d_cg_control.argtypes = [vp, ip, i]
            L.orc3d_cg_iters.argtypes = [vp, ip]
            for n in ("orc3d_get_df", "orc3d_get_uj"):
                getattr(L, n).argtypes = [vp, dp]
            L.orc3d_particle_solv.argtypes = [vp, dp, dp, dp, ip, i, i]
            L.orc3d_particle_solv_vay.argtypes = [vp, dp, dp, dp, ip, i, i]
            L.orc3d_mom_calc_accl.argtypes = [vp, dp, dp, dp, ip, i, i]
            L.orc3d_mom_calc_nvt.argtypes = [vp, dp, dp, ip]
            L.orc3d_bc_mom.argtypes = [vp, dp]
            L.orc3d_ele_cur.argtypes = [vp, dp, dp, dp, ip, i, i]
            L.orc3d_bc_curre.argtypes = [vp, dp, i, i]
            L.orc3d_bc_dfield.argtypes = [vp, dp, i, i]
            L.orc3d_bc_injection.argtypes = [vp, dp, ip, i, i, d]
            L.orc3d_field_fdtd_i.argtypes = [vp, dp, dp, dp, ip, i, i]
            L.orc3d_bc_particle_x.argtypes = [vp, dp, ip]
            L.orc3d_bc_particle_yz.argtypes = [vp, dp, ip]
            L.orc3d_sort_bucket.argtypes = [vp, dp, dp, ip, ip, i, i]
            L.orc3d_energy.argtypes = [vp, dp, dp, ip, dp]
        _lib = L
    return _lib


def _p(a, dtype):
    assert a.dtype == dtype, (a.dtype, dtype)
    assert a.flags.f_contiguous or a.ndim == 1, "reference-layout arrays must be Fortran ordered"
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle2D:
    """One oracle instance = the SAVEd module state of particle/field/sort/boundary."""

    def __init__(self, *, nx, ny, np_cap, nsp=2, ndim=6, delx=1.0, delt=0.5, c=1.0, q, r, gfac=0.501,
                 bc="periodic", threads=1, nxgs=2, nygs=2):
        self.nx, self.ny, self.np, self.nsp, self.ndim = nx, ny, np_cap, nsp, ndim
        self.nxgs, self.nxge = nxgs, nxgs + nx - 1
        self.nygs, self.nyge = nygs, nygs + ny - 1
        self.nxs, self.nxe = self.nxgs, self.nxge
        self.bc = {"periodic": BC_PERIODIC, "reconnection": BC_RECONNECTION, "shock": BC_SHOCK}[bc]
        self.u0 = 0.0  # upstream four-velocity of the shock injection boundary
        q = np.ascontiguousarray(q, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        self._h = lib().orc2d_create(ndim, np_cap, nsp, self.nxgs, self.nxge, self.nygs, self.nyge, self.nygs,
                                     self.nyge, delx, delt, c, _p(q, np.float64), _p(r, np.float64), gfac, self.bc)
        lib().orc2d_set_threads(self._h, threads)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc2d_destroy(h)
            self._h = None

    def set_threads(self, n):
        lib().orc2d_set_threads(self._h, n)

    def cg_control(self, fixed=None, ite_max=100):
        if fixed is None:
            lib().orc2d_cg_control(self._h, None, ite_max)
        else:
            f = np.ascontiguousarray(fixed, dtype=np.int32)
            lib().orc2d_cg_control(self._h, _p(f, np.int32), ite_max)

    def cg_iters(self):
        out = np.zeros(3, np.int32)
        lib().orc2d_cg_iters(self._h, _p(out, np.int32))
        return out

    def field_shape(self, ncomp=6):
        return (ncomp, self.nx + 4, self.ny + 4)

    def get_df(self):
        out = np.zeros(self.field_shape(6), order="F")
        lib().orc2d_get_df(self._h, _p(out, np.float64))
        return out

    def set_df(self, df):
        lib().orc2d_set_df(self._h, _p(np.asfortranarray(df, dtype=np.float64), np.float64))

    def get_uj(self):
        out = np.zeros(self.field_shape(3), order="F")
        lib().orc2d_get_uj(self._h, _p(out, np.float64))
        return out

    # ---- the module procedures ----
    def particle_solv(self, gp, up, uf, cumcnt):
        return lib().orc2d_particle_solv(self._h, _p(gp, np.float64), _p(up, np.float64), _p(uf, np.float64),
                                         _p(cumcnt, np.int32), self.nxs, self.nxe)

    def particle_solv_vay(self, gp, up, uf, cumcnt):
        return lib().orc2d_particle_solv_vay(self._h, _p(gp, np.float64), _p(up, np.float64), _p(uf, np.float64),
                                             _p(cumcnt, np.int32), self.nxs, self.nxe)

    def mom_shape(self):
        """mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp)"""
        return (7, self.nx + 2, self.ny + 2, self.nsp)

    def mom_calc_accl(self, gp, up, uf, cumcnt):
        return lib().orc2d_mom_calc_accl(self._h, _p(gp, np.float64), _p(up, np.float64), _p(uf, np.float64),
                                         _p(cumcnt, np.int32), self.nxs, self.nxe)

    def mom_calc_nvt(self, mom, up, np2):
        return lib().orc2d_mom_calc_nvt(self._h, _p(mom, np.float64), _p(up, np.float64), _p(np2, np.int32))

    def bc_mom(self, mom):
        return lib().orc2d_bc_mom(self._h, _p(mom, np.float64))

    def set_window(self, nxs, nxe):
        """the active x window nxs..nxe that the driver passes to every call (the shock
        driver's expanding box, 2d/proj/shock/app.f90:276-277, 615-625)"""
        self.nxs, self.nxe = int(nxs), int(nxe)

    def bc_injection(self, up, np2, u0=None):
        return lib().orc2d_bc_injection(self._h, _p(up, np.float64), _p(np2, np.int32), self.nxs, self.nxe,
                                        self.u0 if u0 is None else u0)

    def moments(self, st):
        """The driver's diagnostic block (2d/proj/weibel/app.f90:121-123) on a State2D:
        mom_calc__accl into st.gp, mom_calc__nvt from st.gp, bc__mom.  Returns (status, mom)."""
        mom = np.zeros(self.mom_shape(), order="F")
        rc = self.mom_calc_accl(st.gp, st.up, st.uf, st.cumcnt)
        rc = rc or self.mom_calc_nvt(mom, st.gp, st.np2)
        rc = rc or self.bc_mom(mom)
        return rc, mom

    def ele_cur(self, uj, up, gp, cumcnt):
        return lib().orc2d_ele_cur(self._h, _p(uj, np.float64), _p(up, np.float64), _p(gp, np.float64),
                                   _p(cumcnt, np.int32), self.nxs, self.nxe)

    def bc_curre(self, uj):
        return lib().orc2d_bc_curre(self._h, _p(uj, np.float64), self.nxs, self.nxe)

    def bc_dfield(self, df):
        return lib().orc2d_bc_dfield(self._h, _p(df, np.float64), self.nxs, self.nxe)

    def cgm(self, db, gkl):
        return lib().orc2d_cgm(self._h, _p(db, np.float64), _p(gkl, np.float64), self.nxs, self.nxe)

    def field_fdtd_i(self, uf, up, gp, cumcnt):
        return lib().orc2d_field_fdtd_i(self._h, _p(uf, np.float64), _p(up, np.float64), _p(gp, np.float64),
                                        _p(cumcnt, np.int32), self.nxs, self.nxe)

    def bc_particle_x(self, up, np2):
        return lib().orc2d_bc_particle_x(self._h, _p(up, np.float64), _p(np2, np.int32), self.nxs, self.nxe)

    def bc_particle_y(self, up, np2):
        return lib().orc2d_bc_particle_y(self._h, _p(up, np.float64), _p(np2, np.int32))

    def sort_bucket(self, gp, up, cumcnt, np2):
        return lib().orc2d_sort_bucket(self._h, _p(gp, np.float64), _p(up, np.float64), _p(cumcnt, np.int32),
                                       _p(np2, np.int32), self.nxs, self.nxe)

    def energy(self, up, uf, np2):
        out = np.zeros(self.nsp + 2)
        lib().orc2d_energy(self._h, _p(up, np.float64), _p(uf, np.float64), _p(np2, np.int32),
                           _p(out, np.float64))
        return out

    def step(self, st, pusher="boris"):
        """One reference time step on a State2D, in the driver's call order
        (2d/proj/weibel/app.f90:102-107; reconnection: 2d/proj/reconnection/app.f90:101-106);
        pusher="vay" calls particle__solv_vay in place of particle__solv."""
        push = self.particle_solv_vay if pusher == "vay" else self.particle_solv
        rc = push(st.gp, st.up, st.uf, st.cumcnt)
        if self.bc == BC_RECONNECTION:
            rc = rc or self.bc_particle_x(st.gp, st.np2)
        if self.bc == BC_SHOCK:  # 2d/proj/shock/app.f90:110-115
            rc = rc or self.bc_injection(st.gp, st.np2)
        rc = rc or self.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt)
        if self.bc == BC_PERIODIC:
            rc = rc or self.bc_particle_x(st.gp, st.np2)
        rc = rc or self.bc_particle_y(st.gp, st.np2)
        rc = rc or self.sort_bucket(st.up, st.gp, st.cumcnt, st.np2)
        return rc


class Oracle3D:
    """3D oracle instance: the SAVEd module state of particle/field/sort/boundary; bc "periodic"
    (3d/common/boundary_periodic.f90) or "reconnection" (conducting walls in x,
    3d/proj/reconnection/boundary_reconnection.f90)."""

    def __init__(self, *, nx, ny, nz, np_cap, nsp=2, ndim=7, delx=1.0, delt=0.5, c=1.0, q, r, gfac=0.501,
                 threads=1, nxgs=2, nygs=2, nzgs=2, bc="periodic"):
        self.nx, self.ny, self.nz, self.np, self.nsp, self.ndim = nx, ny, nz, np_cap, nsp, ndim
        self.nxgs, self.nxge = nxgs, nxgs + nx - 1
        self.nygs, self.nyge = nygs, nygs + ny - 1
        self.nzgs, self.nzge = nzgs, nzgs + nz - 1
        self.nxs, self.nxe = self.nxgs, self.nxge
        q = np.ascontiguousarray(q, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        self._h = lib().orc3d_create(ndim, np_cap, nsp, self.nxgs, self.nxge, self.nygs, self.nyge, self.nzgs,
                                     self.nzge, self.nygs, self.nyge, self.nzgs, self.nzge, delx, delt, c,
                                     _p(q, np.float64), _p(r, np.float64), gfac)
        lib().orc3d_set_threads(self._h, threads)
        self.bc = bc
        self.u0 = 0.0
        lib().orc3d_set_bc(self._h, {"periodic": 0, "reconnection": 1, "shock": 2}[bc])

    def set_window(self, nxs, nxe):
        """the active x window nxs..nxe the shock driver passes (3d/proj/shock/app.f90:112-117, 654)"""
        self.nxs, self.nxe = int(nxs), int(nxe)

    def bc_injection(self, up, np2, u0=None):
        return lib().orc3d_bc_injection(self._h, _p(up, np.float64), _p(np2, np.int32), self.nxs, self.nxe,
                                        self.u0 if u0 is None else u0)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc3d_destroy(h)
            self._h = None

    def set_threads(self, n):
        lib().orc3d_set_threads(self._h, n)

    def cg_control(self, fixed=None, ite_max=100):
        if fixed is None:
            lib().orc3d_cg_control(self._h, None, ite_max)
        else:
            f = np.ascontiguousarray(fixed, dtype=np.int32)
            lib().orc3d_cg_control(self._h, _p(f, np.int32), ite_max)

    def cg_iters(self):
        out = np.zeros(3, np.int32)
        lib().orc3d_cg_iters(self._h, _p(out, np.int32))
        return out

    def field_shape(self, ncomp=6):
        return (ncomp, self.nx + 4, self.ny + 4, self.nz + 4)

    def get_df(self):
        out = np.zeros(self.field_shape(6), order="F")
        lib().orc3d_get_df(self._h, _p(out, np.float64))
        return out

    def get_uj(self):
        out = np.zeros(self.field_shape(3), order="F")
        lib().orc3d_get_uj(self._h, _p(out, np.float64))
        return out

    def particle_solv(self, gp, up, uf, cumcnt):
        return lib().orc3d_particle_solv(self._h, _p(gp, np.float64), _p(up, np.float64), _p(uf, np.float64),
                                         _p(cumcnt, np.int32), self.nxs, self.nxe)

    def particle_solv_vay(self, gp, up, uf, cumcnt):
        return lib().orc3d_particle_solv_vay(self._h, _p(gp, np.float64), _p(up, np.float64), _p(uf, np.float64),
                                             _p(cumcnt, np.int32), self.nxs, self.nxe)

    def mom_shape(self):
        """mom(7, nxgs-1:nxge+1, nys-1:nye+1, nzs-1:nze+1, nsp)"""
        return (7, self.nx + 2, self.ny + 2, self.nz + 2, self.nsp)

    def mom_calc_accl(self, gp, up, uf, cumcnt):
        return lib().orc3d_mom_calc_accl(self._h, _p(gp, np.float64), _p(up, np.float64), _p(uf, np.float64),
                                         _p(cumcnt, np.int32), self.nxs, self.nxe)

    def mom_calc_nvt(self, mom, up, np2):
        return lib().orc3d_mom_calc_nvt(self._h, _p(mom, np.float64), _p(up, np.float64), _p(np2, np.int32))

    def bc_mom(self, mom):
        return lib().orc3d_bc_mom(self._h, _p(mom, np.float64))

    def moments(self, st):
        """The 3D driver's diagnostic block (3d/proj/weibel/app.f90:122-124) on a State3D.
        Returns (status, mom)."""
        mom = np.zeros(self.mom_shape(), order="F")
        rc = self.mom_calc_accl(st.gp, st.up, st.uf, st.cumcnt)
        rc = rc or self.mom_calc_nvt(mom, st.gp, st.np2)
        rc = rc or self.bc_mom(mom)
        return rc, mom

    def ele_cur(self, uj, up, gp, cumcnt):
        return lib().orc3d_ele_cur(self._h, _p(uj, np.float64), _p(up, np.float64), _p(gp, np.float64),
                                   _p(cumcnt, np.int32), self.nxs, self.nxe)

    def bc_curre(self, uj):
        return lib().orc3d_bc_curre(self._h, _p(uj, np.float64), self.nxs, self.nxe)

    def bc_dfield(self, df):
        return lib().orc3d_bc_dfield(self._h, _p(df, np.float64), self.nxs, self.nxe)

    def field_fdtd_i(self, uf, up, gp, cumcnt):
        return lib().orc3d_field_fdtd_i(self._h, _p(uf, np.float64), _p(up, np.float64), _p(gp, np.float64),
                                        _p(cumcnt, np.int32), self.nxs, self.nxe)

    def bc_particle_x(self, up, np2):
        return lib().orc3d_bc_particle_x(self._h, _p(up, np.float64), _p(np2, np.int32))

    def bc_particle_yz(self, up, np2):
        return lib().orc3d_bc_particle_yz(self._h, _p(up, np.float64), _p(np2, np.int32))

    def sort_bucket(self, gp, up, cumcnt, np2):
        return lib().orc3d_sort_bucket(self._h, _p(gp, np.float64), _p(up, np.float64), _p(cumcnt, np.int32),
                                       _p(np2, np.int32), self.nxs, self.nxe)

    def energy(self, up, uf, np2):
        out = np.zeros(self.nsp + 2)
        lib().orc3d_energy(self._h, _p(up, np.float64), _p(uf, np.float64), _p(np2, np.int32),
                           _p(out, np.float64))
        return out

    def step(self, st, pusher="boris"):
        """One reference time step on a State3D, in the driver's call order
        (3d/proj/weibel/app.f90:103-108; reconnection, particle_x before the field solve:
        3d/proj/reconnection/app.f90:103-108); pusher="vay" calls particle__solv_vay."""
        push = self.particle_solv_vay if pusher == "vay" else self.particle_solv
        rc = push(st.gp, st.up, st.uf, st.cumcnt)
        if self.bc == "reconnection":
            rc = rc or self.bc_particle_x(st.gp, st.np2)
        if self.bc == "shock":  # 3d/proj/shock/app.f90:112-117: injection, no particle_x
            rc = rc or self.bc_injection(st.gp, st.np2)
        rc = rc or self.field_fdtd_i(st.uf, st.up, st.gp, st.cumcnt)
        if self.bc == "periodic":
            rc = rc or self.bc_particle_x(st.gp, st.np2)
        rc = rc or self.bc_particle_yz(st.gp, st.np2)
        rc = rc or self.sort_bucket(st.up, st.gp, st.cumcnt, st.np2)
        return rc
