"""Host-side mirror of WumingPIC's 2D module interface over the C ABI.

``Pic2D`` holds one device context and exposes the reference's procedure
names (particle__solv, field__fdtd_i, bc__particle_x, bc__particle_y,
sort__bucket) acting on device-resident state, plus the reference-layout state
exchange a Fortran driver needs at its I/O points.  Errors that the reference
reports with ``stop`` raise ``WpicError`` carrying the status code.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .loader import Plasma2D, State2D, empty_state2d


def _ptr(a, dtype):
    assert a.dtype == dtype and (a.flags.f_contiguous or a.ndim == 1), (a.dtype, a.flags)
    return a.ctypes.data_as(ctypes.c_void_p)


class Pic2D:
    def __init__(self, plasma: Plasma2D, precision="fp64", stream=None, device_cap=0):
        self.p = plasma
        q, r = plasma.charges()
        prm = _lib.WpicParams()
        prm.ndim, prm.np, prm.nsp = plasma.ndim, plasma.np_cap, plasma.nsp
        prm.nxgs, prm.nxge = plasma.nxgs, plasma.nxge
        prm.nygs, prm.nyge = plasma.nygs, plasma.nyge
        prm.nys, prm.nye = plasma.nygs, plasma.nyge
        prm.delx, prm.delt, prm.c, prm.gfac = plasma.delx, plasma.delt, plasma.c, plasma.gfac
        prm.q[0], prm.q[1] = q[0], q[1]
        prm.r[0], prm.r[1] = r[0], r[1]
        prm.bc_kind = {"periodic": _lib.BC_PERIODIC, "reconnection": _lib.BC_RECONNECTION,
                       "shock": _lib.BC_SHOCK}[plasma.bc]
        prm.precision = {"fp64": _lib.FP64, "fp64_exact": _lib.FP64_EXACT, "mixed": _lib.MIXED}[precision]
        prm.device_cap = int(device_cap)
        self.precision = precision
        h = ctypes.c_void_p()
        check(lib().wpic_init_2d(ctypes.byref(h), ctypes.byref(prm), ctypes.c_void_p(stream or 0)), "wpic_init_2d")
        self._h = h
        if plasma.bc == "shock":
            self.set_window(plasma.nxgs, plasma.nxe)
            self.set_injection(plasma.u0)

    def close(self):
        if getattr(self, "_h", None):
            lib().wpic_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    # ---- state exchange (reference layout) ----
    def put_state(self, st: State2D, gp=False):
        check(lib().wpic_put_particles(self._h, 0, _ptr(st.up, np.float64), _ptr(st.np2, np.int32),
                                       _ptr(st.cumcnt, np.int32)), "put up")
        if gp:
            check(lib().wpic_put_particles(self._h, 1, _ptr(st.gp, np.float64), _ptr(st.np2, np.int32), None),
                  "put gp")
        check(lib().wpic_put_fields(self._h, _ptr(st.uf, np.float64)), "put uf")

    def get_state(self, st: State2D = None) -> State2D:
        if st is None:
            st = empty_state2d(self.p)
        check(lib().wpic_get_particles(self._h, 0, _ptr(st.up, np.float64), _ptr(st.np2, np.int32),
                                       _ptr(st.cumcnt, np.int32)), "get up")
        if self.precision != "mixed":
            check(lib().wpic_get_particles(self._h, 1, _ptr(st.gp, np.float64), None, None), "get gp")
        check(lib().wpic_get_fields(self._h, _ptr(st.uf, np.float64)), "get uf")
        return st

    def put_particles(self, which, up, np2, cumcnt=None):
        check(lib().wpic_put_particles(self._h, which, _ptr(up, np.float64), _ptr(np2, np.int32),
                                       None if cumcnt is None else _ptr(cumcnt, np.int32)), "put particles")

    def get_particles(self, which):
        p = self.p
        up = np.zeros((p.ndim, p.np_cap, p.ny, p.nsp), order="F")
        np2 = np.zeros((p.ny, p.nsp), np.int32, order="F")
        cc = np.zeros((p.nx + 1, p.ny, p.nsp), np.int32, order="F")
        check(lib().wpic_get_particles(self._h, which, _ptr(up, np.float64), _ptr(np2, np.int32),
                                       _ptr(cc, np.int32)), "get particles")
        return up, np2, cc

    def put_fields(self, uf):
        check(lib().wpic_put_fields(self._h, _ptr(np.asfortranarray(uf), np.float64)), "put uf")

    def get_fields(self):
        uf = np.zeros((6, self.p.nx + 4, self.p.ny + 4), order="F")
        check(lib().wpic_get_fields(self._h, _ptr(uf, np.float64)), "get uf")
        return uf

    def get_df(self):
        df = np.zeros((6, self.p.nx + 4, self.p.ny + 4), order="F")
        check(lib().wpic_get_df(self._h, _ptr(df, np.float64)), "get df")
        return df

    def put_df(self, df):
        check(lib().wpic_put_df(self._h, _ptr(np.asfortranarray(df), np.float64)), "put df")

    def get_uj(self):
        uj = np.zeros((3, self.p.nx + 4, self.p.ny + 4), order="F")
        check(lib().wpic_get_uj(self._h, _ptr(uj, np.float64)), "get uj")
        return uj

    # ---- the module procedures ----
    def particle__solv(self):
        check(lib().wpic_particle_solv(self._h), "particle__solv")

    def cg_tolerance(self, rtol, ite_max=1000):
        """CG stopping tolerance relative to ||b|| (the reference's 1e-6) and iteration limit"""
        check(lib().wpic_cg_tolerance(self._h, float(rtol), int(ite_max)), "cg_tolerance")

    def adjoint(self, nsteps, every, lam_uf_final):
        """Run nsteps steps from the current state and return the gradient of a scalar with
        respect to the initial particles (layout of up) and fields (layout of uf), given its
        gradient with respect to the final fields."""
        p = self.p
        lam_uf_final = np.asfortranarray(lam_uf_final, dtype=np.float64)
        lup = np.zeros((p.ndim, p.np_cap, p.ny, p.nsp), order="F")
        luf = np.zeros((6, p.nx + 4, p.ny + 4), order="F")
        check(lib().wpic_adjoint(self._h, int(nsteps), int(every), _ptr(lam_uf_final, np.float64),
                                 _ptr(lup, np.float64), _ptr(luf, np.float64)), "adjoint")
        return lup, luf

    def adjoint_precision(self, precision):
        """Arithmetic of the reverse push and deposit sweeps: "fp64" (default) or "mixed"
        (FP32 per particle along the recorded FP64 trajectory; fields, adjoint CG and all
        accumulations in FP64)."""
        code = {"fp64": _lib.FP64, "fp64_exact": _lib.FP64_EXACT, "mixed": _lib.MIXED}[precision]
        check(lib().wpic_adjoint_precision(self._h, code), "adjoint_precision")

    def adjoint_keep_fields(self, keep=True):
        """Keep every recorded step's field state (default) so that the reverse sweep
        recomputes a segment by pushing and sorting only; False recomputes the full steps.
        Both give the same gradient bit for bit; read by the next adjoint_record."""
        check(lib().wpic_adjoint_keep_fields(self._h, int(bool(keep))), "adjoint_keep_fields")

    def adjoint_record(self, nsteps, every):
        """The forward half of ``adjoint``: run nsteps steps keeping the state every `every` steps."""
        check(lib().wpic_adjoint_record(self._h, int(nsteps), int(every)), "adjoint_record")

    def adjoint_reverse(self, lam_uf_final):
        """The reverse half of ``adjoint`` for the recorded run: (lam_up0, lam_uf0)."""
        p = self.p
        lam_uf_final = np.asfortranarray(lam_uf_final, dtype=np.float64)
        lup = np.zeros((p.ndim, p.np_cap, p.ny, p.nsp), order="F")
        luf = np.zeros((6, p.nx + 4, p.ny + 4), order="F")
        check(lib().wpic_adjoint_reverse(self._h, _ptr(lam_uf_final, np.float64), _ptr(lup, np.float64),
                                         _ptr(luf, np.float64)), "adjoint_reverse")
        return lup, luf

    def adjoint_selfcheck(self):
        """relative <L x, y> - <x, L^T y> of the adjoint's transposed field operators
        (fold, ghost copies, E update, RHS, averaging); overwrites the fields"""
        out = np.zeros(5)
        check(lib().wpic_adjoint_selfcheck(self._h, _ptr(out, np.float64)), "adjoint_selfcheck")
        return out

    def adjoint_pushcheck(self, h=1e-6):
        """(central difference, adjoint) of the push along a random field direction"""
        out = np.zeros(2)
        check(lib().wpic_adjoint_pushcheck(self._h, float(h), _ptr(out, np.float64)), "adjoint_pushcheck")
        return out

    def adjoint_depositcheck(self, h=1e-6):
        """(central difference, adjoint) of the deposit along random particle directions"""
        out = np.zeros(2)
        check(lib().wpic_adjoint_depositcheck(self._h, float(h), _ptr(out, np.float64)), "adjoint_depositcheck")
        return out

    def adjoint_chaincheck(self, h=1e-6):
        """(central difference, adjoint) of fields -> push -> deposit along random fields"""
        out = np.zeros(2)
        check(lib().wpic_adjoint_chaincheck(self._h, float(h), _ptr(out, np.float64)), "adjoint_chaincheck")
        return out

    def set_window(self, nxs, nxe):
        """the active x window nxs..nxe (the shock driver's expanding box)"""
        check(lib().wpic_set_window(self._h, int(nxs), int(nxe)), "set_window")

    def set_injection(self, u0):
        check(lib().wpic_set_injection(self._h, float(u0)), "set_injection")

    def bc__injection(self, u0):
        check(lib().wpic_bc_injection(self._h, float(u0)), "bc__injection")

    def particle__solv_vay(self):
        check(lib().wpic_particle_solv_vay(self._h), "particle__solv_vay")

    def set_pusher(self, name):
        """the push of the fused step: "boris" (particle__solv) or "vay" (particle__solv_vay)"""
        check(lib().wpic_set_pusher(self._h, {"boris": _lib.PUSH_BORIS, "vay": _lib.PUSH_VAY}[name]), "set_pusher")

    def field__fdtd_i(self):
        check(lib().wpic_field_fdtd_i(self._h), "field__fdtd_i")

    def ele_cur(self):
        check(lib().wpic_ele_cur(self._h), "ele_cur")

    def bc__particle_x(self):
        check(lib().wpic_bc_particle_x(self._h), "bc__particle_x")

    def bc__particle_y(self):
        check(lib().wpic_bc_particle_y(self._h), "bc__particle_y")

    def sort__bucket(self):
        check(lib().wpic_sort_bucket(self._h), "sort__bucket")

    def step(self, nsteps=1):
        check(lib().wpic_step(self._h, int(nsteps)), "step")

    # ---- moments (mom_calc__accl, mom_calc__nvt, bc__mom) ----
    def mom_shape(self):
        """mom(7, nxgs-1:nxge+1, nys-1:nye+1[, nzs-1:nze+1], nsp)"""
        return (7, self.p.nx + 2, self.p.ny + 2, self.p.nsp)

    def mom_calc__accl(self):
        check(lib().wpic_mom_calc_accl(self._h), "mom_calc__accl")

    def mom_calc__nvt(self, from_gp=True):
        check(lib().wpic_mom_calc_nvt(self._h, 1 if from_gp else 0), "mom_calc__nvt")

    def bc__mom(self):
        check(lib().wpic_bc_mom(self._h), "bc__mom")

    def get_mom(self):
        out = np.zeros(self.mom_shape(), order="F")
        check(lib().wpic_get_mom(self._h, _ptr(out, np.float64)), "get_mom")
        return out

    def moments(self, to_host=True):
        """accl + nvt + bc__mom; returns the host copy (or None with to_host=False)"""
        if not to_host:
            check(lib().wpic_moments(self._h, None), "moments")
            return None
        out = np.zeros(self.mom_shape(), order="F")
        check(lib().wpic_moments(self._h, _ptr(out, np.float64)), "moments")
        return out

    def energy(self):
        out = np.zeros(self.p.nsp + 2)
        check(lib().wpic_energy(self._h, _ptr(out, np.float64)), "energy")
        return out

    def cg_control(self, fixed=None, ite_max=100):
        if fixed is None:
            check(lib().wpic_cg_control(self._h, None, ite_max))
        else:
            f = np.ascontiguousarray(fixed, dtype=np.int32)
            check(lib().wpic_cg_control(self._h, _ptr(f, np.int32), ite_max))

    def cg_iters(self):
        out = np.zeros(3, np.int32)
        check(lib().wpic_cg_iters(self._h, _ptr(out, np.int32)))
        return out

    def load_weibel(self, seed=None):
        """Device-side seeded loading of the plasma described by self.p."""
        p = self.p
        b0 = np.ascontiguousarray(p.b0, dtype=np.float64)
        check(lib().wpic_load_weibel_2d(self._h, p.ppc, int(p.seed if seed is None else seed), p.drift,
                                        p.drift_axis, p.u_thi, p.u_the, _ptr(b0, np.float64)), "load")

    def num_particles(self):
        return lib().wpic_num_particles(self._h)

    def synchronize(self):
        check(lib().wpic_synchronize(self._h))

    # ---- stage timing ----
    def timing(self, enable=True):
        check(lib().wpic_timing_enable(self._h, 1 if enable else 0))

    def stage_times(self):
        n = lib().wpic_num_stages()
        ms = np.zeros(n)
        ln = np.zeros(n, np.int64)
        check(lib().wpic_timing_get(self._h, _ptr(ms, np.float64), _ptr(ln, np.int64), n))
        return {lib().wpic_stage_name(k).decode(): (float(ms[k]), int(ln[k])) for k in range(n)}
