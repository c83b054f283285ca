"""ctypes binding of libwumingpic_gb300.so (the C ABI in include/wumingpic_gb300.h).

The library is built in-tree by ``__graft_entry__.build()``.  There is no CPU
fallback: if the shared library is missing, or no CUDA device is usable, the
calls fail with an exception.
"""
import ctypes
import os

from . import _build

LIB_PATH = _build.LIB_PATH

# status codes (include/wumingpic_gb300.h)
OK = 0
CG_NOT_CONVERGED = 1
CAPACITY = 2
OUT_OF_RANGE = 3
MOVED_TOO_FAR = 4
NONFINITE = 5
BAD_ARGUMENT = 6
CUDA_ERROR = 7
NOT_INITIALISED = 8
STAGING_TIMEOUT = 9

BC_PERIODIC = 0
BC_RECONNECTION = 1
BC_SHOCK = 2
FP64 = 0
FP64_EXACT = 1
MIXED = 2
PUSH_BORIS = 0
PUSH_VAY = 1


class WpicParams(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int), ("np", ctypes.c_int), ("nsp", ctypes.c_int),
        ("nxgs", ctypes.c_int), ("nxge", ctypes.c_int), ("nygs", ctypes.c_int), ("nyge", ctypes.c_int),
        ("nys", ctypes.c_int), ("nye", ctypes.c_int),
        ("delx", ctypes.c_double), ("delt", ctypes.c_double), ("c", ctypes.c_double), ("gfac", ctypes.c_double),
        ("q", ctypes.c_double * 2), ("r", ctypes.c_double * 2),
        ("bc_kind", ctypes.c_int), ("precision", ctypes.c_int), ("device_cap", ctypes.c_int),
    ]


class WpicParams3D(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int), ("np", ctypes.c_int), ("nsp", ctypes.c_int),
        ("nxgs", ctypes.c_int), ("nxge", ctypes.c_int), ("nygs", ctypes.c_int), ("nyge", ctypes.c_int),
        ("nzgs", ctypes.c_int), ("nzge", ctypes.c_int),
        ("nys", ctypes.c_int), ("nye", ctypes.c_int), ("nzs", ctypes.c_int), ("nze", ctypes.c_int),
        ("delx", ctypes.c_double), ("delt", ctypes.c_double), ("c", ctypes.c_double), ("gfac", ctypes.c_double),
        ("q", ctypes.c_double * 2), ("r", ctypes.c_double * 2),
        ("precision", ctypes.c_int), ("device_cap", ctypes.c_int), ("bc_kind", ctypes.c_int),
    ]


class WpicError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = status_string(status)
        super().__init__(f"{where}: wpic status {status} ({msg})" if where else f"wpic status {status} ({msg})")


_lib = None


def lib():
    """Load the CUDA library; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"CUDA library not built: {LIB_PATH}; run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
        L.wpic_init_2d.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(WpicParams), vp]
        L.wpic_finalize.argtypes = [vp]
        L.wpic_put_particles.argtypes = [vp, i, vp, vp, vp]
        L.wpic_get_particles.argtypes = [vp, i, vp, vp, vp]
        for n in ("wpic_put_fields", "wpic_get_fields", "wpic_put_df", "wpic_get_df", "wpic_get_uj"):
            getattr(L, n).argtypes = [vp, vp]
        L.wpic_set_pusher.argtypes = [vp, i]
        L.wpic_set_window.argtypes = [vp, i, i]
        L.wpic_cg_tolerance.argtypes = [vp, ctypes.c_double, i]
        L.wpic_adjoint.argtypes = [vp, i, i, vp, vp, vp]
        L.wpic_adjoint_record.argtypes = [vp, i, i]
        L.wpic_adjoint_precision.argtypes = [vp, i]
        L.wpic_adjoint_keep_fields.argtypes = [vp, i]
        L.wpic_adjoint_reverse.argtypes = [vp, vp, vp, vp]
        L.wpic_adjoint_selfcheck.argtypes = [vp, vp]
        L.wpic_adjoint_pushcheck.argtypes = [vp, ctypes.c_double, vp]
        L.wpic_adjoint_depositcheck.argtypes = [vp, ctypes.c_double, vp]
        L.wpic_adjoint_chaincheck.argtypes = [vp, ctypes.c_double, vp]
        L.wpic_set_injection.argtypes = [vp, ctypes.c_double]
        L.wpic_bc_injection.argtypes = [vp, ctypes.c_double]
        L.wpic3d_set_pusher.argtypes = [vp, i]
        L.wpic3d_set_window.argtypes = [vp, i, i]
        L.wpic3d_set_injection.argtypes = [vp, ctypes.c_double]
        L.wpic3d_bc_injection.argtypes = [vp, ctypes.c_double]
        for pre in ("wpic", "wpic3d"):
            getattr(L, pre + "_mom_calc_accl").argtypes = [vp]
            getattr(L, pre + "_mom_calc_nvt").argtypes = [vp, i]
            getattr(L, pre + "_bc_mom").argtypes = [vp]
            getattr(L, pre + "_get_mom").argtypes = [vp, vp]
            getattr(L, pre + "_moments").argtypes = [vp, vp]
        for n in ("wpic_particle_solv", "wpic_particle_solv_vay", "wpic_field_fdtd_i", "wpic_ele_cur",
                  "wpic_bc_particle_x",
                  "wpic_bc_particle_y", "wpic_sort_bucket", "wpic_synchronize"):
            getattr(L, n).argtypes = [vp]
        L.wpic_step.argtypes = [vp, i]
        L.wpic_energy.argtypes = [vp, vp]
        L.wpic_cg_control.argtypes = [vp, vp, i]
        L.wpic_cg_iters.argtypes = [vp, vp]
        L.wpic_load_weibel_2d.argtypes = [vp, i, ctypes.c_uint64, d, i, d, d, vp]
        L.wpic_timing_enable.argtypes = [vp, i]
        L.wpic_timing_get.argtypes = [vp, vp, vp, i]
        L.wpic_stage_name.argtypes = [i]
        L.wpic_stage_name.restype = ctypes.c_char_p
        L.wpic_num_stages.argtypes = []
        L.wpic_num_particles.argtypes = [vp]
        L.wpic_num_particles.restype = ll
        L.wpic_measure_fma_peak.argtypes = [i, vp]
        L.wpic_host_register.argtypes = [vp, ctypes.c_size_t]
        L.wpic_host_unregister.argtypes = [vp]
        L.wpic_status_string.argtypes = [i]
        L.wpic_status_string.restype = ctypes.c_char_p
        # 3D
        L.wpic3d_init.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(WpicParams3D), vp]
        L.wpic3d_finalize.argtypes = [vp]
        L.wpic3d_put_particles.argtypes = [vp, i, vp, vp, vp]
        L.wpic3d_get_particles.argtypes = [vp, i, vp, vp, vp]
        for n in ("wpic3d_put_fields", "wpic3d_get_fields", "wpic3d_put_df", "wpic3d_get_df", "wpic3d_get_uj"):
            getattr(L, n).argtypes = [vp, vp]
        for n in ("wpic3d_particle_solv", "wpic3d_particle_solv_vay", "wpic3d_field_fdtd_i", "wpic3d_ele_cur",
                  "wpic3d_bc_particle_x",
                  "wpic3d_bc_particle_yz",
                  "wpic3d_sort_bucket", "wpic3d_synchronize"):
            getattr(L, n).argtypes = [vp]
        L.wpic3d_step.argtypes = [vp, i]
        L.wpic3d_energy.argtypes = [vp, vp]
        L.wpic3d_cg_control.argtypes = [vp, vp, i]
        L.wpic3d_cg_iters.argtypes = [vp, vp]
        L.wpic3d_load_weibel.argtypes = [vp, i, ctypes.c_uint64, d, i, d, d]
        L.wpic3d_num_particles.argtypes = [vp]
        L.wpic3d_num_particles.restype = ll
        _lib = L
    return _lib


def fma_peak_gflops(fp64=True):
    out = ctypes.c_double()
    check(lib().wpic_measure_fma_peak(1 if fp64 else 0, ctypes.byref(out)), "fma peak")
    return out.value


def host_register(arr):
    """Page-lock a numpy array's buffer for fast host<->device copies."""
    check(lib().wpic_host_register(arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes), "host_register")


def host_unregister(arr):
    check(lib().wpic_host_unregister(arr.ctypes.data_as(ctypes.c_void_p)), "host_unregister")


def status_string(status):
    try:
        return lib().wpic_status_string(int(status)).decode()
    except ImportError:
        return "library not built"


def check(status, where=""):
    if status != OK:
        raise WpicError(status, where)
    return status
