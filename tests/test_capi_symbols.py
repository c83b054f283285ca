"""The C-ABI library builds, loads without a GPU and exports every function
declared in include/*.h."""
import ctypes
import glob
import os
import re

from wumingpic_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(wpic(?:3d)?_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("wpic_init_2d", "wpic_particle_solv", "wpic_field_fdtd_i", "wpic_bc_particle_x",
              "wpic_bc_particle_y", "wpic_sort_bucket", "wpic_step", "wpic_energy",
              "wpic3d_init", "wpic3d_particle_solv", "wpic3d_field_fdtd_i", "wpic3d_bc_particle_x",
              "wpic3d_bc_particle_yz", "wpic3d_sort_bucket", "wpic3d_step", "wpic3d_energy"):
        assert n in names, n


def test_library_exports_every_declared_symbol():
    path = _build.build_library()
    lib = ctypes.CDLL(path)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_without_gpu():
    lib = ctypes.CDLL(_build.build_library())
    lib.wpic_status_string.restype = ctypes.c_char_p
    assert lib.wpic_status_string(0) == b"ok"
    assert b"capacity" in lib.wpic_status_string(2)
    lib.wpic_num_stages.restype = ctypes.c_int
    assert lib.wpic_num_stages() >= 5
    assert b"finalise" in lib.wpic_status_string(9)


def test_c_driver_builds_and_links_without_gpu():
    """The C program that drives the header in the Weibel driver's order compiles against the
    header, links against the library and answers a wrong command line before any device call."""
    import subprocess
    exe = _build.build_driver()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "usage" in r.stderr
