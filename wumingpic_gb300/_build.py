"""In-tree build of the CUDA library and of the CPU oracle.

Both are plain compiler invocations run in parallel (no cmake, no setuptools):
  * wumingpic_gb300/_build/libwumingpic_gb300.so  -- the sm_103a kernels and the C ABI
    declared in include/wumingpic_gb300.h (nvcc, one -gencode);
  * oracle/_build/liboracle.so                    -- the CPU restatement used as checker
    (g++ -ffp-contract=off -frounding-math, OpenMP);
  * wumingpic_gb300/_build/wpic_driver2d           -- a C program that calls the C ABI in the
    2D Weibel driver's order (gcc, linked against the library).
Object files are rebuilt only when a source or header is newer.
"""
import glob
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "wumingpic_gb300")
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libwumingpic_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation units of the library and their extra flags.  The *_exact units are
# compiled without FMA contraction so that their arithmetic is the reference's
# operation-by-operation (bit-exact parity mode).
CUDA_UNITS = {
    "capi.cu": [],
    "kernels_fast.cu": [],
    "kernels_exact.cu": ["-fmad=false"],
    "kernels_common.cu": [],
    "mixed2d.cu": [],
    "probe.cu": [],
    "no_alloc.cu": [],
    "capi3d.cu": [],
    "kernels3d_common.cu": [],
    "mixed3d.cu": [],
    "adjoint2d.cu": [],
}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run_parallel(jobs):
    procs = []
    for cmd in jobs:
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errs = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errs.append(" ".join(cmd) + "\n" + out.decode(errors="replace"))
        elif out.strip():
            sys.stderr.write(out.decode(errors="replace"))
    if errs:
        raise RuntimeError("build failed:\n" + "\n".join(errs))


def build_library(verbose=False, extra=()):
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    nvcc = _nvcc()
    objs, jobs = [], []
    for unit, flags in CUDA_UNITS.items():
        src = os.path.join(CSRC, unit)
        if not os.path.exists(src):
            continue
        obj = os.path.join(LIB_DIR, unit.replace(".cu", ".o"))
        objs.append(obj)
        if _newer(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                   "-Xcompiler", "-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC, "--expt-relaxed-constexpr",
                   *flags, *extra, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    _run_parallel(jobs)
    if _newer(LIB_PATH, objs):
        _run_parallel([[nvcc, *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lcudart"]])
    return LIB_PATH


DRIVER_SRC = os.path.join(PKG, "driver", "wpic_driver2d.c")
DRIVER_BIN = os.path.join(LIB_DIR, "wpic_driver2d")


def build_driver():
    """The C driver program, linked against the built library (run path next to it)."""
    hdr = os.path.join(ROOT, "include", "wumingpic_gb300.h")
    if _newer(DRIVER_BIN, [DRIVER_SRC, hdr, LIB_PATH]):
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"), DRIVER_SRC,
               "-L", LIB_DIR, "-lwumingpic_gb300", "-Wl,-rpath,$ORIGIN", "-lm", "-o", DRIVER_BIN]
        _run_parallel([cmd])
    return DRIVER_BIN


def build_oracle():
    out_dir = os.path.join(ORACLE_DIR, "_build")
    os.makedirs(out_dir, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(ORACLE_DIR, "*.cpp")))
    if _newer(ORACLE_LIB, srcs):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-frounding-math", "-fno-fast-math", *srcs, "-o", ORACLE_LIB]
        _run_parallel([cmd])
    return ORACLE_LIB


def build_all(verbose=False):
    """Compile oracle and library concurrently."""
    import threading
    err = []

    def _o():
        try:
            build_oracle()
        except Exception as e:  # noqa: BLE001
            err.append(e)

    t = threading.Thread(target=_o)
    t.start()
    build_library(verbose=verbose)
    build_driver()
    t.join()
    if err:
        raise err[0]


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
