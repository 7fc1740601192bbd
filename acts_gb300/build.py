"""In-tree build of the native libraries.

* acts_gb300/_lib/libcudakalman.so — the CUDA fitter and its C ABI
  (nvcc, sm_103a only).
* acts_gb300/_lib/libckgen.so — the synthetic event generator (g++).
* oracle/_build/libkforacle.so — the CPU oracle used by tests and the CPU
  baseline (make -C oracle).
* acts_gb300/_acts_gb300_ext*.so — the pybind11 module of
  makeKalmanFitterFunction over the C ABI, when pybind11 is importable
  (skipped otherwise; acts_gb300.track_fitting covers the same through
  ctypes).

Nothing is installed outside the repository; outputs are git-ignored.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not os.path.exists(NVCC):
    NVCC = shutil.which("nvcc") or NVCC
CXX = os.environ.get("CXX", "g++")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

# translation units of libcudakalman.so
CUDA_SOURCES = ["ck_kernels_fp64.cu", "ck_kernels_mixed.cu", "ck_units.cu", "ck_api.cu", "ck_static.cu",
                "ck_server.cu", "ck_extrapolate.cu", "ck_reverse_fp64.cu", "ck_reverse_mixed.cu",
                "ck_propagate.cu", "ck_ckf.cu", "ck_simulate.cu"]
CUDA_HEADERS = ["ck_device.cuh", "ck_fitter.cuh", "ck_internal.h", "ck_api_internal.h", "ck_launch.h",
                "ck_simulate.h"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_generator(force=False):
    os.makedirs(LIBDIR, exist_ok=True)
    out = os.path.join(LIBDIR, "libckgen.so")
    src = os.path.join(CSRC, "ck_generate.cpp")
    deps = [src, os.path.join(CSRC, "ck_simulate.h"), os.path.join(INCLUDE, "ckgen.h"),
            os.path.join(INCLUDE, "cudakalman.h")]
    if force or _stale(out, deps):
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + INCLUDE, "-I" + CSRC, src,
              "-o", out, "-lpthread"])
    return out


def build_pybind(force=False):
    """The pybind11 module, linked against libcudakalman.so (rpath $ORIGIN/_lib).
    Returns its path, or None when pybind11 is not importable."""
    try:
        import pybind11
    except ImportError:
        return None
    import sysconfig

    out = os.path.join(HERE, "_acts_gb300_ext" + sysconfig.get_config_var("EXT_SUFFIX"))
    src = os.path.join(CSRC, "ck_pybind.cpp")
    if force or _stale(out, [src, os.path.join(INCLUDE, "cudakalman.h")]):
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden",
              "-I" + INCLUDE, "-I" + pybind11.get_include(),
              "-I" + sysconfig.get_paths()["include"], src, "-o", out,
              "-L" + LIBDIR, "-lcudakalman", "-Wl,-rpath,$ORIGIN/_lib"])
    return out


def build_oracle(force=False):
    odir = os.path.join(ROOT, "oracle")
    if force:
        _run(["make", "-C", odir, "clean"])
    _run(["make", "-C", odir])
    return os.path.join(odir, "_build", "libkforacle.so")


def nvcc_flags(extra=()):
    return [NVCC, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-I" + INCLUDE, "-I" + CSRC, "--expt-relaxed-constexpr"] + list(extra)


def build_cuda(force=False, verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    out = os.path.join(LIBDIR, "libcudakalman.so")
    headers = [os.path.join(CSRC, h) for h in CUDA_HEADERS] + [os.path.join(INCLUDE, "cudakalman.h")]
    objs = []
    jobs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(objdir, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = nvcc_flags(["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
            jobs.append(cmd)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(out, objs):
        _run([NVCC, GENCODE, "-shared", "-o", out] + objs + ["-lcudart", "-lpthread"])
    return out, logs


def build_all(force=False, oracle=True, verbose=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        f_gen = ex.submit(build_generator, force)
        f_ora = ex.submit(build_oracle, force) if oracle else None
        f_cuda = ex.submit(build_cuda, force, verbose)
        res = {"generator": f_gen.result(), "cuda": f_cuda.result()[0]}
        if f_ora is not None:
            res["oracle"] = f_ora.result()
    res["pybind"] = build_pybind(force)
    return res


if __name__ == "__main__":
    force = "--force" in sys.argv
    verbose = "-v" in sys.argv
    if "--generator" in sys.argv:
        print(build_generator(force))
    elif "--oracle" in sys.argv:
        print(build_oracle(force))
    else:
        if verbose:
            out, logs = build_cuda(force, True)
            for l in logs:
                print(l)
        print(build_all(force, verbose=False))
