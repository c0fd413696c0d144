"""Build the GB300 extension in-tree.

Outputs (git-ignored, rebuilt on every host, since GB300 hosts are aarch64 and build hosts may
be x86-64):
  hoomd-blue_gb300/hoomd_gb300/libhoomd_gb300.so   CUDA kernels + the C ABI (include/hoomd_gb300.h)
  hoomd-blue_gb300/hoomd_gb300/_hoomd_gb300*.so    C++ host engine behind pybind11; calls the
                                                   kernels only through the C ABI

Every CUDA translation unit is compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``), in parallel, with ``-lineinfo``. The pybind11 headers come from
the pybind11 package when installed, else from torch's bundled copy.
"""

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys
import sysconfig

PKG_ROOT = pathlib.Path(__file__).resolve().parent
REPO = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
OUT = PKG_ROOT / "hoomd_gb300"
BUILD = PKG_ROOT / "_build"
INCLUDE = REPO / "include"

CUDA_HOME = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["box_common.cu", "nlist.cu", "integrate.cu", "pair_lj.cu", "pair_table.cu",
              "pair_example.cu", "pair_radial.cu", "pair_radial_q.cu", "pair_dpd.cu", "sfc_sort.cu", "thermo_noalloc.cu", "replica.cu", "snapshot_io.cu",
              "mlp.cu"]
HOST_SOURCES = ["engine.cc", "npt.cc", "ensemble.cc", "surrogate.cc", "module.cc"]
LIB_NAME = "libhoomd_gb300.so"


def _ext_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def _pybind11_include():
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        import torch
        return str(pathlib.Path(torch.__file__).parent / "include")


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [INCLUDE / "hoomd_gb300.h"]


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _cu_obj(src, verbose, extra):
    obj = BUILD / (pathlib.Path(src).stem + ".o")
    if _stale(obj, [CSRC / src] + _headers()):
        _run([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--compiler-options", "-fPIC",
              "-I", str(INCLUDE), "-I", str(CSRC), *extra, "-c", str(CSRC / src), "-o", str(obj)],
             verbose)
    return obj


def _host_obj(src, verbose):
    obj = BUILD / (pathlib.Path(src).stem + ".o")
    if _stale(obj, [CSRC / src] + _headers()):
        _run(["g++", "-O2", "-fPIC", "-std=c++17", "-fvisibility=hidden",
              f"-I{sysconfig.get_paths()['include']}", f"-I{_pybind11_include()}",
              f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CUDA_HOME / 'include'}", "-c", str(CSRC / src),
              "-o", str(obj)], verbose)
    return obj


def build(verbose=False, ptxas_verbose=False):
    """Compile everything that is out of date; returns the paths of the two shared objects."""
    BUILD.mkdir(parents=True, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    jobs = min(len(CU_SOURCES) + len(HOST_SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        cu = [ex.submit(_cu_obj, s, verbose, extra) for s in CU_SOURCES]
        host = [ex.submit(_host_obj, s, verbose) for s in HOST_SOURCES]
        cu_objs = [f.result() for f in cu]
        host_objs = [f.result() for f in host]
    lib = OUT / LIB_NAME
    if _stale(lib, cu_objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(lib), *map(str, cu_objs), "-lcudart"], verbose)
    ext = OUT / ("_hoomd_gb300" + _ext_suffix())
    if _stale(ext, host_objs + [lib]):
        _run(["g++", "-shared", "-o", str(ext), *map(str, host_objs), f"-L{OUT}", "-lhoomd_gb300",
              f"-L{CUDA_HOME / 'lib64'}", "-lcudart", "-Wl,-rpath,$ORIGIN",
              f"-Wl,-rpath,{CUDA_HOME / 'lib64'}"], verbose)
    return lib, ext


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in OUT.glob("*.so"):
        p.unlink()


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build(verbose=True, ptxas_verbose="--ptxas" in sys.argv)
