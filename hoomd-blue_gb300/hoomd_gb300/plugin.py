"""Building pair-evaluator plugins (the reference's example_plugins/pair_plugin, built there by
its CMakeLists.txt against an installed HOOMD-blue).

A plugin is an evaluator header written to the reference's evaluator concept
(example_plugins/pair_plugin/EvaluatorPairExample.h), a kernel file that instantiates
``hoomd::md::kernel::gpu_compute_pair_forces<Evaluator>`` and a module file that calls
``hoomd::md::detail::export_PotentialPairGPU<Evaluator>(m, "PotentialPair<Name>GPU")`` -- the
same three files as the reference's plugin, compiled here against the headers of this
repository's include/ directory (hoomd/HOOMDMath.h, hoomd/md/PotentialPair.h,
hoomd/md/PotentialPairGPU.h, hoomd/md/PotentialPairGPU.cuh), for sm_103a, with ENABLE_HIP
defined as the reference's GPU build defines it. The result is a Python extension module; a
``hoomd_gb300.md.pair.Pair`` subclass names it as ``_ext_module`` and its engine class as
``_cpp_class_name``.
"""

import concurrent.futures as cf
import os
import pathlib
import subprocess
import sysconfig

PKG = pathlib.Path(__file__).resolve().parent
INCLUDE = PKG.parent.parent / "include"
CSRC = PKG.parent / "csrc"
CUDA_HOME = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _pybind11_include():
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        import torch
        return str(pathlib.Path(torch.__file__).parent / "include")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(map(str, cmd)), flush=True)
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"plugin build failed:\n{' '.join(map(str, cmd))}\n{r.stdout}\n"
                           f"{r.stderr}")


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(pathlib.Path(d).stat().st_mtime > t for d in deps)


def _sdk_headers():
    return (list(INCLUDE.rglob("*.h")) + list(INCLUDE.rglob("*.cuh")) + list(CSRC.glob("*.cuh"))
            + list(CSRC.glob("*.h")))


def build_pair_plugin(module_name, kernel_sources, module_sources, out_dir, include_dirs=(),
                      verbose=False):
    """Compile a pair-evaluator plugin into ``out_dir/<module_name><EXT_SUFFIX>`` and return its
    path. ``kernel_sources`` are the .cu files (nvcc), ``module_sources`` the pybind11 module
    files (host compiler); ``include_dirs`` are searched before this library's headers. Out of
    date objects only are rebuilt."""
    out_dir = pathlib.Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    lib_dir = PKG
    if not (lib_dir / "libhoomd_gb300.so").exists():
        raise RuntimeError("libhoomd_gb300.so is not built (run __graft_entry__.build())")
    incs = [f"-I{d}" for d in include_dirs] + [f"-I{INCLUDE}", f"-I{CSRC}"]
    deps = _sdk_headers()
    for d in include_dirs:
        deps += list(pathlib.Path(d).glob("*.h"))
    jobs = []

    def cu(src):
        obj = out_dir / (pathlib.Path(src).stem + ".cu.o")
        if _stale(obj, [src] + deps):
            _run([CUDA_HOME / "bin" / "nvcc", *ARCH, "-O3", "-lineinfo", "-std=c++17",
                  "--compiler-options", "-fPIC", "-DENABLE_HIP", *incs, "-c", src, "-o", obj],
                 verbose)
        return obj

    def cc(src):
        obj = out_dir / (pathlib.Path(src).stem + ".cc.o")
        if _stale(obj, [src] + deps):
            _run(["g++", "-O2", "-fPIC", "-std=c++17", "-fvisibility=hidden", "-DENABLE_HIP",
                  *incs, f"-I{sysconfig.get_paths()['include']}", f"-I{_pybind11_include()}",
                  f"-I{CUDA_HOME / 'include'}", "-c", src, "-o", obj], verbose)
        return obj

    with cf.ThreadPoolExecutor(max(1, len(kernel_sources) + len(module_sources))) as ex:
        jobs = [ex.submit(cu, s) for s in kernel_sources] + [ex.submit(cc, s)
                                                            for s in module_sources]
        objs = [j.result() for j in jobs]
    target = out_dir / (module_name + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))
    if _stale(target, objs + [lib_dir / "libhoomd_gb300.so"]):
        _run(["g++", "-shared", "-o", target, *objs, f"-L{lib_dir}", "-lhoomd_gb300",
              f"-L{CUDA_HOME / 'lib64'}", "-lcudart", f"-Wl,-rpath,{lib_dir}",
              f"-Wl,-rpath,{CUDA_HOME / 'lib64'}"], verbose)
    return target


def load_pair_plugin(module_name, path):
    """Import the plugin module built at ``path``."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(module_name, str(path))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod
