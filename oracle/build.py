"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles this project's CPU restatement ``oracle/md_oracle.cc`` into
  ``oracle/_build/libmd_oracle.so``. It needs only g++ and runs on any host.
* ``build_ref()`` compiles ``oracle/ref_shim.cc`` against the reference's own unmodified headers
  (``hoomd/HOOMDMath.h``, ``hoomd/BoxDim.h``, ``hoomd/md/EvaluatorPairLJ.h``,
  ``hoomd/md/EvaluatorPairTable.h``, ``example_plugins/pair_plugin/EvaluatorPairExample.h``), read
  in place from the reference source tree, into ``oracle/_ref/libhoomd_ref_eval_f{32,64}.so``. It
  runs only where that tree and pybind11/Python headers exist; elsewhere it does nothing.
* ``build_gsd_ref()`` compiles the reference's own GSD library ``hoomd/extern/gsd.c`` (a
  self-contained C file, read in place) with the flat ctypes shim ``oracle/gsd_ref_shim.c`` into
  ``oracle/_ref/libgsd_ref.so``, where the reference tree exists. The rest
  of the reference (cell list, neighbour list, pair loop, integrator) cannot be compiled in
  isolation: it needs the absent git submodules (nano-signal-slot, random123, ...) and Eigen3.

Run ``python oracle/build.py`` or call the functions; both are idempotent (mtime checked).
"""

import os
import pathlib
import subprocess
import sys
import sysconfig

HERE = pathlib.Path(__file__).resolve().parent
# the reference source tree: $HOOMD_REFERENCE_ROOT, else a directory named "reference" beside
# this repository's root
REF_ROOT = pathlib.Path(os.environ.get("HOOMD_REFERENCE_ROOT",
                                       str(HERE.parent.parent / "reference")))

ORACLE_SRC = HERE / "md_oracle.cc"
ORACLE_LIB = HERE / "_build" / "libmd_oracle.so"
SHIM_SRC = HERE / "ref_shim.cc"
REF_DIR = HERE / "_ref"


def _stale(target, sources):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_oracle(verbose=False):
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if not _stale(ORACLE_LIB, [ORACLE_SRC]):
        return ORACLE_LIB
    cmd = ["g++", "-O3", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-fopenmp",
           str(ORACLE_SRC), "-o", str(ORACLE_LIB)]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return ORACLE_LIB


def _pybind11_include():
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        pass
    try:
        import torch  # torch ships the pybind11 headers
        inc = pathlib.Path(torch.__file__).parent / "include"
        if (inc / "pybind11").exists():
            return str(inc)
    except ImportError:
        pass
    return None


def ref_available():
    return (REF_ROOT / "hoomd" / "md" / "EvaluatorPairLJ.h").exists()


def build_ref(verbose=False):
    """Compile the reference-header shim, when the reference source tree is present."""
    if not ref_available():
        return None
    pyinc = sysconfig.get_paths()["include"]
    pbinc = _pybind11_include()
    if pbinc is None or not pathlib.Path(pyinc, "Python.h").exists():
        return None
    REF_DIR.mkdir(parents=True, exist_ok=True)
    outs = []
    procs = []
    for prec in (64, 32):
        out = REF_DIR / f"libhoomd_ref_eval_f{prec}.so"
        outs.append(out)
        if not _stale(out, [SHIM_SRC]):
            continue
        cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off",
               f"-DHOOMD_LONGREAL_SIZE={prec}", "-DHOOMD_SHORTREAL_SIZE=32", f"-I{REF_ROOT}",
               f"-I{pyinc}", f"-I{pbinc}", str(SHIM_SRC), "-o", str(out)]
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference shim build failed")
    return outs


GSD_SHIM_SRC = HERE / "gsd_ref_shim.c"
GSD_REF_LIB = REF_DIR / "libgsd_ref.so"


def build_gsd_ref(verbose=False):
    """Compile hoomd/extern/gsd.c with the ctypes shim, when the reference tree is present."""
    src = REF_ROOT / "hoomd" / "extern" / "gsd.c"
    if not src.exists():
        return None
    REF_DIR.mkdir(parents=True, exist_ok=True)
    if not _stale(GSD_REF_LIB, [GSD_SHIM_SRC]):
        return GSD_REF_LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11",
           f"-I{REF_ROOT / 'hoomd' / 'extern'}", str(GSD_SHIM_SRC), str(src), "-o",
           str(GSD_REF_LIB)]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return GSD_REF_LIB


if __name__ == "__main__":
    build_oracle(verbose=True)
    r = build_ref(verbose=True)
    g = build_gsd_ref(verbose=True)
    print("oracle:", ORACLE_LIB, "reference shim:", r, "reference gsd:", g)
    sys.exit(0)
