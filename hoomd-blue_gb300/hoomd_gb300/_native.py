"""Load the compiled engine. There is no fallback: without the CUDA extension nothing runs."""

import importlib
import pathlib

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "libhoomd_gb300.so"

try:
    _hoomd_gb300 = importlib.import_module("hoomd_gb300._hoomd_gb300")
except ImportError as exc:  # pragma: no cover - exercised only when the build is missing
    raise ImportError(
        "hoomd_gb300: the CUDA extension is not built (run `python hoomd-blue_gb300/build.py` "
        "or __graft_entry__.build()); there is no CPU fallback") from exc
