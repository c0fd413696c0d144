"""CPU-only helpers shared by the tests (no torch, no GPU)."""

import ctypes

import numpy as np

from hoomd_gb300 import abi


def pack_table_cpu(U, F):
    """gb_table_pack through the C ABI (a host-only function)."""
    U = np.ascontiguousarray(U, np.float64)
    F = np.ascontiguousarray(F, np.float64)
    out = np.zeros((len(U), 4), np.float32)
    abi.check(abi.load().gb_table_pack(U.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       F.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       len(U), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
              "gb_table_pack")
    return out
