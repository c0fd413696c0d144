"""Test infrastructure: the reference's own GSD library (hoomd/extern/gsd.c, built by
``oracle.build.build_gsd_ref`` into oracle/_ref/libgsd_ref.so) through ctypes.

``available()`` is False where the reference tree was absent at build time; the tests that use
this module skip then. Only tests import it.
"""

import ctypes

import numpy as np

from oracle import build as _build

_TYPES = {1: np.uint8, 2: np.uint16, 3: np.uint32, 4: np.uint64, 5: np.int8, 6: np.int16,
          7: np.int32, 8: np.int64, 9: np.float32, 10: np.float64}
_CODES = {np.dtype(v): k for k, v in _TYPES.items()}
_lib = None


def available():
    return _load() is not None


def _load():
    global _lib
    if _lib is None:
        path = _build.build_gsd_ref()
        if path is None or not path.exists():
            return None
        L = ctypes.CDLL(str(path))
        vp, cp, u64, u32 = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint32
        L.rg_open.restype = vp
        L.rg_open.argtypes = [cp, ctypes.c_int]
        L.rg_create.restype = vp
        L.rg_create.argtypes = [cp, cp, cp, ctypes.c_uint, ctypes.c_uint]
        L.rg_close.argtypes = [vp]
        L.rg_nframes.restype = u64
        L.rg_nframes.argtypes = [vp]
        L.rg_header.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32), cp, cp]
        L.rg_find.argtypes = [vp, u64, cp, ctypes.POINTER(u64), ctypes.POINTER(u32),
                              ctypes.POINTER(ctypes.c_uint8)]
        L.rg_read.argtypes = [vp, u64, cp, vp]
        L.rg_write.argtypes = [vp, cp, ctypes.c_int, u64, u32, vp]
        L.rg_end_frame.argtypes = [vp]
        L.rg_match.restype = vp  # the library's own pointer, passed back as ``prev``
        L.rg_match.argtypes = [vp, cp, vp]
        _lib = L
    return _lib


class RefGSD:
    """A GSD file opened by the reference library (mode 'r', 'a', or 'w' to create)."""

    def __init__(self, name, mode="r", application="ref", schema="hoomd", version=(1, 4)):
        L = _load()
        if mode == "w":
            self.h = L.rg_create(str(name).encode(), application.encode(), schema.encode(),
                                 *version)
        else:
            self.h = L.rg_open(str(name).encode(), 0 if mode == "r" else 1)
        if not self.h:
            raise RuntimeError(f"reference gsd could not open {name}")
        self.L = L

    @property
    def nframes(self):
        return int(self.L.rg_nframes(self.h))

    def header(self):
        gv, sv = ctypes.c_uint32(), ctypes.c_uint32()
        app, sch = ctypes.create_string_buffer(64), ctypes.create_string_buffer(64)
        self.L.rg_header(self.h, ctypes.byref(gv), ctypes.byref(sv), app, sch)
        return dict(gsd_version=(gv.value >> 16, gv.value & 0xFFFF),
                    schema_version=(sv.value >> 16, sv.value & 0xFFFF),
                    application=app.value.decode(), schema=sch.value.decode())

    def find(self, frame, name):
        N, M, t = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint8()
        if not self.L.rg_find(self.h, frame, name.encode(), ctypes.byref(N), ctypes.byref(M),
                              ctypes.byref(t)):
            return None
        return int(N.value), int(M.value), int(t.value)

    def read(self, frame, name):
        f = self.find(frame, name)
        if f is None:
            raise KeyError(name)
        N, M, t = f
        a = np.empty(N * M, _TYPES[t])
        if N * M == 0:
            # gsd_read_chunk reports an empty chunk as corrupt; the gsd Python layer returns an
            # empty array without calling it, as here
            return a if M == 1 else a.reshape(N, M)
        r = self.L.rg_read(self.h, frame, name.encode(), a.ctypes.data_as(ctypes.c_void_p))
        if r != 0:
            raise RuntimeError(f"gsd_read_chunk failed ({r})")
        return a if M == 1 else a.reshape(N, M)

    def write(self, name, data):
        a = np.ascontiguousarray(data)
        if a.ndim == 0:
            a = a.reshape(1)
        N = a.shape[0]
        M = 1 if a.ndim == 1 else a.shape[1]
        r = self.L.rg_write(self.h, name.encode(), _CODES[a.dtype], N, M,
                            a.ctypes.data_as(ctypes.c_void_p))
        if r != 0:
            raise RuntimeError(f"gsd_write_chunk failed ({r})")

    def end_frame(self):
        r = self.L.rg_end_frame(self.h)
        if r != 0:
            raise RuntimeError(f"gsd_end_frame failed ({r})")

    def names(self, match=""):
        out = []
        prev = None
        while True:
            n = self.L.rg_match(self.h, match.encode(), prev)
            if not n:
                return out
            out.append(ctypes.string_at(n).decode())
            prev = n

    def close(self):
        if self.h:
            self.L.rg_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
