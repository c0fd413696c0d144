"""ctypes front end for oracle/_ref/libhoomd_ref_eval_f{32,64}.so -- test infrastructure only.

Those libraries are the reference's own header-only maths (BoxDim, EvaluatorPairLJ,
EvaluatorPairTable, EvaluatorPairExample) compiled unmodified (see oracle/build.py). They exist only
where the reference source tree was present at build time; ``available()`` says whether they do.
"""

import ctypes
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
_libs = {}


def path(prec):
    return HERE / "_ref" / f"libhoomd_ref_eval_f{prec}.so"


def available():
    return path(32).exists() and path(64).exists()


def lib(prec):
    if prec not in _libs:
        L = ctypes.CDLL(str(path(prec)))
        assert L.ref_scalar_size() == prec // 8
        _libs[prec] = L
    return _libs[prec]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _eval(prec, fn, rsq, *args):
    rsq = np.ascontiguousarray(rsq, np.float64)
    n = len(rsq)
    f = np.zeros(n)
    e = np.zeros(n)
    ok = np.zeros(n, np.int32)
    getattr(lib(prec), fn)(n, _p(rsq), *args, _p(f), _p(e), _p(ok))
    return f, e, ok.astype(bool)


def lj_eval(rsq, rcutsq, sigma, epsilon, shift=False, prec=32):
    d = ctypes.c_double
    return _eval(prec, "ref_lj_eval", rsq, d(rcutsq), d(sigma), d(epsilon), int(shift))


def lj_lrc(rcutsq, sigma, epsilon, prec=32):
    out = np.zeros(2)
    d = ctypes.c_double
    lib(prec).ref_lj_lrc(d(rcutsq), d(sigma), d(epsilon), _p(out))
    return out


def table_eval(rsq, rcutsq, rmin, V, F, prec=32):
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.float64)
    d = ctypes.c_double
    return _eval(prec, "ref_table_eval", rsq, d(rcutsq), d(rmin), len(V), _p(V), _p(F))


def example_eval(rsq, rcutsq, k, sigma, shift=False, prec=32):
    d = ctypes.c_double
    return _eval(prec, "ref_example_eval", rsq, d(rcutsq), d(k), d(sigma), int(shift))


def _box(box, periodic):
    b = np.zeros(6)
    b[: len(box)] = box
    return b, np.asarray(periodic, np.int32)


def min_image(v, box, prec=32, periodic=(1, 1, 1)):
    v = np.ascontiguousarray(v, np.float64).copy()
    b, p = _box(box, periodic)
    lib(prec).ref_min_image(len(v), _p(b), _p(p), _p(v))
    return v


def wrap(v, img, box, prec=32, periodic=(1, 1, 1)):
    v = np.ascontiguousarray(v, np.float64).copy()
    img = np.ascontiguousarray(img, np.int32).copy()
    b, p = _box(box, periodic)
    lib(prec).ref_wrap(len(v), _p(b), _p(p), _p(v), _p(img))
    return v, img


def make_fraction(v, box, prec=32, periodic=(1, 1, 1)):
    v = np.ascontiguousarray(v, np.float64).copy()
    b, p = _box(box, periodic)
    lib(prec).ref_make_fraction(len(v), _p(b), _p(p), _p(v))
    return v


def nearest_plane_distance(box, prec=32, periodic=(1, 1, 1)):
    out = np.zeros(3)
    b, p = _box(box, periodic)
    lib(prec).ref_nearest_plane_distance(_p(b), _p(p), _p(out))
    return out
