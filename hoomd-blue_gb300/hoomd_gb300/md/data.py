"""Per-type-pair parameters (hoomd/data/typeparam.py, parameterdicts.py), trimmed to what the pair
forces and the neighbour list use: keys are unordered type pairs, a list in either position sets
every combination, and values are validated against the expected keys."""

import itertools

import numpy as np


def _expand(key):
    if not isinstance(key, tuple) or len(key) != 2:
        raise KeyError(f"type-pair parameters are keyed by (type, type) tuples, got {key!r}")
    a, b = key
    a = [a] if isinstance(a, str) else list(a)
    b = [b] if isinstance(b, str) else list(b)
    return [tuple(sorted(p)) for p in itertools.product(a, b)]


class TypePairDict:
    """Mapping (type_a, type_b) -> value, symmetric in the pair."""

    def __init__(self, default=None, validator=None):
        self._d = {}
        self.default = default
        self._validator = validator
        self._on_change = None

    def __setitem__(self, key, value):
        if self._validator is not None:
            value = self._validator(value)
        for k in _expand(key):
            self._d[k] = value
        if self._on_change is not None:
            self._on_change(key)

    def __getitem__(self, key):
        ks = _expand(key)
        if len(ks) != 1:
            return {k: self[k] for k in ks}
        k = ks[0]
        if k in self._d:
            return self._d[k]
        if self.default is not None:
            return self.default
        raise KeyError(f"{key} has not been set")

    def __contains__(self, key):
        return all(k in self._d for k in _expand(key))

    def get(self, key, default=None):
        try:
            return self[key]
        except KeyError:
            return default

    def keys(self):
        return self._d.keys()

    def to_base(self):
        return dict(self._d)


def dict_validator(required, optional=None, arrays=()):
    optional = optional or {}

    def check(value):
        if not isinstance(value, dict):
            raise TypeError("pair parameters must be a dict")
        out = dict(optional)
        out.update(value)
        missing = [k for k in required if k not in out]
        if missing:
            raise ValueError(f"missing required parameter(s) {missing}")
        extra = [k for k in out if k not in required and k not in optional]
        if extra:
            raise ValueError(f"unexpected parameter(s) {extra}")
        for k in out:
            if k in arrays:
                out[k] = np.ascontiguousarray(out[k], np.float64)
            else:
                out[k] = float(out[k])
        return out

    return check


def nonnegative_real(v):
    v = float(v)
    if v < 0:
        raise ValueError("value must be non-negative")
    return v


class TypeDict:
    """Mapping particle type -> value (a TypeParameter with len_keys=1); a list key sets each
    type in it."""

    def __init__(self, default=None, validator=None):
        self._d = {}
        self.default = default
        self._validator = validator
        self._on_change = None

    @staticmethod
    def _keys(key):
        return [key] if isinstance(key, str) else list(key)

    def __setitem__(self, key, value):
        if self._validator is not None:
            value = self._validator(value)
        for k in self._keys(key):
            self._d[k] = value
        if self._on_change is not None:
            self._on_change(key)

    def __getitem__(self, key):
        ks = self._keys(key)
        if len(ks) != 1 or not isinstance(key, str):
            return {k: self[k] for k in ks}
        if key in self._d:
            return self._d[key]
        if self.default is not None:
            return self.default
        raise KeyError(f"{key} has not been set")

    def __contains__(self, key):
        return all(k in self._d for k in self._keys(key))

    def keys(self):
        return self._d.keys()

    def to_base(self):
        return dict(self._d)
