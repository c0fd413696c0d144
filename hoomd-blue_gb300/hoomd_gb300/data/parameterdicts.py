"""TypeParameterDict (hoomd/data/parameterdicts.py): the specification of one type parameter's
values. Each keyword names a key of the value dict: a type (float, int, str, bool) makes the key
required and converts it; any other value makes the key optional with that default. ``len_keys``
is 1 for per-type and 2 for per-type-pair parameters."""

import numpy as np

from hoomd_gb300.md.data import TypeDict, TypePairDict

_TYPES = (float, int, str, bool)


class TypeParameterDict:
    def __init__(self, *args, len_keys, **kwargs):
        if args:
            raise TypeError("TypeParameterDict takes its keys as keyword arguments")
        if len_keys not in (1, 2):
            raise ValueError("len_keys must be 1 or 2")
        self.len_keys = len_keys
        self.spec = dict(kwargs)

    def _validate(self, value):
        if not isinstance(value, dict):
            raise TypeError("type parameters are given as a dict")
        out = {}
        for k, spec in self.spec.items():
            if k in value:
                v = value[k]
                if isinstance(spec, type) and spec in _TYPES:
                    v = spec(v)
                elif isinstance(v, (list, tuple, np.ndarray)):
                    v = np.ascontiguousarray(v, np.float64)
                out[k] = v
            elif isinstance(spec, type):
                raise ValueError(f"missing required parameter {k!r}")
            else:
                out[k] = spec
        extra = [k for k in value if k not in self.spec]
        if extra:
            raise ValueError(f"unexpected parameter(s) {extra}")
        return out

    def make_container(self):
        """The per-type (TypeDict) or per-type-pair (TypePairDict) mapping of validated values."""
        if self.len_keys == 1:
            return TypeDict(validator=self._validate)
        return TypePairDict(validator=self._validate)
