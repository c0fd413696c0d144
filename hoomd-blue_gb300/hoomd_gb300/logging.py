"""Logging (hoomd/logging.py): named quantities of simulation objects, for writers.

A loggable class lists its quantities in ``_loggables`` (name -> category) and its namespace in
``_log_namespace``; ``Logger.add`` collects them (hoomd/logging.py:594-700). ``Logger.log()``
returns the nested ``{namespace: {quantity: (value, category)}}`` dictionary the reference's
writers read; ``hoomd_gb300.write.GSD`` stores scalar, sequence, string and per-particle values
as ``log/<namespace>/<quantity>`` chunks (hoomd/write/gsd.py:427-520).
"""

import numpy as np


class LoggerCategories:
    """The reference's logging categories (hoomd/logging.py:26-120), as names."""

    scalar = "scalar"
    sequence = "sequence"
    string = "string"
    strings = "strings"
    object = "object"
    angle = "angle"
    bond = "bond"
    constraint = "constraint"
    dihedral = "dihedral"
    improper = "improper"
    pair = "pair"
    particle = "particle"
    ALL = ("scalar", "sequence", "string", "strings", "object", "angle", "bond", "constraint",
           "dihedral", "improper", "pair", "particle")


_GSD_CATEGORIES = ("scalar", "sequence", "string", "strings", "angle", "bond", "constraint",
                   "dihedral", "improper", "pair", "particle")


def _namespace(obj):
    ns = getattr(obj, "_log_namespace", None)
    if ns is not None:
        return tuple(ns)
    mod = type(obj).__module__.split(".")
    if mod and mod[0] == "hoomd_gb300":
        mod = mod[1:]
    return tuple(mod) + (type(obj).__name__,)


class Logger:
    """hoomd.logging.Logger: ``add(obj, quantities=None, user_name=None)`` logs an object's
    quantities (all of them, or the named ones) in the categories the logger accepts."""

    def __init__(self, categories=None, only_default=True):
        cats = LoggerCategories.ALL if categories is None else tuple(categories)
        for c in cats:
            if c not in LoggerCategories.ALL:
                raise ValueError(f"unknown logger category {c!r}")
        self.categories = cats
        self.only_default = only_default
        self._quantities = {}  # namespace tuple -> (getter, category)

    def add(self, obj, quantities=None, user_name=None):
        table = getattr(type(obj), "_loggables", None)
        if not table:
            raise ValueError(f"{type(obj).__name__} has no loggable quantities")
        names = list(table) if quantities is None else list(quantities)
        ns = _namespace(obj)
        if user_name is not None:
            ns = ns[:-1] + (str(user_name),)
        added = []
        for q in names:
            if q not in table:
                raise ValueError(f"{type(obj).__name__} does not log {q!r}")
            cat = table[q]
            if cat not in self.categories:
                if quantities is not None:
                    raise ValueError(f"{q!r} has category {cat!r}, not accepted by this logger")
                continue
            key = ns + (q,)
            self._quantities[key] = (lambda o=obj, q=q: getattr(o, q), cat)
            added.append(key)
        return added

    def remove(self, obj=None, quantities=None, user_name=None):
        if obj is None:
            for q in quantities or []:
                self._quantities.pop(tuple(q) if not isinstance(q, str) else (q,), None)
            return
        ns = _namespace(obj)
        if user_name is not None:
            ns = ns[:-1] + (str(user_name),)
        for key in list(self._quantities):
            if key[:-1] == ns and (quantities is None or key[-1] in quantities):
                del self._quantities[key]

    def __setitem__(self, namespace, value):
        """``logger[ns] = (callable, category)`` or ``(obj, attribute, category)``."""
        ns = (namespace,) if isinstance(namespace, str) else tuple(namespace)
        if len(value) == 2:
            fn, cat = value
            getter = fn
        else:
            o, attr, cat = value
            getter = (lambda o=o, a=attr: getattr(o, a))
        if cat not in LoggerCategories.ALL:
            raise ValueError(f"unknown logger category {cat!r}")
        self._quantities[ns] = (getter, cat)

    def __getitem__(self, namespace):
        ns = (namespace,) if isinstance(namespace, str) else tuple(namespace)
        return self._quantities[ns]

    def __contains__(self, namespace):
        ns = (namespace,) if isinstance(namespace, str) else tuple(namespace)
        return ns in self._quantities

    def __iter__(self):
        return iter(self._quantities)

    def __len__(self):
        return len(self._quantities)

    def keys(self):
        return self._quantities.keys()

    def log(self):
        """Current values: ``{ns0: {ns1: ... {quantity: (value, category)}}}``."""
        out = {}
        for key, (getter, cat) in self._quantities.items():
            d = out
            for k in key[:-1]:
                d = d.setdefault(k, {})
            d[key[-1]] = (getter(), cat)
        return out

    def _gsd_chunks(self):
        """(name, array) pairs for the ``log/`` chunks of a GSD frame."""
        out = []
        for key, (getter, cat) in self._quantities.items():
            if cat not in _GSD_CATEGORIES:
                continue
            v = getter()
            if v is None:
                continue
            if cat == "string":
                a = np.frombuffer(str(v).encode() + b"\0", np.uint8)
            elif cat == "strings":
                from hoomd_gb300.gsd.hoomd import encode_types
                a = encode_types([str(s) for s in v])
            else:
                a = np.asarray(v)
                if a.dtype == np.bool_:
                    a = a.astype(np.uint8)
                if a.ndim == 0:
                    a = a.reshape(1)
            out.append(("/".join(key), a))
        return out
