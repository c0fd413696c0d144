"""Writers (hoomd/write). ``GSD`` writes the system state to a GSD file with the ``hoomd`` schema,
as hoomd.write.GSD (hoomd/write/gsd.py:59) over GSDDumpWriter (hoomd/GSDDumpWriter.cc) does:

* frame 0 holds every per-particle quantity that is not at its schema default, the box, N, the
  dimensions, the type names and the topology sections that have members;
* later frames hold the step and the quantities in ``dynamic`` (categories ``'property'``: box,
  N, position, orientation; ``'momentum'``: velocity, angmom, image; ``'attribute'``: types,
  typeid, mass, charge, diameter, body, moment_inertia; ``'topology'``; or single chunk names).
  A dynamic quantity that is all default is left out unless frame 0 stored it
  (hoomd/GSDDumpWriter.cc:1352-1430), so a reader's fall-back to frame 0 stays correct;
* positions are written wrapped into the box, with the images (hoomd/GSDDumpWriter.cc:1120-1140);
* ``diameter`` is written only with ``write_diameter = True``;
* ``log/<namespace>/<quantity>`` chunks carry a ``hoomd_gb300.logging.Logger``'s scalar,
  sequence and per-particle quantities.

The file layer is hoomd_gb300.gsd.fl.
"""

import os

import numpy as np

from hoomd_gb300 import filter as _filter
from hoomd_gb300.gsd import fl
from hoomd_gb300.gsd import hoomd as gh
from hoomd_gb300.trigger import as_trigger

_CATEGORIES = {
    "property": ("configuration/box", "particles/N", "particles/position",
                 "particles/orientation"),
    "momentum": ("particles/velocity", "particles/angmom", "particles/image"),
    "attribute": ("particles/types", "particles/typeid", "particles/mass", "particles/charge",
                  "particles/diameter", "particles/body", "particles/moment_inertia"),
}
_CHUNKS = {c for v in _CATEGORIES.values() for c in v}
# per-particle chunks in the order GSDDumpWriter writes them: (snapshot field, gsd field)
_PARTICLE_ORDER = ("typeid", "mass", "charge", "diameter", "body", "moment_inertia", "position",
                   "orientation", "velocity", "angmom", "image")
_GSD_TYPES = {name: (dt, m) for name, dt, m, _ in gh.PARTICLE_FIELDS}


def _expand_dynamic(dynamic):
    out = {"configuration/box", "particles/N", "particles/position", "particles/orientation"}
    topology = False
    for d in dynamic:
        d = str(d)
        if d in _CATEGORIES:
            out.update(_CATEGORIES[d])
        elif d == "topology":
            topology = True
        elif d in _CHUNKS:
            out.add(d)
        else:
            raise ValueError(f"invalid dynamic quantity {d!r}")
    return out, topology


class GSD:
    """hoomd.write.GSD: write frames of the system state every ``trigger`` steps.

    ``mode``: ``'ab'`` appends (creating the file when needed), ``'wb'`` overwrites, ``'xb'``
    creates and fails when the file exists. ``truncate=True`` empties the file when the writer
    attaches. ``filter`` selects the particles written; only ``hoomd.filter.All`` is supported.
    """

    def __init__(self, trigger, filename, filter=_filter.All(), mode="ab", truncate=False,
                 dynamic=None, logger=None):
        self.trigger = as_trigger(trigger)
        self.filename = os.fspath(filename)
        if not isinstance(filter, _filter.All):
            raise ValueError("GSD writes the group of all particles (hoomd.filter.All)")
        self.filter = filter
        if mode not in ("ab", "wb", "xb"):
            raise ValueError(f"invalid GSD file mode {mode!r}")
        self.mode = mode
        self.truncate = bool(truncate)
        self.dynamic = ["property"] if dynamic is None else list(dynamic)
        _expand_dynamic(self.dynamic)
        self.logger = logger
        self.write_diameter = False
        self.maximum_write_buffer_size = 64 * 1024 * 1024
        self._file = None
        self._simulation = None

    # -- attachment ----------------------------------------------------------------------------
    def _attach(self, simulation):
        if self._file is not None:
            return
        self._simulation = simulation
        self._file = _open(self.filename, self.mode)
        if self.truncate:
            self._file.truncate()
        self._nondefault = _nondefault(self._file)

    def _detach(self):
        if self._file is not None:
            self._file.close()
        self._file = None
        self._simulation = None

    def flush(self):
        """Sync the file (frames are complete on disk after each write)."""
        if self._file is None:
            raise RuntimeError("The GSD file is unavailable until the simulation runs for 0 or "
                               "more steps.")
        self._file.flush()

    # -- writing -------------------------------------------------------------------------------
    def _write(self, timestep):
        state = self._simulation.state
        _write_frame(self._file, state.get_snapshot(), int(timestep), self.dynamic,
                     self._nondefault, self.write_diameter, self.logger)

    @staticmethod
    def write(state, filename, filter=_filter.All(), mode="wb", logger=None):
        """Write the current state to ``filename`` as a one-frame file (modes 'wb' and 'xb')."""
        if mode not in ("wb", "xb"):
            raise ValueError(f"Invalid GSD.write file mode: {mode}")
        if not isinstance(filter, _filter.All):
            raise ValueError("GSD writes the group of all particles (hoomd.filter.All)")
        with _open(filename, mode) as f:
            _write_frame(f, state.get_snapshot(), state._simulation.timestep, ["property"],
                         {}, False, logger)


def _open(filename, mode):
    return fl.GSDFile(filename, {"ab": "a", "wb": "w", "xb": "x"}[mode],
                      application=gh.APPLICATION, schema=gh.SCHEMA,
                      schema_version=gh.SCHEMA_VERSION)


def _nondefault(f):
    """Which per-particle chunks frame 0 of an existing file stored
    (GSDDumpWriter::populateNonDefault, hoomd/GSDDumpWriter.cc:1021-1055)."""
    if f.schema != gh.SCHEMA or f.schema_version >= (2, 0):
        raise RuntimeError(f"GSD: invalid schema in {f.name}")
    if f.nframes == 0:
        return {}
    return {"particles/" + n: f.chunk_exists(0, "particles/" + n) for n in _PARTICLE_ORDER}


def _wrap(pos, image, box):
    """Wrap positions into the box in FP64, counting the crossings in the images."""
    Lx, Ly, Lz, xy, xz, yz = box
    pos = pos.copy()
    image = image.copy()
    dims = [(2, Lz), (1, Ly), (0, Lx)]
    for axis, L in dims:
        if L == 0:
            continue
        n = np.floor((pos[:, axis] + 0.5 * L) / L)
        if axis == 2:
            pos[:, 0] -= n * xz * Lz
            pos[:, 1] -= n * yz * Lz
        elif axis == 1:
            pos[:, 0] -= n * xy * Ly
        pos[:, axis] -= n * L
        image[:, axis] += n.astype(np.int32)
    return pos, image


def _write_frame(f, snap, step, dynamic, nondefault, write_diameter, logger):
    first = f.nframes == 0
    dyn, topology = _expand_dynamic(dynamic)
    p = snap.particles
    N = p.N
    box = np.array(snap.configuration.box, np.float64)
    f.write_chunk("configuration/step", np.array([step], np.uint64))
    if first:
        f.write_chunk("configuration/dimensions",
                      np.array([snap.configuration.dimensions], np.uint8))
    if first or "configuration/box" in dyn:
        f.write_chunk("configuration/box", box.astype(np.float32))
    if first or "particles/N" in dyn:
        f.write_chunk("particles/N", np.array([N], np.uint32))
    if first or "particles/types" in dyn:
        f.write_chunk("particles/types", gh.encode_types(list(p.types)))
    pos, image = _wrap(np.asarray(p.position, np.float64), np.asarray(p.image, np.int32),
                       box)
    values = {name: getattr(p, name) for name in _PARTICLE_ORDER}
    values["position"] = pos
    values["image"] = image
    for name in _PARTICLE_ORDER:
        chunk = "particles/" + name
        if name == "diameter" and not write_diameter:
            continue
        if not (first or chunk in dyn):
            continue
        dt, m = _GSD_TYPES[name]
        v = np.ascontiguousarray(values[name], dt).reshape((N,) if m == 1 else (N, m))
        all_default = N == 0 or np.array_equal(v, gh.default_array(name, N))
        if all_default and not (not first and nondefault.get(chunk, False)):
            continue
        f.write_chunk(chunk, v)
        if first:
            nondefault[chunk] = True
    if first or topology:
        for sec, m, typed in gh.TOPOLOGY_SECTIONS:
            g = getattr(snap, sec)
            if g.N == 0:
                continue
            f.write_chunk(sec + "/N", np.array([g.N], np.uint32))
            if typed:
                f.write_chunk(sec + "/types", gh.encode_types(list(g.types)))
                f.write_chunk(sec + "/typeid", np.asarray(g.typeid, np.uint32))
            else:
                f.write_chunk(sec + "/value", np.asarray(g.value, np.float32))
            f.write_chunk(sec + "/group", np.asarray(g.group, np.uint32).reshape(g.N, m))
    if logger is not None:
        for name, value in logger._gsd_chunks():
            f.write_chunk("log/" + name, value)
    f.end_frame()
