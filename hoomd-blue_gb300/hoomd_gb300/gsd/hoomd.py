"""The ``hoomd`` schema of GSD files (gsd.hoomd): frames of particle and topology data.

Chunk names, element types and defaults follow the schema that HOOMD-blue writes and reads
(hoomd/GSDDumpWriter.cc:440-760, hoomd/GSDReader.cc:98-320): ``configuration/step`` (uint64),
``configuration/dimensions`` (uint8), ``configuration/box`` (6 float32), ``particles/N`` (uint32),
``particles/types`` (uint8 rows of NUL-padded names), per-particle float32 ``mass``, ``charge``,
``diameter``, ``moment_inertia`` (3), ``position`` (3), ``orientation`` (4), ``velocity`` (3),
``angmom`` (4), uint32 ``typeid``, int32 ``body`` and ``image`` (3), and for each topology section
``N``, ``types``, ``typeid`` and ``group`` (constraints carry float32 ``value`` instead), plus
``log/*`` quantities.

A chunk missing from a frame takes its value from frame 0, and failing that the schema default;
a per-particle chunk of frame 0 is used only when its length matches the frame's N.
"""

import numpy as np

from hoomd_gb300.gsd import fl

SCHEMA = "hoomd"
APPLICATION = "hoomd_gb300"
SCHEMA_VERSION = (1, 4)

# (chunk, numpy type, columns, default value) of each per-particle quantity
PARTICLE_FIELDS = (
    ("typeid", np.uint32, 1, 0),
    ("mass", np.float32, 1, 1.0),
    ("charge", np.float32, 1, 0.0),
    ("diameter", np.float32, 1, 1.0),
    ("body", np.int32, 1, -1),
    ("moment_inertia", np.float32, 3, 0.0),
    ("position", np.float32, 3, 0.0),
    ("orientation", np.float32, 4, (1.0, 0.0, 0.0, 0.0)),
    ("velocity", np.float32, 3, 0.0),
    ("angmom", np.float32, 4, 0.0),
    ("image", np.int32, 3, 0),
)
# topology sections: (name, particles per group, typed)
TOPOLOGY_SECTIONS = (("bonds", 2, True), ("angles", 3, True), ("dihedrals", 4, True),
                     ("impropers", 4, True), ("constraints", 2, False), ("pairs", 2, True))
DEFAULT_BOX = (1.0, 1.0, 1.0, 0.0, 0.0, 0.0)


def default_array(field, N):
    """The schema default of a per-particle quantity for N particles."""
    for name, dt, m, d in PARTICLE_FIELDS:
        if name == field:
            shape = (N,) if m == 1 else (N, m)
            a = np.empty(shape, dt)
            a[...] = d
            return a
    raise KeyError(field)


def encode_types(types):
    """Type names as the uint8 rows of a ``*/types`` chunk (longest name + NUL per row)."""
    width = max([len(t.encode()) for t in types] + [0]) + 1
    a = np.zeros((len(types), width), np.uint8)
    for i, t in enumerate(types):
        b = t.encode()
        a[i, :len(b)] = np.frombuffer(b, np.uint8)
    return a


def decode_types(a):
    a = np.asarray(a, np.uint8)
    if a.ndim == 1:
        a = a.reshape(len(a), 1)
    return [bytes(row).split(b"\0", 1)[0].decode() for row in a]


class ConfigurationData:
    def __init__(self):
        self.step = None
        self.dimensions = None
        self.box = None

    def validate(self):
        self.step = 0 if self.step is None else int(self.step)
        box = np.asarray(DEFAULT_BOX if self.box is None else self.box, np.float32).reshape(6)
        self.box = box
        if self.dimensions is None:
            self.dimensions = 2 if box[2] == 0 else 3
        self.dimensions = int(self.dimensions)


class ParticleData:
    def __init__(self):
        self.N = 0
        self.types = None
        for name, *_ in PARTICLE_FIELDS:
            setattr(self, name, None)

    def validate(self):
        N = int(self.N)
        self.N = N
        self.types = ["A"] if self.types is None else [str(t) for t in self.types]
        for name, dt, m, d in PARTICLE_FIELDS:
            v = getattr(self, name)
            if v is None:
                continue
            shape = (N,) if m == 1 else (N, m)
            v = np.ascontiguousarray(v, dt).reshape(shape)
            setattr(self, name, v)


class BondData:
    def __init__(self, M, typed=True):
        self.M = M
        self._typed = typed
        self.N = 0
        self.types = None
        self.typeid = None
        self.value = None
        self.group = None

    def validate(self):
        N = int(self.N)
        self.N = N
        if self._typed:
            self.types = [] if self.types is None else [str(t) for t in self.types]
            self.typeid = (np.zeros(N, np.uint32) if self.typeid is None
                           else np.ascontiguousarray(self.typeid, np.uint32).reshape(N))
        else:
            self.value = (np.zeros(N, np.float32) if self.value is None
                          else np.ascontiguousarray(self.value, np.float32).reshape(N))
        self.group = (np.zeros((N, self.M), np.uint32) if self.group is None
                      else np.ascontiguousarray(self.group, np.uint32).reshape(N, self.M))


class Frame:
    """One frame of a ``hoomd``-schema GSD file (gsd.hoomd.Frame); unset quantities are None
    and take the schema default (or frame 0's value when read from a file)."""

    def __init__(self):
        self.configuration = ConfigurationData()
        self.particles = ParticleData()
        for name, m, typed in TOPOLOGY_SECTIONS:
            setattr(self, name, BondData(m, typed))
        self.log = {}

    def validate(self):
        self.configuration.validate()
        self.particles.validate()
        for name, *_ in TOPOLOGY_SECTIONS:
            getattr(self, name).validate()


def _equal(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a, b)


class HOOMDTrajectory:
    """A sequence of frames in a GSD file (gsd.hoomd.HOOMDTrajectory): ``len``, indexing and
    slicing read frames; ``append`` writes one."""

    def __init__(self, file):
        if file.schema != SCHEMA:
            raise RuntimeError(f"{file.name}: schema {file.schema!r} is not {SCHEMA!r}")
        if file.schema_version >= (2, 0):
            raise RuntimeError(f"{file.name}: unsupported hoomd schema version "
                               f"{file.schema_version}")
        self.file = file
        self._frame0 = None

    def __len__(self):
        return self.file.nframes

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.file.close()

    def close(self):
        self.file.close()

    def flush(self):
        self.file.flush()

    def truncate(self):
        self.file.truncate()
        self._frame0 = None

    def __iter__(self):
        for i in range(len(self)):
            yield self._read_frame(i)

    def __getitem__(self, key):
        if isinstance(key, slice):
            return [self._read_frame(i) for i in range(*key.indices(len(self)))]
        i = int(key)
        if i < 0:
            i += len(self)
        if not 0 <= i < len(self):
            raise IndexError(f"frame {key} is out of range ({len(self)} frames)")
        return self._read_frame(i)

    # -- reading -------------------------------------------------------------------------------
    def _chunk(self, frame, name, N=None):
        """Chunk ``name`` of ``frame``, else of frame 0, else None; a chunk whose length is not
        ``N`` (when given) counts as missing (hoomd/GSDReader.cc:107-138)."""
        f = self.file
        src = frame if f.chunk_exists(frame, name) else 0 if f.chunk_exists(0, name) else None
        if src is None:
            return None
        a = f.read_chunk(src, name)
        if N is not None and len(a) != N:
            return None
        return a

    def _read_frame(self, i):
        fr = Frame()
        c = fr.configuration
        v = self._chunk(i, "configuration/step")
        c.step = 0 if v is None else int(v[0])
        v = self._chunk(i, "configuration/dimensions")
        c.dimensions = 3 if v is None else int(v[0])
        v = self._chunk(i, "configuration/box")
        c.box = np.array(DEFAULT_BOX if v is None else v, np.float32)
        if c.dimensions == 2:
            c.box[[2, 4, 5]] = 0.0
        p = fr.particles
        v = self._chunk(i, "particles/N")
        p.N = 0 if v is None else int(v[0])
        v = self._chunk(i, "particles/types")
        p.types = ["A"] if v is None else decode_types(v)
        for name, dt, m, d in PARTICLE_FIELDS:
            v = self._chunk(i, "particles/" + name, p.N)
            setattr(p, name, default_array(name, p.N) if v is None
                    else np.asarray(v, dt).reshape((p.N,) if m == 1 else (p.N, m)))
        for sec, m, typed in TOPOLOGY_SECTIONS:
            g = getattr(fr, sec)
            v = self._chunk(i, sec + "/N")
            g.N = 0 if v is None else int(v[0])
            if typed:
                v = self._chunk(i, sec + "/types")
                g.types = [] if v is None else decode_types(v)
                v = self._chunk(i, sec + "/typeid", g.N)
                g.typeid = np.zeros(g.N, np.uint32) if v is None else np.asarray(v, np.uint32)
            else:
                v = self._chunk(i, sec + "/value", g.N)
                g.value = np.zeros(g.N, np.float32) if v is None else np.asarray(v, np.float32)
            v = self._chunk(i, sec + "/group", g.N)
            g.group = (np.zeros((g.N, m), np.uint32) if v is None
                       else np.asarray(v, np.uint32).reshape(g.N, m))
        for name in self.file.find_matching_chunk_names("log/"):
            v = self._chunk(i, name)
            if v is not None:
                fr.log[name[4:]] = v
        return fr

    # -- writing -------------------------------------------------------------------------------
    def _initial(self):
        if self._frame0 is None and len(self) > 0:
            self._frame0 = self._read_frame(0)
        return self._frame0

    def append(self, frame):
        """Write ``frame`` as the next frame. Frame 0 stores the quantities that differ from the
        schema defaults; later frames store those that differ from frame 0."""
        frame.validate()
        f = self.file
        first = len(self) == 0
        ref = None if first else self._initial()

        def put(name, value, default):
            if first:
                if default is None or not _equal(value, default):
                    f.write_chunk(name, value)
            elif not _equal(value, default):
                f.write_chunk(name, value)

        c = frame.configuration
        f.write_chunk("configuration/step", np.array([c.step], np.uint64))
        put("configuration/dimensions", np.array([c.dimensions], np.uint8),
            np.array([3], np.uint8) if first else np.array([ref.configuration.dimensions],
                                                            np.uint8))
        put("configuration/box", c.box,
            np.array(DEFAULT_BOX, np.float32) if first else ref.configuration.box)
        p = frame.particles
        put("particles/N", np.array([p.N], np.uint32),
            np.array([0], np.uint32) if first else np.array([ref.particles.N], np.uint32))
        if first:
            if p.types != ["A"]:
                f.write_chunk("particles/types", encode_types(p.types))
        elif p.types != ref.particles.types:
            f.write_chunk("particles/types", encode_types(p.types))
        for name, dt, m, d in PARTICLE_FIELDS:
            v = getattr(p, name)
            if v is None:
                continue
            base = default_array(name, p.N)
            if not first and ref.particles.N == p.N:
                base = getattr(ref.particles, name)
            put("particles/" + name, v, base)
        for sec, m, typed in TOPOLOGY_SECTIONS:
            g = getattr(frame, sec)
            r = None if first else getattr(ref, sec)
            put(sec + "/N", np.array([g.N], np.uint32),
                np.array([0 if first else r.N], np.uint32))
            if typed:
                if (first and g.types) or (not first and g.types != r.types):
                    f.write_chunk(sec + "/types", encode_types(g.types))
                put(sec + "/typeid", g.typeid,
                    np.zeros(g.N, np.uint32) if first or r.N != g.N else r.typeid)
            else:
                put(sec + "/value", g.value,
                    np.zeros(g.N, np.float32) if first or r.N != g.N else r.value)
            put(sec + "/group", g.group,
                np.zeros((g.N, m), np.uint32) if first or r.N != g.N else r.group)
        for name, v in frame.log.items():
            f.write_chunk("log/" + name, np.asarray(v))
        f.end_frame()
        if first:
            self._frame0 = None


def open(name, mode="r"):  # noqa: A001
    """gsd.hoomd.open: a ``HOOMDTrajectory`` over a GSD file with the ``hoomd`` schema."""
    f = fl.GSDFile(name, mode, application=APPLICATION, schema=SCHEMA,
                   schema_version=SCHEMA_VERSION)
    return HOOMDTrajectory(f)
