"""Snapshots (hoomd/snapshot.py): the host-side, tag-ordered copy of the system state."""

import numpy as np


class Communicator:
    """One process drives one GPU: rank 0 of 1."""

    rank = 0
    num_ranks = 1

    def barrier(self):
        pass


class _Configuration:
    def __init__(self):
        self._box = [0.0] * 6
        self.dimensions = 3

    @property
    def box(self):
        return list(self._box)

    @box.setter
    def box(self, b):
        b = list(b) + [0.0] * (6 - len(b))
        self._box = [float(x) for x in b[:6]]
        self.dimensions = 2 if self._box[2] == 0 else 3


class _Particles:
    def __init__(self):
        self._N = 0
        self.types = ["A"]
        self._alloc(0)

    def _alloc(self, N):
        self.position = np.zeros((N, 3), np.float64)
        self.velocity = np.zeros((N, 3), np.float64)
        self.typeid = np.zeros(N, np.uint32)
        self.mass = np.ones(N, np.float64)
        self.image = np.zeros((N, 3), np.int32)
        # carried with the particles (GSD files, snapshots) but not used by the pair step; each
        # is created at its default on first access, so a field nobody touched is known to hold
        # its default without looking at N values
        self._passive = {}

    def _adopt(self, N, arrays):
        """Take ``arrays`` (name -> array of the right shape, owned by this snapshot from now
        on) as the particle data of N particles; passive fields not given hold their defaults."""
        self._N = int(N)
        self._passive = {}
        for name, m in PARTICLE_FIELDS:
            a = arrays.get(name)
            if name in PASSIVE_DEFAULTS:
                if a is not None:
                    self._passive[name] = a
                continue
            if a is None:
                raise ValueError(f"_adopt: {name} is required")
            setattr(self, name, a)

    def _passive_array(self, name):
        """The passive field ``name`` if it was ever accessed or set, else None (all defaults)."""
        return self._passive.get(name)

    @property
    def N(self):
        return self._N

    @N.setter
    def N(self, n):
        self._N = int(n)
        self._alloc(self._N)


def _passive_property(name):
    def get(self):
        a = self._passive.get(name)
        if a is None:
            a = self._passive[name] = passive_default(name, self._N)
        return a

    def set(self, value):
        self._passive[name] = value
    return property(get, set, doc=f"snapshot.particles.{name} (created at its default on first "
                                  f"access)")


class _Group:
    """A topology section (hoomd.Snapshot.bonds, angles, dihedrals, constraints, pairs): N groups
    of ``size`` particle tags with a type id (constraints carry a value instead)."""

    def __init__(self, size, typed=True):
        self._size = size
        self._typed = typed
        self.types = []
        self.N = 0

    @property
    def N(self):
        return self._N

    @N.setter
    def N(self, n):
        self._N = int(n)
        self.group = np.zeros((self._N, self._size), np.uint32)
        if self._typed:
            self.typeid = np.zeros(self._N, np.uint32)
        else:
            self.value = np.zeros(self._N, np.float64)


# per-particle quantities the MD step carries but does not change, with their default values
PASSIVE_DEFAULTS = {"charge": (1, np.float64, 0.0), "diameter": (1, np.float64, 1.0),
                    "body": (1, np.int32, -1), "moment_inertia": (3, np.float64, 0.0),
                    "orientation": (4, np.float64, (1.0, 0.0, 0.0, 0.0)),
                    "angmom": (4, np.float64, 0.0)}


def passive_default(name, N):
    """A fresh array of N default values of the passive field ``name``."""
    m, dt, v = PASSIVE_DEFAULTS[name]
    shape = (N,) if m == 1 else (N, m)
    if np.ndim(v) == 0 and v == 0:
        return np.zeros(shape, dt)
    a = np.empty(shape, dt)
    a[...] = v
    return a


def is_passive_default(name, a):
    """True when every entry of ``a`` holds the default of the passive field ``name``."""
    m, dt, v = PASSIVE_DEFAULTS[name]
    a = np.asarray(a)
    if a.size == 0:
        return True
    if np.ndim(v) == 0:
        return not np.any(a != v) if v != 0 else not np.any(a)
    return not np.any(a[:, 0] != v[0]) and not np.any(a[:, 1:])


for _name in PASSIVE_DEFAULTS:
    setattr(_Particles, _name, _passive_property(_name))

PARTICLE_FIELDS = (("position", 3), ("velocity", 3), ("typeid", 1), ("mass", 1), ("image", 3),
                   ("charge", 1), ("diameter", 1), ("body", 1), ("moment_inertia", 3),
                   ("orientation", 4), ("angmom", 4))
TOPOLOGY_SECTIONS = ("bonds", "angles", "dihedrals", "impropers", "constraints", "pairs")


class Snapshot:
    """hoomd.Snapshot: the particle fields of the hoomd schema and the topology sections that
    the neighbour list's exclusions read."""

    def __init__(self, communicator=None):
        self.communicator = communicator or Communicator()
        self.configuration = _Configuration()
        self.particles = _Particles()
        self.bonds = _Group(2)
        self.angles = _Group(3)
        self.dihedrals = _Group(4)
        self.impropers = _Group(4)
        self.constraints = _Group(2, typed=False)
        self.pairs = _Group(2)

    def validate(self):
        p = self.particles
        N = p.N
        for name, m in PARTICLE_FIELDS:
            shape = (N,) if m == 1 else (N, m)
            a = p._passive_array(name) if name in PASSIVE_DEFAULTS else getattr(p, name)
            if a is not None and np.shape(a) != shape:
                raise ValueError(f"snapshot.particles.{name} must have shape {shape}")
        if N and int(np.max(p.typeid)) >= len(p.types):
            raise ValueError("typeid refers to a type not in snapshot.particles.types")
        for name in TOPOLOGY_SECTIONS:
            g = getattr(self, name)
            if np.shape(g.group) != (g.N, g._size):
                raise ValueError(f"snapshot.{name}.group must have shape {(g.N, g._size)}")
            if g.N and int(np.max(g.group)) >= N:
                raise ValueError(f"snapshot.{name}.group refers to a particle tag >= N")

    @classmethod
    def from_gsd_frame(cls, gsd_snap, communicator=None):
        """A snapshot from a ``gsd.hoomd.Frame`` (hoomd/snapshot.py:465-520): quantities the
        frame leaves unset keep the snapshot defaults."""
        gsd_snap.validate()
        snap = cls(communicator)
        c = gsd_snap.configuration
        snap.configuration.box = [float(x) for x in c.box]
        gp = gsd_snap.particles
        snap.particles.N = int(gp.N)
        if gp.types is not None:
            snap.particles.types = list(gp.types)
        for name, _ in PARTICLE_FIELDS:
            v = getattr(gp, name, None)
            if v is not None:
                getattr(snap.particles, name)[:] = v
        for name in TOPOLOGY_SECTIONS:
            src = getattr(gsd_snap, name, None)
            if src is None:
                continue
            dst = getattr(snap, name)
            dst.N = int(src.N)
            if dst._typed:
                dst.types = list(src.types or [])
                if src.typeid is not None:
                    dst.typeid[:] = src.typeid
            elif src.value is not None:
                dst.value[:] = src.value
            if src.group is not None:
                dst.group[:] = src.group
        return snap
