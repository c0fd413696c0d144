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

    @property
    def N(self):
        return self._N

    @N.setter
    def N(self, n):
        self._N = int(n)
        self._alloc(self._N)


class Snapshot:
    """hoomd.Snapshot with the particle fields the MD step uses."""

    def __init__(self, communicator=None):
        self.communicator = communicator or Communicator()
        self.configuration = _Configuration()
        self.particles = _Particles()

    def validate(self):
        p = self.particles
        N = p.N
        for name, shape in (("position", (N, 3)), ("velocity", (N, 3)), ("typeid", (N,)),
                            ("mass", (N,)), ("image", (N, 3))):
            if np.shape(getattr(p, name)) != shape:
                raise ValueError(f"snapshot.particles.{name} must have shape {shape}")
        if N and int(np.max(p.typeid)) >= len(p.types):
            raise ValueError("typeid refers to a type not in snapshot.particles.types")
