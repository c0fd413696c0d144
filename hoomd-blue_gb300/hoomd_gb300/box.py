"""Simulation box (hoomd/box.py): lengths and tilt factors, periodic in every direction."""

import numpy as np


class Box:
    def __init__(self, Lx, Ly, Lz=0, xy=0, xz=0, yz=0):
        self.Lx, self.Ly, self.Lz = float(Lx), float(Ly), float(Lz)
        self.xy, self.xz, self.yz = float(xy), float(xz), float(yz)

    @classmethod
    def cube(cls, L):
        return cls(L, L, L)

    @classmethod
    def square(cls, L):
        return cls(L, L, 0)

    @classmethod
    def from_box(cls, box):
        if isinstance(box, Box):
            return cls(*box.to_list())
        b = list(box) + [0] * (6 - len(box))
        return cls(*b[:6])

    def to_list(self):
        return [self.Lx, self.Ly, self.Lz, self.xy, self.xz, self.yz]

    @property
    def L(self):
        return np.array([self.Lx, self.Ly, self.Lz])

    @property
    def is2D(self):
        return self.Lz == 0

    @property
    def dimensions(self):
        return 2 if self.is2D else 3

    @property
    def volume(self):
        return self.Lx * self.Ly * (1.0 if self.is2D else self.Lz)

    @property
    def periodic(self):
        return np.array([True, True, True])

    def __eq__(self, other):
        return isinstance(other, Box) and self.to_list() == other.to_list()

    def __repr__(self):
        return "hoomd_gb300.Box(Lx={}, Ly={}, Lz={}, xy={}, xz={}, yz={})".format(*self.to_list())
