"""Tuners (hoomd/tune). ParticleSorter reorders particles along a Hilbert curve
(hoomd/tune/sorter.py:14, hoomd/SFCPackTuner.cc)."""

import math

from hoomd_gb300.trigger import Periodic, as_trigger


class ParticleSorter:
    """Sort particles in space-filling-curve order every ``trigger`` steps.

    ``grid`` is the number of lattice bins per box side (rounded up to a power of two here, at
    most 512 in 3D and 4096 in 2D); the reference's default is 256 in 3D and 4096 in 2D
    (hoomd/SFCPackTuner.cc:34-42).
    """

    def __init__(self, trigger=200, grid=None):
        self.trigger = as_trigger(trigger)
        if not isinstance(self.trigger, Periodic) or self.trigger.phase != 0:
            raise ValueError("ParticleSorter supports Periodic(period) triggers")
        self.grid = None if grid is None else int(grid)

    def _grid_bits(self, dimensions):
        grid = self.grid if self.grid is not None else (4096 if dimensions == 2 else 256)
        top = 12 if dimensions == 2 else 9
        return max(1, min(top, int(math.ceil(math.log2(max(2, grid))))))

    @property
    def grid_bits(self):
        return self._grid_bits(3)
