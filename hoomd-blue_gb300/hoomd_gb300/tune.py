"""Tuners (hoomd/tune). ParticleSorter reorders particles along a Hilbert curve
(hoomd/tune/sorter.py:14, hoomd/SFCPackTuner.cc)."""

import math

from hoomd_gb300.trigger import Periodic, as_trigger


class ParticleSorter:
    """Sort particles in space-filling-curve order every ``trigger`` steps.

    ``grid`` is the number of lattice bins per box side (rounded up to a power of two here,
    at most 512); the reference's default is 256.
    """

    def __init__(self, trigger=200, grid=None):
        self.trigger = as_trigger(trigger)
        if not isinstance(self.trigger, Periodic) or self.trigger.phase != 0:
            raise ValueError("ParticleSorter supports Periodic(period) triggers")
        self.grid = 256 if grid is None else int(grid)

    @property
    def grid_bits(self):
        return max(1, min(9, int(math.ceil(math.log2(max(2, self.grid))))))
