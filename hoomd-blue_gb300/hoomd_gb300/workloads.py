"""Seeded synthetic systems for the benchmark configurations as ``Snapshot`` objects.

The generators live in the numpy-only module ``synthetic_systems`` (shared with the CPU
reference timing, which must not load this package); each function here returns the same
system as a ``hoomd_gb300.Snapshot``.
"""

import synthetic_systems as _S
from synthetic_systems import (KOB_ANDERSEN, mixture_tables, sc_positions,  # noqa: F401
                               table_potential)

from hoomd_gb300.snapshot import Snapshot


def to_snapshot(system):
    """A ``synthetic_systems.HostSystem`` (or any object with its attributes) as a Snapshot; a
    Snapshot is returned unchanged."""
    if isinstance(system, Snapshot):
        return system
    s = Snapshot()
    s.configuration.box = list(system.configuration.box)
    p = system.particles
    s.particles.N = p.N
    s.particles.types = list(p.types)
    s.particles.position[:] = p.position
    s.particles.typeid[:] = p.typeid
    s.particles.velocity[:] = p.velocity
    return s


def lj_fluid_sc(n=16, density=0.84, jitter=0.05, seed=1, types=("A",)):
    return to_snapshot(_S.lj_fluid_sc(n, density, jitter, seed, types))


def lj_fluid_fcc(m=64, density=0.84, jitter=0.05, seed=1):
    return to_snapshot(_S.lj_fluid_fcc(m, density, jitter, seed))


def binary_mixture(N=262144, density=1.2, frac_a=0.8, jitter=0.05, seed=1):
    return to_snapshot(_S.binary_mixture(N, density, frac_a, jitter, seed))


def multitype_system(N=524288, ntypes=32, density=0.8, jitter=0.05, seed=1):
    return to_snapshot(_S.multitype_system(N, ntypes, density, jitter, seed))


def replica_systems(count=256, n_min=500, n_max=20000, rho=(0.7, 0.9), kT=(0.8, 2.0),
                    jitter=0.05, seed=4):
    """[(snapshot, kT, seed)] for ``count`` replicas drawn from one seeded generator."""
    return [(to_snapshot(h), kt, sd) for h, kt, sd in
            _S.replica_systems(count, n_min, n_max, rho, kT, jitter, seed)]


def _snapshot(pos, L, types, typeid):
    """N particles at ``pos`` in a cubic box of side L, as a Snapshot."""
    return to_snapshot(_S.HostSystem(pos, L, types, typeid))
