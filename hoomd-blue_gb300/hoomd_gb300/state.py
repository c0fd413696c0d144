"""System state (hoomd/state.py), held on the GPU by the engine's ParticleData."""

import copy

import numpy as np

from hoomd_gb300._native import _hoomd_gb300
from hoomd_gb300.box import Box
from hoomd_gb300.snapshot import Snapshot, is_passive_default


class State:
    def __init__(self, simulation, snapshot):
        snapshot.validate()
        self._simulation = simulation
        self._types = list(snapshot.particles.types)
        self._dimensions = snapshot.configuration.dimensions
        p = snapshot.particles
        self._cpp_pdata = _hoomd_gb300.ParticleData(
            int(p.N), len(self._types), int(self._dimensions),
            [float(x) for x in snapshot.configuration.box], [1, 1, 1])
        self._cpp_pdata.seed = simulation.seed & 0xFFFF
        self._cpp_pdata.types = list(self._types)
        self._cpp_pdata.timestep = simulation._initial_timestep
        self._topology = _copy_topology(snapshot)
        self._topology_version = 0
        self._passive = _copy_passive(snapshot)
        self._counts = None
        self._upload(snapshot)

    def _upload(self, snapshot):
        p = snapshot.particles
        q = self._passive.get("charge")  # None: every charge at its default, 0
        self._cpp_pdata.setParticles(
            np.ascontiguousarray(p.position, np.float64),
            np.ascontiguousarray(p.velocity, np.float64),
            np.ascontiguousarray(p.mass, np.float64),
            np.ascontiguousarray(p.typeid, np.uint32),
            np.ascontiguousarray(p.image, np.int32),
            None if q is None else np.ascontiguousarray(q, np.float64))
        self._counts = None
        self._simulation._state_changed()

    def _type_counts(self):
        """Number of particles of each type."""
        if self._counts is None:
            tid = np.asarray(self._cpp_pdata.getParticles()["typeid"], np.int64)
            self._counts = np.bincount(tid, minlength=len(self._types))
        return self._counts

    @property
    def N_particles(self):
        return self._cpp_pdata.N

    @property
    def particle_types(self):
        return list(self._types)

    @property
    def types(self):
        return dict(particle_types=self.particle_types)

    @property
    def box(self):
        return Box.from_box(self._cpp_pdata.getBox())

    @property
    def dimensions(self):
        return self._dimensions

    def get_snapshot(self):
        d = self._cpp_pdata.getParticles()
        s = Snapshot()
        s.configuration.box = self._cpp_pdata.getBox()
        s.particles.types = self.particle_types
        # the engine's fresh tag-ordered arrays become the snapshot's; passive fields are copied
        # where they differ from their defaults and created at their defaults otherwise
        arrays = {k: d[k] for k in ("position", "velocity", "mass", "typeid", "image")}
        for name, v in self._passive.items():
            arrays[name] = v.copy()
        s.particles._adopt(self.N_particles, arrays)
        for name, g in self._topology.items():
            setattr(s, name, copy.deepcopy(g))
        return s

    def set_snapshot(self, snapshot):
        if snapshot.particles.N != self.N_particles:
            raise RuntimeError("set_snapshot: the number of particles may not change")
        if list(snapshot.particles.types) != self._types:
            raise RuntimeError("set_snapshot: particle types may not change")
        if list(snapshot.configuration.box) != list(self._cpp_pdata.getBox()):
            raise RuntimeError("set_snapshot: box changes are not supported")
        snapshot.validate()
        # no bonds, angles, ... before or after: the topology (and the exclusions built from it)
        # stays as it is without copying the empty sections
        if not (all(getattr(snapshot, k).N == 0 for k in _SECTIONS)
                and all(self._topology[k].N == 0 for k in _SECTIONS)):
            topology = _copy_topology(snapshot)
            if not _same_topology(topology, self._topology):
                self._topology = topology
                self._topology_version += 1
        self._passive = _copy_passive(snapshot)
        self._upload(snapshot)

    def thermalize_particle_momenta(self, filter, kT):
        """Gaussian velocities at kT with zero total momentum (hoomd/state.py:759)."""
        self._cpp_pdata.thermalize(float(kT), self._simulation.timestep)
        self._simulation._state_changed(velocities_only=True)


_SECTIONS = ("bonds", "angles", "dihedrals", "impropers", "constraints", "pairs")
# per-particle quantities the MD step does not change: kept on the host in tag order
_PASSIVE = ("charge", "diameter", "body", "moment_inertia", "orientation", "angmom")


def _copy_passive(snapshot):
    """Host copies of the passive fields that differ from their defaults (a field the snapshot
    never created holds its defaults)."""
    out = {}
    p = snapshot.particles
    for name in _PASSIVE:
        a = p._passive_array(name) if hasattr(p, "_passive_array") else getattr(p, name)
        if a is not None and not is_passive_default(name, a):
            out[name] = np.array(a, copy=True)
    return out


def _copy_topology(snapshot):
    return {name: copy.deepcopy(getattr(snapshot, name)) for name in _SECTIONS}


def _same_topology(a, b):
    return all(a[k].N == b[k].N and np.array_equal(a[k].group, b[k].group) for k in _SECTIONS)
