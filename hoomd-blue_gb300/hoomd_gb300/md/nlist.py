"""Neighbour lists (hoomd/md/nlist.py:87-420). ``Cell`` builds a binned full neighbour list on the
GPU; parity with the reference is per-particle neighbour sets, bit for bit at FP32."""

import numpy as np

from hoomd_gb300._native import _hoomd_gb300
from hoomd_gb300.md.data import TypePairDict, nonnegative_real
from hoomd_gb300.operation import AutotunedObject


def excluded_pairs(topology, exclusions, N):
    """Unordered excluded tag pairs (M, 2), sorted and unique, from the snapshot topology
    (hoomd/md/NeighborList.cc:560-760, the exclusion kinds documented in hoomd/md/nlist.py:55-73):
    'bond', 'constraint', 'special_pair' the groups themselves, 'angle' the first and third
    member, 'dihedral' the first and fourth, '1-3' / '1-4' particles two / three bonds apart."""
    out = []

    def add(a, b):
        a, b = np.asarray(a, np.int64), np.asarray(b, np.int64)
        m = a != b
        out.append(np.stack([np.minimum(a[m], b[m]), np.maximum(a[m], b[m])], 1))

    if 'body' in exclusions:
        pass  # no rigid bodies in this state: nothing to exclude
    bonds = topology["bonds"].group.astype(np.int64)
    if 'bond' in exclusions and len(bonds):
        add(bonds[:, 0], bonds[:, 1])
    if 'constraint' in exclusions and topology["constraints"].N:
        g = topology["constraints"].group
        add(g[:, 0], g[:, 1])
    if 'special_pair' in exclusions and topology["pairs"].N:
        g = topology["pairs"].group
        add(g[:, 0], g[:, 1])
    if 'angle' in exclusions and topology["angles"].N:
        g = topology["angles"].group
        add(g[:, 0], g[:, 2])
    if 'dihedral' in exclusions and topology["dihedrals"].N:
        g = topology["dihedrals"].group
        add(g[:, 0], g[:, 3])
    if ('1-3' in exclusions or '1-4' in exclusions) and len(bonds):
        nbr = [[] for _ in range(N)]
        for a, b in bonds:
            nbr[a].append(b)
            nbr[b].append(a)
        for i in range(N):
            for j in nbr[i]:
                for k in nbr[j]:
                    if k == i:
                        continue
                    if '1-3' in exclusions:
                        add([i], [k])
                    if '1-4' in exclusions:
                        for m in nbr[k]:
                            if m != j and m != i:
                                add([i], [m])
    if not out:
        return np.zeros((0, 2), np.uint32)
    return np.unique(np.concatenate(out), axis=0).astype(np.uint32)


class NeighborList(AutotunedObject):
    _loggables = {"num_builds": "scalar", "shortest_rebuild": "scalar", "dimensions": "sequence",
                  "allocated_particles_per_cell": "scalar"}

    def __init__(self, buffer, exclusions, rebuild_check_delay, check_dist, mesh, default_r_cut):
        exclusions = tuple(exclusions)
        bad = [e for e in exclusions if e not in ('bond', 'angle', 'constraint', 'dihedral',
                                                   'special_pair', 'body', '1-3', '1-4',
                                                   'meshbond')]
        if bad:
            raise ValueError(f"invalid exclusions {bad}")
        if mesh is not None:
            raise NotImplementedError("mesh exclusions are outside the short-range LJ/Table path")
        self._cpp_obj = None
        self.buffer = buffer
        self.exclusions = exclusions
        self.rebuild_check_delay = rebuild_check_delay
        self.check_dist = check_dist
        self.r_cut = TypePairDict(default=float(default_r_cut), validator=nonnegative_real)
        self.r_cut._on_change = self._r_cut_changed
        self._simulation = None
        self._ex_version = -1

    @property
    def buffer(self):
        """Buffer width r_buff; a new value applies from the next run (the list is rebuilt)."""
        return self._buffer

    @buffer.setter
    def buffer(self, value):
        value = float(value)
        if value < 0:
            raise ValueError("buffer must be non-negative")
        self._buffer = value
        if self._cpp_obj is not None:
            self._cpp_obj.r_buff = value
            if self._simulation is not None:
                self._simulation._state_changed()

    @property
    def rebuild_check_delay(self):
        """Check whether the list needs a rebuild only every this many steps after a build
        (NeighborList::shouldCheckDistance); 0 with ``check_dist=False`` rebuilds every step."""
        return self._rebuild_check_delay

    @rebuild_check_delay.setter
    def rebuild_check_delay(self, value):
        value = int(value)
        if value < 0:
            raise ValueError("rebuild_check_delay must be non-negative")
        self._rebuild_check_delay = value
        if self._cpp_obj is not None:
            self._cpp_obj.rebuild_check_delay = value
            self._simulation._state_changed()

    @property
    def check_dist(self):
        """Decide rebuilds by the distance check (True) or rebuild every ``rebuild_check_delay``
        steps (False)."""
        return self._check_dist

    @check_dist.setter
    def check_dist(self, value):
        self._check_dist = bool(value)
        if self._cpp_obj is not None:
            self._cpp_obj.check_dist = self._check_dist
            self._simulation._state_changed()

    @property
    def dangerous_builds(self):
        """Builds found necessary at the first check after a delayed-check period: particles
        may have moved further than half the buffer before the check (the reference's
        'dangerous neighborlist build' notice)."""
        sim = self._simulation
        if sim is None or sim._cpp_integrator is None:
            return 0
        return int(sim._cpp_integrator.status()["dangerous_builds"])

    def _r_cut_changed(self, key):
        if self._cpp_obj is None:
            return
        types = self._simulation.state.particle_types
        for i, a in enumerate(types):
            for j, b in enumerate(types):
                if j >= i:
                    self._cpp_obj.setRCut(i, j, float(self.r_cut[(a, b)]))
        self._simulation._state_changed()

    def _apply_exclusions(self, state):
        pairs = excluded_pairs(state._topology, self.exclusions, state.N_particles)
        self._cpp_obj.setExclusions(pairs)
        self._ex_version = state._topology_version

    def _attach(self, simulation):
        if self._cpp_obj is not None and self._simulation is simulation:
            return self._cpp_obj
        self._simulation = simulation
        state = simulation.state
        self._cpp_obj = _hoomd_gb300.NeighborListGPUBinned(state._cpp_pdata, self.buffer)
        self._cpp_obj.rebuild_check_delay = self.rebuild_check_delay
        self._cpp_obj.check_dist = self.check_dist
        types = state.particle_types
        for i, a in enumerate(types):
            for j, b in enumerate(types):
                if j >= i:
                    self._cpp_obj.setRCut(i, j, float(self.r_cut[(a, b)]))
        self._extra_attach()
        self._apply_exclusions(state)
        return self._cpp_obj

    def _extra_attach(self):
        pass

    def _detach(self):
        self._cpp_obj = None

    @property
    def _attached(self):
        return self._cpp_obj is not None

    def pair_list(self, full=False):
        """Unordered (tag_i, tag_j) pairs currently in the list (the reference's getPairList)."""
        if self._cpp_obj is None:
            raise RuntimeError("the neighbour list has not been computed yet")
        return self._cpp_obj.getPairList(bool(full))

    @property
    def local_pair_list(self):
        """Unordered pairs of the list as the engine's current particle indices, not tags
        (hoomd/md/nlist.py local_pair_list)."""
        if self._cpp_obj is None:
            raise RuntimeError("the neighbour list has not been computed yet")
        return self._cpp_obj.getPairList(False, True)

    @property
    def shortest_rebuild(self):
        """Smallest number of timesteps between two builds since the last Simulation.run
        (NeighborList::getSmallestRebuild: capped at 99; 100 when fewer than two builds)."""
        sim = self._simulation
        if sim is None or sim._cpp_integrator is None:
            raise RuntimeError("shortest_rebuild is available after Simulation.run")
        return int(sim._cpp_integrator.status()["shortest_rebuild"])

    @property
    def num_builds(self):
        sim = self._simulation
        if sim is None or sim._cpp_integrator is None:
            return 0
        return int(sim._cpp_integrator.status()["n_builds"])

    @property
    def dimensions(self):
        d = self._cpp_obj.getDim()
        return (d[0], d[1], d[2])

    @property
    def allocated_particles_per_cell(self):
        return self._cpp_obj.getNmax()


class Cell(NeighborList):
    """hoomd.md.nlist.Cell(buffer, exclusions=('bond',), rebuild_check_delay=1,
    check_dist=True, deterministic=False, mesh=None, default_r_cut=0.0)."""

    def __init__(self, buffer, exclusions=('bond',), rebuild_check_delay=1, check_dist=True,
                 deterministic=False, mesh=None, default_r_cut=0.0):
        super().__init__(buffer, exclusions, rebuild_check_delay, check_dist, mesh,
                         default_r_cut)
        self.deterministic = bool(deterministic)

    def _extra_attach(self):
        self._cpp_obj.deterministic = self.deterministic
