"""Neighbour lists (hoomd/md/nlist.py:87-420). ``Cell`` builds a binned full neighbour list on the
GPU; parity with the reference is per-particle neighbour sets, bit for bit at FP32."""

from hoomd_gb300._native import _hoomd_gb300
from hoomd_gb300.md.data import TypePairDict, nonnegative_real


class NeighborList:
    def __init__(self, buffer, exclusions, rebuild_check_delay, check_dist, mesh, default_r_cut):
        exclusions = tuple(exclusions)
        bad = [e for e in exclusions if e not in ('bond', 'angle', 'constraint', 'dihedral',
                                                   'special_pair', 'body', '1-3', '1-4',
                                                   'meshbond')]
        if bad:
            raise ValueError(f"invalid exclusions {bad}")
        if mesh is not None:
            raise NotImplementedError("mesh exclusions are outside the short-range LJ/Table path")
        if int(rebuild_check_delay) != 1 or not bool(check_dist):
            raise NotImplementedError("only rebuild_check_delay=1 with check_dist=True (the "
                                      "reference's defaults) is implemented")
        self.buffer = float(buffer)
        if self.buffer < 0:
            raise ValueError("buffer must be non-negative")
        self.exclusions = exclusions
        self.rebuild_check_delay = int(rebuild_check_delay)
        self.check_dist = bool(check_dist)
        self.r_cut = TypePairDict(default=float(default_r_cut), validator=nonnegative_real)
        self._cpp_obj = None
        self._simulation = None

    def _attach(self, simulation):
        if self._cpp_obj is not None and self._simulation is simulation:
            return self._cpp_obj
        self._simulation = simulation
        state = simulation.state
        self._cpp_obj = _hoomd_gb300.NeighborListGPUBinned(state._cpp_pdata, self.buffer)
        types = state.particle_types
        for i, a in enumerate(types):
            for j, b in enumerate(types):
                if j >= i:
                    self._cpp_obj.setRCut(i, j, float(self.r_cut[(a, b)]))
        self._extra_attach()
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
