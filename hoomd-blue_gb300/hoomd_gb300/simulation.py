"""Simulation (hoomd/simulation.py): owns the state and the operations and runs the step loop."""

import time

from hoomd_gb300.snapshot import Snapshot
from hoomd_gb300.state import State


class Operations:
    """hoomd.Operations: the integrator, computes and tuners attached to a simulation."""

    def __init__(self, simulation):
        self._simulation = simulation
        self._integrator = None
        self.computes = []
        self.tuners = []
        self.updaters = []
        self.writers = []

    @property
    def integrator(self):
        return self._integrator

    @integrator.setter
    def integrator(self, integrator):
        if self._integrator is not None:
            self._integrator._detach()
        self._integrator = integrator
        if integrator is not None:
            integrator._simulation = self._simulation
        self._simulation._detach_all()

    def __iadd__(self, op):
        self.add(op)
        return self

    def add(self, op):
        from hoomd_gb300.tune import ParticleSorter
        if isinstance(op, ParticleSorter):
            self.tuners.append(op)
        else:
            self.computes.append(op)
        self._simulation._detach_all()


class Simulation:
    def __init__(self, device, seed=None):
        self.device = device
        self._seed = 0 if seed is None else int(seed)
        self._initial_timestep = 0
        self._state = None
        self.operations = Operations(self)
        self._cpp_integrator = None
        self._walltime = 0.0
        self._tps = 0.0

    @property
    def seed(self):
        return self._seed

    @seed.setter
    def seed(self, v):
        self._seed = int(v) & 0xFFFF
        if self._state is not None:
            self._state._cpp_pdata.seed = self._seed

    @property
    def state(self):
        return self._state

    @property
    def timestep(self):
        if self._state is None:
            return self._initial_timestep
        return int(self._state._cpp_pdata.timestep)

    @timestep.setter
    def timestep(self, t):
        if self._state is not None:
            raise RuntimeError("timestep can only be set before the state is created")
        self._initial_timestep = int(t)

    @property
    def tps(self):
        """Timesteps per second of the last run (System::updateTPS, hoomd/System.cc:183-189)."""
        return self._tps

    @property
    def walltime(self):
        return self._walltime

    def create_state_from_snapshot(self, snapshot):
        if self._state is not None:
            raise RuntimeError("Cannot initialize more than once")
        self._state = State(self, snapshot)

    def _state_changed(self, velocities_only=False):
        # positions or velocities changed outside the engine: prepare again (rebuild the
        # neighbour list, recompute forces, thermodynamics and the Bussi factor) before the
        # next run, as the reference's prepRun does
        self._needs_prep = True

    def _detach_all(self):
        self._cpp_integrator = None
        for op in self.operations.computes:
            if hasattr(op, "_detach"):
                op._detach()

    def _attach(self):
        integ = self.operations.integrator
        if integ is None:
            # no integrator: neighbour lists added as computes are built on their own
            from hoomd_gb300.md.nlist import NeighborList
            for op in self.operations.computes:
                if isinstance(op, NeighborList):
                    op._attach(self).buildNow()
            return None
        if self._cpp_integrator is None:
            self._cpp_integrator = integ._attach(self)
            sorter = next((t for t in self.operations.tuners if hasattr(t, "grid_bits")), None)
            if sorter is not None:
                self._cpp_integrator.setSorter(sorter.trigger.period, sorter.grid_bits)
            self._needs_prep = True
        for f in integ.forces:
            nl = getattr(f, "nlist", None)
            if nl is not None and nl._cpp_obj is not None and \
                    nl._ex_version != self._state._topology_version:
                nl._apply_exclusions(self._state)
                self._needs_prep = True
        if getattr(self, "_needs_prep", False):
            self._cpp_integrator.prepRun()
            self._needs_prep = False
        for op in self.operations.computes:
            op._simulation = self
        return self._cpp_integrator

    def run(self, steps, write_at_start=False):
        """Advance the simulation by ``steps`` timesteps (hoomd/simulation.py:485-562)."""
        if self._state is None:
            raise RuntimeError("Cannot run before state is set.")
        steps = int(steps)
        if steps < 0:
            raise ValueError("steps must be non-negative")
        cpp = self._attach()
        t0 = time.perf_counter()
        if steps and cpp is None:
            self._state._cpp_pdata.timestep = self.timestep + steps
        elif steps:
            cpp.run(steps)
            cpp.synchronize()
        dt = time.perf_counter() - t0
        self._walltime += dt
        if steps and dt > 0:
            self._tps = steps / dt
        for op in self.operations.computes:
            if hasattr(op, "_invalidate"):
                op._invalidate()
