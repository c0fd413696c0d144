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

    def _tuned_objects(self):
        integ = self._integrator
        out = []
        if integ is not None:
            for f in integ.forces:
                out.append(f)
                if getattr(f, "nlist", None) is not None and f.nlist not in out:
                    out.append(f.nlist)
        return [o for o in out if getattr(o, "_cpp_obj", None) is not None]

    @property
    def is_tuning_complete(self):
        """hoomd.Operations.is_tuning_complete: every attached object's kernel parameters are
        settled."""
        if self._simulation._cpp_integrator is None:
            from hoomd_gb300.error import DataAccessError
            raise DataAccessError("is_tuning_complete")
        return all(o.is_tuning_complete for o in self._tuned_objects())

    def tune_kernel_parameters(self):
        """hoomd.Operations.tune_kernel_parameters: search every attached object's kernel
        parameters at the start of the next run."""
        if self._simulation._cpp_integrator is None:
            raise RuntimeError("Call Simulation.run() before tune_kernel_parameters.")
        for o in self._tuned_objects():
            o.tune_kernel_parameters()

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
        elif hasattr(op, "_write"):
            self.writers.append(op)
            return
        else:
            self.computes.append(op)
        self._simulation._detach_all()


class Simulation:
    _loggables = {"timestep": "scalar", "tps": "scalar", "walltime": "scalar",
                  "final_timestep": "scalar", "initial_timestep": "scalar"}
    _log_namespace = ("Simulation",)

    def __init__(self, device, seed=None):
        self.device = device
        self._seed = 0 if seed is None else int(seed)
        self._initial_timestep = 0
        self._timestep_set = False
        self._run_start = 0
        self._run_end = 0
        self._state = None
        self.operations = Operations(self)
        self._cpp_integrator = None
        self._walltime = 0.0
        self._tps = 0.0
        # hoomd/simulation.py always_compute_pressure: kept for scripts that set it; the virial
        # is computed whenever a pressure is asked for, so it changes nothing here
        self.always_compute_pressure = False

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
        t = int(t)
        if not 0 <= t < 2 ** 64:
            raise ValueError("timestep must be a non-negative 64-bit integer")
        self._initial_timestep = t
        self._timestep_set = True

    @property
    def initial_timestep(self):
        """The timestep at the start of the last run."""
        return self._run_start

    @property
    def final_timestep(self):
        """The timestep at which the last (or current) run ends."""
        return self._run_end

    @property
    def tps(self):
        """Timesteps per second of the last run (System::updateTPS, hoomd/System.cc:183-189)."""
        return self._tps

    @property
    def walltime(self):
        return self._walltime

    def create_state_from_snapshot(self, snapshot):
        """Create the state from a ``Snapshot`` or a ``gsd.hoomd.Frame``
        (hoomd/simulation.py:242-290)."""
        if self._state is not None:
            raise RuntimeError("Cannot initialize more than once")
        if not isinstance(snapshot, Snapshot):
            snapshot = Snapshot.from_gsd_frame(snapshot)
        self._state = State(self, snapshot)

    def create_state_from_gsd(self, filename, frame=-1):
        """Create the state from frame ``frame`` of a GSD file (negative values count from the
        end) as hoomd/simulation.py:188-240 with GSDReader (hoomd/GSDReader.cc:40-90): when the
        timestep was not set, it becomes the frame's ``configuration/step``."""
        if self._state is not None:
            raise RuntimeError("Cannot initialize more than once\n")
        from hoomd_gb300.gsd import hoomd as gh
        with gh.open(filename, "r") as traj:
            n = len(traj)
            i = n - abs(int(frame)) if frame < 0 and abs(int(frame)) <= n else abs(int(frame))
            if i >= n:
                raise RuntimeError(f"Cannot read frame {i} {filename} only has {n} frames.")
            fr = traj[i]
        if fr.particles.N == 0:
            raise RuntimeError("Cannot read a file with 0 particles.")
        if not self._timestep_set:
            self._initial_timestep = int(fr.configuration.step)
        self.create_state_from_snapshot(Snapshot.from_gsd_frame(fr))

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
            self._attach_compute_forces()
            return None
        if self._cpp_integrator is None:
            self._cpp_integrator = integ._attach(self)
            sorter = next((t for t in self.operations.tuners if hasattr(t, "grid_bits")), None)
            if sorter is not None:
                self._cpp_integrator.setSorter(sorter.trigger.period,
                                               sorter._grid_bits(self.state.dimensions))
            self._needs_prep = True
        for f in integ.forces:
            nl = getattr(f, "nlist", None)
            if nl is not None and nl._cpp_obj is not None and \
                    nl._ex_version != self._state._topology_version:
                nl._apply_exclusions(self._state)
                self._needs_prep = True
        for f in list(integ.forces) + list(self.operations.computes):
            if getattr(f, "_pending", False) and getattr(f, "_cpp_obj", None) is not None:
                f._send_params()
                f._pending = False
                # the next run's preparation recomputes the forces at the current positions
                # with the new parameters (IntegratorTwoStep::prepRun; the accelerations of
                # the last step are kept, as there)
                self._needs_prep = True
        if getattr(self, "_needs_prep", False):
            for f in integ.forces:
                if getattr(f, "_cpp_obj", None) is not None and hasattr(f, "_update_tail"):
                    f._update_tail()
            # the particle state or parameters changed: the engine's setters of values its
            # captured step graphs hold drop those graphs themselves, so they are kept here
            self._cpp_integrator.prepRun(True)
            self._needs_prep = False
        for op in self.operations.computes:
            op._simulation = self
        self._attach_compute_forces()
        return self._cpp_integrator

    def _attach_compute_forces(self):
        """Pair forces in ``operations.computes`` that no integrator holds are evaluated on
        their own at the current positions when read (hoomd's forces are computes too)."""
        from hoomd_gb300.md.pair import Pair
        for op in self.operations.computes:
            if isinstance(op, Pair) and op._cpp_obj is None:
                op._attach(self, op.nlist._attach(self))
                op._standalone = True

    def _advance(self, cpp, steps):
        if cpp is None:
            self._state._cpp_pdata.timestep = self.timestep + steps
        else:
            cpp.run(steps)

    def run(self, steps, write_at_start=False):
        """Advance the simulation by ``steps`` timesteps (hoomd/simulation.py:485-562).

        Writers run after each step whose new timestep their trigger selects, and at the
        starting timestep too with ``write_at_start`` (System::run, hoomd/System.cc:80-190);
        the steps between two writes run as one engine call."""
        if self._state is None:
            raise RuntimeError("Cannot run before state is set.")
        steps = int(steps)
        if steps < 0:
            raise ValueError("steps must be non-negative")
        cpp = self._attach()
        if cpp is not None and hasattr(cpp, "resetBuildStats"):
            cpp.resetBuildStats()  # shortest_rebuild counts from this run
        writers = list(self.operations.writers)
        for w in writers:
            w._attach(self)
        start = self.timestep
        self._run_start = start
        self._run_end = start + steps
        t0 = time.perf_counter()
        if write_at_start:
            for w in writers:
                if w.trigger(start):
                    w._write(start)
        t = start
        end = start + steps
        while t < end:
            nxt = min([w.trigger._next(t, end) for w in writers] + [end])
            self._advance(cpp, nxt - t)
            t = nxt
            fire = [w for w in writers if w.trigger(t)]
            if fire and cpp is not None:
                cpp.synchronize()
            for w in fire:
                w._write(t)
        if steps and cpp is not None:
            cpp.synchronize()
        dt = time.perf_counter() - t0
        self._walltime += dt
        if steps and dt > 0:
            self._tps = steps / dt
        for op in self.operations.computes:
            if hasattr(op, "_invalidate"):
                op._invalidate()
