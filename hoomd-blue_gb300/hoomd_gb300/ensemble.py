"""Replica ensembles: many independent LJ systems advanced together on one GPU.

The reference has no batched interface: R independent systems are R ``hoomd.Simulation``
objects, each with its own ``md.nlist.Cell``, ``md.pair.LJ`` and ``md.methods.ConstantVolume``
(Bussi thermostat or NVE), run one after another. ``ReplicaEnsemble`` takes the same per-system
inputs -- a snapshot (positions, velocities, masses, box), a kT, tau and seed per replica -- with
one shared LJ potential, buffer and time step, and advances every replica with ONE persistent
kernel launch per ``run`` (C ABI: ``gb_replicas_run``), replayed from a CUDA graph. Each replica
follows the single-system path step for step: the same half steps, the same distance check and
neighbour-list sets, the same Bussi draws (Philox key (45, timestep, seed), counter 0).

The launch shape (threads per CTA, number of persistent CTAs) changes no result, so
``autotune`` times candidate shapes on live steps, as ``hoomd.tune`` tunes kernel block sizes.
"""

import numpy as np

from hoomd_gb300._native import _hoomd_gb300 as _cpp
from hoomd_gb300.snapshot import Snapshot


class ReplicaEnsemble:
    """Independent single-type LJ replicas sharing one potential and time step.

    Args:
        dt: time step.
        r_cut: LJ cutoff (``default_r_cut``).
        buffer: neighbour-list buffer (``nlist.Cell(buffer=...)``).
        epsilon, sigma: LJ parameters of the one type pair.
        mode: ``"none"`` or ``"shift"`` (``pair.LJ(mode=...)``).
    """

    def __init__(self, dt, r_cut=2.5, buffer=0.4, epsilon=1.0, sigma=1.0, mode="none"):
        modes = {"none": 0, "shift": 1}
        if mode not in modes:
            raise ValueError("mode must be 'none' or 'shift'")
        self.dt = float(dt)
        self._cpp = _cpp.ReplicaEnsembleGPU(float(dt), float(r_cut), float(buffer),
                                            float(epsilon), float(sigma), modes[mode])
        self._boxes = []

    def add_replica(self, snapshot, kT=None, tau=0.0, seed=0, timestep=0):
        """Add one system. ``kT`` = None runs it NVE; otherwise ConstantVolume with
        ``thermostats.Bussi(kT, tau)``. Returns the replica's index."""
        p = snapshot.particles
        box = snapshot.configuration.box
        if snapshot.configuration.dimensions != 3:
            raise ValueError("replicas are three-dimensional")
        if len(p.types) != 1:
            raise ValueError("replicas have one particle type")
        bussi = kT is not None
        r = self._cpp.addReplica(
            np.asarray(p.position, np.float64), np.asarray(p.velocity, np.float64),
            np.asarray(p.mass, np.float64), np.asarray(p.image, np.int32),
            np.asarray(box[:3], np.float64), np.asarray(box[3:6], np.float64), bussi,
            float(kT) if bussi else 1.0, float(tau), int(seed), int(timestep))
        self._boxes.append(list(box))
        return r

    def run(self, steps):
        """Advance every replica by ``steps`` time steps."""
        self._cpp.run(int(steps))

    def autotune(self, steps=20, repeats=2):
        """Time every launch shape on ``steps`` live steps (``repeats`` times, best kept), keep
        the fastest. Advances every replica. Returns the table of trials."""
        out = self._cpp.autotune(int(steps), int(repeats))
        return [dict(block_size=b, grid_size=g, ms_per_step=t) for b, g, t in out]

    def set_launch(self, block_size, grid_size=0):
        self._cpp.setLaunch(int(block_size), int(grid_size))

    @property
    def count(self):
        return self._cpp.count

    @property
    def total_particles(self):
        return self._cpp.total_particles

    @property
    def launch(self):
        return dict(block_size=self._cpp.block_size, grid_size=self._cpp.grid_size)

    @property
    def launch_count(self):
        return self._cpp.launch_count

    @property
    def n_regrowths(self):
        return self._cpp.n_regrowths

    @property
    def last_run_ms(self):
        return self._cpp.last_run_ms

    def thermo(self, r):
        """Energies after the last step of replica ``r`` (ComputeThermo quantities)."""
        rec = self._cpp.record(int(r))
        K = rec["kinetic_energy"]
        return dict(timestep=rec["timestep"], kinetic_energy=K,
                    potential_energy=rec["potential_energy"],
                    kinetic_temperature=2.0 * K / rec["dof"] if rec["dof"] > 0 else 0.0,
                    n_builds=rec["n_builds"])

    def record(self, r):
        return self._cpp.record(int(r))

    def get_snapshot(self, r):
        d = self._cpp.getParticles(int(r))
        s = Snapshot()
        s.configuration.box = self._boxes[r]
        N = len(d["position"])
        s.particles.N = N
        s.particles.position[:] = d["position"]
        s.particles.velocity[:] = d["velocity"][:, :3]
        s.particles.mass[:] = d["velocity"][:, 3]
        s.particles.image[:] = d["image"]
        return s

    def forces(self, r):
        return self._cpp.getParticles(int(r))["force"][:, :3]

    def energies(self, r):
        return self._cpp.getParticles(int(r))["force"][:, 3]

    def neighbor_sets(self, r):
        """Sorted neighbour indices of every particle of replica ``r`` (tests)."""
        nl = self._cpp.neighborList(int(r))
        return [np.sort(row[row >= 0]) for row in nl]
