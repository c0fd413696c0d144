"""hoomd_gb300: HOOMD-blue's short-range MD step, GB300-native.

The package mirrors the part of ``hoomd``'s Python API that drives the short-range MD hot path,
so a script written for HOOMD-blue runs after ``import hoomd_gb300 as hoomd``::

    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(snapshot)
    cell = hoomd.md.nlist.Cell(buffer=0.4)
    lj = hoomd.md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[('A', 'A')] = dict(epsilon=1, sigma=1)
    nvt = hoomd.md.methods.ConstantVolume(
        filter=hoomd.filter.All(), thermostat=hoomd.md.methods.thermostats.Bussi(kT=1.5))
    sim.operations.integrator = hoomd.md.Integrator(dt=0.005, methods=[nvt], forces=[lj])
    sim.run(1000)

Everything below the Python objects runs in the compiled engine (hoomd_gb300/_hoomd_gb300*.so,
C++) on hand-written sm_103a kernels reached through the C ABI of include/hoomd_gb300.h
(hoomd_gb300/libhoomd_gb300.so). There is no CPU path.
"""

from hoomd_gb300._native import _hoomd_gb300  # noqa: F401  (fails loudly when not built)
from hoomd_gb300 import device, error, filter, operation, trigger, tune  # noqa: E402
from hoomd_gb300.box import Box  # noqa: E402
from hoomd_gb300.snapshot import Snapshot  # noqa: E402
from hoomd_gb300.simulation import Simulation  # noqa: E402
from hoomd_gb300.state import State  # noqa: E402
from hoomd_gb300 import md  # noqa: E402
from hoomd_gb300 import gsd, logging, write  # noqa: E402
from hoomd_gb300.ensemble import ReplicaEnsemble  # noqa: E402
from hoomd_gb300 import surrogate  # noqa: E402

__version__ = "0.1.0"

__all__ = ["Box", "ReplicaEnsemble", "Snapshot", "Simulation", "State", "device", "filter", "gsd",
           "logging", "md", "surrogate", "trigger", "tune", "write"]
