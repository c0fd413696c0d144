"""GSD through a simulation on the GPU: hoomd.write.GSD on a trigger during a run,
Simulation.create_state_from_gsd, checkpoint and resume, and logged quantities."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from hoomd_gb300.gsd import hoomd as gh  # noqa: E402


def lj_sim(snap_or_file, seed=2, frame=-1, timestep=None):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    if timestep is not None:
        sim.timestep = timestep
    if isinstance(snap_or_file, str):
        sim.create_state_from_gsd(snap_or_file, frame=frame)
    else:
        sim.create_state_from_snapshot(snap_or_file)
    cell = md.nlist.Cell(buffer=0.4)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    nvt = md.methods.ConstantVolume(
        filter=hoomd.filter.All(), thermostat=md.methods.thermostats.Bussi(kT=1.2))
    sim.operations.integrator = md.Integrator(dt=0.005, forces=[lj], methods=[nvt])
    return sim, lj


def test_writer_trigger_and_resume(tmp_path):
    path = str(tmp_path / "traj.gsd")
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=1)
    snap.particles.charge[:] = np.linspace(-1, 1, snap.particles.N)
    sim, lj = lj_sim(snap)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.2)
    w = hoomd.write.GSD(trigger=hoomd.trigger.Periodic(40), filename=path, mode="wb",
                        dynamic=["property", "momentum"])
    sim.operations.writers.append(w)
    sim.run(120, write_at_start=True)
    end = sim.state.get_snapshot()
    w.flush()
    with gh.open(path) as t:
        assert [f.configuration.step for f in t] == [0, 40, 80, 120]
        last = t[-1]
        assert np.array_equal(last.particles.position, end.particles.position.astype(np.float32))
        assert np.array_equal(last.particles.velocity, end.particles.velocity.astype(np.float32))
        assert np.array_equal(last.particles.image, end.particles.image)
        assert np.array_equal(last.particles.charge, snap.particles.charge.astype(np.float32))
    # resume from step 40 and run to 120: the same trajectory within FP32 round-off (the
    # neighbour list is rebuilt at the restart, so sums may run in another order)
    sim2, _ = lj_sim(path, frame=1)
    assert sim2.timestep == 40
    sim2.run(80)
    s2 = sim2.state.get_snapshot()
    box = np.array(snap.configuration.box[:3])
    u1 = end.particles.position + end.particles.image * box
    u2 = s2.particles.position + s2.particles.image * box
    assert np.abs(u1 - u2).max() < 2e-3
    assert np.array_equal(s2.particles.charge, end.particles.charge.astype(np.float32))
    # an explicit timestep wins over the file's step
    sim3, _ = lj_sim(path, frame=-1, timestep=7)
    assert sim3.timestep == 7


def test_static_write_round_trip(tmp_path):
    path = str(tmp_path / "one.gsd")
    snap = workloads.lj_fluid_sc(6, density=0.7, jitter=0.05, seed=3)
    snap.particles.types = ["A", "B"]
    snap.particles.typeid[::2] = 1
    snap.particles.mass[:] = 1.5
    snap.particles.diameter[:] = 0.8
    snap.bonds.N = 2
    snap.bonds.types = ["b"]
    snap.bonds.group[:] = [[0, 1], [2, 3]]
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(snap)
    hoomd.write.GSD.write(state=sim.state, filename=path)
    sim2 = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim2.create_state_from_gsd(path)
    a, b = sim.state.get_snapshot(), sim2.state.get_snapshot()
    assert b.particles.types == ["A", "B"]
    assert np.array_equal(a.particles.typeid, b.particles.typeid)
    assert np.array_equal(a.particles.position.astype(np.float32),
                          b.particles.position.astype(np.float32))
    assert np.allclose(b.particles.mass, 1.5)
    assert np.allclose(b.particles.diameter, 1.0)  # diameter is written only on request
    assert b.bonds.N == 2 and np.array_equal(b.bonds.group, [[0, 1], [2, 3]])


def test_logged_thermodynamics(tmp_path):
    path = str(tmp_path / "log.gsd")
    snap = workloads.lj_fluid_sc(8, density=0.8, jitter=0.05, seed=4)
    sim, lj = lj_sim(snap)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.2)
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    logger = hoomd.logging.Logger(categories=["scalar"])
    logger.add(thermo, quantities=["kinetic_energy", "potential_energy"])
    logger.add(sim, quantities=["timestep"])
    sim.operations.writers.append(
        hoomd.write.GSD(trigger=25, filename=path, mode="wb", logger=logger))
    sim.run(50)
    with gh.open(path) as t:
        assert len(t) == 2
        log = t[-1].log
        assert log["Simulation/timestep"][0] == 50
        assert np.isclose(log["md/compute/ThermodynamicQuantities/potential_energy"][0],
                          thermo.potential_energy)
        assert np.isclose(log["md/compute/ThermodynamicQuantities/kinetic_energy"][0],
                          thermo.kinetic_energy)
