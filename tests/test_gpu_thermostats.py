"""ConstantVolume thermostats Berendsen and MTTK (hoomd/md/methods/thermostats.py,
hoomd/md/Thermostat.h): trajectories against the oracle's runs on the fused and the unfused step
paths, the MTTK conserved quantity, temperature control, and the thermostat state API."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402


def make_sim(snap, thermostat, fused=True, seed=5, dt=0.005, mode="none"):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    cell = md.nlist.Cell(buffer=0.4)
    forces = []
    for eps in ((1.0,) if fused else (1.0, 0.0)):
        f = md.pair.LJ(nlist=cell, default_r_cut=2.5, mode=mode)
        for a in snap.particles.types:
            for b in snap.particles.types:
                f.params[(a, b)] = dict(epsilon=eps, sigma=1.0)
        forces.append(f)
    cv = md.methods.ConstantVolume(hoomd.filter.All(), thermostat=thermostat)
    sim.operations.integrator = md.Integrator(dt=dt, forces=forces, methods=[cv])
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    return sim, thermo


def oracle_run(s0, steps, thermostat, kT, tau, state=(0.0, 0.0), seed=5):
    N = s0.particles.N
    pos4 = O.make_pos4(s0.particles.position, s0.particles.typeid, 32)
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, :3] = s0.particles.velocity
    vel4[:, 3] = s0.particles.mass
    ref = O.Sim(pos4, vel4, s0.particles.image, np.arange(N), tuple(s0.configuration.box),
                [[2.5]], 0.4, 0.005, kind="lj", params=[[1.0, 1.0]], kT=kT, tau=tau, seed=seed,
                thermostat=thermostat, mttk_state=state)
    ref.run(steps)
    return ref


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("kind", ["berendsen", "mttk"])
def test_trajectory_vs_oracle(kind, fused):
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=6)
    th = (md.methods.thermostats.Berendsen(kT=1.0, tau=0.3) if kind == "berendsen"
          else md.methods.thermostats.MTTK(kT=1.0, tau=0.3))
    sim, thermo = make_sim(snap, th, fused=fused)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 2.0)
    sim.run(0)
    s0 = sim.state.get_snapshot()
    sim.run(25)
    ref = oracle_run(s0, 25, kind, 1.0, 0.3)
    s1 = sim.state.get_snapshot()
    r = ref.get()
    box = np.array(s0.configuration.box[:3])
    ug = s1.particles.position + s1.particles.image * box
    uo = r["pos"][:, :3].astype(np.float64) + r["image"] * box
    assert np.abs(ug - uo).max() < 1e-3
    assert np.abs(s1.particles.velocity - r["vel"][:, :3]).max() < 1e-2
    st = ref.stats()
    assert np.isclose(thermo.kinetic_energy, st["kinetic_energy"], rtol=1e-4)
    if kind == "mttk":
        xi, eta = th.translational_dof
        rxi, reta = ref.mttk_state
        assert np.isclose(xi, rxi, rtol=1e-4, atol=1e-7)
        assert np.isclose(eta, reta, rtol=1e-4, atol=1e-9)


def test_mttk_conserved_quantity():
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=7)
    th = md.methods.thermostats.MTTK(kT=1.2, tau=0.5)
    sim, thermo = make_sim(snap, th, dt=0.002, mode="shift")
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 2.0)
    sim.run(0)
    H0 = thermo.kinetic_energy + thermo.potential_energy + th.energy
    Hs, Ts = [], []
    for _ in range(40):
        sim.run(100)
        Hs.append(thermo.kinetic_energy + thermo.potential_energy + th.energy)
        Ts.append(thermo.kinetic_temperature)
    N = snap.particles.N
    assert max(abs(h - H0) for h in Hs) / N < 2e-3
    assert abs(np.mean(Ts[10:]) - 1.2) < 0.08
    assert th.translational_dof != (0.0, 0.0)


def test_berendsen_relaxes_to_kT():
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=8)
    sim, thermo = make_sim(snap, md.methods.thermostats.Berendsen(kT=1.0, tau=0.2))
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 2.5)
    sim.run(2000)
    T = []
    for _ in range(20):
        sim.run(20)
        T.append(thermo.kinetic_temperature)
    assert abs(np.mean(T) - 1.0) < 0.02


def test_berendsen_needs_momenta():
    snap = workloads.lj_fluid_sc(6, density=0.8, jitter=0.05, seed=9)
    sim, _ = make_sim(snap, md.methods.thermostats.Berendsen(kT=1.0, tau=0.2))
    with pytest.raises(RuntimeError, match="Berendsen thermostat requires non-zero"):
        sim.run(1)


def test_mttk_state_api():
    snap = workloads.lj_fluid_sc(8, density=0.8, jitter=0.05, seed=10)
    th = md.methods.thermostats.MTTK(kT=1.0, tau=0.4)
    sim, thermo = make_sim(snap, th)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.0)
    th.translational_dof = (0.3, -0.2)
    sim.run(0)
    assert th.translational_dof == (0.3, -0.2)
    dof = thermo.degrees_of_freedom
    assert np.isclose(th.energy, dof * 1.0 * (0.3 ** 2 * 0.4 ** 2 / 2 - 0.2))
    th.thermalize_dof()
    xi, eta = th.translational_dof
    assert xi != 0.3 and eta == -0.2
    assert abs(xi) < 6.0 / np.sqrt(dof * 0.4 ** 2)
    sim.run(10)
    assert th.translational_dof[1] != -0.2
