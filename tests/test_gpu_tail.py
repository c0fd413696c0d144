"""LJ tail corrections (PotentialPair::computeTailCorrection, hoomd/md/PotentialPair.h:255-341),
written after the reference's tests (hoomd/md/pytest/test_potential.py:1172-1291): the energy and
pressure of two particles against the analytic corrections, the shift-mode restriction, the
keyword only on LJ, and a barostat that holds the corrected pressure."""

import numpy as np
import pytest

import hoomd_gb300 as hoomd
from hoomd_gb300 import md, workloads


def two_particle_snapshot(d=1.0, L=20.0):
    s = hoomd.Snapshot()
    s.configuration.box = [L, L, L, 0, 0, 0]
    s.particles.N = 2
    s.particles.position[:] = [[-d / 2, 0, 0.1], [d / 2, 0, 0.1]]
    s.particles.types = ["A"]
    return s


def lj_energy(r, sig, eps):
    return 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)


def energy_correction(sigma, epsilon, r_cut, rho, N):
    lj1 = 4.0 * epsilon * sigma ** 12.0
    lj2 = 4.0 * epsilon * sigma ** 6.0
    return 2 * N * np.pi * rho * (lj1 / 9 / r_cut ** 9 - lj2 / 3 / r_cut ** 3)


def pressure_correction(sigma, epsilon, r_cut, rho):
    lj1 = 4.0 * epsilon * sigma ** 12.0
    lj2 = 4.0 * epsilon * sigma ** 6.0
    return 4 / 6 * rho ** 2 * np.pi * (lj1 * 4 / 3 / r_cut ** 9 - lj2 * 2 / r_cut ** 3)


@pytest.mark.gpu
def test_tail_corrections():
    sigma, epsilon, d_pair, r_cut = 1.0, 0.5, 1.5, 2.0
    v1 = np.array([0.46168675, -0.21020661, 0.21240303])
    res = {}
    for tail in (True, False):
        snap = two_particle_snapshot(d=d_pair)
        snap.particles.velocity[0] = v1
        snap.particles.velocity[1] = -v1
        sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
        sim.create_state_from_snapshot(snap)
        lj = md.pair.LJ(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=r_cut, mode="none",
                        tail_correction=tail)
        lj.params[("A", "A")] = dict(sigma=sigma, epsilon=epsilon)
        sim.operations.integrator = md.Integrator(
            dt=0.005, forces=[lj], methods=[md.methods.Langevin(hoomd.filter.All(), kT=1)])
        sim.always_compute_pressure = True
        thermo = md.compute.ThermodynamicQuantities(filter=hoomd.filter.All())
        sim.operations.computes.append(thermo)
        sim.run(0)
        res[tail] = (thermo.potential_energy, thermo.pressure, lj.energy, lj.additional_energy,
                     lj.additional_virial)
    N, volume = 2, 20.0 ** 3
    rho = N / volume
    dE = energy_correction(sigma, epsilon, r_cut, rho, N)
    dP = pressure_correction(sigma, epsilon, r_cut, rho)
    ke = 0.5 * 2 * np.dot(v1, v1)
    ljf = 24 * epsilon / d_pair * (2 * (sigma / d_pair) ** 12 - (sigma / d_pair) ** 6)
    p0 = (2 * ke / 3 + ljf * d_pair / 3) / volume
    e_true, p_true, elj_true, add_e, add_w = res[True]
    e_false, p_false, elj_false, add_e0, add_w0 = res[False]
    np.testing.assert_allclose(e_false, lj_energy(d_pair, sigma, epsilon), rtol=1e-6)
    np.testing.assert_allclose(e_true, lj_energy(d_pair, sigma, epsilon) + dE, rtol=1e-6)
    np.testing.assert_allclose(p_false, p0, rtol=1e-6)
    np.testing.assert_allclose(p_true, p0 + dP, rtol=1e-6)
    assert e_true < e_false and p_true < p_false
    # the force's own energy carries the correction as its additional energy
    np.testing.assert_allclose(add_e, dE, rtol=1e-12)
    np.testing.assert_allclose(elj_true, elj_false + dE, rtol=1e-6)
    assert add_e0 == 0.0 and add_w0 == [0.0] * 6
    np.testing.assert_allclose(add_w[0], dP * volume, rtol=1e-12)
    assert add_w[1] == add_w[2] == add_w[4] == 0.0 and add_w[0] == add_w[3] == add_w[5]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["none", "shift", "xplor"])
def test_shift_mode_with_lrc(mode):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(two_particle_snapshot(d=0.5))
    lj = md.pair.LJ(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5, mode=mode,
                    tail_correction=True)
    lj.params[("A", "A")] = dict(sigma=1, epsilon=0.5)
    sim.operations.integrator = md.Integrator(
        dt=0.005, forces=[lj], methods=[md.methods.Langevin(hoomd.filter.All(), kT=1)])
    if mode != "none":
        with pytest.raises(RuntimeError):
            sim.run(1)
    else:
        sim.run(1)


def test_lrc_non_lj():
    with pytest.raises(TypeError):
        md.pair.Gaussian(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5, mode="none",
                         tail_correction=True)


@pytest.mark.gpu
def test_barostat_holds_the_corrected_pressure():
    """With the correction the barostat's pressure tensor includes dP, so the measured (corrected)
    pressure settles at the target and the density rises above the uncorrected run's."""
    snap = workloads.lj_fluid_sc(8, density=0.7, jitter=0.05, seed=5)
    vols = {}
    for tail in (True, False):
        sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=3)
        sim.create_state_from_snapshot(snap)
        sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.2)
        lj = md.pair.LJ(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5, mode="none",
                        tail_correction=tail)
        lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
        npt = md.methods.ConstantPressure(
            hoomd.filter.All(), S=1.0, tauS=1.0, couple="xyz",
            thermostat=md.methods.thermostats.MTTK(kT=1.2, tau=0.5))
        sim.operations.integrator = md.Integrator(dt=0.004, forces=[lj], methods=[npt])
        thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
        sim.operations.computes.append(thermo)
        sim.run(3000)
        P, V = [], []
        for _ in range(60):
            sim.run(50)
            P.append(thermo.pressure)
            V.append(sim.state.box.volume)
        vols[tail] = np.mean(V)
        assert abs(np.mean(P) - 1.0) < 0.15, (tail, np.mean(P))
    assert vols[True] < vols[False]
