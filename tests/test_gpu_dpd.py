"""DPD thermostat pair forces (hoomd.md.pair.DPD, DPDLJ; PotentialPairDPDThermo): the conservative
parts against DPDConservative and LJ, the full force (drag and random parts with the reference's
Philox streams, Seed(22, timestep, seed), Counter(min tag, max tag)) against an FP64 brute force,
momentum conservation and the thermostat's temperature."""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402


def sim_with(snap, forces, seed=3, dt=0.005, kT=None):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    if kT is not None:
        sim.state.thermalize_particle_momenta(hoomd.filter.All(), kT)
    sim.operations.integrator = md.Integrator(
        dt=dt, forces=forces, methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    return sim


def alpha(tag_i, tag_j, timestep, seed):
    """UniformDistribution<float>(-1, 1) of the pair's Philox stream, in FP32 as the kernel."""
    a, b = min(tag_i, tag_j), max(tag_i, tag_j)
    o = O.philox([0, 0, b, a], O.seed_key(22, timestep, seed))
    u = (int(o[0]) << 32) | int(o[1])
    f = np.float32(u) * np.float32(2.0 ** -64) + np.float32(2.0 ** -65)
    return float(np.float32(-1.0) + np.float32(2.0) * f)


def test_conservative_parts():
    snap = workloads.lj_fluid_sc(8, density=0.8, jitter=0.05, seed=1)
    nl = md.nlist.Cell(buffer=0.4)
    dpd = md.pair.DPD(nlist=nl, kT=1.0, default_r_cut=1.5)
    dpd.params[("A", "A")] = dict(A=25.0, gamma=0.0)
    cons = md.pair.DPDConservative(nlist=nl, default_r_cut=1.5)
    cons.params[("A", "A")] = dict(A=25.0)
    sim_with(snap, [dpd, cons], kT=1.0).run(0)
    assert np.allclose(dpd.forces, cons.forces, rtol=1e-5, atol=1e-4)
    assert math.isclose(dpd.energy, cons.energy, rel_tol=1e-5)
    nl2 = md.nlist.Cell(buffer=0.4)
    dlj = md.pair.DPDLJ(nlist=nl2, kT=1.0, default_r_cut=2.5, mode="shift")
    dlj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, gamma=0.0)
    lj = md.pair.LJ(nlist=nl2, default_r_cut=2.5, mode="shift")
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim_with(snap, [dlj, lj], kT=1.0).run(0)
    assert np.allclose(dlj.forces, lj.forces, rtol=1e-5, atol=1e-4)
    assert math.isclose(dlj.energy, lj.energy, rel_tol=1e-5)


@pytest.mark.parametrize("kind", ["DPD", "DPDLJ"])
def test_full_force_vs_fp64(kind):
    snap = workloads.lj_fluid_sc(7, density=0.85, jitter=0.05, seed=2)
    nl = md.nlist.Cell(buffer=0.3)
    rc, kT, gam, dt, seed = (1.2 if kind == "DPD" else 2.5), 1.3, 4.5, 0.005, 11
    if kind == "DPD":
        f = md.pair.DPD(nlist=nl, kT=kT, default_r_cut=rc)
        f.params[("A", "A")] = dict(A=10.0, gamma=gam)
    else:
        f = md.pair.DPDLJ(nlist=nl, kT=kT, default_r_cut=rc)
        f.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, gamma=gam)
    sim = sim_with(snap, [f], seed=seed, dt=dt, kT=1.0)
    sim.run(0)
    s = sim.state.get_snapshot()
    pos = np.asarray(s.particles.position, np.float32).astype(np.float64)
    vel = np.asarray(s.particles.velocity, np.float32).astype(np.float64)
    N, L = len(pos), s.configuration.box[0]
    F = np.zeros((N, 3))
    for i in range(N):
        d = pos[i] - pos
        d -= L * np.rint(d / L)
        r2 = (d * d).sum(1)
        for j in np.flatnonzero((r2 < rc * rc) & (r2 > 0)):
            r = math.sqrt(r2[j])
            w = 1.0 / r - 1.0 / rc
            if kind == "DPD":
                fd = 10.0 * w
            else:
                ir6 = 1.0 / r2[j] ** 3
                fd = (12.0 * 4 * ir6 * ir6 - 6.0 * 4 * ir6) / r2[j]
            rdotv = d[j] @ (vel[i] - vel[j])
            fd -= gam * rdotv * w * w
            fd += math.sqrt(6.0 * kT * gam / dt) * w * alpha(i, j, 0, seed)
            F[i] += d[j] * fd
    Fg = f.forces
    scale = np.abs(F).max()
    assert np.all(np.abs(Fg - F) <= 1e-4 * np.abs(F) + 2e-5 * scale)


def test_thermostat_and_momentum():
    snap = workloads.lj_fluid_sc(10, density=3.0, jitter=0.05, seed=4)
    f = md.pair.DPD(nlist=md.nlist.Cell(buffer=0.3), kT=1.0, default_r_cut=1.0)
    f.params[("A", "A")] = dict(A=25.0, gamma=4.5)
    sim = sim_with(snap, [f], dt=0.02, kT=0.3)
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.run(500)
    T = []
    for _ in range(40):
        sim.run(25)
        T.append(thermo.kinetic_temperature)
    assert abs(np.mean(T) - 1.0) < 0.05, np.mean(T)
    s = sim.state.get_snapshot()
    P = (s.particles.velocity * s.particles.mass[:, None]).sum(0)
    assert np.abs(P).max() < 1e-2 * math.sqrt(s.particles.N)
