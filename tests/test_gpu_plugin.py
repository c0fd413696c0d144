"""A pair evaluator built as a plugin module runs on this library's kernels (the reference's
example_plugins/pair_plugin path: evaluator header + kernel instantiation + module export +
Python class with _ext_module / _cpp_class_name).

The plugin is the Hertz evaluator of tests/pair_plugin/, written to the reference's evaluator
concept (EvaluatorPairExample.h). Checks: the two-particle closed form over distances,
parameters and shift modes (after example_plugins/pair_plugin/pytest/test_example_pair.py, at
the FP32 tolerance of this library), the parameters read back through getParams, forces,
energies and virials of a dense system against an FP64 brute force, the energy between two sets,
and a fused NVE run that conserves energy.
"""

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from plugin_util import hertz_pair_class  # noqa: E402

HertzPair, _MOD = hertz_pair_class()


def hertz(r, eps, sigma):
    """(V, -dV/dr) of the Hertz potential, FP64."""
    gap = np.clip(1.0 - r / sigma, 0.0, None)
    return eps * gap ** 2.5, 2.5 * eps / sigma * gap ** 1.5


def two_particles(d, L=20.0):
    s = hoomd.Snapshot()
    s.configuration.box = [L, L, L, 0, 0, 0]
    s.particles.N = 2
    s.particles.types = ["A"]
    s.particles.position[:] = [[-d / 2, 0, 0.1], [d / 2, 0, 0.1]]
    return s


def simulation(snap, force, kT=None, dt=0.002):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=3)
    sim.create_state_from_snapshot(snap)
    th = None if kT is None else md.methods.thermostats.Bussi(kT=kT)
    sim.operations.integrator = md.Integrator(
        dt=dt, forces=[force], methods=[md.methods.ConstantVolume(hoomd.filter.All(), th)])
    return sim


@pytest.mark.parametrize("d, eps, sigma, mode", list(itertools.product(
    np.linspace(0.1, 2.0, 3), [0.5, 2.0, 5.0], [0.5, 1.0, 1.5], ["none", "shift"])))
def test_two_particle_closed_form(d, eps, sigma, mode):
    f = HertzPair(md.nlist.Cell(buffer=0.4), default_r_cut=sigma, mode=mode)
    f.params[("A", "A")] = dict(epsilon=eps, sigma=sigma)
    sim = simulation(two_particles(d), f)
    sim.run(0)
    snap = sim.state.get_snapshot()
    dx = snap.particles.position[1] - snap.particles.position[0]
    r = np.linalg.norm(dx)
    V, F = hertz(r, eps, sigma) if r < sigma else (0.0, 0.0)
    # at r_cut = sigma the shift is V(sigma) = 0
    fvec = F * dx / r
    np.testing.assert_allclose(f.forces, [-fvec, fvec], rtol=1e-5, atol=1e-6 * max(1.0, F))
    np.testing.assert_allclose(f.energies, [V / 2, V / 2], rtol=1e-5, atol=1e-7)


def test_parameters_round_trip_and_evaluator_name():
    f = HertzPair(md.nlist.Cell(buffer=0.4), default_r_cut=1.1)
    f.params[("A", "A")] = dict(epsilon=1.25, sigma=1.1)
    sim = simulation(two_particles(0.9), f)
    sim.run(0)
    got = f._cpp_obj.getParams(("A", "A"))
    assert got == {"epsilon": pytest.approx(1.25), "sigma": pytest.approx(1.1)}
    assert f._cpp_obj.getRCut(("A", "A")) == pytest.approx(1.1)
    assert f._cpp_obj.mode == "none"
    assert f._cpp_obj.evaluator_name == "hertz"


def _dense_system():
    snap = workloads.lj_fluid_sc(10, density=1.3, jitter=0.1, seed=12)
    return snap, snap.configuration.box[0]


def _brute(pos, L, eps, sigma):
    d = pos[:, None, :] - pos[None, :, :]
    d -= L * np.rint(d / L)
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, np.inf)
    V, F = hertz(r, eps, sigma)
    inside = r < sigma
    V = np.where(inside, V, 0.0)
    fdr = np.where(inside, F / r, 0.0)
    forces = (fdr[..., None] * d).sum(1)
    energies = 0.5 * V.sum(1)
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    vir = np.stack([0.5 * (fdr * d[..., a] * d[..., b]).sum(1) for a, b in pairs], 1)
    return forces, energies, vir, V


def test_dense_system_vs_fp64_brute_force():
    snap, L = _dense_system()
    f = HertzPair(md.nlist.Cell(buffer=0.3), default_r_cut=1.0)
    f.params[("A", "A")] = dict(epsilon=3.0, sigma=1.0)
    sim = simulation(snap, f)
    sim.operations.computes.append(md.compute.ThermodynamicQuantities(hoomd.filter.All()))
    sim.run(0)
    pos = sim.state.get_snapshot().particles.position
    F, E, W, V = _brute(pos, L, 3.0, 1.0)
    tol = dict(rtol=1e-5, atol=1e-5 * np.abs(F).max())
    np.testing.assert_allclose(f.forces, F, **tol)
    np.testing.assert_allclose(f.energies, E, rtol=1e-5, atol=1e-5 * np.abs(E).max())
    np.testing.assert_allclose(f.virials, W, rtol=1e-5, atol=1e-5 * np.abs(W).max())
    # energy between two sets (the plugin's energy-between-sets kernel)
    tags = np.arange(len(pos))
    a, b = tags[::3], np.setdiff1d(tags, tags[::3])
    assert f.compute_energy(a, b) == pytest.approx(V[np.ix_(a, b)].sum(), rel=2e-5)


def test_fused_nve_run_conserves_energy():
    snap, L = _dense_system()
    f = HertzPair(md.nlist.Cell(buffer=0.3), default_r_cut=1.0)
    f.params[("A", "A")] = dict(epsilon=3.0, sigma=1.0)
    sim = simulation(snap, f, dt=0.002)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.0)
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.run(0)
    e0 = thermo.kinetic_energy + thermo.potential_energy
    sim.run(500)
    e1 = thermo.kinetic_energy + thermo.potential_energy
    assert np.isfinite(e1)
    assert abs(e1 - e0) < 2e-3 * abs(e0)
    assert sim._cpp_integrator.launch_count > 0
