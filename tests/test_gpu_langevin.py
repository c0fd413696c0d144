"""Langevin dynamics (hoomd.md.methods.Langevin, hoomd/md/TwoStepLangevin.cc).

Bars: the step-one (NVE order) and step-two kernels bit-exact against the FP32 oracle through the
C ABI, including the Philox random forces; the fused pair-kernel epilogue bit-exact against the
unfused step two; a short trajectory within FP32 round-off of the oracle's run; and, as the
reference's own tests check (hoomd/md/pytest/test_methods.py), the kinetic temperature
settling at kT, the reservoir tally closing the energy balance, and no motion along z in 2D."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import abi, md, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402
from gpu_util import dev, host, p, stream, zeros  # noqa: E402


def state(N=5000, seed=3, ntypes=2):
    rng = np.random.default_rng(seed)
    L = 20.0
    pos4 = O.make_pos4(rng.uniform(-0.5, 0.5, (N, 3)) * L, rng.integers(0, ntypes, N), 32)
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, :3] = rng.normal(0, 2.0, (N, 3))
    vel4[:, 3] = rng.uniform(0.5, 2.0, N)
    acc = rng.normal(0, 50.0, (N, 3)).astype(np.float32)
    img = rng.integers(-2, 3, (N, 3)).astype(np.int32)
    tags = rng.permutation(N).astype(np.uint32)
    force = rng.normal(0, 30, (N, 4)).astype(np.float32)
    return pos4, vel4, acc, img, tags, force, (L, L, L, 0, 0, 0)


def test_nve_order_step_one_bitexact():
    L_ = abi.load()
    pos4, vel4, acc, img, tags, force, box6 = state()
    N = len(pos4)
    dp, dv, da, di = dev(pos4), dev(vel4), dev(acc), dev(img)
    a = abi.StepOneArgs(d_pos=p(dp), d_vel=p(dv), d_accel=p(da), d_image=p(di), N=N,
                        box=abi.make_box(box6[:3]), dt=0.005, scale=0.5, nve_order=1)
    abi.check(L_.gb_md_step_one(ctypes.byref(a), stream()), "step one")
    po, vo, io = O.nve_step_one(pos4, vel4, acc, img, box6, 0.005, prec=32)
    assert np.array_equal(host(dp), po)
    assert np.array_equal(host(dv), vo)  # the scale is ignored in the NVE order
    assert np.array_equal(host(di), io)


@pytest.mark.parametrize("ndim", [3, 2])
def test_langevin_step_two_bitexact(ndim):
    L_ = abi.load()
    pos4, vel4, acc, img, tags, force, box6 = state()
    N = len(pos4)
    gamma = np.array([0.7, 2.5], np.float32)
    kT, dt, seed, ts = 1.3, 0.005, 1234, 987654321
    dv, da = dev(vel4), dev(np.zeros((N, 3), np.float32))
    dp, dt_, df, dg = dev(pos4), dev(tags.view(np.int32)), dev(force), dev(gamma)
    dts = dev(np.array([ts], np.int64))
    scratch = zeros(L_.gb_md_step_scratch_bytes(N) // 4 + 1)
    thermo = dev(np.zeros(3, np.float64))
    res = dev(np.array([0.25], np.float64))
    abi.check(L_.gb_langevin_step_two(p(dv), p(da), p(df), p(dp), p(dt_), p(dg), N, dt, kT, ndim,
                                      seed, p(dts), p(scratch), p(thermo), p(res), stream()),
              "langevin step two")
    vo, ao, e = O.langevin_step_two(vel4, pos4, tags, force, gamma.astype(np.float64), kT, dt,
                                    seed, ts, ndim=ndim, prec=32)
    assert np.array_equal(host(dv), vo)
    assert np.array_equal(host(da).reshape(-1, 3), ao)
    th = host(thermo)
    assert np.isclose(th[0], O.kinetic_energy(vo), rtol=1e-12)
    assert np.isclose(th[1], force[:, 3].astype(np.float64).sum(), rtol=1e-12)
    # the reservoir: the FP64 sum of F_bd . v against the oracle's FP32 sum
    assert np.isclose(host(res)[0], 0.25 - e * dt, rtol=1e-4, atol=1e-6)
    assert int(host(dts)[0]) == ts + 1


def make_sim(snap, gamma=(1.0,), kT=1.2, tally=False, seed=7, fused=True, dt=0.005):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    cell = md.nlist.Cell(buffer=0.4)
    forces = []
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    for a in snap.particles.types:
        for b in snap.particles.types:
            lj.params[(a, b)] = dict(epsilon=1.0, sigma=1.0)
    forces.append(lj)
    if not fused:
        # a second, zero force sends the step through the unfused path
        zero = md.pair.LJ(nlist=cell, default_r_cut=2.5)
        for a in snap.particles.types:
            for b in snap.particles.types:
                zero.params[(a, b)] = dict(epsilon=0.0, sigma=1.0)
        forces.append(zero)
    lang = md.methods.Langevin(hoomd.filter.All(), kT=kT, tally_reservoir_energy=tally)
    for t, g in zip(snap.particles.types, gamma):
        lang.gamma[t] = g
    sim.operations.integrator = md.Integrator(dt=dt, forces=forces, methods=[lang])
    return sim, lang


def test_fused_equals_unfused():
    """The fused pair-kernel epilogue and the separate step-two kernel: after one step the
    positions are identical (step one is shared) and the velocities differ only by the order of
    the force sums of the two pair-kernel launch shapes; after 30 steps still within FP32
    round-off."""
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=1)
    out = {}
    for fused in (True, False):
        sim, _ = make_sim(snap, fused=fused)
        sim.run(1)
        s1 = sim.state.get_snapshot()
        sim.run(29)
        s30 = sim.state.get_snapshot()
        out[fused] = (s1.particles.position.copy(), s1.particles.velocity.copy(),
                      s30.particles.position.copy(), s30.particles.velocity.copy())
    a, b = out[True], out[False]
    assert np.array_equal(a[0], b[0])
    assert np.allclose(a[1], b[1], rtol=1e-5, atol=1e-5)
    assert np.allclose(a[2], b[2], rtol=0, atol=1e-4)
    assert np.allclose(a[3], b[3], rtol=1e-3, atol=1e-3)


def test_trajectory_vs_oracle():
    """20 steps against the oracle's Langevin run (same Philox streams): the force sums differ
    only in order, so the trajectories agree to FP32 round-off."""
    snap = workloads.binary_mixture(N=1000, density=1.0, seed=2)
    gam = (0.5, 2.0)
    sim, _ = make_sim(snap, gamma=gam, kT=1.1, seed=9)
    sim.run(0)
    s0 = sim.state.get_snapshot()
    N = s0.particles.N
    pos4 = O.make_pos4(s0.particles.position, s0.particles.typeid, 32)
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, :3] = s0.particles.velocity
    vel4[:, 3] = s0.particles.mass
    ref = O.Sim(pos4, vel4, s0.particles.image, np.arange(N), tuple(s0.configuration.box),
                [[2.5, 2.5], [2.5, 2.5]], 0.4, 0.005, kind="lj", params=[[1.0, 1.0]] * 4,
                kT=1.1, seed=9, langevin=list(gam))
    sim.run(20)
    ref.run(20)
    s1 = sim.state.get_snapshot()
    r = ref.get()
    box = np.array(s0.configuration.box[:3])
    ug = s1.particles.position + s1.particles.image * box
    uo = r["pos"][:, :3].astype(np.float64) + r["image"] * box
    assert np.abs(ug - uo).max() < 1e-3
    assert np.abs(s1.particles.velocity - r["vel"][:, :3]).max() < 1e-2


def test_temperature_settles_at_kT():
    snap = workloads.lj_fluid_sc(12, density=0.7, jitter=0.05, seed=3)
    sim, _ = make_sim(snap, kT=1.5, seed=11)
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.run(0)
    assert thermo.degrees_of_freedom == 3 * snap.particles.N  # momentum is not conserved
    sim.run(2000)
    T = []
    for _ in range(60):
        sim.run(50)
        T.append(thermo.kinetic_temperature)
    assert abs(np.mean(T) - 1.5) < 0.03, np.mean(T)


def test_reservoir_closes_the_energy_balance():
    """KE + PE + reservoir energy stays constant up to the integrator's error."""
    snap = workloads.lj_fluid_sc(10, density=0.7, jitter=0.05, seed=4)
    sim, lang = make_sim(snap, kT=1.0, tally=True, dt=0.002)
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 3.0)
    sim.run(0)
    e0 = thermo.kinetic_energy + thermo.potential_energy
    assert lang.reservoir_energy == 0.0
    sim.run(2000)
    e1 = thermo.kinetic_energy + thermo.potential_energy
    res = lang.reservoir_energy
    assert abs(e1 - e0) > 100.0  # the bath took the excess heat
    assert abs((e1 + res) - e0) < 0.05 * abs(e1 - e0), (e0, e1, res)


def test_two_dimensions_stays_planar():
    s = hoomd.Snapshot()
    n = 24
    g = (np.arange(n) - n / 2 + 0.5) * 1.1
    x, y = np.meshgrid(g, g)
    s.configuration.box = [n * 1.1, n * 1.1, 0, 0, 0, 0]
    s.particles.N = n * n
    s.particles.position[:, 0] = x.ravel()
    s.particles.position[:, 1] = y.ravel()
    sim, _ = make_sim(s, kT=1.0)
    sim.run(300)
    out = sim.state.get_snapshot()
    assert np.all(out.particles.position[:, 2] == 0.0)
    assert np.all(out.particles.velocity[:, 2] == 0.0)
