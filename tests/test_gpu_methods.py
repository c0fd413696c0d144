"""Brownian, OverdampedViscous and DisplacementCapped (hoomd.md.methods; hoomd/md/TwoStepBD.cc,
TwoStepConstantVolume.cc): step one through the C ABI against the FP32 oracle (positions bit-exact,
including the Philox random forces; Brownian velocities, drawn with Box-Muller, to FP32 round-off),
and through the Python API the reference's physical checks: free diffusion at D = kT / gamma,
overdamped relaxation lowering the energy, capped displacements."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import abi, md, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402
from gpu_util import dev, host, p, stream  # noqa: E402


def state(N=4000, seed=5, ntypes=2):
    rng = np.random.default_rng(seed)
    L = 20.0
    pos4 = O.make_pos4(rng.uniform(-0.5, 0.5, (N, 3)) * L, rng.integers(0, ntypes, N), 32)
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, :3] = rng.normal(0, 2.0, (N, 3))
    vel4[:, 3] = rng.uniform(0.5, 2.0, N)
    acc = rng.normal(0, 500.0, (N, 3)).astype(np.float32)
    img = rng.integers(-2, 3, (N, 3)).astype(np.int32)
    tags = rng.permutation(N).astype(np.uint32)
    force = rng.normal(0, 30, (N, 4)).astype(np.float32)
    return pos4, vel4, acc, img, tags, force, (L, L, L, 0, 0, 0)


@pytest.mark.parametrize("noiseless", [False, True])
@pytest.mark.parametrize("ndim", [3, 2])
def test_bd_step_one_vs_oracle(noiseless, ndim):
    L_ = abi.load()
    pos4, vel4, acc, img, tags, force, box6 = state()
    N = len(pos4)
    gamma = np.array([0.8, 3.0], np.float32)
    kT, dt, seed, ts = 1.4, 0.002, 77, 123456789
    dp, dv, da, di = dev(pos4), dev(vel4), dev(acc), dev(img)
    df, dtag, dg = dev(force), dev(tags.view(np.int32)), dev(gamma)
    a = abi.StepOneArgs(d_pos=p(dp), d_vel=p(dv), d_accel=p(da), d_image=p(di), N=N,
                        box=abi.make_box(box6[:3]), dt=dt, scale=1.0, brownian=1,
                        d_bd_force=p(df), d_tag=p(dtag), d_gamma=p(dg), bd_kT=kT, ndim=ndim,
                        seed=seed, timestep=ts, noiseless=int(noiseless))
    abi.check(L_.gb_md_step_one(ctypes.byref(a), stream()), "bd step one")
    po, vo, io = O.bd_step_one(pos4, vel4, force, img, tags, gamma.astype(np.float64), box6, kT,
                               dt, seed, ts, ndim=ndim, noiseless=noiseless, prec=32)
    assert np.array_equal(host(dp), po)
    assert np.array_equal(host(di), io)
    v = host(dv)
    if noiseless:
        assert np.array_equal(v, vo)
    else:
        assert np.allclose(v[:, :3], vo[:, :3], rtol=2e-5, atol=2e-6)
        assert np.array_equal(v[:, 3], vel4[:, 3])
    if ndim == 2:
        assert np.all(v[:, 2] == 0.0)


def test_displacement_capped_step_one_vs_oracle():
    L_ = abi.load()
    pos4, vel4, acc, img, tags, force, box6 = state()
    N = len(pos4)
    dt, limit = 0.005, 0.02
    dp, dv, da, di = dev(pos4), dev(vel4), dev(acc), dev(img)
    a = abi.StepOneArgs(d_pos=p(dp), d_vel=p(dv), d_accel=p(da), d_image=p(di), N=N,
                        box=abi.make_box(box6[:3]), dt=dt, scale=1.0, max_displacement=limit)
    abi.check(L_.gb_md_step_one(ctypes.byref(a), stream()), "capped step one")
    po, vo, io = O.cv_step_one_capped(pos4, vel4, acc, img, box6, dt, 1.0, limit, prec=32)
    assert np.array_equal(host(dp), po)
    assert np.array_equal(host(dv), vo)
    v = host(dv)[:, :3].astype(np.float64)
    capped = np.linalg.norm(v, axis=1) * dt
    assert capped.max() <= limit * (1 + 1e-5)
    assert (capped > 0.99 * limit).sum() > N // 10  # the cap was active for many particles


def free_particles(n=16, L=40.0, seed=1):
    """A dilute gas with a zero pair force: only the method moves the particles."""
    s = workloads.lj_fluid_sc(n, density=(n ** 3) / L ** 3, jitter=0.05, seed=seed)
    return s


def make_sim(snap, method, seed=3, dt=0.005, eps=0.0, mode="none"):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    lj = md.pair.LJ(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5, mode=mode)
    lj.params[("A", "A")] = dict(epsilon=eps, sigma=1.0)
    sim.operations.integrator = md.Integrator(dt=dt, forces=[lj], methods=[method])
    return sim, lj


def test_brownian_free_diffusion():
    """Mean squared displacement of free particles: 6 D t with D = kT / gamma."""
    snap = free_particles()
    kT, gamma, dt, steps = 1.5, 2.0, 0.005, 400
    bd = md.methods.Brownian(hoomd.filter.All(), kT=kT)
    bd.gamma["A"] = gamma
    sim, _ = make_sim(snap, bd, dt=dt)
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.run(0)
    s0 = sim.state.get_snapshot()
    assert thermo.degrees_of_freedom == 3 * snap.particles.N
    sim.run(steps)
    s1 = sim.state.get_snapshot()
    box = np.array(snap.configuration.box[:3])
    u0 = s0.particles.position + s0.particles.image * box
    u1 = s1.particles.position + s1.particles.image * box
    msd = ((u1 - u0) ** 2).sum(1).mean()
    expect = 6 * kT / gamma * dt * steps
    assert abs(msd / expect - 1) < 0.05, (msd, expect)
    # velocities are drawn from the Maxwell-Boltzmann distribution at kT
    assert abs(thermo.kinetic_temperature - kT) < 0.05 * kT


def test_overdamped_viscous_relaxes():
    """With no noise the energy decreases monotonically and v = F / gamma."""
    snap = workloads.lj_fluid_sc(8, density=1.0, jitter=0.05, seed=2)
    ov = md.methods.OverdampedViscous(hoomd.filter.All(), default_gamma=5.0)
    sim, lj = make_sim(snap, ov, dt=0.0005, eps=1.0, mode="shift")
    sim.run(0)
    e = [lj.energy]
    for _ in range(20):
        sim.run(20)
        e.append(lj.energy)
    assert all(b <= a + 1e-6 * abs(a) for a, b in zip(e, e[1:]))
    assert e[-1] < e[0]
    s = sim.state.get_snapshot()
    F = lj.forces
    # the velocities are the forces of the previous step over gamma: same scale, same direction
    cos = (s.particles.velocity * F).sum(1) / (
        np.linalg.norm(s.particles.velocity, axis=1) * np.linalg.norm(F, axis=1) + 1e-30)
    assert np.median(cos) > 0.99


def test_displacement_capped_limits_steps():
    snap = workloads.lj_fluid_sc(8, density=1.0, jitter=0.25, seed=4)
    dc = md.methods.DisplacementCapped(hoomd.filter.All(), maximum_displacement=1e-3)
    sim, lj = make_sim(snap, dc, dt=0.005, eps=1.0)
    sim.run(0)
    for _ in range(5):
        s0 = sim.state.get_snapshot()
        sim.run(1)
        s1 = sim.state.get_snapshot()
        box = np.array(snap.configuration.box[:3])
        d = (s1.particles.position + s1.particles.image * box) - (
            s0.particles.position + s0.particles.image * box)
        # FP32 positions near 4 carry 5e-7 of rounding
        assert np.linalg.norm(d, axis=1).max() <= 1e-3 + 2e-6
