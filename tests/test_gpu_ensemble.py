"""Replica ensembles on the GPU (the persistent batched launch, C ABI gb_replicas_run), checked
against the CPU oracle replica by replica, against the single-system engine, and against itself
under other launch shapes and after neighbour-list regrowth."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402


def system(N, density, kT, seed):
    """One replica as workloads.replica_systems makes them, with a given size and density."""
    rng = np.random.default_rng(seed)
    L = (N / density) ** (1.0 / 3.0)
    m = int(np.ceil(N ** (1.0 / 3.0) - 1e-9))
    sites = np.sort(rng.choice(m ** 3, N, replace=False))
    pos = workloads.sc_positions(m, L / m)[sites] + rng.uniform(-0.05, 0.05, (N, 3))
    vel = rng.normal(0.0, np.sqrt(kT), (N, 3))
    vel -= vel.mean(axis=0)
    s = workloads._snapshot(pos, L, ("A",), np.zeros(N, np.uint32))
    s.particles.velocity[:] = vel
    return s


# (N, density, kT, seed): a two-cell-per-side box (N = 300 at 0.9), and uneven sizes
SPECS = [(300, 0.9, 1.2, 1), (1000, 0.7, 0.8, 2), (3000, 0.84, 2.0, 3), (8000, 0.8, 1.5, 4),
         (517, 0.75, 1.0, 5)]


def ensemble(specs=SPECS, bussi=True, mode="none", dt=0.005, capacity=None, launch=None,
             stencil=1):
    ens = hoomd.ReplicaEnsemble(dt=dt, r_cut=2.5, buffer=0.4, mode=mode)
    ens._cpp.setStencil(stencil)
    if capacity:
        ens._cpp.setStartCapacity(capacity)
    snaps = []
    for N, rho, kT, seed in specs:
        s = system(N, rho, kT, seed)
        snaps.append(s)
        ens.add_replica(s, kT=kT if bussi else None, seed=seed)
    if launch:
        ens.set_launch(*launch)
    return ens, snaps


def state(ens, r):
    d = ens._cpp.getParticles(r)
    return d["position"], d["velocity"], d["image"], d["force"]


@pytest.mark.parametrize("stencil", [1, 2])
def test_first_build_and_forces_match_oracle(stencil):
    ens, snaps = ensemble(stencil=stencil)
    ens.run(0)
    # 6.93-wide box: cells of r_list give two per side, of r_list / 2 four per side; both are
    # fewer than the stencil's 2S + 1 cells, so every cell of each axis is searched once
    assert ens.record(0)["dim"] == ([2, 2, 2] if stencil == 1 else [4, 4, 4])
    assert ens.record(0)["stencil"] == stencil
    for r, s in enumerate(snaps):
        N = s.particles.N
        box = tuple(s.configuration.box)
        pos32 = O.make_pos4(s.particles.position, np.zeros(N), 32)
        n, l, h, _ = O.build_nlist(pos32, box, [[2.5]], 0.4, full=True, prec=32)
        ref_sets = O.neighbor_sets(n, l, h)
        got = ens.neighbor_sets(r)
        assert all(np.array_equal(a, b) for a, b in zip(got, ref_sets)), r
        pos64 = O.make_pos4(pos32[:, :3].astype(np.float64), np.zeros(N), 64)
        n, l, h, _ = O.build_nlist(pos64, box, [[2.5]], 0.4, full=False, prec=64)
        fo, _ = O.pair_forces("lj", pos64, box, [[1.0, 1.0]], [[6.25]], n, l, h,
                              third_law=True, compute_virial=False, prec=64)
        _, vel, _, F = state(ens, r)
        floor = 1e-5 * np.abs(fo[:, :3]).max()
        err = np.abs(F[:, :3] - fo[:, :3])
        tol = 1e-5 * np.abs(fo[:, :3]) + floor
        f32, _ = O.pair_forces("lj", pos32, box, [[1.0, 1.0]], [[6.25]], n, l, h,
                               third_law=True, compute_virial=False, prec=32)
        err32 = np.abs(f32[:, :3] - fo[:, :3])
        bad = err > tol
        assert not bad.any(), (r, int(bad.sum()), float((err / tol).max()), float(err.max()),
                               float(err32.max()), float((err32 / tol).max()),
                               int((err32 > tol).sum()))
        th = ens.thermo(r)
        assert np.isclose(th["potential_energy"], fo[:, 3].sum(), rtol=1e-5)
        v32 = np.asarray(s.particles.velocity, np.float32).astype(np.float64)
        assert np.isclose(th["kinetic_energy"], 0.5 * (v32 ** 2).sum(), rtol=1e-12)
        assert th["timestep"] == 0


@pytest.mark.parametrize("bussi", [False, True])
def test_trajectories_match_oracle(bussi):
    """20 steps of each replica vs the oracle's FP32 run of the same system (NVE, or Bussi with
    the same seed: the same Philox draws)."""
    specs = SPECS[:3]
    ens, snaps = ensemble(specs, bussi=bussi)
    ens.run(20)
    for r, (s, (N, rho, kT, seed)) in enumerate(zip(snaps, specs)):
        pos4 = O.make_pos4(s.particles.position, np.zeros(N), 32)
        vel4 = np.ones((N, 4), np.float32)
        vel4[:, :3] = s.particles.velocity
        ref = O.Sim(pos4, vel4, np.zeros((N, 3), np.int32), np.arange(N), s.configuration.box,
                    [[2.5]], 0.4, 0.005, params=[[1.0, 1.0]], full=True, prec=32, bussi=bussi,
                    kT=kT, seed=seed)
        ref.run(20)
        o = ref.get()
        p, v, im, _ = state(ens, r)
        box = np.array(s.configuration.box[:3])
        assert np.abs((p + im * box) - (o["pos"][:, :3] + o["image"] * box)).max() < 1e-3
        assert np.abs(v[:, :3] - o["vel"][:, :3]).max() < 1e-2
        assert ens.thermo(r)["timestep"] == 20


def test_launch_shape_changes_nothing():
    """Neighbour order, force sums and energy sums do not depend on the launch shape: the
    trajectories are bit-identical."""
    out = []
    for launch in [(128, 0), (1024, 0), (768, 0), (256, 7), (512, 1)]:
        ens, _ = ensemble(launch=launch)
        ens.run(150)
        out.append([state(ens, r) + (ens.thermo(r),) for r in range(len(SPECS))])
    for other in out[1:]:
        for a, b in zip(out[0], other):
            for x, y in zip(a[:4], b[:4]):
                assert np.array_equal(x, y)
            assert a[4] == b[4]


def test_overflow_regrowth_is_exact():
    """A start capacity of 8 neighbours overflows at the first build: the kernel stops each
    replica where it was, the host grows its block and relaunches; the result equals a run
    that never overflowed, bit for bit."""
    a, _ = ensemble()
    a.run(200)
    b, _ = ensemble(capacity=8)
    b.run(200)
    assert b.n_regrowths >= 1 and a.n_regrowths == 0
    for r in range(len(SPECS)):
        for x, y in zip(state(a, r), state(b, r)):
            assert np.array_equal(x, y)
        assert a.thermo(r) == b.thermo(r)


def test_bussi_temperatures():
    specs = [(800, 0.8, 0.8, 11), (1500, 0.7, 1.4, 12), (600, 0.9, 2.0, 13)]
    ens, _ = ensemble(specs)
    ens.run(300)
    T = {r: [] for r in range(3)}
    for _ in range(25):
        ens.run(20)
        for r in range(3):
            T[r].append(ens.thermo(r)["kinetic_temperature"])
    for r, (N, rho, kT, seed) in enumerate(specs):
        assert abs(np.mean(T[r]) - kT) < 0.04 * kT, (r, np.mean(T[r]), kT)
        assert ens.record(r)["dof"] == 3 * N - 3


def test_nve_energy_conservation():
    specs = [(2000, 0.84, 1.5, 21), (4000, 0.8, 1.2, 22)]
    ens, _ = ensemble(specs, bussi=False, mode="shift", dt=0.004)
    ens.run(20)
    e0 = [ens.thermo(r)["kinetic_energy"] + ens.thermo(r)["potential_energy"] for r in range(2)]
    ens.run(1500)
    for r, (N, *_rest) in enumerate(specs):
        th = ens.thermo(r)
        assert th["n_builds"] > 10
        assert abs(th["kinetic_energy"] + th["potential_energy"] - e0[r]) / N < 2e-3


def test_matches_single_system_engine():
    """One replica vs the same system through hoomd.Simulation (Bussi, same seed): the two
    engines differ only in summation order."""
    N, rho, kT, seed = 3000, 0.84, 1.5, 7
    s = system(N, rho, kT, seed)
    ens = hoomd.ReplicaEnsemble(dt=0.005, r_cut=2.5, buffer=0.4)
    ens.add_replica(s, kT=kT, seed=seed)
    ens.run(25)
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(s)
    cell = md.nlist.Cell(buffer=0.4)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim.operations.integrator = md.Integrator(
        dt=0.005, forces=[lj], methods=[md.methods.ConstantVolume(
            hoomd.filter.All(), thermostat=md.methods.thermostats.Bussi(kT=kT))])
    sim.run(25)
    p, v, im, _ = state(ens, 0)
    s1 = sim.state.get_snapshot()
    box = np.array(s.configuration.box[:3])
    assert np.abs((p + im * box) - (s1.particles.position + s1.particles.image * box)).max() < 1e-3
    assert np.abs(v[:, :3] - s1.particles.velocity).max() < 1e-2


def test_autotune_keeps_trajectory():
    a, _ = ensemble(SPECS[:3])
    trials = a.autotune(steps=4, repeats=1)
    assert len(trials) >= 4
    assert a.launch["block_size"] in (128, 256, 512, 1024)
    steps = a.thermo(0)["timestep"]
    assert steps == 4 * 2 * len(trials)
    b, _ = ensemble(SPECS[:3])
    b.run(steps)
    for r in range(3):
        for x, y in zip(state(a, r), state(b, r)):
            assert np.array_equal(x, y)


def test_errors():
    s = system(400, 0.8, 1.0, 3)
    ens = hoomd.ReplicaEnsemble(dt=0.005)
    s.particles.velocity[:] = 0.0
    ens.add_replica(s, kT=1.0)
    with pytest.raises(RuntimeError, match="non-zero initial momenta"):
        ens.run(1)
    s = system(400, 0.8, 1.0, 3)
    s.particles.position[5] = [1e3, 0, 0]
    ens = hoomd.ReplicaEnsemble(dt=0.005)
    ens.add_replica(s, kT=1.0)
    with pytest.raises(RuntimeError, match="no longer in the simulation box"):
        ens.run(1)
    small = system(100, 0.9, 1.0, 3)  # L = 4.8 < 2 r_list
    with pytest.raises(ValueError, match="too small"):
        hoomd.ReplicaEnsemble(dt=0.005).add_replica(small, kT=1.0)


def test_benchmark_ensemble_first_lists_and_forces():
    """All 256 replicas of the benchmark ensemble (N 500-20,000, density 0.7-0.9, 2.6 M particles,
    the seeded systems of the replicas_256 configuration): after the first build every replica's
    neighbour sets equal the FP32 oracle's, and its forces are no worse against the FP64 oracle
    than the FP32 oracle's (largest error at most 1.5x the FP32 oracle's, values outside 1e-5
    relative at most twice as many, plus the terms of pairs at the cut-off). The replica kernel
    shifts particle i by its image before subtracting, which is closer to FP64 than the
    reference's subtract-then-shift order at FP32, so the FP64 oracle is the reference here."""
    import os

    cores = os.cpu_count() or 1
    systems = workloads.replica_systems(count=256, n_min=500, n_max=20000, seed=4)
    ens = hoomd.ReplicaEnsemble(dt=0.005, r_cut=2.5, buffer=0.4)
    for snap, kT, seed in systems:
        ens.add_replica(snap, kT=kT, seed=seed)
    ens.run(0)
    for r, (s, _, _) in enumerate(systems):
        N = s.particles.N
        box = tuple(s.configuration.box)
        pos32 = O.make_pos4(s.particles.position, np.zeros(N), 32)
        n, l, h, _ = O.build_nlist(pos32, box, [[2.5]], 0.4, full=True, prec=32, nthreads=cores)
        ref = O.neighbor_sets(n, l, h)
        got = ens.neighbor_sets(r)
        assert [len(x) for x in got] == [len(x) for x in ref], r
        assert np.array_equal(np.concatenate(got), np.concatenate(ref)), r
        kw = dict(third_law=False, compute_virial=False, nthreads=cores)
        f32, _ = O.pair_forces("lj", pos32, box, [[1.0, 1.0]], np.float32([[6.25]]), n, l, h,
                               prec=32, **kw)
        b32, _ = O.pair_forces("lj", pos32, box, [[1.0, 1.0]], np.float32([[6.25]]), n, l, h,
                               prec=32, abs_terms=2, **kw)
        pos64 = O.make_pos4(pos32[:, :3].astype(np.float64), np.zeros(N), 64)
        n, l, h, _ = O.build_nlist(pos64, box, [[2.5]], 0.4, full=True, prec=64, nthreads=cores)
        f64, _ = O.pair_forces("lj", pos64, box, [[1.0, 1.0]], [[6.25]], n, l, h, prec=64, **kw)
        b64, _ = O.pair_forces("lj", pos64, box, [[1.0, 1.0]], [[6.25]], n, l, h, prec=64,
                               abs_terms=2, **kw)
        _, _, _, F = state(ens, r)
        ref = f64[:, :3]
        band = b64[:, :3] + b32[:, :3].astype(np.float64)
        e_gpu = np.abs(F[:, :3] - ref)
        e_32 = np.abs(f32[:, :3].astype(np.float64) - ref)
        assert (e_gpu <= 1.5 * e_32.max() + band + 1e-7 * np.abs(ref).max()).all(), (
            r, float(e_gpu.max()), float(e_32.max()))
        plain = 1e-5 * np.abs(ref) + 1e-5 * np.abs(ref).max() + band
        out_gpu, out_32 = int((e_gpu > plain).sum()), int((e_32 > plain).sum())
        assert out_gpu <= 2 * out_32 + 1e-4 * e_gpu.size, (r, out_gpu, out_32)
