"""End-to-end GPU tests through the hoomd-style Python API, written like the reference's own tests
(hoomd/md/pytest/test_potential.py, test_nlist.py, example_plugins/pair_plugin/pytest), checked
against the golden fixtures and the CPU oracle."""

import itertools
import json
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402
from gpu_util import assert_close_cond  # noqa: E402

GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def two_particle_snapshot(d=1.0, L=20.0):
    s = hoomd.Snapshot()
    s.configuration.box = [L, L, L, 0, 0, 0]
    s.particles.N = 2
    s.particles.position[:] = [[-d / 2, 0, 0.1], [d / 2, 0, 0.1]]
    s.particles.types = ["A"]
    return s


def make_sim(snap, seed=22765):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    return sim


@pytest.mark.parametrize("pot", ["LJ", "Table"])
def test_force_energy_accuracy(pot):
    """hoomd/md/pytest/test_potential.py:952-1058 on the golden fixture."""
    fe = json.load(open(GOLD / "forces_and_energies_lj_table.json"))[pot]
    for i, params in enumerate(fe["params"]):
        cls = getattr(md.pair, pot)
        f = cls(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5)
        f.params[("A", "A")] = params
        sim = make_sim(two_particle_snapshot(d=0.75))
        sim.operations.integrator = md.Integrator(
            dt=0.005, forces=[f], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
        sim.run(0)
        for k, d in enumerate([0.75, 1.5]):
            snap = sim.state.get_snapshot()
            snap.particles.position[0] = [0, 0, 0.1]
            snap.particles.position[1] = [0, 0, d + 0.1]
            sim.state.set_snapshot(snap)
            e = f.energies
            forces = f.forces
            ref_e = fe["energies"][i][k]
            assert np.isclose(e.sum(), ref_e, rtol=1e-5, atol=1e-6 if ref_e == 0 else 0)
            assert np.allclose(forces[0], np.array([0, 0, 1.0]) * fe["forces"][i][k], rtol=1e-5,
                               atol=1e-5)


def test_true_pair_list():
    """hoomd/md/pytest/test_nlist.py:221-372 (standalone Cell compute, r_cut 1.1, buffer 0)."""
    truth = set(frozenset(p) for p in json.load(open(GOLD / "true_pair_list_sc7.json")))
    s = hoomd.Snapshot()
    s.configuration.box = [7, 7, 7, 0, 0, 0]
    s.particles.N = 343
    s.particles.position[:] = workloads.sc_positions(7, 1.0)
    sim = make_sim(s)
    nlist = md.nlist.Cell(buffer=0.0, default_r_cut=1.1)
    sim.operations.computes.append(nlist)
    sim.run(0)
    got = set(frozenset(map(int, p)) for p in nlist.pair_list())
    assert got == truth
    # nothing has reordered the particles, so the indices of local_pair_list are the tags
    local = nlist.local_pair_list
    assert len(local) == len(truth) and np.all(local[:, 0] < local[:, 1])
    assert set(frozenset(map(int, p)) for p in local) == truth


def harm_force_and_energy(dx, k, sigma, r_cut, shift=False):
    dr = np.linalg.norm(dx)
    if dr >= r_cut:
        return np.zeros(3), 0.0
    f = k * (sigma - dr) * np.asarray(dx, np.float64) / dr
    e = 0.5 * k * (sigma - dr) ** 2
    if shift:
        e -= 0.5 * k * (r_cut - sigma) ** 2
    return f, e


@pytest.mark.parametrize("distance, k, sigma, mode",
                         list(itertools.product(np.linspace(0.1, 2.0, 3), [0.5, 2.0, 5.0],
                                                [0.5, 1.0, 1.5], ["none", "shift"])))
def test_example_pair_plugin(distance, k, sigma, mode):
    """example_plugins/pair_plugin/pytest/test_example_pair.py."""
    sim = make_sim(two_particle_snapshot(d=distance))
    cell = md.nlist.Cell(buffer=0.4)
    ex = md.pair.ExamplePair(cell, default_r_cut=sigma, mode=mode)
    ex.params[("A", "A")] = dict(k=k, sigma=sigma)
    sim.operations.integrator = md.Integrator(
        dt=0.001, forces=[ex], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    sim.run(0)
    snap = sim.state.get_snapshot()
    vec = snap.particles.position[1] - snap.particles.position[0]
    f, e = harm_force_and_energy(vec, k, sigma, sigma, mode == "shift")
    np.testing.assert_array_almost_equal(ex.forces, [-f, f], decimal=5)
    np.testing.assert_array_almost_equal(ex.energies, [e / 2, e / 2], decimal=5)


def lj_sim(snap, kT=None, dt=0.005, mode="none", sorter=None, seed=5, thermalize=1.5):
    sim = make_sim(snap, seed)
    if thermalize:
        sim.state.thermalize_particle_momenta(hoomd.filter.All(), thermalize)
    cell = md.nlist.Cell(buffer=0.4)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5, mode=mode)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    th = None if kT is None else md.methods.thermostats.Bussi(kT=kT)
    sim.operations.integrator = md.Integrator(
        dt=dt, forces=[lj], methods=[md.methods.ConstantVolume(hoomd.filter.All(), th)])
    if sorter:
        sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=sorter))
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    return sim, lj, cell, thermo


def test_run0_forces_match_fp64_oracle():
    snap = workloads.lj_fluid_sc(16)
    sim, lj, cell, thermo = lj_sim(snap, thermalize=None)
    sim.run(0)
    pos4 = O.make_pos4(sim.state.get_snapshot().particles.position, np.zeros(4096), 64)
    box = tuple(snap.configuration.box)
    n, l, h, _ = O.build_nlist(pos4, box, [[2.5]], 0.4, full=False, prec=64)
    fo, vo = O.pair_forces("lj", pos4, box, [[1.0, 1.0]], [[6.25]], n, l, h, third_law=True,
                           compute_virial=True, prec=64)
    F = lj.forces
    floor = 1e-5 * np.abs(fo[:, :3]).max()
    assert np.all(np.abs(F - fo[:, :3]) <= 1e-5 * np.abs(fo[:, :3]) + floor)
    assert np.isclose(lj.energy, fo[:, 3].sum(), rtol=1e-5)
    V = lj.virials
    assert np.all(np.abs(V - vo.T) <= 1e-5 * np.abs(vo.T) + 1e-5 * np.abs(vo).max())
    assert np.isclose(thermo.potential_energy, fo[:, 3].sum(), rtol=1e-5)


def test_trajectory_matches_oracle_short_nve():
    """20 NVE steps: GPU FP32 vs the oracle's FP32 CPU run from the same state (per-particle
    positions agree to FP32 round-off amplified by the dynamics)."""
    snap = workloads.lj_fluid_sc(12, density=0.84)
    N = snap.particles.N
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    s0 = sim.state.get_snapshot()
    sim.run(20)
    s1 = sim.state.get_snapshot()
    pos4 = O.make_pos4(s0.particles.position, np.zeros(N), 32)
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, :3] = s0.particles.velocity
    vel4[:, 3] = 1.0
    ref = O.Sim(pos4, vel4, np.zeros((N, 3), np.int32), np.arange(N), snap.configuration.box,
                [[2.5]], 0.4, 0.005, params=[[1.0, 1.0]], full=True, prec=32)
    ref.run(20)
    r = ref.get()
    box = np.array(snap.configuration.box[:3])
    unwrapped_gpu = s1.particles.position + s1.particles.image * box
    unwrapped_ref = r["pos"][:, :3] + r["image"] * box
    assert np.abs(unwrapped_gpu - unwrapped_ref).max() < 1e-3
    assert np.abs(s1.particles.velocity - r["vel"][:, :3]).max() < 1e-2


def test_nve_energy_conservation():
    snap = workloads.lj_fluid_sc(16)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, mode="shift", thermalize=1.5, dt=0.004)
    sim.run(50)
    e0 = thermo.kinetic_energy + thermo.potential_energy
    sim.run(2000)
    e1 = thermo.kinetic_energy + thermo.potential_energy
    assert cell.num_builds > 10
    assert abs(e1 - e0) / snap.particles.N < 2e-3


def test_bussi_thermostat_temperature():
    snap = workloads.lj_fluid_sc(16)
    sim, lj, cell, thermo = lj_sim(snap, kT=1.5, thermalize=0.5)
    sim.run(300)
    Ts = []
    for _ in range(20):
        sim.run(20)
        Ts.append(thermo.kinetic_temperature)
    assert abs(np.mean(Ts) - 1.5) < 0.05
    assert thermo.degrees_of_freedom == 3 * snap.particles.N - 3


def test_sorter_does_not_change_physics():
    snap = workloads.lj_fluid_sc(14)
    out = []
    for sorter in (None, 7):
        sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0, sorter=sorter)
        sim.run(30)
        out.append((sim.state.get_snapshot(), lj.forces))
    (s_a, f_a), (s_b, f_b) = out
    box = np.array(snap.configuration.box[:3])
    ua = s_a.particles.position + s_a.particles.image * box
    ub = s_b.particles.position + s_b.particles.image * box
    assert np.abs(ua - ub).max() < 1e-3
    assert np.abs(f_a - f_b).max() < 1e-2 * max(1.0, np.abs(f_a).max())


def test_overflow_rolls_back_and_matches():
    """Start the cell list and neighbour list exactly full: the melting lattice overflows inside
    a replayed run, the engine restores its checkpoint, grows and repeats the run. The result
    must equal a run that never overflowed."""
    snap = workloads.lj_fluid_sc(14)
    res = []
    for tight in (False, True):
        sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=2.0)
        sim.run(0)
        if tight:
            pos4 = O.make_pos4(sim.state.get_snapshot().particles.position, np.zeros(14 ** 3), 32)
            box = tuple(snap.configuration.box)
            n, _, _, info = O.build_nlist(pos4, box, [[2.5]], 0.4, full=True, prec=32)
            need = int(n.max())
            cell._cpp_obj.setStartCapacity(int(info["cell_size"].max()), [need])
            sim._needs_prep = True
        sim.run(200)
        integ = sim._cpp_integrator
        res.append((sim.state.get_snapshot(), integ.n_rollbacks))
    (a, rb_a), (b, rb_b) = res
    assert rb_a == 0 and rb_b >= 1
    assert np.abs(a.particles.position - b.particles.position).max() < 5e-2


def test_graphs_follow_list_reallocation():
    """A neighbour list rebuilt with larger buffers outside a run (here: new capacities and a
    build on request) moves the buffers the captured step graphs address; the next run must
    capture new graphs and give the same trajectory as a run without the extra build."""
    snap = workloads.lj_fluid_sc(12)
    res = []
    for rebuild in (False, True):
        sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.5)
        sim.run(60)
        integ = sim._cpp_integrator
        assert integ.graphCount() >= 1
        if rebuild:
            gen = cell._cpp_obj.alloc_generation
            cell._cpp_obj.setStartCapacity(int(cell._cpp_obj.getNmax()) + 16,
                                           [int(n) + 64 for n in cell._cpp_obj.getNmaxPerType()])
            cell._cpp_obj.buildNow()
            assert cell._cpp_obj.alloc_generation > gen
        sim.run(60)
        assert integ.graphGeneration() == cell._cpp_obj.alloc_generation
        res.append(sim.state.get_snapshot())
    box = np.array(snap.configuration.box[:3])
    ua, ub = [s.particles.position + s.particles.image * box for s in res]
    assert np.abs(ua - ub).max() < 1e-3


@pytest.mark.parametrize("kT", [None, 1.2])
def test_conditional_build_graphs_match_gated_kernels(kT):
    """The captured step graphs put the neighbour-list build in a conditional node that runs
    only on rebuild steps; graphs that launch the gated build kernels every step must give the
    same trajectory bit for bit (deterministic cell list) and the same number of builds, across
    chunks, a sort and a run continued from the first."""
    snap = workloads.lj_fluid_sc(16)
    res = []
    for conditional in (True, False):
        sim = make_sim(snap, seed=9)
        sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.5)
        cell = md.nlist.Cell(buffer=0.3, deterministic=True)
        lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
        lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
        th = None if kT is None else md.methods.thermostats.Bussi(kT=kT)
        sim.operations.integrator = md.Integrator(
            dt=0.005, forces=[lj], methods=[md.methods.ConstantVolume(hoomd.filter.All(), th)])
        sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=150))
        sim.run(0)
        integ = sim._cpp_integrator
        integ.conditional_build = conditional
        l0 = integ.launch_count
        sim.run(230)
        nb = cell.num_builds
        sim.run(70)
        nb += cell.num_builds
        res.append((sim.state.get_snapshot(), nb, integ.launch_count - l0))
    (a, nb_a, la), (b, nb_b, lb) = res
    assert nb_a == nb_b and nb_a >= 5
    assert np.array_equal(a.particles.position, b.particles.position)
    assert np.array_equal(a.particles.velocity, b.particles.velocity)
    assert np.array_equal(a.particles.image, b.particles.image)
    # the gated graphs launch every build kernel on all 300 steps, the conditional ones only on
    # the rebuild steps (plus one kernel a step that sets the condition)
    assert la < lb


def _schedule_run(r_buff, delay, dist_check, steps=40):
    """The 512-particle fluid of the oracle's schedule test, run through the API."""
    from test_oracle import sc_lattice
    pos, (L, _, _) = sc_lattice(8, 1.2, 0.05, seed=3)
    N = len(pos)
    vel = np.zeros((N, 4), np.float32)
    vel[:, 3] = 1.0
    vel = O.thermalize(vel, np.arange(N), 1.5, 0, 9, prec=32)
    snap = hoomd.Snapshot()
    snap.configuration.box = [L, L, L, 0, 0, 0]
    snap.particles.N = N
    snap.particles.types = ["A"]
    snap.particles.position[:] = np.asarray(pos, np.float32)
    snap.particles.velocity[:] = vel[:, :3]
    sim = make_sim(snap)
    cell = md.nlist.Cell(buffer=r_buff, rebuild_check_delay=delay, check_dist=dist_check)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim.operations.integrator = md.Integrator(
        dt=0.005, forces=[lj], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    sim.run(steps)
    return sim, cell


@pytest.mark.parametrize("r_buff,delay,dist_check,builds,dangerous", [
    (0.002, 4, True, 10, 10),   # thin buffer: every check after the delay finds the list stale
    (0.002, 4, False, 10, 0),   # no distance check: a build every 4 steps, never dangerous
    (0.4, 0, False, 40, 0),     # delay 0 without the distance check: every step
    (0.002, 1, True, 40, 0),    # the default schedule with the thin buffer: every step
])
def test_rebuild_check_schedule(r_buff, delay, dist_check, builds, dangerous, capfd):
    """rebuild_check_delay / check_dist (NeighborList::needsUpdating,
    hoomd/md/NeighborList.cc:1313-1418) on the GPU: the same builds and dangerous builds as the
    oracle's schedule on the same system, and the reference's notice for dangerous builds."""
    sim, cell = _schedule_run(r_buff, delay, dist_check)
    assert (cell.num_builds, cell.dangerous_builds) == (builds, dangerous)
    assert sim._cpp_integrator.status()["last_update"] == 40
    err = capfd.readouterr().err
    assert ("dangerous neighbor list build" in err) == (dangerous > 0)
    if delay > 1:
        assert cell.shortest_rebuild == delay


@pytest.mark.parametrize("method", ["langevin", "constant_volume"])
def test_rebuild_check_schedule_on_the_unfused_path(method):
    """Two pair forces summed take the unfused step, which advances the device step counter too
    (the Langevin half itself, a separate kernel after ConstantVolume's), so the rebuild schedule
    and the build statistics follow the steps there as well."""
    from test_oracle import sc_lattice
    pos, (L, _, _) = sc_lattice(8, 1.2, 0.05, seed=3)
    snap = hoomd.Snapshot()
    snap.configuration.box = [L, L, L, 0, 0, 0]
    snap.particles.N = len(pos)
    snap.particles.types = ["A"]
    snap.particles.position[:] = np.asarray(pos, np.float32)
    sim = make_sim(snap)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.5)
    cell = md.nlist.Cell(buffer=0.002, rebuild_check_delay=4, check_dist=False)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    g = md.pair.Gaussian(nlist=cell, default_r_cut=2.0)
    g.params[("A", "A")] = dict(epsilon=0.1, sigma=0.5)
    forces = [lj, g]
    if method == "constant_volume":
        m = md.methods.ConstantVolume(hoomd.filter.All())
    else:
        m = md.methods.Langevin(hoomd.filter.All(), kT=1.5)
    sim.operations.integrator = md.Integrator(dt=0.005, forces=forces, methods=[m])
    sim.run(40)
    assert cell.num_builds == 10 and cell.dangerous_builds == 0
    assert cell.shortest_rebuild == 4
    assert sim._cpp_integrator.status()["last_update"] == 40
    assert sim._cpp_integrator.status()["timestep"] == 40


def test_delayed_check_matches_oracle():
    """A check every third step with the 0.4 buffer: the GPU builds as often as the oracle from
    the same state, never dangerously, and the trajectory follows the oracle's."""
    from test_oracle import _schedule_sim
    sim, cell = _schedule_run(0.4, 3, True, steps=60)
    ref = _schedule_sim(0.4, 3, True, steps=60)
    st = ref.stats()
    assert cell.num_builds == st["checked_builds"] and cell.dangerous_builds == 0
    assert cell.shortest_rebuild >= 3
    snap = sim.state.get_snapshot()
    pos = snap.particles.position + snap.particles.image * snap.configuration.box[:3]
    r = ref.get()
    L = np.array(snap.configuration.box[:3])
    ref_pos = r["pos"][:, :3] + r["image"] * L
    assert np.abs(pos - ref_pos).max() < 1e-3


def test_kernel_parameters_and_tuning():
    """AutotunedObject (hoomd/operation.py:391-497) on the pair force and the list: the values in
    use, setting them (validated), and the search, which times every candidate launch
    configuration on the live state and keeps the fastest. Forces and neighbour sets do not
    depend on the configuration beyond FP32 summation order."""
    snap = workloads.lj_fluid_sc(16)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.5)
    with pytest.raises(hoomd.error.DataAccessError):
        _ = lj.kernel_parameters
    sim.run(0)
    assert lj.kernel_parameters == {"pair": (256, 8)}  # 4096 particles: 8 lanes per particle
    assert cell.kernel_parameters == {"nlist": (128, 32)}
    assert lj.is_tuning_complete and cell.is_tuning_complete
    assert sim.operations.is_tuning_complete
    with pytest.raises(ValueError):
        lj.kernel_parameters = {"pair": (64, 1)}
    with pytest.raises(KeyError):
        cell.kernel_parameters = {"pair": (64,)}
    pairs0 = {tuple(p) for p in np.sort(cell.pair_list(), axis=1)}
    f0 = lj.forces

    sim.operations.tune_kernel_parameters()
    assert not sim.operations.is_tuning_complete
    sim.run(10)
    assert sim.operations.is_tuning_complete
    samples = sim._cpp_integrator.lastTuning()
    pair = {(s[1], s[2]): s[3] for s in samples if s[0] == "pair"}
    nl = {(s[1], s[2]): s[3] for s in samples if s[0] == "nlist"}
    assert len(pair) == 6 and len(nl) == 6 and all(s[3] > 0 for s in samples)

    def kept_rule(times, kept, default):
        # the fastest, unless it is within 2 % of the default, which then stays
        fastest = min(times, key=times.get)
        return kept == fastest or (kept == default and times[fastest] >= 0.98 * times[default])

    assert kept_rule(pair, lj.kernel_parameters["pair"], (256, 8))
    assert kept_rule(nl, cell.kernel_parameters["nlist"], (128, 32))

    sim2, lj2, cell2, _ = lj_sim(snap, kT=None, thermalize=1.5)
    sim2.run(0)
    for pcfg, ncfg in [((128, 1), (32, 1)), ((256, 4), (64, 32)), ((128, 8), (128, 1)),
                       ((256, 1), (32, 32))]:
        lj2.kernel_parameters = {"pair": pcfg}
        cell2.kernel_parameters = {"nlist": ncfg}
        sim2.run(0)
        assert lj2.kernel_parameters == {"pair": pcfg}
        assert {tuple(p) for p in np.sort(cell2.pair_list(), axis=1)} == pairs0
        assert np.allclose(lj2.forces, f0, rtol=1e-5, atol=1e-5 * np.abs(f0).max())


def test_adding_to_operations():
    """hoomd/md/pytest/test_potential.py:1296-1305: a force added to the operations (no
    integrator) is a compute evaluated at the current positions."""
    sim = make_sim(two_particle_snapshot(d=0.5))
    lj = md.pair.LJ(nlist=md.nlist.Cell(0.4))
    lj.r_cut.default = 2.5
    lj.params.default = {"epsilon": 1.0, "sigma": 1.0}
    sim.operations += lj
    sim.run(0)
    assert lj.energy != 0
    e = 4 * (0.5 ** -12 - 0.5 ** -6)
    assert lj.energy == pytest.approx(e, rel=1e-5)
    f = lj.forces
    fmag = 24 * (2 * 0.5 ** -13 - 0.5 ** -7)
    assert f[1, 0] == pytest.approx(fmag, rel=1e-5) and f[0, 0] == pytest.approx(-fmag, rel=1e-5)
    assert lj.virials.shape == (2, 6)
    assert np.array_equal(lj.torques, np.zeros((2, 3)))
    assert lj.additional_energy == 0.0 and lj.additional_virial == [0.0] * 6
    logger = hoomd.logging.Logger(categories=["scalar", "sequence"])
    logger.add(lj, quantities=["energy", "additional_energy", "additional_virial"])
    logged = logger.log()["md"]["pair"]["LJ"]
    assert logged["energy"] == (pytest.approx(e, rel=1e-5), "scalar")
    assert logged["additional_energy"] == (0.0, "scalar")
    assert logged["additional_virial"] == ([0.0] * 6, "sequence")


@pytest.mark.parametrize("name,params", [
    ("LJ", dict(epsilon=1.5, sigma=1.1)),
    ("Gaussian", dict(epsilon=1.0, sigma=0.8)),
    ("Yukawa", dict(epsilon=2.0, kappa=1.5)),
    ("Morse", dict(D0=1.0, alpha=2.0, r0=1.1)),
    ("Mie", dict(epsilon=1.0, sigma=1.0, n=12, m=6))])
def test_shift(name, params):
    """hoomd/md/pytest/test_potential.py:1349-1390: two forces used as computes, one shifted,
    at r just inside r_cut: the shifted energy is much closer to zero."""
    r_cut = 2.0
    pots = []
    for mode in ("none", "shift"):
        p = getattr(md.pair, name)(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=r_cut)
        p.params[("A", "A")] = params
        p.mode = mode
        pots.append(p)
    sim = make_sim(two_particle_snapshot(d=r_cut - 1e-3))
    sim.operations.computes.extend(pots)
    sim.run(0)
    V, V_shifted = pots[0].energy, pots[1].energy
    assert V != 0
    assert V_shifted == pytest.approx(0, abs=max(abs(V) / 1e2, 1e-8))


def test_force_in_integrator_and_computes():
    """A force held by the integrator and listed as a compute is evaluated once, by the
    integrator; a second, compute-only copy with the same parameters agrees with it."""
    snap = workloads.lj_fluid_sc(8)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    sim.operations.computes.append(lj)
    other = md.pair.LJ(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5)
    other.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim.operations.computes.append(other)
    sim.run(20)
    assert not getattr(lj, "_standalone", False) and other._standalone
    assert np.allclose(other.forces, lj.forces, rtol=1e-4, atol=1e-4)
    assert other.energy == pytest.approx(lj.energy, rel=1e-5)


def test_nan_position_raises_with_tag():
    snap = workloads.lj_fluid_sc(8)
    snap.particles.position[17] = [np.nan, 0, 0]
    sim, lj, cell, thermo = lj_sim(snap, thermalize=None)
    with pytest.raises(RuntimeError, match="tag 17 has NaN"):
        sim.run(0)


def test_bussi_requires_momenta():
    snap = workloads.lj_fluid_sc(8)
    sim, lj, cell, thermo = lj_sim(snap, kT=1.0, thermalize=None)
    with pytest.raises(RuntimeError, match="non-zero initial momenta"):
        sim.run(1)


def test_multiple_forces_general_path():
    """Two LJ forces sharing one list run through the unfused path; their sum equals one LJ with
    epsilon doubled."""
    snap = workloads.lj_fluid_sc(10)
    sim1, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0, seed=3)
    lj.params[("A", "A")] = dict(epsilon=2.0, sigma=1.0)
    sim1.run(10)
    sim2 = make_sim(snap, 3)
    sim2.state.thermalize_particle_momenta(hoomd.filter.All(), 1.0)
    cell2 = md.nlist.Cell(buffer=0.4)
    a = md.pair.LJ(nlist=cell2, default_r_cut=2.5)
    b = md.pair.LJ(nlist=cell2, default_r_cut=2.5)
    a.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    b.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim2.operations.integrator = md.Integrator(
        dt=0.005, forces=[a, b], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    sim2.run(10)
    p1 = sim1.state.get_snapshot().particles.position
    p2 = sim2.state.get_snapshot().particles.position
    assert np.abs(p1 - p2).max() < 1e-4


def _brute_energy_sets(pos, L, tags1, tags2, V, r_cut):
    """FP64 sum of V(r) over i in tags1, j in tags2 within r_cut (minimum image, cubic box)."""
    a = pos[np.asarray(tags1)][:, None, :] - pos[np.asarray(tags2)][None, :, :]
    a -= L * np.rint(a / L)
    r = np.sqrt((a ** 2).sum(-1))
    m = r < r_cut
    return V(r[m]).sum()


@pytest.mark.parametrize("kind", ["lj_xplor", "lj_shift", "yukawa"])
def test_compute_energy_between_sets(kind):
    """Pair.compute_energy (hoomd/md/pair/pair.py, PotentialPair::computeEnergyBetweenSets):
    the sum over i in one set and j in the other, against an FP64 brute force."""
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.1, seed=11)
    N = snap.particles.N
    L = snap.configuration.box[0]
    sim = make_sim(snap)
    rc, ron = 2.5, 2.0
    if kind.startswith("lj"):
        f = md.pair.LJ(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=rc,
                       mode="xplor" if kind == "lj_xplor" else "shift")
        f.params[("A", "A")] = dict(epsilon=1.2, sigma=0.9)
        f.r_on[("A", "A")] = ron

        def V0(r):
            return 4 * 1.2 * ((0.9 / r) ** 12 - (0.9 / r) ** 6)
        if kind == "lj_xplor":
            def V(r):
                s = np.where(r < ron, 1.0, (rc ** 2 - r ** 2) ** 2 * (rc ** 2 + 2 * r ** 2 - 3 * ron ** 2)
                             / (rc ** 2 - ron ** 2) ** 3)
                return V0(r) * s
        else:
            def V(r):
                return V0(r) - V0(rc)
    else:
        f = md.pair.Yukawa(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=rc)
        f.params[("A", "A")] = dict(epsilon=2.0, kappa=1.5)

        def V(r):
            return 2.0 * np.exp(-1.5 * r) / r
    sim.operations.computes.append(f)
    sim.run(0)
    tags = np.arange(N)
    t1, t2 = tags[0::2], tags[1::2]
    pos = sim.state.get_snapshot().particles.position.astype(np.float32).astype(np.float64)
    want = _brute_energy_sets(pos, L, t1, t2, V, rc)
    got = f.compute_energy(t1, t2)
    assert got == pytest.approx(want, rel=2e-5)
    # a subset against the rest, and the symmetry of the two sets
    s1, s2 = tags[:137], tags[137:]
    assert f.compute_energy(s1, s2) == pytest.approx(f.compute_energy(s2, s1), rel=1e-5)
    assert f.compute_energy(s1, s2) == pytest.approx(
        _brute_energy_sets(pos, L, s1, s2, V, rc), rel=2e-5)


def _brute_energy_tag_lists(pos, L, tags1, tags2, V, r_cut):
    """The reference's double loop over the two tag lists (hoomd/md/PotentialPair.h:833-990):
    every (tag in tags1, tag in tags2) combination, duplicates and shared tags included, no
    exclusions; V(r) within r_cut, minimum image, FP64."""
    a = pos[np.asarray(tags1)][:, None, :] - pos[np.asarray(tags2)][None, :, :]
    a -= L * np.rint(a / L)
    r = np.sqrt((a ** 2).sum(-1))
    return V(r[r < r_cut]).sum()


def test_compute_energy_counts_excluded_and_repeated_pairs():
    """compute_energy applies no exclusions (bonded pairs count), counts a tag as often as it
    appears, counts both orders of a pair when both tags are in both sets, and adds V(0) for a
    tag paired with itself, as the reference's double loop does."""
    snap = workloads.lj_fluid_sc(8, density=0.84, jitter=0.05, seed=3)
    N = snap.particles.N
    b = [(i, i + 1) for i in range(0, N - 1, 2)]
    snap.bonds.N = len(b)
    snap.bonds.types = ["b"]
    snap.bonds.group[:] = b
    L = snap.configuration.box[0]
    sim = make_sim(snap)
    rc = 2.5
    f = md.pair.Gaussian(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=rc)  # bonds excluded
    f.params[("A", "A")] = dict(epsilon=1.3, sigma=0.8)

    def V(r):
        return 1.3 * np.exp(-0.5 * r * r / 0.64)
    sim.operations.computes.append(f)
    sim.run(0)
    pos = sim.state.get_snapshot().particles.position.astype(np.float32).astype(np.float64)
    tags = np.arange(N)
    # disjoint: every bonded pair (2k, 2k+1) joins the two sets
    t1, t2 = tags[0::2], tags[1::2]
    assert f.compute_energy(t1, t2) == pytest.approx(
        _brute_energy_tag_lists(pos, L, t1, t2, V, rc), rel=2e-5)
    # overlapping sets with repeated tags
    s1 = np.concatenate([tags[:200], [3, 3, 7, 150]])
    s2 = np.concatenate([tags[100:300], [150, 3]])
    want = _brute_energy_tag_lists(pos, L, s1, s2, V, rc)
    assert f.compute_energy(s1, s2) == pytest.approx(want, rel=2e-5)
    assert f.compute_energy(s2, s1) == pytest.approx(want, rel=2e-5)
    assert f.compute_energy(s1, []) == 0.0


def test_shortest_rebuild():
    """nlist.Cell.shortest_rebuild (NeighborList::getSmallestRebuild): the smallest period
    between builds since the last run, at most the mean period; 100 before two builds."""
    snap = workloads.lj_fluid_sc(12, density=0.84)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.5)
    with pytest.raises(RuntimeError):
        _ = cell.shortest_rebuild
    sim.run(1)
    assert cell.shortest_rebuild == 100
    b0 = cell.num_builds
    sim.run(600)
    nb = cell.num_builds - b0
    assert nb >= 10
    shortest = cell.shortest_rebuild
    assert 1 <= shortest <= 600 / nb
    sim.run(0)
    assert cell.shortest_rebuild == 100  # restarted by the run


def test_parameters_changed_between_runs():
    """Pair parameters and r_cut set after the simulation started take effect at the next run
    (the reference's TypeParameters write through to the attached C++ object)."""
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=4)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    sim.run(5)
    e1 = lj.energy
    lj.params[("A", "A")] = dict(epsilon=2.0, sigma=1.0)
    sim.run(0)
    assert lj.energy == pytest.approx(2 * e1, rel=1e-5)
    lj.r_cut[("A", "A")] = 1.5
    sim.run(0)
    pos = sim.state.get_snapshot().particles.position.astype(np.float32).astype(np.float64)
    L = snap.configuration.box[0]
    N = len(pos)
    tags = np.arange(N)
    want = 0.0
    for i in range(N):
        d = pos[i] - pos[i + 1:]
        d -= L * np.rint(d / L)
        r = np.sqrt((d ** 2).sum(1))
        r = r[r < 1.5]
        want += (4 * 2.0 * (r ** -12 - r ** -6)).sum()
    assert lj.energy == pytest.approx(want, rel=1e-5)
    sim.run(10)  # the shorter list and the new parameters in the captured step
    assert np.isfinite(lj.energy)
    del tags


def test_buffer_changed_between_runs():
    """A new nlist.Cell buffer applies from the next run: the list holds the neighbours within
    the new r_cut + buffer, and the step keeps running."""
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=5)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    sim.run(5)
    integ = sim._cpp_integrator
    n0 = integ.sumNNeigh()
    cell.buffer = 0.8
    sim.run(0)
    n1 = sim._cpp_integrator.sumNNeigh()
    rho = snap.particles.N / snap.configuration.box[0] ** 3
    expect = snap.particles.N * rho * 4 / 3 * np.pi * (2.5 + 0.8) ** 3
    assert n1 > n0 and abs(n1 / expect - 1) < 0.05
    e = lj.energy
    sim.run(20)
    assert np.isfinite(lj.energy) and abs(lj.energy - e) < 0.2 * abs(e)


def test_forces_appended_after_a_run():
    """Forces appended to (or removed from) integrator.forces after a run take part in the next
    run, as the reference's synced lists do."""
    snap = workloads.lj_fluid_sc(8, density=0.8, jitter=0.05, seed=6)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    sim.run(5)
    pe1 = thermo.potential_energy
    lj2 = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj2.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim.operations.integrator.forces.append(lj2)
    sim.run(0)
    assert thermo.potential_energy == pytest.approx(2 * pe1, rel=1e-5)
    sim.operations.integrator.forces.remove(lj2)
    # a removed force no longer reports values from the discarded engine
    with pytest.raises(RuntimeError, match="available after"):
        _ = lj2.energy
    sim.run(0)
    assert thermo.potential_energy == pytest.approx(pe1, rel=1e-5)
    sim.run(10)
    assert np.isfinite(thermo.potential_energy)
    with pytest.raises(RuntimeError, match="available after"):
        _ = lj2.forces


def test_particles_on_the_hi_face_keep_their_neighbours():
    """Particles one FP32 ulp inside the hi faces (a wrapped position lands there when a
    particle crosses the lo face by less than half an ulp): their fractional coordinate rounds to
    1; the engine's list must still hold all their partners across the boundary, so the forces
    match the oracle's."""
    # density 0.8: a box whose FP32 fraction of L/2 - 1 ulp rounds to exactly 1
    snap = workloads.lj_fluid_sc(16, density=0.8)
    L = np.float32(snap.configuration.box[0])
    inside = float(np.nextafter(np.float32(L / np.float32(2)), np.float32(0)))
    assert O.make_fraction(np.float32([[inside, 0, 0]]), snap.configuration.box, 32)[0, 0] >= 1
    rng = np.random.default_rng(8)
    P = snap.particles.position
    moved = 0
    for i in rng.permutation(snap.particles.N):
        axes = [(0,), (1,), (2,), (0, 1), (1, 2), (0, 1, 2)][moved % 6]
        trial = P[i].copy()
        trial[list(axes)] = inside
        d = P - trial
        d -= float(L) * np.rint(d / float(L))
        r = np.sqrt((d ** 2).sum(1))
        r[i] = np.inf
        if r.min() > 0.45:  # apart from every other particle (lattice spacing 1.08)
            P[i] = trial
            moved += 1
        if moved == 18:
            break
    sim, lj, cell, thermo = lj_sim(snap, thermalize=None)
    sim.run(0)
    pos = sim.state.get_snapshot().particles.position
    assert (np.abs(pos - inside) == 0).any()
    box = tuple(snap.configuration.box)
    # the FP32 oracle (same FP32 differences of coordinates near L/2) and the magnitude sums of
    # the FP64 terms bound the comparison; a missing partner would be off by a whole pair force
    p32 = O.make_pos4(pos, np.zeros(len(pos)), 32)
    n, l, h, _ = O.build_nlist(p32, box, [[2.5]], 0.4, full=True, prec=32)
    f32, _ = O.pair_forces("lj", p32, box, [[1.0, 1.0]], np.float32([[6.25]]), n, l, h, prec=32)
    # cut-off band at FP32 too: across the boundary the FP32 r^2 can sit a few 1e-6 from FP64's
    fb32, _ = O.pair_forces("lj", p32, box, [[1.0, 1.0]], np.float32([[6.25]]), n, l, h,
                            prec=32, abs_terms=2)
    p64 = O.make_pos4(pos, np.zeros(len(pos)), 64)
    n, l, h, _ = O.build_nlist(p64, box, [[2.5]], 0.4, full=True, prec=64)
    fa, _ = O.pair_forces("lj", p64, box, [[1.0, 1.0]], [[6.25]], n, l, h, prec=64, abs_terms=1)
    fb, _ = O.pair_forces("lj", p64, box, [[1.0, 1.0]], [[6.25]], n, l, h, prec=64, abs_terms=2)
    assert_close_cond(lj.forces, f32[:, :3], fa[:, :3], band=fb[:, :3] + fb32[:, :3],
                      what="hi-face forces")


def test_params_changed_between_runs_recompute_forces():
    """Parameters set after a run are sent before the next one, and that run's preparation
    recomputes the forces at the current positions with them (IntegratorTwoStep::prepRun,
    hoomd/md/IntegratorTwoStep.cc:262-275: the net force is always recomputed; the
    accelerations of the last step are kept, as there)."""
    snap = workloads.lj_fluid_sc(8, density=0.8, jitter=0.05, seed=6)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    sim.run(5)
    lj.params[("A", "A")] = dict(epsilon=2.0, sigma=1.0)
    sim.run(0)
    f_now = lj.forces
    # a fresh simulation from the same state with epsilon = 2 from the start
    snap2 = sim.state.get_snapshot()
    sim2, lj_b, cell2, thermo2 = lj_sim(snap2, kT=None, thermalize=None)
    lj_b.params[("A", "A")] = dict(epsilon=2.0, sigma=1.0)
    sim2.run(0)
    assert np.allclose(f_now, lj_b.forces, rtol=1e-5, atol=1e-5 * np.abs(f_now).max())
    assert thermo.potential_energy == pytest.approx(thermo2.potential_energy, rel=1e-6)

def test_snapshot_round_trip_on_the_device():
    """get_snapshot / set_snapshot convert on the device (takeSnapshot / initializeFromSnapshot's
    per-particle loops): values come back as their FP32 roundings in tag order, positions out of
    the box are wrapped with their images counted, a snapshot written into a sorted system keeps
    its order and gives the oracle's forces, and a type id out of range is refused."""
    snap = workloads.lj_fluid_sc(12, density=0.84, jitter=0.05, seed=21)
    N = snap.particles.N
    L = snap.configuration.box[0]
    sim, lj, cell, thermo = lj_sim(snap, kT=1.5, sorter=10)
    sim.run(25)  # sorted twice: index order is no longer tag order
    s = sim.state.get_snapshot()
    rng = np.random.default_rng(3)
    pos = s.particles.position + rng.uniform(-0.02, 0.02, (N, 3))
    pos[0] += [L, 0, 0]          # one box length beyond +x
    pos[1] += [0, -1.2 * L, 0]   # beyond -y by more than the box
    vel = rng.normal(size=(N, 3))
    mass = rng.uniform(0.5, 2.0, N)
    s.particles.position[:] = pos
    s.particles.velocity[:] = vel
    s.particles.mass[:] = mass
    img0 = s.particles.image.copy()
    sim.state.set_snapshot(s)
    out = sim.state.get_snapshot()
    f32 = np.float32
    want = pos.astype(f32).astype(np.float64)
    shift = np.zeros((N, 3))
    shift[0, 0] = -L
    k = 2 if pos[1, 1] + L < -L / 2 else 1  # box lengths added to bring it in
    shift[1, 1] = k * L
    assert np.allclose(out.particles.position, want + shift, atol=2e-5)
    assert np.array_equal(out.particles.image[0], img0[0] + [1, 0, 0])
    assert np.array_equal(out.particles.image[1], img0[1] + [0, -k, 0])
    assert np.array_equal(out.particles.image[2:], img0[2:])
    assert np.array_equal(out.particles.velocity, vel.astype(f32).astype(np.float64))
    assert np.array_equal(out.particles.mass, mass.astype(f32).astype(np.float64))
    assert np.array_equal(out.particles.typeid, s.particles.typeid)
    sim.run(0)
    p = out.particles.position
    pos4 = O.make_pos4(p, np.zeros(N), 64)
    box = tuple(snap.configuration.box)
    n, l, h, _ = O.build_nlist(pos4, box, [[2.5]], 0.4, full=False, prec=64)
    fo, _ = O.pair_forces("lj", pos4, box, [[1.0, 1.0]], [[6.25]], n, l, h, third_law=True,
                          compute_virial=False, prec=64)
    assert np.allclose(lj.forces, fo[:, :3], rtol=1e-5, atol=1e-5 * np.abs(fo[:, :3]).max())
    bad = sim.state.get_snapshot()
    bad.particles.typeid[7] = 3
    with pytest.raises(Exception):
        sim.state._upload(bad)


def test_time_step_change_after_a_run_applies():
    """A new Integrator.dt set between runs reaches the captured fused steps (they hold the time
    step): the second run equals a fresh simulation started from the same state at the new dt."""
    snap = workloads.lj_fluid_sc(8, density=0.8, jitter=0.05, seed=13)
    sim, lj, cell, thermo = lj_sim(snap, kT=None, thermalize=1.0)
    sim.run(10)
    mid = sim.state.get_snapshot()
    sim.operations.integrator.dt = 0.0025
    sim.run(10)
    a = sim.state.get_snapshot()
    sim2, lj2, cell2, thermo2 = lj_sim(mid, kT=None, dt=0.0025, thermalize=None)
    sim2.run(10)
    b = sim2.state.get_snapshot()
    assert np.allclose(a.particles.position, b.particles.position, atol=1e-4)
    assert np.allclose(a.particles.velocity, b.particles.velocity, atol=1e-3)
    # and a state written back between runs keeps the same captured steps valid
    sim.state.set_snapshot(mid)
    sim.run(10)
    c = sim.state.get_snapshot()
    assert np.allclose(c.particles.position, b.particles.position, atol=1e-4)
