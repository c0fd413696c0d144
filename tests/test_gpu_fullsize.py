"""Parity at the benchmark configurations' own sizes.

Each system is built from the same seeds as the benchmark:

* the 1,048,576-particle LJ fluid (64^3 FCC, density 0.84, r_cut 2.5, buffer 0.4);
* the 262,144-particle Kob-Andersen mixture (80:20, density 1.2, r_cut 2.5 sigma_ij, buffer 0.3);
* the 524,288-particle 32-type system with 528 tabulated potentials (density 0.8, r_cut 3.0,
  buffer 0.4).

For each, the GPU neighbour list (cell list + the candidate-stream build through the C ABI, the
layout and build the engine runs) must equal the FP32 oracle's full list as per-particle sorted sets, bit
for bit. One evaluation of the pair forces, per-particle energies and virials over that list is
then held to two bars:

* against the FP32 oracle (the reference's arithmetic at HOOMD_LONGREAL_SIZE=32 on the same
  FP32 positions): within 1e-5 of the sum of the magnitudes of the terms of each value (the
  only differences left are the evaluator's reciprocal and the summation order), plus the terms
  of pairs within 1e-6 relative of r_cut^2 at FP64 or at FP32 (LJ does not vanish at r_cut in
  mode "none", and whether such a pair counts turns on the last bit of r^2);
* against the FP64 oracle: no worse than the FP32 oracle itself (largest error at most 1.5x
  the FP32 oracle's; values outside 1e-5 relative at most twice as many as the FP32 oracle's,
  plus 1e-4 of the values).

A bar of 1e-5 relative to the FP64 value alone cannot be met by any FP32 evaluation of these
dense systems: the difference x_i - x_j of FP32 coordinates up to L/2 ~ 54 is off by up to
~4e-6, and the r^-13 LJ force of a close pair magnifies that thirteen-fold, so the FP32 oracle
itself misses it on about 0.2 % of the Kob-Andersen force components.

This follows the reference's CPU-vs-GPU list comparison
(hoomd/md/test/test_neighborlist.cc:1060-1148) and its force/energy accuracy test
(hoomd/md/pytest/test_potential.py:952-1058), at full size. The oracle runs on every host core
(OpenMP); the comparisons are vectorised over particle chunks.

The 1M-particle fluid, the Kob-Andersen mixture and the 32-type Table system are also checked
after 200 steps of the product's own run (Bussi, Hilbert sort every 100 steps, the benchmark's settings): the engine's
forces, energies and virials through the Python API against the oracles at the resulting
positions, with the same bars.
"""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import synthetic_systems as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from gpu_util import (RTOL, GpuNlist, assert_close_cond, compare_neighbor_sets,  # noqa: E402
                      gpu_pair_forces, table_params)

CORES = os.cpu_count() or 1


def _pos4(system):
    p = system.particles
    return O.make_pos4(p.position, p.typeid, 32), tuple(system.configuration.box)


def _lj_case(system, pairs):
    """pairs: {(i, j): (epsilon, sigma, r_cut)} -> (r_cut matrix, oracle/ABI params)."""
    nt = len(system.particles.types)
    rc = np.zeros((nt, nt))
    par = np.zeros((nt * nt, 2))
    for (i, j), (eps, sig, r) in pairs.items():
        for a, b in ((i, j), (j, i)):
            rc[a, b] = r
            par[a * nt + b] = (sig, eps)
    return rc, par


def _systems():
    fcc = S.lj_fluid_fcc(m=64, density=0.84, jitter=0.05, seed=1)
    ka = S.binary_mixture(N=262144, density=1.2, seed=1)
    t32 = S.multitype_system(N=524288, ntypes=32, density=0.8, seed=1)
    return {
        "lj_fcc_1m": (fcc, "lj", _lj_case(fcc, {(0, 0): (1.0, 1.0, 2.5)}), 0.4),
        "ka_262k": (ka, "lj", _lj_case(ka, {(0, 0): (1.0, 1.0, 2.5), (0, 1): (1.5, 0.8, 2.0),
                                            (1, 1): (0.5, 0.88, 2.2)}), 0.3),
        "table32_524k": (t32, "table", None, 0.4),
    }


@pytest.fixture(scope="module")
def systems():
    return _systems()


@pytest.mark.parametrize("case", ["lj_fcc_1m", "ka_262k", "table32_524k"])
def test_fullsize_nlist_and_forces_vs_oracle(systems, case):
    system, kind, lj, r_buff = systems[case]
    pos4, box6 = _pos4(system)
    N = len(pos4)
    nt = len(system.particles.types)
    if kind == "lj":
        rc, par = lj
        tables = opar = odata = None
    else:
        tabs = S.mixture_tables(32, r_min=0.8, r_cut=3.0, width=1000, seed=2)
        recs, data, opar, odata = table_params(
            nt, {k: (v["r_min"], v["U"], v["F"]) for k, v in tabs.items()})
        tables = (recs, data)
        rc = np.full((nt, nt), 3.0)
        par = None

    # neighbour sets: GPU (interleaved column-major list, candidate-stream build) vs FP32 oracle
    nl = GpuNlist(pos4, box6, rc, r_buff, layout="col4")
    n_o, l_o, h_o, info = O.build_nlist(pos4, box6, rc, r_buff, full=True, prec=32,
                                        nthreads=CORES)
    assert nl.dim == info["dim"].tolist()
    nn_g = nl.n_neigh.cpu().numpy().view(np.uint32)
    nl_g = nl.nlist.cpu().numpy().view(np.uint32)
    ho = h_o.astype(np.int64)
    bad = compare_neighbor_sets(nn_g, nl_g, nl.word_index(), n_o, l_o, lambda i, k: ho[i] + k)
    assert len(bad) == 0, f"{case}: {len(bad)} of {N} particles' sets differ, first {bad[:5]}"
    sum_n = int(n_o.astype(np.int64).sum())
    assert sum_n > 50 * N  # a dense liquid: tens of neighbours each

    # one force evaluation over the GPU list vs the FP32 and FP64 oracles
    f, v = gpu_pair_forces(nl, kind, par, rc, virial=True, tables=tables)
    oparams = opar if kind == "table" else par
    f32, v32 = O.pair_forces(kind, pos4, box6, oparams, (rc ** 2).astype(np.float32), n_o, l_o,
                             h_o, third_law=False, compute_virial=True,
                             tdata=None if odata is None else odata.astype(np.float32), prec=32,
                             nthreads=CORES)
    del l_o, h_o, ho
    pos64 = pos4.astype(np.float64)
    pos64[:, 3] = O.types_as_w(O.pos_index_bits(pos4[:, 3], 32), 64)
    check_against_oracles(kind, pos64, box6, oparams, rc, r_buff, odata,
                          (f[:, :3], f[:, 3], v), (f32[:, :3], f32[:, 3], v32), case)


def check_against_oracles(kind, pos64, box6, oparams, rc, r_buff, odata, got, f32, case, ndim=3):
    """got / f32: (forces (N, 3), energies (N,), virials (6, N)) of the GPU and of the FP32
    oracle; the FP64 oracle's values, the sums of term magnitudes and the cut-off band terms are
    computed here. The band is taken both at FP64 and at FP32: for a pair across a periodic
    boundary the FP32 difference x_i - x_j of coordinates near +-L/2 carries a rounding of up to
    ~L 2^-24, so its FP32 r^2 can sit several 1e-6 (relative) from the FP64 one, and the pairs
    that the two FP32 evaluations may count differently are those whose FP32 r^2 is near r_cut^2."""
    n6, l6, h6, _ = O.build_nlist(pos64, box6, rc, r_buff, full=True, ndim=ndim, prec=64,
                                  nthreads=CORES)
    kw = dict(third_law=False, compute_virial=True, tdata=odata, prec=64, nthreads=CORES)
    fo, vo = O.pair_forces(kind, pos64, box6, oparams, rc ** 2, n6, l6, h6, **kw)
    fa, va = O.pair_forces(kind, pos64, box6, oparams, rc ** 2, n6, l6, h6, abs_terms=1, **kw)
    fb, vb = O.pair_forces(kind, pos64, box6, oparams, rc ** 2, n6, l6, h6, abs_terms=2, **kw)
    del n6, l6, h6
    pos32 = O.make_pos4(pos64[:, :3], O.pos_index_bits(pos64[:, 3], 64), 32)
    n3, l3, h3, _ = O.build_nlist(pos32, box6, rc, r_buff, full=True, ndim=ndim, prec=32,
                                  nthreads=CORES)
    kw32 = dict(kw, prec=32)
    fb32, vb32 = O.pair_forces(kind, pos32, box6, oparams, np.float32(rc ** 2), n3, l3, h3,
                               abs_terms=2, **kw32)
    del n3, l3, h3
    fb = fb + fb32.astype(np.float64)
    vb = vb + vb32.astype(np.float64)
    ref = (fo[:, :3], fo[:, 3], vo)
    absref = (fa[:, :3], fa[:, 3], va)
    bands = (fb[:, :3], fb[:, 3], vb)
    for name, g, r32, r64, a, b in zip(("force", "energy", "virial"), got, f32, ref, absref,
                                       bands):
        g = np.asarray(g, np.float64)
        r32 = np.asarray(r32, np.float64)
        assert_close_cond(g, r32, a, band=b, what=f"{case} {name} vs FP32 oracle")
        e_gpu = np.abs(g - r64)
        e_32 = np.abs(r32 - r64)
        over = e_gpu - (1.5 * e_32.max() + b + 1e-7 * np.abs(r64).max())
        assert (over <= 0).all(), (
            f"{case} {name}: GPU error vs FP64 {e_gpu.max():.3e} beyond 1.5 x the FP32 oracle's "
            f"{e_32.max():.3e} plus the cut-off band")
        plain = RTOL * np.abs(r64) + RTOL * np.abs(r64).max()
        out_gpu, out_32 = int((e_gpu > plain + b).sum()), int((e_32 > plain + b).sum())
        assert out_gpu <= 2 * out_32 + 1e-4 * e_gpu.size, (
            f"{case} {name}: {out_gpu} values outside 1e-5 relative of FP64 on the GPU against "
            f"{out_32} for the FP32 oracle")


def test_fullsize_fcc_after_run_vs_oracle():
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md
    from hoomd_gb300.workloads import to_snapshot

    system = S.lj_fluid_fcc(m=64, density=0.84, jitter=0.05, seed=1)
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(to_snapshot(system))
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.5)
    cell = md.nlist.Cell(buffer=0.4)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim.operations.integrator = md.Integrator(dt=0.005, forces=[lj], methods=[
        md.methods.ConstantVolume(hoomd.filter.All(), md.methods.thermostats.Bussi(kT=1.5))])
    sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=100))
    sim.run(200)
    F, E, W = lj.forces, lj.energies, lj.virials
    snap = sim.state.get_snapshot()
    box6 = tuple(snap.configuration.box)
    pos4 = O.make_pos4(snap.particles.position, snap.particles.typeid, 32)
    rc = np.array([[2.5]])
    n, l, h, _ = O.build_nlist(pos4, box6, rc, 0.4, full=True, prec=32, nthreads=CORES)
    f32, v32 = O.pair_forces("lj", pos4, box6, [[1.0, 1.0]], np.float32([[6.25]]), n, l, h,
                             third_law=False, compute_virial=True, prec=32, nthreads=CORES)
    del l, h
    assert cell.num_builds >= 2
    pos64 = pos4.astype(np.float64)
    pos64[:, 3] = O.types_as_w(O.pos_index_bits(pos4[:, 3], 32), 64)
    check_against_oracles("lj", pos64, box6, [[1.0, 1.0]], rc, 0.4, None,
                          (F, E, W.T), (f32[:, :3], f32[:, 3], v32), "fcc after 200 steps")


def test_fullsize_ka_after_run_vs_oracle():
    """The 262,144-particle Kob-Andersen mixture after 200 steps of the product's own run (Bussi
    at kT 0.8, dt 0.003, Hilbert sort every 100 steps, the benchmark's settings): the engine's
    forces, energies and virials through the Python API against the oracles at the resulting
    positions, with the per-type-pair cut-offs and parameters of the mixture."""
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md
    from hoomd_gb300.workloads import to_snapshot

    system = S.binary_mixture(N=262144, density=1.2, seed=1)
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(to_snapshot(system))
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 0.8)
    cell = md.nlist.Cell(buffer=0.3)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    pairs = {("A", "A"): (1.0, 1.0, 2.5), ("A", "B"): (1.5, 0.8, 2.0),
             ("B", "B"): (0.5, 0.88, 2.2)}
    for key, (eps, sig, r) in pairs.items():
        lj.params[key] = dict(epsilon=eps, sigma=sig)
        lj.r_cut[key] = r
    sim.operations.integrator = md.Integrator(dt=0.003, forces=[lj], methods=[
        md.methods.ConstantVolume(hoomd.filter.All(), md.methods.thermostats.Bussi(kT=0.8))])
    sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=100))
    sim.run(200)
    F, E, W = lj.forces, lj.energies, lj.virials
    snap = sim.state.get_snapshot()
    box6 = tuple(snap.configuration.box)
    pos4 = O.make_pos4(snap.particles.position, snap.particles.typeid, 32)
    rc, par = _lj_case(system, {(0, 0): (1.0, 1.0, 2.5), (0, 1): (1.5, 0.8, 2.0),
                                (1, 1): (0.5, 0.88, 2.2)})
    n, l, h, _ = O.build_nlist(pos4, box6, rc, 0.3, full=True, prec=32, nthreads=CORES)
    f32, v32 = O.pair_forces("lj", pos4, box6, par, (rc ** 2).astype(np.float32), n, l, h,
                             third_law=False, compute_virial=True, prec=32, nthreads=CORES)
    del l, h
    assert cell.num_builds >= 2
    pos64 = pos4.astype(np.float64)
    pos64[:, 3] = O.types_as_w(O.pos_index_bits(pos4[:, 3], 32), 64)
    check_against_oracles("lj", pos64, box6, par, rc, 0.3, None,
                          (F, E, W.T), (f32[:, :3], f32[:, 3], v32), "ka after 200 steps")


def test_fullsize_table32_after_run_vs_oracle():
    """The 524,288-particle 32-type system after 200 steps of the product's own run with its 528
    tabulated potentials (Bussi at kT 1.5, dt 0.004, Hilbert sort every 100 steps, the
    benchmark's settings): forces, energies and virials against the oracles at the resulting
    positions."""
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md
    from hoomd_gb300.workloads import to_snapshot

    system = S.multitype_system(N=524288, ntypes=32, density=0.8, seed=1)
    tabs = S.mixture_tables(32, r_min=0.8, r_cut=3.0, width=1000, seed=2)
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(to_snapshot(system))
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.5)
    cell = md.nlist.Cell(buffer=0.4)
    tab = md.pair.Table(nlist=cell, default_r_cut=3.0)
    types = system.particles.types
    for (i, j), v in tabs.items():
        tab.params[(types[i], types[j])] = dict(r_min=v["r_min"], U=v["U"], F=v["F"])
    sim.operations.integrator = md.Integrator(dt=0.004, forces=[tab], methods=[
        md.methods.ConstantVolume(hoomd.filter.All(), md.methods.thermostats.Bussi(kT=1.5))])
    sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=100))
    sim.run(200)
    F, E, W = tab.forces, tab.energies, tab.virials
    snap = sim.state.get_snapshot()
    box6 = tuple(snap.configuration.box)
    pos4 = O.make_pos4(snap.particles.position, snap.particles.typeid, 32)
    nt = len(types)
    _, _, opar, odata = table_params(nt, {k: (v["r_min"], v["U"], v["F"])
                                          for k, v in tabs.items()})
    rc = np.full((nt, nt), 3.0)
    n, l, h, _ = O.build_nlist(pos4, box6, rc, 0.4, full=True, prec=32, nthreads=CORES)
    f32, v32 = O.pair_forces("table", pos4, box6, opar, (rc ** 2).astype(np.float32), n, l, h,
                             third_law=False, compute_virial=True,
                             tdata=odata.astype(np.float32), prec=32, nthreads=CORES)
    del l, h
    assert cell.num_builds >= 2
    pos64 = pos4.astype(np.float64)
    pos64[:, 3] = O.types_as_w(O.pos_index_bits(pos4[:, 3], 32), 64)
    check_against_oracles("table", pos64, box6, opar, rc, 0.4, odata,
                          (F, E, W.T), (f32[:, :3], f32[:, 3], v32), "table32 after 200 steps")


def _plane_system(N, L, seed):
    """N particles on a jittered square lattice in the plane z = 0 (a 2D box, Lz = 1)."""
    rng = np.random.default_rng(seed)
    n = int(round(np.sqrt(N)))
    g = (np.arange(n) + 0.5) / n - 0.5
    f = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    f = f + rng.uniform(-0.1 / n, 0.1 / n, f.shape)
    pos = np.zeros((len(f), 3))
    pos[:, :2] = f * L
    return O.make_pos4(pos, np.zeros(len(f)), 32), (L, L, 1.0, 0.0, 0.0, 0.0)


@pytest.mark.parametrize("case", ["triclinic_110k", "plane_250k"])
def test_medium_tilted_and_planar_systems_vs_oracle(case):
    """The boxes the benchmark configurations leave out, at a size where every cell of the grid
    is exercised many times: a two-type system of 110,592 particles in a triclinic box (tilts
    0.2, -0.15, 0.1; the builds' tilted image arithmetic) and a 2D system of 250,000 particles
    (the 2D cell grid and stencil). Neighbour sets bit-exact against the FP32 oracle, forces,
    energies and virials held to the FP32 and FP64 oracles as for the benchmark systems."""
    if case == "triclinic_110k":
        rng = np.random.default_rng(4)
        n = 48
        g = (np.arange(n) + 0.5) / n - 0.5
        f = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        f = f + rng.uniform(-0.1 / n, 0.1 / n, f.shape)
        L, (xy, xz, yz) = 52.0, (0.2, -0.15, 0.1)
        x = f[:, 0] * L + xy * f[:, 1] * L + xz * f[:, 2] * L
        y = f[:, 1] * L + yz * f[:, 2] * L
        z = f[:, 2] * L
        types = rng.integers(0, 2, len(f))
        pos4 = O.make_pos4(np.stack([x, y, z], 1), types, 32)
        box6 = (L, L, L, xy, xz, yz)
        rc, par = np.array([[2.5, 2.0], [2.0, 2.2]]), np.array([[1.0, 1.0], [0.8, 1.5],
                                                                 [0.8, 1.5], [0.88, 0.5]])
        ndim, r_buff = 3, 0.4
    else:
        pos4, box6 = _plane_system(250000, 560.0, seed=6)
        rc, par = np.array([[2.5]]), np.array([[1.0, 1.0]])
        ndim, r_buff = 2, 0.4
    nl = GpuNlist(pos4, box6, rc, r_buff, layout="col4", ndim=ndim)
    n_o, l_o, h_o, info = O.build_nlist(pos4, box6, rc, r_buff, full=True, ndim=ndim, prec=32,
                                        nthreads=CORES)
    assert nl.dim == info["dim"].tolist()
    nn_g = nl.n_neigh.cpu().numpy().view(np.uint32)
    nl_g = nl.nlist.cpu().numpy().view(np.uint32)
    ho = h_o.astype(np.int64)
    bad = compare_neighbor_sets(nn_g, nl_g, nl.word_index(), n_o, l_o, lambda i, k: ho[i] + k)
    assert len(bad) == 0, f"{case}: {len(bad)} particles' sets differ, first {bad[:5]}"
    assert int(n_o.astype(np.int64).sum()) > 10 * len(pos4)
    f, v = gpu_pair_forces(nl, "lj", par, rc, virial=True)
    f32, v32 = O.pair_forces("lj", pos4, box6, par, (rc ** 2).astype(np.float32), n_o, l_o, h_o,
                             third_law=False, compute_virial=True, prec=32, nthreads=CORES)
    pos64 = pos4.astype(np.float64)
    pos64[:, 3] = O.types_as_w(O.pos_index_bits(pos4[:, 3], 32), 64)
    check_against_oracles("lj", pos64, box6, par, rc, r_buff, None, (f[:, :3], f[:, 3], v),
                          (f32[:, :3], f32[:, 3], v32), case, ndim=ndim)
