"""GPU parity of every kernel, called through the C ABI (hoomd_gb300.abi) with torch-allocated
device buffers, against the CPU oracle on identical inputs.

Bars: neighbour lists bit-exact as per-particle sorted sets (FP32 oracle, same FP32 positions);
integrator half steps bit-exact (FP32 oracle); forces, energies and virials within 1e-5 relative
of the FP64 oracle with an absolute floor of 1e-5 x max|F| (the tolerance is written in
``assert_close_f64``); FP64 reductions to 1e-12.
"""

import ctypes
import json
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from hoomd_gb300 import abi, workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402
from gpu_util import (GpuNlist, dev, gpu_pair_forces, host, lj_params_dev, p, stream,  # noqa: E402
                      table_params, zeros)

GOLD = pathlib.Path(__file__).resolve().parent / "golden"
from gpu_util import RTOL, assert_close_f64  # noqa: E402,F401


def random_system(N, L, ntypes=1, seed=0, tilts=(0, 0, 0), lattice=False):
    """N particles at uniform random fractional coordinates, or (lattice=True) on a jittered
    n^3 simple-cubic grid of fractional coordinates (no overlapping pairs), mapped into the
    (possibly triclinic) box."""
    rng = np.random.default_rng(seed)
    if lattice:
        n = int(round(N ** (1 / 3)))
        g = (np.arange(n) + 0.5) / n - 0.5
        f = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        f = f + rng.uniform(-0.1 / n, 0.1 / n, f.shape)
        N = len(f)
    else:
        f = rng.uniform(-0.5, 0.5, (N, 3))
    Lx, Ly, Lz = L
    xy, xz, yz = tilts
    # fractional -> Cartesian (BoxDim::makeCoordinates)
    x = f[:, 0] * Lx + xy * f[:, 1] * Ly + xz * f[:, 2] * Lz
    y = f[:, 1] * Ly + yz * f[:, 2] * Lz
    z = f[:, 2] * Lz
    types = rng.integers(0, ntypes, N)
    return O.make_pos4(np.stack([x, y, z], 1), types, 32), (Lx, Ly, Lz, xy, xz, yz)


def dense_system():
    """Cells holding more than 32 particles (the tiled builds take own particles in passes of 32):
    2600 uniform particles in a 14^3 box (4^3 cells of 3.5, ≈ 41 a cell) and a cluster of 120 in
    one cell at a corner of the box, two types."""
    rng = np.random.default_rng(11)
    L = 14.0
    uni = rng.uniform(-L / 2, L / 2, (2600, 3))
    clu = rng.uniform(-L / 2, -L / 2 + 3.0, (120, 3))
    pos = np.concatenate([uni, clu])
    types = rng.integers(0, 2, len(pos))
    return O.make_pos4(pos, types, 32), (L, L, L, 0.0, 0.0, 0.0)


def snap_pos4(snap):
    return O.make_pos4(snap.particles.position, snap.particles.typeid, 32), \
        tuple(snap.configuration.box)


def hi_face_system():
    """The 4096-particle fluid with particles placed on the hi faces of the box at FP32: exactly
    at L/2 and one ulp inside, on each axis and on edges and a corner. Their fractional
    coordinate rounds to 1, where the reference's cell list wraps the bin index to 0; their
    neighbours lie across the periodic boundary (a wrapped FP32 position lands there when a
    particle crosses the lo face by less than half an ulp)."""
    pos4, box6 = snap_pos4(workloads.lj_fluid_sc(16))
    L = np.float32(box6[0])
    hi = np.float32(L / np.float32(2))
    inside = np.nextafter(hi, np.float32(0))
    rng = np.random.default_rng(5)
    moved = 0
    for i in rng.permutation(len(pos4)):
        v = hi if moved % 2 == 0 else inside
        axes = [(0,), (1,), (2,), (0, 1), (1, 2), (0, 1, 2)][moved % 6]
        trial = pos4[i, :3].astype(np.float64)
        trial[list(axes)] = v
        d = pos4[:, :3].astype(np.float64) - trial
        d -= float(L) * np.rint(d / float(L))
        r = np.sqrt((d ** 2).sum(1))
        r[i] = np.inf
        if r.min() > 0.45:  # apart from every other particle (lattice spacing 1.06)
            pos4[i, list(axes)] = v
            moved += 1
        if moved == 24:
            break
    return pos4, box6


NLIST_CASES = {
    "sc7_rcut1.1": lambda: (O.make_pos4(workloads.sc_positions(7, 1.0), np.zeros(343), 32),
                            (7.0, 7.0, 7.0, 0, 0, 0), [[1.1]], 0.0),
    "random700_dims332": lambda: random_system(700, (9.3, 10.1, 8.0)) + ([[2.5]], 0.4),
    "lj4096": lambda: snap_pos4(workloads.lj_fluid_sc(16)) + ([[2.5]], 0.4),
    "binary3000": lambda: (lambda s: snap_pos4(s) + (
        [[2.5, 2.0], [2.0, 2.2]], 0.3))(workloads.binary_mixture(N=3375, density=1.2)),
    "triclinic1728": lambda: random_system(1728, (11.0, 12.0, 13.0), 2, seed=4,
                                           tilts=(0.3, -0.2, 0.1), lattice=True)
    + ([[2.5, 1.5], [1.5, 2.0]], 0.4),
    "random60k": lambda: random_system(60000, (41.0, 41.0, 41.0), seed=7) + ([[2.5]], 0.4),
    "hi_face4096": lambda: hi_face_system() + ([[2.5]], 0.4),
    "dense2720": lambda: dense_system() + ([[2.5, 2.0], [2.0, 2.2]], 0.4),
}


@pytest.mark.parametrize("case", sorted(NLIST_CASES))
@pytest.mark.parametrize("layout", ["col", "col4", "col_lane", "col4_lane", "colw", "col4w",
                                    "flat"])
def test_nlist_bitexact_vs_oracle(case, layout):
    pos4, box6, rc, rb = NLIST_CASES[case]()
    nl = GpuNlist(pos4, box6, rc, rb, layout=layout)
    n_o, l_o, h_o, info = O.build_nlist(pos4, box6, rc, rb, full=True, prec=32)
    assert nl.dim == info["dim"].tolist()
    got = nl.sets()
    want = O.neighbor_sets(n_o, l_o, h_o)
    bad = [i for i in range(len(pos4)) if not np.array_equal(got[i], want[i])]
    assert not bad, f"{len(bad)} particles differ, first {bad[:5]}"


def test_true_pair_list_golden_gpu():
    truth = set(frozenset(x) for x in json.load(open(GOLD / "true_pair_list_sc7.json")))
    pos4, box6, rc, rb = NLIST_CASES["sc7_rcut1.1"]()
    nl = GpuNlist(pos4, box6, rc, rb)
    got = set()
    for i, s in enumerate(nl.sets()):
        for j in s:
            got.add(frozenset((i, int(j))))
    assert got == truth


def test_nlist_deterministic_mode_is_reproducible():
    pos4, box6, rc, rb = NLIST_CASES["lj4096"]()
    a = GpuNlist(pos4, box6, rc, rb, deterministic=True)
    b = GpuNlist(pos4, box6, rc, rb, deterministic=True)
    assert np.array_equal(host(a.nlist), host(b.nlist))
    assert np.array_equal(host(a.n_neigh), host(b.n_neigh))
    # each cell's slots are in particle-index order
    xyzf = host(a.xyzf).reshape(-1, a.Nmax_cell, 4)
    cs = host(a.cell_size)
    idx = xyzf[..., 3].copy().view(np.uint32)
    for c in range(len(cs)):
        assert np.all(np.diff(idx[c, : cs[c]].astype(np.int64)) > 0)


def oracle_forces_f64(pos4, box6, kind, params, rc, shift=0, r_on=None, tdata=None):
    pos64 = pos4.astype(np.float64)
    pos64[:, 3] = O.types_as_w(O.pos_index_bits(pos4[:, 3], 32), 64)
    rc = np.atleast_2d(rc)
    n, l, h, _ = O.build_nlist(pos64, box6, rc, 0.4, full=True, prec=64)
    ro = None if r_on is None else np.atleast_2d(r_on) ** 2
    return O.pair_forces(kind, pos64, box6, params, rc ** 2, n, l, h, third_law=False,
                         compute_virial=True, shift_mode=shift, ronsq=ro, tdata=tdata, prec=64)


@pytest.mark.parametrize("layout,tpp", [("col", 0), ("col4", 0), ("flat", 1), ("flat", 4),
                                        ("flat", 8), ("flat", 32)])
def test_lj_forces_vs_fp64_oracle(layout, tpp):
    pos4, box6, rc, rb = NLIST_CASES["lj4096"]()
    nl = GpuNlist(pos4, box6, rc, rb, layout=layout)
    par = np.array([[1.0, 1.0]])
    f, v = gpu_pair_forces(nl, "lj", par, rc, tpp=tpp)
    fo, vo = oracle_forces_f64(pos4, box6, "lj", par, rc)
    assert_close_f64(f[:, :3], fo[:, :3], what="force")
    assert_close_f64(f[:, 3], fo[:, 3], what="energy")
    assert_close_f64(v, vo, what="virial")


@pytest.mark.parametrize("tpp", [1, 4, 8])
@pytest.mark.parametrize("case", ["lj4096", "binary3000"])
def test_interleaved_threads_per_particle_vs_fp64_oracle(tpp, case):
    """Groups of 1, 4 or 8 lanes per particle on the interleaved list (no virial, so the split
    kernel runs), single and two types."""
    pos4, box6, rc, rb = NLIST_CASES[case]()
    if case == "binary3000":
        rc = np.array([[2.5, 2.0], [2.0, 2.2]])
        par = np.array([[1.0, 1.0], [0.8, 1.5], [0.8, 1.5], [0.88, 0.5]])
    else:
        par = np.array([[1.0, 1.0]])
    nl = GpuNlist(pos4, box6, rc, rb, layout="col4")
    f, _ = gpu_pair_forces(nl, "lj", par, rc, virial=False, shift=1, tpp=tpp)
    fo, _ = oracle_forces_f64(pos4, box6, "lj", par, rc, shift=1)
    assert_close_f64(f[:, :3], fo[:, :3], what="force")
    assert_close_f64(f[:, 3], fo[:, 3], what="energy")


@pytest.mark.parametrize("layout", ["col", "col4"])
@pytest.mark.parametrize("shift", [0, 1, 2])
def test_lj_binary_shift_modes_vs_fp64_oracle(shift, layout):
    pos4, box6, rc, rb = NLIST_CASES["binary3000"]()
    rc = np.array([[2.5, 2.0], [2.0, 2.2]])
    ron = np.array([[2.0, 1.5], [1.5, 1.8]])
    par = np.array([[1.0, 1.0], [0.8, 1.5], [0.8, 1.5], [0.88, 0.5]])
    nl = GpuNlist(pos4, box6, rc, rb, layout=layout)
    f, v = gpu_pair_forces(nl, "lj", par, rc, shift=shift, r_on=ron)
    fo, vo = oracle_forces_f64(pos4, box6, "lj", par, rc, shift=shift, r_on=ron)
    assert_close_f64(f[:, :3], fo[:, :3], what="force")
    assert_close_f64(f[:, 3], fo[:, 3], what="energy")
    assert_close_f64(v, vo, what="virial")


@pytest.mark.parametrize("layout", ["col", "col4"])
def test_lj_triclinic_vs_fp64_oracle(layout):
    pos4, box6, rc, rb = NLIST_CASES["triclinic1728"]()
    rc = np.array([[2.5, 1.5], [1.5, 2.0]])
    par = np.array([[1.0, 0.5], [0.9, 1.0], [0.9, 1.0], [1.1, 0.7]])
    nl = GpuNlist(pos4, box6, rc, rb, layout=layout)
    f, v = gpu_pair_forces(nl, "lj", par, rc)
    fo, vo = oracle_forces_f64(pos4, box6, "lj", par, rc)
    assert_close_f64(f[:, :3], fo[:, :3], what="force")
    assert_close_f64(f[:, 3], fo[:, 3], what="energy")


@pytest.mark.parametrize("layout", ["col", "col4"])
def test_table_multitype_vs_fp64_oracle(layout):
    nt = 4
    snap = workloads.multitype_system(N=4096, ntypes=nt, density=0.8)
    pos4, box6 = snap_pos4(snap)
    tabs = workloads.mixture_tables(nt, width=1000)
    tables = {k: (v["r_min"], v["U"], v["F"]) for k, v in tabs.items()}
    recs, data, opar, odata = table_params(nt, tables)
    rc = np.full((nt, nt), 3.0)
    nl = GpuNlist(pos4, box6, rc, 0.4, layout=layout)
    f, v = gpu_pair_forces(nl, "table", None, rc, tables=(recs, data))
    fo, vo = oracle_forces_f64(pos4, box6, "table", opar, rc, tdata=odata)
    assert_close_f64(f[:, :3], fo[:, :3], what="force")
    assert_close_f64(f[:, 3], fo[:, 3], what="energy")
    assert_close_f64(v, vo, what="virial")


@pytest.mark.parametrize("kind", ["LJ", "Table"])
def test_forces_and_energies_golden_through_abi(kind):
    fe = json.load(open(GOLD / "forces_and_energies_lj_table.json"))[kind]
    for i, prm in enumerate(fe["params"]):
        for k, d in enumerate([0.75, 1.5]):
            pos4 = O.make_pos4(np.array([[0, 0, 0.1], [0, 0, d + 0.1]]), [0, 0], 32)
            nl = GpuNlist(pos4, (20.0, 20.0, 20.0, 0, 0, 0), [[2.5]], 0.4)
            if kind == "LJ":
                f, _ = gpu_pair_forces(nl, "lj", [[prm["sigma"], prm["epsilon"]]], [[2.5]])
            else:
                recs, data, _, _ = table_params(1, {(0, 0): (prm["r_min"], prm["U"], prm["F"])})
                f, _ = gpu_pair_forces(nl, "table", None, [[2.5]], tables=(recs, data))
            e = float(f[:, 3].astype(np.float64).sum())
            ref_e = fe["energies"][i][k]
            assert np.isclose(e, ref_e, rtol=1e-5, atol=1e-6 if ref_e == 0 else 0), (i, d, e)
            assert np.allclose(f[0, :3], np.array([0, 0, 1.0]) * fe["forces"][i][k], rtol=1e-5,
                               atol=1e-5)


@pytest.mark.parametrize("layout", ["col", "col4"])
def test_example_evaluator_vs_oracle(layout):
    pos4, box6, rc, rb = NLIST_CASES["random700_dims332"]()
    par = np.array([[2.0, 1.2]])
    nl = GpuNlist(pos4, box6, [[1.5]], rb, layout=layout)
    for shift in (0, 1):
        f, v = gpu_pair_forces(nl, "example", par, [[1.5]], shift=shift)
        fo, vo = oracle_forces_f64(pos4, box6, "example", par, [[1.5]], shift=shift)
        assert_close_f64(f[:, :3], fo[:, :3], what="force")
        assert_close_f64(f[:, 3], fo[:, 3], what="energy")


def _integrator_state(N=5000, seed=3):
    rng = np.random.default_rng(seed)
    L = 20.0
    pos4 = O.make_pos4(rng.uniform(-0.5, 0.5, (N, 3)) * L, np.zeros(N), 32)
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, :3] = rng.normal(0, 2.0, (N, 3))
    vel4[:, 3] = rng.uniform(0.5, 2.0, N)
    acc = rng.normal(0, 50.0, (N, 3)).astype(np.float32)
    img = rng.integers(-2, 3, (N, 3)).astype(np.int32)
    return pos4, vel4, acc, img, (L, L, L, 0, 0, 0)


def test_step_one_and_two_bitexact_vs_oracle():
    L_ = abi.load()
    pos4, vel4, acc, img, box6 = _integrator_state()
    N = len(pos4)
    box = abi.make_box(box6[:3])
    dt, s = 0.005, 0.9876
    dp, dv, da, di = dev(pos4), dev(vel4), dev(acc), dev(img)
    abi.check(L_.gb_cv_step_one(p(dp), p(dv), p(da), p(di), N, ctypes.byref(box), dt, s, None,
                                stream()), "step one")
    po, vo, io = O.cv_step_one(pos4, vel4, acc, img, box6, dt, s, prec=32)
    assert np.array_equal(host(dp), po)
    assert np.array_equal(host(dv), vo)
    assert np.array_equal(host(di), io)
    force = np.random.default_rng(5).normal(0, 30, (N, 4)).astype(np.float32)
    df = dev(force)
    abi.check(L_.gb_cv_step_two(p(dv), p(da), p(df), N, dt, 1.0, None, stream()), "step two")
    vo2, ao2 = O.cv_step_two(vo, force, dt, 1.0, prec=32)
    assert np.array_equal(host(dv), vo2)
    assert np.array_equal(host(da).reshape(-1, 3), ao2)


def test_fused_step_one_sets_rebuild_flag():
    L_ = abi.load()
    pos4, vel4, acc, img, box6 = _integrator_state(N=1000)
    N = len(pos4)
    box = abi.make_box(box6[:3])
    dp, dv, da, di = dev(pos4), dev(vel4), dev(np.zeros_like(acc)), dev(img)
    last = dev(pos4)
    flag = zeros(1)
    rcmax = dev(np.array([2.5], np.float32))
    for dt, expect in ((1e-6, 0), (0.5, 1)):
        a = abi.StepOneArgs(d_pos=p(dp), d_vel=p(dv), d_accel=p(da), d_image=p(di), N=N, box=box,
                            dt=dt, scale=1.0, d_last_pos=p(last), d_rcut_max=p(rcmax), r_buff=0.4,
                            d_rebuild=p(flag))
        abi.check(L_.gb_md_step_one(ctypes.byref(a), stream()), "md step one")
        assert int(host(flag)[0]) == expect


def test_thermo_reduce_fp64():
    L_ = abi.load()
    pos4, vel4, acc, img, box6 = _integrator_state(N=300001)
    N = len(vel4)
    force = np.random.default_rng(1).normal(0, 3, (N, 4)).astype(np.float32)
    vir = np.random.default_rng(2).normal(0, 3, (6, N)).astype(np.float32)
    scratch = zeros(L_.gb_thermo_scratch_bytes(N), torch.uint8)
    out = zeros(3, torch.float64)
    dv, df, dvir = dev(vel4), dev(force), dev(vir)
    for _ in range(2):  # the counter word is left zero for the next call
        abi.check(L_.gb_thermo_reduce(p(dv), p(df), p(dvir), N, N, p(scratch), p(out), stream()),
                  "thermo")
        r = host(out)
        v = vel4.astype(np.float64)
        ke = 0.5 * np.sum(v[:, 3] * (v[:, :3] ** 2).sum(1))
        assert np.isclose(r[0], ke, rtol=1e-12)
        assert np.isclose(r[1], force[:, 3].astype(np.float64).sum(), rtol=1e-12, atol=1e-9)
        w = (vir[0].astype(np.float64) + vir[3] + vir[5]).sum() / 3
        assert np.isclose(r[2], w, rtol=1e-11, atol=1e-9)


def test_bussi_factor_matches_oracle():
    L_ = abi.load()
    out = zeros(1, torch.float64)
    for K, dof, tau, kT, ts, seed in [(150.0, 297.0, 0.0, 1.5, 7, 22765), (1.2e6, 3145725.0, 0.0,
                                      1.5, 123456, 3), (50.0, 60.0, 0.5, 0.8, 99, 1)]:
        dk = dev(np.array([K], np.float64))
        abi.check(L_.gb_bussi_factor(p(dk), dof, 0.005, tau, kT, ts, seed, 0, p(out), stream()),
                  "bussi")
        want = O.bussi_factor(K, dof, 0.005, tau, kT, ts, seed, 0)
        assert np.isclose(host(out)[0], want, rtol=1e-9), (host(out)[0], want)


def test_thermalize_vs_oracle():
    L_ = abi.load()
    N = 20000
    vel4 = np.zeros((N, 4), np.float32)
    vel4[:, 3] = np.random.default_rng(0).uniform(0.5, 2.0, N)
    tags = np.arange(N, dtype=np.uint32)
    dv, dt_ = dev(vel4), dev(tags)
    scratch = zeros(L_.gb_thermo_scratch_bytes(N), torch.uint8)
    abi.check(L_.gb_thermalize(p(dv), p(dt_), N, 1.5, 0, 22765, 3, p(scratch), stream()),
              "thermalize")
    v = host(dv)
    vo = O.thermalize(vel4, tags, 1.5, 0, 22765, prec=32)
    # same Philox stream; sincospif / logf on the GPU vs sinf / logf on the host: a few ulp
    assert np.allclose(v[:, :3], vo[:, :3], rtol=1e-5, atol=1e-5)
    mom = (v[:, 3:4].astype(np.float64) * v[:, :3]).sum(0)
    assert np.all(np.abs(mom) < 1e-2)


def test_sfc_order_is_deterministic_permutation_with_locality():
    L_ = abi.load()
    snap = workloads.lj_fluid_fcc(m=16)
    pos4, box6 = snap_pos4(snap)
    N = len(pos4)
    rng = np.random.default_rng(0)
    perm = rng.permutation(N)
    pos4 = pos4[perm]
    box = abi.make_box(box6[:3])
    need = L_.gb_sfc_scratch_bytes(N, 8)
    scratch = zeros(need, torch.uint8)
    orders = []
    for _ in range(2):
        order = zeros(N)
        abi.check(L_.gb_sfc_order(p(dev(pos4)), N, ctypes.byref(box), 8, p(order), p(scratch),
                                  need, stream()), "sfc")
        orders.append(host(order).astype(np.int64))
    assert np.array_equal(orders[0], orders[1])
    assert np.array_equal(np.sort(orders[0]), np.arange(N))
    xyz = pos4[orders[0], :3].astype(np.float64)
    step = np.linalg.norm(np.diff(xyz, axis=0), axis=1)
    # consecutive particles are neighbours in space (a lattice spacing is ~1.2 here)
    assert np.median(step) < 2.0
    # gather applies the order
    dst = zeros(4 * N, torch.float32)
    src = dev(pos4)
    abi.check(L_.gb_gather(p(dst), p(src), p(dev(orders[0].astype(np.uint32))), N, 16, stream()),
              "gather")
    assert np.array_equal(host(dst).reshape(-1, 4), pos4[orders[0]])


SORT_CASES = {
    "fcc16k_shuffled": lambda: (lambda s: snap_pos4(s))(workloads.lj_fluid_fcc(m=16)),
    "random60k": lambda: random_system(60000, (41.0, 41.0, 41.0), seed=7),
    "triclinic1728": lambda: random_system(1728, (11.0, 12.0, 13.0), 2, seed=4,
                                           tilts=(0.3, -0.2, 0.1), lattice=True),
    "fcc1m": lambda: snap_pos4(workloads.lj_fluid_fcc(m=64)),
    "hi_face4096": lambda: hi_face_system(),
}


@pytest.mark.parametrize("case", sorted(SORT_CASES))
@pytest.mark.parametrize("grid_bits", [8, 5])
def test_sfc_order_equals_oracle(case, grid_bits):
    """The particle sort's permutation is the reference's (SFCPackTuner::getSortedOrder3D:
    Hilbert traversal of the grid, ties by old index), element for element."""
    L_ = abi.load()
    pos4, box6 = SORT_CASES[case]()
    N = len(pos4)
    pos4 = pos4[np.random.default_rng(1).permutation(N)]
    box = abi.make_box(box6[:3], box6[3:])
    need = L_.gb_sfc_scratch_bytes(N, grid_bits)
    scratch = zeros(need, torch.uint8)
    order = zeros(N)
    abi.check(L_.gb_sfc_order(p(dev(pos4)), N, ctypes.byref(box), grid_bits, p(order),
                              p(scratch), need, stream()), "sfc")
    want = O.sfc_order(pos4, box6, grid=1 << grid_bits)
    got = host(order).astype(np.uint32)
    assert np.array_equal(got, want), f"{(got != want).sum()} of {N} positions differ"


def test_sfc_order_2d_equals_oracle():
    """2D: the reference's row-major bin order on a 4096 grid (getSortedOrder2D)."""
    L_ = abi.load()
    rng = np.random.default_rng(9)
    N = 20000
    xy = rng.uniform(-50.0, 50.0, (N, 2))
    pos4 = O.make_pos4(np.column_stack([xy, np.zeros(N)]), np.zeros(N), 32)
    box = abi.make_box((100.0, 100.0, 1.0), (0, 0, 0))
    need = L_.gb_sfc_scratch_bytes_dim(N, 12, 2)
    scratch = zeros(need, torch.uint8)
    order = zeros(N)
    abi.check(L_.gb_sfc_order_dim(p(dev(pos4)), N, ctypes.byref(box), 12, 2, p(order),
                                  p(scratch), need, stream()), "sfc 2d")
    want = O.sfc_order(pos4, (100.0, 100.0, 1.0, 0, 0, 0), grid=4096, ndim=2)
    assert np.array_equal(host(order).astype(np.uint32), want)


def test_needs_update_kernel():
    L_ = abi.load()
    pos4, vel4, acc, img, box6 = _integrator_state(N=2000)
    N = len(pos4)
    box = abi.make_box(box6[:3])
    last = dev(pos4)
    moved = pos4.copy()
    flag = zeros(1)
    rcmax = dev(np.array([2.5], np.float32))
    lam = (ctypes.c_float * 3)(1, 1, 1)
    abi.check(L_.gb_nlist_needs_update(p(flag), p(last), p(dev(moved)), N, ctypes.byref(box),
                                       p(rcmax), 0.4, 1, 1.0, lam, 1, stream()), "check")
    assert int(host(flag)[0]) == 0
    moved[123, 0] += 0.21  # >= r_buff / 2
    abi.check(L_.gb_nlist_needs_update(p(flag), p(last), p(dev(moved)), N, ctypes.byref(box),
                                       p(rcmax), 0.4, 1, 1.0, lam, 7, stream()), "check")
    assert int(host(flag)[0]) == 7


def test_bussi_predrawn_ring_gives_the_same_factor():
    """gb_bussi_draws fills the ring with each timestep's (normal, 2*gamma); the factor formed
    from them equals the oracle's per-step Bussi factor (same Philox stream, same algorithm)."""
    L_ = abi.load()
    ring_size, count, t0 = 64, 40, 1000
    ring = zeros(2 * ring_size, torch.float64)
    ts = dev(np.array([t0], np.int64))
    dof, seed, K, dt, kT = 3.0 * 4096 - 3, 22765, 5000.0, 0.005, 1.5
    abi.check(L_.gb_bussi_draws(p(ts), count, dof, seed, 0, p(ring), ring_size, stream()),
              "draws")
    r = host(ring).reshape(-1, 2)
    for k in range(count):
        t = t0 + 1 + k
        n, g = r[t % ring_size]
        v = kT / 2.0 / K
        factor = np.sqrt(v * (g + n * n))  # tau = 0: time_decay_factor = 0
        assert np.isclose(factor, O.bussi_factor(K, dof, dt, 0.0, kT, t, seed, 0), rtol=1e-9)


@pytest.mark.parametrize("case", ["lj4096", "binary3000", "triclinic1728", "random60k",
                                  "hi_face4096", "dense2720"])
@pytest.mark.parametrize("layout", ["col", "col4"])
def test_tiled_builds_are_identical(case, layout):
    """The candidate-stream, lane-per-particle and warp-per-cell tiled builds write the same
    neighbours in the same order (so the force sums, and with them trajectories, do not depend on
    which one ran). The cell lists are built in the deterministic (sorted) mode, so all three read
    the same cell order."""
    pos4, box6, rc, rb = NLIST_CASES[case]()
    a = GpuNlist(pos4, box6, rc, rb, layout=layout, deterministic=True)
    N = len(pos4)
    na, la = host(a.n_neigh), host(a.nlist)
    k = np.arange(int(na.max()))[None, :]
    i = np.arange(N)[:, None]
    if layout == "col4":
        idx = ((k // 4) * a.stride + i) * 4 + k % 4
    else:
        idx = k * a.stride + i
    valid = k < na[:, None]
    for form in ("_lane", "w"):
        b = GpuNlist(pos4, box6, rc, rb, layout=layout + form, deterministic=True)
        nb, lb = host(b.n_neigh), host(b.nlist)
        assert np.array_equal(na, nb), form
        assert np.array_equal(la[idx][valid], lb[idx][valid]), form
