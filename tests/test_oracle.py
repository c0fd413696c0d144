"""Pin the CPU oracle (oracle/md_oracle.cc) before trusting it.

1. Against the reference's own golden vectors (tests/golden/, copied from the reference's pytest
   fixtures): forces_and_energies.json LJ/Table entries and true_pair_list.json.
2. Bit-for-bit against the reference's own header-only maths compiled unmodified
   (tests/golden/ref_vectors.npz; live on random inputs too when oracle/_ref is present).
3. Against the published Philox4x32-10 known-answer vectors (random123 is absent from the
   reference checkout) and the distributional facts the reference's own RNG tests check.
4. Against independent brute-force restatements (O(N^2) neighbour search, finite differences).
"""

import json
import pathlib

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refshim

GOLD = pathlib.Path(__file__).resolve().parent / "golden"
Z = np.load(GOLD / "ref_vectors.npz")


def sc_lattice(n, a=1.0, r=0.0, seed=0):
    """hoomd/conftest.py:203-253 lattice_snapshot_factory (same meshgrid ordering -> same tags)."""
    ranges = [np.arange(-n / 2, n / 2) for _ in range(3)]
    x, y, z = np.meshgrid(*ranges)
    pos = (np.vstack((x.flatten(), y.flatten(), z.flatten())).T + 0.5) * a
    if r > 0:
        pos += np.random.default_rng(seed).uniform(-r, r, size=pos.shape)
    return pos, (n * a,) * 3


# --- 3. random numbers ------------------------------------------------------------------------------

def test_philox_known_answers():
    # Published Philox4x32-10 known-answer vectors (Salmon et al. SC'11 / random123 kat_vectors).
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert O.philox(ctr, key).tolist() == want


def test_seed_key_packing():
    # hoomd/RandomNumbers.h:136-168 layout: id | seed1 seed0 | timestep bits 32-39 ; timestep low
    # word. The reference's own KAT (hoomd/test/random_numbers_test.cc:456-461) checks this packing.
    key = O.seed_key(0xAB, 0x0000_00CD_1234_5678, 0xBEEF)
    assert key[0] == (0xAB << 24) | (0xBEEF << 8) | 0xCD
    assert key[1] == 0x12345678


def test_normal_and_gamma_moments():
    x = O.normal_draws(200, 1, 7, 3, 200000)
    assert abs(x.mean()) < 0.01 and abs(x.std() - 1) < 0.01
    for alpha in (0.5, 1.5, 40.0, 1.5e6):
        g = O.gamma_draws(201, 2, 7, 4, alpha, 20000 if alpha < 1e3 else 2000)
        assert abs(g.mean() / alpha - 1) < 5 * np.sqrt(1 / alpha / len(g)) + 1e-9
        assert abs(g.var() / alpha - 1) < 0.1


def test_bussi_factor_samples_canonical_ke():
    # With tau = 0, K' = s^2 K is a fresh draw of (kT/2) * chi^2_dof (Bussi et al. 2007).
    dof, kT, K = 300.0, 1.5, 123.0
    s = np.array([O.bussi_factor(K, dof, 0.005, 0.0, kT, t, 5, 0) for t in range(20000)])
    Kn = s * s * K
    assert abs(Kn.mean() / (0.5 * kT * dof) - 1) < 0.01
    assert abs(Kn.var() / (0.5 * kT * kT * dof) - 1) < 0.06
    assert O.bussi_factor(K, dof, 0.0, 0.0, kT, 3, 5, 0) == 1.0


def test_thermalize_zero_momentum_and_temperature():
    N = 20000
    vel = np.zeros((N, 4), np.float64)
    vel[:, 3] = 1.0
    v = O.thermalize(vel, np.arange(N), 1.5, 0, 22765, prec=64)
    assert np.allclose(v[:, :3].sum(0), 0, atol=1e-9)
    T = (v[:, :3] ** 2).sum() / (3 * N - 3)
    assert abs(T / 1.5 - 1) < 0.02


# --- 2. evaluators and geometry vs the reference's headers ------------------------------------------

@pytest.mark.parametrize("prec", [32, 64])
def test_lj_bitexact_vs_reference(prec):
    c = 0
    while f"lj{c}_case" in Z:
        sigma, eps, rcutsq, shift = Z[f"lj{c}_case"]
        f, e, ok = O.lj_eval(Z[f"lj{c}_rsq"], rcutsq, sigma, eps, bool(shift), prec)
        assert np.array_equal(ok, Z[f"lj{c}_ok{prec}"])
        assert np.array_equal(f.astype(np.float64), Z[f"lj{c}_f{prec}"])
        assert np.array_equal(e.astype(np.float64), Z[f"lj{c}_e{prec}"])
        lrc = O.lj_lrc(rcutsq, sigma, eps, prec).astype(np.float64)
        assert np.allclose(lrc, Z[f"lj{c}_lrc{prec}"], rtol=1e-6 if prec == 32 else 1e-14)
        c += 1
    assert c >= 5


@pytest.mark.parametrize("prec", [32, 64])
def test_table_bitexact_vs_reference(prec):
    c = 0
    while f"tab{c}_case" in Z:
        rmin, rcutsq, width = Z[f"tab{c}_case"]
        f, e, ok = O.table_eval(Z[f"tab{c}_rsq"], rcutsq, rmin, Z[f"tab{c}_U"], Z[f"tab{c}_F"], prec)
        assert np.array_equal(ok, Z[f"tab{c}_ok{prec}"])
        assert np.array_equal(f.astype(np.float64), Z[f"tab{c}_f{prec}"])
        assert np.array_equal(e.astype(np.float64), Z[f"tab{c}_e{prec}"])
        c += 1
    assert c >= 5


@pytest.mark.parametrize("prec", [32, 64])
def test_example_bitexact_vs_reference(prec):
    c = 0
    while f"ex{c}_case" in Z:
        k, sigma, rcutsq, shift = Z[f"ex{c}_case"]
        f, e, ok = O.example_eval(Z[f"ex{c}_rsq"], rcutsq, k, sigma, bool(shift), prec)
        assert np.array_equal(ok, Z[f"ex{c}_ok{prec}"])
        assert np.array_equal(f.astype(np.float64), Z[f"ex{c}_f{prec}"])
        assert np.array_equal(e.astype(np.float64), Z[f"ex{c}_e{prec}"])
        c += 1


@pytest.mark.parametrize("prec", [32, 64])
def test_geometry_bitexact_vs_reference(prec):
    R = np.float32 if prec == 32 else np.float64
    c = 0
    while f"box{c}_b6" in Z:
        b6, per = Z[f"box{c}_b6"], Z[f"box{c}_per"]
        # host (branch) form bit-exact; device (rint) form equal within one image
        mi = O.min_image(Z[f"box{c}_mi_in"].astype(R), b6, prec, False, per)
        assert np.array_equal(mi.astype(np.float64), Z[f"box{c}_mi{prec}"])
        mr = O.min_image(Z[f"box{c}_mi_in"].astype(R), b6, prec, True, per)
        L = b6[:3]
        inner = np.all(np.abs(Z[f"box{c}_mi{prec}"]) < 0.499 * L, axis=1)
        assert np.allclose(mr[inner], Z[f"box{c}_mi{prec}"][inner], rtol=0,
                           atol=4 * np.finfo(R).eps * L.max())
        wv, wi = O.wrap(Z[f"box{c}_wrap_in"].astype(R), Z[f"box{c}_wrap_img"], b6, prec, per)
        assert np.array_equal(wv.astype(np.float64), Z[f"box{c}_wrap{prec}"])
        assert np.array_equal(wi, Z[f"box{c}_wrapimg{prec}"])
        fr = O.make_fraction(Z[f"box{c}_frac_in"].astype(R), b6, prec, per)
        assert np.array_equal(fr.astype(np.float64), Z[f"box{c}_frac{prec}"])
        npd = O.nearest_plane_distance(b6, prec, per)
        assert np.array_equal(npd.astype(np.float64), Z[f"box{c}_npd{prec}"])
        c += 1


@pytest.mark.skipif(not refshim.available(), reason="reference headers not built here")
@pytest.mark.parametrize("prec", [32, 64])
def test_live_random_vs_reference(prec):
    rng = np.random.default_rng(prec)
    for _ in range(20):
        sigma, eps = rng.uniform(0.5, 1.5), rng.uniform(0.1, 2)
        rc = rng.uniform(1.5, 3.5)
        rsq = rng.uniform(0.3, (1.1 * rc) ** 2, 1000)
        a = O.lj_eval(rsq, rc * rc, sigma, eps, True, prec)
        b = refshim.lj_eval(rsq, rc * rc, sigma, eps, True, prec)
        assert np.array_equal(a[0].astype(np.float64), b[0])
        assert np.array_equal(a[1].astype(np.float64), b[1])


# --- 1. golden vectors ------------------------------------------------------------------------------

def two_particle_forces(kind, params, d, prec, r_cut=2.5, L=20.0):
    """Reference test geometry: particles at (0,0,0.1) and (0,0,d+0.1) in an L=20 box."""
    xyz = np.array([[0, 0, 0.1], [0, 0, d + 0.1]])
    pos4 = O.make_pos4(xyz, [0, 0], prec)
    n, nl, head, _ = O.build_nlist(pos4, (L, L, L), [[r_cut]], 0.4, full=True, prec=prec)
    if kind == "lj":
        p = np.array([[params["sigma"], params["epsilon"]]])
        f, v = O.pair_forces("lj", pos4, (L, L, L), p, [[r_cut * r_cut]], n, nl, head, prec=prec)
    else:
        U = np.asarray(params["U"], np.float64)
        F = np.asarray(params["F"], np.float64)
        p = np.array([[params["r_min"], len(U), 0]])
        f, v = O.pair_forces("table", pos4, (L, L, L), p, [[r_cut * r_cut]], n, nl, head,
                             tdata=np.concatenate([U, F]), prec=prec)
    return f


def isclose(value, reference, rtol=5e-6):
    # hoomd/md/pytest/test_potential.py:994-1006 (auto atol)
    atol = 1e-6 if reference == 0 else 0
    return np.isclose(value, reference, rtol=rtol, atol=atol)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("kind", ["LJ", "Table"])
def test_forces_and_energies_golden(kind, prec):
    fe = json.load(open(GOLD / "forces_and_energies_lj_table.json"))[kind]
    for i, params in enumerate(fe["params"]):
        for k, d in enumerate([0.75, 1.5]):
            f = two_particle_forces(kind.lower(), params, d, prec)
            e_tot = float(f[:, 3].astype(np.float64).sum())
            rtol = 5e-6 if prec == 64 else 2e-5
            assert isclose(e_tot, fe["energies"][i][k], rtol), (i, d, e_tot)
            want = np.array([0, 0, 1.0]) * fe["forces"][i][k]
            assert np.allclose(f[0, :3], want, rtol=rtol, atol=1e-6 if prec == 64 else 1e-5)
            # Newton's third law between the two particles
            assert np.allclose(f[1, :3], -f[0, :3], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("full", [True, False])
def test_true_pair_list_golden(prec, full):
    truth = set(frozenset(p) for p in json.load(open(GOLD / "true_pair_list_sc7.json")))
    pos, L = sc_lattice(7, 1.0)
    pos4 = O.make_pos4(pos, np.zeros(len(pos)), prec)
    n, nl, head, _ = O.build_nlist(pos4, L, [[1.1]], 0.0, full=full, prec=prec)
    got = set()
    for i, s in enumerate(O.neighbor_sets(n, nl, head)):
        for j in s:
            got.add(frozenset((i, int(j))))
    assert got == truth
    assert n.sum() == (2 if full else 1) * len(truth)


# --- 4. independent restatements -------------------------------------------------------------------

def brute_force_sets(pos4, L, r_list, prec):
    R = np.float32 if prec == 32 else np.float64
    p = pos4[:, :3].astype(R)
    Lr = np.asarray(L, R)
    Linv = (R(1) / Lr).astype(R)
    out = []
    for i in range(len(p)):
        d = (p[i] - p).astype(R)
        # device minImage form, z then y then x (orthorhombic), no FMA contraction in numpy
        d = (d - Lr * np.rint(d * Linv)).astype(R)
        rsq = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        m = rsq <= R(r_list) * R(r_list)
        m[i] = False
        out.append(np.nonzero(m)[0])
    return out


@pytest.mark.parametrize("prec", [32, 64])
def test_nlist_vs_brute_force(prec):
    rng = np.random.default_rng(3)
    L = (9.3, 10.1, 8.0)
    N = 700
    xyz = (rng.uniform(-0.5, 0.5, (N, 3)) * L)
    pos4 = O.make_pos4(xyz, np.zeros(N), prec)
    r_cut, r_buff = 2.5, 0.4
    n, nl, head, info = O.build_nlist(pos4, L, [[r_cut]], r_buff, full=True, prec=prec)
    R = np.float32 if prec == 32 else np.float64
    r_list = R(R(r_cut) + R(r_buff))
    bf = brute_force_sets(pos4, L, r_list, prec)
    got = O.neighbor_sets(n, nl, head)
    mismatch = [i for i in range(N) if not np.array_equal(got[i], bf[i])]
    assert not mismatch
    # 8.0/2.9 -> 2 cells in z: the deduplicated-adjacency path is exercised
    assert list(info["dim"]) == [3, 3, 2]


def test_cell_adj_dedup_small_dims():
    adj = O.cell_adj([2, 3, 1])
    assert adj.shape == (6, 6)
    for row in adj:
        assert list(row) == sorted(set(row))
    adj = O.cell_adj([5, 5, 5])
    assert adj.shape == (125, 27)


@pytest.mark.parametrize("prec", [32, 64])
def test_half_list_third_law_matches_full(prec):
    rng = np.random.default_rng(11)
    L = (8.0, 8.0, 8.0)
    pos, _ = sc_lattice(6, 8.0 / 6, 0.1, seed=5)
    pos4 = O.make_pos4(pos, rng.integers(0, 2, len(pos)), prec)
    rc = np.array([[2.5, 2.0], [2.0, 2.2]])
    par = np.array([[1.0, 1.0], [1.5, 0.8], [1.5, 0.8], [0.5, 0.88]])
    par = par[:, [1, 0]]  # (sigma, epsilon)
    out = {}
    for full in (True, False):
        n, nl, head, _ = O.build_nlist(pos4, L, rc, 0.3, full=full, prec=prec)
        out[full] = O.pair_forces("lj", pos4, L, par, rc * rc, n, nl, head, third_law=not full,
                                  compute_virial=True, prec=prec)
    tol = 2e-4 if prec == 32 else 1e-10
    for a, b in zip(out[True], out[False]):
        assert np.allclose(a, b, rtol=tol, atol=tol * np.abs(a).max())


def test_lj_force_is_minus_energy_gradient():
    # hoomd/md/pytest/test_potential.py:858-949: F = -dE/dr by finite differences, rtol 1e-5
    r = np.linspace(0.9, 2.4, 40)
    h = 1e-6
    f, _, _ = O.lj_eval(r * r, 6.25, 1.0, 1.0, prec=64)
    _, ep, _ = O.lj_eval((r + h) ** 2, 6.25, 1.0, 1.0, prec=64)
    _, em, _ = O.lj_eval((r - h) ** 2, 6.25, 1.0, 1.0, prec=64)
    assert np.allclose(f * r, -(ep - em) / (2 * h), rtol=1e-5, atol=1e-7)


def test_nve_energy_conservation_fp64():
    pos, L = sc_lattice(8, 1.6, 0.05, seed=1)
    N = len(pos)
    pos4 = O.make_pos4(pos - 0.0, np.zeros(N), 64)
    vel = np.zeros((N, 4))
    vel[:, 3] = 1.0
    vel = O.thermalize(vel, np.arange(N), 1.0, 0, 9, prec=64)
    sim = O.Sim(pos4, vel, np.zeros((N, 3), np.int32), np.arange(N), L, [[2.5]], 0.4, 0.002,
                params=[[1.0, 1.0]], shift_mode=1, prec=64)
    sim.run(1)
    s0 = sim.stats()
    e0 = s0["kinetic_energy"] + s0["potential_energy"]
    sim.run(400)
    s1 = sim.stats()
    e1 = s1["kinetic_energy"] + s1["potential_energy"]
    assert s1["n_builds"] > 2
    assert abs(e1 - e0) / N < 2e-3


def test_bussi_thermostat_holds_temperature():
    pos, L = sc_lattice(8, 1.6, 0.05, seed=2)
    N = len(pos)
    pos4 = O.make_pos4(pos, np.zeros(N), 32)
    vel = np.zeros((N, 4), np.float32)
    vel[:, 3] = 1.0
    vel = O.thermalize(vel, np.arange(N), 0.5, 0, 9, prec=32)
    sim = O.Sim(pos4, vel, np.zeros((N, 3), np.int32), np.arange(N), L, [[2.5]], 0.4, 0.005,
                params=[[1.0, 1.0]], bussi=True, kT=1.5, seed=9, prec=32)
    sim.run(300)
    T = 2 * sim.stats()["kinetic_energy"] / (3 * N - 3)
    assert abs(T - 1.5) < 0.3


def _schedule_sim(r_buff, delay, dist_check, steps=40):
    """NeighborList::needsUpdating's schedule (hoomd/md/NeighborList.cc:1313-1418) in the
    oracle: a fluid run of ``steps`` steps with the given buffer and rebuild-check settings."""
    pos, L = sc_lattice(8, 1.2, 0.05, seed=3)
    N = len(pos)
    pos4 = O.make_pos4(pos, np.zeros(N), 32)
    vel = np.zeros((N, 4), np.float32)
    vel[:, 3] = 1.0
    vel = O.thermalize(vel, np.arange(N), 1.5, 0, 9, prec=32)
    sim = O.Sim(pos4, vel, np.zeros((N, 3), np.int32), np.arange(N), L, [[2.5]], r_buff, 0.005,
                params=[[1.0, 1.0]], prec=32)
    sim.set_check(delay, dist_check)
    sim.run(steps)
    return sim


def test_oracle_rebuild_check_schedule():
    # a buffer so thin that every check finds the list stale: with a delay of 4 the list is
    # built at steps 4, 8, ..., 40, each at the first check after the delay (dangerous)
    st = _schedule_sim(0.002, 4, True).stats()
    assert (st["checked_builds"], st["dangerous_builds"], st["last_update"]) == (10, 10, 40)
    # without the distance check: the same builds, none of them dangerous
    st = _schedule_sim(0.002, 4, False).stats()
    assert (st["checked_builds"], st["dangerous_builds"], st["last_update"]) == (10, 0, 40)
    # rebuild_check_delay = 0 without the distance check: every step
    st = _schedule_sim(0.4, 0, False).stats()
    assert (st["checked_builds"], st["dangerous_builds"]) == (40, 0)
    # the default (check every step) with the thin buffer: a build every step, none dangerous
    st = _schedule_sim(0.002, 1, True).stats()
    assert (st["checked_builds"], st["dangerous_builds"]) == (40, 0)
    # check_dist=False with rebuild_check_delay = 1 still checks the distance (the reference's
    # condition only skips the check for a delay of 0 or above 1)
    a = _schedule_sim(0.4, 1, False).stats()
    b = _schedule_sim(0.4, 1, True).stats()
    assert a["checked_builds"] == b["checked_builds"] < 40


def test_oracle_delayed_check_keeps_the_physics():
    """With a buffer wide enough for the delay, a list checked every third step holds every
    pair within r_cut, so the trajectory follows the every-step one to FP32 round-off."""
    a = _schedule_sim(0.4, 3, True, steps=60)
    b = _schedule_sim(0.4, 1, True, steps=60)
    sa, sb = a.stats(), b.stats()
    assert sa["dangerous_builds"] == 0
    assert sa["checked_builds"] <= 60 // 3
    assert np.abs(a.get()["pos"][:, :3] - b.get()["pos"][:, :3]).max() < 1e-3
