"""Neighbour-list exclusions (hoomd.md.nlist.Cell(exclusions=...), gb_nlist_filter): the list is
the oracle's set at r_list minus the excluded tag pairs, forces skip excluded pairs, and the
exclusions follow the particles through the Hilbert sort."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402
from hoomd_gb300.md.nlist import excluded_pairs  # noqa: E402
from oracle import oracle as O  # noqa: E402


def chains(n=10, length=10, density=0.84, seed=3):
    """Lattice particles bonded into chains of consecutive tags (lattice neighbours along x)."""
    s = workloads.lj_fluid_sc(n, density=density, jitter=0.05, seed=seed)
    N = s.particles.N
    b = [(i, i + 1) for i in range(N - 1) if (i + 1) % length != 0]
    s.bonds.N = len(b)
    s.bonds.types = ["b"]
    s.bonds.group[:] = b
    return s


def make(snap, exclusions, sorter=None, dt=0.004):
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=4)
    sim.create_state_from_snapshot(snap)
    cell = md.nlist.Cell(buffer=0.4, exclusions=exclusions)
    lj = md.pair.LJ(nlist=cell, default_r_cut=2.5)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    sim.operations.integrator = md.Integrator(
        dt=dt, forces=[lj], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    if sorter:
        sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=sorter))
    return sim, lj, cell


def topology(snap):
    return {k: getattr(snap, k) for k in ("bonds", "angles", "dihedrals", "impropers",
                                          "constraints", "pairs")}


@pytest.mark.parametrize("exclusions", [(), ("bond",), ("bond", "1-3"), ("bond", "1-3", "1-4")])
def test_pair_list_is_oracle_set_minus_exclusions(exclusions):
    snap = chains()
    N = snap.particles.N
    sim, lj, cell = make(snap, exclusions)
    sim.run(0)
    pos4 = O.make_pos4(sim.state.get_snapshot().particles.position, np.zeros(N), 32)
    n, l, h, _ = O.build_nlist(pos4, tuple(snap.configuration.box), [[2.5]], 0.4, full=False,
                               prec=32)
    ref = set()
    for i, js in enumerate(O.neighbor_sets(n, l, h)):
        for j in js:
            ref.add((min(i, int(j)), max(i, int(j))))
    ex = set(map(tuple, excluded_pairs(topology(snap), exclusions, N).tolist()))
    if exclusions:
        assert ex & ref  # some excluded pairs are within r_list (1-4 ones are just beyond it)
    got = set((int(a), int(b)) for a, b in np.sort(cell.pair_list(), axis=1))
    assert got == ref - ex


def brute_lj(pos, L, ex, rc=2.5):
    N = len(pos)
    F = np.zeros((N, 3))
    E = 0.0
    for i in range(N):
        d = pos[i] - pos
        d -= L * np.rint(d / L)
        r2 = (d * d).sum(1)
        m = (r2 < rc * rc) & (r2 > 0)
        for j in ex.get(i, ()):
            m[j] = False
        ir6 = 1.0 / r2[m] ** 3
        fd = 24 * ir6 * (2 * ir6 - 1) / r2[m]
        F[i] = (fd[:, None] * d[m]).sum(0)
        E += 0.5 * (4 * ir6 * (ir6 - 1)).sum()
    return F, E


def test_forces_skip_excluded_pairs():
    snap = chains(8)
    N = snap.particles.N
    sim, lj, cell = make(snap, ("bond", "1-3"))
    sim.run(0)
    pos = np.asarray(sim.state.get_snapshot().particles.position, np.float32).astype(np.float64)
    ex = {}
    for a, b in excluded_pairs(topology(snap), ("bond", "1-3"), N).tolist():
        ex.setdefault(a, []).append(b)
        ex.setdefault(b, []).append(a)
    Fo, Eo = brute_lj(pos, snap.configuration.box[0], ex)
    F = lj.forces
    scale = np.abs(Fo).max()
    assert np.all(np.abs(F - Fo) <= 1e-5 * np.abs(Fo) + 1e-5 * scale)
    assert np.isclose(lj.energy, Eo, rtol=1e-5)


def test_exclusions_follow_the_sort():
    """With the Hilbert sort permuting indices every 7 steps, the trajectory equals the unsorted
    one (exclusion rows are rebuilt for the new indices)."""
    snap = chains(10)
    out = []
    for sorter in (None, 7):
        sim, lj, cell = make(snap, ("bond",), sorter=sorter)
        sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.0)
        sim.run(30)
        out.append(sim.state.get_snapshot())
    a, b = out
    box = np.array(snap.configuration.box[:3])
    ua = a.particles.position + a.particles.image * box
    ub = b.particles.position + b.particles.image * box
    assert np.abs(ua - ub).max() < 1e-3
    assert a.bonds.N == snap.bonds.N and np.array_equal(a.bonds.group, snap.bonds.group)
