"""The reference's other radial pair potentials (one kernel family, gb_pair_forces_radial) through
the hoomd-style API: the reference's own golden values (hoomd/md/pytest/forces_and_energies.json,
harness hoomd/md/pytest/test_potential.py:952-1058), and many-particle forces against an FP64
brute-force sum of the closed forms written out below."""

import json
import math
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import hoomd_gb300 as hoomd  # noqa: E402
from hoomd_gb300 import md, workloads  # noqa: E402

GOLD = json.load(open(pathlib.Path(__file__).resolve().parent / "golden"
                      / "forces_and_energies_radial.json"))
NAMES = [k for k in GOLD if not k.startswith("_")]


def two_particles(d, L=20.0, charge=0.0):
    s = hoomd.Snapshot()
    s.configuration.box = [L, L, L, 0, 0, 0]
    s.particles.N = 2
    s.particles.types = ["A"]
    s.particles.position[:] = [[0, 0, 0.1], [0, 0, d + 0.1]]
    s.particles.charge[:] = charge
    return s


def potential(name, params, mode="none", r_cut=2.5):
    cls = getattr(md.pair, name)
    f = cls(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=r_cut, mode=mode)
    f.params[("A", "A")] = params
    return f


@pytest.mark.parametrize("name", NAMES)
def test_force_energy_accuracy(name):
    ent = GOLD[name]
    for i, params in enumerate(ent["params"]):
        f = potential(name, params)
        sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
        # unit charges for Ewald, as the reference's harness sets them
        sim.create_state_from_snapshot(two_particles(0.75, charge=1.0 if name == "Ewald" else 0.0))
        sim.operations.integrator = md.Integrator(
            dt=0.005, forces=[f], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
        sim.run(0)
        for k, d in enumerate([0.75, 1.5]):
            e_ref, f_ref = ent["energies"][i][k], ent["forces"][i][k]
            if isinstance(e_ref, str) or isinstance(f_ref, str):
                continue  # infinite inside the hard core (TWF)
            snap = sim.state.get_snapshot()
            snap.particles.position[0] = [0, 0, 0.1]
            snap.particles.position[1] = [0, 0, d + 0.1]
            sim.state.set_snapshot(snap)
            E = float(np.sum(f.energies, dtype=np.float64))
            F = f.forces[0]
            # 2e-5 relative, with a 5e-8 floor for FP32 cancellation (DLVO's energy at 1.5 is
            # 4.5e-4 from terms near 1e-2)
            tol = 2e-5 * abs(e_ref) + (1e-6 if e_ref == 0 else 5e-8)
            assert abs(E - e_ref) <= tol, (name, i, d, E, e_ref)
            assert np.allclose(F, [0, 0, f_ref], rtol=2e-5, atol=1e-6), (name, i, d, F, f_ref)


def closed_form(name, p):
    """V(r) in float64, the same closed forms as hoomd/md/EvaluatorPair*.h."""
    def lj(r, s, e, n=12, m=6):
        return 4 * e * ((s / r) ** n - (s / r) ** m)

    if name == "Gaussian":
        return lambda r: p["epsilon"] * np.exp(-r ** 2 / (2 * p["sigma"] ** 2))
    if name == "Yukawa":
        return lambda r: p["epsilon"] * np.exp(-p["kappa"] * r) / r
    if name == "Morse":
        return lambda r: p["D0"] * (np.exp(-2 * p["alpha"] * (r - p["r0"]))
                                    - 2 * np.exp(-p["alpha"] * (r - p["r0"])))
    if name == "ForceShiftedLJ":
        rc = 2.5
        h = 1e-7
        frc = -(lj(rc + h, p["sigma"], p["epsilon"]) - lj(rc - h, p["sigma"], p["epsilon"])) / (2 * h)
        return lambda r: lj(r, p["sigma"], p["epsilon"]) + (r - rc) * frc
    if name in ("Mie", "ExpandedMie"):
        n, m = p["n"], p["m"]
        pre = (n / (n - m)) * (n / m) ** (m / (n - m)) * p["epsilon"]
        dl = p.get("delta", 0.0)
        return lambda r: pre * ((p["sigma"] / (r - dl)) ** n - (p["sigma"] / (r - dl)) ** m)
    if name == "ExpandedLJ":
        return lambda r: lj(r - p["delta"], p["sigma"], p["epsilon"])
    if name == "Buckingham":
        return lambda r: p["A"] * np.exp(-r / p["rho"]) - p["C"] / r ** 6
    if name == "LJ1208":
        return lambda r: lj(r, p["sigma"], p["epsilon"], 12, 8)
    if name == "LJ0804":
        return lambda r: lj(r, p["sigma"], p["epsilon"], 8, 4)
    if name == "LJGauss":
        return lambda r: (1 / r ** 12 - 2 / r ** 6
                          - p["epsilon"] * np.exp(-(r - p["r0"]) ** 2 / (2 * p["sigma"] ** 2)))
    if name == "ExpandedGaussian":
        return lambda r: p["epsilon"] * np.exp(-(r - p["delta"]) ** 2 / (2 * p["sigma"] ** 2))
    if name == "OPP":
        return lambda r: (p["C1"] * r ** -p["eta1"]
                          + p["C2"] * r ** -p["eta2"] * np.cos(p["k"] * r - p["phi"]))
    if name == "DPDConservative":
        rc = 2.5
        return lambda r: p["A"] * (rc - r) - p["A"] / (2 * rc) * (rc * rc - r * r)
    if name == "DLVO":
        k, Z, A, a1, a2 = (p[x] for x in ("kappa", "Z", "A", "a1", "a2"))
        rs, rd, rp = a1 + a2, a1 - a2, a1 * a2
        return lambda r: (rp / rs * Z * np.exp(-k * (r - rs)) - rp * A / 3 / (r * r - rs * rs)
                          - rp * A / 3 / (r * r - rd * rd)
                          - A / 6 * np.log((r * r - rs * rs) / (r * r - rd * rd)))
    if name == "Fourier":
        rc = 2.5
        a = [sum((-1) ** n * p["a"][n - 2] for n in range(2, 5))] + list(p["a"])
        b = [sum(n * (-1) ** n * p["b"][n - 2] for n in range(2, 5))] + list(p["b"])
        return lambda r: r ** -12 + sum(a[n - 1] * np.cos(n * np.pi * r / rc)
                                        + b[n - 1] * np.sin(n * np.pi * r / rc)
                                        for n in range(1, 5)) / r ** 2
    if name == "Moliere":
        Z, aF = p["qi"] * p["qj"], p["aF"]
        return lambda r: Z / r * (0.35 * np.exp(-0.3 * r / aF) + 0.55 * np.exp(-1.2 * r / aF)
                                  + 0.1 * np.exp(-6.0 * r / aF))
    if name == "ZBL":
        Z, aF = p["qi"] * p["qj"], p["aF"]
        return lambda r: Z / r * (0.1818 * np.exp(-3.2 * r / aF) + 0.5099 * np.exp(-0.9423 * r / aF)
                                  + 0.2802 * np.exp(-0.4029 * r / aF)
                                  + 0.02817 * np.exp(-0.2016 * r / aF))
    if name == "Ewald":
        from scipy.special import erfc
        k, a = p["kappa"], p.get("alpha", 0.0)
        return lambda r: 0.5 * (erfc(k * r + a / (2 * k)) * np.exp(a * r)
                                + erfc(k * r - a / (2 * k)) * np.exp(-a * r)) / r
    if name == "ReactionField":
        rc, erf = 2.5, p["eps_rf"]
        fac = (0.5 if erf == 0 else (erf - 1) / (2 * erf + 1)) / rc ** 3
        return lambda r: p["epsilon"] * (1 / r + fac * r * r)
    assert name == "TWF"
    return lambda r: (4 * p["epsilon"] / p["alpha"] ** 2
                      * (1 / ((r / p["sigma"]) ** 2 - 1) ** 6
                         - p["alpha"] / ((r / p["sigma"]) ** 2 - 1) ** 3))


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("mode", ["none", "shift"])
def test_many_particle_forces_vs_fp64(name, mode):
    """A jittered lattice (nearest neighbours at 1.07 - 1.17, clear of the TWF hard core) through
    the unfused kernel; per-particle forces and the total energy against an FP64 brute force."""
    if mode == "shift" and "shift" not in getattr(md.pair, name)._accepted_modes:
        pytest.skip(f"{name} does not accept mode 'shift'")
    p = dict(GOLD[name]["params"][1 if len(GOLD[name]["params"]) > 1 else 0])
    snap = workloads.lj_fluid_sc(8, density=0.7, jitter=0.05, seed=4)
    charged = name == "Ewald"
    if charged:
        snap.particles.charge[:] = np.random.default_rng(5).choice([-1.0, 0.5, 1.0],
                                                                  snap.particles.N)
    f = potential(name, p, mode=mode)
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1)
    sim.create_state_from_snapshot(snap)
    sim.operations.integrator = md.Integrator(
        dt=0.005, forces=[f], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    sim.run(0)
    pos = np.asarray(sim.state.get_snapshot().particles.position, np.float32).astype(np.float64)
    q = np.asarray(snap.particles.charge, np.float32).astype(np.float64) if charged else None
    L = snap.configuration.box[0]
    V = closed_form(name, p)
    N = len(pos)
    Fo = np.zeros((N, 3))
    Eo = 0.0
    rc = 2.5
    vshift = V(rc) if mode == "shift" else 0.0
    h = 1e-6
    for i in range(N):
        d = pos[i] - pos
        d -= L * np.rint(d / L)
        r = np.sqrt((d * d).sum(1))
        m = (r < rc) & (r > 0)
        rr = r[m]
        qq = q[i] * q[m] if charged else 1.0
        F = -(V(rr + h) - V(rr - h)) / (2 * h) * qq
        Fo[i] = ((F / rr)[:, None] * d[m]).sum(0)
        Eo += 0.5 * ((V(rr) - vshift) * qq).sum()
    Fg = f.forces
    scale = np.abs(Fo).max()
    assert np.all(np.abs(Fg - Fo) <= 1e-4 * np.abs(Fo) + 1e-5 * scale), name
    assert math.isclose(f.energy, Eo, rel_tol=1e-4, abs_tol=1e-5 * N), (f.energy, Eo)


def test_fused_nve_with_morse_conserves_energy():
    """One radial force alone runs on the fused graph path (pair kernel + step two + FP64 sums)."""
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=2)
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=2)
    sim.create_state_from_snapshot(snap)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), 0.5)
    f = potential("Morse", dict(D0=1.0, alpha=3.0, r0=1.1), mode="shift")
    sim.operations.integrator = md.Integrator(
        dt=0.002, forces=[f], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.run(20)
    e0 = thermo.kinetic_energy + thermo.potential_energy
    sim.run(1000)
    e1 = thermo.kinetic_energy + thermo.potential_energy
    assert abs(e1 - e0) / snap.particles.N < 1e-3


def test_reaction_field_with_charges_and_sort():
    """ReactionField with use_charge=True scales each pair by q_i q_j; the charges follow the
    particles through the Hilbert sort (a sorted run equals an unsorted one)."""
    snap = workloads.lj_fluid_sc(10, density=0.8, jitter=0.05, seed=8)
    rng = np.random.default_rng(3)
    snap.particles.charge[:] = rng.choice([-1.0, 1.0], snap.particles.N)
    p = dict(epsilon=0.3, eps_rf=2.0, use_charge=True)
    out = []
    for sorter in (None, 5):
        sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=2)
        sim.create_state_from_snapshot(snap)
        sim.state.thermalize_particle_momenta(hoomd.filter.All(), 1.0)
        f = md.pair.ReactionField(nlist=md.nlist.Cell(buffer=0.4), default_r_cut=2.5)
        f.params[("A", "A")] = p
        lj = md.pair.LJ(nlist=f.nlist, default_r_cut=2.5)
        lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
        sim.operations.integrator = md.Integrator(
            dt=0.004, forces=[lj, f], methods=[md.methods.ConstantVolume(hoomd.filter.All())])
        if sorter:
            sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=sorter))
        sim.run(0)
        if sorter is None:
            pos = np.asarray(sim.state.get_snapshot().particles.position, np.float32)
            pos = pos.astype(np.float64)
            L = snap.configuration.box[0]
            V = closed_form("ReactionField", p)
            q = snap.particles.charge
            E = 0.0
            for i in range(len(pos)):
                d = pos[i] - pos
                d -= L * np.rint(d / L)
                r = np.sqrt((d * d).sum(1))
                m = (r < 2.5) & (r > 0)
                E += 0.5 * (V(r[m]) * q[i] * q[m]).sum()
            assert math.isclose(f.energy, E, rel_tol=1e-4, abs_tol=1e-4)
        sim.run(20)
        out.append(sim.state.get_snapshot())
    a, b = out
    box = np.array(snap.configuration.box[:3])
    ua = a.particles.position + a.particles.image * box
    ub = b.particles.position + b.particles.image * box
    assert np.abs(ua - ub).max() < 1e-3
    assert np.array_equal(a.particles.charge, b.particles.charge)
