"""Generate the golden fixtures in tests/golden/ from the reference (run where the HOOMD-blue
source tree is present; the fixtures are committed so that test hosts never need that tree).

Outputs
-------
forces_and_energies_lj_table.json, forces_and_energies_radial.json
    The ``LJ`` and ``Table`` entries (and, in the second file, those of the fourteen radial
    potentials of ``RADIAL``) of the reference's Mathematica-computed fixture
    ``hoomd/md/pytest/forces_and_energies.json`` (force and energy of two particles at
    r = 0.75 and 1.5, r_cut = 2.5), used by the reference's ``test_force_energy_accuracy``
    (``hoomd/md/pytest/test_potential.py:952-1058``).
true_pair_list_sc7.json
    The reference's ``hoomd/md/pytest/true_pair_list.json``: the 1029 unordered tag pairs of a
    7x7x7 simple-cubic lattice (a = 1) within r_cut = 1.1, buffer 0
    (``hoomd/md/pytest/test_nlist.py:221-372``).
ref_vectors.npz
    Outputs of the reference's own header-only maths, compiled unmodified at FP32 and FP64
    (oracle/_ref, see oracle/build.py), on seeded random inputs: EvaluatorPairLJ,
    EvaluatorPairTable, EvaluatorPairExample, BoxDim::minImage / wrap / makeFraction /
    getNearestPlaneDistance.

Usage: ``python tests/golden/make_golden.py`` (after ``python oracle/build.py``).
"""

import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from oracle import build as obuild  # noqa: E402
from oracle import refshim  # noqa: E402

REF = obuild.REF_ROOT

LJ_CASES = [  # (sigma, epsilon, r_cut, shift)
    (1.0, 1.0, 2.5, 0), (1.0, 1.0, 2.5, 1), (0.5, 0.0005, 2.5, 0), (1.5, 0.0015, 2.5, 1),
    (0.8, 1.5, 2.0, 0), (0.88, 0.5, 2.2, 1), (1.0, 0.0, 2.5, 0),
]
EXAMPLE_CASES = [(k, s, s, shift) for k in (0.5, 2.0, 5.0) for s in (0.5, 1.0, 1.5)
                 for shift in (0, 1)]
BOXES = [  # (box6, periodic)
    ((16.957, 16.957, 16.957, 0, 0, 0), (1, 1, 1)),
    ((10.0, 12.0, 15.0, 0, 0, 0), (1, 1, 1)),
    ((10.0, 11.0, 12.0, 0.3, -0.2, 0.1), (1, 1, 1)),
    ((9.0, 9.5, 10.0, 0, 0, 0), (1, 0, 1)),
]


def c5_table(rng, r_min=0.8, r_cut=3.0, width=1000):
    """One C5-style table: LJ + Yukawa + Gaussian with F = -dU/dr analytic."""
    r = np.linspace(r_min, r_cut, width, endpoint=False)
    eps, sig = rng.uniform(0.5, 1.5), rng.uniform(0.8, 1.2)
    A, kappa = rng.uniform(-2, 2), rng.uniform(0.5, 3)
    G, w = rng.uniform(0, 2), rng.uniform(0.1, 0.4)
    sr6 = (sig / r) ** 6
    U = 4 * eps * (sr6 * sr6 - sr6) + A * np.exp(-kappa * r) / r + G * np.exp(-0.5 * (r / w) ** 2)
    F = (4 * eps * (12 * sr6 * sr6 - 6 * sr6) / r + A * np.exp(-kappa * r) * (kappa * r + 1) / r**2
         + G * np.exp(-0.5 * (r / w) ** 2) * r / w**2)
    return U, F


def table_index_safe_f32(rsq, rcutsq, rmin, width):
    """True where the FP32 reference evaluation stays inside the table (value_i < width)."""
    f = np.float32
    r = np.sqrt(f(rsq))
    rcut = np.sqrt(f(rcutsq))
    dr = (rcut - f(rmin)) / f(width)
    vf = (r - f(rmin)) / dr
    inside = (f(rsq) < f(rcutsq)) & (r >= f(rmin))
    return ~inside | (np.floor(vf) < width)


# the radial potentials served by gb_pair_forces_radial
RADIAL = ("Gaussian", "Yukawa", "Morse", "ForceShiftedLJ", "Mie", "ExpandedMie", "ExpandedLJ",
          "Buckingham", "LJ1208", "LJ0804", "LJGauss", "ExpandedGaussian", "OPP", "TWF",
          "DPDConservative", "DLVO", "Fourier", "Moliere", "ZBL", "ReactionField", "Ewald")


def main():
    if not obuild.ref_available():
        raise SystemExit("reference source tree not found")
    obuild.build_ref()
    assert refshim.available()
    rng = np.random.default_rng(20261204)

    fe = json.load(open(REF / "hoomd/md/pytest/forces_and_energies.json"))
    out = {k: fe[k] for k in ("LJ", "Table")}
    out["_source"] = "hoomd/md/pytest/forces_and_energies.json (LJ, Table entries)"
    json.dump(out, open(HERE / "forces_and_energies_lj_table.json", "w"), indent=1)
    out = {k: fe[k] for k in RADIAL}
    out["_source"] = "hoomd/md/pytest/forces_and_energies.json (" + ", ".join(RADIAL) + ")"
    json.dump(out, open(HERE / "forces_and_energies_radial.json", "w"), indent=1)

    pairs = json.load(open(REF / "hoomd/md/pytest/true_pair_list.json"))
    json.dump(pairs, open(HERE / "true_pair_list_sc7.json", "w"))

    z = {}
    # LJ
    for c, (sigma, eps, rcut, shift) in enumerate(LJ_CASES):
        rsq = rng.uniform((0.6 * sigma) ** 2, (1.2 * rcut) ** 2, 256)
        rsq[:4] = [rcut * rcut, np.nextafter(rcut * rcut, 0), (0.75) ** 2, 1.5**2]
        z[f"lj{c}_case"] = np.array([sigma, eps, rcut * rcut, shift])
        z[f"lj{c}_rsq"] = rsq
        for prec in (32, 64):
            f, e, ok = refshim.lj_eval(rsq, rcut * rcut, sigma, eps, bool(shift), prec)
            z[f"lj{c}_f{prec}"], z[f"lj{c}_e{prec}"], z[f"lj{c}_ok{prec}"] = f, e, ok
            z[f"lj{c}_lrc{prec}"] = refshim.lj_lrc(rcut * rcut, sigma, eps, prec)
    # Table: the three fixture tables plus two C5-style random tables
    tables = [(p["r_min"], np.array(p["U"]), np.array(p["F"]), 2.5) for p in fe["Table"]["params"]]
    for _ in range(2):
        U, F = c5_table(rng)
        tables.append((0.8, U, F, 3.0))
    for c, (rmin, U, F, rcut) in enumerate(tables):
        width = len(U)
        rsq = rng.uniform((0.9 * rmin) ** 2, (1.05 * rcut) ** 2, 512)
        dr = (rcut - rmin) / width
        edges = [rmin**2, (rmin + 0.5 * dr) ** 2, (rcut - 0.5 * dr) ** 2, rcut**2,
                 np.nextafter(rmin**2, 0), 0.75**2, 1.5**2]
        rsq[: len(edges)] = edges
        safe = table_index_safe_f32(rsq, rcut * rcut, rmin, width)
        rsq = rsq[safe]
        z[f"tab{c}_case"] = np.array([rmin, rcut * rcut, width])
        z[f"tab{c}_U"], z[f"tab{c}_F"], z[f"tab{c}_rsq"] = U, F, rsq
        for prec in (32, 64):
            f, e, ok = refshim.table_eval(rsq, rcut * rcut, rmin, U, F, prec)
            z[f"tab{c}_f{prec}"], z[f"tab{c}_e{prec}"], z[f"tab{c}_ok{prec}"] = f, e, ok
    # Example plugin evaluator
    for c, (k, sigma, rcut, shift) in enumerate(EXAMPLE_CASES):
        rsq = rng.uniform(0.05**2, (1.2 * rcut) ** 2, 64)
        z[f"ex{c}_case"] = np.array([k, sigma, rcut * rcut, shift])
        z[f"ex{c}_rsq"] = rsq
        for prec in (32, 64):
            f, e, ok = refshim.example_eval(rsq, rcut * rcut, k, sigma, bool(shift), prec)
            z[f"ex{c}_f{prec}"], z[f"ex{c}_e{prec}"], z[f"ex{c}_ok{prec}"] = f, e, ok
    # Geometry
    for c, (b6, per) in enumerate(BOXES):
        L = np.array(b6[:3])
        z[f"box{c}_b6"], z[f"box{c}_per"] = np.array(b6), np.array(per)
        v = rng.uniform(-0.95, 0.95, (256, 3)) * L
        z[f"box{c}_mi_in"] = v
        x = rng.uniform(-0.6, 0.6, (256, 3)) * L
        img = rng.integers(-3, 4, (256, 3)).astype(np.int32)
        z[f"box{c}_wrap_in"], z[f"box{c}_wrap_img"] = x, img
        q = rng.uniform(-0.5, 0.5, (256, 3)) * L
        z[f"box{c}_frac_in"] = q
        for prec in (32, 64):
            # vectors rounded to the working precision first, as a HOOMD build would hold them
            R = np.float32 if prec == 32 else np.float64
            z[f"box{c}_mi{prec}"] = refshim.min_image(v.astype(R), b6, prec, per)
            wv, wi = refshim.wrap(x.astype(R), img, b6, prec, per)
            z[f"box{c}_wrap{prec}"], z[f"box{c}_wrapimg{prec}"] = wv, wi
            z[f"box{c}_frac{prec}"] = refshim.make_fraction(q.astype(R), b6, prec, per)
            z[f"box{c}_npd{prec}"] = refshim.nearest_plane_distance(b6, prec, per)
    np.savez_compressed(HERE / "ref_vectors.npz", **z)
    print("wrote", sorted(p.name for p in HERE.iterdir()))


if __name__ == "__main__":
    main()
