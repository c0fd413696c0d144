"""Pair forces (hoomd/md/pair/pair.py): ``Pair`` with ``LJ``, ``Table``, the other radial
potentials, DPD, and ``ExamplePair``, the evaluator of the reference's pair-plugin template
(example_plugins/pair_plugin/EvaluatorPairExample.h).

Attribute names, parameter keys, accepted modes and the per-particle outputs (``forces``,
``energies``, ``virials``, ``energy``) follow the reference. On attach each force looks up its
engine class as the reference does (hoomd/md/pair/pair.py:126-146): ``_ext_module`` (this
package's compiled module, or a plugin's own module) and ``_cpp_class_name`` + "GPU", constructed
from the state and the neighbour list; every type pair's parameters then go through the engine
object's ``setParams((a, b), dict)``, ``setRCut`` and ``setROn`` (PotentialPair<E>'s pybind
methods, hoomd/md/PotentialPair.h:1017-1036). A plugin's Python class declares its parameters
with ``hoomd_gb300.data.TypeParameter`` / ``TypeParameterDict`` and ``_add_typeparam``, as
example_plugins/pair_plugin/pair.py does.
"""

import numpy as np

from hoomd_gb300._native import _hoomd_gb300
from hoomd_gb300.md.data import TypePairDict, dict_validator, nonnegative_real
from hoomd_gb300.operation import AutotunedObject

_MODES = {"none": 0, "shift": 1, "xplor": 2}


class Pair(AutotunedObject):
    """Base pair force (hoomd/md/pair/pair.py:18-161)."""

    _accepted_modes = ("none", "shift", "xplor")
    _ext_module = _hoomd_gb300
    _cpp_class_name = None
    _loggables = {"energy": "scalar", "energies": "particle", "forces": "particle",
                  "torques": "particle", "virials": "particle", "additional_energy": "scalar",
                  "additional_virial": "sequence"}

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
        self.r_cut = TypePairDict(default=None if default_r_cut is None else float(default_r_cut),
                                  validator=nonnegative_real)
        self.r_on = TypePairDict(default=float(default_r_on), validator=nonnegative_real)
        if mode not in self._accepted_modes:
            raise ValueError(f"mode must be one of {self._accepted_modes}")
        self._mode = mode
        self.nlist = nlist
        self._cpp_obj = None
        self._simulation = None

    @property
    def mode(self):
        return self._mode

    @mode.setter
    def mode(self, m):
        if m not in self._accepted_modes:
            raise ValueError(f"mode must be one of {self._accepted_modes}")
        self._mode = m
        if self._cpp_obj is not None:
            self._cpp_obj.mode = m
            self._update_tail()

    def _tail_coefficients(self, state):
        """(energy, virial) tail-correction coefficients: the energy and each diagonal virial
        term are these over the volume. Forces without a tail correction have none."""
        return 0.0, 0.0

    def _update_tail(self):
        """Recompute the tail-correction coefficients from the attached state."""
        if self._cpp_obj is None:
            return
        e, w = self._tail_coefficients(self._simulation.state)
        self._cpp_obj.setTailCorrection(float(e), float(w))

    @property
    def additional_energy(self):
        """Energy not attributed to particles (the tail correction; hoomd/md/force.py:97)."""
        self._require_run()
        return self._cpp_obj.tailEnergy()

    @property
    def additional_virial(self):
        """Virial not attributed to particles, (xx, xy, xz, yy, yz, zz)."""
        self._require_run()
        w = self._cpp_obj.tailVirial()
        return [w, 0.0, 0.0, w, 0.0, w]

    def _add_typeparam(self, typeparam):
        """Expose a ``hoomd_gb300.data.TypeParameter`` as the attribute of its name (the
        reference's Operation._add_typeparam)."""
        setattr(self, typeparam.name, typeparam.make_container())

    def _cpp_params(self, value):
        """The dict handed to the engine object's setParams for one type pair."""
        return dict(value)

    def _attach(self, simulation, cpp_nlist):
        self._simulation = simulation
        self._standalone = False
        state = simulation.state
        cls = getattr(self._ext_module, self._cpp_class_name + "GPU")
        self._cpp_obj = cls(state._cpp_pdata, cpp_nlist)
        self._cpp_obj.mode = self._mode
        types = state.particle_types
        if self._cpp_obj.useCharge is False:
            self._cpp_obj.useCharge = bool(self._needs_charge(types))
        self._send_params()
        # parameters set after attaching reach the engine before the next step
        for d in (self.params, self.r_cut, self.r_on):
            if hasattr(d, "_on_change"):
                d._on_change = self._typeparam_changed
        return self._cpp_obj

    def _send_params(self):
        """Every type pair's parameters, r_cut and r_on to the engine object."""
        types = self._simulation.state.particle_types
        for i, a in enumerate(types):
            for j, b in enumerate(types):
                if j < i:
                    continue
                try:
                    value = self.params[(a, b)]
                except KeyError:
                    raise RuntimeError(f"{type(self).__name__}: params[({a!r}, {b!r})] is not set")
                self._cpp_obj.setParams((a, b), self._cpp_params(value))
                try:
                    rc = self.r_cut[(a, b)]
                except KeyError:
                    raise RuntimeError(f"{type(self).__name__}: r_cut[({a!r}, {b!r})] is not set")
                self._cpp_obj.setRCut((a, b), float(rc))
                self._cpp_obj.setROn((a, b), float(self.r_on[(a, b)]))
        self._update_tail()

    def _typeparam_changed(self, key):
        if self._cpp_obj is None:
            return
        try:
            self._send_params()
            self._pending = False
            # forces at the current positions are recomputed with the new values at the next run
            self._simulation._state_changed()
        except RuntimeError:
            self._pending = True  # other pairs still unset: sent, or reported, at the next run

    def _detach(self):
        self._cpp_obj = None

    def _needs_charge(self, types):
        """True when every pair is scaled by q_i q_j (the reference's needsCharge())."""
        return False

    def _require_run(self, virial=False):
        if self._cpp_obj is None or self._simulation is None:
            raise RuntimeError("forces are available after Simulation.run")
        self._simulation._attach()
        if getattr(self, "_standalone", False):
            # a compute, not held by an integrator: evaluate at the current positions
            self._cpp_obj.compute(bool(virial))

    @property
    def forces(self):
        """(N, 3) forces in tag order."""
        self._require_run()
        return self._cpp_obj.getForces()

    def compute_energy(self, tags1, tags2):
        """Energy between two sets of particles, U = sum over every tag in tags1 and every tag
        in tags2 of V_ij(r) (hoomd/md/pair/pair.py compute_energy, PotentialPair::
        computeEnergyBetweenSets): no exclusions apply, repeated tags count each time, and a tag
        in both lists is also paired with itself, as in the reference. Summed on the GPU."""
        if self._cpp_obj is None or self._simulation is None:
            raise RuntimeError("compute_energy is available after Simulation.run")
        self._simulation._attach()
        t1 = np.asarray(tags1, dtype=np.int64).ravel()
        t2 = np.asarray(tags2, dtype=np.int64).ravel()
        if (t1 < 0).any() or (t2 < 0).any():
            raise ValueError("compute_energy: tags are non-negative")
        return self._cpp_obj.computeEnergyBetweenSets(t1, t2)

    @property
    def torques(self):
        """(N, 3) torques: zero for these isotropic pair forces."""
        self._require_run()
        return np.zeros((self._simulation.state.N_particles, 3))

    @property
    def energies(self):
        """(N,) per-particle energies (half of each pair energy) in tag order."""
        self._require_run()
        return self._cpp_obj.getEnergies()

    @property
    def virials(self):
        """(N, 6) per-particle virials (xx, xy, xz, yy, yz, zz) in tag order."""
        self._require_run(virial=True)
        return self._cpp_obj.getVirials()

    @property
    def energy(self):
        """Total energy of this force: the additional energy plus the per-particle energies
        summed in FP64 on the device (ForceCompute::calcEnergySum)."""
        self._require_run()
        return self._cpp_obj.tailEnergy() + self._cpp_obj.energySum()


class LJ(Pair):
    """Lennard-Jones (hoomd/md/pair/pair.py:163-228); params: epsilon, sigma."""

    _cpp_class_name = "PotentialPairLJ"

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none',
                 tail_correction=False):
        super().__init__(nlist, default_r_cut, default_r_on, mode)
        self._tail_correction = bool(tail_correction)
        self.params = TypePairDict(validator=dict_validator(("epsilon", "sigma")))

    @property
    def tail_correction(self):
        """Whether the isotropic integrated long-range tail correction is applied."""
        return self._tail_correction

    @tail_correction.setter
    def tail_correction(self, value):
        self._tail_correction = bool(value)
        if self._cpp_obj is not None:
            self._cpp_obj.tail_correction = self._tail_correction
        self._update_tail()

    def _attach(self, simulation, cpp_nlist):
        obj = super()._attach(simulation, cpp_nlist)
        obj.tail_correction = self._tail_correction
        return obj

    def _tail_coefficients(self, state):
        """PotentialPair::computeTailCorrection (hoomd/md/PotentialPair.h:255-341) with the LJ
        integrals of EvaluatorPairLJ::evalEnergyLRCIntegral / evalPressureLRCIntegral
        (hoomd/md/EvaluatorPairLJ.h:213-248). Over the volume V: energy
        sum_ij 2 pi N_i (N_j / V) I_E, pressure sum_ij (4/6) pi (N_i / V)(N_j / V) I_P, and each
        diagonal virial term D V dP / 3."""
        if not self._tail_correction:
            return 0.0, 0.0
        if self._mode != "none":
            raise RuntimeError(
                'Pair potential shift mode must be "none" to apply tail corrections.')
        types, counts, dimensions = state.particle_types, state._type_counts(), state.dimensions
        e = w = 0.0
        for i, a in enumerate(types):
            for j, b in enumerate(types):
                rc = float(self.r_cut[(a, b)])
                if rc == 0.0:
                    continue
                p = self.params[(a, b)]
                lj1 = 4.0 * p["epsilon"] * p["sigma"] ** 12
                lj2 = 4.0 * p["epsilon"] * p["sigma"] ** 6
                rc3inv = 1.0 / (rc * rc) ** 1.5
                rc9inv = rc3inv ** 3
                i_e = lj1 / 9.0 * rc9inv - lj2 / 3.0 * rc3inv
                i_p = lj1 * 4.0 / 3.0 * rc9inv - lj2 * 2.0 * rc3inv
                e += 2.0 * np.pi * counts[i] * counts[j] * i_e
                w += dimensions / 3.0 * (4.0 / 6.0) * np.pi * counts[i] * counts[j] * i_p
        return e, w


class Table(Pair):
    """Tabulated potential (hoomd/md/pair/pair.py:520-619); params: r_min, U, F. Mode 'none'."""

    _cpp_class_name = "PotentialPairTable"
    _accepted_modes = ("none",)

    def __init__(self, nlist, default_r_cut=None):
        super().__init__(nlist, default_r_cut=default_r_cut, default_r_on=0, mode='none')
        self.params = TypePairDict(validator=dict_validator(("r_min", "U", "F"),
                                                            arrays=("U", "F")))

    def _cpp_params(self, v):
        U = np.asarray(v["U"], np.float64)
        F = np.asarray(v["F"], np.float64)
        if U.shape != F.shape or U.ndim != 1:
            raise RuntimeError("The length of V and F arrays must be equal.")
        if len(U) == 0:
            raise RuntimeError("The length of V and F must not be zero.")
        return dict(r_min=float(v["r_min"]), U=U, F=F)


class ExamplePair(Pair):
    """The reference's pair-plugin example evaluator: V = k/2 (sigma - r)^2 inside r_cut
    (example_plugins/pair_plugin/pair.py:15-28); params: k, sigma."""

    _cpp_class_name = "PotentialPairExample"

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
        super().__init__(nlist, default_r_cut, default_r_on, mode)
        self.params = TypePairDict(validator=dict_validator(("k", "sigma")))


class TableSurrogate(Pair):
    """Radial MLP stand-in for a multi-type ``Table`` (the reference has no counterpart; it
    replaces hoomd/md/EvaluatorPairTable.h's spline gathers). ``surrogate`` is a trained
    :class:`hoomd_gb300.surrogate.Surrogate`; its r_cut applies to every type pair and pairs
    closer than its r_min feel no force, as in ``Table``. Mode 'none', no virials. On attach the
    force becomes a PotentialPairGPU of kind MLP (gb_mlp_forces in include/hoomd_gb300.h)."""

    _accepted_modes = ("none",)

    def __init__(self, nlist, surrogate):
        super().__init__(nlist, default_r_cut=surrogate.r_cut, default_r_on=0, mode='none')
        self.surrogate = surrogate

    def _attach(self, simulation, cpp_nlist):
        self._simulation = simulation
        self._standalone = False
        state = simulation.state
        ntypes = len(state.particle_types)
        if ntypes != self.surrogate.ntypes:
            raise RuntimeError(f"the surrogate was trained for {self.surrogate.ntypes} types, "
                               f"the state has {ntypes}")
        self._cpp_obj = _hoomd_gb300.PotentialPairGPU(state._cpp_pdata, cpp_nlist,
                                                      _hoomd_gb300.PairKind.MLP)
        self._cpp_obj.setSurrogate(self.surrogate._cpp)
        for i in range(ntypes):
            for j in range(i, ntypes):
                self._cpp_obj.setRCut(i, j, float(self.surrogate.r_cut))
        return self._cpp_obj

    @property
    def virials(self):
        raise RuntimeError("TableSurrogate does not compute virials")


class _Radial(Pair):
    """The reference's other radial pair potentials, one GPU kernel family (``gb_pair_forces_radial``
    in include/hoomd_gb300.h selects the closed form by kind). Parameter keys and modes follow
    hoomd.md.pair."""

    _keys = ()

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
        super().__init__(nlist, default_r_cut, default_r_on, mode)
        self.params = TypePairDict(validator=dict_validator(self._keys))


# the reference's engine class of each radial potential (hoomd/md/pair/pair.py _cpp_class_name)
_CPP_NAMES = {"Gaussian": "PotentialPairGauss", "DPDConservative": "PotentialPairConservativeDPD"}


def _radial(name, kind, keys, doc, modes=("none", "shift", "xplor")):
    cls = type(name, (_Radial,), {"_radial_kind": kind, "_keys": tuple(keys),
                                  "_accepted_modes": modes, "__doc__": doc,
                                  "_cpp_class_name": _CPP_NAMES.get(name,
                                                                    "PotentialPair" + name)})
    cls.__module__ = __name__
    return cls


Gaussian = _radial("Gaussian", 0, ("epsilon", "sigma"),
                   "Gaussian (hoomd/md/pair/pair.py, EvaluatorPairGauss.h): eps exp(-r^2/2 sigma^2).")
Yukawa = _radial("Yukawa", 1, ("epsilon", "kappa"),
                 "Yukawa (EvaluatorPairYukawa.h): eps exp(-kappa r)/r.")
Morse = _radial("Morse", 2, ("D0", "alpha", "r0"),
                "Morse (EvaluatorPairMorse.h): D0 [e^(-2 alpha (r-r0)) - 2 e^(-alpha (r-r0))].")
ForceShiftedLJ = _radial("ForceShiftedLJ", 3, ("sigma", "epsilon"),
                         "Force-shifted LJ (EvaluatorPairForceShiftedLJ.h).", ("none",))
Mie = _radial("Mie", 4, ("epsilon", "sigma", "n", "m"), "Mie n-m (EvaluatorPairMie.h).")
ExpandedMie = _radial("ExpandedMie", 5, ("epsilon", "sigma", "n", "m", "delta"),
                      "Mie at r - delta (EvaluatorPairExpandedMie.h).")
ExpandedLJ = _radial("ExpandedLJ", 6, ("sigma", "epsilon", "delta"),
                     "LJ at r - delta (EvaluatorPairExpandedLJ.h).")
Buckingham = _radial("Buckingham", 7, ("A", "rho", "C"),
                     "Buckingham (EvaluatorPairBuckingham.h): A exp(-r/rho) - C/r^6.")
LJ1208 = _radial("LJ1208", 8, ("sigma", "epsilon"), "12-8 Lennard-Jones (EvaluatorPairLJ1208.h).")
LJ0804 = _radial("LJ0804", 9, ("sigma", "epsilon"), "8-4 Lennard-Jones (EvaluatorPairLJ0804.h).")
LJGauss = _radial("LJGauss", 10, ("epsilon", "sigma", "r0"),
                  "Lennard-Jones-Gauss (EvaluatorPairLJGauss.h).")
ExpandedGaussian = _radial("ExpandedGaussian", 11, ("epsilon", "sigma", "delta"),
                           "Gaussian at r - delta (EvaluatorPairExpandedGaussian.h).")
OPP = _radial("OPP", 12, ("C1", "C2", "eta1", "eta2", "k", "phi"),
              "Oscillating pair potential (EvaluatorPairOPP.h).")
TWF = _radial("TWF", 13, ("sigma", "epsilon", "alpha"),
              "Ten Wolde-Frenkel (EvaluatorPairTWF.h); infinite for r <= sigma.")
DPDConservative = _radial("DPDConservative", 14, ("A",),
                          "Conservative DPD force (EvaluatorPairDPDThermoDPD.h): "
                          "A (r_c - r) - A (r_c^2 - r^2) / (2 r_c).", ("none",))
DLVO = _radial("DLVO", 15, ("kappa", "Z", "A", "a1", "a2"),
               "DLVO colloid force (EvaluatorPairDLVO.h): screened repulsion and sphere-sphere "
               "van der Waals attraction of radii a1, a2.", ("none", "shift"))
Moliere = _radial("Moliere", 17, ("qi", "qj", "aF"),
                  "Moliere screened Coulomb (EvaluatorPairMoliere.h).")
ZBL = _radial("ZBL", 18, ("qi", "qj", "aF"),
              "Ziegler-Biersack-Littmark screened Coulomb (EvaluatorPairZBL.h).", ("none",))


class Fourier(_Radial):
    """Fourier pair force (EvaluatorPairFourier.h): 1/r^12 + sum over n = 1..4 of
    [a_n cos(n pi r / r_c) + b_n sin(n pi r / r_c)] / r^2, with ``a`` and ``b`` the three
    coefficients of n = 2, 3, 4 (those of n = 1 make the force and energy vanish at r_c)."""

    _radial_kind = 16
    _cpp_class_name = "PotentialPairFourier"
    _accepted_modes = ("none", "xplor")

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
        super().__init__(nlist, default_r_cut, default_r_on, mode)
        self.params = TypePairDict(validator=dict_validator(("a", "b"), arrays=("a", "b")))


class ReactionField(_Radial):
    """Reaction-field electrostatics (EvaluatorPairReactionField.h):
    eps [1/r + (eps_rf - 1)/(2 eps_rf + 1) r^2 / r_c^3], times q_i q_j with ``use_charge=True``;
    eps_rf = 0 stands for an infinite dielectric. ``use_charge`` must be the same for every type
    pair (one kernel instantiation scales all pairs or none)."""

    _radial_kind = 19
    _cpp_class_name = "PotentialPairReactionField"

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
        super().__init__(nlist, default_r_cut, default_r_on, mode)
        self.params = TypePairDict(validator=dict_validator(("epsilon", "eps_rf"),
                                                            optional={"use_charge": False}))

    def _needs_charge(self, types):
        flags = {bool(self.params[(a, b)].get("use_charge")) for a in types for b in types}
        if len(flags) > 1:
            raise NotImplementedError("ReactionField: use_charge must be the same for every "
                                      "type pair")
        return flags.pop()


class Ewald(_Radial):
    """Real-space part of the Ewald sum (EvaluatorPairEwald.h): q_i q_j [erfc(kappa r +
    alpha / 2 kappa) e^{alpha r} + erfc(kappa r - alpha / 2 kappa) e^{-alpha r}] / 2r; alpha = 0
    is the plain erfc(kappa r) / r. Reads the particle charges."""

    _radial_kind = 20
    _cpp_class_name = "PotentialPairEwald"
    _keys = ("kappa", "alpha")
    _accepted_modes = ("none",)

    def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
        super().__init__(nlist, default_r_cut, default_r_on, mode)
        self.params = TypePairDict(validator=dict_validator(("kappa",), optional={"alpha": 0.0}))

    def _needs_charge(self, types):
        return True


class _DPDBase(Pair):
    """DPD thermostat pair forces (hoomd/md/pair/pair.py DPD, DPDLJ; PotentialPairDPDThermo):
    a conservative force plus the drag and random forces of the DPD thermostat at ``kT``, whose
    random numbers come from both particles' tags and the timestep. They read the velocities, so
    the integrator runs them on its unfused path."""


    def __init__(self, nlist, kT, default_r_cut=None, mode='none'):
        super().__init__(nlist, default_r_cut, 0.0, mode)
        self._kT = float(kT)

    @property
    def kT(self):
        return self._kT

    @kT.setter
    def kT(self, v):
        self._kT = float(v)
        if self._cpp_obj is not None:
            self._cpp_obj.dpdKT = self._kT

    def _attach(self, simulation, cpp_nlist):
        obj = super()._attach(simulation, cpp_nlist)
        obj.dpdKT = self._kT
        return obj


class DPD(_DPDBase):
    """DPD (EvaluatorPairDPDThermoDPD.h): conservative force A (1 - r/r_c), drag
    -gamma w^2 (r . v) / r and random force sqrt(6 gamma kT / dt) w alpha, w = 1 - r/r_c."""

    _cpp_class_name = "PotentialPairDPDThermoDPD"
    _accepted_modes = ("none",)

    def __init__(self, nlist, kT, default_r_cut=None):
        super().__init__(nlist, kT, default_r_cut, 'none')
        self.params = TypePairDict(validator=dict_validator(("A", "gamma")))


class DPDLJ(_DPDBase):
    """DPD thermostat with a Lennard-Jones conservative force (EvaluatorPairDPDThermoLJ.h)."""

    _cpp_class_name = "PotentialPairDPDThermoLJ"
    _accepted_modes = ("none", "shift")

    def __init__(self, nlist, kT, default_r_cut=None, mode='none'):
        super().__init__(nlist, kT, default_r_cut, mode)
        self.params = TypePairDict(validator=dict_validator(("epsilon", "sigma", "gamma")))
