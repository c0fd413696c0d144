"""Integration methods (hoomd/md/methods/methods.py): ConstantVolume (NVE without a thermostat, NVT
with one), ConstantPressure, DisplacementCapped, Langevin, Brownian and OverdampedViscous, each over
the group of
all particles."""

from hoomd_gb300.filter import All
from hoomd_gb300.md.data import TypeDict, nonnegative_real
from hoomd_gb300.md.methods import thermostats  # noqa: F401


class Method:
    _loggables = {}


class ConstantVolume(Method):
    def __init__(self, filter, thermostat=None):
        if not isinstance(filter, All):
            raise NotImplementedError("ConstantVolume integrates the group of all particles")
        self.filter = filter
        self._thermostat = thermostat
        self._cpp_integ = None

    @property
    def thermostat(self):
        return self._thermostat

    @thermostat.setter
    def thermostat(self, t):
        self._thermostat = t
        if self._cpp_integ is not None:
            self._apply(self._cpp_integ)

    def _apply(self, integ):
        if self._thermostat is None:
            integ.setNoThermostat()
        else:
            self._thermostat._apply(integ)

    def _attach(self, integ, state=None):
        self._cpp_integ = integ
        if self._thermostat is not None and state is not None:
            self._thermostat._simulation = state._simulation
        self._apply(integ)


class NVE(ConstantVolume):
    """The reference's legacy NVE alias: ConstantVolume without a thermostat."""

    def __init__(self, filter):
        super().__init__(filter, thermostat=None)


def _gamma_r(v):
    v = tuple(float(x) for x in v)
    if len(v) != 3 or min(v) < 0:
        raise ValueError("gamma_r is three non-negative numbers")
    return v


class Langevin(Method):
    """Langevin dynamics (hoomd/md/methods/methods.py:637-833, hoomd/md/TwoStepLangevin.cc).

    Translational degrees of freedom only: drag ``gamma[type]`` and a uniform random force of
    variance 2 kT gamma / dt per direction, velocity-Verlet halves in the reference's order. The
    random numbers follow the reference's streams (Philox, Seed(25, timestep, seed), Counter(tag)),
    so a trajectory is a function of the seed and the initial state. ``kT`` is a constant.
    ``gamma_r`` is accepted for the rotational degrees of freedom, which this path does not
    integrate. ``reservoir_energy`` is tallied with ``tally_reservoir_energy=True``.
    """

    _loggables = {"reservoir_energy": "scalar"}

    def __init__(self, filter, kT, tally_reservoir_energy=False, default_gamma=1.0,
                 default_gamma_r=(1.0, 1.0, 1.0)):
        if not isinstance(filter, All):
            raise NotImplementedError("Langevin integrates the group of all particles")
        self.filter = filter
        self._kT = float(kT)
        self._tally = bool(tally_reservoir_energy)
        self.gamma = TypeDict(default=float(default_gamma), validator=nonnegative_real)
        self.gamma_r = TypeDict(default=_gamma_r(default_gamma_r), validator=_gamma_r)
        self.gamma._on_change = self.gamma_r._on_change = lambda key: self._reapply()
        self._cpp_integ = None
        self._types = None

    @property
    def kT(self):
        return self._kT

    @kT.setter
    def kT(self, v):
        self._kT = float(v)
        self._reapply()

    @property
    def tally_reservoir_energy(self):
        return self._tally

    @tally_reservoir_energy.setter
    def tally_reservoir_energy(self, v):
        self._tally = bool(v)
        self._reapply()

    @property
    def reservoir_energy(self):
        if self._cpp_integ is None:
            raise RuntimeError("reservoir_energy is available after the simulation runs")
        return self._cpp_integ.reservoir_energy

    def _reapply(self):
        if self._cpp_integ is not None:
            self._apply(self._cpp_integ)

    def _apply(self, integ):
        gam = [float(self.gamma[t]) for t in self._types]
        integ.setLangevin(self._kT, gam, self._tally)

    def _attach(self, integ, state=None):
        self._types = list(state.particle_types)
        self._cpp_integ = integ
        self._apply(integ)


class DisplacementCapped(ConstantVolume):
    """ConstantVolume without a thermostat whose step one caps each particle's displacement at
    ``maximum_displacement`` (hoomd/md/methods/methods.py:583-635, TwoStepConstantVolume.cc:44-52);
    a constant here."""

    def __init__(self, filter, maximum_displacement):
        super().__init__(filter, thermostat=None)
        self._max = float(maximum_displacement)

    @property
    def maximum_displacement(self):
        return self._max

    @maximum_displacement.setter
    def maximum_displacement(self, v):
        self._max = float(v)
        if self._cpp_integ is not None:
            self._cpp_integ.setMaxDisplacement(self._max)

    def _apply(self, integ):
        super()._apply(integ)
        integ.setMaxDisplacement(self._max)


class Brownian(Method):
    """Brownian dynamics (hoomd/md/methods/methods.py:835-1023, hoomd/md/TwoStepBD.cc): each step
    x += (F + F_r) dt / gamma with a uniform random force of variance 2 kT gamma / dt per
    direction, and velocities drawn from the Maxwell-Boltzmann distribution at kT (they carry
    no dynamics). The random numbers follow the reference's stream (Seed(24, timestep, seed),
    Counter(tag)). Translational degrees of freedom only; ``kT`` is a constant."""

    _noiseless = False

    def __init__(self, filter, kT, default_gamma=1.0, default_gamma_r=(1.0, 1.0, 1.0)):
        if not isinstance(filter, All):
            raise NotImplementedError(f"{type(self).__name__} integrates the group of all "
                                      "particles")
        self.filter = filter
        self._kT = float(kT)
        self.gamma = TypeDict(default=float(default_gamma), validator=nonnegative_real)
        self.gamma_r = TypeDict(default=_gamma_r(default_gamma_r), validator=_gamma_r)
        self.gamma._on_change = self.gamma_r._on_change = lambda key: self._reapply()
        self._cpp_integ = None
        self._types = None

    @property
    def kT(self):
        return self._kT

    @kT.setter
    def kT(self, v):
        self._kT = float(v)
        self._reapply()

    def _reapply(self):
        if self._cpp_integ is not None:
            self._apply(self._cpp_integ)

    def _apply(self, integ):
        integ.setBrownian(self._kT, [float(self.gamma[t]) for t in self._types],
                          self._noiseless)

    def _attach(self, integ, state=None):
        self._types = list(state.particle_types)
        self._cpp_integ = integ
        self._apply(integ)


class OverdampedViscous(Brownian):
    """Overdamped viscous dynamics (hoomd/md/methods/methods.py:1025-1160): Brownian dynamics
    without the random force, x += F dt / gamma and v = F / gamma."""

    _noiseless = True

    def __init__(self, filter, default_gamma=1.0, default_gamma_r=(1.0, 1.0, 1.0)):
        super().__init__(filter, 0.0, default_gamma, default_gamma_r)


_COUPLE = {"none": 0, "xy": 1, "xz": 2, "yz": 3, "xyz": 4}


class ConstantPressure(Method):
    """Constant pressure (hoomd/md/methods/methods.py:177-580, TwoStepConstantPressure.cc): the
    MTK barostat with box degrees of freedom ``box_dof`` = (x, y, z, xy, xz, yz), couplings
    ``couple`` ("xyz", "xy", "xz", "yz", "none"), time constant ``tauS`` and Langevin damping
    ``gamma`` of the barostat, with the MTTK thermostat or none. ``S`` is the target stress: one
    number (hydrostatic pressure) or six (xx, yy, zz, yz, xz, xy), constants here. Translational
    degrees of freedom only; ``rescale_all`` has no effect (the group is all particles)."""

    _loggables = {"barostat_energy": "scalar"}

    def __init__(self, filter, S, tauS, couple, thermostat=None,
                 box_dof=(True, True, True, False, False, False), rescale_all=False, gamma=0.0):
        if not isinstance(filter, All):
            raise NotImplementedError("ConstantPressure integrates the group of all particles")
        if thermostat is not None and not isinstance(thermostat, thermostats.MTTK):
            raise NotImplementedError("ConstantPressure runs with the MTTK thermostat or none")
        if couple not in _COUPLE:
            raise ValueError(f"couple must be one of {tuple(_COUPLE)}")
        self.filter = filter
        self.S = S
        self.tauS = float(tauS)
        self.couple = couple
        self.thermostat = thermostat
        self.box_dof = [bool(x) for x in box_dof]
        if len(self.box_dof) != 6:
            raise ValueError("box_dof has six entries")
        self.rescale_all = bool(rescale_all)
        self.gamma = float(gamma)
        self._barostat_dof = (0.0,) * 6
        self._cpp_integ = None

    @staticmethod
    def _stress(S):
        try:
            v = [float(x) for x in S]
        except TypeError:
            v = [float(S)] * 3 + [0.0] * 3
        if len(v) != 6:
            raise ValueError("S is one number or six")
        return v

    @property
    def barostat_dof(self):
        if self._cpp_integ is None:
            return self._barostat_dof
        return tuple(self._cpp_integ.getBarostatDOF())

    @barostat_dof.setter
    def barostat_dof(self, v):
        v = tuple(float(x) for x in v)
        if len(v) != 6:
            raise ValueError("barostat_dof has six entries")
        self._barostat_dof = v
        if self._cpp_integ is not None:
            self._cpp_integ.setBarostatDOF(list(v))

    @property
    def barostat_energy(self):
        if self._cpp_integ is None:
            raise RuntimeError("barostat_energy is available after the simulation runs")
        return self._cpp_integ.barostatEnergy()

    def thermalize_barostat_dof(self):
        raise NotImplementedError("thermalize_barostat_dof is not available on this path")

    def _apply(self, integ):
        if self.thermostat is None:
            integ.setNoThermostat()
        else:
            self.thermostat._apply(integ)
        integ.setNPT(self._stress(self.S), self.tauS, _COUPLE[self.couple],
                     [int(x) for x in self.box_dof], self.gamma)
        integ.setBarostatDOF(list(self._barostat_dof))

    def _attach(self, integ, state=None):
        if self._cpp_integ is not None and self._cpp_integ is not integ:
            self._barostat_dof = tuple(self._cpp_integ.getBarostatDOF())
        self._cpp_integ = integ
        if self.thermostat is not None and state is not None:
            self.thermostat._simulation = state._simulation
        self._apply(integ)
