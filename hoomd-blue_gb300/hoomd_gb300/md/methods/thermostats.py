"""Thermostats of ConstantVolume (hoomd/md/methods/thermostats.py, hoomd/md/Thermostat.h).

* ``Bussi``: stochastic velocity rescaling; the factor is drawn on the GPU each step (Philox key
  Seed(45, timestep, seed), counter = tag of the first member) from the FP64 kinetic energy.
* ``Berendsen``: rescaling by sqrt(1 + dt/tau (kT/T - 1)) at step one, from the kinetic
  temperature at the start of the step.
* ``MTTK``: the Nose-Hoover chain of length one of Martyna, Tuckerman, Tobias and Klein; both
  halves scale by exp(-xi dt/2), and (xi, eta) advance on the GPU after step one from the
  half-step kinetic temperature.

All thermostat arithmetic is FP64 on the device; nothing leaves the GPU inside a run.
"""


class Thermostat:
    _loggables = {}

    def __init__(self, kT):
        self.kT = float(kT)
        self._cpp = None


class Bussi(Thermostat):
    def __init__(self, kT, tau=0.0):
        super().__init__(kT)
        self.tau = float(tau)

    def _apply(self, integ):
        self._cpp = integ
        integ.setBussi(self.kT, self.tau)


class Berendsen(Thermostat):
    def __init__(self, kT, tau):
        super().__init__(kT)
        self.tau = float(tau)
        if self.tau <= 0:
            raise ValueError("tau must be positive")

    def _apply(self, integ):
        self._cpp = integ
        integ.setBerendsen(self.kT, self.tau)


class MTTK(Thermostat):
    """hoomd.md.methods.thermostats.MTTK(kT, tau): ``translational_dof`` is the thermostat's
    (xi, eta); ``energy`` its contribution to the conserved quantity; ``thermalize_dof()`` draws
    xi from its equilibrium distribution (hoomd/md/Thermostat.h:273-300)."""

    _loggables = {"energy": "scalar"}

    def __init__(self, kT, tau):
        super().__init__(kT)
        self.tau = float(tau)
        if self.tau <= 0:
            raise ValueError("tau must be positive")
        self._state = (0.0, 0.0)
        self._simulation = None

    def _apply(self, integ):
        if self._cpp is not None and self._cpp is not integ:
            self._state = tuple(self._cpp.getMTTKState())  # carry (xi, eta) to a new integrator
        self._cpp = integ
        integ.setMTTK(self.kT, self.tau)
        integ.setMTTKState(*self._state)

    @property
    def translational_dof(self):
        if self._cpp is None:
            return self._state
        return tuple(self._cpp.getMTTKState())

    @translational_dof.setter
    def translational_dof(self, v):
        xi, eta = (float(x) for x in v)
        self._state = (xi, eta)
        if self._cpp is not None:
            self._cpp.setMTTKState(xi, eta)

    @property
    def rotational_dof(self):
        return (0.0, 0.0)

    @property
    def energy(self):
        if self._cpp is None:
            raise RuntimeError("the thermostat energy is available after the simulation runs")
        return self._cpp.mttkEnergy()

    def thermalize_dof(self):
        if self._cpp is None or self._simulation is None:
            raise RuntimeError("call thermalize_dof after the simulation has run")
        self._cpp.thermalizeMTTK(self._simulation.timestep)
        self._state = tuple(self._cpp.getMTTKState())
