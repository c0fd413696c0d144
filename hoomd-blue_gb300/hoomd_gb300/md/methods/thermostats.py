"""Thermostats (hoomd/md/methods/thermostats.py:244-333): Bussi stochastic velocity rescaling.
The rescale factor is drawn on the GPU each step (Philox key Seed(45, timestep, seed), counter =
tag of the first member), from the FP64 kinetic energy reduced on the GPU."""


class Thermostat:
    pass


class Bussi(Thermostat):
    def __init__(self, kT, tau=0.0):
        self.kT = float(kT)
        self.tau = float(tau)

    def _apply(self, integ):
        integ.setBussi(self.kT, self.tau)
