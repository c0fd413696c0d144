"""ThermodynamicQuantities (hoomd/md/compute.py; C++ hoomd/md/ComputeThermo.cc:76-290): kinetic and
potential energy, temperature and pressure of all particles, reduced on the GPU in FP64."""

from hoomd_gb300.filter import All


class ThermodynamicQuantities:
    _loggables = {q: "scalar" for q in (
        "kinetic_energy", "translational_kinetic_energy", "potential_energy",
        "degrees_of_freedom", "translational_degrees_of_freedom", "kinetic_temperature",
        "volume", "pressure")}

    def __init__(self, filter):
        if not isinstance(filter, All):
            raise NotImplementedError("thermodynamic quantities are computed over all particles")
        self.filter = filter
        self._simulation = None

    def _attach_to(self, sim):
        self._simulation = sim

    def _thermo(self, virial=False):
        sim = self._simulation
        if sim is None:
            raise RuntimeError("add the compute to simulation.operations.computes first")
        cpp = sim._attach()
        return cpp.thermo(bool(virial)), cpp

    def _detach(self):
        pass

    @property
    def kinetic_energy(self):
        return self._thermo()[0][0]

    @property
    def translational_kinetic_energy(self):
        return self.kinetic_energy

    @property
    def potential_energy(self):
        return self._thermo()[0][1]

    @property
    def degrees_of_freedom(self):
        return self._thermo()[1].dof()

    @property
    def translational_degrees_of_freedom(self):
        return self.degrees_of_freedom

    @property
    def kinetic_temperature(self):
        (ke, _, _), cpp = self._thermo()
        dof = cpp.dof()
        return 2.0 * ke / dof if dof > 0 else 0.0

    @property
    def volume(self):
        return self._simulation.state.box.volume

    @property
    def pressure(self):
        """P = (2 K / D + W) / V with W = (virial xx + yy + zz) / D (ComputeThermo.cc)."""
        (ke, _, w), cpp = self._thermo(True)
        D = self._simulation.state.dimensions
        return (2.0 * ke / D + w * 3.0 / D) / self.volume
