"""Integration methods (hoomd/md/methods/methods.py:85-176): ConstantVolume, which is NVE without a
thermostat and NVT with one."""

from hoomd_gb300.filter import All
from hoomd_gb300.md.methods import thermostats  # noqa: F401


class Method:
    pass


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

    def _attach(self, integ):
        self._cpp_integ = integ
        self._apply(integ)


class NVE(ConstantVolume):
    """The reference's legacy NVE alias: ConstantVolume without a thermostat."""

    def __init__(self, filter):
        super().__init__(filter, thermostat=None)
