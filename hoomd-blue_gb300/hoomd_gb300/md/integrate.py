"""The MD integrator (hoomd/md/integrate.py:128-296): velocity Verlet two-step integration with
one method (ConstantVolume or Langevin) over all particles and any number of pair forces sharing
one neighbour list."""

from hoomd_gb300._native import _hoomd_gb300


class Integrator:
    def __init__(self, dt, integrate_rotational_dof=False, forces=None, constraints=None,
                 methods=None, rigid=None, half_step_hook=None):
        if integrate_rotational_dof:
            raise NotImplementedError("rotational degrees of freedom are outside this path")
        if constraints or rigid is not None or half_step_hook is not None:
            raise NotImplementedError("constraints, rigid bodies and half-step hooks are "
                                      "outside this path")
        self._dt = float(dt)
        self.forces = list(forces or [])
        self.methods = list(methods or [])
        self.integrate_rotational_dof = False
        self._simulation = None
        self._cpp_obj = None
        self._cpp_nlist = None

    @property
    def dt(self):
        return self._dt

    @dt.setter
    def dt(self, v):
        self._dt = float(v)
        if self._cpp_obj is not None:
            self._cpp_obj.dt = self._dt

    def _attach(self, simulation):
        if len(self.methods) != 1:
            raise NotImplementedError("exactly one integration method is supported")
        if not self.forces:
            raise RuntimeError("the integrator needs at least one force")
        nl = self.forces[0].nlist
        if any(f.nlist is not nl for f in self.forces):
            raise NotImplementedError("all pair forces must share one neighbour list")
        self._simulation = simulation
        cpp_nl = nl._attach(simulation)
        self._cpp_nlist = cpp_nl
        integ = _hoomd_gb300.IntegratorTwoStep(simulation.state._cpp_pdata, cpp_nl, self._dt)
        for f in self.forces:
            integ.addForce(f._attach(simulation, cpp_nl))
        self.methods[0]._attach(integ, simulation.state)
        self._cpp_obj = integ
        return integ

    def _detach(self):
        self._cpp_obj = None
        for f in self.forces:
            f._detach()
        if self.forces:
            self.forces[0].nlist._detach()
