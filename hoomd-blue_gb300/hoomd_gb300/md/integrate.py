"""The MD integrator (hoomd/md/integrate.py:128-296): velocity Verlet two-step integration with
one method (ConstantVolume or Langevin) over all particles and any number of pair forces sharing
one neighbour list."""

from hoomd_gb300._native import _hoomd_gb300


class _SyncedList(list):
    """A list whose changes detach the integrator, so the next run attaches the new contents
    (the reference's SyncedList behaviour for ``forces`` and ``methods``)."""

    def __init__(self, items, on_change):
        super().__init__(items)
        self._on_change = on_change

    def _changed(self):
        self._on_change()


def _wrap(name):
    base = getattr(list, name)

    def method(self, *args, **kwargs):
        out = base(self, *args, **kwargs)
        self._changed()
        return out
    method.__name__ = name
    return method


for _name in ("append", "extend", "insert", "remove", "pop", "clear", "__setitem__",
              "__delitem__", "__iadd__", "sort", "reverse"):
    setattr(_SyncedList, _name, _wrap(_name))


class Integrator:
    def __init__(self, dt, integrate_rotational_dof=False, forces=None, constraints=None,
                 methods=None, rigid=None, half_step_hook=None):
        if integrate_rotational_dof:
            raise NotImplementedError("rotational degrees of freedom are outside this path")
        if constraints or rigid is not None or half_step_hook is not None:
            raise NotImplementedError("constraints, rigid bodies and half-step hooks are "
                                      "outside this path")
        self._dt = float(dt)
        self._forces = _SyncedList(forces or [], self._contents_changed)
        self._methods = _SyncedList(methods or [], self._contents_changed)
        self.integrate_rotational_dof = False
        self._simulation = None
        self._cpp_obj = None
        self._cpp_nlist = None
        self._attached_forces = []

    def _contents_changed(self):
        if self._simulation is not None and self._cpp_obj is not None:
            # forces taken out of the list lose their engine objects (reading them raises until
            # they are attached again); the ones still listed are re-attached at the next run
            current = {id(f) for f in self._forces}
            for f in self._attached_forces:
                if id(f) not in current:
                    f._detach()
            self._detach()
            self._simulation._detach_all()

    @property
    def forces(self):
        return self._forces

    @forces.setter
    def forces(self, items):
        self._forces = _SyncedList(items, self._contents_changed)
        self._contents_changed()

    @property
    def methods(self):
        return self._methods

    @methods.setter
    def methods(self, items):
        self._methods = _SyncedList(items, self._contents_changed)
        self._contents_changed()

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
        integ.notice_level = int(getattr(simulation.device, "notice_level", 2))
        for f in self.forces:
            integ.addForce(f._attach(simulation, cpp_nl))
        self._attached_forces = list(self.forces)
        self.methods[0]._attach(integ, simulation.state)
        self._cpp_obj = integ
        return integ

    def _detach(self):
        self._cpp_obj = None
        for f in self.forces:
            f._detach()
        if self.forces:
            self.forces[0].nlist._detach()
