"""Triggers (hoomd/trigger.py): boolean functions of the timestep that schedule writers and
tuners. ``_next(t, end)`` gives the first step in (t, end] that fires, else ``end``, so the run
loop can hand the steps in between to the engine in one call."""


class Trigger:
    def __call__(self, timestep):
        raise NotImplementedError

    def _next(self, t, end):
        for s in range(t + 1, end + 1):
            if self(s):
                return s
        return end


class Periodic(Trigger):
    """Fires when (timestep - phase) % period == 0."""

    def __init__(self, period, phase=0):
        self.period = int(period)
        self.phase = int(phase)
        if self.period < 1:
            raise ValueError("period must be positive")

    def __call__(self, timestep):
        return (timestep - self.phase) % self.period == 0

    def _next(self, t, end):
        s = t + 1 + (self.phase - (t + 1)) % self.period
        return min(s, end)


class On(Trigger):
    """Fires only at ``timestep``."""

    def __init__(self, timestep):
        self.timestep = int(timestep)

    def __call__(self, timestep):
        return timestep == self.timestep

    def _next(self, t, end):
        return self.timestep if t < self.timestep <= end else end


class Before(Trigger):
    """Fires for timesteps before ``timestep``."""

    def __init__(self, timestep):
        self.timestep = int(timestep)

    def __call__(self, timestep):
        return timestep < self.timestep

    def _next(self, t, end):
        return t + 1 if t + 1 < self.timestep and t + 1 <= end else end


class After(Trigger):
    """Fires for timesteps after ``timestep``."""

    def __init__(self, timestep):
        self.timestep = int(timestep)

    def __call__(self, timestep):
        return timestep > self.timestep

    def _next(self, t, end):
        return min(max(t + 1, self.timestep + 1), end)


class Not(Trigger):
    def __init__(self, trigger):
        self.trigger = trigger

    def __call__(self, timestep):
        return not self.trigger(timestep)


class And(Trigger):
    def __init__(self, triggers):
        self.triggers = list(triggers)

    def __call__(self, timestep):
        return all(t(timestep) for t in self.triggers)


class Or(Trigger):
    def __init__(self, triggers):
        self.triggers = list(triggers)

    def __call__(self, timestep):
        return any(t(timestep) for t in self.triggers)

    def _next(self, t, end):
        return min([tr._next(t, end) for tr in self.triggers] + [end])


def as_trigger(t):
    if isinstance(t, Trigger):
        return t
    return Periodic(int(t))
