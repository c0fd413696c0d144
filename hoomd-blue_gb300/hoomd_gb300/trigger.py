"""Triggers (hoomd/trigger.py)."""


class Trigger:
    def __call__(self, timestep):
        raise NotImplementedError


class Periodic(Trigger):
    """Fires when (timestep - phase) % period == 0."""

    def __init__(self, period, phase=0):
        self.period = int(period)
        self.phase = int(phase)

    def __call__(self, timestep):
        return (timestep - self.phase) % self.period == 0


def as_trigger(t):
    if isinstance(t, Trigger):
        return t
    return Periodic(int(t))
