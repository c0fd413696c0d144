"""Particle filters (hoomd/filter). The hot path integrates the group of all particles."""


class ParticleFilter:
    pass


class All(ParticleFilter):
    """hoomd.filter.All: every particle."""

    def __eq__(self, other):
        return isinstance(other, All)

    def __hash__(self):
        return hash("All")
