"""Molecular dynamics (hoomd/md): neighbour lists, pair forces, the integrator and its methods."""

from hoomd_gb300.md import compute, methods, nlist, pair  # noqa: F401
from hoomd_gb300.md.integrate import Integrator  # noqa: F401
