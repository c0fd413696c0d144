"""GSD files: ``fl`` is the file layer (gsd.fl), ``hoomd`` the particle schema (gsd.hoomd)."""

from hoomd_gb300.gsd import fl, hoomd  # noqa: F401

__all__ = ["fl", "hoomd"]
