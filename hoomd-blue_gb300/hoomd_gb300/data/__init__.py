"""Parameter containers (hoomd/data): the type-parameter classes a pair plugin's Python module
uses to declare its parameters (example_plugins/pair_plugin/pair.py)."""

from hoomd_gb300.data import parameterdicts, typeparam  # noqa: F401
from hoomd_gb300.data.parameterdicts import TypeParameterDict  # noqa: F401
from hoomd_gb300.data.typeparam import TypeParameter  # noqa: F401
