"""Python class of the Hertz pair plugin, declared as the reference's plugin declares its pair
force (example_plugins/pair_plugin/pair.py): the engine class by module and name, the accepted
modes, and the per-type-pair parameters as a TypeParameter."""

from hoomd_gb300.data.parameterdicts import TypeParameterDict
from hoomd_gb300.data.typeparam import TypeParameter
from hoomd_gb300.md import pair


def make_pair_class(ext_module):
    """The HertzPair class over the built plugin module ``ext_module``."""

    class HertzPair(pair.Pair):
        """Hertzian soft spheres: V = epsilon (1 - r/sigma)^(5/2) for r < sigma."""

        _ext_module = ext_module
        _cpp_class_name = "PotentialPairHertz"
        _accepted_modes = ("none", "shift", "xplor")

        def __init__(self, nlist, default_r_cut=None, default_r_on=0., mode='none'):
            super().__init__(nlist, default_r_cut, default_r_on, mode)
            params = TypeParameter('params', 'particle_types',
                                   TypeParameterDict(epsilon=float, sigma=float, len_keys=2))
            self._add_typeparam(params)

    return HertzPair
