"""Builds the Hertz pair plugin of tests/pair_plugin/ (an evaluator written to the reference's
plugin concept) into tests/pair_plugin/_build/ and returns its module and Pair class."""

import pathlib

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "pair_plugin"
BUILD = SRC / "_build"


def build_hertz(verbose=False):
    from hoomd_gb300 import plugin
    path = plugin.build_pair_plugin("_hertz_plugin", [SRC / "PotentialPairHertzGPUKernel.cu"],
                                    [SRC / "module.cc"], BUILD / "hertz", include_dirs=[SRC],
                                    verbose=verbose)
    return plugin.load_pair_plugin("_hertz_plugin", path)


def hertz_pair_class():
    import importlib.util
    mod = build_hertz()
    spec = importlib.util.spec_from_file_location("hertz_pair", str(SRC / "pair.py"))
    pmod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pmod)
    return pmod.make_pair_class(mod), mod
