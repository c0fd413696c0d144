"""Pair-evaluator plugins build against this library's plugin headers (no GPU needed: nvcc
compiles for sm_103a here).

* The Hertz plugin of tests/pair_plugin/ -- an evaluator header, kernel file, module file and
  Python class laid out as the reference's example_plugins/pair_plugin -- compiles into a module
  that exports PotentialPairHertzGPU (the engine class) and PotentialPairHertz (the CPU class,
  which refuses: there is no CPU device).
* Where the reference source tree is present, the reference's own example plugin sources
  (example_plugins/pair_plugin/EvaluatorPairExample.h, PotentialPairExampleGPUKernel.cu,
  module.cc) compile unchanged, read in place, into a module with the same two names.
"""

import pathlib

import pytest

from plugin_util import BUILD, build_hertz


def test_hertz_plugin_builds_and_registers():
    mod = build_hertz()
    assert callable(mod.PotentialPairHertzGPU)
    with pytest.raises(RuntimeError, match="no CPU device"):
        mod.PotentialPairHertz()


def _reference_plugin_dir():
    from oracle import build
    d = pathlib.Path(build.REF_ROOT) / "example_plugins" / "pair_plugin"
    return d if (d / "EvaluatorPairExample.h").exists() else None


@pytest.mark.skipif(_reference_plugin_dir() is None, reason="reference source tree not present")
def test_reference_example_plugin_compiles_unchanged():
    from hoomd_gb300 import plugin
    d = _reference_plugin_dir()
    path = plugin.build_pair_plugin("_pair_plugin", [d / "PotentialPairExampleGPUKernel.cu"],
                                    [d / "module.cc"], BUILD / "reference_example")
    mod = plugin.load_pair_plugin("_pair_plugin", path)
    assert callable(mod.PotentialPairExampleGPU)
    with pytest.raises(RuntimeError, match="no CPU device"):
        mod.PotentialPairExample()
