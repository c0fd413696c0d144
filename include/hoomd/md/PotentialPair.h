// hoomd/md/PotentialPair.h for pair-evaluator plugins built against hoomd_gb300.
//
// The reference's plugin module also registers the CPU class of its evaluator
// (detail::export_PotentialPair<Evaluator>(m, "PotentialPair<Name>"),
// example_plugins/pair_plugin/module.cc). This library runs on the GPU only: the name is
// registered, and calling it raises an error that points at the GPU class.
#pragma once

#include "hoomd/HOOMDMath.h"

#include <stdexcept>
#include <string>

#include <pybind11/pybind11.h>

namespace hoomd
    {
namespace md
    {
namespace detail
    {
template<class evaluator> void export_PotentialPair(pybind11::module& m, const std::string& name)
    {
    const std::string gpu = name + "GPU";
    m.def(
        name.c_str(),
        [gpu](pybind11::args, pybind11::kwargs) -> pybind11::object {
            throw std::runtime_error("hoomd_gb300 has no CPU device; the pair force runs as " + gpu);
        });
    }

    } // end namespace detail
    } // end namespace md
    } // end namespace hoomd
