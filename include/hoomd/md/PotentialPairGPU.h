// hoomd/md/PotentialPairGPU.h for pair-evaluator plugins built against hoomd_gb300.
//
// The reference's plugin module (example_plugins/pair_plugin/module.cc) registers its evaluator
// with
//     hoomd::md::detail::export_PotentialPairGPU<Evaluator>(m, "PotentialPair<Name>GPU");
// Here that call adds to the plugin module a constructor of the same name. Called as the
// reference's Python layer calls the class (hoomd/md/pair/pair.py:126-146: the state's particle
// data and the neighbour list), it returns the engine's pair force for this evaluator, an object
// of hoomd_gb300's compiled module with the reference's methods (setParams((a, b), dict),
// getParams, setRCut / getRCut, setROn / getROn, mode, tail_correction). Parameters cross as the
// evaluator's own param_type, built by its param_type(pybind11::dict, bool) constructor and read
// back by its asDict(); the kernels are those of the plugin's kernel file, which instantiates
// gpu_compute_pair_forces<Evaluator> (hoomd/md/PotentialPairGPU.cuh).
#pragma once

#include "hoomd/HOOMDMath.h"
#include "hoomd/md/PotentialPairGPU.cuh"

#include <cstring>
#include <stdexcept>
#include <string>

#include <pybind11/pybind11.h>

namespace hoomd
    {
namespace md
    {
namespace detail
    {
template<class evaluator> int gb_plugin_entry(gb_pair_plugin_call* call, const void* d_params)
    {
    kernel::gpu_compute_pair_forces<evaluator>(
        *call, static_cast<const typename evaluator::param_type*>(d_params));
    return call->status;
    }

template<class evaluator>
void export_PotentialPairGPU(pybind11::module& m, const std::string& name)
    {
    using param_type = typename evaluator::param_type;
    static const std::string evaluator_name = evaluator::getName();
    static const gb_pair_plugin record = {GB_PAIR_PLUGIN_ABI, (uint32_t)sizeof(param_type),
                                          &gb_plugin_entry<evaluator>, evaluator_name.c_str()};
    pybind11::object to_bytes = pybind11::cpp_function([](pybind11::dict d) {
        param_type p(d, false);
        return pybind11::bytes(reinterpret_cast<const char*>(&p), sizeof(p));
    });
    pybind11::object to_dict = pybind11::cpp_function([](pybind11::bytes b) {
        const std::string s = b;
        if (s.size() != sizeof(param_type))
            throw std::invalid_argument("parameter record of the wrong size");
        param_type p;
        std::memcpy(static_cast<void*>(&p), s.data(), sizeof(p));
        return p.asDict();
    });
    m.def(
        name.c_str(),
        [to_bytes, to_dict](pybind11::object particle_data, pybind11::object nlist) {
            pybind11::object engine = pybind11::module_::import("hoomd_gb300._hoomd_gb300");
            return engine.attr("PotentialPairPluginGPU")(
                particle_data, nlist,
                pybind11::capsule(const_cast<gb_pair_plugin*>(&record), "gb_pair_plugin"),
                to_bytes, to_dict);
        },
        pybind11::arg("sysdef"), pybind11::arg("nlist"));
    }

    } // end namespace detail
    } // end namespace md
    } // end namespace hoomd
