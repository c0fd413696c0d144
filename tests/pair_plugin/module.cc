// Module file of the Hertz pair plugin, registered as the reference's plugin module registers
// its evaluator (example_plugins/pair_plugin/module.cc).
#include "EvaluatorPairHertz.h"

#include "hoomd/md/PotentialPair.h"
#include <pybind11/pybind11.h>
#ifdef ENABLE_HIP
#include "hoomd/md/PotentialPairGPU.h"
#endif

namespace hoomd
    {
namespace md
    {

PYBIND11_MODULE(_hertz_plugin, m)
    {
    detail::export_PotentialPair<EvaluatorPairHertz>(m, "PotentialPairHertz");
#ifdef ENABLE_HIP
    detail::export_PotentialPairGPU<EvaluatorPairHertz>(m, "PotentialPairHertzGPU");
#endif
    }

    } // end namespace md
    } // end namespace hoomd
