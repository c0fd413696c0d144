// Kernel file of the Hertz pair plugin: the explicit instantiation the reference's plugin kernel
// file makes (example_plugins/pair_plugin/PotentialPairExampleGPUKernel.cu).
#include "EvaluatorPairHertz.h"
#include "hoomd/md/PotentialPairGPU.cuh"

namespace hoomd
    {
namespace md
    {
namespace kernel
    {
template __attribute__((visibility("default"))) hipError_t
gpu_compute_pair_forces<EvaluatorPairHertz>(const pair_args_t& pair_args,
                                            const EvaluatorPairHertz::param_type* d_params);
    } // end namespace kernel
    } // end namespace md
    } // end namespace hoomd
