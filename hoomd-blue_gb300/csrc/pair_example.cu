// Pair-force entry points for EvaluatorExample (one translation unit per evaluator, as the reference
// instantiates one PotentialPairGPUKernel per evaluator, hoomd/md/CMakeLists.txt:505-550).
#include "fused_step.h"
#include "pair_kernel.cuh"

using namespace gb;

extern "C"
    {
    int gb_pair_forces_example(const gb_pair_args* args, const gb_example_param* d_params, void* stream)
        {
        FuseArgs none {};
        return launch_pair<EvalExample, false>(args, d_params, nullptr, none, (cudaStream_t)stream);
        }

    int gb_md_pair_step_example(const gb_pair_args* args, const gb_example_param* d_params, const gb_step_fuse* fuse, void* stream)
        {
        FuseArgs fz;
        int rc = make_fuse_args(args, fuse, fz);
        if (rc != GB_OK)
            return rc;
        return launch_pair<EvalExample, true>(args, d_params, nullptr, fz, (cudaStream_t)stream);
        }

    int gb_pair_energy_sets_example(const gb_pair_args* args, const gb_example_param* d_params,
                                  const gb_energy_sets* sets, double* d_partials, void* stream)
        {
        return launch_energy_sets<EvalExample>(args, d_params, nullptr, sets, d_partials,
                                        (cudaStream_t)stream);
        }
    }
