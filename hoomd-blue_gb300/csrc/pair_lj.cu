// Pair-force entry points for EvaluatorLJ (one translation unit per evaluator, as the reference
// instantiates one PotentialPairGPUKernel per evaluator, hoomd/md/CMakeLists.txt:505-550).
#include "fused_step.h"
#include "pair_kernel.cuh"

using namespace gb;

extern "C"
    {
    int gb_pair_forces_lj(const gb_pair_args* args, const gb_lj_param* d_params, void* stream)
        {
        FuseArgs none {};
        return launch_pair<EvalLJ, false>(args, d_params, nullptr, none, (cudaStream_t)stream);
        }

    int gb_md_pair_step_lj(const gb_pair_args* args, const gb_lj_param* d_params, const gb_step_fuse* fuse, void* stream)
        {
        FuseArgs fz;
        int rc = make_fuse_args(args, fuse, fz);
        if (rc != GB_OK)
            return rc;
        return launch_pair<EvalLJ, true>(args, d_params, nullptr, fz, (cudaStream_t)stream);
        }

    int gb_pair_energy_sets_lj(const gb_pair_args* args, const gb_lj_param* d_params,
                               const gb_energy_sets* sets, double* d_partials, void* stream)
        {
        return launch_energy_sets<EvalLJ>(args, d_params, nullptr, sets, d_partials,
                                          (cudaStream_t)stream);
        }

    unsigned int gb_pair_energy_sets_blocks(unsigned int N)
        {
        return energy_sets_blocks(N);
        }
    }
