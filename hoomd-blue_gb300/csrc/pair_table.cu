// Pair-force entry points for EvaluatorTable (one translation unit per evaluator, as the reference
// instantiates one PotentialPairGPUKernel per evaluator, hoomd/md/CMakeLists.txt:505-550).
#include "fused_step.h"
#include "pair_kernel.cuh"

using namespace gb;

extern "C"
    {
    int gb_pair_forces_table(const gb_pair_args* args, const gb_table_param* d_params, const float* d_table, void* stream)
        {
        FuseArgs none {};
        return launch_pair<EvalTable, false>(args, d_params, d_table, none, (cudaStream_t)stream);
        }

    int gb_md_pair_step_table(const gb_pair_args* args, const gb_table_param* d_params, const float* d_table, const gb_step_fuse* fuse, void* stream)
        {
        FuseArgs fz;
        int rc = make_fuse_args(args, fuse, fz);
        if (rc != GB_OK)
            return rc;
        return launch_pair<EvalTable, true>(args, d_params, d_table, fz, (cudaStream_t)stream);
        }

    int gb_pair_energy_sets_table(const gb_pair_args* args, const gb_table_param* d_params,
                                  const float* d_table,
                                  const gb_energy_sets* sets, double* d_partials, void* stream)
        {
        return launch_energy_sets<EvalTable>(args, d_params, d_table, sets, d_partials,
                                        (cudaStream_t)stream);
        }
    }
