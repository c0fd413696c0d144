// Pair-force entry points for the radial evaluator family (EvalRadial): the reference builds one
// PotentialPairGPU instantiation per evaluator (hoomd/md/CMakeLists.txt:505-550); here the
// fourteen closed forms share one instantiation set, selected per force by gb_radial_param.kind.
#include "fused_step.h"
#include "pair_kernel.cuh"

using namespace gb;

extern "C"
    {
    int gb_pair_forces_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                              void* stream)
        {
        FuseArgs none {};
        return launch_pair<EvalRadial, false>(args, d_params, nullptr, none,
                                              (cudaStream_t)stream);
        }

    int gb_md_pair_step_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                               const gb_step_fuse* fuse, void* stream)
        {
        FuseArgs fz;
        int rc = make_fuse_args(args, fuse, fz);
        if (rc != GB_OK)
            return rc;
        return launch_pair<EvalRadial, true>(args, d_params, nullptr, fz, (cudaStream_t)stream);
        }
    }
