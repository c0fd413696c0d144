// Pair-force entry points for the radial evaluator family (EvalRadial): the reference builds one
// PotentialPairGPU instantiation per evaluator (hoomd/md/CMakeLists.txt:505-550); here the
// closed forms share one instantiation set, selected per force by gb_radial_param.kind. With
// per-particle charges (args->d_charge) the charged instantiation set of pair_radial_q.cu runs.
#include "fused_step.h"
#include "pair_kernel.cuh"

namespace gb
{
int radial_charged(const gb_pair_args* args, const gb_radial_param* d_params, const FuseArgs& fz,
                   bool fused, cudaStream_t s);
int radial_energy_sets_charged(const gb_pair_args* args, const gb_radial_param* d_params,
                               const gb_energy_sets* sets, double* d_partials, cudaStream_t s);
}

using namespace gb;

extern "C"
    {
    int gb_pair_forces_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                              void* stream)
        {
        FuseArgs none {};
        if (args && args->d_charge)
            return radial_charged(args, d_params, none, false, (cudaStream_t)stream);
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
        if (args->d_charge)
            return radial_charged(args, d_params, fz, true, (cudaStream_t)stream);
        return launch_pair<EvalRadial, true>(args, d_params, nullptr, fz, (cudaStream_t)stream);
        }

    int gb_pair_energy_sets_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                                   const gb_energy_sets* sets, double* d_partials, void* stream)
        {
        if (args && args->d_charge)
            return radial_energy_sets_charged(args, d_params, sets, d_partials,
                                              (cudaStream_t)stream);
        return launch_energy_sets<EvalRadial>(args, d_params, nullptr, sets, d_partials,
                                              (cudaStream_t)stream);
        }
    }
