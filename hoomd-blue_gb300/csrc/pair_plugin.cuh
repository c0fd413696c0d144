// Pair kernels for an evaluator written to the reference's concept
// (example_plugins/pair_plugin/EvaluatorPairExample.h): gb_pair_plugin_call dispatch onto this
// library's force, fused-step and energy-between-sets kernels. Included by the plugin's kernel
// translation unit through hoomd/md/PotentialPairGPU.cuh.
#pragma once

#include "fused_step.h"
#include "pair_kernel.cuh"

namespace gb
{
// The reference's evaluator interface seen through this library's: a three-argument
// constructor (no shared-data pointer), no per-pair parameter preparation, needsCharge() known
// on the device only. The host-side checks therefore take every plugin evaluator as charge-free;
// the engine passes the particle charges to every plugin call, so an evaluator that reads them
// finds them.
template<class E> struct PluginEval
    {
    using param_type = typename E::param_type;
    E e;
    __device__ __forceinline__ PluginEval(float rsq, float rcutsq, const param_type& p,
                                          const float*)
        : e(rsq, rcutsq, p)
        {
        }
    __device__ __forceinline__ static void prepare_param(param_type&, float) { }
    __host__ __device__ static bool needsCharge()
        {
#ifdef __CUDA_ARCH__
        return E::needsCharge();
#else
        return false;
#endif
        }
    __device__ __forceinline__ void setCharge(float qi, float qj)
        {
        e.setCharge(qi, qj);
        }
    __device__ __forceinline__ bool evalForceAndEnergy(float& force_divr, float& pair_eng,
                                                       bool energy_shift)
        {
        return e.evalForceAndEnergy(force_divr, pair_eng, energy_shift);
        }
    };

template<class E> int plugin_call(gb_pair_plugin_call* c, const typename E::param_type* d_params)
    {
    GB_REQUIRE(c && c->args, "pair plugin: null call");
    GB_REQUIRE(c->args->d_charge, "pair plugin: the particle charges are required (an evaluator "
                                  "may read them)");
    const cudaStream_t s = (cudaStream_t)c->stream;
    switch (c->op)
        {
    case 0:
        {
        FuseArgs none {};
        return launch_pair<PluginEval<E>, false>(c->args, d_params, nullptr, none, s);
        }
    case 1:
        {
        FuseArgs fz;
        const int rc = make_fuse_args(c->args, c->fuse, fz);
        if (rc != GB_OK)
            return rc;
        return launch_pair<PluginEval<E>, true>(c->args, d_params, nullptr, fz, s);
        }
    case 2:
        return launch_energy_sets<PluginEval<E>>(c->args, d_params, nullptr, c->sets,
                                                 c->d_partials, s);
    default:
        return fail(GB_ERR_INVALID, "pair plugin: op must be 0, 1 or 2");
        }
    }
} // namespace gb
