// hoomd/md/PotentialPairGPU.cuh for pair-evaluator plugins built against hoomd_gb300.
//
// The reference's plugin kernel file (example_plugins/pair_plugin/PotentialPairExampleGPUKernel.cu)
// explicitly instantiates
//     template hipError_t gpu_compute_pair_forces<Evaluator>(const pair_args_t&,
//                                                            const Evaluator::param_type*);
// (the driver of hoomd/md/PotentialPairGPU.cuh:579-656). Here the same instantiation compiles
// this library's pair kernels (interleaved and head-list forms, the fused pair step and the
// energy between two sets) for the evaluator; pair_args_t is the gb_pair_plugin_call of
// include/hoomd_gb300.h, whose `op` selects the kernel. Compile with nvcc, -I on this include
// directory and on the package's csrc directory; link against libhoomd_gb300.so.
#pragma once

#include "hoomd/HOOMDMath.h"

#include <cuda_runtime.h>

#include "hoomd_gb300.h"

#if !defined(HIP_INCLUDE_HIP_HIP_RUNTIME_H) && !defined(HOOMD_GB300_HIP_ERROR)
#define HOOMD_GB300_HIP_ERROR
typedef cudaError_t hipError_t;
#endif

#ifdef __CUDACC__
#include "pair_plugin.cuh"
#endif

namespace hoomd
    {
namespace md
    {
namespace kernel
    {
typedef gb_pair_plugin_call pair_args_t;

//! One call of the evaluator's kernels; pair_args.status receives the gb_status.
template<class evaluator>
hipError_t gpu_compute_pair_forces(const pair_args_t& pair_args,
                                   const typename evaluator::param_type* d_params)
#ifdef __CUDACC__
    {
    pair_args_t& c = const_cast<pair_args_t&>(pair_args);
    c.status = gb::plugin_call<evaluator>(&c, d_params);
    return c.status == GB_OK ? cudaSuccess : cudaErrorInvalidValue;
    }
#else
    ;
#endif

    } // end namespace kernel
    } // end namespace md
    } // end namespace hoomd
