// The radial evaluator family with per-particle charges (EvalRadialQ: every pair scaled by
// q_i q_j), in its own translation unit so that it compiles in parallel with the uncharged set.
#include "fused_step.h"
#include "pair_kernel.cuh"

namespace gb
{
int radial_charged(const gb_pair_args* args, const gb_radial_param* d_params, const FuseArgs& fz,
                   bool fused, cudaStream_t s)
    {
    if (fused)
        return launch_pair<EvalRadialQ, true>(args, d_params, nullptr, fz, s);
    return launch_pair<EvalRadialQ, false>(args, d_params, nullptr, fz, s);
    }

int radial_energy_sets_charged(const gb_pair_args* args, const gb_radial_param* d_params,
                               const gb_energy_sets* sets, double* d_partials, cudaStream_t s)
    {
    return launch_energy_sets<EvalRadialQ>(args, d_params, nullptr, sets, d_partials, s);
    }
} // namespace gb
