// Pair evaluators for the GB300 pair kernel, following the reference's evaluator concept
// (example_plugins/pair_plugin/EvaluatorPairExample.h): a POD param_type per type pair, a
// constructor from (rsq, rcutsq, param), needsCharge/setCharge, and
// evalForceAndEnergy(force_divr, pair_eng, energy_shift) returning false when the pair does not
// interact. Two additions: the constructor also receives `ext`, a device pointer to shared
// read-only data (the packed table bins for Table; unused by LJ and Example), because the
// reference's ManagedArray members have no equivalent in a plain C-ABI parameter struct; and a
// static prepare_param(param, rcutsq) that a kernel applies once per type pair when it stages
// the parameters (derived constants, e.g. the Table's 1/dr).
//
// A plugin evaluator is added by writing a struct with this interface and instantiating
// gb::launch_pair<Evaluator>() from pair_kernel.cuh.
#pragma once

#include "gb_device.cuh"

namespace gb
{

// Reciprocal with one MUFU instruction (rcp.approx.ftz.f32, < 1 ulp error): enough for FP32 forces
// held to 1e-5 relative, and a quarter of the instructions of the IEEE-rounded reciprocal.
__device__ __forceinline__ float rcp_approx(float x)
    {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
    }

// hoomd/md/EvaluatorPairLJ.h:162-211. Branch free: the terms are computed for every pair and
// selected, so lanes of a warp that fall inside and outside r_cut do not diverge.
struct EvalLJ
    {
    using param_type = gb_lj_param;
    __device__ __forceinline__ static void prepare_param(param_type&, float) { }
    float rsq, rcutsq, lj1, lj2;
    __device__ __forceinline__ EvalLJ(float rsq_, float rcutsq_, const param_type& p,
                                      const float*)
        : rsq(rsq_), rcutsq(rcutsq_), lj1(p.epsilon_x_4 * p.sigma_6 * p.sigma_6),
          lj2(p.epsilon_x_4 * p.sigma_6)
        {
        }
    static constexpr bool needsCharge()
        {
        return false;
        }
    __device__ __forceinline__ void setCharge(float, float) { }
    __device__ __forceinline__ bool evalForceAndEnergy(float& force_divr, float& pair_eng,
                                                       bool energy_shift) const
        {
        const bool in = rsq < rcutsq && lj1 != 0.0f;
        const float r2inv = rcp_approx(rsq);
        const float r6inv = r2inv * r2inv * r2inv;
        const float fd = r2inv * r6inv * (12.0f * lj1 * r6inv - 6.0f * lj2);
        float pe = r6inv * (lj1 * r6inv - lj2);
        if (energy_shift)
            {
            const float rcut2inv = rcp_approx(rcutsq);
            const float rcut6inv = rcut2inv * rcut2inv * rcut2inv;
            pe -= rcut6inv * (lj1 * rcut6inv - lj2);
            }
        force_divr = in ? fd : force_divr;
        pair_eng = in ? pe : pair_eng;
        return in;
        }
    };

// hoomd/md/EvaluatorPairTable.h:151-194: linear interpolation on width points spaced
// dr = (r_cut - r_min)/width, V1 = F1 = 0 in the last bin. Each bin is one packed quad
// (V[k], F[k], V[k+1], F[k+1]), so a pair reads 16 bytes. 1/dr is derived once per type pair
// (prepare_param) and r, 1/r come from one reciprocal square root; value_i is clamped to width-1
// (at FP32, r just below r_cut can round (r - rmin)/dr up to width, where the reference reads one
// past the end of its table). Branch free: out-of-range lanes read a valid bin and are discarded.
struct EvalTable
    {
    using param_type = gb_table_param;
    float rsq, rcutsq, rmin, inv_dr;
    unsigned int width;
    const float4* bins;
    // per type pair, once per block: keep 1/dr in the reserved word
    __device__ __forceinline__ static void prepare_param(param_type& p, float rcutsq)
        {
        const float rcut = sqrtf(rcutsq);
        const float inv = (float)p.width / (rcut - p.rmin);
        p.reserved = __float_as_uint(inv);
        }
    __device__ __forceinline__ EvalTable(float rsq_, float rcutsq_, const param_type& p,
                                         const float* table)
        : rsq(rsq_), rcutsq(rcutsq_), rmin(p.rmin), width(p.width),
          bins(reinterpret_cast<const float4*>(table) + p.offset)
        {
        inv_dr = __uint_as_float(p.reserved);
        }
    static constexpr bool needsCharge()
        {
        return false;
        }
    __device__ __forceinline__ void setCharge(float, float) { }
    __device__ __forceinline__ bool evalForceAndEnergy(float& force_divr, float& pair_eng,
                                                       bool) const
        {
        const float rinv = rsqrtf(rsq);
        const float r = rsq * rinv;
        const bool in = rsq < rcutsq && r >= rmin && rsq > 0.0f;
        const float value_f = fmaxf((r - rmin) * inv_dr, 0.0f);
        unsigned int value_i = (unsigned int)value_f;
        value_i = min(value_i, width - 1);
        const float4 q = __ldg(bins + value_i);
        const float f = value_f - (float)value_i;
        const float Vr = q.x + f * (q.z - q.x);
        const float Fr = q.y + f * (q.w - q.y);
        force_divr = in ? Fr * rinv : force_divr;
        pair_eng = in ? Vr : pair_eng;
        return in;
        }
    };

// example_plugins/pair_plugin/EvaluatorPairExample.h:82-142 (harmonic spring)
struct EvalExample
    {
    using param_type = gb_example_param;
    __device__ __forceinline__ static void prepare_param(param_type&, float) { }
    float rsq, rcutsq, k, sigma;
    __device__ __forceinline__ EvalExample(float rsq_, float rcutsq_, const param_type& p,
                                           const float*)
        : rsq(rsq_), rcutsq(rcutsq_), k(p.k), sigma(p.sigma)
        {
        }
    static constexpr bool needsCharge()
        {
        return false;
        }
    __device__ __forceinline__ void setCharge(float, float) { }
    __device__ __forceinline__ bool evalForceAndEnergy(float& force_divr, float& pair_eng,
                                                       bool energy_shift) const
        {
        if (rsq < rcutsq)
            {
            const float r = sqrtf(rsq);
            const float rinv = 1.0f / r;
            const float overlap = sigma - r;
            force_divr = k * overlap * rinv;
            pair_eng = 0.5f * k * overlap * overlap;
            if (energy_shift)
                {
                const float rcut = sqrtf(rcutsq);
                const float cut_overlap = sigma - rcut;
                pair_eng -= 0.5f * k * cut_overlap * cut_overlap;
                }
            return true;
            }
        return false;
        }
    };

} // namespace gb
