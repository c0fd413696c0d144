// Pair evaluators for the GB300 pair kernel, following the reference's evaluator concept
// (example_plugins/pair_plugin/EvaluatorPairExample.h): a POD param_type per type pair, a
// constructor from (rsq, rcutsq, param), needsCharge/setCharge, and
// evalForceAndEnergy(force_divr, pair_eng, energy_shift) returning false when the pair does not
// interact. One addition: the constructor also receives `ext`, a device pointer to shared
// read-only data (the flat table array for Table; unused by LJ and Example), because the
// reference's ManagedArray members have no equivalent in a plain C-ABI parameter struct.
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

// hoomd/md/EvaluatorPairTable.h:151-194. Linear interpolation on width points spaced
// (r_cut - r_min)/width; V1 = F1 = 0 in the last bin. value_i is clamped to width-1: at FP32, r
// just below r_cut can round (r - rmin)/dr up to width, where the reference reads one past the
// end of its table.
struct EvalTable
    {
    using param_type = gb_table_param;
    float rsq, rcutsq, rmin;
    unsigned int width;
    const float* V;
    const float* F;
    __device__ __forceinline__ EvalTable(float rsq_, float rcutsq_, const param_type& p,
                                         const float* table)
        : rsq(rsq_), rcutsq(rcutsq_), rmin(p.rmin), width(p.width), V(table + p.offset),
          F(table + p.offset + p.width)
        {
        }
    static constexpr bool needsCharge()
        {
        return false;
        }
    __device__ __forceinline__ void setCharge(float, float) { }
    __device__ __forceinline__ bool evalForceAndEnergy(float& force_divr, float& pair_eng,
                                                       bool) const
        {
        const float r = sqrtf(rsq);
        if (rsq >= rcutsq || r < rmin)
            return false;
        const float rcut = sqrtf(rcutsq);
        const float delta_r = (rcut - rmin) / (float)width;
        const float value_f = (r - rmin) / delta_r;
        unsigned int value_i = (unsigned int)floorf(value_f);
        if (value_i >= width)
            value_i = width - 1;
        const float V0 = __ldg(V + value_i);
        const float F0 = __ldg(F + value_i);
        float V1 = 0.0f, F1 = 0.0f;
        if (value_i + 1 < width)
            {
            V1 = __ldg(V + value_i + 1);
            F1 = __ldg(F + value_i + 1);
            }
        const float f = value_f - (float)value_i;
        const float Vr = V0 + f * (V1 - V0);
        const float Fr = F0 + f * (F1 - F0);
        if (rsq > 0.0f)
            force_divr = Fr / r;
        pair_eng = Vr;
        return true;
        }
    };

// example_plugins/pair_plugin/EvaluatorPairExample.h:82-142 (harmonic spring)
struct EvalExample
    {
    using param_type = gb_example_param;
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
