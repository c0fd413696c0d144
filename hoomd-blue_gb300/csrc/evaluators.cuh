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
// gb::launch_pair<Evaluator>() from pair_kernel.cuh; pair_example.cu is a complete example.
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
    __host__ __device__ static constexpr bool needsCharge()
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
    __host__ __device__ static constexpr bool needsCharge()
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
    __host__ __device__ static constexpr bool needsCharge()
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

// The reference's other radial evaluators (hoomd/md/EvaluatorPair{Gauss,Yukawa,Morse,
// ForceShiftedLJ,Mie,ExpandedMie,ExpandedLJ,Buckingham,LJ1208,LJ0804,LJGauss,ExpandedGaussian,
// OPP,TWF}.h) as one evaluator: the kind is uniform per force, so the switch costs one
// non-divergent branch per pair and the whole family shares one set of kernel instantiations.
// Each kind writes V(r) and F(r) = -dV/dr from its closed form; shift mode subtracts V(r_cut).
// The closed forms are one out-of-line function, so every kernel variant shares its code.
// Q = true multiplies every pair's force and energy by q_i q_j (Ewald, ReactionField with
// use_charge): the closed forms below are written for unit charges, and all of them are linear
// in q_i q_j.
template<bool Q> struct EvalRadialT
    {
    using param_type = gb_radial_param;
    // derived per type pair: the Mie prefactor, or F(r_cut) of the force-shifted LJ
    __device__ __forceinline__ static void prepare_param(param_type& p, float rcutsq)
        {
        if (p.kind == GB_RADIAL_MIE || p.kind == GB_RADIAL_EXPANDED_MIE)
            {
            const float n = p.v[2], m = p.v[3];
            p.aux = (n / (n - m)) * powf(n / m, m / (n - m)) * p.v[0];
            }
        else if (p.kind == GB_RADIAL_FORCE_SHIFTED_LJ)
            {
            float V, F;
            p.aux = 0.0f;
            eval(p, sqrtf(rcutsq), V, F);
            p.aux = F;
            }
        else if (p.kind == GB_RADIAL_DPD_CONSERVATIVE || p.kind == GB_RADIAL_FOURIER
                 || p.kind == GB_RADIAL_REACTION_FIELD)
            p.aux = sqrtf(rcutsq); // r_cut enters the functional form
        }
    float rsq, rcutsq;
    param_type p;
    float qiqj = 1.0f;
    __device__ __forceinline__ EvalRadialT(float rsq_, float rcutsq_, const param_type& p_,
                                           const float*)
        : rsq(rsq_), rcutsq(rcutsq_), p(p_)
        {
        }
    __host__ __device__ static constexpr bool needsCharge()
        {
        return Q;
        }
    __device__ __forceinline__ void setCharge(float qi, float qj)
        {
        if (Q)
            qiqj = qi * qj;
        }

    // (s/x)^n - style LJ of exponents (n, m) with prefactor c: V and F at distance x = r - delta
    __device__ __forceinline__ static void lj_nm(float c, float sigma, float x, int n, int m,
                                                 float& V, float& F)
        {
        const float q = sigma / x;
        const float q2 = q * q, q4 = q2 * q2;
        float qn, qm;
        if (n == 12)
            {
            const float q6 = q4 * q2;
            qn = q6 * q6;
            qm = m == 6 ? q6 : q4 * q4;
            }
        else // n == 8, m == 4
            {
            qn = q4 * q4;
            qm = q4;
            }
        V = c * (qn - qm);
        F = c * ((float)n * qn - (float)m * qm) / x;
        }

    __device__ __noinline__ static void eval(const param_type& p, float r, float& V, float& F)
        {
        const float* v = p.v;
        switch (p.kind)
            {
            case GB_RADIAL_GAUSS:
                {
                const float is2 = 1.0f / (v[1] * v[1]);
                const float e = v[0] * expf(-0.5f * r * r * is2);
                V = e;
                F = e * r * is2;
                break;
                }
            case GB_RADIAL_YUKAWA:
                {
                const float e = v[0] * expf(-v[1] * r) / r;
                V = e;
                F = e * (v[1] * r + 1.0f) / r;
                break;
                }
            case GB_RADIAL_MORSE:
                {
                const float e1 = expf(-v[1] * (r - v[2]));
                V = v[0] * (e1 * e1 - 2.0f * e1);
                F = 2.0f * v[0] * v[1] * (e1 * e1 - e1);
                break;
                }
            case GB_RADIAL_FORCE_SHIFTED_LJ:
                {
                // F = F_LJ(r) - F_LJ(r_cut); aux = F_LJ(r_cut) (0 while it is being derived).
                // The energy's (r - r_cut) F_LJ(r_cut) term is added by evalForceAndEnergy.
                lj_nm(4.0f * v[1], v[0], r, 12, 6, V, F);
                F -= p.aux;
                break;
                }
            case GB_RADIAL_MIE:
            case GB_RADIAL_EXPANDED_MIE:
                {
                const float x = p.kind == GB_RADIAL_EXPANDED_MIE ? r - v[4] : r;
                const float q = v[1] / x;
                const float qn = powf(q, v[2]), qm = powf(q, v[3]);
                V = p.aux * (qn - qm);
                F = p.aux * (v[2] * qn - v[3] * qm) / x;
                break;
                }
            case GB_RADIAL_EXPANDED_LJ:
                lj_nm(4.0f * v[1], v[0], r - v[2], 12, 6, V, F);
                break;
            case GB_RADIAL_BUCKINGHAM:
                {
                const float ir2 = 1.0f / (r * r), ir6 = ir2 * ir2 * ir2;
                const float e = v[0] * expf(-r / v[1]);
                V = e - v[2] * ir6;
                F = e / v[1] - 6.0f * v[2] * ir6 / r;
                break;
                }
            case GB_RADIAL_LJ1208:
                lj_nm(4.0f * v[1], v[0], r, 12, 8, V, F);
                break;
            case GB_RADIAL_LJ0804:
                lj_nm(4.0f * v[1], v[0], r, 8, 4, V, F);
                break;
            case GB_RADIAL_LJ_GAUSS:
                {
                const float ir2 = 1.0f / (r * r), ir6 = ir2 * ir2 * ir2;
                const float d = r - v[2];
                const float is2 = 1.0f / (v[1] * v[1]);
                const float g = v[0] * expf(-0.5f * d * d * is2);
                V = ir6 * ir6 - 2.0f * ir6 - g;
                F = (12.0f * ir6 * ir6 - 12.0f * ir6) / r - g * d * is2;
                break;
                }
            case GB_RADIAL_EXPANDED_GAUSS:
                {
                const float d = r - v[2];
                const float is2 = 1.0f / (v[1] * v[1]);
                const float e = v[0] * expf(-0.5f * d * d * is2);
                V = e;
                F = e * d * is2;
                break;
                }
            case GB_RADIAL_OPP:
                {
                const float a = v[0] * powf(r, -v[2]);
                const float b = v[1] * powf(r, -v[3]);
                const float arg = v[4] * r - v[5];
                const float c = cosf(arg), s = sinf(arg);
                V = a + b * c;
                F = (v[2] * a + v[3] * b * c) / r + v[4] * b * s;
                break;
                }
            case GB_RADIAL_DPD_CONSERVATIVE:
                {
                const float rc = p.aux;
                V = v[0] * (rc - r) - 0.5f * v[0] / rc * (rc * rc - r * r);
                F = v[0] * (1.0f - r / rc);
                break;
                }
            case GB_RADIAL_DLVO:
                {
                const float kappa = v[0], Z = v[1], A = v[2], a1 = v[3], a2 = v[4];
                if (kappa == 0.0f)
                    {
                    V = F = 0.0f;
                    break;
                    }
                const float radsum = a1 + a2, radsub = a1 - a2, radprod = a1 * a2;
                const float radsumsq = a1 * a1 + a2 * a2, radsubsq = a1 * a1 - a2 * a2;
                const float r2 = r * r;
                const float rmdsqs = r2 - radsum * radsum, rmdsqm = r2 - radsub * radsub;
                const float rep = kappa * radprod / radsum * Z * expf(-kappa * (r - radsum));
                const float t1 = r2 * r2 + radsubsq * radsubsq - 2.0f * r2 * radsumsq;
                const float atr_divr = -32.0f * A / 3.0f * radprod * radprod * radprod / (t1 * t1);
                F = rep + atr_divr * r;
                V = rep / kappa - radprod / rmdsqs * A / 3.0f - radprod / rmdsqm * A / 3.0f
                    - logf(rmdsqs / rmdsqm) * A / 6.0f;
                break;
                }
            case GB_RADIAL_FOURIER:
                {
                const float rc = p.aux;
                const float k = 3.14159265358979f / rc;
                const float x = r * k;
                const float ir = 1.0f / r, ir2 = ir * ir, ir3 = ir * ir2;
                const float ir12 = ir3 * ir3 * ir3 * ir3;
                // the n = 1 coefficients follow from V(r_c) = 0 and V'(r_c) = 0
                float a1s = 0.0f, b1s = 0.0f;
                for (int n = 2; n < 5; n++)
                    {
                    const float sgn = (n & 1) ? -1.0f : 1.0f;
                    a1s += sgn * v[n - 2];
                    b1s += (float)n * sgn * v[n + 1];
                    }
                float s, c;
                sincosf(x, &s, &c);
                float four = a1s * c + b1s * s;
                float dfour = a1s * s - b1s * c; // -(d/dx) of the n = 1 terms
                for (int n = 2; n < 5; n++)
                    {
                    sincosf((float)n * x, &s, &c);
                    four += v[n - 2] * c + v[n + 1] * s;
                    dfour += (float)n * (v[n - 2] * s - v[n + 1] * c);
                    }
                V = ir12 + ir2 * four;
                F = 12.0f * ir12 * ir + ir2 * k * dfour + 2.0f * ir3 * four;
                break;
                }
            case GB_RADIAL_MOLIERE:
            case GB_RADIAL_ZBL:
                {
                const float Zsq = v[0] * v[1], aF = v[2];
                if (Zsq == 0.0f || aF == 0.0f)
                    {
                    V = F = 0.0f;
                    break;
                    }
                const float x = r / aF;
                float e = 0.0f, de = 0.0f;
                if (p.kind == GB_RADIAL_MOLIERE)
                    {
                    const float e1 = 0.35f * expf(-0.3f * x), e2 = 0.55f * expf(-1.2f * x),
                                e3 = 0.1f * expf(-6.0f * x);
                    e = e1 + e2 + e3;
                    de = 0.3f * e1 + 1.2f * e2 + 6.0f * e3;
                    }
                else
                    {
                    const float e1 = 0.1818f * expf(-3.2f * x), e2 = 0.5099f * expf(-0.9423f * x),
                                e3 = 0.2802f * expf(-0.4029f * x),
                                e4 = 0.02817f * expf(-0.2016f * x);
                    e = e1 + e2 + e3 + e4;
                    de = 3.2f * e1 + 0.9423f * e2 + 0.4029f * e3 + 0.2016f * e4;
                    }
                V = Zsq / r * e;
                F = Zsq / (r * r) * e + Zsq / r * de / aF;
                break;
                }
            case GB_RADIAL_EWALD:
                {
                // real-space Ewald sum with a Gaussian-smeared screening alpha
                // (EvaluatorPairEwald.h:121-148), unit charges
                const float kappa = v[0], alpha = v[1];
                const float a1 = kappa * r + alpha / (2.0f * kappa);
                const float a2 = kappa * r - alpha / (2.0f * kappa);
                const float e1 = expf(alpha * r), e2 = expf(-alpha * r);
                const float c1 = erfcf(a1), c2 = erfcf(a2);
                const float val = 0.5f * (c1 * e1 + c2 * e2) / r;
                V = val;
                F = (val + e2 * 2.0f * kappa * expf(-a2 * a2) * 0.564189583547756f
                     + alpha * 0.5f * e2 * c2 - alpha * 0.5f * e1 * c1)
                    / r;
                break;
                }
            case GB_RADIAL_REACTION_FIELD:
                {
                const float eps = v[0], epsrf = v[1], rc = p.aux;
                const float rc3inv = 1.0f / (rc * rc * rc);
                const float eps_fac = epsrf == 0.0f ? 0.5f * rc3inv
                                                    : (epsrf - 1.0f) / (2.0f * epsrf + 1.0f) * rc3inv;
                V = eps * (1.0f / r + eps_fac * r * r);
                F = eps * (1.0f / (r * r) - 2.0f * eps_fac * r);
                break;
                }
            default: // GB_RADIAL_TWF
                {
                const float is2 = 1.0f / (v[0] * v[0]);
                const float t = r * r * is2 - 1.0f;
                const float it3 = 1.0f / (t * t * t);
                const float pre = 4.0f * v[1] / (v[2] * v[2]);
                V = pre * (it3 * it3 - v[2] * it3);
                F = pre * (6.0f * it3 * it3 - 3.0f * v[2] * it3) / t * 2.0f * r * is2;
                break;
                }
            }
        }

    __device__ __forceinline__ bool evalForceAndEnergy(float& force_divr, float& pair_eng,
                                                       bool energy_shift) const
        {
        if (!(rsq < rcutsq))
            return false;
        const float r = sqrtf(rsq);
        float V, F;
        eval(p, r, V, F);
        if (p.kind == GB_RADIAL_FORCE_SHIFTED_LJ)
            V += (r - sqrtf(rcutsq)) * p.aux;
        if (energy_shift)
            {
            float Vc, Fc;
            eval(p, sqrtf(rcutsq), Vc, Fc);
            V -= Vc;
            }
        force_divr = F / r;
        pair_eng = V;
        if (Q)
            {
            force_divr *= qiqj;
            pair_eng *= qiqj;
            }
        return true;
        }
    };
using EvalRadial = EvalRadialT<false>;
using EvalRadialQ = EvalRadialT<true>;

} // namespace gb
