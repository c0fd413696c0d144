// DPD thermostat pair forces (the reference's PotentialPairDPDThermo with EvaluatorPairDPDThermoDPD
// and EvaluatorPairDPDThermoLJ): one thread per particle over the column-major list interleaved
// by 4. Beside the neighbour's position the pair needs its velocity and tag; the random number of
// a pair is drawn from both tags in a fixed order, so i and j compute equal and opposite forces
// from the same draw without sharing any state.
#include "gb_device.cuh"
#include "gb_host.h"
#include "rng.cuh"

namespace gb
{
namespace
{
template<bool LJ, bool MULTI, bool VIRIAL>
__global__ void __launch_bounds__(256)
    k_pair_dpd(float4* __restrict__ d_force, float* __restrict__ d_virial, size_t pitch,
               unsigned int N, const float4* __restrict__ d_pos,
               const float4* __restrict__ d_vel, const uint32_t* __restrict__ d_tag, gb_box box,
               const unsigned int* __restrict__ d_n_neigh, const uint4* __restrict__ d_nlist4,
               uint64_t stride, const gb_dpd_param* __restrict__ d_params,
               const float* __restrict__ d_rcutsq, unsigned int ntypes, bool shift,
               uint64_t timestep, uint16_t seed, float dt, float kT, bool ortho)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N)
        return;
    const float4 pi = __ldg(d_pos + i);
    const float4 vi = __ldg(d_vel + i);
    const uint32_t tagi = __ldg(d_tag + i);
    const unsigned int ti = __float_as_uint(pi.w);
    const unsigned int nn = d_n_neigh[i];
    float fx = 0.f, fy = 0.f, fz = 0.f, pe = 0.f;
    float vxx = 0.f, vxy = 0.f, vxz = 0.f, vyy = 0.f, vyz = 0.f, vzz = 0.f;
    for (unsigned int k = 0; k < nn; k++)
        {
        const unsigned int j = __ldg(reinterpret_cast<const unsigned int*>(
                                         d_nlist4 + (uint64_t)(k >> 2) * stride + i)
                                     + (k & 3u));
        const float4 pj = __ldg(d_pos + j);
        float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        if (ortho)
            min_image_ortho(box, dx, dy, dz);
        else
            min_image(box, dx, dy, dz);
        const float rsq = dx * dx + dy * dy + dz * dz;
        const unsigned int tp = MULTI ? ti * ntypes + __float_as_uint(pj.w) : 0u;
        const float rcutsq = __ldg(d_rcutsq + tp);
        if (!(rsq < rcutsq))
            continue;
        const gb_dpd_param p = d_params[tp];
        if (LJ && p.lj1 == 0.0f)
            continue;
        const float4 vj = __ldg(d_vel + j);
        const uint32_t tagj = __ldg(d_tag + j);
        const float rdotv = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
        const float rinv = rsqrtf(rsq);
        const float rcutinv = rsqrtf(rcutsq);
        Philox rng(22, timestep, seed, min(tagi, tagj), max(tagi, tagj));
        const float alpha = uniform_m11_f(rng);
        float force_divr, pair_eng;
        if (LJ)
            {
            const float r2inv = 1.0f / rsq;
            const float r6inv = r2inv * r2inv * r2inv;
            force_divr = r2inv * r6inv * (12.0f * p.lj1 * r6inv - 6.0f * p.lj2);
            pair_eng = r6inv * (p.lj1 * r6inv - p.lj2);
            if (shift)
                {
                const float rc2inv = 1.0f / rcutsq;
                const float rc6inv = rc2inv * rc2inv * rc2inv;
                pair_eng -= rc6inv * (p.lj1 * rc6inv - p.lj2);
                }
            }
        else
            {
            const float r = 1.0f / rinv, rcut = 1.0f / rcutinv;
            force_divr = p.a * (rinv - rcutinv);
            pair_eng = p.a * (rcut - r) - 0.5f * p.a * rcutinv * (rcutsq - rsq);
            }
        const float force_divr_cons = force_divr;
        const float w = rinv - rcutinv;
        force_divr -= p.gamma * rdotv * w * w;
        force_divr += rsqrtf(dt / (kT * p.gamma * 6.0f)) * w * alpha;
        fx += dx * force_divr;
        fy += dy * force_divr;
        fz += dz * force_divr;
        pe += pair_eng;
        if (VIRIAL)
            {
            const float h = 0.5f * force_divr_cons;
            vxx += dx * dx * h;
            vxy += dx * dy * h;
            vxz += dx * dz * h;
            vyy += dy * dy * h;
            vyz += dy * dz * h;
            vzz += dz * dz * h;
            }
        }
    d_force[i] = make_float4(fx, fy, fz, 0.5f * pe);
    if (VIRIAL)
        {
        d_virial[0 * pitch + i] = vxx;
        d_virial[1 * pitch + i] = vxy;
        d_virial[2 * pitch + i] = vxz;
        d_virial[3 * pitch + i] = vyy;
        d_virial[4 * pitch + i] = vyz;
        d_virial[5 * pitch + i] = vzz;
        }
    }

template<bool LJ, bool MULTI>
void launch_dpd(const gb_pair_args& a, const gb_dpd_param* d_params, const float* d_vel,
                const uint32_t* d_tag, uint64_t timestep, uint16_t seed, float dt, float kT,
                cudaStream_t s)
    {
    const bool ortho = a.box.xy == 0.0f && a.box.xz == 0.0f && a.box.yz == 0.0f;
    auto kern = a.compute_virial ? k_pair_dpd<LJ, MULTI, true> : k_pair_dpd<LJ, MULTI, false>;
    kern<<<div_up(a.N, 256), 256, 0, s>>>(
        reinterpret_cast<float4*>(a.d_force), a.d_virial, a.virial_pitch, a.N,
        reinterpret_cast<const float4*>(a.d_pos), reinterpret_cast<const float4*>(d_vel), d_tag,
        a.box, a.d_n_neigh, reinterpret_cast<const uint4*>(a.d_nlist), a.stride, d_params,
        a.d_rcutsq, a.ntypes, a.shift_mode == 1, timestep, seed, dt, kT, ortho);
    }
} // namespace
} // namespace gb

using namespace gb;

extern "C"
    {
    int gb_pair_forces_dpd(const gb_pair_args* args, const gb_dpd_param* d_params,
                           const float* d_vel, const uint32_t* d_tag, int lj, uint64_t timestep,
                           uint16_t seed, float dt, float kT, void* stream)
        {
        GB_REQUIRE(args, "gb_pair_forces_dpd: null args");
        const gb_pair_args& a = *args;
        GB_REQUIRE(a.d_force && a.d_pos && a.d_n_neigh && a.d_nlist && a.d_rcutsq && d_params
                       && d_vel && d_tag,
                   "gb_pair_forces_dpd: null device pointer");
        GB_REQUIRE(!a.d_head_list && a.interleave == 4 && a.stride >= a.N,
                   "gb_pair_forces_dpd: column-major list interleaved by 4 required");
        GB_REQUIRE(!a.compute_virial || (a.d_virial && a.virial_pitch >= a.N),
                   "gb_pair_forces_dpd: virial requested without a buffer of pitch >= N");
        GB_REQUIRE(a.shift_mode <= 1, "gb_pair_forces_dpd: shift_mode 0 or 1");
        GB_REQUIRE(a.ntypes >= 1, "gb_pair_forces_dpd: ntypes >= 1");
        if (a.N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        const bool multi = a.ntypes > 1;
        if (lj)
            multi ? launch_dpd<true, true>(a, d_params, d_vel, d_tag, timestep, seed, dt, kT, s)
                  : launch_dpd<true, false>(a, d_params, d_vel, d_tag, timestep, seed, dt, kT, s);
        else
            multi ? launch_dpd<false, true>(a, d_params, d_vel, d_tag, timestep, seed, dt, kT, s)
                  : launch_dpd<false, false>(a, d_params, d_vel, d_tag, timestep, seed, dt, kT, s);
        return check_launch("gb_pair_forces_dpd");
        }
    }
