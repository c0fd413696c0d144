// The pair-force kernel template (PotentialPair<Evaluator> on GB300) and its launcher.
//
// Replaces gpu_compute_pair_forces_shared_kernel (hoomd/md/PotentialPairGPU.cuh:140-404).
// Layouts: with a column-major neighbour list (head(i) = i, stride >= N) one thread owns one
// particle and neighbour k of 32 consecutive particles is one 128-byte load, so the index stream
// -- the dominant HBM traffic -- is read exactly once, coalesced, with no shuffle reductions.
// With the reference's flat head-list layout, groups of TPP threads share a particle and reduce
// with warp shuffles, as the reference does. Per-pair parameters, r_cut^2 and r_on^2 are staged
// in shared memory when there is more than one type and held in registers otherwise.
//
// FUSE adds the integrator's second half step and the FP64 thermodynamic reductions to the
// epilogue (TwoStepConstantVolume step two, hoomd/md/TwoStepConstantVolumeGPU.cu:166-205; thermo,
// hoomd/md/ComputeThermo.cc:76-290): the force never makes a round trip through HBM before it is
// used, and the last block to finish reduces the per-block partial sums in a fixed order and
// draws the Bussi factor for the next step on the device (no host synchronisation per step).
#pragma once

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "evaluators.cuh"
#include "gb_device.cuh"
#include "gb_host.h"
#include "rng.cuh"

namespace gb
{

// Epilogue state for the fused step (device pointers are caller-owned).
struct FuseArgs
    {
    float4* vel;            // float4[N] in/out
    float* accel;           // float3[N] out
    float dt;
    const double* d_scale2; // step-two rescale factor (NULL = 1)
    double* partials;       // [3 * gridDim.x] scratch
    unsigned int* counter;  // zero before the launch; left zero
    double* out;            // [3]: KE, PE, W
    int bussi;              // draw the factor for the next step into d_factor
    double dof, tau, kT, dt_d;
    uint16_t seed;
    uint32_t instance_id;
    uint64_t* d_timestep;   // current step; advanced by one by the last block
    double* d_factor;
    uint32_t* d_status;     // bit 0: Bussi with zero kinetic energy
    uint32_t* d_rebuild_reset;
    const double2* d_ring;  // optional pre-drawn Bussi draws, indexed by timestep % ring_size
    unsigned int ring_size;
    int langevin;           // Langevin step two instead of the rescaled one
    const uint32_t* tag;    // [N] tags (Langevin random-number counters)
    const float4* pos;      // [N] positions, type in w
    const float* gamma;     // [ntypes] drag coefficients
    float lkT;
    unsigned int ndim;
    double* d_reservoir;    // optional Langevin reservoir energy
    int berendsen;          // draw-free Berendsen factor for the next step one into d_factor
    int brownian;           // no second half (Brownian dynamics): sums only
    };

template<int TPP> __device__ __forceinline__ double block_sum_d(double v, double* s_red)
    {
    v = warp_sum(v);
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    if (lane == 0)
        s_red[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0)
        {
        const int nw = blockDim.x / 32;
        r = (lane < nw) ? s_red[lane] : 0.0;
        r = warp_sum(r);
        }
    __syncthreads();
    return r; // valid in thread 0
    }

// Step two of the integrator for particle gi from its net force (fx, fy, fz_), and the
// particle's FP64 terms of the step's sums: 2 KE, PE, and for Langevin F_bd . v.
__device__ __forceinline__ void fuse_step_two(const FuseArgs& fz, unsigned int gi, float fx,
                                              float fy, float fz_, float pe, double& ke_d,
                                              double& pe_d, double& w_d)
    {
    float4 v = fz.vel[gi];
    if (fz.brownian)
        {
        ke_d = (double)v.w
               * ((double)v.x * (double)v.x + (double)v.y * (double)v.y
                  + (double)v.z * (double)v.z);
        pe_d = (double)pe;
        return;
        }
    const float minv = __frcp_rn(v.w);
    float ax, ay, az;
    if (fz.langevin)
        {
        // hoomd/md/TwoStepLangevin.cc:248-292: F_bd = r * sqrt(6 gamma kT / dt) - gamma v with
        // r uniform in [-1, 1] (three draws, Seed(25, timestep, seed), Counter(tag)),
        // a = (F + F_bd) / m, v += (a / 2) dt
        const unsigned int type = __float_as_uint(__ldg(fz.pos + gi).w);
        const float gamma = __ldg(fz.gamma + type);
        const float coeff
            = __fsqrt_rn(__fdiv_rn(__fmul_rn(__fmul_rn(6.0f, gamma), fz.lkT), fz.dt));
        Philox rng(25, *fz.d_timestep, fz.seed, __ldg(fz.tag + gi));
        const float rx = uniform_m11_f(rng);
        const float ry = uniform_m11_f(rng);
        const float rz = uniform_m11_f(rng);
        const float bx = __fsub_rn(__fmul_rn(rx, coeff), __fmul_rn(gamma, v.x));
        const float by = __fsub_rn(__fmul_rn(ry, coeff), __fmul_rn(gamma, v.y));
        const float bz
            = fz.ndim < 3 ? 0.0f : __fsub_rn(__fmul_rn(rz, coeff), __fmul_rn(gamma, v.z));
        ax = __fmul_rn(__fadd_rn(fx, bx), minv);
        ay = __fmul_rn(__fadd_rn(fy, by), minv);
        az = __fmul_rn(__fadd_rn(fz_, bz), minv);
        v.x = __fadd_rn(v.x, __fmul_rn(__fmul_rn(0.5f, ax), fz.dt));
        v.y = __fadd_rn(v.y, __fmul_rn(__fmul_rn(0.5f, ay), fz.dt));
        v.z = __fadd_rn(v.z, __fmul_rn(__fmul_rn(0.5f, az), fz.dt));
        w_d = (double)bx * (double)v.x + (double)by * (double)v.y + (double)bz * (double)v.z;
        }
    else
        {
        // a = F/m, v = v*s + dt/2 * a (TwoStepConstantVolume.cc:213-261 order)
        ax = __fmul_rn(fx, minv);
        ay = __fmul_rn(fy, minv);
        az = __fmul_rn(fz_, minv);
        const float s2 = fz.d_scale2 ? (float)*fz.d_scale2 : 1.0f;
        const float hdt = __fmul_rn(0.5f, fz.dt);
        v.x = __fadd_rn(__fmul_rn(v.x, s2), __fmul_rn(hdt, ax));
        v.y = __fadd_rn(__fmul_rn(v.y, s2), __fmul_rn(hdt, ay));
        v.z = __fadd_rn(__fmul_rn(v.z, s2), __fmul_rn(hdt, az));
        }
    fz.vel[gi] = v;
    fz.accel[3 * (size_t)gi + 0] = ax;
    fz.accel[3 * (size_t)gi + 1] = ay;
    fz.accel[3 * (size_t)gi + 2] = az;
    ke_d = (double)v.w
           * ((double)v.x * (double)v.x + (double)v.y * (double)v.y + (double)v.z * (double)v.z);
    pe_d = (double)pe;
    }

__device__ inline void fuse_finish(const FuseArgs& fz, double ke, double pe, double w)
    {
    __shared__ double s_red[32];
    __shared__ bool s_last;
    ke = block_sum_d<1>(ke, s_red);
    pe = block_sum_d<1>(pe, s_red);
    w = block_sum_d<1>(w, s_red);
    if (threadIdx.x == 0)
        {
        fz.partials[3 * blockIdx.x + 0] = ke;
        fz.partials[3 * blockIdx.x + 1] = pe;
        fz.partials[3 * blockIdx.x + 2] = w;
        __threadfence();
        const unsigned int done = atomicAdd(fz.counter, 1u);
        s_last = (done == gridDim.x - 1);
        }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    // last block: fixed-order reduction of the partials (deterministic)
    double a = 0.0, b = 0.0, c = 0.0;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x)
        {
        a += __ldcg(fz.partials + 3 * k + 0);
        b += __ldcg(fz.partials + 3 * k + 1);
        c += __ldcg(fz.partials + 3 * k + 2);
        }
    a = block_sum_d<1>(a, s_red);
    b = block_sum_d<1>(b, s_red);
    c = block_sum_d<1>(c, s_red);
    if (threadIdx.x == 0)
        {
        const double K = 0.5 * a;
        fz.out[0] = K;
        fz.out[1] = b;
        fz.out[2] = fz.langevin ? 0.0 : c / 3.0;
        // the Langevin tally: c = sum of F_bd . v (hoomd/md/TwoStepLangevin.cc:396-412)
        if (fz.langevin && fz.d_reservoir)
            *fz.d_reservoir -= c * fz.dt_d;
        if (fz.berendsen)
            {
            if (fz.dof != 0.0 && K <= 0.0)
                {
                atomicOr(fz.d_status, 2u);
                *fz.d_factor = 1.0;
                }
            else
                *fz.d_factor = berendsen_factor_d(K, fz.dof, fz.dt_d, fz.tau, fz.kT);
            }
        if (fz.bussi)
            {
            const uint64_t next = *fz.d_timestep + 1;
            if (K <= 0.0)
                {
                atomicOr(fz.d_status, 1u);
                *fz.d_factor = 1.0;
                }
            else if (fz.d_ring)
                *fz.d_factor = bussi_factor_from_draws(K, fz.dof, fz.dt_d, fz.tau, fz.kT,
                                                       fz.d_ring[next % fz.ring_size]);
            else
                *fz.d_factor = bussi_factor_d(K, fz.dof, fz.dt_d, fz.tau, fz.kT, next, fz.seed,
                                              fz.instance_id);
            }
        if (fz.d_timestep)
            *fz.d_timestep += 1;
        if (fz.d_rebuild_reset)
            *fz.d_rebuild_reset = 0u;
        *fz.counter = 0;
        }
    }

// Template parameters select the data path (evaluator, threads per particle, layout, type
// tables, fused epilogue); shift mode, virial and box shape are uniform runtime branches.
// XPLOR smoothing between r_on and r_cut (applied by the reference's force loop,
// hoomd/md/PotentialPair.h:711-737). With w = r_cut^2 - r_on^2 and u = r_cut^2 - r^2, the energy is
// multiplied by S = u^2 (r_cut^2 + 2 r^2 - 3 r_on^2) / w^3, and since dS/d(r^2) =
// -6 u (r^2 - r_on^2) / w^3, the force over r becomes S F/r + 12 V u (r^2 - r_on^2) / w^3.
__device__ __forceinline__ void xplor_smooth(float rsq, float rcutsq, float ronsq,
                                             float& force_divr, float& pair_eng)
    {
    const float w = rcutsq - ronsq;
    const float inv_w3 = 1.0f / (w * w * w);
    const float u = rcutsq - rsq;
    const float smooth = u * u * (rcutsq + 2.0f * rsq - 3.0f * ronsq) * inv_w3;
    const float slope = 12.0f * u * (rsq - ronsq) * inv_w3;
    force_divr = smooth * force_divr + slope * pair_eng;
    pair_eng *= smooth;
    }

template<class Eval, int TPP, bool FLAT, bool MULTI, bool FUSE>
__global__ void __launch_bounds__(256)
    k_pair(float4* __restrict__ d_force, float* __restrict__ d_virial, size_t pitch,
           unsigned int N, const float4* __restrict__ d_pos, gb_box box,
           const unsigned int* __restrict__ d_n_neigh, const unsigned int* __restrict__ d_nlist,
           const uint64_t* __restrict__ d_head_list, uint64_t stride,
           const typename Eval::param_type* __restrict__ d_params,
           const float* __restrict__ d_rcutsq, const float* __restrict__ d_ronsq,
           unsigned int ntypes, const float* __restrict__ ext,
           const float* __restrict__ d_charge, int SHIFT, bool VIRIAL, bool ORTHO, FuseArgs fz)
    {
    using P = typename Eval::param_type;
    extern __shared__ __align__(16) unsigned char s_raw[];
    P* s_params = reinterpret_cast<P*>(s_raw);
    const unsigned int np = ntypes * ntypes;
    float* s_rcutsq = reinterpret_cast<float*>(s_raw + sizeof(P) * np);
    float* s_ronsq = s_rcutsq + np;
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < np; t += blockDim.x)
            {
            P pt = d_params[t];
            Eval::prepare_param(pt, d_rcutsq[t]);
            s_params[t] = pt;
            s_rcutsq[t] = d_rcutsq[t];
            if (SHIFT == 2)
                s_ronsq[t] = d_ronsq[t];
            }
        __syncthreads();
        }
    P p0;
    float rc0 = 0.0f, ro0 = 0.0f;
    if (!MULTI)
        {
        p0 = d_params[0];
        rc0 = d_rcutsq[0];
        Eval::prepare_param(p0, rc0);
        if (SHIFT == 2)
            ro0 = d_ronsq[0];
        }

    const unsigned int gi = blockIdx.x * (blockDim.x / TPP) + threadIdx.x / TPP;
    const unsigned int lane = threadIdx.x % TPP;
    const bool active = gi < N;

    float fx = 0.f, fy = 0.f, fz_ = 0.f, pe = 0.f;
    float vxx = 0.f, vxy = 0.f, vxz = 0.f, vyy = 0.f, vyz = 0.f, vzz = 0.f;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active)
        {
        const unsigned int nn = d_n_neigh[gi];
        pi = __ldg(d_pos + gi);
        const unsigned int ti = __float_as_uint(pi.w);
        const uint64_t head = FLAT ? d_head_list[gi] : (uint64_t)gi;
        const uint64_t step = FLAT ? 1ull : stride;
        auto pair = [&](unsigned int j) {
            const float4 pj = __ldg(d_pos + j);
            float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            if (ORTHO)
                min_image_ortho(box, dx, dy, dz);
            else
                min_image(box, dx, dy, dz);
            const float rsq = dx * dx + dy * dy + dz * dz;
            const P* param;
            float rcutsq, ronsq = 0.0f;
            if (MULTI)
                {
                const unsigned int tp = ti * ntypes + __float_as_uint(pj.w);
                param = s_params + tp;
                rcutsq = s_rcutsq[tp];
                if (SHIFT == 2)
                    ronsq = s_ronsq[tp];
                }
            else
                {
                param = &p0;
                rcutsq = rc0;
                ronsq = ro0;
                }
            bool energy_shift = (SHIFT == 1) || (SHIFT == 2 && ronsq > rcutsq);
            float force_divr = 0.0f, pair_eng = 0.0f;
            Eval eval(rsq, rcutsq, *param, ext);
            if (Eval::needsCharge())
                eval.setCharge(__ldg(d_charge + gi), __ldg(d_charge + j));
            eval.evalForceAndEnergy(force_divr, pair_eng, energy_shift);
            if (SHIFT == 2)
                {
                if (rsq >= ronsq && rsq < rcutsq)
                    xplor_smooth(rsq, rcutsq, ronsq, force_divr, pair_eng);
                }
            if (VIRIAL)
                {
                const float force_div2r = 0.5f * force_divr;
                vxx += dx * dx * force_div2r;
                vxy += dx * dy * force_div2r;
                vxz += dx * dz * force_div2r;
                vyy += dy * dy * force_div2r;
                vyz += dy * dz * force_div2r;
                vzz += dz * dz * force_div2r;
                }
            fx += dx * force_divr;
            fy += dy * force_divr;
            fz_ += dz * force_divr;
            pe += pair_eng;
        };
        unsigned int k = lane;
        // four independent index loads and gathers in flight per thread
        for (; k + 3 * TPP < nn; k += 4 * TPP)
            {
            const unsigned int j0 = __ldg(d_nlist + head + (uint64_t)k * step);
            const unsigned int j1 = __ldg(d_nlist + head + (uint64_t)(k + TPP) * step);
            const unsigned int j2 = __ldg(d_nlist + head + (uint64_t)(k + 2 * TPP) * step);
            const unsigned int j3 = __ldg(d_nlist + head + (uint64_t)(k + 3 * TPP) * step);
            pair(j0);
            pair(j1);
            pair(j2);
            pair(j3);
            }
        for (; k < nn; k += TPP)
            pair(__ldg(d_nlist + head + (uint64_t)k * step));
        pe *= 0.5f;
        }
    if (TPP > 1)
        {
        fx = group_sum<TPP>(fx);
        fy = group_sum<TPP>(fy);
        fz_ = group_sum<TPP>(fz_);
        pe = group_sum<TPP>(pe);
        if (VIRIAL)
            {
            vxx = group_sum<TPP>(vxx);
            vxy = group_sum<TPP>(vxy);
            vxz = group_sum<TPP>(vxz);
            vyy = group_sum<TPP>(vyy);
            vyz = group_sum<TPP>(vyz);
            vzz = group_sum<TPP>(vzz);
            }
        }
    double ke_d = 0.0, pe_d = 0.0, w_d = 0.0;
    if (active && lane == 0)
        {
        d_force[gi] = make_float4(fx, fy, fz_, pe);
        if (VIRIAL)
            {
            d_virial[0 * pitch + gi] = vxx;
            d_virial[1 * pitch + gi] = vxy;
            d_virial[2 * pitch + gi] = vxz;
            d_virial[3 * pitch + gi] = vyy;
            d_virial[4 * pitch + gi] = vyz;
            d_virial[5 * pitch + gi] = vzz;
            w_d = (double)vxx + (double)vyy + (double)vzz;
            }
        if (FUSE)
            fuse_step_two(fz, gi, fx, fy, fz_, pe, ke_d, pe_d, w_d);
        }
    if (FUSE)
        fuse_finish(fz, ke_d, pe_d, w_d);
    }

// Fast path for the column-major list interleaved by 4 (gb_nlist_args.interleave = 4): one thread
// per particle reads four neighbour indices with one 16-byte streaming load (a warp reads 512
// contiguous bytes), keeps the next two index batches in flight while the current four position
// gathers and pair evaluations run, and masks the tail of the list by substituting the particle
// itself (a valid address) and discarding its result.
__device__ __forceinline__ uint4 ld_stream_u4(const uint4* p)
    {
    return __ldcs(p);
    }

// bytes of the per-type tables at the start of the kernel's dynamic shared memory, rounded to 16
template<class P> __host__ __device__ inline size_t i4_param_bytes(unsigned int ntypes, bool multi)
    {
    return multi ? ((sizeof(P) + 2 * sizeof(float)) * ntypes * ntypes + 15) / 16 * 16 : 0;
    }

// TPP > 1 (small systems): TPP consecutive lanes share one particle, lane l taking the groups of
// four neighbours b = l, l + TPP, ... (the reference's threads-per-particle split,
// hoomd/md/PotentialPairGPU.cuh:140-404), and the partial sums meet by shuffles.
template<class Eval, bool MULTI, bool ORTHO, bool FUSE, bool VIRIAL, bool XPLOR, int TPP = 1>
__global__ void __launch_bounds__(256, (FUSE || VIRIAL || XPLOR) ? 4 : 5)
    k_pair_i4(float4* __restrict__ d_force, float* __restrict__ d_virial, size_t pitch,
              unsigned int N, const float4* __restrict__ d_pos, gb_box box,
              const unsigned int* __restrict__ d_n_neigh, const uint4* __restrict__ d_nlist4,
              uint64_t stride, const typename Eval::param_type* __restrict__ d_params,
              const float* __restrict__ d_rcutsq, const float* __restrict__ d_ronsq,
              unsigned int ntypes, const float* __restrict__ ext,
              const float* __restrict__ d_charge, bool SHIFT1, FuseArgs fz)
    {
    using P = typename Eval::param_type;
    extern __shared__ __align__(16) unsigned char s_raw[];
    P* s_params = reinterpret_cast<P*>(s_raw);
    const unsigned int np = ntypes * ntypes;
    float* s_rcutsq = reinterpret_cast<float*>(s_raw + sizeof(P) * np);
    float* s_ronsq = s_rcutsq + np;
    // largest r_cut^2 of any type pair (non-negative floats order as their bit patterns)
    __shared__ unsigned int s_rcmax[8];
    unsigned int rcmax_bits = 0;
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < np; t += blockDim.x)
            {
            P pt = d_params[t];
            Eval::prepare_param(pt, d_rcutsq[t]);
            s_params[t] = pt;
            s_rcutsq[t] = d_rcutsq[t];
            rcmax_bits = max(rcmax_bits, __float_as_uint(fmaxf(d_rcutsq[t], 0.0f)));
            if (XPLOR)
                s_ronsq[t] = d_ronsq[t];
            }
        rcmax_bits = __reduce_max_sync(0xffffffffu, rcmax_bits);
        if (threadIdx.x % 32 == 0)
            s_rcmax[threadIdx.x / 32] = rcmax_bits;
        __syncthreads();
        for (unsigned int w = 0; w < blockDim.x / 32; w++)
            rcmax_bits = max(rcmax_bits, s_rcmax[w]);
        }
    P p0;
    float rc0 = 0.0f, ro0 = 0.0f;
    if (!MULTI)
        {
        p0 = d_params[0];
        rc0 = d_rcutsq[0];
        Eval::prepare_param(p0, rc0);
        if (XPLOR)
            ro0 = d_ronsq[0];
        rcmax_bits = __float_as_uint(fmaxf(rc0, 0.0f));
        }
    // Wrap-free warps. A particle at least r_cut (plus a margin) from every face of an
    // orthorhombic box has all its partners within r_cut at their stored positions without an
    // image shift, so minimum image changes no pair inside r_cut; a pair that it would shift
    // lies beyond r_cut either way (the raw separation then exceeds L - r_cut >= r_cut) and
    // contributes zero. Warps whose particles all qualify skip the image arithmetic.
    const float rcmax = sqrtf(__uint_as_float(rcmax_bits)) * 1.001f + 1e-6f;
    const float hx = 0.5f * box.L[0] - rcmax, hy = 0.5f * box.L[1] - rcmax,
                hz = 0.5f * box.L[2] - rcmax;

    const unsigned int sub = threadIdx.x % TPP;
    // Resident grid: each warp walks chunks of 32 threads, warp w of the grid taking chunks
    // w, w + W, ... (W = warps in the grid), so a block meets its FP64 reduction barrier once,
    // after several chunks, instead of after one chunk whose slowest warp holds the rest.
    double ke_d = 0.0, pe_d = 0.0, w_d = 0.0;
    const uint64_t grid_threads = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
         t0 < (uint64_t)N * TPP; t0 += grid_threads)
    {
    const unsigned int i = (unsigned int)((t0 + (threadIdx.x & 31u)) / TPP);
    const bool active = i < N;
    float fx = 0.f, fy = 0.f, fz_ = 0.f, pe = 0.f;
    float vxx = 0.f, vxy = 0.f, vxz = 0.f, vyy = 0.f, vyz = 0.f, vzz = 0.f;
    const float4 pi = active ? __ldg(d_pos + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool wrap_free
        = ORTHO
          && __all_sync(0xffffffffu, !active
                                         || (fabsf(pi.x) < hx && fabsf(pi.y) < hy
                                             && fabsf(pi.z) < hz));
    if (active)
        {
        const unsigned int nn = d_n_neigh[i];
        const unsigned int ti = __float_as_uint(pi.w);
        // minimum image with fused multiply-adds (forces are held to a tolerance; only the
        // neighbour-list build needs minImage's exact roundings); every direction periodic
        const float Lx = box.L[0], Ly = box.L[1], Lz = box.L[2];
        const float Lix = box.Linv[0], Liy = box.Linv[1], Liz = box.Linv[2];
        const float Lzxz = box.L[2] * box.xz, Lzyz = box.L[2] * box.yz, Lyxy = box.L[1] * box.xy;
        const float qi = Eval::needsCharge() ? __ldg(d_charge + i) : 0.0f;
        auto pair = [&](auto wrap, const float4 pj, unsigned int j, bool valid) {
            float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            if (ORTHO)
                {
                if (decltype(wrap)::value)
                    {
                    dx -= Lx * rintf(dx * Lix);
                    dy -= Ly * rintf(dy * Liy);
                    dz -= Lz * rintf(dz * Liz);
                    }
                }
            else
                {
                const float iz = rintf(dz * Liz);
                dz -= Lz * iz;
                dy -= Lzyz * iz;
                dx -= Lzxz * iz;
                const float iy = rintf(dy * Liy);
                dy -= Ly * iy;
                dx -= Lyxy * iy;
                dx -= Lx * rintf(dx * Lix);
                }
            const float rsq = dx * dx + dy * dy + dz * dz;
            const P* param;
            float rcutsq, ronsq = 0.0f;
            if (MULTI)
                {
                const unsigned int tp = ti * ntypes + __float_as_uint(pj.w);
                param = s_params + tp;
                rcutsq = s_rcutsq[tp];
                if (XPLOR)
                    ronsq = s_ronsq[tp];
                }
            else
                {
                param = &p0;
                rcutsq = rc0;
                ronsq = ro0;
                }
            const bool energy_shift = XPLOR ? (ronsq > rcutsq) : SHIFT1;
            float force_divr = 0.0f, pair_eng = 0.0f;
            Eval eval(rsq, rcutsq, *param, ext);
            if (Eval::needsCharge())
                eval.setCharge(qi, __ldg(d_charge + j));
            eval.evalForceAndEnergy(force_divr, pair_eng, energy_shift);
            if (XPLOR && rsq >= ronsq && rsq < rcutsq)
                xplor_smooth(rsq, rcutsq, ronsq, force_divr, pair_eng);
            if (!valid)
                {
                force_divr = 0.0f;
                pair_eng = 0.0f;
                }
            if (VIRIAL)
                {
                const float force_div2r = 0.5f * force_divr;
                vxx += dx * dx * force_div2r;
                vxy += dx * dy * force_div2r;
                vxz += dx * dz * force_div2r;
                vyy += dy * dy * force_div2r;
                vyz += dy * dz * force_div2r;
                vzz += dz * dz * force_div2r;
                }
            fx += dx * force_divr;
            fy += dy * force_divr;
            fz_ += dz * force_divr;
            pe += pair_eng;
        };
        // full groups of four with no per-pair masking, then the partial last group; index
        // loads run two groups ahead of the four independent position gathers
        const unsigned int nfull = nn >> 2;
        const unsigned int rem = nn & 3u;
        const uint4* p4 = d_nlist4 + i;
        auto walk = [&](auto wrap) {
            const uint4 self = make_uint4(i, i, i, i);
            if (TPP > 1)
                {
                // groups sub, sub + TPP, ...; the partial last group belongs to lane nfull % TPP
                for (unsigned int b = sub; b < nfull; b += TPP)
                    {
                    const uint4 jc = ld_stream_u4(p4 + (uint64_t)b * stride);
                    const float4 q0 = __ldg(d_pos + jc.x);
                    const float4 q1 = __ldg(d_pos + jc.y);
                    const float4 q2 = __ldg(d_pos + jc.z);
                    const float4 q3 = __ldg(d_pos + jc.w);
                    pair(wrap, q0, jc.x, true);
                    pair(wrap, q1, jc.y, true);
                    pair(wrap, q2, jc.z, true);
                    pair(wrap, q3, jc.w, true);
                    }
                if (rem && sub == nfull % TPP)
                    {
                    const uint4 jc = ld_stream_u4(p4 + (uint64_t)nfull * stride);
                    const float4 q0 = __ldg(d_pos + jc.x);
                    const float4 q1 = __ldg(d_pos + (rem > 1 ? jc.y : i));
                    const float4 q2 = __ldg(d_pos + (rem > 2 ? jc.z : i));
                    pair(wrap, q0, jc.x, true);
                    pair(wrap, q1, rem > 1 ? jc.y : i, rem > 1);
                    pair(wrap, q2, rem > 2 ? jc.z : i, rem > 2);
                    }
                }
            uint4 jA = self, jB = self;
            if (TPP == 1 && nfull > 0)
                jA = ld_stream_u4(p4);
            if (TPP == 1 && nfull > 1)
                jB = ld_stream_u4(p4 + stride);
            for (unsigned int b = 0; TPP == 1 && b < nfull; b++)
                {
                const uint4 jc = jA;
                jA = jB;
                if (b + 2 < nfull)
                    jB = ld_stream_u4(p4 + (uint64_t)(b + 2) * stride);
                const float4 q0 = __ldg(d_pos + jc.x);
                const float4 q1 = __ldg(d_pos + jc.y);
                const float4 q2 = __ldg(d_pos + jc.z);
                const float4 q3 = __ldg(d_pos + jc.w);
                pair(wrap, q0, jc.x, true);
                pair(wrap, q1, jc.y, true);
                pair(wrap, q2, jc.z, true);
                pair(wrap, q3, jc.w, true);
                }
            if (TPP == 1 && rem)
                {
                const uint4 jc = ld_stream_u4(p4 + (uint64_t)nfull * stride);
                const float4 q0 = __ldg(d_pos + jc.x);
                const float4 q1 = __ldg(d_pos + (rem > 1 ? jc.y : i));
                const float4 q2 = __ldg(d_pos + (rem > 2 ? jc.z : i));
                pair(wrap, q0, jc.x, true);
                pair(wrap, q1, rem > 1 ? jc.y : i, rem > 1);
                pair(wrap, q2, rem > 2 ? jc.z : i, rem > 2);
                }
        };
        if (wrap_free)
            walk(std::false_type {});
        else
            walk(std::true_type {});
        pe *= 0.5f;
        }
    if (TPP > 1)
        {
        fx = group_sum<TPP>(fx);
        fy = group_sum<TPP>(fy);
        fz_ = group_sum<TPP>(fz_);
        pe = group_sum<TPP>(pe);
        if (VIRIAL)
            {
            vxx = group_sum<TPP>(vxx);
            vxy = group_sum<TPP>(vxy);
            vxz = group_sum<TPP>(vxz);
            vyy = group_sum<TPP>(vyy);
            vyz = group_sum<TPP>(vyz);
            vzz = group_sum<TPP>(vzz);
            }
        }
    if (active && sub == 0)
        {
        d_force[i] = make_float4(fx, fy, fz_, pe);
        double ke_i = 0.0, pe_i = 0.0, w_i = 0.0;
        if (VIRIAL)
            {
            d_virial[0 * pitch + i] = vxx;
            d_virial[1 * pitch + i] = vxy;
            d_virial[2 * pitch + i] = vxz;
            d_virial[3 * pitch + i] = vyy;
            d_virial[4 * pitch + i] = vyz;
            d_virial[5 * pitch + i] = vzz;
            w_i = (double)vxx + (double)vyy + (double)vzz;
            }
        if (FUSE)
            {
            fuse_step_two(fz, i, fx, fy, fz_, pe, ke_i, pe_i, w_i);
            ke_d += ke_i;
            pe_d += pe_i;
            w_d += w_i;
            }
        }
    }
    if (FUSE)
        fuse_finish(fz, ke_d, pe_d, w_d);
    }

// Blocks of one kernel resident on the current GPU at once (SM count x blocks per SM), cached
// per kernel, block size, dynamic shared memory size and device.
struct ResidentGrid
    {
    int dev = -1;
    size_t smem = ~size_t(0);
    unsigned int blk = 0;
    unsigned int n = 0;
    unsigned int blocks(const void* kern, unsigned int block, size_t smem_bytes)
        {
        int d = 0;
        cudaGetDevice(&d);
        if (d != dev || smem_bytes != smem || block != blk)
            {
            int sms = 0, per_sm = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)block, smem_bytes);
            n = (unsigned int)std::max(1, sms * std::max(1, per_sm));
            dev = d;
            smem = smem_bytes;
            blk = block;
            }
        return n;
        }
    };

template<class Eval, bool MULTI, bool ORTHO, bool FUSE, bool VIRIAL, bool XPLOR, int TPP = 1>
int launch_pair_i4_inst(const gb_pair_args& a, const typename Eval::param_type* d_params,
                        const float* ext, const FuseArgs& fz, cudaStream_t s)
    {
    const unsigned int block = a.block_size ? a.block_size : 256u;
    const size_t smem = i4_param_bytes<typename Eval::param_type>(a.ntypes, MULTI);
    auto kern = k_pair_i4<Eval, MULTI, ORTHO, FUSE, VIRIAL, XPLOR, TPP>;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // no more blocks than fit on the GPU at once (the kernel loops over the rest)
    static thread_local ResidentGrid cache;
    const unsigned int grid = std::min<unsigned long long>(
        div_up((unsigned long long)a.N * TPP, block),
        cache.blocks(reinterpret_cast<const void*>(kern), block, smem));
    kern<<<grid, block, smem, s>>>(reinterpret_cast<float4*>(a.d_force), a.d_virial,
                                   a.virial_pitch, a.N, reinterpret_cast<const float4*>(a.d_pos),
                                   a.box, a.d_n_neigh, reinterpret_cast<const uint4*>(a.d_nlist),
                                   a.stride, d_params, a.d_rcutsq, a.d_ronsq, a.ntypes, ext,
                                   a.d_charge, a.shift_mode == 1, fz);
    return check_launch("pair force kernel (interleaved list)");
    }

template<class Eval, bool MULTI, bool ORTHO, bool FUSE>
int dispatch_pair_i4_vx(const gb_pair_args& a, const typename Eval::param_type* d_params,
                        const float* ext, const FuseArgs& fz, cudaStream_t s)
    {
    const bool xplor = a.shift_mode == 2;
    // threads per particle: explicit 1, 4 or 8, or by system size (enough lanes to fill the GPU)
    unsigned int tpp = a.threads_per_particle;
    if (tpp == 0)
        tpp = a.N <= 16384 ? 8u : (a.N <= 65536 ? 4u : 1u);
    if (!xplor && !a.compute_virial && ORTHO && tpp > 1)
        {
        if (tpp == 8)
            return launch_pair_i4_inst<Eval, MULTI, ORTHO, FUSE, false, false, 8>(a, d_params, ext, fz, s);
        return launch_pair_i4_inst<Eval, MULTI, ORTHO, FUSE, false, false, 4>(a, d_params, ext, fz, s);
        }
    if (FUSE)
        {
        // the fused step never needs the virial
        return xplor ? launch_pair_i4_inst<Eval, MULTI, ORTHO, FUSE, false, true>(a, d_params, ext, fz, s)
                     : launch_pair_i4_inst<Eval, MULTI, ORTHO, FUSE, false, false>(a, d_params, ext, fz, s);
        }
    if (a.compute_virial)
        return xplor ? launch_pair_i4_inst<Eval, MULTI, ORTHO, false, true, true>(a, d_params, ext, fz, s)
                     : launch_pair_i4_inst<Eval, MULTI, ORTHO, false, true, false>(a, d_params, ext, fz, s);
    return xplor ? launch_pair_i4_inst<Eval, MULTI, ORTHO, false, false, true>(a, d_params, ext, fz, s)
                 : launch_pair_i4_inst<Eval, MULTI, ORTHO, false, false, false>(a, d_params, ext, fz, s);
    }

template<class Eval, bool FUSE>
int dispatch_pair_i4(const gb_pair_args& a, const typename Eval::param_type* d_params,
                     const float* ext, const FuseArgs& fz, cudaStream_t s)
    {
    GB_REQUIRE(a.shift_mode <= 2, "pair force: shift_mode must be 0, 1 or 2");
    GB_REQUIRE(a.block_size == 0 || a.block_size == 128 || a.block_size == 256,
               "pair force: the interleaved-list kernel runs 128- or 256-thread blocks");
    GB_REQUIRE(!(FUSE && a.compute_virial), "fused step: the virial is not computed");
    GB_REQUIRE(a.box.periodic[0] && a.box.periodic[1] && a.box.periodic[2],
               "pair force: the interleaved-list kernel needs a box periodic in every direction");
    const bool ortho = a.box.xy == 0.0f && a.box.xz == 0.0f && a.box.yz == 0.0f;
    if (a.ntypes > 1)
        return ortho ? dispatch_pair_i4_vx<Eval, true, true, FUSE>(a, d_params, ext, fz, s)
                     : dispatch_pair_i4_vx<Eval, true, false, FUSE>(a, d_params, ext, fz, s);
    return ortho ? dispatch_pair_i4_vx<Eval, false, true, FUSE>(a, d_params, ext, fz, s)
                 : dispatch_pair_i4_vx<Eval, false, false, FUSE>(a, d_params, ext, fz, s);
    }

template<class Eval, int TPP, bool FLAT, bool MULTI, bool FUSE>
int launch_pair_inst(const gb_pair_args& a, const typename Eval::param_type* d_params,
                     const float* ext, const FuseArgs& fz, unsigned int block,
                     cudaStream_t s)
    {
    const unsigned int per_block = block / TPP;
    const unsigned int grid = div_up(a.N, per_block);
    size_t smem = 0;
    if (MULTI)
        smem = (sizeof(typename Eval::param_type) + 2 * sizeof(float)) * a.ntypes * a.ntypes;
    auto kern = k_pair<Eval, TPP, FLAT, MULTI, FUSE>;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const bool ortho = a.box.xy == 0.0f && a.box.xz == 0.0f && a.box.yz == 0.0f;
    kern<<<grid, block, smem, s>>>(reinterpret_cast<float4*>(a.d_force), a.d_virial,
                                   a.virial_pitch, a.N, reinterpret_cast<const float4*>(a.d_pos),
                                   a.box, a.d_n_neigh, a.d_nlist, a.d_head_list, a.stride,
                                   d_params, a.d_rcutsq, a.d_ronsq, a.ntypes, ext, a.d_charge,
                                   (int)a.shift_mode, a.compute_virial != 0, ortho, fz);
    return check_launch("pair force kernel");
    }

template<class Eval, int TPP, bool FLAT, bool FUSE>
int dispatch_pair_flags(const gb_pair_args& a, const typename Eval::param_type* d_params,
                        const float* ext, const FuseArgs& fz, unsigned int block,
                        cudaStream_t s)
    {
    GB_REQUIRE(a.shift_mode <= 2, "pair force: shift_mode must be 0, 1 or 2");
    if (a.ntypes > 1)
        return launch_pair_inst<Eval, TPP, FLAT, true, FUSE>(a, d_params, ext, fz, block, s);
    return launch_pair_inst<Eval, TPP, FLAT, false, FUSE>(a, d_params, ext, fz, block, s);
    }

// Entry for one evaluator: validates and picks the layout / TPP instantiation.
template<class Eval, bool FUSE>
int launch_pair(const gb_pair_args* a, const typename Eval::param_type* d_params,
                const float* ext, const FuseArgs& fz, cudaStream_t s)
    {
    GB_REQUIRE(a, "pair force: null args");
    GB_REQUIRE(a->d_force && a->d_pos && a->d_n_neigh && a->d_nlist && a->d_rcutsq && d_params,
               "pair force: null device pointer");
    GB_REQUIRE(!a->compute_virial || (a->d_virial && a->virial_pitch >= a->N),
               "pair force: virial requested without a buffer of pitch >= N");
    GB_REQUIRE(a->shift_mode != 2 || a->d_ronsq, "pair force: xplor needs r_on^2");
    GB_REQUIRE(a->ntypes >= 1 && a->ntypes <= 64, "pair force: 1 <= ntypes <= 64");
    GB_REQUIRE(a->d_head_list || a->stride >= a->N, "pair force: column-major stride < N");
    GB_REQUIRE(!Eval::needsCharge() || a->d_charge, "pair force: this evaluator needs charges");
    if (a->N == 0)
        return GB_OK;
    unsigned int block = a->block_size ? a->block_size : 256;
    GB_REQUIRE(block % 32 == 0 && block <= 256, "pair force: block size multiple of 32, <= 256");
    const bool flat = a->d_head_list != nullptr;
    unsigned int tpp = a->threads_per_particle;
    if (!flat)
        {
        GB_REQUIRE(a->interleave <= 1 || a->interleave == 4,
                   "pair force: interleave must be 1 or 4");
        GB_REQUIRE(a->interleave == 4 ? (tpp <= 1 || tpp == 4 || tpp == 8) : tpp <= 1,
                   "pair force: column-major lists take 1 thread per particle (interleave 1) or "
                   "1, 4 or 8 (interleave 4)");
        if (a->interleave == 4)
            return dispatch_pair_i4<Eval, FUSE>(*a, d_params, ext, fz, s);
        return dispatch_pair_flags<Eval, 1, false, FUSE>(*a, d_params, ext, fz, block, s);
        }
    if (tpp == 0)
        tpp = 8;
    switch (tpp)
        {
    case 1:
        return dispatch_pair_flags<Eval, 1, true, FUSE>(*a, d_params, ext, fz, block, s);
    case 2:
        return dispatch_pair_flags<Eval, 2, true, FUSE>(*a, d_params, ext, fz, block, s);
    case 4:
        return dispatch_pair_flags<Eval, 4, true, FUSE>(*a, d_params, ext, fz, block, s);
    case 8:
        return dispatch_pair_flags<Eval, 8, true, FUSE>(*a, d_params, ext, fz, block, s);
    case 16:
        return dispatch_pair_flags<Eval, 16, true, FUSE>(*a, d_params, ext, fz, block, s);
    case 32:
        return dispatch_pair_flags<Eval, 32, true, FUSE>(*a, d_params, ext, fz, block, s);
    default:
        return fail(GB_ERR_INVALID, "pair force: threads_per_particle must be a power of two <= 32");
        }
    }

} // namespace gb

namespace gb
{
// PotentialPair::computeEnergyBetweenSets (hoomd/md/PotentialPair.h:833-990, exported as
// computeEnergyBetweenSets; hoomd/md/pair/pair.py compute_energy): the reference loops over every
// tag of set 1 and every tag of set 2 (duplicates and tags in both sets included, no exclusions
// applied) and adds V_ij(r) with the force's shift / XPLOR mode. Here d_mult1[i] / d_mult2[i]
// count how often particle index i's tag appears in each set, and the sum is
//   sum_i m1[i] * ( sum_{j in list(i) + excluded(i)} m2[j] V_ij + m2[i] V_ii(r = 0) ):
// the full list holds every ordered pair within r_list except the excluded ones, which are added
// back from the exclusion rows (each distinct partner once); pairs beyond r_cut contribute
// nothing. The i == j term is the evaluator at zero distance, as the reference evaluates it when
// a tag is in both sets. Each block writes its partial sum to d_partials[blockIdx.x]; the caller
// adds them in order.
template<class Eval, bool XPLOR>
__device__ __forceinline__ double sets_pair_energy(float rsq, unsigned int tp,
                                                   const typename Eval::param_type* d_params,
                                                   const float* d_rcutsq, const float* d_ronsq,
                                                   const float* ext, float qi, float qj,
                                                   bool SHIFT1)
    {
    typename Eval::param_type param = d_params[tp];
    const float rcutsq = d_rcutsq[tp];
    Eval::prepare_param(param, rcutsq);
    const float ronsq = XPLOR ? d_ronsq[tp] : 0.0f;
    float force_divr = 0.0f, pair_eng = 0.0f;
    Eval eval(rsq, rcutsq, param, ext);
    if (Eval::needsCharge())
        eval.setCharge(qi, qj);
    if (!eval.evalForceAndEnergy(force_divr, pair_eng, XPLOR ? (ronsq > rcutsq) : SHIFT1))
        return 0.0;
    if (XPLOR && rsq >= ronsq && rsq < rcutsq)
        xplor_smooth(rsq, rcutsq, ronsq, force_divr, pair_eng);
    return (double)pair_eng;
    }

template<class Eval, bool MULTI, bool XPLOR>
__global__ void __launch_bounds__(256)
    k_energy_sets(unsigned int N, const float4* __restrict__ d_pos, gb_box box,
                  const unsigned int* __restrict__ d_n_neigh, const unsigned int* __restrict__ d_nlist,
                  const uint64_t* __restrict__ d_head_list, uint64_t stride, unsigned int interleave,
                  const typename Eval::param_type* __restrict__ d_params,
                  const float* __restrict__ d_rcutsq, const float* __restrict__ d_ronsq,
                  unsigned int ntypes, const float* __restrict__ ext,
                  const float* __restrict__ d_charge, bool SHIFT1,
                  const uint32_t* __restrict__ d_mult1, const uint32_t* __restrict__ d_mult2,
                  const unsigned int* __restrict__ d_n_ex, const unsigned int* __restrict__ d_ex_list,
                  unsigned int ex_pitch, double* __restrict__ d_partials)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    double u = 0.0;
    const uint32_t m1 = i < N ? d_mult1[i] : 0u;
    if (m1)
        {
        const float4 pi = d_pos[i];
        const unsigned int ti = __float_as_uint(pi.w);
        const float qi = Eval::needsCharge() ? d_charge[i] : 0.0f;
        const unsigned int nn = d_n_neigh[i];
        const unsigned int nex = d_n_ex ? d_n_ex[i] : 0u;
        double ui = 0.0;
        for (unsigned int k = 0; k < nn + nex; k++)
            {
            unsigned int j;
            if (k < nn)
                {
                size_t w;
                if (d_head_list)
                    w = d_head_list[i] + k;
                else if (interleave == 4)
                    w = (((size_t)(k >> 2) * stride + i) << 2) + (k & 3u);
                else
                    w = (size_t)k * stride + i;
                j = d_nlist[w];
                }
            else
                {
                // an excluded partner (filtered out of the list): count each distinct one once
                const unsigned int* row = d_ex_list + (size_t)i * ex_pitch;
                const unsigned int e = k - nn;
                j = row[e];
                bool seen = (j == i);
                for (unsigned int e2 = 0; e2 < e && !seen; e2++)
                    seen = row[e2] == j;
                if (seen)
                    continue;
                }
            const uint32_t m2 = d_mult2[j];
            if (!m2)
                continue;
            const float4 pj = d_pos[j];
            float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            min_image(box, dx, dy, dz);
            const float rsq = dx * dx + dy * dy + dz * dz;
            const unsigned int tp = MULTI ? ti * ntypes + __float_as_uint(pj.w) : 0u;
            ui += (double)m2 * sets_pair_energy<Eval, XPLOR>(
                                   rsq, tp, d_params, d_rcutsq, d_ronsq, ext, qi,
                                   Eval::needsCharge() ? d_charge[j] : 0.0f, SHIFT1);
            }
        const uint32_t m2i = d_mult2[i];
        if (m2i)
            {
            const unsigned int tp = MULTI ? ti * ntypes + ti : 0u;
            ui += (double)m2i * sets_pair_energy<Eval, XPLOR>(0.0f, tp, d_params, d_rcutsq,
                                                              d_ronsq, ext, qi, qi, SHIFT1);
            }
        u = (double)m1 * ui;
        }
    __shared__ double s_red[32];
    u = block_sum_d<1>(u, s_red);
    if (threadIdx.x == 0)
        d_partials[blockIdx.x] = u;
    }

inline unsigned int energy_sets_blocks(unsigned int N)
    {
    return div_up(N > 0 ? N : 1u, 256u);
    }

template<class Eval>
int launch_energy_sets(const gb_pair_args* a, const typename Eval::param_type* d_params,
                       const float* ext, const gb_energy_sets* sets, double* d_partials,
                       cudaStream_t s)
    {
    GB_REQUIRE(a && sets && d_partials, "energy between sets: null argument");
    GB_REQUIRE(sets->d_mult1 && sets->d_mult2, "energy between sets: null multiplicity array");
    GB_REQUIRE(!sets->d_n_ex || (sets->d_ex_list && sets->ex_pitch > 0),
               "energy between sets: exclusion rows need d_ex_list and ex_pitch");
    GB_REQUIRE(a->d_pos && a->d_n_neigh && a->d_nlist && a->d_rcutsq && d_params,
               "energy between sets: null device pointer");
    GB_REQUIRE(a->shift_mode <= 2 && (a->shift_mode != 2 || a->d_ronsq),
               "energy between sets: shift_mode 0, 1 or 2 (xplor needs r_on^2)");
    GB_REQUIRE(a->d_head_list || a->interleave <= 1 || a->interleave == 4,
               "energy between sets: interleave must be 1 or 4");
    GB_REQUIRE(!Eval::needsCharge() || a->d_charge, "energy between sets: charges needed");
    const unsigned int grid = energy_sets_blocks(a->N);
    const bool multi = a->ntypes > 1, xplor = a->shift_mode == 2;
    auto kern = multi ? (xplor ? k_energy_sets<Eval, true, true> : k_energy_sets<Eval, true, false>)
                      : (xplor ? k_energy_sets<Eval, false, true> : k_energy_sets<Eval, false, false>);
    kern<<<grid, 256, 0, s>>>(a->N, reinterpret_cast<const float4*>(a->d_pos), a->box,
                              a->d_n_neigh, a->d_nlist, a->d_head_list, a->stride,
                              a->interleave == 4 ? 4u : 1u, d_params, a->d_rcutsq, a->d_ronsq,
                              a->ntypes, ext, a->d_charge, a->shift_mode == 1, sets->d_mult1,
                              sets->d_mult2, sets->d_n_ex, sets->d_ex_list,
                              sets->d_n_ex ? sets->ex_pitch : 0u, d_partials);
    return check_launch("energy between sets");
    }
} // namespace gb
