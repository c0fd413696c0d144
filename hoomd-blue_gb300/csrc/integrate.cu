// Integrator halves, thermodynamic reductions, Bussi factor and momentum thermalisation.
//
// The half steps use explicit round-to-nearest intrinsics in the order of the reference's CPU
// path (hoomd/md/TwoStepConstantVolume.cc:7-80, 213-261), so one step is bit-identical to the
// FP32 oracle. Reductions widen every per-particle term to double and sum in a fixed order.
#include <cstdint>

#include "fused_step.h"
#include "gb_device.cuh"
#include "gb_host.h"
#include "rng.cuh"

namespace gb
{
namespace
{
// Block sum of three doubles; result valid in thread 0.
__device__ inline void block_sum3(double& a, double& b, double& c)
    {
    __shared__ double s[3][32];
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    if (lane == 0)
        {
        s[0][warp] = a;
        s[1][warp] = b;
        s[2][warp] = c;
        }
    __syncthreads();
    if (warp == 0)
        {
        const int nw = blockDim.x / 32;
        a = lane < nw ? s[0][lane] : 0.0;
        b = lane < nw ? s[1][lane] : 0.0;
        c = lane < nw ? s[2][lane] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        c = warp_sum(c);
        }
    __syncthreads();
    }

// Last-block-done reduction: partials[3*block + k]; returns true in the last block, whose
// thread 0 then holds the totals in a, b, c.
__device__ inline bool reduce3_last(double& a, double& b, double& c, unsigned int* counter,
                                    double* partials)
    {
    __shared__ bool s_last;
    block_sum3(a, b, c);
    if (threadIdx.x == 0)
        {
        partials[3 * blockIdx.x] = a;
        partials[3 * blockIdx.x + 1] = b;
        partials[3 * blockIdx.x + 2] = c;
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
        }
    __syncthreads();
    if (!s_last)
        return false;
    __threadfence();
    a = b = c = 0.0;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x)
        {
        a += __ldcg(partials + 3 * k);
        b += __ldcg(partials + 3 * k + 1);
        c += __ldcg(partials + 3 * k + 2);
        }
    block_sum3(a, b, c);
    if (threadIdx.x == 0)
        *counter = 0;
    return true;
    }

struct StepOneCheck
    {
    const float4* last_pos;
    const float* rcut_max;
    float r_buff;
    uint32_t* rebuild;
    // delayed-check schedule (gb_step_one_args); last_update NULL: check every step
    const uint64_t* check_step;
    const uint64_t* last_update;
    uint32_t delay;
    int dist_check;
    };

// NeighborList::shouldCheckDistance / needsUpdating (hoomd/md/NeighborList.cc:1313-1403) for the
// step T = *check_step + 1: 0 = no rebuild, 1 = rebuild without a check, 2 = distance check
__device__ __forceinline__ int check_schedule(const StepOneCheck& c)
    {
    if (!c.last_update)
        return 2;
    const uint64_t T = *c.check_step + 1, last = *c.last_update;
    if (T < last + c.delay)
        return 0;
    if (c.r_buff < 1e-6f
        || (!c.dist_check && (c.delay == 0 || (c.delay > 1 && T == last + c.delay))))
        return 1;
    return 2;
    }

// Brownian dynamics (TwoStepBD) and the DisplacementCapped limit of step one.
struct StepOneExtra
    {
    float max_disp;           // > 0: cap |v| dt at this length (ConstantVolume order only)
    const float4* force;      // BD: net force
    const uint32_t* tag;      // BD: tags (random-number counters)
    const float* gamma;       // BD: drag per type
    float kT;
    unsigned int ndim;
    uint16_t seed;
    const uint64_t* d_timestep; // BD: current step on the device, or NULL to use timestep
    uint64_t timestep;
    int noiseless;            // OverdampedViscous: no random force, v = F / gamma
    uint32_t* zero;           // words set to zero on the way (the next build's cell counts)
    unsigned int n_zero;
    };

// MTTK thermostat state and the reduction scratch of step one.
struct MttkStep
    {
    double* state;  // xi, eta
    double* scale2; // exp(-xi dt / 2) for step two
    double dof, kT, tau, dt;
    unsigned int* counter;
    double* partials;
    };

template<bool CHECK, bool NVE, bool MTTK, bool BD>
__global__ void k_step_one(float4* __restrict__ pos, float4* __restrict__ vel,
                           const float* __restrict__ accel, int* __restrict__ image,
                           unsigned int N, gb_box box, float dt, float scale,
                           const double* __restrict__ d_scale, StepOneCheck chk, MttkStep mk,
                           StepOneExtra ex)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    for (unsigned int w = j; w < ex.n_zero; w += gridDim.x * blockDim.x)
        ex.zero[w] = 0u;
    bool moved = false;
    __shared__ float s_mttk;
    if (MTTK)
        {
        // exp(-xi dt / 2) of the current xi (hoomd/md/Thermostat.h:148-153), once per block
        if (threadIdx.x == 0)
            s_mttk = (float)exp(-(1.0 / 2.0) * mk.state[0] * mk.dt);
        __syncthreads();
        }
    double ke = 0.0;
    if (j < N)
        {
        const float s = MTTK ? s_mttk : ((!NVE && d_scale) ? (float)*d_scale : scale);
        float4 v = vel[j];
        float4 p = pos[j];
        const float ax = BD ? 0.0f : accel[3 * (size_t)j], ay = BD ? 0.0f : accel[3 * (size_t)j + 1],
                    az = BD ? 0.0f : accel[3 * (size_t)j + 2];
        if (BD)
            {
            // TwoStepBD::integrateStepOne (hoomd/md/TwoStepBD.cc:90-151): three uniform draws
            // from Seed(24, timestep, seed), Counter(tag); x += (F + F_r) dt / gamma with
            // F_r = r sqrt(6 gamma kT / dt); then new velocities from the same stream
            // (NormalDistribution(sqrt(kT / m))), or F / gamma without noise
            const uint64_t ts = ex.d_timestep ? *ex.d_timestep : ex.timestep;
            Philox rng(24, ts, ex.seed, ex.tag[j]);
            const float rx = uniform_m11_f(rng);
            const float ry = uniform_m11_f(rng);
            const float rz = uniform_m11_f(rng);
            const float gamma = ex.gamma[__float_as_uint(p.w)];
            float coeff = __fsqrt_rn(__fdiv_rn(fmul(fmul(6.0f, gamma), ex.kT), dt));
            if (ex.noiseless)
                coeff = 0.0f;
            const float frx = fmul(rx, coeff), fry = fmul(ry, coeff);
            const float frz = ex.ndim < 3 ? 0.0f : fmul(rz, coeff);
            const float4 f = ex.force[j];
            p.x = fadd(p.x, __fdiv_rn(fmul(fadd(f.x, frx), dt), gamma));
            p.y = fadd(p.y, __fdiv_rn(fmul(fadd(f.y, fry), dt), gamma));
            p.z = fadd(p.z, __fdiv_rn(fmul(fadd(f.z, frz), dt), gamma));
            if (ex.noiseless)
                {
                v.x = __fdiv_rn(f.x, gamma);
                v.y = __fdiv_rn(f.y, gamma);
                v.z = ex.ndim > 2 ? __fdiv_rn(f.z, gamma) : 0.0f;
                }
            else
                {
                const float sigma = __fsqrt_rn(__fdiv_rn(ex.kT, v.w));
                v.x = normal_f(rng) * sigma + 0.0f;
                v.y = normal_f(rng) * sigma + 0.0f;
                v.z = ex.ndim > 2 ? normal_f(rng) * sigma + 0.0f : 0.0f;
                }
            }
        else if (NVE)
            {
            // x += v dt + (1/2) a dt^2 ; v += (1/2) a dt   (TwoStepNVEGPU.cu:68-98,
            // TwoStepLangevin.cc:57-81)
            p.x = fadd(p.x, fadd(fmul(v.x, dt), fmul(fmul(fmul(0.5f, ax), dt), dt)));
            p.y = fadd(p.y, fadd(fmul(v.y, dt), fmul(fmul(fmul(0.5f, ay), dt), dt)));
            p.z = fadd(p.z, fadd(fmul(v.z, dt), fmul(fmul(fmul(0.5f, az), dt), dt)));
            v.x = fadd(v.x, fmul(fmul(0.5f, ax), dt));
            v.y = fadd(v.y, fmul(fmul(0.5f, ay), dt));
            v.z = fadd(v.z, fmul(fmul(0.5f, az), dt));
            }
        else
            {
            // v = v + (1/2) a dt ; v *= s ; x += dt v   (TwoStepConstantVolume.cc:37-55)
            v.x = fadd(v.x, fmul(fmul(0.5f, ax), dt));
            v.y = fadd(v.y, fmul(fmul(0.5f, ay), dt));
            v.z = fadd(v.z, fmul(fmul(0.5f, az), dt));
            v.x = fmul(v.x, s);
            v.y = fmul(v.y, s);
            v.z = fmul(v.z, s);
            if (ex.max_disp > 0.0f)
                {
                // DisplacementCapped: |v| dt at most the limit, the documented behaviour of
                // hoomd/md/methods/methods.py:583-598. (The reference's CPU path,
                // TwoStepConstantVolume.cc:44-52, divides by dt once more and its GPU path,
                // TwoStepConstantVolumeGPU.cu:69-74, multiplies by dt instead; neither caps the
                // step at the limit.) With len = |v| dt, v / len * limit has length limit / dt.
                const float len = fmul(__fsqrt_rn(dot3(v.x, v.y, v.z)), dt);
                if (len > ex.max_disp)
                    {
                    v.x = fmul(__fdiv_rn(v.x, len), ex.max_disp);
                    v.y = fmul(__fdiv_rn(v.y, len), ex.max_disp);
                    v.z = fmul(__fdiv_rn(v.z, len), ex.max_disp);
                    }
                }
            p.x = fadd(p.x, fmul(dt, v.x));
            p.y = fadd(p.y, fmul(dt, v.y));
            p.z = fadd(p.z, fmul(dt, v.z));
            }
        int ix = 0, iy = 0, iz = 0;
        wrap(box, p.x, p.y, p.z, ix, iy, iz);
        if (ix | iy | iz)
            {
            image[3 * (size_t)j] += ix;
            image[3 * (size_t)j + 1] += iy;
            image[3 * (size_t)j + 2] += iz;
            }
        vel[j] = v;
        pos[j] = p;
        if (MTTK)
            ke = (double)v.w
                 * ((double)v.x * (double)v.x + (double)v.y * (double)v.y
                    + (double)v.z * (double)v.z);
        const int sched = CHECK ? check_schedule(chk) : 0;
        if (CHECK && sched == 1)
            moved = true;
        if (CHECK && sched == 2)
            {
            // hoomd/md/NeighborListGPU.cu:42-83 with lambda = 1 (fixed box)
            const float4 lp = chk.last_pos[j];
            float dx = fsub(p.x, lp.x), dy = fsub(p.y, lp.y), dz = fsub(p.z, lp.z);
            min_image(box, dx, dy, dz);
            const float rmin = chk.rcut_max[__float_as_uint(p.w)];
            const float rmax = fadd(rmin, chk.r_buff);
            const float delta_max = fmul(fsub(rmax, rmin), 0.5f);
            const float maxsq = (delta_max > 0.0f) ? fmul(delta_max, delta_max) : 0.0f;
            moved = dot3(dx, dy, dz) >= maxsq;
            }
        }
    if (CHECK && __any_sync(0xffffffffu, moved) && (threadIdx.x % 32) == 0)
        *chk.rebuild = 1u;
    if (MTTK)
        {
        // advanceThermostat (hoomd/md/Thermostat.h:162-177) on the half-step kinetic energy
        double b = 0.0, c = 0.0;
        if (reduce3_last(ke, b, c, mk.counter, mk.partials) && threadIdx.x == 0)
            {
            const double T_cur = 2.0 * (0.5 * ke) / mk.dof;
            const double drive = (1.0 / 2.0) * mk.dt / mk.tau / mk.tau * (T_cur / mk.kT - 1.0);
            const double xi_prime = mk.state[0] + drive;
            const double xi = xi_prime + drive;
            mk.state[0] = xi;
            mk.state[1] += xi_prime * mk.dt;
            *mk.scale2 = exp(-(1.0 / 2.0) * xi * mk.dt);
            }
        }
    }

__global__ void k_step_two(float4* __restrict__ vel, float* __restrict__ accel,
                           const float4* __restrict__ net_force, unsigned int N, float dt,
                           float scale, const double* __restrict__ d_scale)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N)
        return;
    const float s = d_scale ? (float)*d_scale : scale;
    float4 v = vel[j];
    const float4 f = net_force[j];
    const float minv = __frcp_rn(v.w);
    const float ax = fmul(f.x, minv), ay = fmul(f.y, minv), az = fmul(f.z, minv);
    v.x = fmul(v.x, s);
    v.y = fmul(v.y, s);
    v.z = fmul(v.z, s);
    const float hdt = fmul(0.5f, dt);
    v.x = fadd(v.x, fmul(hdt, ax));
    v.y = fadd(v.y, fmul(hdt, ay));
    v.z = fadd(v.z, fmul(hdt, az));
    vel[j] = v;
    accel[3 * (size_t)j] = ax;
    accel[3 * (size_t)j + 1] = ay;
    accel[3 * (size_t)j + 2] = az;
    }

// ConstantPressure halves (TwoStepConstantPressure.cc:206-330, 587-640): upper-triangular
// propagators m = (xx, xy, xz, yy, yz, zz) applied as the reference writes them.
struct Tri
    {
    float m[6];
    };

__device__ __forceinline__ void tri_apply(const Tri& t, float& x, float& y, float& z)
    {
    const float nx = fadd(fadd(fmul(t.m[0], x), fmul(t.m[1], y)), fmul(t.m[2], z));
    const float ny = fadd(fmul(t.m[3], y), fmul(t.m[4], z));
    const float nz = fmul(t.m[5], z);
    x = nx;
    y = ny;
    z = nz;
    }

__global__ void k_npt_step_one(float4* __restrict__ pos, float4* __restrict__ vel,
                               const float* __restrict__ accel, int* __restrict__ image,
                               unsigned int N, gb_box box, float dt, float s, Tri mv, Tri mr,
                               Tri mri)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N)
        return;
    float4 v = vel[j];
    float4 p = pos[j];
    const float hdt = __fdiv_rn(dt, 2.0f);
    // v += dt/2 a ; v = M_v v ; v *= s ; r = M_r r ; r += M_r,int v
    v.x = fadd(v.x, fmul(hdt, accel[3 * (size_t)j]));
    v.y = fadd(v.y, fmul(hdt, accel[3 * (size_t)j + 1]));
    v.z = fadd(v.z, fmul(hdt, accel[3 * (size_t)j + 2]));
    tri_apply(mv, v.x, v.y, v.z);
    v.x = fmul(v.x, s);
    v.y = fmul(v.y, s);
    v.z = fmul(v.z, s);
    tri_apply(mr, p.x, p.y, p.z);
    float ix = v.x, iy = v.y, iz = v.z;
    tri_apply(mri, ix, iy, iz);
    p.x = fadd(p.x, ix);
    p.y = fadd(p.y, iy);
    p.z = fadd(p.z, iz);
    int wx = 0, wy = 0, wz = 0;
    wrap(box, p.x, p.y, p.z, wx, wy, wz);
    if (wx | wy | wz)
        {
        image[3 * (size_t)j] += wx;
        image[3 * (size_t)j + 1] += wy;
        image[3 * (size_t)j + 2] += wz;
        }
    vel[j] = v;
    pos[j] = p;
    }

__global__ void k_npt_step_two(float4* __restrict__ vel, float* __restrict__ accel,
                               const float4* __restrict__ net, unsigned int N, float dt, float s,
                               Tri mv)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N)
        return;
    float4 v = vel[j];
    const float4 f = net[j];
    const float minv = __frcp_rn(v.w);
    const float ax = fmul(f.x, minv), ay = fmul(f.y, minv), az = fmul(f.z, minv);
    v.x = fmul(v.x, s);
    v.y = fmul(v.y, s);
    v.z = fmul(v.z, s);
    tri_apply(mv, v.x, v.y, v.z);
    const float hdt = __fdiv_rn(dt, 2.0f);
    v.x = fadd(v.x, fmul(hdt, ax));
    v.y = fadd(v.y, fmul(hdt, ay));
    v.z = fadd(v.z, fmul(hdt, az));
    vel[j] = v;
    accel[3 * (size_t)j] = ax;
    accel[3 * (size_t)j + 1] = ay;
    accel[3 * (size_t)j + 2] = az;
    }

// Kinetic and virial tensors in FP64: per block 13 partial sums (sum m v_a v_b, sum W_ab, PE),
// then one block adds the partials in a fixed order.
constexpr int TENSOR_TERMS = 13;

__global__ void k_tensor_partials(const float4* __restrict__ vel, const float4* __restrict__ force,
                                  const float* __restrict__ virial, size_t pitch, unsigned int N,
                                  double* __restrict__ partials)
    {
    __shared__ double s[TENSOR_TERMS][256 / 32];
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    double t[TENSOR_TERMS];
    for (int k = 0; k < TENSOR_TERMS; k++)
        t[k] = 0.0;
    if (j < N)
        {
        const float4 v = vel[j];
        const double m = v.w, vx = v.x, vy = v.y, vz = v.z;
        t[0] = m * vx * vx;
        t[1] = m * vx * vy;
        t[2] = m * vx * vz;
        t[3] = m * vy * vy;
        t[4] = m * vy * vz;
        t[5] = m * vz * vz;
        if (virial)
            for (int k = 0; k < 6; k++)
                t[6 + k] = (double)virial[k * pitch + j];
        if (force)
            t[12] = (double)force[j].w;
        }
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    for (int k = 0; k < TENSOR_TERMS; k++)
        {
        double x = warp_sum(t[k]);
        if (lane == 0)
            s[k][warp] = x;
        }
    __syncthreads();
    if (threadIdx.x < TENSOR_TERMS)
        {
        double x = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); w++)
            x += s[threadIdx.x][w];
        partials[(size_t)blockIdx.x * TENSOR_TERMS + threadIdx.x] = x;
        }
    }

__global__ void k_tensor_final(const double* __restrict__ partials, unsigned int nblocks,
                               double* __restrict__ out)
    {
    if (threadIdx.x < TENSOR_TERMS)
        {
        double x = 0.0;
        for (unsigned int b = 0; b < nblocks; b++)
            x += partials[(size_t)b * TENSOR_TERMS + threadIdx.x];
        out[threadIdx.x] = x;
        }
    }

__global__ void k_thermo(const float4* __restrict__ vel, const float4* __restrict__ force,
                         const float* __restrict__ virial, size_t pitch, unsigned int N,
                         unsigned int* counter, double* partials, double* out)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0, pe = 0.0, w = 0.0;
    if (j < N)
        {
        const float4 v = vel[j];
        ke = (double)v.w * ((double)v.x * (double)v.x + (double)v.y * (double)v.y
                            + (double)v.z * (double)v.z);
        if (force)
            pe = (double)force[j].w;
        if (virial)
            w = (double)virial[j] + (double)virial[3 * pitch + j] + (double)virial[5 * pitch + j];
        }
    if (reduce3_last(ke, pe, w, counter, partials) && threadIdx.x == 0)
        {
        out[0] = 0.5 * ke;
        out[1] = pe;
        out[2] = w / 3.0;
        }
    }

__global__ void k_bussi_draws(const uint64_t* d_timestep, unsigned int count, double dof,
                              uint16_t seed, uint32_t instance_id, double2* ring,
                              unsigned int ring_size)
    {
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count)
        return;
    const uint64_t ts = *d_timestep + 1 + k;
    ring[ts % ring_size] = bussi_draws_d(dof, ts, seed, instance_id);
    }

__global__ void k_bussi(const double* d_ke, double dof, double dt, double tau, double kT,
                        uint64_t timestep, uint16_t seed, uint32_t instance_id, double* d_factor)
    {
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *d_factor = bussi_factor_d(*d_ke, dof, dt, tau, kT, timestep, seed, instance_id);
    }

__global__ void k_berendsen(const double* d_ke, double dof, double dt, double tau, double kT,
                            double* d_factor, uint32_t* d_status)
    {
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    const double K = *d_ke;
    if (dof != 0.0 && K <= 0.0)
        {
        atomicOr(d_status, 2u);
        *d_factor = 1.0;
        return;
        }
    *d_factor = berendsen_factor_d(K, dof, dt, tau, kT);
    }

__global__ void k_normal_draw(uint8_t id, uint64_t timestep, uint16_t seed, uint32_t counter,
                              double sigma, double* out)
    {
    if (threadIdx.x == 0 && blockIdx.x == 0)
        {
        Philox rng(id, timestep, seed, counter);
        *out = normal_d(rng) * sigma + 0.0;
        }
    }

// hoomd/ParticleGroup.cc:719-746: velocities from NormalDistribution<float>(sqrt(kT/m)) with
// key Seed(35, timestep, seed) and counter = tag; momentum summed in double.
__global__ void k_thermalize_draw(float4* __restrict__ vel, const uint32_t* __restrict__ tag,
                                  unsigned int N, float kT, uint64_t timestep, uint16_t seed,
                                  unsigned int ndim, unsigned int* counter, double* partials,
                                  double* total)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    double px = 0.0, py = 0.0, pz = 0.0;
    if (j < N)
        {
        Philox rng(35, timestep, seed, tag[j]);
        float4 v = vel[j];
        const float sigma = sqrtf(kT / v.w);
        v.x = normal_f(rng) * sigma + 0.0f;
        v.y = normal_f(rng) * sigma + 0.0f;
        v.z = (ndim > 2) ? normal_f(rng) * sigma + 0.0f : 0.0f;
        vel[j] = v;
        px = (double)v.w * v.x;
        py = (double)v.w * v.y;
        pz = (double)v.w * v.z;
        }
    if (reduce3_last(px, py, pz, counter, partials) && threadIdx.x == 0)
        {
        total[0] = px;
        total[1] = py;
        total[2] = pz;
        }
    }

__global__ void k_thermalize_shift(float4* __restrict__ vel, unsigned int N, unsigned int ndim,
                                   const double* __restrict__ total)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N)
        return;
    const float cx = (float)(total[0] / N), cy = (float)(total[1] / N),
                cz = (float)(total[2] / N);
    float4 v = vel[j];
    v.x = v.x - cx / v.w;
    v.y = v.y - cy / v.w;
    if (ndim > 2)
        v.z = v.z - cz / v.w;
    vel[j] = v;
    }
// Langevin step two from the net force, with the step's FP64 sums (last block).
__global__ void k_langevin_two(FuseArgs fz, const float4* __restrict__ net, unsigned int N)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0, pe = 0.0, w = 0.0;
    if (j < N)
        {
        const float4 f = net[j];
        fuse_step_two(fz, j, f.x, f.y, f.z, f.w, ke, pe, w);
        }
    fuse_finish(fz, ke, pe, w);
    }

struct ForcePtrs
    {
    const float4* f[8];
    };

__global__ void k_sum_net_force(float4* __restrict__ net, ForcePtrs fp, unsigned int nf,
                                unsigned int N)
    {
    const unsigned int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N)
        return;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (unsigned int k = 0; k < nf; k++)
        {
        const float4 v = fp.f[k][j];
        s.x += v.x;
        s.y += v.y;
        s.z += v.z;
        s.w += v.w;
        }
    net[j] = s;
    }
} // namespace
} // namespace gb

using namespace gb;

namespace gb
{
namespace
{
// The value of a conditional graph node from a device flag (0 or not): the rebuild flag the
// step's check kernel raised decides whether the node's body (the cell list and neighbour-list
// build) runs in this replay of the graph.
__global__ void k_set_conditional(cudaGraphConditionalHandle handle, const uint32_t* flag)
    {
    cudaGraphSetConditional(handle, *flag != 0u ? 1u : 0u);
    }

__global__ void k_step_counter_advance(uint64_t* step)
    {
    *step += 1;
    }
} // namespace
} // namespace gb

extern "C"
    {
    int gb_graph_set_conditional(uint64_t handle, const uint32_t* d_flag, void* stream)
        {
        GB_REQUIRE(d_flag, "gb_graph_set_conditional: null flag");
        gb::k_set_conditional<<<1, 1, 0, (cudaStream_t)stream>>>(
            (cudaGraphConditionalHandle)handle, d_flag);
        return check_launch("gb_graph_set_conditional");
        }

    int gb_step_counter_advance(uint64_t* d_timestep, void* stream)
        {
        GB_REQUIRE(d_timestep, "gb_step_counter_advance: null counter");
        gb::k_step_counter_advance<<<1, 1, 0, (cudaStream_t)stream>>>(d_timestep);
        return check_launch("gb_step_counter_advance");
        }

    int gb_cv_step_one(float* d_pos, float* d_vel, const float* d_accel, int* d_image,
                       unsigned int N, const gb_box* box, float dt, float scale,
                       const double* d_scale, void* stream)
        {
        GB_REQUIRE(box && (N == 0 || (d_pos && d_vel && d_accel && d_image)),
                   "gb_cv_step_one: null argument");
        if (N == 0)
            return GB_OK;
        StepOneCheck none {nullptr, nullptr, 0.0f, nullptr, nullptr, nullptr, 1u, 1};
        k_step_one<false, false, false, false><<<div_up(N, 256), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<float4*>(d_pos), reinterpret_cast<float4*>(d_vel), d_accel, d_image,
            N, *box, dt, scale, d_scale, none, MttkStep {}, StepOneExtra {});
        return check_launch("gb_cv_step_one");
        }

    int gb_md_step_one(const gb_step_one_args* a, void* stream)
        {
        GB_REQUIRE(a, "gb_md_step_one: null args");
        GB_REQUIRE(a->N == 0 || (a->d_pos && a->d_vel && a->d_accel && a->d_image),
                   "gb_md_step_one: null particle array");
        GB_REQUIRE(!a->d_last_pos || (a->d_rcut_max && a->d_rebuild),
                   "gb_md_step_one: rebuild check needs r_cut max and a flag");
        if (a->N == 0)
            return GB_OK;
        GB_REQUIRE(!a->d_last_update || a->d_check_step,
                   "gb_md_step_one: a check schedule needs the device step counter");
        StepOneCheck chk {reinterpret_cast<const float4*>(a->d_last_pos),
                          a->d_rcut_max,
                          a->r_buff,
                          a->d_rebuild,
                          a->d_check_step,
                          a->d_last_update,
                          a->check_delay,
                          a->check_dist};
        cudaStream_t s = (cudaStream_t)stream;
        const bool mttk = a->d_mttk_state != nullptr;
        GB_REQUIRE(!mttk || (a->d_mttk_scale2 && a->d_mttk_scratch && !a->nve_order),
                   "gb_md_step_one: MTTK needs the step-two factor, scratch and the "
                   "ConstantVolume order");
        MttkStep mk {};
        if (mttk)
            {
            mk.state = a->d_mttk_state;
            mk.scale2 = a->d_mttk_scale2;
            mk.dof = a->mttk_dof;
            mk.kT = a->mttk_kT;
            mk.tau = a->mttk_tau;
            mk.dt = (double)a->dt;
            mk.counter = reinterpret_cast<unsigned int*>(a->d_mttk_scratch);
            mk.partials
                = reinterpret_cast<double*>(reinterpret_cast<char*>(a->d_mttk_scratch) + 256);
            }
        const bool bd = a->brownian != 0;
        GB_REQUIRE(!bd || (a->d_bd_force && a->d_tag && a->d_gamma && !mttk && !a->nve_order),
                   "gb_md_step_one: Brownian dynamics needs the net force, tags and drag "
                   "coefficients, and excludes the other methods");
        StepOneExtra ex {};
        ex.max_disp = (!a->nve_order && !bd) ? a->max_displacement : 0.0f;
        ex.force = reinterpret_cast<const float4*>(a->d_bd_force);
        ex.tag = a->d_tag;
        ex.gamma = a->d_gamma;
        ex.kT = a->bd_kT;
        ex.ndim = a->ndim ? a->ndim : 3u;
        ex.seed = (uint16_t)a->seed;
        ex.d_timestep = a->d_timestep;
        ex.timestep = a->timestep;
        ex.noiseless = a->noiseless;
        ex.zero = a->d_zero_words;
        ex.n_zero = a->d_zero_words ? a->n_zero_words : 0u;
        using K = void (*)(float4*, float4*, const float*, int*, unsigned int, gb_box, float,
                           float, const double*, StepOneCheck, MttkStep, StepOneExtra);
        K kern;
        if (a->d_last_pos)
            kern = bd ? k_step_one<true, false, false, true>
                      : (mttk ? k_step_one<true, false, true, false>
                              : (a->nve_order ? k_step_one<true, true, false, false>
                                              : k_step_one<true, false, false, false>));
        else
            kern = bd ? k_step_one<false, false, false, true>
                      : (mttk ? k_step_one<false, false, true, false>
                              : (a->nve_order ? k_step_one<false, true, false, false>
                                              : k_step_one<false, false, false, false>));
        kern<<<div_up(a->N, 256), 256, 0, s>>>(
            reinterpret_cast<float4*>(a->d_pos), reinterpret_cast<float4*>(a->d_vel), a->d_accel,
            a->d_image, a->N, a->box, a->dt, a->scale, a->d_scale, chk, mk, ex);
        return check_launch("gb_md_step_one");
        }

    int gb_cv_step_two(float* d_vel, float* d_accel, const float* d_net_force, unsigned int N,
                       float dt, float scale, const double* d_scale, void* stream)
        {
        GB_REQUIRE(N == 0 || (d_vel && d_accel && d_net_force), "gb_cv_step_two: null argument");
        if (N == 0)
            return GB_OK;
        k_step_two<<<div_up(N, 256), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<float4*>(d_vel), d_accel, reinterpret_cast<const float4*>(d_net_force),
            N, dt, scale, d_scale);
        return check_launch("gb_cv_step_two");
        }

    int gb_langevin_step_two(float* d_vel, float* d_accel, const float* d_net_force,
                             const float* d_pos, const uint32_t* d_tag, const float* d_gamma,
                             unsigned int N, float dt, float kT, uint32_t ndim, uint16_t seed,
                             uint64_t* d_timestep, void* d_scratch, double* d_thermo,
                             double* d_reservoir, void* stream)
        {
        GB_REQUIRE(d_timestep && d_scratch && d_thermo, "gb_langevin_step_two: null argument");
        GB_REQUIRE(N == 0 || (d_vel && d_accel && d_net_force && d_pos && d_tag && d_gamma),
                   "gb_langevin_step_two: null particle array");
        FuseArgs fz {};
        fz.vel = reinterpret_cast<float4*>(d_vel);
        fz.accel = d_accel;
        fz.dt = dt;
        fz.dt_d = (double)dt;
        fz.counter = reinterpret_cast<unsigned int*>(d_scratch);
        fz.partials = reinterpret_cast<double*>(reinterpret_cast<char*>(d_scratch) + 256);
        fz.out = d_thermo;
        fz.seed = seed;
        fz.d_timestep = d_timestep;
        fz.langevin = 1;
        fz.tag = d_tag;
        fz.pos = reinterpret_cast<const float4*>(d_pos);
        fz.gamma = d_gamma;
        fz.lkT = kT;
        fz.ndim = ndim ? ndim : 3u;
        fz.d_reservoir = d_reservoir;
        k_langevin_two<<<div_up(N > 0 ? N : 1, 256), 256, 0, (cudaStream_t)stream>>>(
            fz, reinterpret_cast<const float4*>(d_net_force), N);
        return check_launch("gb_langevin_step_two");
        }

    int gb_npt_step_one(float* d_pos, float* d_vel, const float* d_accel, int* d_image,
                        unsigned int N, const gb_box* new_box, float dt, float scale,
                        const float* mat_exp_v, const float* mat_exp_r,
                        const float* mat_exp_r_int, void* stream)
        {
        GB_REQUIRE(new_box && mat_exp_v && mat_exp_r && mat_exp_r_int,
                   "gb_npt_step_one: null argument");
        GB_REQUIRE(N == 0 || (d_pos && d_vel && d_accel && d_image),
                   "gb_npt_step_one: null particle array");
        if (N == 0)
            return GB_OK;
        Tri mv, mr, mri;
        for (int k = 0; k < 6; k++)
            {
            mv.m[k] = mat_exp_v[k];
            mr.m[k] = mat_exp_r[k];
            mri.m[k] = mat_exp_r_int[k];
            }
        k_npt_step_one<<<div_up(N, 256), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<float4*>(d_pos), reinterpret_cast<float4*>(d_vel), d_accel, d_image,
            N, *new_box, dt, scale, mv, mr, mri);
        return check_launch("gb_npt_step_one");
        }

    int gb_npt_step_two(float* d_vel, float* d_accel, const float* d_net_force, unsigned int N,
                        float dt, float scale, const float* mat_exp_v, void* stream)
        {
        GB_REQUIRE(mat_exp_v, "gb_npt_step_two: null argument");
        GB_REQUIRE(N == 0 || (d_vel && d_accel && d_net_force),
                   "gb_npt_step_two: null particle array");
        if (N == 0)
            return GB_OK;
        Tri mv;
        for (int k = 0; k < 6; k++)
            mv.m[k] = mat_exp_v[k];
        k_npt_step_two<<<div_up(N, 256), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<float4*>(d_vel), d_accel, reinterpret_cast<const float4*>(d_net_force),
            N, dt, scale, mv);
        return check_launch("gb_npt_step_two");
        }

    size_t gb_thermo_tensor_scratch_bytes(unsigned int N)
        {
        return sizeof(double) * TENSOR_TERMS * (size_t)div_up(N > 0 ? N : 1, 256);
        }

    int gb_thermo_tensor(const float* d_vel, const float* d_force, const float* d_virial,
                         size_t virial_pitch, unsigned int N, void* d_scratch, double* d_out,
                         void* stream)
        {
        GB_REQUIRE(d_vel && d_scratch && d_out, "gb_thermo_tensor: null argument");
        GB_REQUIRE(!d_virial || virial_pitch >= N, "gb_thermo_tensor: virial pitch < N");
        const unsigned int nb = div_up(N > 0 ? N : 1, 256);
        cudaStream_t s = (cudaStream_t)stream;
        k_tensor_partials<<<nb, 256, 0, s>>>(reinterpret_cast<const float4*>(d_vel),
                                             reinterpret_cast<const float4*>(d_force), d_virial,
                                             virial_pitch, N, reinterpret_cast<double*>(d_scratch));
        k_tensor_final<<<1, 32, 0, s>>>(reinterpret_cast<const double*>(d_scratch), nb, d_out);
        return check_launch("gb_thermo_tensor");
        }

    int gb_sum_net_force(float* d_net, const float* const* h_force_ptrs, unsigned int n_forces,
                         unsigned int N, void* stream)
        {
        GB_REQUIRE(d_net && h_force_ptrs, "gb_sum_net_force: null argument");
        GB_REQUIRE(n_forces >= 1 && n_forces <= 8, "gb_sum_net_force: 1 <= n_forces <= 8");
        if (N == 0)
            return GB_OK;
        ForcePtrs fp {};
        for (unsigned int k = 0; k < n_forces; k++)
            {
            GB_REQUIRE(h_force_ptrs[k], "gb_sum_net_force: null force array");
            fp.f[k] = reinterpret_cast<const float4*>(h_force_ptrs[k]);
            }
        k_sum_net_force<<<div_up(N, 256), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<float4*>(d_net), fp, n_forces, N);
        return check_launch("gb_sum_net_force");
        }

    size_t gb_thermo_scratch_bytes(unsigned int N)
        {
        return 256 + 3 * sizeof(double) * (size_t)div_up(N > 0 ? N : 1, 256);
        }

    size_t gb_md_step_scratch_bytes(unsigned int N)
        {
        return step_scratch_bytes(N);
        }

    int gb_thermo_reduce(const float* d_vel, const float* d_force, const float* d_virial,
                         size_t virial_pitch, unsigned int N, void* d_scratch, double* d_out,
                         void* stream)
        {
        GB_REQUIRE(d_vel && d_scratch && d_out, "gb_thermo_reduce: null argument");
        GB_REQUIRE(!d_virial || virial_pitch >= N, "gb_thermo_reduce: virial pitch < N");
        const unsigned int nb = div_up(N > 0 ? N : 1, 256);
        k_thermo<<<nb, 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<const float4*>(d_vel), reinterpret_cast<const float4*>(d_force),
            d_virial, virial_pitch, N, reinterpret_cast<unsigned int*>(d_scratch),
            reinterpret_cast<double*>(reinterpret_cast<char*>(d_scratch) + 256), d_out);
        return check_launch("gb_thermo_reduce");
        }

    int gb_bussi_factor(const double* d_ke, double dof, double dt, double tau, double kT,
                        uint64_t timestep, uint16_t seed, uint32_t instance_id, double* d_factor,
                        void* stream)
        {
        GB_REQUIRE(d_ke && d_factor, "gb_bussi_factor: null argument");
        k_bussi<<<1, 32, 0, (cudaStream_t)stream>>>(d_ke, dof, dt, tau, kT, timestep, seed,
                                                     instance_id, d_factor);
        return check_launch("gb_bussi_factor");
        }

    int gb_bussi_draws(const uint64_t* d_timestep, unsigned int count, double dof, uint16_t seed,
                       uint32_t instance_id, double* d_ring, unsigned int ring_size, void* stream)
        {
        GB_REQUIRE(d_timestep && d_ring, "gb_bussi_draws: null argument");
        GB_REQUIRE(ring_size > 0 && count <= ring_size, "gb_bussi_draws: count > ring_size");
        if (count == 0)
            return GB_OK;
        k_bussi_draws<<<div_up(count, 64), 64, 0, (cudaStream_t)stream>>>(
            d_timestep, count, dof, seed, instance_id, reinterpret_cast<double2*>(d_ring),
            ring_size);
        return check_launch("gb_bussi_draws");
        }

    int gb_berendsen_factor(const double* d_ke, double dof, double dt, double tau, double kT,
                            double* d_factor, uint32_t* d_status, void* stream)
        {
        GB_REQUIRE(d_ke && d_factor && d_status, "gb_berendsen_factor: null argument");
        GB_REQUIRE(tau > 0.0, "gb_berendsen_factor: tau must be positive");
        k_berendsen<<<1, 32, 0, (cudaStream_t)stream>>>(d_ke, dof, dt, tau, kT, d_factor,
                                                        d_status);
        return check_launch("gb_berendsen_factor");
        }

    int gb_normal_draw(uint8_t id, uint64_t timestep, uint16_t seed, uint32_t counter,
                       double sigma, double* d_out, void* stream)
        {
        GB_REQUIRE(d_out, "gb_normal_draw: null argument");
        k_normal_draw<<<1, 32, 0, (cudaStream_t)stream>>>(id, timestep, seed, counter, sigma,
                                                          d_out);
        return check_launch("gb_normal_draw");
        }

    int gb_thermalize(float* d_vel, const uint32_t* d_tag, unsigned int N, double kT,
                      uint64_t timestep, uint16_t seed, unsigned int ndim, void* d_scratch,
                      void* stream)
        {
        GB_REQUIRE(d_vel && d_tag && d_scratch, "gb_thermalize: null argument");
        if (N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        const unsigned int nb = div_up(N, 256);
        unsigned int* counter = reinterpret_cast<unsigned int*>(d_scratch);
        double* total = reinterpret_cast<double*>(reinterpret_cast<char*>(d_scratch) + 64);
        double* partials = reinterpret_cast<double*>(reinterpret_cast<char*>(d_scratch) + 256);
        k_thermalize_draw<<<nb, 256, 0, s>>>(reinterpret_cast<float4*>(d_vel), d_tag, N, (float)kT,
                                             timestep, seed, ndim, counter, partials, total);
        k_thermalize_shift<<<nb, 256, 0, s>>>(reinterpret_cast<float4*>(d_vel), N, ndim, total);
        return check_launch("gb_thermalize");
        }
    }
