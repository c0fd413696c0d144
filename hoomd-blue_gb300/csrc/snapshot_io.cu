// Snapshot transfer on the device: the per-particle part of ParticleData::takeSnapshot and
// ParticleData::initializeFromSnapshot (hoomd/ParticleData.cc), which the reference runs on the
// host. The host side copies the snapshot's arrays (tag order, FP64) to or from one device staging
// block; these kernels convert between that block and the particle arrays the MD step uses
// (index order, FP32 float4), so a million-particle round trip is a few bulk copies and two
// kernels instead of host loops.
//
// Scatter (snapshot -> particles): each tag t goes to index i = rtag[t], the index its particle
// already holds (d_rtag NULL: i = t), so a snapshot written back into a running simulation keeps
// the particles' current order and with it the locality the Hilbert sort gave them. Positions are
// wrapped into the box with the image counts updated, in the order and FP32 arithmetic of the
// host wrap (at most one box length per axis per pass, two passes), as initializeFromSnapshot
// does once.
#include <cstdint>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
__global__ void k_snapshot_gather(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                  const int* __restrict__ image, const uint32_t* __restrict__ tag,
                                  unsigned int N, double* __restrict__ o_pos,
                                  double* __restrict__ o_vel, double* __restrict__ o_mass,
                                  uint32_t* __restrict__ o_typeid, int32_t* __restrict__ o_image)
    {
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += gridDim.x * blockDim.x)
        {
        const unsigned int t = tag[i];
        if (t >= N)
            continue;
        const float4 p = pos[i], v = vel[i];
        o_pos[3 * (size_t)t] = p.x;
        o_pos[3 * (size_t)t + 1] = p.y;
        o_pos[3 * (size_t)t + 2] = p.z;
        o_vel[3 * (size_t)t] = v.x;
        o_vel[3 * (size_t)t + 1] = v.y;
        o_vel[3 * (size_t)t + 2] = v.z;
        o_mass[t] = v.w;
        o_typeid[t] = __float_as_uint(p.w);
        o_image[3 * (size_t)t] = image[3 * (size_t)i];
        o_image[3 * (size_t)t + 1] = image[3 * (size_t)i + 1];
        o_image[3 * (size_t)t + 2] = image[3 * (size_t)i + 2];
        }
    }

__global__ void k_rtag(const uint32_t* __restrict__ tag, unsigned int N, uint32_t* __restrict__ rtag)
    {
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += gridDim.x * blockDim.x)
        {
        const unsigned int t = tag[i];
        if (t < N)
            rtag[t] = i;
        }
    }

// one wrap pass of a coordinate triple (the host form of ParticleData::set_particles): z, then
// y (with the yz tilt), then x (with the xy / xz tilts)
__device__ __forceinline__ void wrap_pass(const gb_box& b, float& x, float& y, float& z, int& ix,
                                          int& iy, int& iz)
    {
    if (b.periodic[2])
        {
        if (z >= b.hi[2])
            {
            z = fsub(z, b.L[2]);
            y = fsub(y, fmul(b.L[2], b.yz));
            x = fsub(x, fmul(b.L[2], b.xz));
            iz++;
            }
        else if (z < b.lo[2])
            {
            z = fadd(z, b.L[2]);
            y = fadd(y, fmul(b.L[2], b.yz));
            x = fadd(x, fmul(b.L[2], b.xz));
            iz--;
            }
        }
    if (b.periodic[1])
        {
        const float ty = fmul(b.yz, z);
        if (y >= fadd(b.hi[1], ty))
            {
            y = fsub(y, b.L[1]);
            x = fsub(x, fmul(b.L[1], b.xy));
            iy++;
            }
        else if (y < fadd(b.lo[1], ty))
            {
            y = fadd(y, b.L[1]);
            x = fadd(x, fmul(b.L[1], b.xy));
            iy--;
            }
        }
    if (b.periodic[0])
        {
        const float tx = fadd(fmul(fsub(b.xz, fmul(b.xy, b.yz)), z), fmul(b.xy, y));
        if (x >= fadd(b.hi[0], tx))
            {
            x = fsub(x, b.L[0]);
            ix++;
            }
        else if (x < fadd(b.lo[0], tx))
            {
            x = fadd(x, b.L[0]);
            ix--;
            }
        }
    }

__global__ void k_snapshot_scatter(const double* __restrict__ s_pos, const double* __restrict__ s_vel,
                                   const double* __restrict__ s_mass,
                                   const uint32_t* __restrict__ s_typeid,
                                   const int32_t* __restrict__ s_image,
                                   const double* __restrict__ s_charge,
                                   const uint32_t* __restrict__ rtag, unsigned int N,
                                   unsigned int ntypes, gb_box box, float4* __restrict__ pos,
                                   float4* __restrict__ vel, int* __restrict__ image,
                                   uint32_t* __restrict__ tag, float* __restrict__ charge,
                                   uint32_t* __restrict__ err)
    {
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < N;
         t += gridDim.x * blockDim.x)
        {
        const unsigned int i = rtag ? rtag[t] : t;
        const uint32_t ty = s_typeid[t];
        if (ty >= ntypes || i >= N)
            {
            atomicMin(err, t);
            continue;
            }
        float x = (float)s_pos[3 * (size_t)t], y = (float)s_pos[3 * (size_t)t + 1],
              z = (float)s_pos[3 * (size_t)t + 2];
        int ix = s_image[3 * (size_t)t], iy = s_image[3 * (size_t)t + 1],
            iz = s_image[3 * (size_t)t + 2];
        wrap_pass(box, x, y, z, ix, iy, iz);
        wrap_pass(box, x, y, z, ix, iy, iz);
        pos[i] = make_float4(x, y, z, __uint_as_float(ty));
        vel[i] = make_float4((float)s_vel[3 * (size_t)t], (float)s_vel[3 * (size_t)t + 1],
                             (float)s_vel[3 * (size_t)t + 2], (float)s_mass[t]);
        image[3 * (size_t)i] = ix;
        image[3 * (size_t)i + 1] = iy;
        image[3 * (size_t)i + 2] = iz;
        tag[i] = t;
        if (s_charge && charge)
            charge[i] = (float)s_charge[t];
        }
    }

unsigned int io_grid(unsigned int N)
    {
    return div_up(N > 0 ? N : 1u, 256u);
    }
} // namespace
} // namespace gb

using namespace gb;

extern "C"
    {
    size_t gb_snapshot_stage_bytes(unsigned int N)
        {
        // pos, vel (3 doubles), mass, charge (double), typeid (u32), image (3 i32), rtag (u32),
        // each section 256-byte aligned
        auto up = [](size_t b) { return (b + 255) / 256 * 256; };
        const size_t n = N;
        return 2 * up(24 * n) + 2 * up(8 * n) + up(4 * n) + up(12 * n) + up(4 * n);
        }

    int gb_snapshot_gather(const float* d_pos, const float* d_vel, const int32_t* d_image,
                           const uint32_t* d_tag, unsigned int N, double* d_out_pos,
                           double* d_out_vel, double* d_out_mass, uint32_t* d_out_typeid,
                           int32_t* d_out_image, void* stream)
        {
        GB_REQUIRE(d_pos && d_vel && d_image && d_tag && d_out_pos && d_out_vel && d_out_mass
                       && d_out_typeid && d_out_image,
                   "gb_snapshot_gather: null argument");
        if (N == 0)
            return GB_OK;
        k_snapshot_gather<<<io_grid(N), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<const float4*>(d_pos), reinterpret_cast<const float4*>(d_vel), d_image,
            d_tag, N, d_out_pos, d_out_vel, d_out_mass, d_out_typeid, d_out_image);
        return check_launch("gb_snapshot_gather");
        }

    int gb_rtag(const uint32_t* d_tag, unsigned int N, uint32_t* d_rtag, void* stream)
        {
        GB_REQUIRE(d_tag && d_rtag, "gb_rtag: null argument");
        if (N == 0)
            return GB_OK;
        k_rtag<<<io_grid(N), 256, 0, (cudaStream_t)stream>>>(d_tag, N, d_rtag);
        return check_launch("gb_rtag");
        }

    int gb_snapshot_scatter(const double* d_in_pos, const double* d_in_vel,
                            const double* d_in_mass, const uint32_t* d_in_typeid,
                            const int32_t* d_in_image, const double* d_in_charge,
                            const uint32_t* d_rtag, unsigned int N, unsigned int ntypes,
                            const gb_box* box, float* d_pos, float* d_vel, int32_t* d_image,
                            uint32_t* d_tag, float* d_charge, uint32_t* d_err, void* stream)
        {
        GB_REQUIRE(d_in_pos && d_in_vel && d_in_mass && d_in_typeid && d_in_image && box && d_pos
                       && d_vel && d_image && d_tag && d_err,
                   "gb_snapshot_scatter: null argument");
        GB_REQUIRE(!d_in_charge || d_charge, "gb_snapshot_scatter: charges need d_charge");
        if (N == 0)
            return GB_OK;
        k_snapshot_scatter<<<io_grid(N), 256, 0, (cudaStream_t)stream>>>(
            d_in_pos, d_in_vel, d_in_mass, d_in_typeid, d_in_image, d_in_charge, d_rtag, N,
            ntypes, *box, reinterpret_cast<float4*>(d_pos), reinterpret_cast<float4*>(d_vel),
            d_image, d_tag, d_charge, d_err);
        return check_launch("gb_snapshot_scatter");
        }
    }
