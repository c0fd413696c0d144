// Device-side geometry and reduction helpers shared by the kernels.
//
// Geometry follows the reference's BoxDim (hoomd/BoxDim.h) at FP32. Every rounding step is an
// explicit __f*_rn intrinsic so that nvcc cannot contract a multiply-add into an FMA: distances
// computed here are bit-identical to the FP32 oracle (compiled with -ffp-contract=off), which is
// what makes neighbour-list membership (dr^2 <= r_list^2) reproducible bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "hoomd_gb300.h"

namespace gb
{

__device__ __forceinline__ float fmul(float a, float b)
    {
    return __fmul_rn(a, b);
    }
__device__ __forceinline__ float fadd(float a, float b)
    {
    return __fadd_rn(a, b);
    }
__device__ __forceinline__ float fsub(float a, float b)
    {
    return __fsub_rn(a, b);
    }

// BoxDim::minImage, device (rint) form: hoomd/BoxDim.h:322-341.
__device__ __forceinline__ void min_image(const gb_box& b, float& x, float& y, float& z)
    {
    if (b.periodic[2])
        {
        float img = rintf(fmul(z, b.Linv[2]));
        z = fsub(z, fmul(b.L[2], img));
        y = fsub(y, fmul(fmul(b.L[2], b.yz), img));
        x = fsub(x, fmul(fmul(b.L[2], b.xz), img));
        }
    if (b.periodic[1])
        {
        float img = rintf(fmul(y, b.Linv[1]));
        y = fsub(y, fmul(b.L[1], img));
        x = fsub(x, fmul(fmul(b.L[1], b.xy), img));
        }
    if (b.periodic[0])
        {
        x = fsub(x, fmul(b.L[0], rintf(fmul(x, b.Linv[0]))));
        }
    }

// Orthorhombic specialisation (tilts zero): identical arithmetic minus the zero tilt terms
// (x - 0*img == x exactly, so results are bit-identical to min_image()).
__device__ __forceinline__ void min_image_ortho(const gb_box& b, float& x, float& y, float& z)
    {
    if (b.periodic[2])
        z = fsub(z, fmul(b.L[2], rintf(fmul(z, b.Linv[2]))));
    if (b.periodic[1])
        y = fsub(y, fmul(b.L[1], rintf(fmul(y, b.Linv[1]))));
    if (b.periodic[0])
        x = fsub(x, fmul(b.L[0], rintf(fmul(x, b.Linv[0]))));
    }

// Packed FP32 pairs (add/sub/mul.rn.f32x2): two independent IEEE round-to-nearest operations
// per instruction, so each half is bit-identical to the scalar __f*_rn form.
__device__ __forceinline__ uint64_t f2pack(float lo, float hi)
    {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
    }
__device__ __forceinline__ void f2unpack(uint64_t v, float& lo, float& hi)
    {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    }
__device__ __forceinline__ uint64_t f2sub(uint64_t a, uint64_t b)
    {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
    }
__device__ __forceinline__ uint64_t f2add(uint64_t a, uint64_t b)
    {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
    }
__device__ __forceinline__ uint64_t f2mul(uint64_t a, uint64_t b)
    {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
    }

__device__ __forceinline__ uint64_t f2fma(uint64_t a, uint64_t b, uint64_t c)
    {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
    }

__device__ __forceinline__ float dot3(float x, float y, float z)
    {
    return fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z));
    }

// dot3 of both halves of packed differences. The squares are packed mul.rn.f32x2 (each half an
// IEEE round-to-nearest product) and the sums scalar __fadd_rn, which is never merged into a
// multiply-add, so each sum adds the rounded squares exactly as the scalar sequence does. The
// sums written as packed add.rn.f32x2 were measured to round differently from the scalar
// sequence on a share of inputs (as if merged with the products; a list membership decided at
// r_list^2 then differed from the reference's by one pair in a million particles).
__device__ __forceinline__ void f2dot3(uint64_t dx, uint64_t dy, uint64_t dz, float& r0,
                                       float& r1)
    {
    float x0, x1, y0, y1, z0, z1;
    f2unpack(f2mul(dx, dx), x0, x1);
    f2unpack(f2mul(dy, dy), y0, y1);
    f2unpack(f2mul(dz, dz), z0, z1);
    r0 = fadd(fadd(x0, y0), z0);
    r1 = fadd(fadd(x1, y1), z1);
    }

// BoxDim::makeFraction with no ghost layer: hoomd/BoxDim.h:276-284.
__device__ __forceinline__ void make_fraction(const gb_box& b, float x, float y, float z,
                                              float& fx, float& fy, float& fz)
    {
    float dx = fsub(x, b.lo[0]);
    float dy = fsub(y, b.lo[1]);
    float dz = fsub(z, b.lo[2]);
    dx = fsub(dx, fadd(fmul(fsub(b.xz, fmul(b.yz, b.xy)), z), fmul(b.xy, y)));
    dy = fsub(dy, fmul(b.yz, z));
    fx = fmul(dx, b.Linv[0]);
    fy = fmul(dy, b.Linv[1]);
    fz = fmul(dz, b.Linv[2]);
    }

// Cell of a position: hoomd/CellList.cc:441-476 (bin index from makeFraction). Returns false
// when the particle is outside the box (fraction outside [-1e-5, 1 + 1e-5)). One deliberate
// difference: where the reference wraps a bin index of dim (a fraction that rounds to 1, i.e. a
// particle within an ulp or so of the hi face) to bin 0, this keeps it in the last bin. The
// neighbour-list builds here take a stencil cell's periodic image from the cell index, which
// needs every particle on its own cell's side of the boundary; a particle at the hi face filed
// in bin 0 would be imaged a box length away from all its partners (the reference finds them by
// minimum image per pair). The neighbour sets are the same either way.
__device__ __forceinline__ bool cell_of(const gb_box& b, const unsigned int* dim, float x, float y,
                                        float z, unsigned int& cell)
    {
    float fx, fy, fz;
    make_fraction(b, x, y, z, fx, fy, fz);
    int ib = (int)fmul(fx, (float)dim[0]);
    int jb = (int)fmul(fy, (float)dim[1]);
    int kb = (int)fmul(fz, (float)dim[2]);
    if ((fx < -0.00001f || fx >= 1.00001f) || (fy < -0.00001f || fy >= 1.00001f)
        || (fz < -0.00001f || fz >= 1.00001f))
        return false;
    if (ib == (int)dim[0] && b.periodic[0])
        ib = (int)dim[0] - 1;
    if (jb == (int)dim[1] && b.periodic[1])
        jb = (int)dim[1] - 1;
    if (kb == (int)dim[2] && b.periodic[2])
        kb = (int)dim[2] - 1;
    if (ib < 0 || ib >= (int)dim[0] || jb < 0 || jb >= (int)dim[1] || kb < 0 || kb >= (int)dim[2])
        return false;
    cell = (unsigned int)((kb * (int)dim[1] + jb) * (int)dim[0] + ib);
    return true;
    }

// BoxDim::wrap (hoomd/BoxDim.h:407-474), no forced flags.
__device__ __forceinline__ void wrap(const gb_box& b, float& x, float& y, float& z, int& ix,
                                     int& iy, int& iz)
    {
    float oy = b.periodic[1] ? fmul(fadd(b.hi[1], b.lo[1]), 0.5f) : 0.0f;
    float oz = b.periodic[2] ? fmul(fadd(b.hi[2], b.lo[2]), 0.5f) : 0.0f;
    if (b.periodic[0])
        {
        float tilt_x = fadd(fmul(fsub(b.xz, fmul(b.xy, b.yz)), fsub(z, oz)), fmul(b.xy, fsub(y, oy)));
        if (x >= fadd(b.hi[0], tilt_x))
            {
            x = fsub(x, b.L[0]);
            ix++;
            }
        else if (x < fadd(b.lo[0], tilt_x))
            {
            x = fadd(x, b.L[0]);
            ix--;
            }
        }
    if (b.periodic[1])
        {
        float tilt_y = fmul(b.yz, fsub(z, oz));
        if (y >= fadd(b.hi[1], tilt_y))
            {
            y = fsub(y, b.L[1]);
            x = fsub(x, fmul(b.L[1], b.xy));
            iy++;
            }
        else if (y < fadd(b.lo[1], tilt_y))
            {
            y = fadd(y, b.L[1]);
            x = fadd(x, fmul(b.L[1], b.xy));
            iy--;
            }
        }
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
    }

__device__ __forceinline__ bool box_is_ortho(const gb_box& b)
    {
    return b.xy == 0.0f && b.xz == 0.0f && b.yz == 0.0f;
    }

template<class T> __device__ __forceinline__ T warp_sum(T v)
    {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
    }

// Sum over groups of TPP consecutive lanes (TPP a power of two <= 32).
template<int TPP, class T> __device__ __forceinline__ T group_sum(T v)
    {
#pragma unroll
    for (int o = TPP / 2; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o, TPP);
    return v;
    }

__device__ __forceinline__ unsigned int float_as_uint(float f)
    {
    return __float_as_uint(f);
    }

} // namespace gb
