// hoomd/HOOMDMath.h for pair-evaluator plugins built against hoomd_gb300.
//
// A plugin evaluator written for the reference (example_plugins/pair_plugin/EvaluatorPairExample.h
// is the template) includes "hoomd/HOOMDMath.h" and uses Scalar, Scalar2/3/4, make_scalar*,
// __int_as_scalar / __scalar_as_int, the fast:: and slow:: math functions, and DEVICE /
// HOSTDEVICE qualifiers selected by __HIPCC__. This header provides those names for this
// library's FP32 path (Scalar = float, HOOMD_LONGREAL_SIZE 32), so such an evaluator compiles
// here without a source change: its kernel translation unit with nvcc (where __HIPCC__ is defined,
// as the reference's HIP layer defines it under nvcc), its module translation unit with the host
// compiler (where pybind11 is available for param_type(pybind11::dict, bool) and asDict()).
#ifndef __HOOMD_MATH_H__
#define __HOOMD_MATH_H__

#if defined(__CUDACC__) && !defined(__HIPCC__)
#define __HIPCC__ 1
#endif

#include <vector_types.h>

#ifndef __HIPCC__
#include <Python.h>
#include <pybind11/pybind11.h>
#endif

#include <cmath>
#include <cstring>

#ifdef __HIPCC__
#define HOSTDEVICE __host__ __device__
#define DEVICE __device__
#else
#define HOSTDEVICE
#define DEVICE
#endif

#ifndef HOOMD_LONGREAL_SIZE
#define HOOMD_LONGREAL_SIZE 32
#endif
#ifndef HOOMD_SHORTREAL_SIZE
#define HOOMD_SHORTREAL_SIZE 32
#endif

namespace hoomd
    {
// the pair kernels here run in FP32 (forces, energies, virials; FP64 only in reductions)
typedef float Scalar;
typedef float2 Scalar2;
typedef float3 Scalar3;
typedef float4 Scalar4;
typedef float LongReal;
typedef float2 LongReal2;
typedef float3 LongReal3;
typedef float4 LongReal4;
typedef float ShortReal;
typedef float2 ShortReal2;
typedef float3 ShortReal3;
typedef float4 ShortReal4;

HOSTDEVICE inline Scalar2 make_scalar2(Scalar x, Scalar y)
    {
    Scalar2 v;
    v.x = x;
    v.y = y;
    return v;
    }

HOSTDEVICE inline Scalar3 make_scalar3(Scalar x, Scalar y, Scalar z)
    {
    Scalar3 v;
    v.x = x;
    v.y = y;
    v.z = z;
    return v;
    }

HOSTDEVICE inline Scalar4 make_scalar4(Scalar x, Scalar y, Scalar z, Scalar w)
    {
    Scalar4 v;
    v.x = x;
    v.y = y;
    v.z = z;
    v.w = w;
    return v;
    }

// an integer carried in the bits of a Scalar (particle types in position.w)
HOSTDEVICE inline Scalar __int_as_scalar(int a)
    {
#ifdef __CUDA_ARCH__
    return ::__int_as_float(a);
#else
    Scalar s;
    std::memcpy(&s, &a, sizeof(s));
    return s;
#endif
    }

HOSTDEVICE inline int __scalar_as_int(Scalar b)
    {
#ifdef __CUDA_ARCH__
    return ::__float_as_int(b);
#else
    int a;
    std::memcpy(&a, &b, sizeof(a));
    return a;
#endif
    }

// fast:: may use the GPU's approximate functions; slow:: keeps the IEEE-rounded forms
namespace fast
    {
HOSTDEVICE inline float sqrt(float x)
    {
#ifdef __CUDA_ARCH__
    return ::sqrtf(x);
#else
    return std::sqrt(x);
#endif
    }
HOSTDEVICE inline float rsqrt(float x)
    {
#ifdef __CUDA_ARCH__
    return ::rsqrtf(x);
#else
    return 1.0f / std::sqrt(x);
#endif
    }
HOSTDEVICE inline float exp(float x)
    {
#ifdef __CUDA_ARCH__
    return ::__expf(x);
#else
    return std::exp(x);
#endif
    }
HOSTDEVICE inline float log(float x)
    {
#ifdef __CUDA_ARCH__
    return ::__logf(x);
#else
    return std::log(x);
#endif
    }
HOSTDEVICE inline float pow(float x, float y)
    {
#ifdef __CUDA_ARCH__
    return ::__powf(x, y);
#else
    return std::pow(x, y);
#endif
    }
HOSTDEVICE inline float sin(float x)
    {
#ifdef __CUDA_ARCH__
    return ::__sinf(x);
#else
    return std::sin(x);
#endif
    }
HOSTDEVICE inline float cos(float x)
    {
#ifdef __CUDA_ARCH__
    return ::__cosf(x);
#else
    return std::cos(x);
#endif
    }
HOSTDEVICE inline void sincos(float x, float& s, float& c)
    {
    s = fast::sin(x);
    c = fast::cos(x);
    }
HOSTDEVICE inline float acos(float x)
    {
#ifdef __CUDA_ARCH__
    return ::acosf(x);
#else
    return std::acos(x);
#endif
    }
HOSTDEVICE inline float erfc(float x)
    {
#ifdef __CUDA_ARCH__
    return ::erfcf(x);
#else
    return std::erfc(x);
#endif
    }
    } // namespace fast

namespace slow
    {
HOSTDEVICE inline float sqrt(float x)
    {
#ifdef __CUDA_ARCH__
    return ::sqrtf(x);
#else
    return std::sqrt(x);
#endif
    }
HOSTDEVICE inline float rsqrt(float x)
    {
    return 1.0f / slow::sqrt(x);
    }
HOSTDEVICE inline float exp(float x)
    {
#ifdef __CUDA_ARCH__
    return ::expf(x);
#else
    return std::exp(x);
#endif
    }
HOSTDEVICE inline float log(float x)
    {
#ifdef __CUDA_ARCH__
    return ::logf(x);
#else
    return std::log(x);
#endif
    }
HOSTDEVICE inline float pow(float x, float y)
    {
#ifdef __CUDA_ARCH__
    return ::powf(x, y);
#else
    return std::pow(x, y);
#endif
    }
HOSTDEVICE inline float sin(float x)
    {
#ifdef __CUDA_ARCH__
    return ::sinf(x);
#else
    return std::sin(x);
#endif
    }
HOSTDEVICE inline float cos(float x)
    {
#ifdef __CUDA_ARCH__
    return ::cosf(x);
#else
    return std::cos(x);
#endif
    }
HOSTDEVICE inline void sincos(float x, float& s, float& c)
    {
    s = slow::sin(x);
    c = slow::cos(x);
    }
HOSTDEVICE inline float acos(float x)
    {
#ifdef __CUDA_ARCH__
    return ::acosf(x);
#else
    return std::acos(x);
#endif
    }
HOSTDEVICE inline float erfc(float x)
    {
#ifdef __CUDA_ARCH__
    return ::erfcf(x);
#else
    return std::erfc(x);
#endif
    }
HOSTDEVICE inline float rint(float x)
    {
#ifdef __CUDA_ARCH__
    return ::rintf(x);
#else
    return std::rint(x);
#endif
    }
    } // namespace slow

    } // namespace hoomd

#endif // __HOOMD_MATH_H__
