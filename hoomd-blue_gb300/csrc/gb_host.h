// Host-side helpers for the C ABI: error recording and launch checking.
#pragma once

#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "hoomd_gb300.h"

namespace gb
{
void set_error(const std::string& msg);

inline int fail(int code, const std::string& msg)
    {
    set_error(msg);
    return code;
    }

// Check the launch that was just issued (configuration errors are reported synchronously by
// cudaGetLastError; execution errors surface at the caller's next synchronisation).
inline int check_launch(const char* what)
    {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(GB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return GB_OK;
    }

inline unsigned int div_up(unsigned long long a, unsigned long long b)
    {
    return (unsigned int)((a + b - 1) / b);
    }

int num_sms();
} // namespace gb

#define GB_REQUIRE(cond, msg)                                                                     \
    do                                                                                            \
        {                                                                                         \
        if (!(cond))                                                                              \
            return ::gb::fail(GB_ERR_INVALID, msg);                                               \
        } while (0)
