// gb_thermo_reduce_noalloc: the FP64 thermodynamic reduction of gb_thermo_reduce, for callers
// that cannot allocate device memory.
//
// Who needs it: a host whose device memory is already handed to its own pool and accounted
// for (a framework that embeds these kernels and forbids side allocations), and a host that must
// not stall other work on the GPU (cudaFree synchronises the whole device). Such a caller cannot
// provide the global scratch buffer that gb_thermo_reduce takes, and must not have the library
// allocate one. This entry point instead uses a fixed scratch array that lives in the library
// image itself: it is created when the library is loaded on a device and stays resident on every
// GPU that loads the library until the process exits.
//
// Limits and rules:
//  * N must not exceed GB_NOALLOC_MAX_N (4,194,304 particles); larger N is rejected with
//    GB_ERR_TOO_LARGE before anything is launched.
//  * The first call in each CUDA context looks up the array's device address
//    (cudaGetSymbolAddress, with that context current) and caches it under the context's id;
//    that is once per device, and once more after a cudaDeviceReset. Make that first call
//    before any stream capture.
//  * All calls share the one array and it keeps the previous call's contents. The call clears
//    the completion counter on its stream before the reduction starts; calls that overlap on the
//    GPU (issued on different streams without ordering between them) race on the array and give
//    wrong results.
//  * No cudaMalloc, cudaFree or allocating library routine is called.
#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
constexpr unsigned int NA_BLOCK = 256;
constexpr unsigned int NA_MAX_BLOCKS = GB_NOALLOC_MAX_N / NA_BLOCK;
// [0, 256): completion counter; [256, ...): 3 doubles of partial sums per block
constexpr size_t NA_BYTES = 256 + 3 * sizeof(double) * (size_t)NA_MAX_BLOCKS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

__device__ inline void na_block_sum3(double& a, double& b, double& c)
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

// Same per-particle terms and the same fixed-order reduction as gb_thermo_reduce.
__global__ void __launch_bounds__(NA_BLOCK)
    k_thermo_noalloc(const float4* __restrict__ vel, const float4* __restrict__ force,
                     const float* __restrict__ virial, size_t pitch, unsigned int N,
                     unsigned char* scratch, double* out)
    {
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch);
    double* partials = reinterpret_cast<double*>(scratch + 256);
    __shared__ bool s_last;
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
    na_block_sum3(ke, pe, w);
    if (threadIdx.x == 0)
        {
        partials[3 * blockIdx.x] = ke;
        partials[3 * blockIdx.x + 1] = pe;
        partials[3 * blockIdx.x + 2] = w;
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
        }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    double a = 0.0, b = 0.0, c = 0.0;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x)
        {
        a += __ldcg(partials + 3 * k);
        b += __ldcg(partials + 3 * k + 1);
        c += __ldcg(partials + 3 * k + 2);
        }
    na_block_sum3(a, b, c);
    if (threadIdx.x == 0)
        {
        out[0] = 0.5 * a;
        out[1] = b;
        out[2] = c / 3.0;
        *counter = 0;
        }
    }

// Device address of g_noalloc_scratch, looked up once per CUDA context. The cache is keyed by
// the driver's context id (cuCtxGetId: unique for the life of the process), not by the device
// ordinal, so a context created after cudaDeviceReset, or another context made current on the
// same device, gets its own lookup instead of a stale address. The two driver functions are
// resolved through the runtime (cudaGetDriverEntryPointByVersion), so the library needs no link
// to libcuda; where they cannot be resolved, the address is looked up on every call.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

std::mutex g_na_mutex;
bool g_na_resolved = false;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
std::vector<std::pair<unsigned long long, void*>> g_na_cache;

// the current context's id, or false when there is none (or the driver functions are missing)
bool current_context_id(unsigned long long* id)
    {
    if (!g_na_resolved)
        {
        g_na_resolved = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q)
                == cudaSuccess
            && q == cudaDriverEntryPointSuccess)
            g_ctx_current = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q)
                == cudaSuccess
            && q == cudaDriverEntryPointSuccess)
            g_ctx_id = (CtxGetIdFn)f;
        cudaGetLastError();
        }
    if (!g_ctx_current || !g_ctx_id)
        return false;
    void* ctx = nullptr;
    if (g_ctx_current(&ctx) != 0 || ctx == nullptr)
        return false;
    return g_ctx_id(ctx, id) == 0;
    }

int noalloc_scratch_ptr(void** ptr)
    {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    unsigned long long id = 0;
    if (current_context_id(&id))
        for (const auto& kv : g_na_cache)
            if (kv.first == id)
                {
                *ptr = kv.second;
                return GB_OK;
                }
    // first call in this context (the lookup also initialises the device's primary context when
    // none is current yet)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
        return fail(GB_ERR_CUDA, std::string("gb_thermo_reduce_noalloc: cudaGetSymbolAddress: ")
                                     + cudaGetErrorString(e));
    if (current_context_id(&id))
        g_na_cache.emplace_back(id, p);
    *ptr = p;
    return GB_OK;
    }
} // namespace
} // namespace gb

using namespace gb;

extern "C"
    {
    int gb_thermo_reduce_noalloc(const float* d_vel, const float* d_force, const float* d_virial,
                                 size_t virial_pitch, unsigned int N, double* d_out,
                                 void* stream)
        {
        GB_REQUIRE(d_vel && d_out, "gb_thermo_reduce_noalloc: null argument");
        GB_REQUIRE(!d_virial || virial_pitch >= N, "gb_thermo_reduce_noalloc: virial pitch < N");
        if (N > GB_NOALLOC_MAX_N)
            return fail(GB_ERR_TOO_LARGE,
                        "gb_thermo_reduce_noalloc: N exceeds GB_NOALLOC_MAX_N (4194304 "
                        "particles); use gb_thermo_reduce with caller-provided scratch");
        void* scratch = nullptr;
        int rc = noalloc_scratch_ptr(&scratch);
        if (rc != GB_OK)
            return rc;
        cudaStream_t s = (cudaStream_t)stream;
        // the counter must start at zero; the array keeps whatever the previous call left
        cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess)
            return fail(GB_ERR_CUDA, std::string("gb_thermo_reduce_noalloc: clearing the "
                                                 "counter: ")
                                         + cudaGetErrorString(e));
        const unsigned int nb = div_up(N > 0 ? N : 1, NA_BLOCK);
        k_thermo_noalloc<<<nb, NA_BLOCK, 0, s>>>(
            reinterpret_cast<const float4*>(d_vel), reinterpret_cast<const float4*>(d_force),
            d_virial, virial_pitch, N, reinterpret_cast<unsigned char*>(scratch), d_out);
        return check_launch("gb_thermo_reduce_noalloc");
        }
    }
