// Space-filling-curve particle sort (replaces SFCPackTunerGPU: hoomd/SFCPackTunerGPU.cu:26-160
// bins particles on a grid^3 lattice, orders them along a Hilbert curve with thrust::sort_by_key
// and gathers every per-particle array).
//
// Here the Hilbert index of each particle's grid cell is computed arithmetically with Skilling's
// transpose algorithm (J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707, 2004)
// instead of the reference's recursive traversal table, and the order is produced by a counting
// sort over the grid^3 buckets: histogram, exclusive scan, scatter. Buckets are far smaller than
// a particle's volume at liquid densities, so ties are rare; a final pass orders the members of
// any shared bucket by old index, which makes the permutation deterministic.
#include <cstdint>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
constexpr unsigned int SCAN_TILE = 4096; // elements per block in the scan (1024 threads x 4)

// Skilling: axes -> transposed Hilbert index, then interleave to a 3*bits-bit key.
__device__ inline uint32_t hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits)
    {
    uint32_t X[3] = {x, y, z};
    const uint32_t M = 1u << (bits - 1);
    // inverse undo
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        {
        const uint32_t P = Q - 1;
        for (int i = 0; i < 3; i++)
            {
            if (X[i] & Q)
                X[0] ^= P;
            else
                {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
                }
            }
        }
    // Gray encode
    for (int i = 1; i < 3; i++)
        X[i] ^= X[i - 1];
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q)
            t ^= Q - 1;
    for (int i = 0; i < 3; i++)
        X[i] ^= t;
    // interleave: bit b of X[i] -> key bit 3*b + (2 - i)
    uint32_t key = 0;
    for (int b = bits - 1; b >= 0; b--)
        for (int i = 0; i < 3; i++)
            key = (key << 1) | ((X[i] >> b) & 1u);
    return key;
    }

__global__ void k_sfc_keys(const float4* __restrict__ pos, unsigned int N, gb_box box, int bits,
                           uint32_t* keys, uint32_t* hist)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N)
        return;
    const float4 p = pos[i];
    float fx, fy, fz;
    make_fraction(box, p.x, p.y, p.z, fx, fy, fz);
    const int G = 1 << bits;
    int c[3] = {(int)(fx * G), (int)(fy * G), (int)(fz * G)};
    for (int d = 0; d < 3; d++)
        c[d] = c[d] < 0 ? 0 : (c[d] >= G ? G - 1 : c[d]);
    const uint32_t key = hilbert3(c[0], c[1], c[2], bits);
    keys[i] = key;
    atomicAdd(&hist[key], 1u);
    }

// Exclusive scan, pass 1: per-tile scan in place, tile totals out.
__global__ void __launch_bounds__(1024) k_scan_tile(uint32_t* data, size_t n, uint32_t* tile_sum)
    {
    __shared__ uint32_t s_warp[32];
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + threadIdx.x * 4;
    uint32_t v[4];
    uint32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
        {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        tsum += v[k];
        }
    // inclusive warp scan of thread sums
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    uint32_t inc = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o)
            inc += y;
        }
    if (lane == 31)
        s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0)
        {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += y;
            }
        s_warp[lane] = w; // inclusive over warps
        }
    __syncthreads();
    uint32_t run = inc - tsum + (warp > 0 ? s_warp[warp - 1] : 0u);
#pragma unroll
    for (int k = 0; k < 4; k++)
        {
        if (base + k < n)
            data[base + k] = run;
        run += v[k];
        }
    if (threadIdx.x == 1023)
        tile_sum[blockIdx.x] = s_warp[31];
    }

// Pass 2: exclusive scan of the tile totals by one block (looping over chunks of 1024).
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* sums, unsigned int ntiles)
    {
    __shared__ uint32_t s[1024];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0)
        s_carry = 0;
    __syncthreads();
    for (unsigned int base = 0; base < ntiles; base += 1024)
        {
        const unsigned int i = base + threadIdx.x;
        const uint32_t v = (i < ntiles) ? sums[i] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (unsigned int o = 1; o < 1024; o <<= 1)
            {
            const uint32_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
            }
        if (i < ntiles)
            sums[i] = s[threadIdx.x] - v + s_carry;
        __syncthreads();
        if (threadIdx.x == 1023)
            s_carry += s[1023];
        __syncthreads();
        }
    }

__global__ void k_scan_add(uint32_t* data, size_t n, const uint32_t* tile_sum)
    {
    const size_t base = (size_t)blockIdx.x * SCAN_TILE;
    const uint32_t add = tile_sum[blockIdx.x];
    for (unsigned int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x)
        if (base + k < n)
            data[base + k] += add;
    }

__global__ void k_sfc_scatter(const uint32_t* __restrict__ keys, unsigned int N, uint32_t* offsets,
                              uint32_t* order)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N)
        return;
    const uint32_t slot = atomicAdd(&offsets[keys[i]], 1u);
    order[slot] = i;
    }

// Deterministic tie-break: positions sharing a key are ordered by old index. The run of equal
// keys starting at a new position is short (buckets hold ~0.1 particles at liquid density).
__global__ void k_sfc_fix_ties(const uint32_t* __restrict__ keys, unsigned int N, uint32_t* order)
    {
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N)
        return;
    const uint32_t k = keys[order[s]];
    if (s > 0 && keys[order[s - 1]] == k)
        return; // not the start of a run
    unsigned int e = s + 1;
    while (e < N && keys[order[e]] == k)
        e++;
    if (e - s < 2)
        return;
    for (unsigned int a = s + 1; a < e; a++)
        {
        const uint32_t v = order[a];
        unsigned int b = a;
        while (b > s && order[b - 1] > v)
            {
            order[b] = order[b - 1];
            b--;
            }
        order[b] = v;
        }
    }

template<class T>
__global__ void k_gather(T* __restrict__ dst, const T* __restrict__ src,
                         const uint32_t* __restrict__ order, unsigned int N)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N)
        dst[i] = src[order[i]];
    }

struct alignas(4) b12
    {
    uint32_t v[3];
    };
} // namespace

static size_t sfc_layout(unsigned int N, int bits, size_t* off_keys, size_t* off_hist,
                         size_t* off_tiles)
    {
    const size_t nbins = (size_t)1 << (3 * bits);
    const size_t ntiles = (nbins + SCAN_TILE - 1) / SCAN_TILE;
    size_t o = 0;
    *off_keys = o;
    o += ((size_t)N * 4 + 255) / 256 * 256;
    *off_hist = o;
    o += (nbins * 4 + 255) / 256 * 256;
    *off_tiles = o;
    o += (ntiles * 4 + 255) / 256 * 256;
    return o;
    }
} // namespace gb

using namespace gb;

extern "C"
    {
    size_t gb_sfc_scratch_bytes(unsigned int N, int grid_bits)
        {
        size_t a, b, c;
        return sfc_layout(N, grid_bits, &a, &b, &c);
        }

    int gb_sfc_order(const float* d_pos, unsigned int N, const gb_box* box, int grid_bits,
                     uint32_t* d_order, void* d_scratch, size_t scratch_bytes, void* stream)
        {
        GB_REQUIRE(box && d_order && d_scratch && (d_pos || N == 0), "gb_sfc_order: null argument");
        GB_REQUIRE(grid_bits >= 1 && grid_bits <= 9, "gb_sfc_order: 1 <= grid_bits <= 9");
        size_t ok, oh, ot;
        const size_t need = sfc_layout(N, grid_bits, &ok, &oh, &ot);
        GB_REQUIRE(scratch_bytes >= need, "gb_sfc_order: scratch too small");
        if (N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        char* base = reinterpret_cast<char*>(d_scratch);
        uint32_t* keys = reinterpret_cast<uint32_t*>(base + ok);
        uint32_t* hist = reinterpret_cast<uint32_t*>(base + oh);
        uint32_t* tiles = reinterpret_cast<uint32_t*>(base + ot);
        const size_t nbins = (size_t)1 << (3 * grid_bits);
        const unsigned int ntiles = (unsigned int)((nbins + SCAN_TILE - 1) / SCAN_TILE);
        if (cudaMemsetAsync(hist, 0, nbins * 4, s) != cudaSuccess)
            return fail(GB_ERR_CUDA, "gb_sfc_order: memset");
        k_sfc_keys<<<div_up(N, 256), 256, 0, s>>>(reinterpret_cast<const float4*>(d_pos), N, *box,
                                                  grid_bits, keys, hist);
        k_scan_tile<<<ntiles, 1024, 0, s>>>(hist, nbins, tiles);
        k_scan_sums<<<1, 1024, 0, s>>>(tiles, ntiles);
        k_scan_add<<<ntiles, 256, 0, s>>>(hist, nbins, tiles);
        k_sfc_scatter<<<div_up(N, 256), 256, 0, s>>>(keys, N, hist, d_order);
        k_sfc_fix_ties<<<div_up(N, 256), 256, 0, s>>>(keys, N, d_order);
        return check_launch("gb_sfc_order");
        }

    int gb_gather(void* d_dst, const void* d_src, const uint32_t* d_order, unsigned int N,
                  unsigned int elem_bytes, void* stream)
        {
        GB_REQUIRE(d_dst && d_src && d_order, "gb_gather: null argument");
        GB_REQUIRE(d_dst != d_src, "gb_gather: in-place gather is not supported");
        if (N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        const unsigned int g = div_up(N, 256);
        switch (elem_bytes)
            {
        case 4:
            k_gather<<<g, 256, 0, s>>>((uint32_t*)d_dst, (const uint32_t*)d_src, d_order, N);
            break;
        case 8:
            k_gather<<<g, 256, 0, s>>>((uint2*)d_dst, (const uint2*)d_src, d_order, N);
            break;
        case 12:
            k_gather<<<g, 256, 0, s>>>((b12*)d_dst, (const b12*)d_src, d_order, N);
            break;
        case 16:
            k_gather<<<g, 256, 0, s>>>((uint4*)d_dst, (const uint4*)d_src, d_order, N);
            break;
        default:
            return fail(GB_ERR_INVALID, "gb_gather: element size must be 4, 8, 12 or 16 bytes");
            }
        return check_launch("gb_gather");
        }
    }
