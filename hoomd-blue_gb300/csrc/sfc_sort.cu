// Space-filling-curve particle sort (replaces SFCPackTunerGPU: hoomd/SFCPackTunerGPU.cu:26-160,
// hoomd/SFCPackTuner.cc:289-486): particles are binned on a grid^3 lattice of the box, ordered by
// the position of their bin along the reference's Hilbert traversal, ties by old index, and every
// per-particle array is gathered into the new order.
//
// The reference builds the traversal as a grid^3 table by recursion (SFCPackTuner::
// generateTraversalOrder): a cube is split into eight octants visited in the order `cell_order`,
// and octant m's own order is cell_order permuted by rule m. Here the position of a bin along
// that traversal is computed directly: the orders the recursion can reach form a small set of
// states, so a state table (state, octant) -> (rank among the eight children, next state), built
// once on the host by walking the rules from the identity order, turns the bin's coordinates into
// its traversal position with one table step per level (8 levels for the default grid of 256).
// The order then comes from a counting sort over the grid^3 buckets: histogram, exclusive scan,
// scatter, and a pass that orders the members of a shared bucket by old index (the reference
// sorts (key, index) pairs). In two dimensions the reference orders bins row by row
// (SFCPackTuner::getSortedOrder2D, grid 4096), and so does this sort.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
constexpr unsigned int SCAN_TILE = 4096; // elements per block in the scan (1024 threads x 4)
constexpr int MAX_STATES = 64;

// Octant o of a cube at (x, y, z) offsets (the reference's istep / jstep / kstep walking tables:
// a Gray-code tour of the eight corners).
constexpr int OCT_X[8] = {0, 0, 0, 0, 1, 1, 1, 1};
constexpr int OCT_Y[8] = {0, 0, 1, 1, 1, 1, 0, 0};
constexpr int OCT_Z[8] = {0, 1, 1, 0, 0, 1, 1, 0};
// Permutation rules: the order inside child m is child[k] = parent[RULE[m][k]]
// (SFCPackTuner.cc permute1 ... permute8).
constexpr int RULE[8][8] = {{0, 3, 4, 7, 6, 5, 2, 1}, {0, 7, 6, 1, 2, 5, 4, 3},
                            {0, 7, 6, 1, 2, 5, 4, 3}, {2, 3, 0, 1, 6, 7, 4, 5},
                            {2, 3, 0, 1, 6, 7, 4, 5}, {4, 3, 2, 5, 6, 1, 0, 7},
                            {4, 3, 2, 5, 6, 1, 0, 7}, {6, 5, 2, 1, 0, 3, 4, 7}};

// rank[state][octant]: which child (0..7) visits that octant; next[state][rank]: the child's state
struct HilbertTable
    {
    uint8_t rank[MAX_STATES][8];
    uint8_t next[MAX_STATES][8];
    };

const HilbertTable& hilbert_table()
    {
    static HilbertTable table;
    static std::once_flag once;
    std::call_once(once, [] {
        std::vector<std::vector<int>> states;
        states.push_back({0, 1, 2, 3, 4, 5, 6, 7});
        std::memset(&table, 0, sizeof(table));
        for (size_t s = 0; s < states.size(); s++)
            {
            const std::vector<int> order = states[s];
            for (int m = 0; m < 8; m++)
                {
                table.rank[s][order[m]] = (uint8_t)m;
                std::vector<int> child(8);
                for (int k = 0; k < 8; k++)
                    child[k] = order[RULE[m][k]];
                size_t c = 0;
                while (c < states.size() && states[c] != child)
                    c++;
                if (c == states.size())
                    states.push_back(child);
                table.next[s][m] = (uint8_t)c;
                }
            }
        });
    return table;
    }

// position of bin (x, y, z) of a 2^bits grid along the traversal
__device__ inline uint32_t hilbert_rank(const HilbertTable& t, uint32_t x, uint32_t y, uint32_t z,
                                        int bits)
    {
    uint32_t key = 0, state = 0;
    for (int b = bits - 1; b >= 0; b--)
        {
        const uint32_t bx = (x >> b) & 1u, by = (y >> b) & 1u, bz = (z >> b) & 1u;
        // octant id from the corner bits (inverse of the Gray-code tour)
        const uint32_t oct = bx ? (by ? 4u + bz : 7u - bz) : (by ? 3u - bz : bz);
        const uint32_t m = t.rank[state][oct];
        key = (key << 3) | m;
        state = t.next[state][m];
        }
    return key;
    }

__global__ void k_sfc_keys(const float4* __restrict__ pos, unsigned int N, gb_box box, int bits,
                           unsigned int ndim, HilbertTable table, uint32_t* keys, uint32_t* hist)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N)
        return;
    const float4 p = pos[i];
    float fx, fy, fz;
    make_fraction(box, p.x, p.y, p.z, fx, fy, fz);
    const uint32_t G = 1u << bits;
    // (unsigned int)(f * grid) % grid, as the reference bins (a fraction that rounds to 1 lands
    // in bin 0)
    const uint32_t cx = __float2uint_rz(fmul(fx, (float)G)) % G;
    const uint32_t cy = __float2uint_rz(fmul(fy, (float)G)) % G;
    uint32_t key;
    if (ndim == 2)
        key = cx * G + cy;
    else
        {
        const uint32_t cz = __float2uint_rz(fmul(fz, (float)G)) % G;
        key = hilbert_rank(table, cx, cy, cz, bits);
        }
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

static size_t sfc_layout(unsigned int N, int bits, unsigned int ndim, size_t* off_keys,
                         size_t* off_hist, size_t* off_tiles)
    {
    const size_t nbins = (size_t)1 << ((ndim == 2 ? 2 : 3) * bits);
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
    size_t gb_sfc_scratch_bytes_dim(unsigned int N, int grid_bits, unsigned int ndim)
        {
        size_t a, b, c;
        return sfc_layout(N, grid_bits, ndim, &a, &b, &c);
        }

    size_t gb_sfc_scratch_bytes(unsigned int N, int grid_bits)
        {
        return gb_sfc_scratch_bytes_dim(N, grid_bits, 3);
        }

    int gb_sfc_order_dim(const float* d_pos, unsigned int N, const gb_box* box, int grid_bits,
                         unsigned int ndim, uint32_t* d_order, void* d_scratch,
                         size_t scratch_bytes, void* stream)
        {
        GB_REQUIRE(box && d_order && d_scratch && (d_pos || N == 0), "gb_sfc_order: null argument");
        GB_REQUIRE(ndim == 2 || ndim == 3, "gb_sfc_order: ndim must be 2 or 3");
        GB_REQUIRE(grid_bits >= 1 && grid_bits <= (ndim == 2 ? 12 : 9),
                   "gb_sfc_order: 1 <= grid_bits <= 9 (3D) or 12 (2D)");
        size_t ok, oh, ot;
        const size_t need = sfc_layout(N, grid_bits, ndim, &ok, &oh, &ot);
        GB_REQUIRE(scratch_bytes >= need, "gb_sfc_order: scratch too small");
        if (N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        char* base = reinterpret_cast<char*>(d_scratch);
        uint32_t* keys = reinterpret_cast<uint32_t*>(base + ok);
        uint32_t* hist = reinterpret_cast<uint32_t*>(base + oh);
        uint32_t* tiles = reinterpret_cast<uint32_t*>(base + ot);
        const size_t nbins = (size_t)1 << ((ndim == 2 ? 2 : 3) * grid_bits);
        const unsigned int ntiles = (unsigned int)((nbins + SCAN_TILE - 1) / SCAN_TILE);
        if (cudaMemsetAsync(hist, 0, nbins * 4, s) != cudaSuccess)
            return fail(GB_ERR_CUDA, "gb_sfc_order: memset");
        k_sfc_keys<<<div_up(N, 256), 256, 0, s>>>(reinterpret_cast<const float4*>(d_pos), N, *box,
                                                  grid_bits, ndim, hilbert_table(), keys, hist);
        k_scan_tile<<<ntiles, 1024, 0, s>>>(hist, nbins, tiles);
        k_scan_sums<<<1, 1024, 0, s>>>(tiles, ntiles);
        k_scan_add<<<ntiles, 256, 0, s>>>(hist, nbins, tiles);
        k_sfc_scatter<<<div_up(N, 256), 256, 0, s>>>(keys, N, hist, d_order);
        k_sfc_fix_ties<<<div_up(N, 256), 256, 0, s>>>(keys, N, d_order);
        return check_launch("gb_sfc_order");
        }

    int gb_sfc_order(const float* d_pos, unsigned int N, const gb_box* box, int grid_bits,
                     uint32_t* d_order, void* d_scratch, size_t scratch_bytes, void* stream)
        {
        return gb_sfc_order_dim(d_pos, N, box, grid_bits, 3, d_order, d_scratch, scratch_bytes,
                                stream);
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
