// Replica ensembles: many independent single-type LJ systems advanced in one persistent launch.
//
// The reference runs one system per Simulation; each of its steps is IntegratorTwoStep::update
// (hoomd/md/IntegratorTwoStep.cc:51-139) with TwoStepConstantVolume (step one, the neighbour-list
// distance check and rebuild, PotentialPair<EvaluatorPairLJ> forces, step two) and the Bussi
// thermostat (hoomd/md/Thermostat.h:357-446). Here one CTA owns one replica at a time and runs
// all of its steps between block barriers:
//
//   step one + distance check      (TwoStepConstantVolume.cc:37-55, NeighborListGPU.cu:42-83)
//   [cell list + neighbour list]   counting sort of the replica into its cells (one shared-memory
//                                  counter per cell, exact sizes, so the cell list cannot
//                                  overflow), slots ordered by particle index, then the binned
//                                  search with the same FP32 roundings as gpu_compute_nlist_binned
//                                  (NeighborListGPUBinned.cu:52-298), so the lists are the same sets
//   pair forces + step two         (PotentialPairGPU.cuh:140-404, TwoStepConstantVolume.cc:213-261)
//   FP64 energy sums, Bussi factor (ComputeThermo.cc:76-290, Thermostat.h:416-446)
//
// The Bussi draws depend only on the timestep, seed and dof, so a window of them is drawn in
// parallel by the whole CTA ahead of the steps that use them. The energy sums run over fixed
// 32-particle chunks in a fixed order, which makes every replica's trajectory independent of the
// block size and of which CTA ran it. CTAs take replicas from a queue with one atomic each and
// never wait for one another; the last CTA to leave resets the queue for the next launch.
#include <cstdint>

#include "evaluators.cuh"
#include "gb_device.cuh"
#include "gb_host.h"
#include "rng.cuh"

namespace gb
{
namespace
{
constexpr uint32_t NO_REPLICA = 0xffffffffu;

struct RepArrays
    {
    float4* pos;
    float4* vel;
    float4* accel;
    int4* image;
    float4* force;
    float4* last_pos;
    uint32_t* n_neigh;
    uint32_t* nlist;
    uint32_t* cellidx; // per particle: its cell at the last build
    float4* sorted;    // particles in cell order: x, y, z, index bits
    double2* chunk;    // per 32 particles: (sum m v^2, sum energy)
    uint64_t* clocks;  // optional per-replica phase cycle counters
    };

constexpr size_t scratch_cellidx(uint64_t n)
    {
    return (n * 4 + 255) / 256 * 256;
    }
constexpr size_t scratch_sorted(uint64_t n)
    {
    return (n * 16 + 255) / 256 * 256;
    }
constexpr size_t scratch_chunk(uint64_t n)
    {
    return ((n + 31) / 32 * 16 + 255) / 256 * 256;
    }

// Candidate-stream search (stream_search): cells of at most STREAM_OCC particles; per warp
// the own particles by pairs (512 B), the plane record (128 B), and the candidate indices and
// ballot masks of up to STREAM_NB blocks of 32 candidates (one plane's stream).
constexpr uint32_t STREAM_OCC = 40;
constexpr uint32_t STREAM_NB = (9 * STREAM_OCC + 31) / 32;
constexpr size_t STREAM_WARP_BYTES = 512 + 128 + 2 * 4 * 32 * STREAM_NB;

__host__ __device__ inline size_t smem_cells_bytes(uint32_t max_cells, uint32_t block)
    {
    // Bussi draws (double2 per thread), cell starts (max_cells + 1), cell counters (max_cells)
    return ((size_t)block * 16 + (size_t)(2 * max_cells + 1) * 4 + 15) / 16 * 16;
    }

__host__ __device__ inline size_t smem_bytes(uint32_t max_cells, uint32_t block)
    {
    return smem_cells_bytes(max_cells, block) + (size_t)(block / 32) * STREAM_WARP_BYTES;
    }

struct RepShared
    {
    gb_replica rep;     // live copy of the replica's record
    uint64_t wbase;     // first timestep of the Bussi draw window
    uint32_t wcount;    // draws in the window
    uint32_t rebuild;   // set by step one when a particle moved far enough
    uint32_t err;       // status bits raised during a build
    uint32_t maxcnt;    // largest neighbour count found by the last build
    uint32_t maxocc;    // most particles in one cell at the last build
    uint32_t wtot[32];  // scan scratch
    long long clk[4];   // cycles in step one, builds, pair step, Bussi draws (thread 0)
    long long t0;       // last phase boundary (thread 0)
    };

// Phase boundary: charge the cycles since the last boundary to phase k (thread 0 only).
__device__ __forceinline__ void stamp(RepShared& sh, int k)
    {
    if (threadIdx.x == 0)
        {
        const long long t1 = clock64();
        sh.clk[k] += t1 - sh.t0;
        sh.t0 = t1;
        }
    }

static_assert(sizeof(gb_replica) % 8 == 0, "gb_replica must be a whole number of doubles");

// Exclusive scan of cnt[0, n) into start[0, n], start[n] = total. Whole block; ends synced.
__device__ void block_scan(const uint32_t* cnt, uint32_t* start, uint32_t n, uint32_t* wtot)
    {
    const uint32_t T = blockDim.x, t = threadIdx.x;
    const uint32_t lane = t % 32, warp = t / 32, nw = T / 32;
    const uint32_t seg = (n + T - 1) / T;
    const uint32_t c0 = min(t * seg, n), c1 = min(c0 + seg, n);
    uint32_t local = 0;
    for (uint32_t c = c0; c < c1; c++)
        local += cnt[c];
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o)
            incl += v;
        }
    if (lane == 31)
        wtot[warp] = incl;
    __syncthreads();
    if (warp == 0)
        {
        const uint32_t v = lane < nw ? wtot[lane] : 0u;
        uint32_t w = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
            if ((int)lane >= o)
                w += u;
            }
        if (lane < nw)
            wtot[lane] = w - v;
        if (lane == nw - 1)
            start[n] = w;
        }
    __syncthreads();
    uint32_t run = wtot[warp] + incl - local;
    for (uint32_t c = c0; c < c1; c++)
        {
        start[c] = run;
        run += cnt[c];
        }
    __syncthreads();
    }

__device__ __forceinline__ uint32_t wrap_index(int c, int n)
    {
    return (uint32_t)(c < 0 ? c + n : (c >= n ? c - n : c));
    }

// Candidate-stream search of one replica (the main build's k_nlist_stream): a warp per cell, the lanes holding 32 candidates of one stencil
// plane's stream (nine cells in the order (row, column), each a run of the cell-ordered array),
// the own particles tested two at a time against them (packed differences and squares, scalar
// sums: the per-thread search's roundings), one ballot mask per own particle and block, then lane
// p appends own particle p's hits in stream order, which is the per-thread search's order. Used
// for orthorhombic replicas with at least four cells a side, stencil 1 and at most STREAM_OCC
// particles a cell (cell images then come from the cell offsets, as in the per-thread search).
// Returns the warp's largest neighbour count.
__device__ __noinline__ uint32_t stream_search(const gb_replica& R, const RepArrays& A,
                                               const uint32_t* s_start, unsigned char* s_stream,
                                               float rlsq)
    {
    const uint32_t lane = threadIdx.x % 32, warp = threadIdx.x / 32, nwarps = blockDim.x / 32;
    const uint32_t dims[3] = {R.dim[0], R.dim[1], R.dim[2]};
    const uint32_t ncell = dims[0] * dims[1] * dims[2];
    const gb_box box = R.box;
    const float4* sorted = A.sorted + R.first;
    uint32_t* nlist = A.nlist + R.nlist_offset;
    const uint32_t Nmax = R.Nmax;
    const uint32_t stride = R.stride;
    const float inf = __int_as_float(0x7f800000);
    unsigned char* base = s_stream + (size_t)warp * STREAM_WARP_BYTES;
    float4* s_oa = reinterpret_cast<float4*>(base);     // (x, x', y, y') of own pairs
    float4* s_ob = s_oa + 16;                           // (z, z', index, index')
    uint32_t* s_plane = reinterpret_cast<uint32_t*>(s_ob + 16); // [0, 10) offsets, [10, 19)
                                                        // run starts, [19, 28) images
    uint32_t* s_cj = s_plane + 32;
    uint32_t* s_mask = s_cj + 32 * STREAM_NB;
    uint32_t my_max = 0;

    for (uint32_t cell = warp; cell < ncell; cell += nwarps)
        {
        const uint32_t c0 = s_start[cell], csize = s_start[cell + 1] - c0;
        const int ci = cell % dims[0], cj = (cell / dims[0]) % dims[1],
                  ck = cell / (dims[0] * dims[1]);
        for (uint32_t ob = 0; ob < csize; ob += 32)
            {
            const uint32_t n_pass = min(csize - ob, 32u);
            const bool active = lane < n_pass;
            float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
            if (active)
                {
                pi = sorted[c0 + ob + lane];
                float* a = reinterpret_cast<float*>(s_oa + lane / 2) + (lane & 1);
                float* bz = reinterpret_cast<float*>(s_ob + lane / 2) + (lane & 1);
                a[0] = pi.x;
                a[2] = pi.y;
                bz[0] = pi.z;
                bz[2] = pi.w;
                }
            const uint32_t i = __float_as_uint(pi.w);
            uint32_t wo = i * 4u;
            const uint32_t jump = stride * 4u - 3u;
            uint32_t cnt = 0;
            for (int pz = -1; pz <= 1; pz++)
                {
                uint32_t q_n = 0;
                bool q_wrap = false;
                if (lane < 9)
                    {
                    const int ox = lane % 3 - 1, oy = lane / 3 - 1;
                    const int x = ci + ox, y = cj + oy, z = ck + pz;
                    const uint32_t q_cell = (wrap_index(z, (int)dims[2]) * dims[1]
                                             + wrap_index(y, (int)dims[1])) * dims[0]
                                            + wrap_index(x, (int)dims[0]);
                    const uint32_t qs = s_start[q_cell];
                    q_n = s_start[q_cell + 1] - qs;
                    const int ix = x >= (int)dims[0] ? 1 : (x < 0 ? -1 : 0);
                    const int iy = y >= (int)dims[1] ? 1 : (y < 0 ? -1 : 0);
                    const int iz = z >= (int)dims[2] ? 1 : (z < 0 ? -1 : 0);
                    q_wrap = ix != 0 || iy != 0 || iz != 0;
                    s_plane[10 + lane] = qs;
                    s_plane[19 + lane] = (uint32_t)((ix + 1) | ((iy + 1) << 2) | ((iz + 1) << 4));
                    }
                uint32_t incl = q_n;
#pragma unroll
                for (int o = 1; o < 16; o <<= 1)
                    {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if ((int)lane >= o)
                        incl += y;
                    }
                if (lane < 9)
                    s_plane[lane] = incl - q_n;
                const uint32_t total = __shfl_sync(0xffffffffu, incl, 8);
                if (lane == 9)
                    s_plane[9] = total;
                const bool plane_wraps = __any_sync(0xffffffffu, q_wrap);
                __syncwarp();
                const uint32_t nb = (total + 31u) / 32u;
                uint32_t q = 0;
                for (uint32_t b = 0; b < nb; b++)
                    {
                    const uint32_t k = 32u * b + lane;
                    float cx = inf, cy = inf, cz = inf, sx = 0.f, sy = 0.f, sz = 0.f;
                    uint32_t cjdx = 0xffffffffu;
                    if (k < total)
                        {
                        while (k >= s_plane[q + 1])
                            q++;
                        const float4 c = sorted[s_plane[10 + q] + (k - s_plane[q])];
                        cx = c.x;
                        cy = c.y;
                        cz = c.z;
                        cjdx = __float_as_uint(c.w);
                        const uint32_t img = s_plane[19 + q];
                        sx = fmul(box.L[0], (float)((int)(img & 3u) - 1));
                        sy = fmul(box.L[1], (float)((int)((img >> 2) & 3u) - 1));
                        sz = fmul(box.L[2], (float)((int)((img >> 4) & 3u) - 1));
                        }
                    s_cj[k] = cjdx;
                    uint32_t* mrow = s_mask + 32u * b;
                    auto test = [&](auto wrap_tag) {
                        constexpr bool wrapped = decltype(wrap_tag)::value;
                        const uint64_t cx2 = f2pack(cx, cx), cy2 = f2pack(cy, cy),
                                       cz2 = f2pack(cz, cz);
                        uint32_t p = 0;
#pragma unroll 2
                        for (; p + 1 < n_pass; p += 2)
                            {
                            const float4 oa = s_oa[p / 2], obz = s_ob[p / 2];
                            uint64_t dx = f2sub(f2pack(oa.x, oa.y), cx2);
                            uint64_t dy = f2sub(f2pack(oa.z, oa.w), cy2);
                            uint64_t dz = f2sub(f2pack(obz.x, obz.y), cz2);
                            if (wrapped)
                                {
                                dx = f2sub(dx, f2pack(sx, sx));
                                dy = f2sub(dy, f2pack(sy, sy));
                                dz = f2sub(dz, f2pack(sz, sz));
                                }
                            float r0, r1;
                            f2dot3(dx, dy, dz, r0, r1);
                            const uint32_t m0 = __ballot_sync(
                                0xffffffffu, r0 <= rlsq && cjdx != __float_as_uint(obz.z));
                            const uint32_t m1 = __ballot_sync(
                                0xffffffffu, r1 <= rlsq && cjdx != __float_as_uint(obz.w));
                            if (lane == 0)
                                *reinterpret_cast<uint2*>(mrow + p) = make_uint2(m0, m1);
                            }
                        for (; p < n_pass; p++)
                            {
                            const float* a = reinterpret_cast<const float*>(s_oa + p / 2) + (p & 1);
                            const float* bz = reinterpret_cast<const float*>(s_ob + p / 2) + (p & 1);
                            float dx = fsub(a[0], cx), dy = fsub(a[2], cy), dz = fsub(bz[0], cz);
                            if (wrapped)
                                {
                                dx = fsub(dx, sx);
                                dy = fsub(dy, sy);
                                dz = fsub(dz, sz);
                                }
                            const bool hit = dot3(dx, dy, dz) <= rlsq
                                             && cjdx != __float_as_uint(bz[2]);
                            const uint32_t m = __ballot_sync(0xffffffffu, hit);
                            if (lane == 0)
                                mrow[p] = m;
                            }
                    };
                    if (plane_wraps)
                        test(std::true_type {});
                    else
                        test(std::false_type {});
                    }
                __syncwarp();
                if (active)
                    {
                    for (uint32_t b = 0; b < nb; b++)
                        {
                        uint32_t m = s_mask[32u * b + lane];
                        const uint32_t* cjb = s_cj + 32u * b;
                        auto put = [&](uint32_t j) {
                            if (cnt < Nmax)
                                nlist[wo] = j;
                            cnt++;
                            wo += (cnt & 3u) ? 1u : jump;
                        };
                        while (m)
                            {
                            const uint32_t t0 = __ffs(m) - 1;
                            m &= m - 1u;
                            const uint32_t t1 = m ? __ffs(m) - 1 : t0;
                            const bool two = m != 0u;
                            m &= m - 1u;
                            const uint32_t j0 = cjb[t0], j1 = cjb[t1];
                            put(j0);
                            if (two)
                                put(j1);
                            }
                        }
                    }
                __syncwarp();
                }
            if (active)
                {
                A.n_neigh[R.first + i] = min(cnt, Nmax);
                A.last_pos[R.first + i] = make_float4(pi.x, pi.y, pi.z, 0.0f);
                my_max = max(my_max, cnt);
                }
            __syncwarp();
            }
        }
    return my_max;
    }

// Cell list + neighbour list of the replica in sh.rep. Sets sh.err / sh.maxcnt; ends synced.
// Not inlined (nor are the other phases): each phase gets its own register allocation.
template<int MAXT>
__device__ __noinline__ void build_lists(RepShared& sh, const RepArrays& A, uint32_t* s_start,
                                         uint32_t* s_cnt, unsigned char* s_stream)
    {
    const gb_replica& R = sh.rep;
    const uint32_t T = blockDim.x, t = threadIdx.x;
    const uint32_t N = R.N;
    const uint32_t dims[3] = {R.dim[0], R.dim[1], R.dim[2]};
    const uint32_t ncell = dims[0] * dims[1] * dims[2];
    const gb_box box = R.box;
    float4* pos = A.pos + R.first;
    uint32_t* cellidx = A.cellidx + R.first;
    float4* sorted = A.sorted + R.first;

    for (uint32_t c = t; c < ncell; c += T)
        s_cnt[c] = 0u;
    if (t == 0)
        {
        sh.err = 0u;
        sh.maxcnt = 0u;
        sh.maxocc = 0u;
        }
    __syncthreads();
    // bin (hoomd/CellListGPU.cu:42-170, without a slot limit)
    for (uint32_t i = t; i < N; i += T)
        {
        const float4 p = pos[i];
        uint32_t c = 0;
        if (isnan(p.x) || isnan(p.y) || isnan(p.z))
            atomicOr(&sh.err, (uint32_t)GB_REPLICA_NAN);
        else if (!cell_of(box, dims, p.x, p.y, p.z, c))
            atomicOr(&sh.err, (uint32_t)GB_REPLICA_OUTSIDE);
        else
            atomicAdd(&s_cnt[c], 1u);
        cellidx[i] = c;
        }
    __syncthreads();
    if (sh.err)
        return;
    block_scan(s_cnt, s_start, ncell, sh.wtot);
    for (uint32_t c = t; c < ncell; c += T)
        s_cnt[c] = s_start[c];
    __syncthreads();
    for (uint32_t i = t; i < N; i += T)
        {
        const float4 p = pos[i];
        const uint32_t slot = atomicAdd(&s_cnt[cellidx[i]], 1u);
        sorted[slot] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
        }
    __syncthreads();
    // slots of a cell in particle-index order (nlist.Cell(deterministic=True))
    uint32_t occ = 0;
    for (uint32_t c = t; c < ncell; c += T)
        {
        const uint32_t b = s_start[c], e = s_start[c + 1];
        occ = max(occ, e - b);
        for (uint32_t a = b + 1; a < e; a++)
            {
            const float4 v = sorted[a];
            const uint32_t key = __float_as_uint(v.w);
            uint32_t k = a;
            while (k > b && __float_as_uint(sorted[k - 1].w) > key)
                {
                sorted[k] = sorted[k - 1];
                k--;
                }
            sorted[k] = v;
            }
        }
    occ = __reduce_max_sync(0xffffffffu, occ);
    if (t % 32 == 0)
        atomicMax(&sh.maxocc, occ);
    __syncthreads();

    // binned search: lanes walk consecutive cell-ordered slots, so a warp mostly shares a
    // stencil. With S = stencil, the cells within S of the particle's cell hold every neighbour
    // (cell width >= r_list / S); along an axis with fewer than 2S + 1 cells every cell is
    // searched once. The cells of one stencil row are consecutive in x, hence their particles
    // are one or two contiguous runs of the cell-ordered array.
    const float r_list = fadd(R.r_cut, R.r_buff);
    const float rlsq = fmul(r_list, r_list);
    const uint32_t Nmax = R.Nmax;
    const uint32_t stride = R.stride;
    uint4* nl4 = reinterpret_cast<uint4*>(A.nlist + R.nlist_offset);
    const bool ortho = box_is_ortho(box);
    const int S = (int)R.stencil;
    const uint32_t span = 2u * (uint32_t)S + 1u;
    const bool full_x = dims[0] < span, full_y = dims[1] < span, full_z = dims[2] < span;
    const int ny = full_y ? (int)dims[1] : (int)span, nz = full_z ? (int)dims[2] : (int)span;
    // With every axis at least 2S + 2 cells wide and no tilt, the image of a candidate is the
    // image of its cell relative to the particle's (-1, 0, +1 per axis, constant along a run),
    // and x_i - x_j - L*img rounds exactly as minImage's x_i - x_j - L*rint((x_i - x_j)/L) for
    // every pair within r_list; otherwise each candidate goes through min_image.
    const bool shifts = ortho && dims[0] >= span + 1 && dims[1] >= span + 1 && dims[2] >= span + 1;
    uint32_t my_max = 0;
    if (shifts && S == 1 && sh.maxocc <= STREAM_OCC)
        my_max = stream_search(R, A, s_start, s_stream, rlsq);
    else
    for (uint32_t s = t; s < N; s += T)
        {
        const float4 pi = sorted[s];
        const uint32_t i = __float_as_uint(pi.w);
        const uint32_t c = cellidx[i];
        const int cx = c % dims[0], cy = (c / dims[0]) % dims[1], cz = c / (dims[0] * dims[1]);
        uint32_t cnt = 0;
        uint4 buf = make_uint4(0u, 0u, 0u, 0u);
        auto store = [&](uint32_t j) {
            if (cnt < Nmax)
                {
                switch (cnt & 3u)
                    {
                    case 0: buf.x = j; break;
                    case 1: buf.y = j; break;
                    case 2: buf.z = j; break;
                    default:
                        buf.w = j;
                        nl4[(size_t)(cnt >> 2) * stride + i] = buf;
                    }
                }
            cnt++;
        };
        // candidates [s_start[c0], s_start[c1]) shifted by (sx, sy, sz); two per step: packed
        // FP32 differences and squares (each half rounds as the scalar operation) and scalar
        // rounded sums (f2dot3)
        auto run = [&](uint32_t c0, uint32_t c1, float sx, float sy, float sz) {
            const uint32_t e = s_start[c1];
            uint32_t a = s_start[c0];
            if (shifts)
                {
                const uint64_t px = f2pack(pi.x, pi.x), py = f2pack(pi.y, pi.y),
                               pz = f2pack(pi.z, pi.z);
                const uint64_t hx = f2pack(sx, sx), hy = f2pack(sy, sy), hz = f2pack(sz, sz);
                for (; a + 1 < e; a += 2)
                    {
                    const float4 q0 = sorted[a], q1 = sorted[a + 1];
                    const uint64_t dx = f2sub(f2sub(px, f2pack(q0.x, q1.x)), hx);
                    const uint64_t dy = f2sub(f2sub(py, f2pack(q0.y, q1.y)), hy);
                    const uint64_t dz = f2sub(f2sub(pz, f2pack(q0.z, q1.z)), hz);
                    float r0, r1;
                    f2dot3(dx, dy, dz, r0, r1);
                    const uint32_t j0 = __float_as_uint(q0.w), j1 = __float_as_uint(q1.w);
                    if (r0 <= rlsq && j0 != i)
                        store(j0);
                    if (r1 <= rlsq && j1 != i)
                        store(j1);
                    }
                if (a < e)
                    {
                    const float4 q = sorted[a];
                    const uint32_t j = __float_as_uint(q.w);
                    const float dx = fsub(fsub(pi.x, q.x), sx), dy = fsub(fsub(pi.y, q.y), sy),
                                dz = fsub(fsub(pi.z, q.z), sz);
                    if (dot3(dx, dy, dz) <= rlsq && j != i)
                        store(j);
                    }
                }
            else
                for (; a < e; a++)
                    {
                    const float4 q = sorted[a];
                    const uint32_t j = __float_as_uint(q.w);
                    float dx = fsub(pi.x, q.x), dy = fsub(pi.y, q.y), dz = fsub(pi.z, q.z);
                    if (ortho)
                        min_image_ortho(box, dx, dy, dz);
                    else
                        min_image(box, dx, dy, dz);
                    if (dot3(dx, dy, dz) <= rlsq && j != i)
                        store(j);
                    }
        };
        for (int kz = 0; kz < nz; kz++)
            {
            const int zu = cz - S + kz;
            const uint32_t z = full_z ? (uint32_t)kz : wrap_index(zu, (int)dims[2]);
            const float sz = full_z ? 0.0f : fmul(box.L[2], zu < 0 ? -1.0f : (zu >= (int)dims[2] ? 1.0f : 0.0f));
            for (int ky = 0; ky < ny; ky++)
                {
                const int yu = cy - S + ky;
                const uint32_t y = full_y ? (uint32_t)ky : wrap_index(yu, (int)dims[1]);
                const float sy = full_y ? 0.0f : fmul(box.L[1], yu < 0 ? -1.0f : (yu >= (int)dims[1] ? 1.0f : 0.0f));
                const uint32_t row = (z * dims[1] + y) * dims[0];
                if (full_x)
                    run(row, row + dims[0], 0.0f, sy, sz);
                else
                    {
                    const int x0 = cx - S, x1 = cx + S;
                    const float L0 = box.L[0];
                    if (x0 < 0)
                        {
                        run(row + (uint32_t)(x0 + (int)dims[0]), row + dims[0], -L0, sy, sz);
                        run(row, row + (uint32_t)(x1 + 1), 0.0f, sy, sz);
                        }
                    else if (x1 >= (int)dims[0])
                        {
                        run(row + (uint32_t)x0, row + dims[0], 0.0f, sy, sz);
                        run(row, row + (uint32_t)(x1 + 1 - (int)dims[0]), L0, sy, sz);
                        }
                    else
                        run(row + (uint32_t)x0, row + (uint32_t)(x1 + 1), 0.0f, sy, sz);
                    }
                }
            }
        const uint32_t stored = min(cnt, Nmax);
        if (stored & 3u)
            nl4[(size_t)(stored >> 2) * stride + i] = buf;
        A.n_neigh[R.first + i] = stored;
        A.last_pos[R.first + i] = make_float4(pi.x, pi.y, pi.z, 0.0f);
        my_max = max(my_max, cnt);
        }
    my_max = __reduce_max_sync(0xffffffffu, my_max);
    if (threadIdx.x % 32 == 0)
        atomicMax(&sh.maxcnt, my_max);
    __syncthreads();
    if (t == 0)
        {
        if (sh.maxcnt > Nmax)
            {
            sh.err |= GB_REPLICA_OVERFLOW;
            sh.rep.needed = sh.maxcnt;
            }
        else
            sh.rep.n_builds += 1;
        }
    __syncthreads();
    }

// Pair forces on every particle; with `step_two` also the second half step. Writes the chunk
// sums of m v^2 and energy; ends synced, with (K, U) in warp 0 lane 0's return value.
// ORTHO (no tilt) is a template parameter so that its loop holds no tilt terms in registers.
template<int MAXT, bool ORTHO>
__device__ __noinline__ double2 pair_forces(const RepShared& sh, const RepArrays& A, bool step_two)
    {
    const gb_replica& R = sh.rep;
    const uint32_t T = blockDim.x;
    const uint32_t lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    const uint32_t N = R.N;
    const float4* pos = A.pos + R.first;
    float4* vel = A.vel + R.first;
    const uint4* nl4 = reinterpret_cast<const uint4*>(A.nlist + R.nlist_offset);
    const uint32_t* n_neigh = A.n_neigh + R.first;
    double2* chunk = A.chunk + R.first / 32;
    const uint64_t stride = R.stride;
    const float rcutsq = fmul(R.r_cut, R.r_cut);
    const bool shift = R.shift_mode == 1u;
    const gb_lj_param lj = R.lj;
    const float Lx = R.box.L[0], Ly = R.box.L[1], Lz = R.box.L[2];
    const float Lix = R.box.Linv[0], Liy = R.box.Linv[1], Liz = R.box.Linv[2];
    const float Lzxz = ORTHO ? 0.0f : R.box.L[2] * R.box.xz,
                Lzyz = ORTHO ? 0.0f : R.box.L[2] * R.box.yz,
                Lyxy = ORTHO ? 0.0f : R.box.L[1] * R.box.xy;
    const float dt = (float)R.dt;
    const float hdt = __fmul_rn(0.5f, dt);

    for (uint32_t base = warp * 32; base < N; base += T)
        {
        const uint32_t i = base + lane;
        double ke = 0.0, pe_d = 0.0;
        if (i < N)
            {
            const float4 pi = pos[i];
            float fx = 0.f, fy = 0.f, fz = 0.f, pe = 0.f;
            auto pair = [&](const float4 pj, bool valid) {
                float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                if (ORTHO)
                    {
                    // shift particle i by its image first, then subtract: when the box is much
                    // wider than r_list, (x_i - k L) and x_j are within a factor of two and their
                    // difference is exact in FP32, whereas x_i - x_j across the boundary loses
                    // the low bits of |x| ~ L/2
                    const float kx = rintf(dx * Lix), ky = rintf(dy * Liy), kz = rintf(dz * Liz);
                    dx = fmaf(-kx, Lx, pi.x) - pj.x;
                    dy = fmaf(-ky, Ly, pi.y) - pj.y;
                    dz = fmaf(-kz, Lz, pi.z) - pj.z;
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
                float force_divr = 0.0f, pair_eng = 0.0f;
                EvalLJ eval(rsq, rcutsq, lj, nullptr);
                eval.evalForceAndEnergy(force_divr, pair_eng, shift);
                if (!valid)
                    {
                    force_divr = 0.0f;
                    pair_eng = 0.0f;
                    }
                fx += dx * force_divr;
                fy += dy * force_divr;
                fz += dz * force_divr;
                pe += pair_eng;
            };
            const uint32_t nn = n_neigh[i];
            const uint32_t nfull = nn >> 2, rem = nn & 3u;
            const uint4* p4 = nl4 + i;
            // index loads run two groups ahead of the position gathers
            const uint4 self = make_uint4(i, i, i, i);
            uint4 jA = self, jB = self;
            if (nfull > 0)
                jA = __ldcs(p4);
            if (nfull > 1)
                jB = __ldcs(p4 + stride);
            for (uint32_t b = 0; b < nfull; b++)
                {
                const uint4 jc = jA;
                jA = jB;
                if (b + 2 < nfull)
                    jB = __ldcs(p4 + (uint64_t)(b + 2) * stride);
                const float4 q0 = pos[jc.x];
                const float4 q1 = pos[jc.y];
                const float4 q2 = pos[jc.z];
                const float4 q3 = pos[jc.w];
                pair(q0, true);
                pair(q1, true);
                pair(q2, true);
                pair(q3, true);
                }
            if (rem)
                {
                const uint4 jc = __ldcs(p4 + (uint64_t)nfull * stride);
                const float4 q0 = pos[jc.x];
                const float4 q1 = pos[rem > 1 ? jc.y : i];
                const float4 q2 = pos[rem > 2 ? jc.z : i];
                pair(q0, true);
                pair(q1, rem > 1);
                pair(q2, rem > 2);
                }
            pe *= 0.5f;
            A.force[R.first + i] = make_float4(fx, fy, fz, pe);
            float4 v = vel[i];
            const float minv = __frcp_rn(v.w);
            const float ax = __fmul_rn(fx, minv), ay = __fmul_rn(fy, minv),
                        az = __fmul_rn(fz, minv);
            if (step_two)
                {
                v.x = __fadd_rn(v.x, __fmul_rn(hdt, ax));
                v.y = __fadd_rn(v.y, __fmul_rn(hdt, ay));
                v.z = __fadd_rn(v.z, __fmul_rn(hdt, az));
                vel[i] = v;
                }
            A.accel[R.first + i] = make_float4(ax, ay, az, 0.0f);
            ke = (double)v.w
                 * ((double)v.x * (double)v.x + (double)v.y * (double)v.y
                    + (double)v.z * (double)v.z);
            pe_d = (double)pe;
            }
        ke = warp_sum(ke);
        pe_d = warp_sum(pe_d);
        if (lane == 0)
            chunk[base / 32] = make_double2(ke, pe_d);
        }
    __syncthreads();
    double2 tot = make_double2(0.0, 0.0);
    if (warp == 0)
        {
        const uint32_t nchunk = (N + 31) / 32;
        double a = 0.0, b = 0.0;
        for (uint32_t c = lane; c < nchunk; c += 32)
            {
            const double2 v = chunk[c];
            a += v.x;
            b += v.y;
            }
        tot.x = warp_sum(a);
        tot.y = warp_sum(b);
        }
    return tot;
    }

// Bussi draws for timesteps [from, from + blockDim.x), capped at the replica's target.
template<int MAXT>
__device__ __noinline__ void draw_window(RepShared& sh, double2* s_draws, uint64_t from)
    {
    const gb_replica& R = sh.rep;
    const uint64_t ts = from + threadIdx.x;
    if (ts <= R.target)
        s_draws[threadIdx.x] = bussi_draws_d(R.dof, ts, (uint16_t)R.seed, 0u);
    __syncthreads();
    if (threadIdx.x == 0)
        {
        sh.wbase = from;
        sh.wcount = blockDim.x;
        }
    __syncthreads();
    }

// Totals after a force evaluation: energies, Bussi factor of the step that starts at `next`.
template<int MAXT>
__device__ __noinline__ void finish_step(RepShared& sh, const double2* s_draws, double2 tot, uint64_t next,
                            bool from_window)
    {
    if (threadIdx.x != 0)
        return;
    gb_replica& R = sh.rep;
    const double K = 0.5 * tot.x;
    R.ke = K;
    R.pe = tot.y;
    if (!R.bussi)
        {
        R.factor = 1.0;
        return;
        }
    if (K <= 0.0)
        {
        R.status |= GB_REPLICA_ZERO_KE;
        R.factor = 1.0;
        return;
        }
    if (from_window)
        R.factor = bussi_factor_from_draws(K, R.dof, R.dt, R.tau, R.kT,
                                           s_draws[next - sh.wbase]);
    else
        R.factor = bussi_factor_d(K, R.dof, R.dt, R.tau, R.kT, next, (uint16_t)R.seed, 0u);
    }

template<int MAXT>
__device__ void run_replica(RepShared& sh, const RepArrays& A, double2* s_draws,
                            uint32_t* s_start, uint32_t* s_cnt, unsigned char* s_stream)
    {
    gb_replica& R = sh.rep;
    const uint32_t T = blockDim.x, t = threadIdx.x;
    if (t == 0)
        {
        sh.wbase = 0;
        sh.wcount = 0;
        sh.rebuild = 0;
        for (int k = 0; k < 4; k++)
            sh.clk[k] = 0;
        sh.t0 = clock64();
        }
    __syncthreads();
    if (R.status)
        return;
    if (!R.prepared)
        {
        // IntegratorTwoStep::prepRun: lists, forces and a = F/m at the current step, thermo,
        // and the factor of the first step (hoomd/md/IntegratorTwoStep.cc:226-298)
        build_lists<MAXT>(sh, A, s_start, s_cnt, s_stream);
        stamp(sh, 1);
        if (sh.err)
            {
            if (t == 0)
                R.status |= sh.err;
            __syncthreads();
            return;
            }
        const double2 tot = box_is_ortho(R.box) ? pair_forces<MAXT, true>(sh, A, false)
                                                : pair_forces<MAXT, false>(sh, A, false);
        finish_step<MAXT>(sh, s_draws, tot, R.timestep, false);
        if (t == 0)
            R.prepared = 1u;
        __syncthreads();
        stamp(sh, 2);
        }
    const float dt = (float)R.dt;
    const gb_box box = R.box;
    const float rmax = fadd(R.r_cut, R.r_buff);
    const float delta_max = fmul(fsub(rmax, R.r_cut), 0.5f);
    const float maxsq = (delta_max > 0.0f) ? fmul(delta_max, delta_max) : 0.0f;
    float4* pos = A.pos + R.first;
    float4* vel = A.vel + R.first;
    const float4* accel = A.accel + R.first;
    int4* image = A.image + R.first;
    const float4* last_pos = A.last_pos + R.first;

    while (R.status == 0u && (R.pending_build || R.timestep < R.target))
        {
        const uint64_t ts = R.timestep;
        const bool window = R.bussi && R.target > ts;
        if (window && (ts + 1 < sh.wbase || ts + 1 >= sh.wbase + sh.wcount))
            {
            draw_window<MAXT>(sh, s_draws, ts + 1);
            stamp(sh, 3);
            }
        if (!R.pending_build)
            {
            const float s = (float)R.factor;
            bool moved = false;
            for (uint32_t j = t; j < R.N; j += T)
                {
                float4 v = vel[j];
                float4 p = pos[j];
                const float4 a = accel[j];
                // v = v + (1/2) a dt ; v *= s ; x += dt v   (TwoStepConstantVolume.cc:37-55)
                v.x = fadd(v.x, fmul(fmul(0.5f, a.x), dt));
                v.y = fadd(v.y, fmul(fmul(0.5f, a.y), dt));
                v.z = fadd(v.z, fmul(fmul(0.5f, a.z), dt));
                v.x = fmul(v.x, s);
                v.y = fmul(v.y, s);
                v.z = fmul(v.z, s);
                p.x = fadd(p.x, fmul(dt, v.x));
                p.y = fadd(p.y, fmul(dt, v.y));
                p.z = fadd(p.z, fmul(dt, v.z));
                int ix = 0, iy = 0, iz = 0;
                wrap(box, p.x, p.y, p.z, ix, iy, iz);
                if (ix | iy | iz)
                    {
                    int4 im = image[j];
                    im.x += ix;
                    im.y += iy;
                    im.z += iz;
                    image[j] = im;
                    }
                vel[j] = v;
                pos[j] = p;
                // hoomd/md/NeighborListGPU.cu:42-83 with lambda = 1 (fixed box)
                const float4 lp = last_pos[j];
                float dx = fsub(p.x, lp.x), dy = fsub(p.y, lp.y), dz = fsub(p.z, lp.z);
                min_image(box, dx, dy, dz);
                moved = moved || dot3(dx, dy, dz) >= maxsq;
                }
            if (__any_sync(0xffffffffu, moved) && t % 32 == 0)
                sh.rebuild = 1u;
            __syncthreads();
            if (t == 0)
                R.pending_build = sh.rebuild;
            __syncthreads();
            stamp(sh, 0);
            }
        if (R.pending_build)
            {
            build_lists<MAXT>(sh, A, s_start, s_cnt, s_stream);
            stamp(sh, 1);
            if (sh.err)
                {
                if (t == 0)
                    R.status |= sh.err;
                __syncthreads();
                break;
                }
            }
        const double2 tot = box_is_ortho(R.box) ? pair_forces<MAXT, true>(sh, A, true)
                                                : pair_forces<MAXT, false>(sh, A, true);
        finish_step<MAXT>(sh, s_draws, tot, ts + 1, window);
        if (t == 0)
            {
            R.timestep = ts + 1;
            R.pending_build = 0u;
            sh.rebuild = 0u;
            }
        __syncthreads();
        stamp(sh, 2);
        }
    }

// MAXT bounds the block size and thereby the registers per thread: 1024 -> 64, 768 -> 80,
// 512 -> 128; the launch picks the smallest MAXT >= block_size.
template<int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
    k_replicas(gb_replica* reps, uint32_t n_rep, const uint32_t* order, uint32_t* queue,
               RepArrays A, uint32_t max_cells)
    {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ RepShared sh;
    __shared__ uint32_t s_r;
    double2* s_draws = reinterpret_cast<double2*>(smem);
    uint32_t* s_start = reinterpret_cast<uint32_t*>(s_draws + blockDim.x);
    uint32_t* s_cnt = s_start + max_cells + 1;
    unsigned char* s_stream = smem + smem_cells_bytes(max_cells, blockDim.x);
    constexpr uint32_t WORDS = sizeof(gb_replica) / 4;
    for (;;)
        {
        if (threadIdx.x == 0)
            {
            const uint32_t q = atomicAdd(&queue[0], 1u);
            s_r = q < n_rep ? order[q] : NO_REPLICA;
            }
        __syncthreads();
        const uint32_t r = s_r;
        if (r == NO_REPLICA || r >= n_rep)
            break;
        uint32_t* dst = reinterpret_cast<uint32_t*>(&sh.rep);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(reps + r);
        for (uint32_t w = threadIdx.x; w < WORDS; w += blockDim.x)
            dst[w] = src[w];
        __syncthreads();
        const bool idle = sh.rep.status == 0u && sh.rep.prepared && !sh.rep.pending_build
                          && sh.rep.timestep >= sh.rep.target;
        if (!idle)
            {
            // cell grid larger than the launch's shared memory: refuse rather than overrun
            if (sh.rep.dim[0] * sh.rep.dim[1] * sh.rep.dim[2] > max_cells)
                {
                if (threadIdx.x == 0)
                    sh.rep.status |= GB_REPLICA_CONFIG;
                __syncthreads();
                }
            else
                {
                run_replica<MAXT>(sh, A, s_draws, s_start, s_cnt, s_stream);
                if (A.clocks && threadIdx.x == 0)
                    for (int k = 0; k < 4; k++)
                        A.clocks[4 * (size_t)r + k] += (uint64_t)sh.clk[k];
                }
            __syncthreads();
            uint32_t* out = reinterpret_cast<uint32_t*>(reps + r);
            for (uint32_t w = threadIdx.x; w < WORDS; w += blockDim.x)
                out[w] = dst[w];
            }
        __syncthreads();
        }
    if (threadIdx.x == 0)
        {
        __threadfence();
        if (atomicAdd(&queue[1], 1u) == gridDim.x - 1)
            {
            queue[0] = 0u;
            queue[1] = 0u;
            }
        }
    }

using ReplicaKernel = void (*)(gb_replica*, uint32_t, const uint32_t*, uint32_t*, RepArrays,
                               uint32_t);

ReplicaKernel kernel_for(uint32_t block)
    {
    if (block <= 512)
        return k_replicas<512>;
    if (block <= 768)
        return k_replicas<768>;
    return k_replicas<1024>;
    }

int launch_shape(uint32_t max_cells, uint32_t block, size_t& smem)
    {
    smem = smem_bytes(max_cells, block);
    if (block < 64 || block > GB_REPLICA_MAX_BLOCK || block % 32 != 0)
        return 0;
    if (smem + sizeof(RepShared) + 64 > 227 * 1024)
        return 0;
    const ReplicaKernel k = kernel_for(block);
    if (smem > 48 * 1024
        && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
               != cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, (int)block, smem) != cudaSuccess)
        return 0;
    return n;
    }
} // namespace
} // namespace gb

using namespace gb;

extern "C"
    {
    size_t gb_replica_scratch_bytes(uint64_t n_slots)
        {
        return scratch_cellidx(n_slots) + scratch_sorted(n_slots) + scratch_chunk(n_slots);
        }

    size_t gb_replica_smem_bytes(uint32_t max_cells, uint32_t block_size)
        {
        const size_t s = smem_bytes(max_cells, block_size);
        return (s + sizeof(RepShared) + 64 > 227 * 1024) ? 0 : s;
        }

    int gb_replica_ctas_per_sm(uint32_t max_cells, uint32_t block_size)
        {
        size_t smem = 0;
        return launch_shape(max_cells, block_size, smem);
        }

    int gb_replicas_run(const gb_replica_batch* b, void* stream)
        {
        GB_REQUIRE(b, "gb_replicas_run: null argument");
        if (b->n_replicas == 0)
            return GB_OK;
        GB_REQUIRE(b->d_replicas && b->d_order && b->d_queue && b->d_pos && b->d_vel
                       && b->d_accel && b->d_image && b->d_force && b->d_last_pos
                       && b->d_n_neigh && b->d_nlist && b->d_scratch,
                   "gb_replicas_run: null device pointer");
        GB_REQUIRE(b->max_cells > 0, "gb_replicas_run: max_cells must be positive");
        size_t smem = 0;
        const int per_sm = launch_shape(b->max_cells, b->block_size, smem);
        if (per_sm <= 0)
            return fail(GB_ERR_UNSUPPORTED,
                        "gb_replicas_run: block_size / max_cells cannot launch");
        uint32_t grid = b->grid_size ? b->grid_size : (uint32_t)(per_sm * num_sms());
        RepArrays A;
        A.pos = reinterpret_cast<float4*>(b->d_pos);
        A.vel = reinterpret_cast<float4*>(b->d_vel);
        A.accel = reinterpret_cast<float4*>(b->d_accel);
        A.image = reinterpret_cast<int4*>(b->d_image);
        A.force = reinterpret_cast<float4*>(b->d_force);
        A.last_pos = reinterpret_cast<float4*>(b->d_last_pos);
        A.n_neigh = b->d_n_neigh;
        A.nlist = b->d_nlist;
        unsigned char* sc = static_cast<unsigned char*>(b->d_scratch);
        A.cellidx = reinterpret_cast<uint32_t*>(sc);
        A.sorted = reinterpret_cast<float4*>(sc + scratch_cellidx(b->n_slots));
        A.chunk = reinterpret_cast<double2*>(sc + scratch_cellidx(b->n_slots)
                                             + scratch_sorted(b->n_slots));
        A.clocks = b->d_phase_clocks;
        kernel_for(b->block_size)<<<grid, b->block_size, smem, (cudaStream_t)stream>>>(
            b->d_replicas, b->n_replicas, b->d_order, b->d_queue, A, b->max_cells);
        return check_launch("gb_replicas_run");
        }
    }
