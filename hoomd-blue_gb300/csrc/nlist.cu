// Cell list and binned neighbour list on GB300.
//
// Cell list (replaces gpu_compute_cell_list, hoomd/CellListGPU.cu:42-170): one thread per
// particle bins it with the reference's makeFraction arithmetic and claims a slot with an atomic.
// Optional deterministic mode sorts each cell's slots by particle index afterwards
// (hoomd/CellListGPU.cu:478-540 does the same with a global thrust sort).
//
// Neighbour list (replaces gpu_compute_nlist_binned, hoomd/md/NeighborListGPUBinned.cu:52-298):
// one warp per cell in every form. The default (k_nlist_stream) puts 32 candidates of the
// cell's stencil in the lanes and tests them against one own particle at a time, a ballot per own
// particle; the other forms put the own particles in the lanes. In the first of those, for each
// of the 27 (or fewer, deduplicated) adjacent cells the warp stages 32 candidates at a time in
// shared memory with one coalesced load, then every lane tests its particle against every staged
// candidate. All lanes walk the same candidate sequence, so there is no divergence in the search
// (the reference's thread-per-particle search diverges whenever a warp straddles cells). Hits are
// written in the column-major layout nlist[k * stride + i] (coalesced across particles in SFC
// order), the same interleaved by four, or the reference's flat head-list layout.
#include <cstdint>
#include <type_traits>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
constexpr int NL_WARPS = 4; // warps per block in the build kernel

// dangerous-build accounting of a delayed rebuild check (gb_cell_list_args)
struct BuildRecord
    {
    uint64_t* dangerous;
    uint32_t delay;
    int dist_check;
    };

// build statistics of one (non-gated-off) build; one thread
__device__ void record_build(uint64_t* count, const uint64_t* timestep, uint64_t* build_steps,
                             const BuildRecord& rec)
    {
    if (count)
        *count += 1;
    if (timestep && build_steps)
        {
        // NeighborList::needsUpdating (hoomd/md/NeighborList.cc:1349-1356, 1388-1414) for the
        // step whose forces follow
        const uint64_t T = *timestep + 1, last = build_steps[0];
        if (last != ~0ull && T > last)
            build_steps[1] = min(build_steps[1], min(T - last, (uint64_t)99));
        if (rec.dangerous && rec.dist_check && rec.delay > 1 && last != ~0ull
            && T == last + rec.delay)
            *rec.dangerous += 1;
        build_steps[0] = T;
        }
    }

__global__ void k_zero_u32(unsigned int* p, size_t n, const uint32_t* gate, uint64_t* count,
                           const uint64_t* timestep, uint64_t* build_steps, BuildRecord rec)
    {
    if (gate && *gate == 0)
        return;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        record_build(count, timestep, build_steps, rec);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = 0;
    }

// stats: the build statistics are kept here (the counts were zeroed by the caller's step)
__global__ void k_cell_bin(const float4* __restrict__ pos, unsigned int N, gb_box box, uint3 dim,
                           unsigned int Nmax, unsigned int* cell_size, float4* xyzf,
                           unsigned int* cell_type, unsigned int* cond, const uint32_t* gate,
                           bool stats, uint64_t* count, const uint64_t* timestep,
                           uint64_t* build_steps, BuildRecord rec)
    {
    if (gate && *gate == 0)
        return;
    if (stats && blockIdx.x == 0 && threadIdx.x == 0)
        record_build(count, timestep, build_steps, rec);
    const unsigned int dims[3] = {dim.x, dim.y, dim.z};
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        {
        float4 p = pos[i];
        if (isnan(p.x) || isnan(p.y) || isnan(p.z))
            {
            atomicMax(&cond[1], i + 1);
            continue;
            }
        unsigned int bin;
        if (!cell_of(box, dims, p.x, p.y, p.z, bin))
            {
            atomicMax(&cond[2], i + 1);
            continue;
            }
        unsigned int slot = atomicAdd(&cell_size[bin], 1u);
        if (slot < Nmax)
            {
            size_t s = (size_t)bin * Nmax + slot;
            xyzf[s] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
            if (cell_type)
                cell_type[s] = __float_as_uint(p.w);
            }
        else
            atomicMax(&cond[0], slot + 1);
        }
    }

// Deterministic slot order: one warp per cell ranks each slot by particle index and scatters.
__global__ void k_cell_sort(const unsigned int* cell_size, float4* xyzf, unsigned int* cell_type,
                            unsigned int ncell, unsigned int Nmax, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int wpb = blockDim.x / 32;
    float4* s_x = reinterpret_cast<float4*>(smem_raw) + (size_t)warp * Nmax;
    unsigned int* s_t = reinterpret_cast<unsigned int*>(reinterpret_cast<float4*>(smem_raw)
                                                        + (size_t)wpb * Nmax)
                        + (size_t)warp * Nmax;
    for (unsigned int cell = blockIdx.x * wpb + warp; cell < ncell; cell += gridDim.x * wpb)
        {
        unsigned int n = min(cell_size[cell], Nmax);
        size_t base = (size_t)cell * Nmax;
        for (unsigned int a = lane; a < n; a += 32)
            {
            s_x[a] = xyzf[base + a];
            if (cell_type)
                s_t[a] = cell_type[base + a];
            }
        __syncwarp();
        for (unsigned int a = lane; a < n; a += 32)
            {
            unsigned int ia = __float_as_uint(s_x[a].w);
            unsigned int rank = 0;
            for (unsigned int b = 0; b < n; b++)
                rank += (__float_as_uint(s_x[b].w) < ia);
            xyzf[base + rank] = s_x[a];
            if (cell_type)
                cell_type[base + rank] = s_t[a];
            }
        __syncwarp();
        }
    }

__global__ void k_cell_adj(uint3 dim, unsigned int ndim, unsigned int width, unsigned int* adj)
    {
    unsigned int ncell = dim.x * dim.y * dim.z;
    for (unsigned int cur = blockIdx.x * blockDim.x + threadIdx.x; cur < ncell;
         cur += gridDim.x * blockDim.x)
        {
        int i = cur % dim.x, j = (cur / dim.x) % dim.y, k = cur / (dim.x * dim.y);
        unsigned int a[27];
        int n = 0;
        int rk = (ndim == 2) ? 0 : 1;
        int mx = dim.x, my = dim.y, mz = dim.z;
        for (int nk = k - rk; nk <= k + rk; nk++)
            for (int nj = j - 1; nj <= j + 1; nj++)
                for (int ni = i - 1; ni <= i + 1; ni++)
                    {
                    int wi = ((ni % mx) + mx) % mx;
                    int wj = ((nj % my) + my) % my;
                    int wk = ((nk % mz) + mz) % mz;
                    a[n++] = (unsigned int)((wk * my + wj) * mx + wi);
                    }
        // insertion sort + unique (hoomd/CellList.cc:390-397)
        for (int x = 1; x < n; x++)
            {
            unsigned int v = a[x];
            int y = x - 1;
            while (y >= 0 && a[y] > v)
                {
                a[y + 1] = a[y];
                y--;
                }
            a[y + 1] = v;
            }
        int u = 0;
        for (int x = 0; x < n; x++)
            if (x == 0 || a[x] != a[x - 1])
                a[u++] = a[x];
        for (int x = 0; x < (int)width && x < u; x++)
            adj[(size_t)cur * width + x] = a[x];
        }
    }

// The build: see the file comment. Template parameters:
//  MULTI  per-pair r_cut / r_list tables (ntypes > 1)
//  LAYOUT 0 = reference flat head-list layout, 1 = column-major, 4 = column-major interleaved by 4
//  MI     minimum-image method: 0 = BoxDim::minImage (rint) general, 1 = rint orthorhombic,
//         2 = exact image shift of the adjacent cell (every dimension has >= 4 cells and is
//         periodic). In case 2 each candidate cell appears once in the 27-cell stencil, so a
//         candidate within r_list of particle i is the minimum image and the rint image equals the
//         cell's image; subtracting the cell's L*img terms in minImage's order (z, then y, then x)
//         reproduces minImage's roundings exactly for every pair that can be in the list, so the
//         dr^2 <= r_list^2 decisions are unchanged while three multiplies and three rints per
//         candidate disappear.
template<bool MULTI, int LAYOUT, int MI>
__global__ void __launch_bounds__(NL_WARPS * 32)
    k_nlist_binned(unsigned int* __restrict__ nlist, unsigned int* __restrict__ n_neigh,
                   float4* __restrict__ last_pos, unsigned int* __restrict__ cond,
                   const uint64_t* __restrict__ head_list, uint64_t stride,
                   const unsigned int* __restrict__ Nmax_t,
                   const unsigned int* __restrict__ cell_size, const float4* __restrict__ xyzf,
                   const unsigned int* __restrict__ cell_type,
                   const unsigned int* __restrict__ cell_adj, uint3 dim, unsigned int ncell,
                   unsigned int Nmax_cell, unsigned int adj_w, gb_box box,
                   const float* __restrict__ r_cut, const float* __restrict__ r_listsq,
                   unsigned int ntypes, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    __shared__ float4 s_cand[NL_WARPS][32];
    __shared__ unsigned int s_ctype[NL_WARPS][32];
    // [2 * ntypes^2] r_cut then r_listsq (MULTI only), stored transposed: entry (a, b) at
    // b * ntypes + a, so the lanes of a warp (own particles of any type) testing one candidate
    // read consecutive words, free of bank conflicts
    extern __shared__ float s_tab[];
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x)
            {
            const unsigned int tt = (t % ntypes) * ntypes + t / ntypes;
            s_tab[tt] = r_cut[t];
            s_tab[ntypes * ntypes + tt] = r_listsq[t];
            }
        __syncthreads();
        }
    const float rc0 = MULTI ? 0.0f : r_cut[0];
    const float rl0 = MULTI ? 0.0f : r_listsq[0];
    const unsigned int Nmax0 = MULTI ? 0u : Nmax_t[0];

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const unsigned int cell = blockIdx.x * NL_WARPS + warp;
    if (cell >= ncell)
        return;
    const int ci = cell % dim.x, cj = (cell / dim.x) % dim.y, ck = cell / (dim.x * dim.y);
    const unsigned int csize = min(cell_size[cell], Nmax_cell);
    for (unsigned int base = 0; base < csize; base += 32)
        {
        const unsigned int own = base + lane;
        const bool active = own < csize;
        float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
        unsigned int i = 0, ti = 0;
        if (active)
            {
            pi = xyzf[(size_t)cell * Nmax_cell + own];
            i = __float_as_uint(pi.w);
            if (MULTI)
                ti = cell_type[(size_t)cell * Nmax_cell + own];
            }
        const unsigned int Nmax_i = MULTI ? (active ? Nmax_t[ti] : 0u) : Nmax0;
        const uint64_t head = (LAYOUT == 0) ? (active ? head_list[i] : 0ull) : (uint64_t)i;
        unsigned int cnt = 0;
        auto store = [&](unsigned int j) {
            if (cnt < Nmax_i)
                {
                if (LAYOUT == 0)
                    nlist[head + cnt] = j;
                else if (LAYOUT == 1)
                    nlist[head + (uint64_t)cnt * stride] = j;
                else
                    nlist[((uint64_t)(cnt >> 2) * stride + i) * 4 + (cnt & 3)] = j;
                }
            cnt++;
        };
        for (unsigned int a = 0; a < adj_w; a++)
            {
            const unsigned int nc = __ldg(cell_adj + (size_t)cell * adj_w + a);
            const unsigned int nsz = min(__ldg(cell_size + nc), Nmax_cell);
            // image of the adjacent cell relative to this one (MI == 2)
            float sz = 0.f, syz = 0.f, sxz = 0.f, sy = 0.f, sxy = 0.f, sx = 0.f;
            if (MI == 2)
                {
                const int ni = nc % dim.x, nj = (nc / dim.x) % dim.y, nk = nc / (dim.x * dim.y);
                const int dx_c = ni - ci, dy_c = nj - cj, dz_c = nk - ck;
                const float ix = dx_c == (int)dim.x - 1 ? -1.f : (dx_c == 1 - (int)dim.x ? 1.f : 0.f);
                const float iy = dy_c == (int)dim.y - 1 ? -1.f : (dy_c == 1 - (int)dim.y ? 1.f : 0.f);
                const float iz = dz_c == (int)dim.z - 1 ? -1.f : (dz_c == 1 - (int)dim.z ? 1.f : 0.f);
                sz = fmul(box.L[2], iz);
                syz = fmul(fmul(box.L[2], box.yz), iz);
                sxz = fmul(fmul(box.L[2], box.xz), iz);
                sy = fmul(box.L[1], iy);
                sxy = fmul(fmul(box.L[1], box.xy), iy);
                sx = fmul(box.L[0], ix);
                }
            for (unsigned int cb = 0; cb < nsz; cb += 32)
                {
                if (cb + lane < nsz)
                    {
                    s_cand[warp][lane] = __ldg(xyzf + (size_t)nc * Nmax_cell + cb + lane);
                    if (MULTI)
                        s_ctype[warp][lane] = __ldg(cell_type + (size_t)nc * Nmax_cell + cb + lane);
                    }
                __syncwarp();
                const unsigned int m = min(32u, nsz - cb);
                if (active)
                    {
#pragma unroll 2
                    for (unsigned int t = 0; t < m; t++)
                        {
                        const float4 c = s_cand[warp][t];
                        const unsigned int j = __float_as_uint(c.w);
                        float dx = fsub(pi.x, c.x), dy = fsub(pi.y, c.y), dz = fsub(pi.z, c.z);
                        if (MI == 2)
                            {
                            dz = fsub(dz, sz);
                            dy = fsub(dy, syz);
                            dx = fsub(dx, sxz);
                            dy = fsub(dy, sy);
                            dx = fsub(dx, sxy);
                            dx = fsub(dx, sx);
                            }
                        else if (MI == 1)
                            min_image_ortho(box, dx, dy, dz);
                        else
                            min_image(box, dx, dy, dz);
                        const float rsq = dot3(dx, dy, dz);
                        float rc, rl;
                        if (MULTI)
                            {
                            const unsigned int tp = s_ctype[warp][t] * ntypes + ti;
                            rc = s_tab[tp];
                            rl = s_tab[ntypes * ntypes + tp];
                            }
                        else
                            {
                            rc = rc0;
                            rl = rl0;
                            }
                        if (rsq <= rl && j != i && rc > 0.0f)
                            store(j);
                        }
                    }
                __syncwarp();
                }
            }
        if (active)
            {
            // stored count is clipped to the capacity so that a consumer launched before the
            // host sees the overflow never reads past the list; cond holds the count needed
            n_neigh[i] = min(cnt, Nmax_i);
            if (cnt > Nmax_i)
                atomicMax(&cond[ti], cnt);
            if (last_pos)
                last_pos[i] = make_float4(pi.x, pi.y, pi.z, 0.0f);
            }
        }
    }

// Tiled build for the common case (every dimension >= 4 cells and periodic, column-major list):
// one warp per cell. For each z-plane of the 3x3x3 stencil the warp stages the nine adjacent
// cells' particles in shared memory together with each cell's exact image shift (the MI == 2
// argument above), then every lane takes one staged candidate and the warp walks the cell's own
// particles. For own particle o, the lanes whose candidate is within r_list form a ballot; each
// writes its candidate at position count(o) + rank, and count(o) (held by lane o) advances by the
// ballot's population. All 32 lanes test a distinct pair in every iteration, the store path is
// one predicated store per lane, and neighbours appear in a fixed order (stencil plane, cell,
// slot), so the list is as deterministic as the cell list it is built from.
constexpr int TILE_WARPS_MAX = 4;

__device__ __forceinline__ unsigned int wrap_cell(int c, int n)
    {
    return (unsigned int)(c < 0 ? c + n : (c >= n ? c - n : c));
    }

template<bool MULTI, int LAYOUT, bool ORTHO>
__global__ void __launch_bounds__(TILE_WARPS_MAX * 32)
    k_nlist_tile(unsigned int* __restrict__ nlist, unsigned int* __restrict__ n_neigh,
                 float4* __restrict__ last_pos, unsigned int* __restrict__ cond, uint64_t stride,
                 const unsigned int* __restrict__ Nmax_t,
                 const unsigned int* __restrict__ cell_size, const float4* __restrict__ xyzf,
                 const unsigned int* __restrict__ cell_type, uint3 dim, unsigned int ncell,
                 unsigned int Nmax_cell, gb_box box, const float* __restrict__ r_cut,
                 const float* __restrict__ r_listsq, unsigned int ntypes, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x / 32;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    // block-wide: type tables (MULTI)
    float* s_tab = reinterpret_cast<float*>(smem);
    const size_t tab_bytes = MULTI ? ((2 * sizeof(float) * ntypes * ntypes + 15) / 16) * 16 : 0;
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x)
            {
            s_tab[t] = r_cut[t];
            s_tab[ntypes * ntypes + t] = r_listsq[t];
            }
        __syncthreads();
        }
    // per-warp region
    const size_t per_warp = (size_t)Nmax_cell * (16 + 16 * 9 + 4 * 9 + 4) + 9 * 6 * 4;
    unsigned char* base = smem + tab_bytes + (size_t)warp * ((per_warp + 15) / 16 * 16);
    float4* s_own = reinterpret_cast<float4*>(base);
    float4* s_cand = s_own + Nmax_cell;
    unsigned int* s_meta = reinterpret_cast<unsigned int*>(s_cand + 9 * Nmax_cell);
    unsigned int* s_otype = s_meta + 9 * Nmax_cell;
    float* s_shift = reinterpret_cast<float*>(s_otype + Nmax_cell);

    const unsigned int cell = blockIdx.x * wpb + warp;
    if (cell >= ncell)
        return;
    const int ci = cell % dim.x, cj = (cell / dim.x) % dim.y, ck = cell / (dim.x * dim.y);
    const unsigned int csize = min(cell_size[cell], Nmax_cell);
    if (csize == 0)
        return;
    for (unsigned int a = lane; a < csize; a += 32)
        {
        s_own[a] = xyzf[(size_t)cell * Nmax_cell + a];
        if (MULTI)
            s_otype[a] = cell_type[(size_t)cell * Nmax_cell + a];
        }
    __syncwarp();
    const float rc0 = MULTI ? 0.0f : r_cut[0];
    const float rl0 = MULTI ? 0.0f : r_listsq[0];
    const unsigned int Nmax0 = MULTI ? 0u : Nmax_t[0];
    const unsigned int lt_mask = (1u << lane) - 1u;
    const size_t row4 = (size_t)stride * 4u; // entries between consecutive groups of four

    for (unsigned int ob = 0; ob < csize; ob += 32)
        {
        const unsigned int nown = min(32u, csize - ob);
        unsigned int my_cnt = 0; // count of own particle ob + lane
        for (int pz = -1; pz <= 1; pz++)
            {
            // stage the nine cells of this plane; lane q < 9 describes cell q
            unsigned int q_cell = 0, q_n = 0;
            if (lane < 9)
                {
                const int ox = lane % 3 - 1, oy = lane / 3 - 1;
                const unsigned int ni = wrap_cell(ci + ox, dim.x);
                const unsigned int nj = wrap_cell(cj + oy, dim.y);
                const unsigned int nk = wrap_cell(ck + pz, dim.z);
                q_cell = (nk * dim.y + nj) * dim.x + ni;
                q_n = min(__ldg(cell_size + q_cell), Nmax_cell);
                // minImage's image rint((x_i - x_j)/L) for this cell: +1 when the stencil wraps
                // past the high face (x_j near the low face, x_i near the high face), -1 past
                // the low face, 0 otherwise
                const float ix = (ci + ox >= (int)dim.x) ? 1.f : (ci + ox < 0 ? -1.f : 0.f);
                const float iy = (cj + oy >= (int)dim.y) ? 1.f : (cj + oy < 0 ? -1.f : 0.f);
                const float iz = (ck + pz >= (int)dim.z) ? 1.f : (ck + pz < 0 ? -1.f : 0.f);
                s_shift[lane * 6 + 0] = fmul(box.L[2], iz);
                s_shift[lane * 6 + 1] = fmul(fmul(box.L[2], box.yz), iz);
                s_shift[lane * 6 + 2] = fmul(fmul(box.L[2], box.xz), iz);
                s_shift[lane * 6 + 3] = fmul(box.L[1], iy);
                s_shift[lane * 6 + 4] = fmul(fmul(box.L[1], box.xy), iy);
                s_shift[lane * 6 + 5] = fmul(box.L[0], ix);
                }
            // exclusive prefix of the nine counts
            unsigned int incl = q_n;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1)
                {
                const unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += y;
                }
            const unsigned int ncand = __shfl_sync(0xffffffffu, incl, 8);
            for (int q = 0; q < 9; q++)
                {
                const unsigned int qc = __shfl_sync(0xffffffffu, q_cell, q);
                const unsigned int qn = __shfl_sync(0xffffffffu, q_n, q);
                const unsigned int qo = __shfl_sync(0xffffffffu, incl - q_n, q);
                for (unsigned int t = lane; t < qn; t += 32)
                    {
                    s_cand[qo + t] = __ldg(xyzf + (size_t)qc * Nmax_cell + t);
                    s_meta[qo + t] = (unsigned int)q
                                     | (MULTI ? (__ldg(cell_type + (size_t)qc * Nmax_cell + t) << 8)
                                              : 0u);
                    }
                }
            __syncwarp();
            for (unsigned int cb = 0; cb < ncand; cb += 32)
                {
                const unsigned int t = cb + lane;
                const bool has = t < ncand;
                float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
                unsigned int meta = 0;
                if (has)
                    {
                    c = s_cand[t];
                    meta = s_meta[t];
                    }
                const unsigned int j = __float_as_uint(c.w);
                const float* sh = s_shift + (meta & 0xffu) * 6;
                const float sz = sh[0], syz = sh[1], sxz = sh[2], sy = sh[3], sxy = sh[4], sx = sh[5];
                const unsigned int tj = meta >> 8;
                // r_cut, r_list^2 and capacity of own particle o
                auto limits = [&](unsigned int o, float& rc, float& rl, unsigned int& nmax_o) {
                    if (MULTI)
                        {
                        const unsigned int ti = s_otype[ob + o];
                        rc = s_tab[ti * ntypes + tj];
                        rl = s_tab[ntypes * ntypes + ti * ntypes + tj];
                        nmax_o = __ldg(Nmax_t + ti);
                        }
                    else
                        {
                        rc = rc0;
                        rl = rl0;
                        nmax_o = Nmax0;
                        }
                };
                // the lanes holding a hit for own particle o write it at count(o) + rank
                auto emit = [&](unsigned int o, unsigned int i, bool hit, unsigned int nmax_o) {
                    const unsigned int bal = __ballot_sync(0xffffffffu, hit);
                    if (bal)
                        {
                        const unsigned int cnt_o = __shfl_sync(0xffffffffu, my_cnt, o);
                        const unsigned int k = cnt_o + __popc(bal & lt_mask);
                        if (hit && k < nmax_o)
                            {
                            if (LAYOUT == 4)
                                nlist[(size_t)(k >> 2) * row4 + (size_t)i * 4u + (k & 3u)] = j;
                            else
                                nlist[(size_t)k * stride + i] = j;
                            }
                        if (lane == (int)o)
                            my_cnt += __popc(bal);
                        }
                };
                unsigned int o = 0;
                if (ORTHO)
                    {
                    // two own particles per step: packed FP32 differences (each half rounds as the
                    // scalar fsub), scalar rounded squares and sums, so the decisions are identical
                    const uint64_t cx2 = f2pack(c.x, c.x), cy2 = f2pack(c.y, c.y),
                                   cz2 = f2pack(c.z, c.z);
                    const uint64_t sx2 = f2pack(sx, sx), sy2 = f2pack(sy, sy), sz2 = f2pack(sz, sz);
                    for (; o + 1 < nown; o += 2)
                        {
                        const float4 p0 = s_own[ob + o], p1 = s_own[ob + o + 1];
                        const uint64_t dx = f2sub(f2sub(f2pack(p0.x, p1.x), cx2), sx2);
                        const uint64_t dy = f2sub(f2sub(f2pack(p0.y, p1.y), cy2), sy2);
                        const uint64_t dz = f2sub(f2sub(f2pack(p0.z, p1.z), cz2), sz2);
                        float rsq0, rsq1;
                        f2dot3(dx, dy, dz, rsq0, rsq1);
                        const unsigned int i0 = __float_as_uint(p0.w), i1 = __float_as_uint(p1.w);
                        float rc, rl;
                        unsigned int nmax_o;
                        limits(o, rc, rl, nmax_o);
                        emit(o, i0, has && rsq0 <= rl && j != i0 && rc > 0.0f, nmax_o);
                        limits(o + 1, rc, rl, nmax_o);
                        emit(o + 1, i1, has && rsq1 <= rl && j != i1 && rc > 0.0f, nmax_o);
                        }
                    }
                for (; o < nown; o++)
                    {
                    const float4 pi = s_own[ob + o];
                    const unsigned int i = __float_as_uint(pi.w);
                    float dx = fsub(pi.x, c.x), dy = fsub(pi.y, c.y), dz = fsub(pi.z, c.z);
                    dz = fsub(dz, sz);
                    if (!ORTHO)
                        {
                        dy = fsub(dy, syz); // tilt terms; exactly zero in an orthorhombic box
                        dx = fsub(dx, sxz);
                        }
                    dy = fsub(dy, sy);
                    if (!ORTHO)
                        dx = fsub(dx, sxy);
                    dx = fsub(dx, sx);
                    const float rsq = dot3(dx, dy, dz);
                    float rc, rl;
                    unsigned int nmax_o;
                    limits(o, rc, rl, nmax_o);
                    emit(o, i, has && rsq <= rl && j != i && rc > 0.0f, nmax_o);
                    }
                }
            __syncwarp();
            }
        if (lane < (int)nown)
            {
            const float4 pi = s_own[ob + lane];
            const unsigned int i = __float_as_uint(pi.w);
            const unsigned int nmax_i = MULTI ? Nmax_t[s_otype[ob + lane]] : Nmax0;
            n_neigh[i] = min(my_cnt, nmax_i);
            if (my_cnt > nmax_i)
                atomicMax(&cond[MULTI ? s_otype[ob + lane] : 0u], my_cnt);
            if (last_pos)
                last_pos[i] = make_float4(pi.x, pi.y, pi.z, 0.0f);
            }
        __syncwarp();
        }
    }

// Lane-per-particle tiled build (same cases as k_nlist_tile): one warp per cell, lane l holds own
// particle ob + l in registers. The nine cells of each stencil plane are staged in shared memory
// as structure-of-arrays (x, y, z, index[, type]), every cell starting at an even slot, so two
// consecutive candidates load as one 8-byte packed pair. Every lane tests its own particle
// against the staged candidates two at a time: packed FP32 differences and squares (each half
// rounds as the scalar operation) and scalar rounded sums (f2dot3), so the decisions are
// bit-identical to the minImage sequence, and writes its hits straight into
// its own row; a cell's exact image shift is applied only when the stencil wraps there (it is
// zero otherwise, and x - 0 is exact). Hits come in the order (plane, cell, slot) of the
// warp-cooperative kernel above, so the lists are the same.
constexpr int LANE_WARPS = 4;

__host__ __device__ inline unsigned int lane_cap(unsigned int Nmax_cell)
    {
    return 9u * (Nmax_cell + 1u) + 1u & ~1u; // even-rounded cells, even total
    }

template<bool MULTI, int LAYOUT, bool ORTHO>
__global__ void __launch_bounds__(LANE_WARPS * 32)
    k_nlist_lane(unsigned int* __restrict__ nlist, unsigned int* __restrict__ n_neigh,
                 float4* __restrict__ last_pos, unsigned int* __restrict__ cond, uint64_t stride,
                 const unsigned int* __restrict__ Nmax_t,
                 const unsigned int* __restrict__ cell_size, const float4* __restrict__ xyzf,
                 const unsigned int* __restrict__ cell_type, uint3 dim, unsigned int ncell,
                 unsigned int Nmax_cell, gb_box box, const float* __restrict__ r_cut,
                 const float* __restrict__ r_listsq, unsigned int ntypes, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x / 32;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    // r_list^2 per type pair, -1 where r_cut is off (MULTI only), stored transposed: entry
    // (a, b) at b * ntypes + a, so the lanes (own particles of any type) testing one candidate
    // read consecutive words, free of bank conflicts
    float* s_tab = reinterpret_cast<float*>(smem);
    const size_t tab_bytes = MULTI ? ((2 * sizeof(float) * ntypes * ntypes + 15) / 16) * 16 : 0;
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x)
            s_tab[(t % ntypes) * ntypes + t / ntypes] = r_cut[t] > 0.0f ? r_listsq[t] : -1.0f;
        __syncthreads();
        }
    const unsigned int cap = lane_cap(Nmax_cell);
    const size_t per_warp = ((size_t)cap * 4u * (MULTI ? 5u : 4u) + 15) / 16 * 16;
    unsigned char* base = smem + tab_bytes + (size_t)warp * per_warp;
    float* s_x = reinterpret_cast<float*>(base);
    float* s_y = s_x + cap;
    float* s_z = s_y + cap;
    unsigned int* s_j = reinterpret_cast<unsigned int*>(s_z + cap);
    unsigned int* s_t = s_j + cap;

    const unsigned int cell = blockIdx.x * wpb + warp;
    if (cell >= ncell)
        return;
    const int ci = cell % dim.x, cj = (cell / dim.x) % dim.y, ck = cell / (dim.x * dim.y);
    const unsigned int csize = min(cell_size[cell], Nmax_cell);
    if (csize == 0)
        return;
    const size_t row4 = (size_t)stride * 4u;

    for (unsigned int ob = 0; ob < csize; ob += 32)
        {
        const bool active = ob + lane < csize;
        float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
        unsigned int ti = 0;
        if (active)
            {
            pi = __ldg(xyzf + (size_t)cell * Nmax_cell + ob + lane);
            if (MULTI)
                ti = __ldg(cell_type + (size_t)cell * Nmax_cell + ob + lane);
            }
        const unsigned int i = __float_as_uint(pi.w);
        const unsigned int nmax_i = active ? __ldg(Nmax_t + (MULTI ? ti : 0u)) : 0u;
        // next free slot of this particle's row (interleaved by four: four consecutive slots, then
        // a jump of one row of groups)
        // (word offsets fit 32 bits: a list of 2^32 words would be 16 GB)
        unsigned int wo = LAYOUT == 4 ? i * 4u : i;
        const unsigned int jump = LAYOUT == 4 ? (unsigned int)row4 - 3u : (unsigned int)stride;
        unsigned int cnt = 0;
        auto put = [&](bool hit, unsigned int j) {
            if (hit && cnt < nmax_i)
                nlist[wo] = j;
            if (hit)
                {
                cnt++;
                if (LAYOUT == 4)
                    wo += (cnt & 3u) ? 1u : jump;
                else
                    wo += jump;
                }
        };
        // r_list^2 of the pair, or -1 (never met) for an inactive lane or a pair without r_cut
        const float rl_single = (!MULTI && active && __ldg(r_cut) > 0.0f) ? __ldg(r_listsq) : -1.0f;
        auto rlim = [&](unsigned int slot) -> float {
            if (MULTI)
                return active ? s_tab[s_t[slot] * ntypes + ti] : -1.0f;
            return rl_single;
        };
        const uint64_t px2 = f2pack(pi.x, pi.x), py2 = f2pack(pi.y, pi.y), pz2 = f2pack(pi.z, pi.z);

        for (int pz = -1; pz <= 1; pz++)
            {
            unsigned int q_cell = 0, q_n = 0;
            if (lane < 9)
                {
                const int ox = lane % 3 - 1, oy = lane / 3 - 1;
                q_cell = (wrap_cell(ck + pz, dim.z) * dim.y + wrap_cell(cj + oy, dim.y)) * dim.x
                         + wrap_cell(ci + ox, dim.x);
                q_n = min(__ldg(cell_size + q_cell), Nmax_cell);
                }
            const unsigned int q_pad = (q_n + 1u) & ~1u;
            unsigned int incl = q_pad;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1)
                {
                const unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += y;
                }
            const unsigned int q_off = incl - q_pad;
            for (int q = 0; q < 9; q++)
                {
                const unsigned int qc = __shfl_sync(0xffffffffu, q_cell, q);
                const unsigned int qn = __shfl_sync(0xffffffffu, q_n, q);
                const unsigned int qo = __shfl_sync(0xffffffffu, q_off, q);
                for (unsigned int t = lane; t < qn; t += 32)
                    {
                    const float4 c = __ldg(xyzf + (size_t)qc * Nmax_cell + t);
                    s_x[qo + t] = c.x;
                    s_y[qo + t] = c.y;
                    s_z[qo + t] = c.z;
                    s_j[qo + t] = __float_as_uint(c.w);
                    if (MULTI)
                        s_t[qo + t] = __ldg(cell_type + (size_t)qc * Nmax_cell + t);
                    }
                }
            __syncwarp();
            for (int q = 0; q < 9; q++)
                {
                const unsigned int qn = __shfl_sync(0xffffffffu, q_n, q);
                const unsigned int qo = __shfl_sync(0xffffffffu, q_off, q);
                const int ox = q % 3 - 1, oy = q / 3 - 1;
                // minImage's image for this cell: +1 past the high face, -1 past the low face
                const float ix = (ci + ox >= (int)dim.x) ? 1.f : (ci + ox < 0 ? -1.f : 0.f);
                const float iy = (cj + oy >= (int)dim.y) ? 1.f : (cj + oy < 0 ? -1.f : 0.f);
                const float iz = (ck + pz >= (int)dim.z) ? 1.f : (ck + pz < 0 ? -1.f : 0.f);
                const bool wrapped = ix != 0.f || iy != 0.f || iz != 0.f;
                const float sz = fmul(box.L[2], iz), sy = fmul(box.L[1], iy), sx = fmul(box.L[0], ix);
                const float syz = ORTHO ? 0.f : fmul(fmul(box.L[2], box.yz), iz);
                const float sxz = ORTHO ? 0.f : fmul(fmul(box.L[2], box.xz), iz);
                const float sxy = ORTHO ? 0.f : fmul(fmul(box.L[1], box.xy), iy);
                // the own particle itself can only be met in the centre cell
                auto scan = [&](auto centre_tag) {
                constexpr bool centre = decltype(centre_tag)::value;
                unsigned int t = 0;
                if (ORTHO)
                    {
                    const uint64_t sx2 = f2pack(sx, sx), sy2 = f2pack(sy, sy), sz2 = f2pack(sz, sz);
                    for (; t + 1 < qn; t += 2)
                        {
                        const unsigned int slot = qo + t;
                        const uint64_t cx = *reinterpret_cast<const uint64_t*>(s_x + slot);
                        const uint64_t cy = *reinterpret_cast<const uint64_t*>(s_y + slot);
                        const uint64_t cz = *reinterpret_cast<const uint64_t*>(s_z + slot);
                        uint64_t dx = f2sub(px2, cx), dy = f2sub(py2, cy), dz = f2sub(pz2, cz);
                        if (wrapped)
                            {
                            dz = f2sub(dz, sz2);
                            dy = f2sub(dy, sy2);
                            dx = f2sub(dx, sx2);
                            }
                        float rsq0, rsq1;
                        f2dot3(dx, dy, dz, rsq0, rsq1);
                        const uint2 jj = *reinterpret_cast<const uint2*>(s_j + slot);
                        put(rsq0 <= rlim(slot) && (!centre || jj.x != i), jj.x);
                        put(rsq1 <= rlim(slot + 1) && (!centre || jj.y != i), jj.y);
                        }
                    }
                for (; t < qn; t++)
                    {
                    const unsigned int slot = qo + t;
                    const unsigned int j = s_j[slot];
                    float dx = fsub(pi.x, s_x[slot]), dy = fsub(pi.y, s_y[slot]),
                          dz = fsub(pi.z, s_z[slot]);
                    if (wrapped)
                        {
                        dz = fsub(dz, sz);
                        if (!ORTHO)
                            {
                            dy = fsub(dy, syz); // tilt terms; exactly zero in an orthorhombic box
                            dx = fsub(dx, sxz);
                            }
                        dy = fsub(dy, sy);
                        if (!ORTHO)
                            dx = fsub(dx, sxy);
                        dx = fsub(dx, sx);
                        }
                    const float rsq = dot3(dx, dy, dz);
                    put(rsq <= rlim(slot) && (!centre || j != i), j);
                    }
                };
                if (pz == 0 && q == 4)
                    scan(std::true_type {});
                else
                    scan(std::false_type {});
                }
            __syncwarp();
            }
        if (active)
            {
            n_neigh[i] = min(cnt, nmax_i);
            if (cnt > nmax_i)
                atomicMax(&cond[MULTI ? ti : 0u], cnt);
            if (last_pos)
                last_pos[i] = make_float4(pi.x, pi.y, pi.z, 0.0f);
            }
        }
    }

// Candidate-stream build (same cases as k_nlist_lane): one warp per cell, the lanes holding
// candidates instead of own particles, so every lane works whatever the cell's occupancy. The
// own particles (the cell's, 32 per pass) sit in shared memory. Each stencil plane's nine cells
// form one stream of candidates in the order (cell, slot); the warp takes 32 of them into its
// lanes' registers, walks the own particles, and records each own particle's test of the 32 as
// one ballot mask. After the plane, lane p takes own particle p and appends the candidates of its
// masks in stream order, so its list is the lane build's list, entry for entry. Distances use the
// lane build's operation order (minImage's, with the cell's exact image shift only where the
// stencil wraps), so the decisions are bit-identical.
constexpr int STREAM_WARPS = 4;

// 32-candidate blocks of one plane's stream, at most
__host__ __device__ inline unsigned int stream_nb(unsigned int Nmax_cell)
    {
    return (9u * Nmax_cell + 31u) / 32u;
    }

// per-warp shared memory (words): own x, y, z, index and type row [32 each], plane record
// [32], candidate indices [32 nb], masks [32 nb]
__host__ __device__ inline size_t stream_warp_bytes(unsigned int Nmax_cell)
    {
    return 4u * 32u * 6u + 2u * 4u * 32u * (size_t)stream_nb(Nmax_cell);
    }

template<bool MULTI, int LAYOUT, bool ORTHO>
__global__ void __launch_bounds__(STREAM_WARPS * 32, 6)
    k_nlist_stream(unsigned int* __restrict__ nlist, unsigned int* __restrict__ n_neigh,
                   float4* __restrict__ last_pos, unsigned int* __restrict__ cond,
                   uint64_t stride, const unsigned int* __restrict__ Nmax_t,
                   const unsigned int* __restrict__ cell_size, const float4* __restrict__ xyzf,
                   const unsigned int* __restrict__ cell_type, uint3 dim, unsigned int ncell,
                   unsigned int Nmax_cell, gb_box box, const float* __restrict__ r_cut,
                   const float* __restrict__ r_listsq, unsigned int ntypes, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x / 32;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    // r_list^2 per type pair (own row, candidate column), -1 where r_cut is off (MULTI only)
    float* s_tab = reinterpret_cast<float*>(smem);
    const size_t tab_bytes = MULTI ? ((sizeof(float) * ntypes * ntypes + 15) / 16) * 16 : 0;
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x)
            s_tab[t] = r_cut[t] > 0.0f ? r_listsq[t] : -1.0f;
        __syncthreads();
        }
    const unsigned int nb_max = stream_nb(Nmax_cell);
    unsigned char* base = smem + tab_bytes + (size_t)warp * stream_warp_bytes(Nmax_cell);
    // own particles by pairs: s_oa[q] = (x, x', y, y') and s_ob[q] = (z, z', index, index') of own
    // particles 2q and 2q + 1, so one 16-byte load gives a packed pair of two coordinates
    float4* s_oa = reinterpret_cast<float4*>(base);
    float4* s_ob = s_oa + 16;
    unsigned int* s_orow = reinterpret_cast<unsigned int*>(s_ob + 16);
    unsigned int* s_plane = s_orow + 32; // [0, 10) offsets, [10, 19) cells, [19, 28) images
    unsigned int* s_cj = s_plane + 32;
    unsigned int* s_mask = s_cj + 32 * nb_max;

    const unsigned int cell = blockIdx.x * wpb + warp;
    if (cell >= ncell)
        return;
    const int ci = cell % dim.x, cj = (cell / dim.x) % dim.y, ck = cell / (dim.x * dim.y);
    const unsigned int csize = min(cell_size[cell], Nmax_cell);
    if (csize == 0)
        return;
    const size_t row4 = (size_t)stride * 4u;
    const float rl_single = (!MULTI && __ldg(r_cut) > 0.0f) ? __ldg(r_listsq) : -1.0f;
    const float inf = __int_as_float(0x7f800000);

    for (unsigned int ob = 0; ob < csize; ob += 32)
        {
        const unsigned int n_pass = min(csize - ob, 32u);
        const bool active = lane < n_pass;
        float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
        unsigned int ti = 0;
        if (active)
            {
            pi = __ldg(xyzf + (size_t)cell * Nmax_cell + ob + lane);
            if (MULTI)
                ti = __ldg(cell_type + (size_t)cell * Nmax_cell + ob + lane);
            float* a = reinterpret_cast<float*>(s_oa + lane / 2) + (lane & 1);
            float* bz = reinterpret_cast<float*>(s_ob + lane / 2) + (lane & 1);
            a[0] = pi.x;
            a[2] = pi.y;
            bz[0] = pi.z;
            bz[2] = pi.w;
            if (MULTI)
                s_orow[lane] = ti * ntypes;
            }
        const unsigned int i = __float_as_uint(pi.w);
        const unsigned int nmax_i = active ? __ldg(Nmax_t + (MULTI ? ti : 0u)) : 0u;
        unsigned int wo = LAYOUT == 4 ? i * 4u : i;
        const unsigned int jump = LAYOUT == 4 ? (unsigned int)row4 - 3u : (unsigned int)stride;
        unsigned int cnt = 0;

        for (int pz = -1; pz <= 1; pz++)
            {
            // the plane's nine cells: offsets of their runs in the stream, cell, image
            unsigned int q_n = 0;
            bool q_wrap = false;
            if (lane < 9)
                {
                const int ox = lane % 3 - 1, oy = lane / 3 - 1;
                const unsigned int q_cell
                    = (wrap_cell(ck + pz, dim.z) * dim.y + wrap_cell(cj + oy, dim.y)) * dim.x
                      + wrap_cell(ci + ox, dim.x);
                q_n = min(__ldg(cell_size + q_cell), Nmax_cell);
                const int ix = (ci + ox >= (int)dim.x) ? 1 : (ci + ox < 0 ? -1 : 0);
                const int iy = (cj + oy >= (int)dim.y) ? 1 : (cj + oy < 0 ? -1 : 0);
                const int iz = (ck + pz >= (int)dim.z) ? 1 : (ck + pz < 0 ? -1 : 0);
                q_wrap = ix != 0 || iy != 0 || iz != 0;
                s_plane[10 + lane] = q_cell;
                s_plane[19 + lane] = (unsigned int)((ix + 1) | ((iy + 1) << 2) | ((iz + 1) << 4));
                }
            unsigned int incl = q_n;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1)
                {
                const unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += y;
                }
            if (lane < 9)
                s_plane[lane] = incl - q_n;
            const unsigned int total = __shfl_sync(0xffffffffu, incl, 8);
            if (lane == 9)
                s_plane[9] = total;
            const bool plane_wraps = __any_sync(0xffffffffu, q_wrap);
            __syncwarp();
            const unsigned int nb = (total + 31u) / 32u;
            unsigned int q = 0;
            for (unsigned int b = 0; b < nb; b++)
                {
                // this lane's candidate: stream entry 32 b + lane
                const unsigned int k = 32u * b + lane;
                float cx = inf, cy = inf, cz = inf;
                unsigned int cjdx = 0xffffffffu, ct = 0;
                float sx = 0.f, sy = 0.f, sz = 0.f, syz = 0.f, sxz = 0.f, sxy = 0.f;
                if (k < total)
                    {
                    while (k >= s_plane[q + 1])
                        q++;
                    const unsigned int qc = s_plane[10 + q];
                    const unsigned int slot = k - s_plane[q];
                    const float4 c = __ldg(xyzf + (size_t)qc * Nmax_cell + slot);
                    cx = c.x;
                    cy = c.y;
                    cz = c.z;
                    cjdx = __float_as_uint(c.w);
                    if (MULTI)
                        ct = __ldg(cell_type + (size_t)qc * Nmax_cell + slot);
                    const unsigned int img = s_plane[19 + q];
                    const float ix = (float)((int)(img & 3u) - 1);
                    const float iy = (float)((int)((img >> 2) & 3u) - 1);
                    const float iz = (float)((int)((img >> 4) & 3u) - 1);
                    sz = fmul(box.L[2], iz);
                    sy = fmul(box.L[1], iy);
                    sx = fmul(box.L[0], ix);
                    if (!ORTHO)
                        {
                        syz = fmul(fmul(box.L[2], box.yz), iz);
                        sxz = fmul(fmul(box.L[2], box.xz), iz);
                        sxy = fmul(fmul(box.L[1], box.xy), iy);
                        }
                    }
                s_cj[k] = cjdx;
                unsigned int* mrow = s_mask + 32u * b;
                auto test = [&](auto wrap_tag) {
                    constexpr bool wrapped = decltype(wrap_tag)::value;
                    unsigned int p = 0;
                    // two own particles per step: packed FP32 differences and squares (each half
                    // rounds as the scalar operation), scalar rounded sums (f2dot3)
                    const uint64_t cx2 = f2pack(cx, cx), cy2 = f2pack(cy, cy), cz2 = f2pack(cz, cz);
#pragma unroll 2
                    for (; p + 1 < n_pass; p += 2)
                        {
                        const float4 oa = s_oa[p / 2], obz = s_ob[p / 2];
                        uint64_t dx = f2sub(f2pack(oa.x, oa.y), cx2);
                        uint64_t dy = f2sub(f2pack(oa.z, oa.w), cy2);
                        uint64_t dz = f2sub(f2pack(obz.x, obz.y), cz2);
                        if (wrapped)
                            {
                            dz = f2sub(dz, f2pack(sz, sz));
                            if (!ORTHO)
                                {
                                dy = f2sub(dy, f2pack(syz, syz));
                                dx = f2sub(dx, f2pack(sxz, sxz));
                                }
                            dy = f2sub(dy, f2pack(sy, sy));
                            if (!ORTHO)
                                dx = f2sub(dx, f2pack(sxy, sxy));
                            dx = f2sub(dx, f2pack(sx, sx));
                            }
                        float r0, r1;
                        f2dot3(dx, dy, dz, r0, r1);
                        const uint2 oi = make_uint2(__float_as_uint(obz.z), __float_as_uint(obz.w));
                        float rl0 = rl_single, rl1 = rl_single;
                        if (MULTI)
                            {
                            const uint2 orow = *reinterpret_cast<const uint2*>(s_orow + p);
                            rl0 = s_tab[orow.x + ct];
                            rl1 = s_tab[orow.y + ct];
                            }
                        const unsigned int m0 = __ballot_sync(0xffffffffu, r0 <= rl0 && cjdx != oi.x);
                        const unsigned int m1 = __ballot_sync(0xffffffffu, r1 <= rl1 && cjdx != oi.y);
                        if (lane == 0)
                            *reinterpret_cast<uint2*>(mrow + p) = make_uint2(m0, m1);
                        }
                    for (; p < n_pass; p++)
                        {
                        const float* a = reinterpret_cast<const float*>(s_oa + p / 2) + (p & 1);
                        const float* bz = reinterpret_cast<const float*>(s_ob + p / 2) + (p & 1);
                        const float4 o = make_float4(a[0], a[2], bz[0], bz[2]);
                        float dx = fsub(o.x, cx), dy = fsub(o.y, cy), dz = fsub(o.z, cz);
                        if (wrapped)
                            {
                            dz = fsub(dz, sz);
                            if (!ORTHO)
                                {
                                dy = fsub(dy, syz);
                                dx = fsub(dx, sxz);
                                }
                            dy = fsub(dy, sy);
                            if (!ORTHO)
                                dx = fsub(dx, sxy);
                            dx = fsub(dx, sx);
                            }
                        const float rsq = dot3(dx, dy, dz);
                        const float rl = MULTI ? s_tab[s_orow[p] + ct] : rl_single;
                        const bool hit = rsq <= rl && cjdx != __float_as_uint(o.w);
                        const unsigned int m = __ballot_sync(0xffffffffu, hit);
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
            // lane p appends own particle p's hits of this plane in stream order
            if (active)
                {
                for (unsigned int b = 0; b < nb; b++)
                    {
                    unsigned int m = s_mask[32u * b + lane];
                    const unsigned int* cjb = s_cj + 32u * b;
                    auto put = [&](unsigned int j) {
                        if (cnt < nmax_i)
                            nlist[wo] = j;
                        cnt++;
                        if (LAYOUT == 4)
                            wo += (cnt & 3u) ? 1u : jump;
                        else
                            wo += jump;
                    };
                    // two hits per iteration: both candidate loads issue before the stores
                    while (m)
                        {
                        const unsigned int t0 = __ffs(m) - 1;
                        m &= m - 1u;
                        const unsigned int t1 = m ? __ffs(m) - 1 : t0;
                        const bool two = m != 0u;
                        m &= m - 1u;
                        const unsigned int j0 = cjb[t0], j1 = cjb[t1];
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
            n_neigh[i] = min(cnt, nmax_i);
            if (cnt > nmax_i)
                atomicMax(&cond[MULTI ? ti : 0u], cnt);
            if (last_pos)
                last_pos[i] = make_float4(pi.x, pi.y, pi.z, 0.0f);
            }
        __syncwarp();
        }
    }

size_t stream_smem_bytes(unsigned int Nmax_cell, unsigned int ntypes, bool multi, int wpb)
    {
    const size_t tab = multi ? ((sizeof(float) * ntypes * ntypes + 15) / 16) * 16 : 0;
    return tab + (size_t)wpb * stream_warp_bytes(Nmax_cell);
    }

size_t lane_smem_bytes(unsigned int Nmax_cell, unsigned int ntypes, bool multi, int wpb)
    {
    const size_t tab = multi ? ((2 * sizeof(float) * ntypes * ntypes + 15) / 16) * 16 : 0;
    const size_t per_warp = ((size_t)lane_cap(Nmax_cell) * 4u * (multi ? 5u : 4u) + 15) / 16 * 16;
    return tab + (size_t)wpb * per_warp;
    }

size_t tile_smem_bytes(unsigned int Nmax_cell, unsigned int ntypes, bool multi, int wpb)
    {
    const size_t tab = multi ? ((2 * sizeof(float) * ntypes * ntypes + 15) / 16) * 16 : 0;
    const size_t per_warp = (size_t)Nmax_cell * (16 + 16 * 9 + 4 * 9 + 4) + 9 * 6 * 4;
    return tab + (size_t)wpb * ((per_warp + 15) / 16 * 16);
    }

template<bool MULTI, int LAYOUT>
bool launch_nlist_tile(const gb_nlist_args& a, unsigned int ncell, cudaStream_t s)
    {
    const bool ortho = a.box.xy == 0.0f && a.box.xz == 0.0f && a.box.yz == 0.0f;
    if (a.nlist_capacity != 0 && a.nlist_capacity <= 0xffffffffull)
        {
        if (a.threads_per_particle != 1)
            {
            // the candidate stream (32 lanes test each own particle), the default
            int wpb2 = a.block_size ? (int)(a.block_size / 32) : STREAM_WARPS;
            size_t smem2 = stream_smem_bytes(a.Nmax_cell, a.ntypes, MULTI, wpb2);
            while (smem2 > 96 * 1024 && wpb2 > 1)
                smem2 = stream_smem_bytes(a.Nmax_cell, a.ntypes, MULTI, --wpb2);
            if (smem2 <= 200 * 1024)
                {
                auto kern2 = ortho ? k_nlist_stream<MULTI, LAYOUT, true>
                                   : k_nlist_stream<MULTI, LAYOUT, false>;
                if (smem2 > 48 * 1024)
                    cudaFuncSetAttribute(kern2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem2);
                kern2<<<div_up(ncell, wpb2), wpb2 * 32, smem2, s>>>(
                    a.d_nlist, a.d_n_neigh, reinterpret_cast<float4*>(a.d_last_pos),
                    a.d_conditions, a.stride, a.d_Nmax, a.d_cell_size,
                    reinterpret_cast<const float4*>(a.d_xyzf), a.d_cell_type,
                    make_uint3(a.dim[0], a.dim[1], a.dim[2]), ncell, a.Nmax_cell, a.box, a.d_r_cut,
                    a.d_r_listsq, a.ntypes, a.d_gate);
                return true;
                }
            }
        int wpb = a.block_size ? (int)(a.block_size / 32) : LANE_WARPS;
        size_t smem = lane_smem_bytes(a.Nmax_cell, a.ntypes, MULTI, wpb);
        while (smem > 96 * 1024 && wpb > 1)
            smem = lane_smem_bytes(a.Nmax_cell, a.ntypes, MULTI, --wpb);
        if (smem > 200 * 1024)
            return false;
        auto kern = ortho ? k_nlist_lane<MULTI, LAYOUT, true> : k_nlist_lane<MULTI, LAYOUT, false>;
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<div_up(ncell, wpb), wpb * 32, smem, s>>>(
            a.d_nlist, a.d_n_neigh, reinterpret_cast<float4*>(a.d_last_pos), a.d_conditions,
            a.stride, a.d_Nmax, a.d_cell_size, reinterpret_cast<const float4*>(a.d_xyzf),
            a.d_cell_type, make_uint3(a.dim[0], a.dim[1], a.dim[2]), ncell, a.Nmax_cell, a.box,
            a.d_r_cut, a.d_r_listsq, a.ntypes, a.d_gate);
        return true;
        }
    int wpb = TILE_WARPS_MAX;
    size_t smem = tile_smem_bytes(a.Nmax_cell, a.ntypes, MULTI, wpb);
    while (smem > 96 * 1024 && wpb > 1)
        smem = tile_smem_bytes(a.Nmax_cell, a.ntypes, MULTI, --wpb);
    if (smem > 200 * 1024)
        return false;
    auto kern = ortho ? k_nlist_tile<MULTI, LAYOUT, true> : k_nlist_tile<MULTI, LAYOUT, false>;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<div_up(ncell, wpb), wpb * 32, smem, s>>>(
        a.d_nlist, a.d_n_neigh, reinterpret_cast<float4*>(a.d_last_pos), a.d_conditions, a.stride,
        a.d_Nmax, a.d_cell_size, reinterpret_cast<const float4*>(a.d_xyzf), a.d_cell_type,
        make_uint3(a.dim[0], a.dim[1], a.dim[2]), ncell, a.Nmax_cell, a.box, a.d_r_cut,
        a.d_r_listsq, a.ntypes, a.d_gate);
    return true;
    }

template<bool MULTI, int LAYOUT, int MI>
void launch_nlist(const gb_nlist_args& a, unsigned int ncell, cudaStream_t s)
    {
    size_t smem = MULTI ? 2 * sizeof(float) * a.ntypes * a.ntypes : 0;
    k_nlist_binned<MULTI, LAYOUT, MI><<<div_up(ncell, NL_WARPS), NL_WARPS * 32, smem, s>>>(
        a.d_nlist, a.d_n_neigh, reinterpret_cast<float4*>(a.d_last_pos), a.d_conditions,
        a.d_head_list, a.stride, a.d_Nmax, a.d_cell_size,
        reinterpret_cast<const float4*>(a.d_xyzf), a.d_cell_type, a.d_cell_adj,
        make_uint3(a.dim[0], a.dim[1], a.dim[2]), ncell, a.Nmax_cell, a.adj_width, a.box,
        a.d_r_cut, a.d_r_listsq, a.ntypes, a.d_gate);
    }

template<bool MULTI, int LAYOUT>
void launch_nlist_mi(const gb_nlist_args& a, unsigned int ncell, cudaStream_t s)
    {
    const bool ortho = a.box.xy == 0.0f && a.box.xz == 0.0f && a.box.yz == 0.0f;
    const bool all_periodic = a.box.periodic[0] && a.box.periodic[1] && a.box.periodic[2];
    // four or more cells per side: an index difference of +-(dim-1) can only be a wrapped
    // neighbour, and rint(dx/L) agrees with the cell image whenever |dx| <= L/2 could matter
    if (a.adj_width == 27 && all_periodic && a.dim[0] >= 4 && a.dim[1] >= 4 && a.dim[2] >= 4)
        launch_nlist<MULTI, LAYOUT, 2>(a, ncell, s);
    else if (ortho)
        launch_nlist<MULTI, LAYOUT, 1>(a, ncell, s);
    else
        launch_nlist<MULTI, LAYOUT, 0>(a, ncell, s);
    }

template<bool MULTI>
void launch_nlist_layout(const gb_nlist_args& a, unsigned int ncell, cudaStream_t s)
    {
    const bool all_periodic = a.box.periodic[0] && a.box.periodic[1] && a.box.periodic[2];
    const bool tiled = !a.d_head_list && a.adj_width == 27 && all_periodic && a.dim[0] >= 4
                       && a.dim[1] >= 4 && a.dim[2] >= 4;
    if (tiled)
        {
        if (a.interleave == 4 ? launch_nlist_tile<MULTI, 4>(a, ncell, s)
                              : launch_nlist_tile<MULTI, 1>(a, ncell, s))
            return;
        }
    if (a.d_head_list)
        launch_nlist_mi<MULTI, 0>(a, ncell, s);
    else if (a.interleave == 4)
        launch_nlist_mi<MULTI, 4>(a, ncell, s);
    else
        launch_nlist_mi<MULTI, 1>(a, ncell, s);
    }

// Stable in-place removal of excluded neighbours (one thread per particle; hoomd's
// gpu_nlist_filter_kernel does the same per particle).
template<int LAYOUT>
__global__ void k_nlist_filter(unsigned int* nlist, unsigned int* n_neigh,
                               const uint64_t* __restrict__ head, uint64_t stride, unsigned int N,
                               const unsigned int* __restrict__ n_ex,
                               const unsigned int* __restrict__ ex_list, unsigned int ex_pitch,
                               const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N)
        return;
    const unsigned int ne = n_ex[i];
    if (ne == 0)
        return;
    auto at = [&](unsigned int k) -> size_t {
        if (LAYOUT == 0)
            return (size_t)head[i] + k;
        if (LAYOUT == 1)
            return (size_t)k * stride + i;
        return ((size_t)(k >> 2) * stride + i) * 4 + (k & 3u);
    };
    const unsigned int* ex = ex_list + (size_t)i * ex_pitch;
    const unsigned int nn = n_neigh[i];
    unsigned int w = 0;
    for (unsigned int k = 0; k < nn; k++)
        {
        const unsigned int j = nlist[at(k)];
        bool drop = false;
        for (unsigned int e = 0; e < ne; e++)
            drop = drop || ex[e] == j;
        if (!drop)
            nlist[at(w++)] = j;
        }
    n_neigh[i] = w;
    }

__global__ void k_needs_update(uint32_t* result, const float4* __restrict__ last_pos,
                               const float4* __restrict__ pos, unsigned int N, gb_box box,
                               const float* __restrict__ rcut_max, float r_buff,
                               float lambda_min, float3 lambda, uint32_t checkn)
    {
    unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool moved = false;
    if (i < N)
        {
        float4 p = pos[i], lp = last_pos[i];
        float dx = fsub(p.x, fmul(lambda.x, lp.x));
        float dy = fsub(p.y, fmul(lambda.y, lp.y));
        float dz = fsub(p.z, fmul(lambda.z, lp.z));
        min_image(box, dx, dy, dz);
        const float rmin = rcut_max[__float_as_uint(p.w)];
        const float rmax = fadd(rmin, r_buff);
        const float delta_max = fmul(fsub(fmul(rmax, lambda_min), rmin), 0.5f);
        const float maxsq = (delta_max > 0.0f) ? fmul(delta_max, delta_max) : 0.0f;
        moved = dot3(dx, dy, dz) >= maxsq;
        }
    if (__any_sync(0xffffffffu, moved) && (threadIdx.x % 32) == 0)
        atomicMax(result, checkn);
    }

// Block-level inclusive scan helpers for the head list.
__global__ void k_head_block(const float4* __restrict__ pos, unsigned int N,
                             const unsigned int* __restrict__ Nmax, uint64_t* head,
                             uint64_t* block_sums)
    {
    __shared__ uint64_t s[1024];
    unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t v = (i < N) ? Nmax[__float_as_uint(pos[i].w)] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (unsigned int o = 1; o < blockDim.x; o <<= 1)
        {
        uint64_t t = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
        }
    if (i < N)
        head[i] = s[threadIdx.x] - v; // exclusive
    if (threadIdx.x == blockDim.x - 1)
        block_sums[blockIdx.x] = s[threadIdx.x];
    }

__global__ void k_head_offsets(uint64_t* block_sums, unsigned int nblocks, uint64_t* total)
    {
    if (threadIdx.x == 0 && blockIdx.x == 0)
        {
        uint64_t run = 0;
        for (unsigned int b = 0; b < nblocks; b++)
            {
            uint64_t t = block_sums[b];
            block_sums[b] = run;
            run += t;
            }
        *total = run;
        }
    }

__global__ void k_head_add(uint64_t* head, unsigned int N, const uint64_t* block_sums)
    {
    unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N)
        head[i] += block_sums[blockIdx.x];
    }
} // namespace
} // namespace gb

using namespace gb;

extern "C"
    {
    int gb_cell_list_build(const gb_cell_list_args* a, void* stream)
        {
        GB_REQUIRE(a, "gb_cell_list_build: null args");
        GB_REQUIRE(a->d_pos || a->N == 0, "gb_cell_list_build: null positions");
        GB_REQUIRE(a->d_cell_size && a->d_xyzf && a->d_conditions,
                   "gb_cell_list_build: null output");
        GB_REQUIRE(a->Nmax > 0, "gb_cell_list_build: Nmax must be > 0");
        const unsigned int ncell = a->dim[0] * a->dim[1] * a->dim[2];
        GB_REQUIRE(ncell > 0, "gb_cell_list_build: empty cell grid");
        cudaStream_t s = (cudaStream_t)stream;
        GB_REQUIRE(!a->d_timestep == !a->d_build_steps,
                   "gb_cell_list_build: the build statistics need both the step and the record");
        const int sms = num_sms();
        const BuildRecord rec {a->d_dangerous, a->check_delay, a->check_dist};
        // with counts_zeroed the binning launch keeps the statistics (and there must be one)
        const bool stats_in_bin = a->counts_zeroed && a->N > 0;
        if (!stats_in_bin)
            k_zero_u32<<<min(div_up(ncell, 256), (unsigned)sms * 8), 256, 0, s>>>(
                a->counts_zeroed ? nullptr : a->d_cell_size, a->counts_zeroed ? 0 : ncell,
                a->d_gate, a->d_build_count, a->d_timestep, a->d_build_steps, rec);
        if (a->N > 0)
            k_cell_bin<<<min(div_up(a->N, 256), (unsigned)sms * 16), 256, 0, s>>>(
                reinterpret_cast<const float4*>(a->d_pos), a->N, a->box,
                make_uint3(a->dim[0], a->dim[1], a->dim[2]), a->Nmax, a->d_cell_size,
                reinterpret_cast<float4*>(a->d_xyzf), a->d_cell_type, a->d_conditions,
                a->d_gate, stats_in_bin, a->d_build_count, a->d_timestep, a->d_build_steps, rec);
        if (a->deterministic)
            {
            const int wpb = 4;
            size_t smem = (size_t)wpb * a->Nmax * (sizeof(float4) + sizeof(unsigned int));
            GB_REQUIRE(smem <= 200 * 1024, "gb_cell_list_build: Nmax too large to sort cells");
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(k_cell_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
            k_cell_sort<<<min(div_up(ncell, wpb), (unsigned)sms * 8), wpb * 32, smem, s>>>(
                a->d_cell_size, reinterpret_cast<float4*>(a->d_xyzf), a->d_cell_type, ncell,
                a->Nmax, a->d_gate);
            }
        return check_launch("gb_cell_list_build");
        }

    int gb_cell_adj_build(const unsigned int dim[3], unsigned int ndim, unsigned int* d_adj,
                          unsigned int* width_out, void* stream)
        {
        GB_REQUIRE(dim && d_adj && width_out, "gb_cell_adj_build: null argument");
        unsigned int nu[3];
        for (int d = 0; d < 3; d++)
            nu[d] = dim[d] > 3 ? 3 : dim[d];
        unsigned int w = (ndim == 2) ? nu[0] * nu[1] : nu[0] * nu[1] * nu[2];
        *width_out = w;
        unsigned int ncell = dim[0] * dim[1] * dim[2];
        GB_REQUIRE(ncell > 0, "gb_cell_adj_build: empty grid");
        k_cell_adj<<<div_up(ncell, 128), 128, 0, (cudaStream_t)stream>>>(
            make_uint3(dim[0], dim[1], dim[2]), ndim, w, d_adj);
        return check_launch("gb_cell_adj_build");
        }

    int gb_nlist_build_binned(const gb_nlist_args* a, void* stream)
        {
        GB_REQUIRE(a, "gb_nlist_build_binned: null args");
        GB_REQUIRE(a->d_nlist && a->d_n_neigh && a->d_conditions && a->d_Nmax,
                   "gb_nlist_build_binned: null output");
        GB_REQUIRE(a->d_cell_size && a->d_xyzf && a->d_cell_adj, "gb_nlist_build_binned: no cells");
        GB_REQUIRE(a->ntypes >= 1 && a->d_r_cut && a->d_r_listsq,
                   "gb_nlist_build_binned: cutoff tables required");
        GB_REQUIRE(a->ntypes == 1 || a->d_cell_type,
                   "gb_nlist_build_binned: cell types required when ntypes > 1");
        GB_REQUIRE(a->d_head_list || a->stride >= a->N,
                   "gb_nlist_build_binned: column-major stride must be >= N");
        GB_REQUIRE(a->adj_width >= 1 && a->adj_width <= 27, "gb_nlist_build_binned: adj width");
        GB_REQUIRE(a->ntypes <= 64, "gb_nlist_build_binned: at most 64 types");
        GB_REQUIRE(a->block_size == 0 || a->block_size == 32 || a->block_size == 64
                       || a->block_size == 128,
                   "gb_nlist_build_binned: block_size must be 32, 64 or 128");
        GB_REQUIRE(a->threads_per_particle == 0 || a->threads_per_particle == 1
                       || a->threads_per_particle == 32,
                   "gb_nlist_build_binned: threads_per_particle must be 1 or 32");
        const unsigned int ncell = a->dim[0] * a->dim[1] * a->dim[2];
        if (ncell == 0 || a->N == 0)
            return GB_OK;
        GB_REQUIRE(a->d_head_list || a->interleave <= 1 || a->interleave == 4,
                   "gb_nlist_build_binned: interleave must be 1 or 4");
        cudaStream_t s = (cudaStream_t)stream;
        if (a->ntypes > 1)
            launch_nlist_layout<true>(*a, ncell, s);
        else
            launch_nlist_layout<false>(*a, ncell, s);
        return check_launch("gb_nlist_build_binned");
        }

    int gb_nlist_needs_update(uint32_t* d_result, const float* d_last_pos, const float* d_pos,
                              unsigned int N, const gb_box* box, const float* d_rcut_max,
                              float r_buff, unsigned int ntypes, float lambda_min,
                              const float lambda[3], uint32_t checkn, void* stream)
        {
        GB_REQUIRE(d_result && box && d_rcut_max && lambda, "gb_nlist_needs_update: null argument");
        (void)ntypes;
        if (N == 0)
            return GB_OK;
        k_needs_update<<<div_up(N, 256), 256, 0, (cudaStream_t)stream>>>(
            d_result, reinterpret_cast<const float4*>(d_last_pos),
            reinterpret_cast<const float4*>(d_pos), N, *box, d_rcut_max, r_buff, lambda_min,
            make_float3(lambda[0], lambda[1], lambda[2]), checkn);
        return check_launch("gb_nlist_needs_update");
        }

    int gb_nlist_filter(unsigned int* d_nlist, unsigned int* d_n_neigh,
                        const uint64_t* d_head_list, uint64_t stride, uint32_t interleave,
                        unsigned int N, const unsigned int* d_n_ex, const unsigned int* d_ex_list,
                        unsigned int ex_pitch, const uint32_t* d_gate, void* stream)
        {
        GB_REQUIRE(d_nlist && d_n_neigh && d_n_ex && d_ex_list, "gb_nlist_filter: null argument");
        GB_REQUIRE(ex_pitch > 0, "gb_nlist_filter: ex_pitch must be positive");
        if (N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        const unsigned int grid = div_up(N, 256);
        if (d_head_list)
            k_nlist_filter<0><<<grid, 256, 0, s>>>(d_nlist, d_n_neigh, d_head_list, stride, N,
                                                   d_n_ex, d_ex_list, ex_pitch, d_gate);
        else
            {
            GB_REQUIRE(stride >= N, "gb_nlist_filter: column-major stride < N");
            if (interleave == 4)
                k_nlist_filter<4><<<grid, 256, 0, s>>>(d_nlist, d_n_neigh, nullptr, stride, N,
                                                       d_n_ex, d_ex_list, ex_pitch, d_gate);
            else
                k_nlist_filter<1><<<grid, 256, 0, s>>>(d_nlist, d_n_neigh, nullptr, stride, N,
                                                       d_n_ex, d_ex_list, ex_pitch, d_gate);
            }
        return check_launch("gb_nlist_filter");
        }

    int gb_nlist_head_list(uint64_t* d_head_list, uint64_t* d_total, const float* d_pos,
                           unsigned int N, const unsigned int* d_Nmax, unsigned int ntypes,
                           void* stream)
        {
        GB_REQUIRE(d_head_list && d_total && d_Nmax, "gb_nlist_head_list: null argument");
        (void)ntypes;
        cudaStream_t s = (cudaStream_t)stream;
        if (N == 0)
            return cudaMemsetAsync(d_total, 0, sizeof(uint64_t), s) == cudaSuccess
                       ? GB_OK
                       : fail(GB_ERR_CUDA, "gb_nlist_head_list: memset");
        const unsigned int nb = div_up(N, 1024);
        // block sums live after the N head entries' worth of scratch in d_total[1..nb]
        k_head_block<<<nb, 1024, 0, s>>>(reinterpret_cast<const float4*>(d_pos), N, d_Nmax,
                                         d_head_list, d_total + 1);
        k_head_offsets<<<1, 1, 0, s>>>(d_total + 1, nb, d_total);
        k_head_add<<<nb, 1024, 0, s>>>(d_head_list, N, d_total + 1);
        return check_launch("gb_nlist_head_list");
        }
    }
