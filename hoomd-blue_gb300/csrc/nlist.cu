// Cell list and binned neighbour list on GB300.
//
// Cell list (replaces gpu_compute_cell_list, hoomd/CellListGPU.cu:42-170): one thread per
// particle bins it with the reference's makeFraction arithmetic and claims a slot with an atomic.
// Optional deterministic mode sorts each cell's slots by particle index afterwards
// (hoomd/CellListGPU.cu:478-540 does the same with a global thrust sort).
//
// Neighbour list (replaces gpu_compute_nlist_binned, hoomd/md/NeighborListGPUBinned.cu:52-298):
// one warp per cell. The warp's lanes own the cell's particles; for each of the 27 (or fewer,
// deduplicated) adjacent cells the warp stages 32 candidates at a time in shared memory with one
// coalesced load, then every lane tests its particle against every staged candidate. All lanes
// walk the same candidate sequence, so there is no divergence in the search (the reference's
// thread-per-particle search diverges whenever a warp straddles cells). Hits are written in the
// column-major layout nlist[k * stride + i] (coalesced across particles in SFC order) or the
// reference's flat head-list layout.
#include <cstdint>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
constexpr int NL_WARPS = 4; // warps per block in the build kernel

__global__ void k_zero_u32(unsigned int* p, size_t n, const uint32_t* gate, uint64_t* count)
    {
    if (gate && *gate == 0)
        return;
    if (count && blockIdx.x == 0 && threadIdx.x == 0)
        *count += 1;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = 0;
    }

__global__ void k_cell_bin(const float4* __restrict__ pos, unsigned int N, gb_box box, uint3 dim,
                           unsigned int Nmax, unsigned int* cell_size, float4* xyzf,
                           unsigned int* cell_type, unsigned int* cond, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
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

// The build: see the file comment. MULTI: per-pair r_cut / r_list tables (ntypes > 1);
// ORTHO: zero tilt factors; FLAT: reference head-list layout instead of column-major.
template<bool MULTI, bool ORTHO, bool FLAT>
__global__ void __launch_bounds__(NL_WARPS * 32)
    k_nlist_binned(unsigned int* __restrict__ nlist, unsigned int* __restrict__ n_neigh,
                   float4* __restrict__ last_pos, unsigned int* __restrict__ cond,
                   const uint64_t* __restrict__ head_list, uint64_t stride,
                   const unsigned int* __restrict__ Nmax_t,
                   const unsigned int* __restrict__ cell_size, const float4* __restrict__ xyzf,
                   const unsigned int* __restrict__ cell_type,
                   const unsigned int* __restrict__ cell_adj, unsigned int ncell,
                   unsigned int Nmax_cell, unsigned int adj_w, gb_box box,
                   const float* __restrict__ r_cut, const float* __restrict__ r_listsq,
                   unsigned int ntypes, const uint32_t* gate)
    {
    if (gate && *gate == 0)
        return;
    __shared__ float4 s_cand[NL_WARPS][32];
    __shared__ unsigned int s_ctype[NL_WARPS][32];
    extern __shared__ float s_tab[]; // [2 * ntypes^2] r_cut then r_listsq (MULTI only)
    if (MULTI)
        {
        for (unsigned int t = threadIdx.x; t < ntypes * ntypes; t += blockDim.x)
            {
            s_tab[t] = r_cut[t];
            s_tab[ntypes * ntypes + t] = r_listsq[t];
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
        const uint64_t head = FLAT ? (active ? head_list[i] : 0ull) : (uint64_t)i;
        const uint64_t step = FLAT ? 1ull : stride;
        unsigned int cnt = 0;
        for (unsigned int a = 0; a < adj_w; a++)
            {
            const unsigned int nc = __ldg(cell_adj + (size_t)cell * adj_w + a);
            const unsigned int nsz = min(__ldg(cell_size + nc), Nmax_cell);
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
                    for (unsigned int t = 0; t < m; t++)
                        {
                        const float4 c = s_cand[warp][t];
                        const unsigned int j = __float_as_uint(c.w);
                        float dx = fsub(pi.x, c.x), dy = fsub(pi.y, c.y), dz = fsub(pi.z, c.z);
                        if (ORTHO)
                            min_image_ortho(box, dx, dy, dz);
                        else
                            min_image(box, dx, dy, dz);
                        const float rsq = dot3(dx, dy, dz);
                        float rc, rl;
                        if (MULTI)
                            {
                            const unsigned int tp = ti * ntypes + s_ctype[warp][t];
                            rc = s_tab[tp];
                            rl = s_tab[ntypes * ntypes + tp];
                            }
                        else
                            {
                            rc = rc0;
                            rl = rl0;
                            }
                        if (rsq <= rl && j != i && rc > 0.0f)
                            {
                            if (cnt < Nmax_i)
                                nlist[head + (uint64_t)cnt * step] = j;
                            cnt++;
                            }
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

template<bool MULTI, bool ORTHO, bool FLAT>
void launch_nlist(const gb_nlist_args& a, unsigned int ncell, cudaStream_t s)
    {
    size_t smem = MULTI ? 2 * sizeof(float) * a.ntypes * a.ntypes : 0;
    k_nlist_binned<MULTI, ORTHO, FLAT><<<div_up(ncell, NL_WARPS), NL_WARPS * 32, smem, s>>>(
        a.d_nlist, a.d_n_neigh, reinterpret_cast<float4*>(a.d_last_pos), a.d_conditions,
        a.d_head_list, a.stride, a.d_Nmax, a.d_cell_size,
        reinterpret_cast<const float4*>(a.d_xyzf), a.d_cell_type, a.d_cell_adj, ncell,
        a.Nmax_cell, a.adj_width, a.box, a.d_r_cut, a.d_r_listsq, a.ntypes, a.d_gate);
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
        const int sms = num_sms();
        k_zero_u32<<<min(div_up(ncell, 256), (unsigned)sms * 8), 256, 0, s>>>(a->d_cell_size,
                                                                             ncell, a->d_gate,
                                                                             a->d_build_count);
        if (a->N > 0)
            k_cell_bin<<<min(div_up(a->N, 256), (unsigned)sms * 16), 256, 0, s>>>(
                reinterpret_cast<const float4*>(a->d_pos), a->N, a->box,
                make_uint3(a->dim[0], a->dim[1], a->dim[2]), a->Nmax, a->d_cell_size,
                reinterpret_cast<float4*>(a->d_xyzf), a->d_cell_type, a->d_conditions,
                a->d_gate);
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
        const unsigned int ncell = a->dim[0] * a->dim[1] * a->dim[2];
        if (ncell == 0 || a->N == 0)
            return GB_OK;
        cudaStream_t s = (cudaStream_t)stream;
        const bool multi = a->ntypes > 1;
        const bool ortho = a->box.xy == 0.0f && a->box.xz == 0.0f && a->box.yz == 0.0f;
        const bool flat = a->d_head_list != nullptr;
        if (multi)
            {
            if (ortho)
                flat ? launch_nlist<true, true, true>(*a, ncell, s)
                     : launch_nlist<true, true, false>(*a, ncell, s);
            else
                flat ? launch_nlist<true, false, true>(*a, ncell, s)
                     : launch_nlist<true, false, false>(*a, ncell, s);
            }
        else
            {
            if (ortho)
                flat ? launch_nlist<false, true, true>(*a, ncell, s)
                     : launch_nlist<false, true, false>(*a, ncell, s);
            else
                flat ? launch_nlist<false, false, true>(*a, ncell, s)
                     : launch_nlist<false, false, false>(*a, ncell, s);
            }
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
