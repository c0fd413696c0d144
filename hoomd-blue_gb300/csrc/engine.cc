// Host engine implementation (see engine.h). Kernels are reached only through the C ABI.
#include "engine.h"
#include "surrogate.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <iostream>
#include <sstream>

namespace gbe
{

void check(int rc, const char* what)
    {
    if (rc != GB_OK)
        throw std::runtime_error(std::string(what) + ": " + gb_last_error());
    }

void cuda_check(cudaError_t e, const char* what)
    {
    if (e != cudaSuccess)
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }

static inline uint32_t f2u(float f)
    {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
    }
static inline float u2f(uint32_t u)
    {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
    }

// ------------------------------------------------------------------------------------------------
// ParticleData
// ------------------------------------------------------------------------------------------------
ParticleData::ParticleData(unsigned int N_, unsigned int ntypes_, unsigned int ndim_,
                           const std::vector<double>& b6, const std::vector<int>& per)
    : N(N_), ntypes(ntypes_), ndim(ndim_)
    {
    if (b6.size() != 6)
        throw std::invalid_argument("box must have 6 entries [Lx, Ly, Lz, xy, xz, yz]");
    if (ntypes == 0)
        throw std::invalid_argument("at least one particle type is required");
    for (int d = 0; d < 6; d++)
        box6[d] = b6[d];
    for (int d = 0; d < 3; d++)
        periodic[d] = per.size() == 3 ? per[d] : 1;
    check(gb_box_make(box6, box6[3], box6[4], box6[5], periodic, &box), "gb_box_make");
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    pos.resize(4 * (size_t)N);
    vel.resize(4 * (size_t)N);
    accel.resize(3 * (size_t)N);
    image.resize(3 * (size_t)N);
    tag.resize(N);
    accel.zero(stream);
    scratch.resize(std::max<size_t>(gb_thermo_scratch_bytes(N), 4096));
    scratch.zero(stream);
    }

ParticleData::Stage ParticleData::stage()
    {
    const size_t need = gb_snapshot_stage_bytes(N) + 256;
    if (io_stage.size() < need)
        io_stage.resize(need);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t n = N;
    char* b = io_stage.get();
    Stage st;
    st.pos = reinterpret_cast<double*>(b);
    b += up(24 * n);
    st.vel = reinterpret_cast<double*>(b);
    b += up(24 * n);
    st.mass = reinterpret_cast<double*>(b);
    b += up(8 * n);
    st.charge = reinterpret_cast<double*>(b);
    b += up(8 * n);
    st.typeid_ = reinterpret_cast<uint32_t*>(b);
    b += up(4 * n);
    st.image = reinterpret_cast<int32_t*>(b);
    b += up(12 * n);
    st.rtag = reinterpret_cast<uint32_t*>(b);
    b += up(4 * n);
    st.err = reinterpret_cast<uint32_t*>(b);
    return st;
    }

// initializeFromSnapshot's per-particle part on the device: one bulk copy per snapshot array into
// the staging block, then gb_snapshot_scatter (conversion to FP32, wrap into the box, images).
void ParticleData::set_particles(const double* p, const double* v, const double* m,
                                 const uint32_t* t, const int32_t* img, const double* q)
    {
    if (!p || !v || !m || !t || !img)
        throw std::invalid_argument("set_particles: position, velocity, mass, typeid and image "
                                    "arrays are required");
    const Stage st = stage();
    const size_t n = N;
    auto h2d = [&](void* dst, const void* src, size_t bytes) {
        if (bytes)
            cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream),
                       "set_particles copy");
    };
    h2d(st.pos, p, 24 * n);
    h2d(st.vel, v, 24 * n);
    h2d(st.mass, m, 8 * n);
    h2d(st.typeid_, t, 4 * n);
    h2d(st.image, img, 12 * n);
    if (charge.size() != N)
        charge.resize(N);
    if (q)
        h2d(st.charge, q, 8 * n);
    else
        charge.zero(stream); // the snapshot's charges are all at their default, 0
    const uint32_t* rt = nullptr;
    if (tags_set)
        {
        check(gb_rtag(tag.get(), N, st.rtag, stream), "gb_rtag");
        rt = st.rtag;
        }
    cuda_check(cudaMemsetAsync(st.err, 0xFF, sizeof(uint32_t), stream), "set_particles err");
    check(gb_snapshot_scatter(st.pos, st.vel, st.mass, st.typeid_, st.image,
                              q ? st.charge : nullptr, rt, N, ntypes, &box, pos.get(), vel.get(),
                              image.get(), tag.get(), q ? charge.get() : nullptr, st.err, stream),
          "gb_snapshot_scatter");
    uint32_t err = 0;
    cuda_check(cudaMemcpyAsync(&err, st.err, sizeof(err), cudaMemcpyDeviceToHost, stream),
               "set_particles err");
    accel.zero(stream);
    accel_set = false;
    cuda_check(cudaStreamSynchronize(stream), "set_particles");
    if (err != 0xFFFFFFFFu)
        throw std::invalid_argument("typeid out of range (particle tag " + std::to_string(err)
                                    + ")");
    tags_set = true;
    }

void ParticleData::set_charges(const double* q)
    {
    const std::vector<uint32_t> r = rtag();
    std::vector<float> h(N);
    for (unsigned int t = 0; t < N; t++)
        h[r[t]] = (float)q[t];
    charge.resize(N);
    charge.upload(h.data(), h.size(), stream);
    cuda_check(cudaStreamSynchronize(stream), "set_charges");
    }

void ParticleData::set_box(const double* b6)
    {
    for (int d = 0; d < 6; d++)
        box6[d] = b6[d];
    check(gb_box_make(box6, box6[3], box6[4], box6[5], periodic, &box), "gb_box_make");
    }

std::vector<uint32_t> ParticleData::rtag()
    {
    std::vector<uint32_t> t(N), r(N);
    tag.download(t.data(), N, stream);
    cuda_check(cudaStreamSynchronize(stream), "rtag");
    for (unsigned int i = 0; i < N; i++)
        r[t[i]] = i;
    return r;
    }

// takeSnapshot's per-particle part on the device: gb_snapshot_gather writes the tag-ordered FP64
// arrays into the staging block, then one bulk copy per array to the host.
void ParticleData::get_particles(double* p, double* v, double* m, uint32_t* t, int32_t* img)
    {
    const Stage st = stage();
    const size_t n = N;
    check(gb_snapshot_gather(pos.get(), vel.get(), image.get(), tag.get(), N, st.pos, st.vel,
                             st.mass, st.typeid_, st.image, stream),
          "gb_snapshot_gather");
    auto d2h = [&](void* dst, const void* src, size_t bytes) {
        if (dst && bytes)
            cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream),
                       "get_particles copy");
    };
    d2h(p, st.pos, 24 * n);
    d2h(v, st.vel, 24 * n);
    d2h(m, st.mass, 8 * n);
    d2h(t, st.typeid_, 4 * n);
    d2h(img, st.image, 12 * n);
    cuda_check(cudaStreamSynchronize(stream), "get_particles");
    }

void ParticleData::thermalize(double kT, uint64_t ts)
    {
    check(gb_thermalize(vel.get(), tag.get(), N, kT, ts, seed, ndim, scratch.get(), stream),
          "gb_thermalize");
    cuda_check(cudaStreamSynchronize(stream), "thermalize");
    }

// ------------------------------------------------------------------------------------------------
// NeighborList (NeighborListGPUBinned + CellListGPU)
// ------------------------------------------------------------------------------------------------
NeighborList::NeighborList(std::shared_ptr<ParticleData> pd, double rb)
    : pdata(std::move(pd)), r_buff((float)rb)
    {
    if (rb < 0.0)
        throw std::invalid_argument("Requested buffer radius is less than zero.");
    own_rcut.assign(pdata->ntypes * pdata->ntypes, 0.0f);
    Nmax.assign(pdata->ntypes, 0);
    cond.resize(3 + 64);
    }

void NeighborList::set_r_cut(unsigned int i, unsigned int j, double r)
    {
    const unsigned int nt = pdata->ntypes;
    own_rcut[i * nt + j] = own_rcut[j * nt + i] = (float)r;
    dirty = true;
    }

void NeighborList::add_consumer(const std::vector<float>* m)
    {
    consumers.push_back(m);
    dirty = true;
    }

void NeighborList::ensure_consumer(const std::vector<float>* m)
    {
    if (std::find(consumers.begin(), consumers.end(), m) == consumers.end())
        add_consumer(m);
    }

void NeighborList::remove_consumer(const std::vector<float>* m)
    {
    const auto n = consumers.size();
    consumers.erase(std::remove(consumers.begin(), consumers.end(), m), consumers.end());
    if (consumers.size() != n)
        dirty = true;
    }

void NeighborList::clear_consumers()
    {
    consumers.clear();
    dirty = true;
    }

// hoomd/md/NeighborList.cc:452-529
void NeighborList::update_rlist()
    {
    const unsigned int nt = pdata->ntypes;
    r_cut = own_rcut;
    for (auto* m : consumers)
        for (unsigned int k = 0; k < nt * nt; k++)
            r_cut[k] = std::max(r_cut[k], (*m)[k]);
    r_listsq.assign(nt * nt, 0.0f);
    rcut_max.assign(nt, 0.0f);
    for (unsigned int i = 0; i < nt; i++)
        {
        float mx = 0.0f;
        for (unsigned int j = 0; j < nt; j++)
            {
            const float rc = r_cut[i * nt + j];
            if (rc > mx)
                mx = rc;
            volatile float rl = (rc > 0.0f) ? rc + r_buff : 0.0f;
            r_listsq[i * nt + j] = rl * rl;
            }
        rcut_max[i] = mx;
        }
    }

void NeighborList::allocate()
    {
    ParticleData& pd = *pdata;
    const unsigned int nt = pd.ntypes;
    alloc_generation++;
    update_rlist();
    float rmax = 0.0f;
    for (float v : rcut_max)
        rmax = std::max(rmax, v);
    const float width = rmax + r_buff;
    if (!(width > 0.0f))
        throw std::runtime_error("Cell: cell width must be non-zero");
    // NeighborList::checkBoxSize (hoomd/md/NeighborList.cc:535-561)
    {
    unsigned int d1[3];
    check(gb_cell_dims(&pd.box, pd.ndim, 1.0f, d1), "gb_cell_dims");
    float npd[3];
    float a = pd.box.xy * pd.box.yz - pd.box.xz;
    npd[0] = pd.box.L[0] / std::sqrt(1.0f + pd.box.xy * pd.box.xy + a * a);
    npd[1] = pd.box.L[1] / std::sqrt(1.0f + pd.box.yz * pd.box.yz);
    npd[2] = pd.box.L[2];
    for (int d = 0; d < (pd.ndim == 3 ? 3 : 2); d++)
        if (pd.periodic[d] && npd[d] <= width * 2.0f)
            {
            std::ostringstream oss;
            oss << "nlist: Simulation box is too small, the neighbor list is searching beyond the "
                   " minimum image: rmax="
                << width;
            throw std::runtime_error(oss.str());
            }
    }
    check(gb_cell_dims(&pd.box, pd.ndim, width, dim), "gb_cell_dims");
    const unsigned int ncell = dim[0] * dim[1] * dim[2];
    adj.resize(27 * (size_t)ncell);
    check(gb_cell_adj_build(dim, pd.ndim, adj.get(), &adj_w, pd.stream), "gb_cell_adj_build");
    // capacities: the reference starts from ceil(N/ncell) and grows on overflow; start with
    // headroom so that replayed runs rarely roll back
    const double per_cell = double(pd.N) / ncell;
    const unsigned int want_cell = (unsigned int)std::ceil(per_cell * 1.6) + 4;
    if (!capacity_fixed)
        Nmax_cell = std::max(Nmax_cell, want_cell);
    const double vol = (pd.ndim == 3) ? double(pd.box.L[0]) * pd.box.L[1] * pd.box.L[2]
                                      : double(pd.box.L[0]) * pd.box.L[1];
    const double rho = pd.N / vol;
    for (unsigned int t = 0; t < nt; t++)
        {
        float rl = 0.0f;
        for (unsigned int j = 0; j < nt; j++)
            rl = std::max(rl, r_listsq[t * nt + j]);
        rl = std::sqrt(rl);
        const double shell = (pd.ndim == 3) ? 4.0 / 3.0 * M_PI * rl * rl * rl : M_PI * rl * rl;
        // several types: each type's rows take the largest count among fewer particles, and a
        // rollback replays a whole chunk, so start those with more room
        const double headroom = nt > 1 ? 1.5 : 1.35;
        unsigned int want = (unsigned int)std::ceil(rho * shell * headroom) + 8;
        want = (want + 3) & ~3u;
        if (!capacity_fixed)
            Nmax[t] = std::max(Nmax[t], want);
        }
    capacity_fixed = false; // a fixed start applies to the first allocation only
    stride = ((uint64_t)pd.N + 31) / 32 * 32;
    const unsigned int nmax_all = *std::max_element(Nmax.begin(), Nmax.end());
    cell_size.resize(ncell);
    xyzf.resize(4 * (size_t)ncell * Nmax_cell);
    cell_type.resize(nt > 1 ? (size_t)ncell * Nmax_cell : 0);
    // the interleaved layout writes whole groups of four: a capacity that is not a multiple of
    // four (a fixed start capacity) still needs its last group allocated
    nlist.resize(std::max<uint64_t>(1, stride * ((nmax_all + 3u) & ~3u)));
    n_neigh.resize(std::max(1u, pd.N));
    n_neigh.zero(pd.stream);
    last_pos.resize(4 * (size_t)std::max(1u, pd.N));
    d_Nmax.resize(nt);
    d_Nmax.upload(Nmax.data(), nt, pd.stream);
    d_r_cut.resize(nt * nt);
    d_r_cut.upload(r_cut.data(), nt * nt, pd.stream);
    d_r_listsq.resize(nt * nt);
    d_r_listsq.upload(r_listsq.data(), nt * nt, pd.stream);
    d_rcut_max.resize(nt);
    d_rcut_max.upload(rcut_max.data(), nt, pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "nlist allocate");
    allocated = true;
    dirty = false;
    }

void NeighborList::enqueue_build(const uint32_t* d_gate, uint64_t* d_build_count,
                                 uint32_t* d_cell_cond, uint32_t* d_nl_cond, cudaStream_t s,
                                 const uint64_t* d_timestep, uint64_t* d_build_steps,
                                 uint64_t* d_dangerous, bool counts_zeroed)
    {
    ParticleData& pd = *pdata;
    gb_cell_list_args c {};
    c.d_dangerous = d_dangerous;
    c.check_delay = rebuild_check_delay;
    c.check_dist = check_dist ? 1 : 0;
    c.d_pos = pd.pos.get();
    c.N = pd.N;
    c.box = pd.box;
    for (int d = 0; d < 3; d++)
        c.dim[d] = dim[d];
    c.Nmax = Nmax_cell;
    c.d_cell_size = cell_size.get();
    c.d_xyzf = xyzf.get();
    c.d_cell_type = pd.ntypes > 1 ? cell_type.get() : nullptr;
    c.d_conditions = d_cell_cond;
    c.d_gate = d_gate;
    c.deterministic = deterministic ? 1 : 0;
    c.d_build_count = d_build_count;
    c.d_timestep = d_timestep;
    c.d_build_steps = d_build_steps;
    c.counts_zeroed = counts_zeroed ? 1 : 0;
    check(gb_cell_list_build(&c, s), "gb_cell_list_build");
    gb_nlist_args a {};
    a.d_nlist = nlist.get();
    a.d_n_neigh = n_neigh.get();
    a.d_last_pos = last_pos.get();
    a.d_conditions = d_nl_cond;
    a.d_head_list = nullptr;
    a.stride = stride;
    a.interleave = 4;
    a.d_Nmax = d_Nmax.get();
    a.d_pos = pd.pos.get();
    a.N = pd.N;
    a.d_cell_size = cell_size.get();
    a.d_xyzf = xyzf.get();
    a.d_cell_type = pd.ntypes > 1 ? cell_type.get() : nullptr;
    a.d_cell_adj = adj.get();
    for (int d = 0; d < 3; d++)
        a.dim[d] = dim[d];
    a.Nmax_cell = Nmax_cell;
    a.adj_width = adj_w;
    a.box = pd.box;
    a.d_r_cut = d_r_cut.get();
    a.d_r_listsq = d_r_listsq.get();
    a.ntypes = pd.ntypes;
    a.d_gate = d_gate;
    a.block_size = kp_block;
    a.threads_per_particle = kp_tpp;
    a.nlist_capacity = nlist.size();
    check(gb_nlist_build_binned(&a, s), "gb_nlist_build_binned");
    if (ex_pitch > 0)
        check(gb_nlist_filter(nlist.get(), n_neigh.get(), nullptr, stride, 4, pd.N, n_ex.get(),
                              ex_list.get(), ex_pitch, d_gate, s),
              "gb_nlist_filter");
    }

void NeighborList::set_exclusions(const std::vector<uint32_t>& tag_pairs)
    {
    if (tag_pairs.size() % 2)
        throw std::invalid_argument("exclusions are (tag, tag) pairs");
    for (uint32_t t : tag_pairs)
        if (t >= pdata->N)
            throw std::invalid_argument("exclusion refers to a tag >= N");
    ex_tags = tag_pairs;
    ex_dirty = true;
    }

// per-index exclusion rows from the tag pairs and the current tag -> index map
void NeighborList::refresh_exclusions()
    {
    ParticleData& pd = *pdata;
    if (!ex_dirty && ex_generation == pd.sort_generation)
        return;
    // new exclusions (not a re-sort of the same ones) may change the row pitch and the buffers
    if (ex_dirty)
        alloc_generation++;
    ex_dirty = false;
    ex_generation = pd.sort_generation;
    if (ex_tags.empty())
        {
        ex_pitch = 0;
        return;
        }
    const std::vector<uint32_t> rtag = pd.rtag();
    std::vector<std::vector<uint32_t>> rows(pd.N);
    for (size_t k = 0; k < ex_tags.size(); k += 2)
        {
        const uint32_t a = rtag[ex_tags[k]], b = rtag[ex_tags[k + 1]];
        rows[a].push_back(b);
        rows[b].push_back(a);
        }
    unsigned int pitch = 1;
    for (auto& r : rows)
        pitch = std::max<unsigned int>(pitch, (unsigned int)r.size());
    std::vector<uint32_t> cnt(pd.N), flat((size_t)pd.N * pitch, 0u);
    for (unsigned int i = 0; i < pd.N; i++)
        {
        cnt[i] = (uint32_t)rows[i].size();
        std::copy(rows[i].begin(), rows[i].end(), flat.begin() + (size_t)i * pitch);
        }
    ex_pitch = pitch;
    n_ex.resize(pd.N);
    ex_list.resize(flat.size());
    n_ex.upload(cnt.data(), cnt.size(), pd.stream);
    ex_list.upload(flat.data(), flat.size(), pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "exclusions");
    }

bool NeighborList::grow(const DevStatus& st)
    {
    bool grew = false;
    if (st.cell_cond[0] > Nmax_cell)
        {
        Nmax_cell = st.cell_cond[0] + std::max(4u, st.cell_cond[0] / 8);
        grew = true;
        }
    std::vector<bool> over(pdata->ntypes, false);
    bool nl_grew = false;
    for (unsigned int t = 0; t < pdata->ntypes; t++)
        if (st.nl_cond[t] > Nmax[t])
            {
            unsigned int want = st.nl_cond[t] + std::max(8u, st.nl_cond[t] / 8);
            Nmax[t] = (want + 3) & ~3u;
            over[t] = true;
            grew = nl_grew = true;
            }
    // the types share one density: when one type's row overflows, the others are near their
    // capacity too, so give every type an eighth more at once instead of one rollback each
    if (nl_grew)
        for (unsigned int t = 0; t < pdata->ntypes; t++)
            if (!over[t])
                Nmax[t] = (Nmax[t] + std::max(8u, Nmax[t] / 8) + 3) & ~3u;
    if (grew)
        {
        allocated = false;
        allocate();
        }
    return grew;
    }

static std::string tag_message(ParticleData& pd, uint32_t index_plus_one, const char* what)
    {
    std::vector<uint32_t> t(pd.N);
    pd.tag.download(t.data(), pd.N, pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "tag lookup");
    std::ostringstream s;
    s << "Particle with unique tag " << t[index_plus_one - 1] << " " << what;
    return s.str();
    }

void NeighborList::build_sync()
    {
    ParticleData& pd = *pdata;
    if (!allocated || dirty)
        allocate();
    refresh_exclusions();
    for (int attempt = 0; attempt < 64; attempt++)
        {
        cond.zero(pd.stream);
        enqueue_build(nullptr, nullptr, cond.get(), cond.get() + 3, pd.stream);
        DevStatus st {};
        std::vector<uint32_t> h(3 + 64);
        cond.download(h.data(), h.size(), pd.stream);
        cuda_check(cudaStreamSynchronize(pd.stream), "nlist build");
        if (h[1])
            throw std::runtime_error(tag_message(pd, h[1], "has NaN for its position."));
        if (h[2])
            throw std::runtime_error(tag_message(pd, h[2], "is no longer in the simulation box."));
        for (int k = 0; k < 3; k++)
            st.cell_cond[k] = h[k];
        for (unsigned int t = 0; t < pd.ntypes; t++)
            st.nl_cond[t] = h[3 + t];
        if (!grow(st))
            return;
        }
    throw std::runtime_error("neighbour list build did not converge");
    }

std::vector<uint32_t> NeighborList::pair_list(bool full, bool local)
    {
    ParticleData& pd = *pdata;
    std::vector<uint32_t> nn(pd.N), t(pd.N), nl(nlist.size());
    n_neigh.download(nn.data(), pd.N, pd.stream);
    nlist.download(nl.data(), nl.size(), pd.stream);
    pd.tag.download(t.data(), pd.N, pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "pair_list");
    std::vector<uint32_t> out;
    for (unsigned int i = 0; i < pd.N; i++)
        for (unsigned int k = 0; k < nn[i]; k++)
            {
            uint32_t j = nl[((size_t)(k >> 2) * stride + i) * 4 + (k & 3)];
            uint32_t a = local ? i : t[i], b = local ? j : t[j];
            if (full || a < b)
                {
                out.push_back(a);
                out.push_back(b);
                }
            }
    return out;
    }

// ------------------------------------------------------------------------------------------------
// PairForce (PotentialPair<Evaluator>GPU)
// ------------------------------------------------------------------------------------------------
PairForce::PairForce(std::shared_ptr<ParticleData> pd, std::shared_ptr<NeighborList> nl,
                     PairKind k)
    : pdata(std::move(pd)), nlist(std::move(nl)), kind(k)
    {
    ntypes = pdata->ntypes;
    const unsigned int np = ntypes * ntypes;
    r_cut.assign(np, 0.0f);
    r_on.assign(np, 0.0f);
    lj.assign(np, gb_lj_param {0.0f, 0.0f});
    ex.assign(np, gb_example_param {0.0f, 0.0f});
    rad.assign(np, gb_radial_param {});
    dpd.assign(np, gb_dpd_param {});
    t_rmin.assign(np, 0.0);
    t_U.assign(np, std::vector<double>(1, 0.0));
    t_F.assign(np, std::vector<double>(1, 0.0));
    force.resize(4 * (size_t)std::max(1u, pdata->N));
    force.zero(pdata->stream);
    }

PairForce::~PairForce()
    {
    // the list keeps a pointer to this force's r_cut matrix while it is a consumer
    if (nlist)
        nlist->remove_consumer(&r_cut);
    }

void PairForce::compute_standalone(bool with_virial)
    {
    nlist->ensure_consumer(&r_cut);
    nlist->build_sync();
    compute(pdata->stream, with_virial);
    cuda_check(cudaStreamSynchronize(pdata->stream), "compute");
    }

// EvaluatorPairDPDThermoDPD / DPDThermoLJ parameters (hoomd/md/EvaluatorPairDPDThermoLJ.h:60-90)
void PairForce::set_params_dpd(unsigned int i, unsigned int j, bool lj, double a_or_eps,
                               double sigma, double gamma)
    {
    gb_dpd_param p {};
    if (lj)
        {
        const double s6 = sigma * sigma * sigma * sigma * sigma * sigma;
        p.lj1 = (float)(4.0 * a_or_eps * s6 * s6);
        p.lj2 = (float)(4.0 * a_or_eps * s6);
        }
    else
        p.a = (float)a_or_eps;
    p.gamma = (float)gamma;
    dpd_lj = lj;
    dpd[i * ntypes + j] = dpd[j * ntypes + i] = p;
    params_dirty = true;
    }

// EvaluatorPairLJ::param_type(sigma, epsilon) at FP32 (hoomd/md/EvaluatorPairLJ.h:125-142)
void PairForce::set_params_lj(unsigned int i, unsigned int j, double sigma, double epsilon)
    {
    const float s = (float)sigma;
    gb_lj_param p;
    p.sigma_6 = s * s * s * s * s * s;
    p.epsilon_x_4 = 4.0f * (float)epsilon;
    lj[i * ntypes + j] = lj[j * ntypes + i] = p;
    params_dirty = true;
    }

void PairForce::set_params_example(unsigned int i, unsigned int j, double k, double sigma)
    {
    ex[i * ntypes + j] = ex[j * ntypes + i] = gb_example_param {(float)k, (float)sigma};
    params_dirty = true;
    }

void PairForce::set_params_radial(unsigned int i, unsigned int j, unsigned int kind,
                                  const std::vector<double>& v)
    {
    if (kind >= GB_RADIAL_KINDS)
        throw std::invalid_argument("unknown radial potential kind");
    if (v.size() > 6)
        throw std::invalid_argument("at most six parameters per type pair");
    gb_radial_param p {};
    for (size_t k = 0; k < v.size(); k++)
        p.v[k] = (float)v[k];
    p.kind = kind;
    rad[i * ntypes + j] = rad[j * ntypes + i] = p;
    params_dirty = true;
    }

void PairForce::set_params_table(unsigned int i, unsigned int j, double r_min,
                                 const std::vector<double>& U, const std::vector<double>& F)
    {
    if (U.size() != F.size())
        throw std::runtime_error("The length of V and F arrays must be equal.");
    if (U.empty())
        throw std::runtime_error("The length of V and F must not be zero.");
    for (auto idx : {i * ntypes + j, j * ntypes + i})
        {
        t_rmin[idx] = r_min;
        t_U[idx] = U;
        t_F[idx] = F;
        }
    params_dirty = true;
    }

// PotentialPair::setRCut / setROn (hoomd/md/PotentialPair.h:444-480): r^2 in Scalar.
void PairForce::set_r_cut(unsigned int i, unsigned int j, double r)
    {
    r_cut[i * ntypes + j] = r_cut[j * ntypes + i] = (float)r;
    params_dirty = true;
    nlist->dirty = true;
    }

void PairForce::set_r_on(unsigned int i, unsigned int j, double r)
    {
    r_on[i * ntypes + j] = r_on[j * ntypes + i] = (float)r;
    params_dirty = true;
    }

void PairForce::upload()
    {
    if (!params_dirty)
        return;
    cudaStream_t s = pdata->stream;
    const unsigned int np = ntypes * ntypes;
    std::vector<float> rc2(np), ro2(np);
    for (unsigned int k = 0; k < np; k++)
        {
        rc2[k] = r_cut[k] * r_cut[k];
        ro2[k] = r_on[k] * r_on[k];
        }
    d_rcutsq.resize(np);
    d_rcutsq.upload(rc2.data(), np, s);
    d_ronsq.resize(np);
    d_ronsq.upload(ro2.data(), np, s);
    if (kind == PairKind::LJ)
        {
        d_params.resize(np * sizeof(gb_lj_param));
        cuda_check(cudaMemcpyAsync(d_params.get(), lj.data(), np * sizeof(gb_lj_param),
                                   cudaMemcpyHostToDevice, s),
                   "params");
        }
    else if (kind == PairKind::Radial)
        {
        d_params.resize(np * sizeof(gb_radial_param));
        cuda_check(cudaMemcpyAsync(d_params.get(), rad.data(), np * sizeof(gb_radial_param),
                                   cudaMemcpyHostToDevice, s),
                   "params");
        }
    else if (kind == PairKind::DPD)
        {
        d_params.resize(np * sizeof(gb_dpd_param));
        cuda_check(cudaMemcpyAsync(d_params.get(), dpd.data(), np * sizeof(gb_dpd_param),
                                   cudaMemcpyHostToDevice, s),
                   "params");
        }
    else if (kind == PairKind::Plugin)
        {
        d_params.resize(std::max<size_t>(1, plugin_params.size()));
        cuda_check(cudaMemcpyAsync(d_params.get(), plugin_params.data(), plugin_params.size(),
                                   cudaMemcpyHostToDevice, s),
                   "params");
        }
    else if (kind == PairKind::Example)
        {
        d_params.resize(np * sizeof(gb_example_param));
        cuda_check(cudaMemcpyAsync(d_params.get(), ex.data(), np * sizeof(gb_example_param),
                                   cudaMemcpyHostToDevice, s),
                   "params");
        }
    else if (kind == PairKind::Table)
        {
        std::vector<gb_table_param> tp(np);
        std::vector<float> data;
        std::map<std::pair<unsigned, unsigned>, uint32_t> seen;
        for (unsigned int i = 0; i < ntypes; i++)
            for (unsigned int j = 0; j < ntypes; j++)
                {
                const unsigned int a = std::min(i, j), b = std::max(i, j);
                const unsigned int idx = i * ntypes + j;
                auto it = seen.find({a, b});
                uint32_t off;
                if (it == seen.end())
                    {
                    // packed bins (V[k], F[k], V[k+1], F[k+1]); offsets count quads
                    off = (uint32_t)(data.size() / 4);
                    const uint32_t w = (uint32_t)t_U[idx].size();
                    std::vector<float> q(4 * (size_t)w);
                    check(gb_table_pack(t_U[idx].data(), t_F[idx].data(), w, q.data()),
                          "gb_table_pack");
                    data.insert(data.end(), q.begin(), q.end());
                    seen[{a, b}] = off;
                    }
                else
                    off = it->second;
                tp[idx] = gb_table_param {(float)t_rmin[idx], (uint32_t)t_U[idx].size(), off, 0u};
                }
        d_params.resize(np * sizeof(gb_table_param));
        cuda_check(cudaMemcpyAsync(d_params.get(), tp.data(), np * sizeof(gb_table_param),
                                   cudaMemcpyHostToDevice, s),
                   "params");
        d_table.resize(data.size());
        d_table.upload(data.data(), data.size(), s);
        }
    cuda_check(cudaStreamSynchronize(s), "pair upload");
    params_dirty = false;
    }

gb_pair_args PairForce::pair_args(bool with_virial)
    {
    ParticleData& pd = *pdata;
    NeighborList& nl = *nlist;
    gb_pair_args a {};
    a.d_force = force.get();
    if (with_virial)
        {
        virial.resize(6 * (size_t)std::max(1u, pd.N));
        a.d_virial = virial.get();
        a.virial_pitch = pd.N;
        }
    a.N = pd.N;
    a.d_pos = pd.pos.get();
    a.box = pd.box;
    a.d_n_neigh = nl.n_neigh.get();
    a.d_nlist = nl.nlist.get();
    a.d_head_list = nullptr;
    a.stride = nl.stride;
    a.interleave = 4;
    a.d_rcutsq = d_rcutsq.get();
    a.d_ronsq = d_ronsq.get();
    a.ntypes = ntypes;
    a.shift_mode = (unsigned int)shift_mode;
    a.compute_virial = with_virial ? 1 : 0;
    a.block_size = kp_block;
    a.threads_per_particle = kp_tpp;
    if (uses_charge)
        {
        if (pd.charge.size() != pd.N)
            throw std::runtime_error("pair force needs particle charges, which are not set");
        a.d_charge = pd.charge.get();
        }
    return a;
    }

void PairForce::compute(cudaStream_t s, bool with_virial)
    {
    upload();
    if (kind == PairKind::MLP)
        {
        if (!mlp)
            throw std::runtime_error("the surrogate pair force has no network");
        if (with_virial)
            throw std::runtime_error("the surrogate pair force does not compute virials");
        if (mlp->ntypes != ntypes)
            throw std::runtime_error("the surrogate was built for another number of types");
        ParticleData& pd = *pdata;
        NeighborList& nl = *nlist;
        const unsigned int nmax = *std::max_element(nl.Nmax.begin(), nl.Nmax.end());
        mlp_scratch.resize(gb_mlp_forces_scratch_bytes(pd.N, nmax));
        gb_mlp_force_args m {};
        m.d_force = force.get();
        m.d_pos = pd.pos.get();
        m.N = pd.N;
        m.box = pd.box;
        m.d_n_neigh = nl.n_neigh.get();
        m.d_nlist = nl.nlist.get();
        m.stride = nl.stride;
        m.Nmax = nmax;
        m.ntypes = ntypes;
        m.r_min = mlp->r_min;
        m.r_cut = mlp->r_cut;
        m.act_split = mlp->act_split;
        m.d_infer = mlp->infer_block();
        m.d_scratch = mlp_scratch.get();
        m.mma_sync = mlp->mma_sync;
        check(gb_mlp_forces(&m, s), "gb_mlp_forces");
        virial_valid = false;
        return;
        }
    gb_pair_args a = pair_args(with_virial);
    int rc;
    if (kind == PairKind::Plugin)
        {
        gb_pair_plugin_call c {};
        c.op = 0;
        c.args = &a;
        c.stream = s;
        rc = plugin_call(c);
        }
    else if (kind == PairKind::LJ)
        rc = gb_pair_forces_lj(&a, (const gb_lj_param*)d_params.get(), s);
    else if (kind == PairKind::Example)
        rc = gb_pair_forces_example(&a, (const gb_example_param*)d_params.get(), s);
    else if (kind == PairKind::Radial)
        rc = gb_pair_forces_radial(&a, (const gb_radial_param*)d_params.get(), s);
    else if (kind == PairKind::DPD)
        rc = gb_pair_forces_dpd(&a, (const gb_dpd_param*)d_params.get(), pdata->vel.get(),
                                pdata->tag.get(), dpd_lj ? 1 : 0, force_timestep, pdata->seed,
                                force_dt, (float)dpd_kT, s);
    else
        rc = gb_pair_forces_table(&a, (const gb_table_param*)d_params.get(), d_table.get(), s);
    check(rc, "pair force");
    virial_valid = with_virial;
    }

double PairForce::energy_between_sets(const std::vector<uint32_t>& tags1,
                                      const std::vector<uint32_t>& tags2)
    {
    if (kind == PairKind::MLP || kind == PairKind::DPD)
        throw std::runtime_error("compute_energy is not available for this pair force");
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    upload();
    nlist->ensure_consumer(&r_cut);
    nlist->build_sync();
    if (tags1.empty() || tags2.empty())
        return 0.0;
    const std::vector<uint32_t> rt = pd.rtag();
    // occurrences of each particle index's tag in the two sets (the reference's double loop
    // over the tag lists counts duplicates and overlaps)
    std::vector<uint32_t> mult((size_t)2 * pd.N, 0u);
    for (int which = 0; which < 2; which++)
        for (uint32_t t : (which == 0 ? tags1 : tags2))
            {
            if (t >= pd.N)
                throw std::invalid_argument("compute_energy: tag out of range");
            mult[(size_t)which * pd.N + rt[t]]++;
            }
    DeviceArray<uint32_t> d_mult;
    d_mult.resize(std::max<size_t>(2, mult.size()));
    d_mult.upload(mult.data(), mult.size(), s);
    nlist->refresh_exclusions();
    gb_energy_sets sets{};
    sets.d_mult1 = d_mult.get();
    sets.d_mult2 = d_mult.get() + pd.N;
    if (nlist->ex_pitch > 0)
        {
        sets.d_n_ex = nlist->n_ex.get();
        sets.d_ex_list = nlist->ex_list.get();
        sets.ex_pitch = nlist->ex_pitch;
        }
    const unsigned int nb = gb_pair_energy_sets_blocks(pd.N);
    DeviceArray<double> parts;
    parts.resize(nb);
    gb_pair_args a = pair_args(false);
    int rc;
    if (kind == PairKind::Plugin)
        {
        gb_pair_plugin_call c {};
        c.op = 2;
        c.args = &a;
        c.sets = &sets;
        c.d_partials = parts.get();
        c.stream = s;
        rc = plugin_call(c);
        }
    else if (kind == PairKind::LJ)
        rc = gb_pair_energy_sets_lj(&a, (const gb_lj_param*)d_params.get(), &sets, parts.get(),
                                    s);
    else if (kind == PairKind::Example)
        rc = gb_pair_energy_sets_example(&a, (const gb_example_param*)d_params.get(), &sets,
                                         parts.get(), s);
    else if (kind == PairKind::Radial)
        rc = gb_pair_energy_sets_radial(&a, (const gb_radial_param*)d_params.get(), &sets,
                                        parts.get(), s);
    else
        rc = gb_pair_energy_sets_table(&a, (const gb_table_param*)d_params.get(), d_table.get(),
                                       &sets, parts.get(), s);
    check(rc, "energy between sets");
    std::vector<double> h(nb);
    parts.download(h.data(), nb, s);
    cuda_check(cudaStreamSynchronize(s), "energy between sets");
    double u = 0.0;
    for (double v : h)
        u += v;
    return u;
    }

int PairForce::plugin_call(gb_pair_plugin_call& c)
    {
    if (!plugin || !plugin->call)
        return GB_ERR_INVALID;
    c.status = GB_OK;
    const int rc = plugin->call(&c, d_params.get());
    return rc != GB_OK ? rc : c.status;
    }

void PairForce::set_params_plugin(unsigned int i, unsigned int j, const void* record, size_t bytes)
    {
    if (kind != PairKind::Plugin || !plugin)
        throw std::logic_error("set_params_plugin: not a plugin pair force");
    if (bytes != plugin->param_size)
        throw std::invalid_argument("plugin parameter record has the wrong size");
    if (i >= ntypes || j >= ntypes)
        throw std::invalid_argument("type index out of range");
    const unsigned char* r = static_cast<const unsigned char*>(record);
    std::copy(r, r + bytes, plugin_params.begin() + (size_t)(i * ntypes + j) * bytes);
    std::copy(r, r + bytes, plugin_params.begin() + (size_t)(j * ntypes + i) * bytes);
    params_dirty = true;
    }

int PairForce::launch_fused(const gb_pair_args& a, const gb_step_fuse& f, cudaStream_t s)
    {
    if (kind == PairKind::Plugin)
        {
        gb_pair_plugin_call c {};
        c.op = 1;
        c.args = &a;
        c.fuse = &f;
        c.stream = s;
        return plugin_call(c);
        }
    if (kind == PairKind::LJ)
        return gb_md_pair_step_lj(&a, (const gb_lj_param*)d_params.get(), &f, s);
    if (kind == PairKind::Example)
        return gb_md_pair_step_example(&a, (const gb_example_param*)d_params.get(), &f, s);
    if (kind == PairKind::Radial)
        return gb_md_pair_step_radial(&a, (const gb_radial_param*)d_params.get(), &f, s);
    if (kind == PairKind::DPD || kind == PairKind::MLP)
        throw std::logic_error("this pair force has no fused step");
    return gb_md_pair_step_table(&a, (const gb_table_param*)d_params.get(), d_table.get(), &f, s);
    }

// ------------------------------------------------------------------------------------------------
// Integrator (IntegratorTwoStep + TwoStepConstantVolume + BussiThermostat + ComputeThermo)
// ------------------------------------------------------------------------------------------------
Integrator::Integrator(std::shared_ptr<ParticleData> pd, std::shared_ptr<NeighborList> nl,
                       double dt_)
    : pdata(std::move(pd)), nlist(std::move(nl)), dt(dt_)
    {
    d_status.resize(1);
    d_status.zero(pdata->stream);
    const uint64_t steps[2] = {~0ull, 100};
    cuda_check(cudaMemcpyAsync(d_status.get()->build_steps, steps, sizeof(steps),
                               cudaMemcpyHostToDevice, pdata->stream),
               "build statistics");
    cuda_check(cudaStreamSynchronize(pdata->stream), "build statistics");
    }

Integrator::~Integrator()
    {
    drop_graphs();
    if (body_stream)
        cudaStreamDestroy(body_stream);
    if (h_builds)
        cudaFreeHost(h_builds);
    }

void Integrator::add_force(std::shared_ptr<PairForce> f)
    {
    if (f->nlist != nlist)
        throw std::invalid_argument("all pair forces of one integrator must share its nlist");
    forces.push_back(std::move(f));
    prepared = false;
    drop_graphs();
    }

void Integrator::set_thermostat_bussi(double kT_, double tau_)
    {
    bussi = true;
    berendsen = mttk = langevin = false;
    kT = kT_;
    tau = tau_;
    prepared = false;
    drop_graphs();
    }

void Integrator::set_thermostat_none()
    {
    bussi = false;
    berendsen = mttk = false;
    langevin = false;
    brownian = false;
    prepared = false;
    drop_graphs();
    }

void Integrator::set_langevin(double kT_, const std::vector<double>& gamma_, bool tally_)
    {
    if (gamma_.size() != pdata->ntypes)
        throw std::invalid_argument("Langevin: one drag coefficient per particle type");
    bussi = false;
    berendsen = mttk = false;
    brownian = false;
    langevin = true;
    tally = tally_;
    langevin_kT = kT_;
    gamma.assign(gamma_.begin(), gamma_.end());
    d_gamma.resize(gamma.size());
    cuda_check(cudaMemcpy(d_gamma.get(), gamma.data(), sizeof(float) * gamma.size(),
                          cudaMemcpyHostToDevice),
               "gamma");
    prepared = false;
    drop_graphs();
    }

void Integrator::set_thermostat_berendsen(double kT_, double tau_)
    {
    if (!(tau_ > 0.0))
        throw std::invalid_argument("Berendsen: tau must be positive");
    berendsen = true;
    bussi = mttk = langevin = false;
    kT = kT_;
    tau = tau_;
    prepared = false;
    drop_graphs();
    }

void Integrator::set_thermostat_mttk(double kT_, double tau_)
    {
    if (!(tau_ > 0.0))
        throw std::invalid_argument("MTTK: tau must be positive");
    mttk = true;
    bussi = berendsen = langevin = false;
    kT = kT_;
    tau = tau_;
    prepared = false;
    drop_graphs();
    }

std::vector<double> Integrator::mttk_state()
    {
    if (prepared)
        {
        DevStatus st = read_status();
        mttk_host[0] = st.mttk[0];
        mttk_host[1] = st.mttk[1];
        }
    return {mttk_host[0], mttk_host[1]};
    }

void Integrator::set_mttk_state(double xi, double eta)
    {
    mttk_host[0] = xi;
    mttk_host[1] = eta;
    if (prepared)
        {
        double v[2] = {xi, eta};
        cuda_check(cudaMemcpyAsync(d_status.get()->mttk, v, sizeof(v), cudaMemcpyHostToDevice,
                                   pdata->stream),
                   "mttk state");
        cuda_check(cudaStreamSynchronize(pdata->stream), "mttk state");
        }
    }

void Integrator::thermalize_mttk(uint64_t timestep)
    {
    // xi ~ Normal(sqrt(1 / (dof tau^2))), Seed(28, timestep, seed), Counter(first tag = 0)
    DeviceArray<double> out;
    out.resize(1);
    const double sigma = std::sqrt(1.0 / (dof() * tau * tau));
    check(gb_normal_draw(28, timestep, pdata->seed, 0u, sigma, out.get(), pdata->stream),
          "gb_normal_draw");
    double xi = 0.0;
    out.download(&xi, 1, pdata->stream);
    cuda_check(cudaStreamSynchronize(pdata->stream), "thermalize");
    const std::vector<double> cur = mttk_state();
    set_mttk_state(xi, cur[1]);
    }

double Integrator::mttk_energy()
    {
    const std::vector<double> st = mttk_state();
    return dof() * kT * (st[0] * st[0] * tau * tau / 2.0 + st[1]);
    }

void Integrator::set_brownian(double kT_, const std::vector<double>& gamma_, bool noiseless)
    {
    if (gamma_.size() != pdata->ntypes)
        throw std::invalid_argument("Brownian: one drag coefficient per particle type");
    for (double g : gamma_)
        if (!(g > 0.0))
            throw std::invalid_argument("Brownian: drag coefficients must be positive");
    bussi = berendsen = mttk = langevin = false;
    brownian = true;
    bd_noiseless = noiseless;
    bd_kT = kT_;
    gamma.assign(gamma_.begin(), gamma_.end());
    d_gamma.resize(gamma.size());
    cuda_check(cudaMemcpy(d_gamma.get(), gamma.data(), sizeof(float) * gamma.size(),
                          cudaMemcpyHostToDevice),
               "gamma");
    prepared = false;
    drop_graphs();
    }

void Integrator::set_max_displacement(double d)
    {
    max_disp = d > 0.0 ? d : 0.0;
    drop_graphs();
    }

double Integrator::reservoir_energy()
    {
    if (!prepared)
        return reservoir;
    return read_status().reservoir;
    }

// Bussi draws for the next k timesteps, in parallel, ahead of a run of fused steps.
static void enqueue_bussi_draws(const Integrator& in, DevStatus* ds, double* ring,
                                unsigned int ring_size, unsigned int k, cudaStream_t s)
    {
    check(gb_bussi_draws(&ds->timestep, k, in.dof(), in.pdata->seed, 0u, ring, ring_size, s),
          "gb_bussi_draws");
    }

void Integrator::set_sorter(uint64_t period, int bits)
    {
    sort_period = period;
    sort_bits = bits;
    }

// IntegratorTwoStep::getTranslationalDOF for one momentum-conserving method on all particles
// (hoomd/md/IntegratorTwoStep.cc:154-199): D*N - D.
double Integrator::dof() const
    {
    // Langevin and Brownian dynamics do not conserve momentum
    // (TwoStepLangevinBase::isMomentumConserving): D*N
    if (langevin || brownian)
        return double(pdata->ndim) * pdata->N;
    return double(pdata->ndim) * pdata->N - double(pdata->ndim);
    }

DevStatus Integrator::read_status()
    {
    DevStatus st;
    cuda_check(cudaMemcpyAsync(&st, d_status.get(), sizeof(DevStatus), cudaMemcpyDeviceToHost,
                               pdata->stream),
               "read status");
    cuda_check(cudaStreamSynchronize(pdata->stream), "read status");
    return st;
    }

void Integrator::drop_graphs()
    {
    for (auto& kv : graphs)
        cudaGraphExecDestroy(kv.second);
    graphs.clear();
    }

// IntegratorTwoStep::prepRun (hoomd/md/IntegratorTwoStep.cc:226-298)
void Integrator::prepare(bool keep_graphs)
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    if (forces.empty())
        throw std::runtime_error("integrator has no forces");
    if (pd.N == 0)
        throw std::runtime_error("Empty integration group.");
    nlist->clear_consumers();
    for (auto& f : forces)
        nlist->add_consumer(&f->r_cut);
    // the build statistics and the check schedule carry over from the last run unless the list
    // must be rebuilt anyway (first run, new r_cut or capacities: the reference's forced update
    // at this step, which the build count leaves out)
    const bool forced = nlist->dirty || !nlist->allocated;
    const DevStatus old = read_status();
    nlist->build_sync();
    if (!keep_graphs)
        drop_graphs();
    for (auto& f : forces)
        {
        f->force_timestep = pd.timestep;
        f->force_dt = (float)dt;
        f->compute(s, compute_virial);
        }
    const float* net = forces[0]->force.get();
    if (forces.size() > 1)
        {
        net_force.resize(4 * (size_t)pd.N);
        std::vector<const float*> ptrs;
        for (auto& f : forces)
            ptrs.push_back(f->force.get());
        check(gb_sum_net_force(net_force.get(), ptrs.data(), (unsigned)ptrs.size(), pd.N, s),
              "gb_sum_net_force");
        net = net_force.get();
        }
    if (!pd.accel_set)
        {
        // Integrator::computeAccelerations: a = F/m (a half step with dt = 0 leaves v as is)
        check(gb_cv_step_two(pd.vel.get(), pd.accel.get(), net, pd.N, 0.0f, 1.0f, nullptr, s),
              "accelerations");
        pd.accel_set = true;
        }
    d_thermo_scratch.resize(gb_thermo_scratch_bytes(pd.N));
    d_thermo_scratch.zero(s);
    d_step_scratch.resize(gb_md_step_scratch_bytes(pd.N));
    d_step_scratch.zero(s);
    d_bussi_ring.resize(2 * (size_t)BUSSI_RING);
    DevStatus st {};
    st.timestep = pd.timestep;
    st.n_builds = old.n_builds;
    st.build_steps[0] = (forced || old.build_steps[0] == ~0ull) ? pd.timestep : old.build_steps[0];
    st.build_steps[1] = old.build_steps[1];
    st.n_dangerous = old.n_dangerous;
    st.factor = 1.0;
    st.reservoir = reservoir;
    st.mttk[0] = mttk_host[0];
    st.mttk[1] = mttk_host[1];
    st.mttk_scale2 = 1.0;
    cuda_check(cudaMemcpyAsync(d_status.get(), &st, sizeof(st), cudaMemcpyHostToDevice, s),
               "status");
    DevStatus* ds = d_status.get();
    check(gb_thermo_reduce(pd.vel.get(), net, nullptr, 0, pd.N, d_thermo_scratch.get(),
                           ds->thermo, s),
          "thermo");
    if (bussi)
        check(gb_bussi_factor(&ds->thermo[0], dof(), dt, tau, kT, pd.timestep, pd.seed, 0u,
                              &ds->factor, s),
              "bussi");
    if (berendsen)
        check(gb_berendsen_factor(&ds->thermo[0], dof(), dt, tau, kT, &ds->factor, &ds->status,
                                  s),
              "berendsen");
    DevStatus back = read_status();
    if (bussi && dof() != 0 && back.thermo[0] == 0.0)
        throw std::runtime_error("Bussi thermostat requires non-zero initial momenta.");
    if (berendsen && (back.status & 2u))
        throw std::runtime_error("Berendsen thermostat requires non-zero initial temperatures");
    prepared = true;
    }

// Arguments of step one (with the rebuild check) for the current method.
gb_step_one_args Integrator::step_one_args(DevStatus* ds) const
    {
    ParticleData& pd = *pdata;
    gb_step_one_args o {};
    o.d_pos = pd.pos.get();
    o.d_vel = pd.vel.get();
    o.d_accel = pd.accel.get();
    o.d_image = pd.image.get();
    o.N = pd.N;
    o.box = pd.box;
    o.dt = (float)dt;
    o.scale = 1.0f;
    o.d_scale = (bussi || berendsen) ? &ds->factor : nullptr;
    o.d_last_pos = nlist->last_pos.get();
    o.d_rcut_max = nlist->d_rcut_max.get();
    o.r_buff = nlist->r_buff;
    o.d_rebuild = &ds->rebuild;
    if (nlist->rebuild_check_delay != 1 || !nlist->check_dist)
        {
        o.d_check_step = &ds->timestep;
        o.d_last_update = &ds->build_steps[0];
        o.check_delay = nlist->rebuild_check_delay;
        o.check_dist = nlist->check_dist ? 1 : 0;
        }
    o.nve_order = langevin ? 1 : 0;
    o.max_displacement = (float)max_disp;
    if (brownian)
        {
        o.brownian = 1;
        o.d_scale = nullptr;
        o.d_bd_force = forces.size() > 1 ? net_force.get() : forces[0]->force.get();
        o.d_tag = pd.tag.get();
        o.d_gamma = d_gamma.get();
        o.bd_kT = (float)bd_kT;
        o.ndim = pd.ndim;
        o.seed = pd.seed;
        o.d_timestep = &ds->timestep;
        o.noiseless = bd_noiseless ? 1 : 0;
        }
    if (mttk)
        {
        o.d_mttk_state = ds->mttk;
        o.d_mttk_scale2 = &ds->mttk_scale2;
        o.mttk_dof = dof();
        o.mttk_kT = kT;
        o.mttk_tau = tau;
        o.d_mttk_scratch = d_thermo_scratch.get();
        }
    return o;
    }

// Arguments of the fused pair kernel's step two for the current method.
gb_step_fuse Integrator::fuse_args(DevStatus* ds) const
    {
    ParticleData& pd = *pdata;
    gb_step_fuse fu {};
    fu.d_vel = pd.vel.get();
    fu.d_accel = pd.accel.get();
    fu.dt = (float)dt;
    fu.d_scale2 = mttk ? &ds->mttk_scale2 : nullptr;
    fu.berendsen = berendsen ? 1 : 0;
    fu.brownian = brownian ? 1 : 0;
    fu.d_scratch = d_step_scratch.get();
    fu.d_thermo = ds->thermo;
    fu.bussi = bussi ? 1 : 0;
    fu.dof = dof();
    fu.tau = tau;
    fu.kT = kT;
    fu.seed = pd.seed;
    fu.instance_id = 0;
    fu.d_timestep = &ds->timestep;
    fu.d_factor = &ds->factor;
    fu.d_status = &ds->status;
    fu.d_rebuild_reset = &ds->rebuild;
    if (bussi)
        {
        fu.d_bussi_ring = d_bussi_ring.get();
        fu.bussi_ring_size = BUSSI_RING;
        }
    if (langevin)
        {
        fu.langevin = 1;
        fu.d_tag = pd.tag.get();
        fu.d_pos = pd.pos.get();
        fu.d_gamma = d_gamma.get();
        fu.langevin_kT = (float)langevin_kT;
        fu.ndim = pd.ndim;
        fu.d_reservoir = tally ? &ds->reservoir : nullptr;
        }
    return fu;
    }

void Integrator::enqueue_step_fused(cudaStream_t s)
    {
    ParticleData& pd = *pdata;
    DevStatus* ds = d_status.get();
    // step one also zeroes the cell counts, so the build's gated launches are two, not three
    gb_step_one_args o = step_one_args(ds);
    o.d_zero_words = nlist->cell_size.get();
    o.n_zero_words = (uint32_t)nlist->cell_size.size();
    check(gb_md_step_one(&o, s), "gb_md_step_one");
    nlist->enqueue_build(&ds->rebuild, &ds->n_builds, ds->cell_cond, ds->nl_cond, s, &ds->timestep,
                         ds->build_steps, &ds->n_dangerous, true);
    PairForce& f = *forces[0];
    gb_pair_args a = f.pair_args(false);
    const gb_step_fuse fu = fuse_args(ds);
    check(f.launch_fused(a, fu, s), "fused pair step");
    }

// One fused step inside a graph capture on stream s, its neighbour-list build in the body of an
// IF conditional node whose value the step's rebuild flag sets (gb_graph_set_conditional).
void Integrator::capture_step_conditional(cudaStream_t s, unsigned long long handle)
    {
    DevStatus* ds = d_status.get();
    const gb_step_one_args o = step_one_args(ds);
    check(gb_md_step_one(&o, s), "gb_md_step_one");
    check(gb_graph_set_conditional(handle, &ds->rebuild, s), "gb_graph_set_conditional");
    cudaStreamCaptureStatus st;
    cudaGraph_t cap = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cuda_check(cudaStreamGetCaptureInfo(s, &st, nullptr, &cap, &deps, nullptr, &ndeps),
               "capture info");
    cudaGraphNodeParams p {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = (cudaGraphConditionalHandle)handle;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    cuda_check(cudaGraphAddNode(&node, cap, deps, nullptr, ndeps, &p), "conditional node");
    cuda_check(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                   cudaStreamSetCaptureDependencies),
               "capture dependencies");
    if (!body_stream)
        cuda_check(cudaStreamCreateWithFlags(&body_stream, cudaStreamNonBlocking), "stream");
    cudaGraph_t body = p.conditional.phGraph_out[0];
    cuda_check(cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal),
               "body capture");
    try
        {
        nlist->enqueue_build(&ds->rebuild, &ds->n_builds, ds->cell_cond, ds->nl_cond,
                             body_stream, &ds->timestep, ds->build_steps, &ds->n_dangerous);
        }
    catch (...)
        {
        cudaStreamEndCapture(body_stream, &body);
        throw;
        }
    cuda_check(cudaStreamEndCapture(body_stream, &body), "body capture end");
    PairForce& f = *forces[0];
    gb_pair_args a = f.pair_args(false);
    const gb_step_fuse fu = fuse_args(ds);
    check(f.launch_fused(a, fu, s), "fused pair step");
    }

void Integrator::enqueue_step_general(cudaStream_t s, uint64_t step)
    {
    ParticleData& pd = *pdata;
    DevStatus* ds = d_status.get();
    gb_step_one_args o = step_one_args(ds);
    if (brownian)
        {
        // the device step counter advances only on the fused path; here the host knows it
        o.d_timestep = nullptr;
        o.timestep = step;
        }
    check(gb_md_step_one(&o, s), "gb_md_step_one");
    nlist->enqueue_build(&ds->rebuild, &ds->n_builds, ds->cell_cond, ds->nl_cond, s, &ds->timestep,
                         ds->build_steps, &ds->n_dangerous);
    for (auto& f : forces)
        {
        // IntegratorTwoStep::update computes the net force for timestep + 1
        f->force_timestep = step + 1;
        f->force_dt = (float)dt;
        f->compute(s, compute_virial);
        }
    const float* net = forces[0]->force.get();
    if (forces.size() > 1)
        {
        std::vector<const float*> ptrs;
        for (auto& f : forces)
            ptrs.push_back(f->force.get());
        check(gb_sum_net_force(net_force.get(), ptrs.data(), (unsigned)ptrs.size(), pd.N, s),
              "gb_sum_net_force");
        net = net_force.get();
        }
    if (langevin)
        {
        check(gb_langevin_step_two(pd.vel.get(), pd.accel.get(), net, pd.pos.get(), pd.tag.get(),
                                   d_gamma.get(), pd.N, (float)dt, (float)langevin_kT, pd.ndim,
                                   pd.seed, &ds->timestep, d_step_scratch.get(), ds->thermo,
                                   tally ? &ds->reservoir : nullptr, s),
              "gb_langevin_step_two");
        }
    else if (brownian)
        {
        // TwoStepBD has no second half; the sums only
        check(gb_thermo_reduce(pd.vel.get(), net, nullptr, 0, pd.N, d_thermo_scratch.get(),
                               ds->thermo, s),
              "thermo");
        }
    else
        {
        check(gb_cv_step_two(pd.vel.get(), pd.accel.get(), net, pd.N, (float)dt, 1.0f,
                             mttk ? &ds->mttk_scale2 : nullptr, s),
              "gb_cv_step_two");
        check(gb_thermo_reduce(pd.vel.get(), net, nullptr, 0, pd.N, d_thermo_scratch.get(),
                               ds->thermo, s),
              "thermo");
        }
    if (!langevin) // the Langevin step two advances the counter itself
        check(gb_step_counter_advance(&ds->timestep, s), "step counter");
    if (bussi)
        check(gb_bussi_factor(&ds->thermo[0], dof(), dt, tau, kT, step + 1, pd.seed, 0u,
                              &ds->factor, s),
              "bussi");
    if (berendsen)
        check(gb_berendsen_factor(&ds->thermo[0], dof(), dt, tau, kT, &ds->factor, &ds->status,
                                  s),
              "berendsen");
    cuda_check(cudaMemsetAsync(&ds->rebuild, 0, sizeof(uint32_t), s), "reset rebuild");
    }

cudaGraphExec_t Integrator::graph_for(unsigned int k)
    {
    // a neighbour list regrown or reallocated outside run_chunk (a forced build, a build for a
    // query) moved the buffers the captured graphs address
    if (nlist->alloc_generation != graph_nlist_generation)
        {
        drop_graphs();
        graph_nlist_generation = nlist->alloc_generation;
        }
    auto it = graphs.find(k);
    if (it != graphs.end())
        return it->second;
    cudaStream_t s = pdata->stream;
    cudaGraph_t g;
    if (k > BUSSI_RING)
        throw std::runtime_error("chunk longer than the Bussi draw ring");
    // with conditional nodes, a step's build runs only when its rebuild check fired (the gated
    // build kernels otherwise cost a wave of empty blocks each, every step); each step's node has
    // a handle of its own (a handle belongs to one conditional node). A runtime that refuses
    // any part of it gets the gated capture instead.
    auto capture = [&](bool conditional) {
        cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
        try
            {
            if (bussi)
                enqueue_bussi_draws(*this, d_status.get(), d_bussi_ring.get(), BUSSI_RING, k, s);
            std::vector<cudaGraphConditionalHandle> handles(conditional ? k : 0);
            if (conditional)
                {
                cudaStreamCaptureStatus st;
                cudaGraph_t cap = nullptr;
                cuda_check(cudaStreamGetCaptureInfo(s, &st, nullptr, &cap, nullptr, nullptr,
                                                    nullptr),
                           "capture info");
                for (unsigned int i = 0; i < k; i++)
                    cuda_check(cudaGraphConditionalHandleCreate(&handles[i], cap, 0, 0),
                               "conditional handle");
                }
            for (unsigned int i = 0; i < k; i++)
                {
                if (conditional)
                    capture_step_conditional(s, handles[i]);
                else
                    enqueue_step_fused(s);
                }
            }
        catch (...)
            {
            g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g)
                cudaGraphDestroy(g);
            throw;
            }
        cuda_check(cudaStreamEndCapture(s, &g), "end capture");
        cudaGraphExec_t e;
        const cudaError_t err = cudaGraphInstantiate(&e, g, 0);
        cudaGraphDestroy(g);
        cuda_check(err, "graph instantiate");
        return e;
    };
    cudaGraphExec_t exec = nullptr;
    if (use_conditional_build)
        {
        try
            {
            exec = capture(true);
            }
        catch (const std::exception&)
            {
            cudaGetLastError();
            use_conditional_build = false;
            }
        }
    if (!exec)
        exec = capture(false);
    graphs[k] = exec;
    return exec;
    }

void Integrator::checkpoint()
    {
    cudaStream_t s = pdata->stream;
    ck_pos.copy_from(pdata->pos, s);
    ck_vel.copy_from(pdata->vel, s);
    ck_accel.copy_from(pdata->accel, s);
    ck_image.copy_from(pdata->image, s);
    ck_status.copy_from(d_status, s);
    }

void Integrator::restore()
    {
    cudaStream_t s = pdata->stream;
    pdata->pos.copy_from(ck_pos, s);
    pdata->vel.copy_from(ck_vel, s);
    pdata->accel.copy_from(ck_accel, s);
    pdata->image.copy_from(ck_image, s);
    d_status.copy_from(ck_status, s);
    }

void Integrator::run_chunk(unsigned int k)
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    const bool fused = forces.size() == 1 && !compute_virial && forces[0]->kind != PairKind::MLP
                       && forces[0]->kind != PairKind::DPD;
    for (int attempt = 0; attempt < 16; attempt++)
        {
        checkpoint();
        DevStatus* ds = d_status.get();
        cuda_check(cudaMemsetAsync(ds->cell_cond, 0, sizeof(ds->cell_cond), s), "zero cond");
        cuda_check(cudaMemsetAsync(ds->nl_cond, 0, sizeof(ds->nl_cond), s), "zero cond");
        cuda_check(cudaMemsetAsync(&ds->status, 0, sizeof(uint32_t), s), "zero status");
        const uint64_t cell_kernels = (nlist->deterministic ? 3 : 2) + (nlist->ex_pitch ? 1 : 0);
        bool conditional = false;
        if (fused && use_graph)
            {
            cudaGraphExec_t exec = graph_for(k);
            conditional = use_conditional_build;
            if (conditional)
                {
                if (!h_builds)
                    cuda_check(cudaHostAlloc((void**)&h_builds, sizeof(uint64_t), 0), "host alloc");
                cuda_check(cudaMemcpyAsync(h_builds, &ds->n_builds, sizeof(uint64_t),
                                           cudaMemcpyDeviceToHost, s),
                           "build count");
                }
            cuda_check(cudaGraphLaunch(exec, s), "graph launch");
            // conditional graphs: step one, the conditional's value and the pair step each step;
            // the build kernels are added below for the builds that ran
            launch_count += conditional
                                ? (uint64_t)k * 3 + (bussi ? 1 : 0)
                                : (uint64_t)k * (1 + cell_kernels + 1 + 1) + (bussi ? 1 : 0);
            }
        else if (fused)
            {
            if (bussi)
                enqueue_bussi_draws(*this, ds, d_bussi_ring.get(), BUSSI_RING, k, s);
            for (unsigned int i = 0; i < k; i++)
                enqueue_step_fused(s);
            launch_count += (uint64_t)k * (1 + cell_kernels + 1 + 1) + (bussi ? 1 : 0);
            }
        else
            {
            if (forces.size() > 1)
                net_force.resize(4 * (size_t)pd.N);
            for (unsigned int i = 0; i < k; i++)
                enqueue_step_general(s, pd.timestep + i);
            launch_count += (uint64_t)k
                            * (1 + cell_kernels + 1 + forces.size() + (forces.size() > 1 ? 1 : 0)
                               + (langevin ? 1 : (brownian ? 2 : 3))
                               + ((bussi || berendsen) ? 1 : 0));
            }
        DevStatus st = read_status();
        if (st.n_dangerous > dangerous_seen && notice_level >= 2)
            {
            // NeighborList::needsUpdating's notice (hoomd/md/NeighborList.cc:1405-1414)
            std::cerr << "notice(2): nlist: " << (st.n_dangerous - dangerous_seen)
                      << " dangerous neighbor list build(s): the first check after "
                         "rebuild_check_delay steps found the list stale. Continuing this "
                         "simulation may produce incorrect results; decrease "
                         "rebuild_check_delay and rerun."
                      << std::endl;
            }
        dangerous_seen = st.n_dangerous;
        if (conditional)
            launch_count += (st.n_builds - *h_builds) * (cell_kernels + 1);
        if (st.cell_cond[1])
            throw std::runtime_error(tag_message(pd, st.cell_cond[1], "has NaN for its position."));
        if (st.cell_cond[2])
            throw std::runtime_error(
                tag_message(pd, st.cell_cond[2], "is no longer in the simulation box."));
        bool overflow = st.cell_cond[0] > nlist->Nmax_cell;
        for (unsigned int t = 0; t < pd.ntypes; t++)
            overflow = overflow || st.nl_cond[t] > nlist->Nmax[t];
        if (overflow)
            {
            restore();
            nlist->grow(st);
            drop_graphs();
            nlist->build_sync();
            n_rollbacks++;
            continue;
            }
        if (st.status & 1u)
            throw std::runtime_error("Bussi thermostat requires non-zero initial momenta.");
        if (st.status & 2u)
            throw std::runtime_error("Berendsen thermostat requires non-zero initial temperatures");
        reservoir = st.reservoir;
        mttk_host[0] = st.mttk[0];
        mttk_host[1] = st.mttk[1];
        pd.timestep += k;
        steps_run += k;
        if (!fused)
            {
            uint64_t ts = pd.timestep;
            cuda_check(cudaMemcpyAsync(&ds->timestep, &ts, sizeof(ts), cudaMemcpyHostToDevice, s),
                       "timestep");
            cuda_check(cudaStreamSynchronize(s), "timestep");
            }
        return;
        }
    throw std::runtime_error("run: repeated neighbour-list overflow");
    }

// SFCPackTuner::update (hoomd/SFCPackTuner.cc:81-118): order, gather every per-particle array,
// then force a neighbour-list rebuild (the reference's notifyParticleSort).
void Integrator::sort_particles()
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    const size_t need = gb_sfc_scratch_bytes_dim(pd.N, sort_bits, pd.ndim == 2 ? 2 : 3);
    if (pd.scratch.size() < need + 4 * (size_t)pd.N + 256)
        {
        pd.scratch.resize(need + 4 * (size_t)pd.N + 256);
        pd.scratch.zero(s);
        }
    uint32_t* order = reinterpret_cast<uint32_t*>(pd.scratch.get() + need);
    check(gb_sfc_order_dim(pd.pos.get(), pd.N, &pd.box, sort_bits, pd.ndim == 2 ? 2 : 3, order,
                           pd.scratch.get(), need, s),
          "gb_sfc_order");
    pd.alt.resize(4 * (size_t)pd.N);
    auto apply = [&](void* arr, unsigned int bytes) {
        check(gb_gather(pd.alt.get(), arr, order, pd.N, bytes, s), "gb_gather");
        cuda_check(cudaMemcpyAsync(arr, pd.alt.get(), (size_t)bytes * pd.N,
                                   cudaMemcpyDeviceToDevice, s),
                   "sort copy");
    };
    apply(pd.pos.get(), 16);
    apply(pd.vel.get(), 16);
    apply(pd.accel.get(), 12);
    apply(pd.image.get(), 12);
    apply(pd.tag.get(), 4);
    if (pd.charge.size() == pd.N)
        apply(pd.charge.get(), 4);
    for (auto& f : forces)
        {
        apply(f->force.get(), 16);
        f->virial_valid = false;
        }
    // Brownian step one reads the summed force of the last step
    if (net_force.size() == 4 * (size_t)pd.N)
        apply(net_force.get(), 16);
    // the old scratch counter words may have been overwritten: re-zero the thermo scratch
    pd.scratch.zero(s);
    pd.sort_generation++;
    nlist->build_sync();
    // a forced update (not counted in num_builds): the reference makes it at the next step's
    // force computation, the step the check schedule and the build periods count from
    DevStatus* ds = d_status.get();
    const uint64_t upd = pd.timestep + 1;
    cuda_check(cudaMemcpyAsync(&ds->build_steps[0], &upd, sizeof(upd), cudaMemcpyHostToDevice, s),
               "last update");
    cuda_check(cudaStreamSynchronize(s), "sort");
    }

// System::run's resetStats (hoomd/System.cc:90, hoomd/md/NeighborList.cc:1420-1426): builds,
// dangerous builds and the smallest period count from the start of each run
void Integrator::reset_build_stats()
    {
    const uint64_t period = 100;
    DevStatus* ds = d_status.get();
    cuda_check(cudaMemcpyAsync(&ds->build_steps[1], &period, sizeof(period),
                               cudaMemcpyHostToDevice, pdata->stream),
               "build statistics");
    cuda_check(cudaMemsetAsync(&ds->n_builds, 0, sizeof(uint64_t), pdata->stream),
               "build statistics");
    cuda_check(cudaMemsetAsync(&ds->n_dangerous, 0, sizeof(uint64_t), pdata->stream),
               "build statistics");
    dangerous_seen = 0;
    cuda_check(cudaStreamSynchronize(pdata->stream), "build statistics");
    }

void Integrator::run(uint64_t nsteps)
    {
    ParticleData& pd = *pdata;
    if (!prepared || nlist->dirty)
        prepare();
    for (auto& f : forces)
        if (f->params_dirty)
            {
            f->upload();
            drop_graphs();
            }
    bool tune = nlist->tune_requested;
    for (auto& f : forces)
        tune = tune || f->tune_requested;
    if (tune && !npt)
        last_tuning = autotune();
    if (npt)
        {
        run_npt(nsteps);
        return;
        }
    uint64_t done = 0;
    while (done < nsteps)
        {
        if (sort_period && pd.timestep % sort_period == 0)
            sort_particles();
        uint64_t k = std::min<uint64_t>(nsteps - done, chunk);
        if (sort_period)
            {
            const uint64_t to_sort = sort_period - (pd.timestep % sort_period);
            k = std::min(k, to_sort);
            }
        run_chunk((unsigned int)k);
        done += k;
        }
    }

double Integrator::sum_n_neigh()
    {
    ParticleData& pd = *pdata;
    std::vector<uint32_t> h(pd.N);
    nlist->n_neigh.download(h.data(), pd.N, pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "n_neigh");
    double s = 0;
    for (uint32_t v : h)
        s += v;
    return s;
    }

std::vector<Integrator::TuneSample> Integrator::autotune()
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    if (!prepared || nlist->dirty)
        prepare();
    checkpoint();
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    DevStatus* ds = d_status.get();
    std::vector<TuneSample> out;
    // Each candidate runs in three interleaved rounds (one untimed launch, then five timed) and
    // keeps its best round mean; the default configuration stays unless another one is at least
    // 2 % faster, so that timing noise does not move a run off the defaults.
    struct Candidate
        {
        unsigned int block, tpp;
        double ms;
        };
    auto search = [&](std::vector<Candidate>& cand, size_t def,
                      const std::function<void(const Candidate&)>& apply,
                      const std::function<void()>& launch) -> size_t {
        for (auto& c : cand)
            c.ms = 1e30;
        for (int round = 0; round < 3; round++)
            for (auto& c : cand)
                {
                apply(c);
                launch();
                cuda_check(cudaEventRecord(e0, s), "record");
                for (int r = 0; r < 5; r++)
                    launch();
                cuda_check(cudaEventRecord(e1, s), "record");
                cuda_check(cudaEventSynchronize(e1), "sync");
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                c.ms = std::min(c.ms, ms / 5.0);
                }
        size_t best = def;
        for (size_t k = 0; k < cand.size(); k++)
            if (cand[k].ms < cand[best].ms)
                best = k;
        return cand[best].ms < 0.98 * cand[def].ms ? best : def;
    };
    try
        {
        if (nlist->tune_requested)
            {
            // a build at the current positions, as the forced build before the run made
            // (block size, threads per own particle); the default is the first
            std::vector<Candidate> cand = {{128u, 32u, 0.0}, {64u, 32u, 0.0}, {32u, 32u, 0.0},
                                           {128u, 1u, 0.0},  {64u, 1u, 0.0},  {32u, 1u, 0.0}};
            const size_t pick = search(
                cand, 0,
                [&](const Candidate& c) {
                    nlist->kp_block = c.block;
                    nlist->kp_tpp = c.tpp;
                },
                [&] {
                    cuda_check(cudaMemsetAsync(ds->cell_cond, 0, sizeof(ds->cell_cond), s),
                               "cond");
                    cuda_check(cudaMemsetAsync(ds->nl_cond, 0, sizeof(ds->nl_cond), s), "cond");
                    nlist->enqueue_build(nullptr, nullptr, ds->cell_cond, ds->nl_cond, s);
                });
            for (const auto& c : cand)
                out.push_back({"nlist", c.block, c.tpp, c.ms});
            nlist->kp_block = cand[pick].block;
            nlist->kp_tpp = cand[pick].tpp;
            nlist->tune_requested = false;
            }
        const bool fused_path = forces.size() == 1 && !compute_virial
                                && forces[0]->kind != PairKind::MLP
                                && forces[0]->kind != PairKind::DPD;
        for (auto& fp : forces)
            {
            PairForce& f = *fp;
            if (!f.tune_requested)
                continue;
            // several lanes per particle serve the interleaved list of an orthorhombic box
            // without XPLOR smoothing or virials
            const bool split = pd.box.xy == 0.0f && pd.box.xz == 0.0f && pd.box.yz == 0.0f
                               && f.shift_mode != 2 && !(compute_virial && !fused_path)
                               && f.kind != PairKind::MLP;
            std::vector<unsigned int> tpps = {1u};
            if (split)
                tpps = {1u, 4u, 8u};
            // the kernel's default: 256 threads, lanes per particle by N
            const unsigned int tpp_def
                = split ? (pd.N <= 16384 ? 8u : (pd.N <= 65536 ? 4u : 1u)) : 1u;
            std::vector<Candidate> cand;
            size_t def = 0;
            for (unsigned int b : {128u, 256u})
                for (unsigned int t : tpps)
                    {
                    if (b == 256u && t == tpp_def)
                        def = cand.size();
                    cand.push_back({b, t, 0.0});
                    }
            const size_t pick = search(
                cand, def,
                [&](const Candidate& c) {
                    f.kp_block = c.block;
                    f.kp_tpp = c.tpp;
                },
                [&] {
                    if (fused_path)
                        {
                        gb_pair_args a = f.pair_args(false);
                        const gb_step_fuse fu = fuse_args(ds);
                        check(f.launch_fused(a, fu, s), "fused pair step");
                        }
                    else
                        f.compute(s, compute_virial);
                });
            for (const auto& c : cand)
                out.push_back({"pair", c.block, c.tpp, c.ms});
            f.kp_block = cand[pick].block;
            f.kp_tpp = cand[pick].tpp;
            f.tune_requested = false;
            }
        }
    catch (...)
        {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        restore();
        throw;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    restore();
    // the candidates' forces were computed at the restored positions; recompute them with the
    // kept configuration so that every array matches it
    for (auto& f : forces)
        f->compute(s, compute_virial);
    drop_graphs();
    cuda_check(cudaStreamSynchronize(s), "autotune");
    return out;
    }

std::vector<double> Integrator::time_phases(unsigned int reps)
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    if (!prepared || nlist->dirty)
        prepare();
    if (forces.size() != 1)
        throw std::runtime_error("time_phases: one pair force (the fused path) required");
    checkpoint();
    cudaEvent_t ev[4];
    for (auto& e : ev)
        cuda_check(cudaEventCreate(&e), "event");
    std::vector<double> acc(3, 0.0);
    DevStatus* ds = d_status.get();
    for (unsigned int r = 0; r < reps; r++)
        {
        const gb_step_one_args o = step_one_args(ds);
        cuda_check(cudaEventRecord(ev[0], s), "record");
        check(gb_md_step_one(&o, s), "gb_md_step_one");
        cuda_check(cudaEventRecord(ev[1], s), "record");
        // time a real rebuild: open the gate (outside the timed interval)
        uint32_t one = 1;
        cuda_check(cudaMemcpyAsync(&ds->rebuild, &one, sizeof(one), cudaMemcpyHostToDevice, s),
                   "gate");
        cuda_check(cudaMemsetAsync(ds->cell_cond, 0, sizeof(ds->cell_cond), s), "cond");
        cuda_check(cudaMemsetAsync(ds->nl_cond, 0, sizeof(ds->nl_cond), s), "cond");
        cuda_check(cudaEventRecord(ev[2], s), "record");
        nlist->enqueue_build(&ds->rebuild, &ds->n_builds, ds->cell_cond, ds->nl_cond, s);
        cuda_check(cudaEventRecord(ev[3], s), "record");
        cuda_check(cudaEventSynchronize(ev[3]), "sync");
        float t01, t23;
        cudaEventElapsedTime(&t01, ev[0], ev[1]);
        cudaEventElapsedTime(&t23, ev[2], ev[3]);
        PairForce& f = *forces[0];
        gb_pair_args a = f.pair_args(false);
        const gb_step_fuse fu = fuse_args(ds);
        if (bussi)
            enqueue_bussi_draws(*this, ds, d_bussi_ring.get(), BUSSI_RING, 1, s);
        cuda_check(cudaEventRecord(ev[0], s), "record");
        if (f.kind == PairKind::MLP || f.kind == PairKind::DPD)
            {
            // unfused: forces, step two, thermo and the Bussi factor as enqueue_step_general
            f.compute(s, false);
            check(gb_cv_step_two(pd.vel.get(), pd.accel.get(), f.force.get(), pd.N, (float)dt,
                                 1.0f, nullptr, s),
                  "gb_cv_step_two");
            check(gb_thermo_reduce(pd.vel.get(), f.force.get(), nullptr, 0, pd.N,
                                   d_thermo_scratch.get(), ds->thermo, s),
                  "thermo");
            if (bussi)
                check(gb_bussi_factor(&ds->thermo[0], dof(), dt, tau, kT, pd.timestep + 1,
                                      pd.seed, 0u, &ds->factor, s),
                      "bussi");
            }
        else
            check(f.launch_fused(a, fu, s), "fused pair step");
        cuda_check(cudaEventRecord(ev[1], s), "record");
        cuda_check(cudaEventSynchronize(ev[1]), "sync");
        float t_pair;
        cudaEventElapsedTime(&t_pair, ev[0], ev[1]);
        acc[0] += t01;
        acc[1] += t23;
        acc[2] += t_pair;
        }
    for (auto& e : ev)
        cudaEventDestroy(e);
    for (auto& v : acc)
        v /= reps;
    restore();
    nlist->build_sync();
    // the force arrays belong to the restored positions again
    for (auto& f : forces)
        f->compute(s, false);
    cuda_check(cudaStreamSynchronize(s), "time_phases");
    return acc;
    }

std::vector<double> Integrator::thermo(bool with_virial)
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    if (!prepared)
        prepare();
    if (with_virial)
        for (auto& f : forces)
            if (!f->virial_valid)
                f->compute(s, true);
    d_thermo_scratch.resize(gb_thermo_scratch_bytes(pd.N));
    DeviceArray<double> out;
    out.resize(3);
    double ke = 0, pe = 0, w = 0;
    for (size_t k = 0; k < forces.size(); k++)
        {
        PairForce& f = *forces[k];
        check(gb_thermo_reduce(pd.vel.get(), f.force.get(), with_virial ? f.virial.get() : nullptr,
                               pd.N, pd.N, d_thermo_scratch.get(), out.get(), s),
              "thermo");
        double h[3];
        out.download(h, 3, s);
        cuda_check(cudaStreamSynchronize(s), "thermo");
        ke = h[0];
        // tail corrections: energy, and the same term on each diagonal of the virial (W is the
        // trace over 3)
        pe += h[1] + f.tail_energy / f.box_volume();
        w += h[2] + f.tail_virial / f.box_volume();
        }
    return {ke, pe, w};
    }

double PairForce::energy_sum()
    {
    ParticleData& pd = *pdata;
    const size_t need = gb_thermo_scratch_bytes(pd.N);
    if (d_esum_scratch.size() != need)
        {
        d_esum_scratch.resize(need);
        d_esum_scratch.zero(pd.stream); // the reduction's counter word starts at zero
        }
    d_esum.resize(3);
    check(gb_thermo_reduce(pd.vel.get(), force.get(), nullptr, pd.N, pd.N, d_esum_scratch.get(),
                           d_esum.get(), pd.stream),
          "energy sum");
    double h[3];
    d_esum.download(h, 3, pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "energy sum");
    return h[1];
    }

double PairForce::box_volume() const
    {
    const double* b = pdata->box6;
    return pdata->ndim == 2 ? b[0] * b[1] : b[0] * b[1] * b[2];
    }

} // namespace gbe
