// Host engine of replica ensembles (layout, launches, overflow regrowth, launch-shape tuning).
#include "ensemble.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <numeric>
#include <sstream>
#include <stdexcept>

namespace gbe
{

static constexpr uint32_t CELL_CAP = 16384; // cells per replica held in shared memory
static constexpr double PI = 3.14159265358979323846;

ReplicaEnsemble::ReplicaEnsemble(double dt_, double r_cut_, double r_buff_, double epsilon,
                                 double sigma, int shift_mode_)
    : dt(dt_), r_cut(r_cut_), r_buff(r_buff_), shift_mode(shift_mode_)
    {
    if (!(r_cut_ > 0.0))
        throw std::invalid_argument("r_cut must be positive");
    if (!(r_buff_ >= 0.0))
        throw std::invalid_argument("buffer must be non-negative");
    if (shift_mode_ != 0 && shift_mode_ != 1)
        throw std::invalid_argument("mode must be 'none' or 'shift'");
    // PairForce::set_params_lj at FP32 (hoomd/md/EvaluatorPairLJ.h:125-142)
    const float s = (float)sigma;
    lj.sigma_6 = s * s * s * s * s * s;
    lj.epsilon_x_4 = 4.0f * (float)epsilon;
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
    cuda_check(cudaEventCreate(&ev0), "event");
    cuda_check(cudaEventCreate(&ev1), "event");
    }

ReplicaEnsemble::~ReplicaEnsemble()
    {
    drop_graph();
    if (pin_reps)
        cudaFreeHost(pin_reps);
    if (pin_targets)
        cudaFreeHost(pin_targets);
    if (ev0)
        cudaEventDestroy(ev0);
    if (ev1)
        cudaEventDestroy(ev1);
    if (stream)
        {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
        }
    }

void ReplicaEnsemble::drop_graph()
    {
    if (graph)
        cudaGraphExecDestroy(graph);
    graph = nullptr;
    }

void ReplicaEnsemble::set_launch(uint32_t block, uint32_t grid)
    {
    if (block < 64 || block > GB_REPLICA_MAX_BLOCK || block % 32)
        throw std::invalid_argument("block_size must be a multiple of 32 in [64, 1024]");
    block_size = block;
    grid_size = grid;
    drop_graph();
    }

void ReplicaEnsemble::set_stencil(uint32_t s)
    {
    if (!h_reps.empty())
        throw std::runtime_error("set the stencil before adding replicas");
    if (s != 1 && s != 2)
        throw std::invalid_argument("stencil must be 1 or 2");
    stencil = s;
    }

void ReplicaEnsemble::set_start_capacity(uint32_t nmax)
    {
    if (allocated)
        throw std::runtime_error("set the start capacity before the first run");
    start_capacity = (nmax + 3) & ~3u;
    for (auto& r : h_reps)
        r.Nmax = std::max(4u, start_capacity);
    }

uint32_t ReplicaEnsemble::add(unsigned int N, const double* pos, const double* vel,
                              const double* mass, const int32_t* image, const double L[3],
                              const double tilt[3], bool bussi, double kT, double tau,
                              uint32_t seed, uint64_t timestep)
    {
    if (allocated)
        throw std::runtime_error("replicas can only be added before the first run");
    if (N == 0)
        throw std::invalid_argument("a replica needs at least one particle");
    if (bussi && N < 2)
        throw std::invalid_argument("Bussi needs at least two particles (dof = 3N - 3)");
    gb_replica r;
    std::memset(&r, 0, sizeof(r));
    const int periodic[3] = {1, 1, 1};
    check(gb_box_make(L, tilt ? tilt[0] : 0.0, tilt ? tilt[1] : 0.0, tilt ? tilt[2] : 0.0,
                      periodic, &r.box),
          "box");
    const float rl = (float)r_cut + (float)r_buff;
    uint32_t dim[3];
    check(gb_cell_dims(&r.box, 3, rl, dim), "cell dims");
    if (dim[0] < 2 || dim[1] < 2 || dim[2] < 2)
        throw std::invalid_argument(
            "Simulation box is too small: every width must be at least 2 (r_cut + buffer)");
    // stencil 2 (cells of r_list / 2, 125 searched) tests 42 % fewer candidates than stencil 1
    // (cells of r_list, 27 searched) but its lanes diverge more: a warp's particles sit in ~10
    // cells instead of ~2. Stencil 1 builds faster in the one-thread-per-particle search.
    r.stencil = stencil;
    float width = rl / (float)stencil;
    check(gb_cell_dims(&r.box, 3, width, dim), "cell dims");
    while ((uint64_t)dim[0] * dim[1] * dim[2] > CELL_CAP)
        {
        width *= 1.25f;
        check(gb_cell_dims(&r.box, 3, width, dim), "cell dims");
        }
    r.N = N;
    r.stride = (N + 31) / 32 * 32;
    std::copy(dim, dim + 3, r.dim);
    r.lj = lj;
    r.r_cut = (float)r_cut;
    r.r_buff = (float)r_buff;
    r.shift_mode = (uint32_t)shift_mode;
    r.bussi = bussi ? 1u : 0u;
    r.seed = seed & 0xffffu;
    r.dt = dt;
    r.kT = kT;
    r.tau = tau;
    r.dof = 3.0 * N - 3.0;
    r.timestep = timestep;
    r.target = timestep;
    r.factor = 1.0;
    // capacity from the mean count in the r_list sphere, with room for fluctuations
    const double vol = (double)r.box.L[0] * r.box.L[1] * r.box.L[2];
    const double nbar = 4.0 / 3.0 * PI * (double)rl * rl * rl * (N / vol);
    uint32_t nmax = (uint32_t)std::ceil(1.25 * nbar + 8.0);
    if (start_capacity)
        nmax = start_capacity;
    r.Nmax = std::max(4u, (nmax + 3) & ~3u);
    h_reps.push_back(r);

    std::vector<float> p(4 * (size_t)N), v(4 * (size_t)N);
    std::vector<int32_t> im(4 * (size_t)N, 0);
    for (size_t i = 0; i < N; i++)
        {
        for (int k = 0; k < 3; k++)
            {
            p[4 * i + k] = (float)pos[3 * i + k];
            v[4 * i + k] = (float)vel[3 * i + k];
            if (image)
                im[4 * i + k] = image[3 * i + k];
            }
        p[4 * i + 3] = 0.0f; // type 0 (bits)
        v[4 * i + 3] = (float)mass[i];
        }
    h_pos.push_back(std::move(p));
    h_vel.push_back(std::move(v));
    h_img.push_back(std::move(im));
    total_N += N;
    return (uint32_t)(h_reps.size() - 1);
    }

void ReplicaEnsemble::allocate()
    {
    const uint32_t R = count();
    if (R == 0)
        throw std::runtime_error("the ensemble has no replicas");
    uint64_t first = 0, nl = 0;
    max_cells = 1;
    for (auto& r : h_reps)
        {
        r.first = first;
        first += r.stride;
        r.nlist_offset = nl;
        nl += (uint64_t)r.stride * r.Nmax;
        max_cells = std::max(max_cells, r.dim[0] * r.dim[1] * r.dim[2]);
        }
    n_slots = first;
    arena_used = nl;
    // largest replicas first: the queue hands the longest jobs out before the short ones
    std::vector<uint32_t> order(R);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return h_reps[a].N > h_reps[b].N; });

    d_reps.resize(R);
    d_order.resize(R);
    d_queue.resize(2);
    d_pos.resize(4 * n_slots);
    d_vel.resize(4 * n_slots);
    d_accel.resize(4 * n_slots);
    d_force.resize(4 * n_slots);
    d_last_pos.resize(4 * n_slots);
    d_image.resize(4 * n_slots);
    d_n_neigh.resize(n_slots);
    d_nlist.resize(nl + nl / 4 + 4);
    d_scratch.resize(gb_replica_scratch_bytes(n_slots));
    d_clocks.resize(4 * (size_t)R);
    d_clocks.zero(stream);
    for (auto* a : {&d_pos, &d_vel, &d_accel, &d_force, &d_last_pos})
        a->zero(stream);
    d_image.zero(stream);
    d_n_neigh.zero(stream);
    d_queue.zero(stream);
    for (uint32_t k = 0; k < R; k++)
        {
        const gb_replica& r = h_reps[k];
        const size_t n4 = 4 * (size_t)r.N;
        cuda_check(cudaMemcpyAsync(d_pos.get() + 4 * r.first, h_pos[k].data(), n4 * 4,
                                   cudaMemcpyHostToDevice, stream),
                   "upload positions");
        cuda_check(cudaMemcpyAsync(d_vel.get() + 4 * r.first, h_vel[k].data(), n4 * 4,
                                   cudaMemcpyHostToDevice, stream),
                   "upload velocities");
        cuda_check(cudaMemcpyAsync(d_image.get() + 4 * r.first, h_img[k].data(), n4 * 4,
                                   cudaMemcpyHostToDevice, stream),
                   "upload images");
        }
    d_order.upload(order.data(), R, stream);
    d_reps.upload(h_reps.data(), R, stream);
    cuda_check(cudaMallocHost((void**)&pin_reps, sizeof(gb_replica) * R), "pinned records");
    cuda_check(cudaMallocHost((void**)&pin_targets, sizeof(uint64_t) * R), "pinned targets");
    cuda_check(cudaStreamSynchronize(stream), "upload");
    h_pos.clear();
    h_vel.clear();
    h_img.clear();
    allocated = true;
    }

// Enqueues: targets H2D (a strided copy into the records' target fields), the persistent kernel,
// the records D2H. Recorded once into a graph and replayed.
void ReplicaEnsemble::launch_once()
    {
    const uint32_t R = count();
    auto enqueue = [&]() {
        cuda_check(cudaMemcpy2DAsync(reinterpret_cast<char*>(d_reps.get()) + offsetof(gb_replica, target),
                                     sizeof(gb_replica), pin_targets,
                                     sizeof(uint64_t), sizeof(uint64_t), R,
                                     cudaMemcpyHostToDevice, stream),
                   "targets");
        gb_replica_batch b {};
        b.d_replicas = d_reps.get();
        b.n_replicas = R;
        b.d_order = d_order.get();
        b.d_queue = d_queue.get();
        b.d_pos = d_pos.get();
        b.d_vel = d_vel.get();
        b.d_accel = d_accel.get();
        b.d_image = d_image.get();
        b.d_force = d_force.get();
        b.d_last_pos = d_last_pos.get();
        b.d_n_neigh = d_n_neigh.get();
        b.d_nlist = d_nlist.get();
        b.d_scratch = d_scratch.get();
        b.n_slots = n_slots;
        b.max_cells = max_cells;
        b.block_size = block_size;
        b.grid_size = grid_size;
        b.d_phase_clocks = d_clocks.get();
        check(gb_replicas_run(&b, stream), "gb_replicas_run");
        cuda_check(cudaMemcpyAsync(pin_reps, d_reps.get(), sizeof(gb_replica) * R,
                                   cudaMemcpyDeviceToHost, stream),
                   "records");
    };
    cuda_check(cudaEventRecord(ev0, stream), "event");
    if (use_graph)
        {
        if (!graph)
            {
            cudaGraph_t g;
            cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal),
                       "begin capture");
            try
                {
                enqueue();
                }
            catch (...)
                {
                cudaStreamEndCapture(stream, &g);
                throw;
                }
            cuda_check(cudaStreamEndCapture(stream, &g), "end capture");
            cuda_check(cudaGraphInstantiate(&graph, g, 0), "graph instantiate");
            cudaGraphDestroy(g);
            }
        cuda_check(cudaGraphLaunch(graph, stream), "graph launch");
        }
    else
        enqueue();
    cuda_check(cudaEventRecord(ev1, stream), "event");
    cuda_check(cudaStreamSynchronize(stream), "replica run");
    launch_count += 1;
    }

void ReplicaEnsemble::sync_records()
    {
    std::memcpy(h_reps.data(), pin_reps, sizeof(gb_replica) * count());
    }

static const char* status_text(uint32_t st)
    {
    if (st & GB_REPLICA_NAN)
        return "has a particle with NaN for its position";
    if (st & GB_REPLICA_OUTSIDE)
        return "has a particle that is no longer in the simulation box";
    if (st & GB_REPLICA_ZERO_KE)
        return "uses the Bussi thermostat, which requires non-zero initial momenta";
    return "has a cell grid larger than the launch supports";
    }

void ReplicaEnsemble::run(uint64_t steps)
    {
    if (!allocated)
        allocate();
    const uint32_t R = count();
    for (uint32_t k = 0; k < R; k++)
        pin_targets[k] = h_reps[k].timestep + steps;
    double ms = 0.0;
    for (int attempt = 0; attempt < 32; attempt++)
        {
        launch_once();
        float t = 0.0f;
        cuda_check(cudaEventElapsedTime(&t, ev0, ev1), "elapsed");
        ms += t;
        sync_records();
        bool regrow = false;
        for (uint32_t k = 0; k < R; k++)
            {
            gb_replica& r = h_reps[k];
            const uint32_t st = r.status;
            if (st & ~GB_REPLICA_OVERFLOW)
                {
                std::ostringstream m;
                m << "replica " << k << " " << status_text(st) << ".";
                throw std::runtime_error(m.str());
                }
            if (st & GB_REPLICA_OVERFLOW)
                {
                // NeighborList::grow's headroom; a fresh block at the end of the arena
                const uint32_t want = r.needed + std::max(8u, r.needed / 8);
                r.Nmax = (want + 3) & ~3u;
                r.nlist_offset = arena_used;
                arena_used += (uint64_t)r.stride * r.Nmax;
                r.status = 0u;
                r.needed = 0u;
                regrow = true;
                }
            }
        if (!regrow)
            {
            last_run_ms = ms;
            return;
            }
        n_regrowths++;
        if (arena_used > d_nlist.size())
            {
            DeviceArray<uint32_t> bigger;
            bigger.resize(arena_used + arena_used / 4);
            const uint64_t keep = d_nlist.size();
            cuda_check(cudaMemcpyAsync(bigger.get(), d_nlist.get(), keep * sizeof(uint32_t),
                                       cudaMemcpyDeviceToDevice, stream),
                       "grow neighbour arena");
            cuda_check(cudaStreamSynchronize(stream), "grow neighbour arena");
            d_nlist.swap(bigger);
            drop_graph();
            }
        d_reps.upload(h_reps.data(), R, stream);
        }
    throw std::runtime_error("run: repeated neighbour-list overflow");
    }

std::vector<TuneResult> ReplicaEnsemble::autotune(uint32_t steps_per_trial, uint32_t repeats)
    {
    if (!allocated)
        allocate();
    int dev = 0, sms = 0;
    cuda_check(cudaGetDevice(&dev), "device");
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SMs");
    std::vector<TuneResult> out;
    const uint32_t blocks[] = {128, 256, 512, 768, 1024};
    TuneResult best {block_size, grid_size, 1e300};
    for (uint32_t b : blocks)
        {
        const int occ = gb_replica_ctas_per_sm(max_cells, b);
        for (int c = 1; c <= occ && c <= 8; c++)
            {
            set_launch(b, (uint32_t)(c * sms));
            run(steps_per_trial); // records the graph for this shape
            double t = 1e300;
            for (uint32_t k = 0; k < std::max(1u, repeats); k++)
                {
                run(steps_per_trial);
                t = std::min(t, last_run_ms / steps_per_trial);
                }
            out.push_back({b, (uint32_t)(c * sms), t});
            if (t < best.ms_per_step)
                best = out.back();
            }
        }
    set_launch(best.block_size, best.grid_size);
    return out;
    }

gb_replica ReplicaEnsemble::record(uint32_t r)
    {
    if (r >= count())
        throw std::out_of_range("replica index");
    return h_reps[r];
    }

void ReplicaEnsemble::get_particles(uint32_t k, double* pos, double* vel, int32_t* image,
                                    double* force)
    {
    if (k >= count())
        throw std::out_of_range("replica index");
    if (!allocated)
        allocate();
    const gb_replica& r = h_reps[k];
    const size_t n4 = 4 * (size_t)r.N;
    std::vector<float> p(n4), v(n4), f(n4);
    std::vector<int32_t> im(n4);
    d_pos.download_at(p.data(), 4 * r.first, n4, stream);
    d_vel.download_at(v.data(), 4 * r.first, n4, stream);
    d_force.download_at(f.data(), 4 * r.first, n4, stream);
    d_image.download_at(im.data(), 4 * r.first, n4, stream);
    cuda_check(cudaStreamSynchronize(stream), "download");
    for (size_t i = 0; i < r.N; i++)
        for (int c = 0; c < 4; c++)
            {
            if (c < 3)
                {
                pos[3 * i + c] = p[4 * i + c];
                vel[4 * i + c] = v[4 * i + c];
                image[3 * i + c] = im[4 * i + c];
                }
            else
                vel[4 * i + 3] = v[4 * i + 3];
            force[4 * i + c] = f[4 * i + c];
            }
    }

std::vector<uint64_t> ReplicaEnsemble::phase_clocks()
    {
    std::vector<uint64_t> h(d_clocks.size());
    d_clocks.download(h.data(), h.size(), stream);
    cuda_check(cudaStreamSynchronize(stream), "download");
    return h;
    }

std::vector<uint32_t> ReplicaEnsemble::neighbor_counts(uint32_t k)
    {
    if (k >= count())
        throw std::out_of_range("replica index");
    const gb_replica& r = h_reps[k];
    std::vector<uint32_t> n(r.N);
    d_n_neigh.download_at(n.data(), r.first, r.N, stream);
    cuda_check(cudaStreamSynchronize(stream), "download");
    return n;
    }

std::vector<uint32_t> ReplicaEnsemble::neighbor_list(uint32_t k)
    {
    if (k >= count())
        throw std::out_of_range("replica index");
    const gb_replica& r = h_reps[k];
    std::vector<uint32_t> n = neighbor_counts(k);
    const size_t words = (size_t)r.stride * r.Nmax;
    std::vector<uint32_t> blk(words);
    d_nlist.download_at(blk.data(), r.nlist_offset, words, stream);
    cuda_check(cudaStreamSynchronize(stream), "download");
    std::vector<uint32_t> out((size_t)r.N * r.Nmax, 0xffffffffu);
    for (size_t i = 0; i < r.N; i++)
        for (uint32_t c = 0; c < n[i]; c++)
            out[i * r.Nmax + c] = blk[((size_t)(c / 4) * r.stride + i) * 4 + c % 4];
    return out;
    }

} // namespace gbe
