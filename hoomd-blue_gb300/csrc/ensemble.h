// Host engine of replica ensembles: many independent single-type LJ systems (each the
// reference's Simulation + Cell nlist + pair.LJ + ConstantVolume/Bussi) advanced together by one
// persistent kernel launch per run (gb_replicas_run), replayed from a CUDA graph.
//
// Layout: all replicas share the per-particle arrays (replica r owns [first_r, first_r + N_r),
// first_r a multiple of 32) and one neighbour-list arena in which each replica has its own
// column-major, interleaved-by-4 block of stride_r x Nmax_r words. When a replica's list
// overflows, the kernel stops that replica where it was (after step one, before the build), the
// host gives it a larger block at the end of the arena (the other replicas' blocks never move,
// so their lists stay valid) and the launch is repeated; only the stopped replicas have work left,
// and they resume exactly where they stopped, so a run with overflows gives the same trajectory
// bit for bit as one without.
//
// The launch shape (threads per CTA, persistent CTAs) does not change any result, so the tuner
// times candidate shapes on live steps, as the reference's Autotuner does (hoomd/Autotuner.h).
#pragma once

#include <cstdint>
#include <vector>

#include "engine.h"

namespace gbe
{

struct TuneResult
    {
    uint32_t block_size;
    uint32_t grid_size;
    double ms_per_step;
    };

class ReplicaEnsemble
    {
    public:
    ReplicaEnsemble(double dt, double r_cut, double r_buff, double epsilon, double sigma,
                    int shift_mode);
    ~ReplicaEnsemble();
    ReplicaEnsemble(const ReplicaEnsemble&) = delete;
    ReplicaEnsemble& operator=(const ReplicaEnsemble&) = delete;

    // Adds a replica: N positions and velocities (3N doubles each, inside the box), masses (N),
    // images (3N or empty), box lengths and tilts. Returns its index. Only before the first run.
    uint32_t add(unsigned int N, const double* pos, const double* vel, const double* mass,
                 const int32_t* image, const double L[3], const double tilt[3], bool bussi,
                 double kT, double tau, uint32_t seed, uint64_t timestep);

    void run(uint64_t steps);
    std::vector<TuneResult> autotune(uint32_t steps_per_trial, uint32_t repeats);
    void set_launch(uint32_t block_size, uint32_t grid_size);
    void set_start_capacity(uint32_t nmax); // first neighbour capacity (tests of regrowth)
    void set_stencil(uint32_t s);           // 1: cells of r_list; 2: cells of r_list / 2

    // per-replica readback (host order of the replica's particles)
    void get_particles(uint32_t r, double* pos, double* vel, int32_t* image, double* force);
    std::vector<uint32_t> neighbor_counts(uint32_t r);
    // SM cycles each replica's CTA spent per phase since allocation, [4 * count()]: step one,
    // neighbour-list builds, pair step (+ step two, sums, factor), Bussi draws
    std::vector<uint64_t> phase_clocks();
    std::vector<uint32_t> neighbor_list(uint32_t r); // N x n_neigh_max, -1 padded rows
    gb_replica record(uint32_t r);

    uint32_t count() const
        {
        return (uint32_t)h_reps.size();
        }
    uint64_t total_particles() const
        {
        return total_N;
        }
    uint32_t block_size = 512;
    uint32_t grid_size = 0;      // 0 = every CTA that fits at once
    uint64_t launch_count = 0;   // kernels launched (graph replays included)
    uint64_t n_regrowths = 0;    // relaunches after neighbour-list overflow
    bool use_graph = true;
    uintptr_t stream_handle() const
        {
        return (uintptr_t)stream;
        }
    double last_run_ms = 0.0;    // device time of the last run's launches (CUDA events)

    private:
    void allocate();
    void launch_once();
    void drop_graph();
    void sync_records();

    double dt, r_cut, r_buff;
    gb_lj_param lj;
    int shift_mode;
    uint32_t start_capacity = 0;
    uint32_t stencil = 1;
    bool allocated = false;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    std::vector<gb_replica> h_reps;           // host copy of the records
    std::vector<std::vector<float>> h_pos, h_vel;
    std::vector<std::vector<int32_t>> h_img;
    uint64_t total_N = 0, n_slots = 0, arena_used = 0;
    uint32_t max_cells = 1;
    gb_replica* pin_reps = nullptr;           // pinned staging for records
    uint64_t* pin_targets = nullptr;          // pinned targets (read by the graph's copy node)
    DeviceArray<gb_replica> d_reps;
    DeviceArray<uint32_t> d_order, d_queue, d_n_neigh, d_nlist;
    DeviceArray<float> d_pos, d_vel, d_accel, d_force, d_last_pos;
    DeviceArray<int32_t> d_image;
    DeviceArray<char> d_scratch;
    DeviceArray<uint64_t> d_clocks;
    };

} // namespace gbe
