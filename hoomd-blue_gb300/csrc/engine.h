// Host engine: the C++ operation classes of the short-range MD step on one GPU.
//
// These mirror the reference's host classes (ParticleData/SystemDefinition,
// NeighborListGPUBinned + CellListGPU, PotentialPair<Evaluator>GPU, IntegratorTwoStep +
// TwoStepConstantVolumeGPU + BussiThermostat + ComputeThermoGPU, SFCPackTunerGPU). They own the
// device arrays (plain cudaMalloc buffers, the role GlobalArray plays in the reference) and
// launch work only through the C ABI of include/hoomd_gb300.h.
//
// Differences from the reference's control flow, all invisible to the physics:
//  * no host synchronisation per step: the rebuild decision, the overflow conditions and the
//    Bussi factor live on the device; runs of steps are captured into a CUDA graph and replayed;
//  * overflow of the cell list or neighbour list inside a replayed run is detected after the run
//    from the device condition words; the state is then restored from a checkpoint taken before
//    the run, capacities grow (with headroom) and the run is repeated. The reference instead
//    re-runs the build immediately (hoomd/md/NeighborList.cc:412-427), which needs a host read
//    after every build.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "hoomd_gb300.h"

namespace gbe
{

void check(int rc, const char* what);
void cuda_check(cudaError_t e, const char* what);

template<class T> class DeviceArray
    {
    public:
    DeviceArray() = default;
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    ~DeviceArray()
        {
        release();
        }
    void resize(size_t n)
        {
        if (n == m_n)
            return;
        release();
        if (n)
            cuda_check(cudaMalloc((void**)&m_ptr, n * sizeof(T)), "cudaMalloc");
        m_n = n;
        }
    void release()
        {
        if (m_ptr)
            cudaFree(m_ptr);
        m_ptr = nullptr;
        m_n = 0;
        }
    T* get() const
        {
        return m_ptr;
        }
    size_t size() const
        {
        return m_n;
        }
    size_t bytes() const
        {
        return m_n * sizeof(T);
        }
    void upload(const T* h, size_t n, cudaStream_t s)
        {
        if (n > m_n)
            throw std::runtime_error("DeviceArray::upload: too many elements");
        if (n)
            cuda_check(cudaMemcpyAsync(m_ptr, h, n * sizeof(T), cudaMemcpyHostToDevice, s),
                       "upload");
        }
    void download(T* h, size_t n, cudaStream_t s) const
        {
        if (n > m_n)
            throw std::runtime_error("DeviceArray::download: too many elements");
        if (n)
            cuda_check(cudaMemcpyAsync(h, m_ptr, n * sizeof(T), cudaMemcpyDeviceToHost, s),
                       "download");
        }
    void download_at(T* h, size_t offset, size_t n, cudaStream_t s) const
        {
        if (offset + n > m_n)
            throw std::runtime_error("DeviceArray::download_at: out of range");
        if (n)
            cuda_check(cudaMemcpyAsync(h, m_ptr + offset, n * sizeof(T), cudaMemcpyDeviceToHost,
                                       s),
                       "download");
        }
    void swap(DeviceArray& o)
        {
        std::swap(m_ptr, o.m_ptr);
        std::swap(m_n, o.m_n);
        }
    void zero(cudaStream_t s)
        {
        if (m_n)
            cuda_check(cudaMemsetAsync(m_ptr, 0, m_n * sizeof(T), s), "memset");
        }
    void copy_from(const DeviceArray& o, cudaStream_t s)
        {
        resize(o.m_n);
        if (m_n)
            cuda_check(cudaMemcpyAsync(m_ptr, o.m_ptr, m_n * sizeof(T), cudaMemcpyDeviceToDevice, s),
                       "d2d copy");
        }

    private:
    T* m_ptr = nullptr;
    size_t m_n = 0;
    };

// Device-resident control block: one D2H copy per replayed run reads all of it.
struct DevStatus
    {
    uint32_t cell_cond[3]; // needed Nmax, NaN index+1, out-of-box index+1
    uint32_t rebuild;      // rebuild gate for the current step
    uint32_t status;       // bit 0: Bussi, bit 1: Berendsen with zero kinetic energy
    uint32_t pad[3];
    uint64_t timestep;
    uint64_t n_builds;
    // step of the last build (NeighborList m_last_updated_tstep), smallest period between
    // builds (capped at 99)
    uint64_t build_steps[2];
    uint64_t n_dangerous; // dangerous builds (delayed checks that found the list stale)
    double factor;         // Bussi rescale factor for the next step one
    double thermo[3];      // KE, PE, W after the last step
    double reservoir;      // Langevin reservoir energy (tally_reservoir_energy)
    double mttk[2];        // MTTK thermostat xi, eta
    double mttk_scale2;    // MTTK step-two factor of the current step
    uint32_t nl_cond[64];  // per-type neighbours needed on overflow
    };

class ParticleData
    {
    public:
    ParticleData(unsigned int N, unsigned int ntypes, unsigned int ndim,
                 const std::vector<double>& box6, const std::vector<int>& periodic);
    // host arrays in tag order: pos xyz (3N), vel xyz (3N), mass (N), typeid (N), image (3N),
    // optional charge (N). Particles that already exist keep their current index (a snapshot
    // written back keeps the sorted order); positions are wrapped into the box.
    void set_particles(const double* pos, const double* vel, const double* mass,
                       const uint32_t* typeid_, const int32_t* image,
                       const double* charge = nullptr);
    void get_particles(double* pos, double* vel, double* mass, uint32_t* typeid_,
                       int32_t* image);
    std::vector<uint32_t> rtag(); // tag -> index
    void set_box(const double* b6); // [Lx, Ly, Lz, xy, xz, yz]
    // per-particle charges in tag order (kept in index order on the device, sorted with the
    // particles); read by the pair forces that need them
    void set_charges(const double* q);
    void thermalize(double kT, uint64_t timestep);

    unsigned int N, ntypes, ndim;
    double box6[6];
    int periodic[3];
    gb_box box;
    uint16_t seed = 0;
    uint64_t timestep = 0;
    bool accel_set = false;
    cudaStream_t stream = nullptr;
    DeviceArray<float> pos, vel, accel, alt, charge;
    DeviceArray<int32_t> image;
    DeviceArray<uint32_t> tag;
    DeviceArray<char> scratch;
    DeviceArray<char> io_stage; // snapshot staging block (gb_snapshot_stage_bytes(N) + 256)
    bool tags_set = false;      // the particles exist (tags hold a permutation of 0..N-1)
    std::vector<std::string> type_names; // particle type names, by type id (when known)
    uint64_t sort_generation = 0;

    private:
    // section pointers of io_stage: pos, vel, mass, charge, typeid, image, rtag, error word
    struct Stage
        {
        double *pos, *vel, *mass, *charge;
        uint32_t* typeid_;
        int32_t* image;
        uint32_t *rtag, *err;
        };
    Stage stage();
    };

class NeighborList
    {
    public:
    NeighborList(std::shared_ptr<ParticleData> pdata, double r_buff);
    void set_r_cut(unsigned int i, unsigned int j, double r); // the nlist's own r_cut matrix
    void add_consumer(const std::vector<float>* rcut_matrix);
    // add unless already present; remove every entry of one matrix (its owner is going away)
    void ensure_consumer(const std::vector<float>* rcut_matrix);
    void remove_consumer(const std::vector<float>* rcut_matrix);
    void clear_consumers();
    void update_rlist();        // NeighborList::updateRList
    void allocate();            // cell grid, adjacency, capacities
    void build_sync();          // forced build with host-side overflow retry
    void enqueue_build(const uint32_t* d_gate, uint64_t* d_build_count, uint32_t* d_cell_cond,
                       uint32_t* d_nl_cond, cudaStream_t s, const uint64_t* d_timestep = nullptr,
                       uint64_t* d_build_steps = nullptr, uint64_t* d_dangerous = nullptr,
                       bool counts_zeroed = false);
    bool grow(const DevStatus& st); // returns true when a capacity grew
    // pairs of the list as tags (or as the current particle indices with local = true)
    std::vector<uint32_t> pair_list(bool full, bool local = false);
    std::vector<uint32_t> dims() const
        {
        return {dim[0], dim[1], dim[2]};
        }

    std::shared_ptr<ParticleData> pdata;
    float r_buff;
    bool deterministic = false;
    unsigned int rebuild_check_delay = 1;
    bool check_dist = true;
    std::vector<float> own_rcut;
    std::vector<const std::vector<float>*> consumers;
    std::vector<float> r_cut, r_listsq, rcut_max;
    unsigned int dim[3] = {0, 0, 0};
    unsigned int adj_w = 0, Nmax_cell = 0;
    std::vector<uint32_t> Nmax;
    uint64_t stride = 0;
    bool allocated = false;
    bool dirty = true; // r_cut or capacities changed: graphs must be rebuilt
    bool capacity_fixed = false; // start from exactly Nmax_cell / Nmax (tests of the growth path)
    // kernel parameters (Autotuner): threads per block of the tiled build and threads testing
    // each own particle (32 = candidate stream, 1 = lane per particle; 0 = defaults); a search on
    // the live state runs at the next run when requested
    unsigned int kp_block = 0, kp_tpp = 0;
    bool tune_requested = false;
    // exclusions (NeighborList::addExclusion / filterNlist): unordered tag pairs, and per
    // particle index the excluded indices (rebuilt when a sort permutes the indices)
    void set_exclusions(const std::vector<uint32_t>& tag_pairs);
    void refresh_exclusions();
    std::vector<uint32_t> ex_tags;
    unsigned int ex_pitch = 0;
    uint64_t ex_generation = ~0ull;
    // incremented whenever allocate() replaces the device buffers (captured graphs hold their
    // addresses, so graphs captured under an older generation must not be replayed)
    uint64_t alloc_generation = 0;
    bool ex_dirty = false;
    DeviceArray<uint32_t> n_ex, ex_list;
    DeviceArray<float> d_r_cut, d_r_listsq, d_rcut_max, xyzf, last_pos;
    DeviceArray<uint32_t> cell_size, cell_type, adj, n_neigh, d_Nmax, cond;
    // column-major, interleaved by 4: neighbour k of particle i at ((k/4)*stride + i)*4 + k%4
    DeviceArray<uint32_t> nlist;
    };

enum class PairKind
    {
    LJ = 0,
    Table = 1,
    Example = 2,
    MLP = 3, // radial MLP surrogate of Table (unfused path: pair list + tensor-core tiles)
    Radial = 4, // the other radial evaluators (gb_radial_param.kind)
    DPD = 5, // DPD thermostat pair forces (unfused: they read the velocities step two writes)
    Plugin = 6 // an evaluator compiled in a plugin module (gb_pair_plugin)
    };

class MlpSurrogate;

class PairForce
    {
    public:
    PairForce(std::shared_ptr<ParticleData> pdata, std::shared_ptr<NeighborList> nlist,
              PairKind kind);
    ~PairForce();
    PairForce(const PairForce&) = delete;
    PairForce& operator=(const PairForce&) = delete;
    // forces at the current positions outside an integrator (a force used as a compute): makes
    // this force's r_cut part of its list's r_list, builds the list and computes
    void compute_standalone(bool with_virial);
    // PotentialPair::computeEnergyBetweenSets: sum of V_ij over i in tags1, j in tags2, on the
    // device from a freshly built list
    double energy_between_sets(const std::vector<uint32_t>& tags1,
                               const std::vector<uint32_t>& tags2);
    void set_params_lj(unsigned int i, unsigned int j, double sigma, double epsilon);
    void set_params_example(unsigned int i, unsigned int j, double k, double sigma);
    void set_params_radial(unsigned int i, unsigned int j, unsigned int kind,
                           const std::vector<double>& v);
    // DPD (lj = false: A) or DPDLJ (lj = true: epsilon, sigma), drag gamma
    void set_params_dpd(unsigned int i, unsigned int j, bool lj, double a_or_eps, double sigma,
                        double gamma);
    void set_params_table(unsigned int i, unsigned int j, double r_min,
                          const std::vector<double>& U, const std::vector<double>& F);
    void set_r_cut(unsigned int i, unsigned int j, double r);
    void set_r_on(unsigned int i, unsigned int j, double r);
    void upload();
    void compute(cudaStream_t s, bool virial);
    int launch_fused(const gb_pair_args& a, const gb_step_fuse& f, cudaStream_t s);
    gb_pair_args pair_args(bool virial);

    std::shared_ptr<ParticleData> pdata;
    std::shared_ptr<NeighborList> nlist;
    PairKind kind;
    int shift_mode = 0;
    bool uses_charge = false; // the evaluator scales pairs by q_i q_j (d_charge in the args)
    // Isotropic long-range tail correction (PotentialPair::computeTailCorrection): the energy and
    // each diagonal virial term it adds are these coefficients over the box volume
    double tail_energy = 0.0, tail_virial = 0.0;
    double box_volume() const;
    unsigned int ntypes;
    std::vector<float> r_cut, r_on;
    std::vector<gb_lj_param> lj;
    std::vector<gb_example_param> ex;
    std::vector<gb_radial_param> rad;
    std::vector<gb_dpd_param> dpd;
    bool dpd_lj = false;
    double dpd_kT = 1.0;
    uint64_t force_timestep = 0; // timestep of the force evaluation (DPD random numbers)
    float force_dt = 0.0f;       // integrator time step (DPD random force amplitude)
    std::vector<double> t_rmin;
    std::vector<std::vector<double>> t_U, t_F;
    bool params_dirty = true;
    // kernel parameters (Autotuner): block size and threads per particle of the pair kernel
    // (0 = the kernel's defaults); a search on the live state runs at the next run when requested
    unsigned int kp_block = 0, kp_tpp = 0;
    bool tune_requested = false;
    std::shared_ptr<MlpSurrogate> mlp;
    // plugin evaluator: its record and ntypes^2 parameter records of param_size bytes each
    const gb_pair_plugin* plugin = nullptr;
    std::vector<unsigned char> plugin_params;
    void set_params_plugin(unsigned int i, unsigned int j, const void* record, size_t bytes);
    int plugin_call(gb_pair_plugin_call& c);
    DeviceArray<char> d_params, mlp_scratch, d_esum_scratch;
    DeviceArray<float> d_rcutsq, d_ronsq, d_table, force, virial;
    DeviceArray<double> d_esum;
    // sum of the per-particle energies of the last computed forces (FP64, on the device)
    double energy_sum();
    bool virial_valid = false;
    };

class Integrator
    {
    public:
    Integrator(std::shared_ptr<ParticleData> pdata, std::shared_ptr<NeighborList> nlist,
               double dt);
    ~Integrator();
    void add_force(std::shared_ptr<PairForce> f);
    void set_thermostat_bussi(double kT, double tau);
    void set_thermostat_none();
    // TwoStepLangevin (translational part): per-type drag coefficients, constant kT
    void set_langevin(double kT, const std::vector<double>& gamma, bool tally);
    double reservoir_energy();
    // ConstantVolume thermostats: Berendsen and MTTK (Nose-Hoover), hoomd/md/Thermostat.h
    void set_thermostat_berendsen(double kT, double tau);
    void set_thermostat_mttk(double kT, double tau);
    std::vector<double> mttk_state();               // xi, eta
    void set_mttk_state(double xi, double eta);
    void thermalize_mttk(uint64_t timestep);         // MTTKThermostat::thermalizeThermostat
    double mttk_energy();                            // MTTKThermostat::getThermostatEnergy
    // TwoStepBD (Brownian; noiseless = OverdampedViscous), translational part
    void set_brownian(double kT, const std::vector<double>& gamma, bool noiseless);
    // DisplacementCapped: limit of |v| dt in the ConstantVolume step one (0 = none)
    void set_max_displacement(double d);
    // ConstantPressure (TwoStepConstantPressure, MTK barostat), translational part; thermostat
    // none or MTTK. S = (xx, yy, zz, yz, xz, xy); couple 0 none, 1 xy, 2 xz, 3 yz, 4 xyz;
    // flags = box_dof (x, y, z, xy, xz, yz)
    void set_npt(const std::vector<double>& S, double tauS, int couple,
                 const std::vector<int>& box_dof, double gamma);
    std::vector<double> barostat_dof();             // (nu_xx, nu_xy, nu_xz, nu_yy, nu_yz, nu_zz)
    void set_barostat_dof(const std::vector<double>& nu);
    double barostat_energy();
    // FP64 sums over all forces: kinetic tensor (6), virial tensor (6), potential energy
    std::vector<double> thermo_tensor();
    void set_sorter(uint64_t period, int grid_bits);
    void set_chunk(unsigned int steps)
        {
        chunk = steps ? (steps > 1024 ? 1024 : steps) : 1;
        }
    // IntegratorTwoStep::prepRun. keep_graphs: only the particle state changed since the step
    // graphs were captured (positions, velocities, images, charges), so they stay valid; every
    // setter of a value the graphs hold (time step, thermostat, parameters) drops them itself
    void prepare(bool keep_graphs = false);
    void run(uint64_t nsteps);
    std::vector<double> thermo(bool with_virial); // KE, PE, W (W only when with_virial)
    double dof() const;
    DevStatus read_status();

    std::shared_ptr<ParticleData> pdata;
    std::shared_ptr<NeighborList> nlist;
    std::vector<std::shared_ptr<PairForce>> forces;
    double dt;
    bool bussi = false;
    double kT = 1.0, tau = 0.0;
    bool langevin = false, tally = false;
    bool berendsen = false, mttk = false;
    bool brownian = false, bd_noiseless = false;
    double bd_kT = 1.0;
    double max_disp = 0.0;
    bool npt = false;
    double npt_S[6] = {0, 0, 0, 0, 0, 0}, npt_tauS = 1.0, npt_gamma = 0.0;
    int npt_couple = 4;
    unsigned int npt_flags = 7;
    double nu[6] = {0, 0, 0, 0, 0, 0}; // xx, xy, xz, yy, yz, zz
    double mat_v[6], mat_r[6], mat_ri[6];
    std::vector<double> npt_tensor;     // thermo_tensor() at the last full step
    double mttk_host[2] = {0.0, 0.0}; // xi, eta carried across prepare()
    double langevin_kT = 1.0;
    std::vector<float> gamma;
    double reservoir = 0.0; // host copy, carried across prepare()
    uint64_t sort_period = 0;
    int sort_bits = 8;
    unsigned int chunk = 50;
    bool use_graph = true;
    // captured fused steps put the neighbour-list build in the body of a conditional graph node
    // (run only on rebuild steps) instead of launching the gated build kernels every step; falls
    // back to the gated kernels when the runtime refuses conditional nodes. Off by default: on
    // the 1M-particle fluid the conditional nodes cost more per step (0.296 against 0.290 ms at
    // one build in eight steps) than the early-exit blocks of the gated kernels they remove.
    bool use_conditional_build = false;
    cudaStream_t body_stream = nullptr; // captures the conditional node bodies
    uint64_t* h_builds = nullptr;       // page-locked copy of the build count at a chunk's start
    bool compute_virial = false;
    bool prepared = false;
    uint64_t n_rollbacks = 0;
    uint64_t steps_run = 0;
    uint64_t launch_count = 0; // kernels this engine launched (graph replays included)
    int notice_level = 2;      // the device's notice level (dangerous-build notices at >= 2)
    uint64_t dangerous_seen = 0;
    // average device time (ms) of each phase of one fused step, launched outside the graph on
    // the engine's stream with CUDA events: [step one + rebuild check, cell list + neighbour
    // list build, fused pair step]; the state is checkpointed before and restored after
    std::vector<double> time_phases(unsigned int reps);
    // the Autotuner's search (hoomd/Autotuner.h:49-668) for every pair force and the list that
    // asked for one: each candidate launch configuration timed on the current state (the state
    // restored afterwards), the fastest kept; returns {name, block, tpp, ms} per candidate
    struct TuneSample
        {
        std::string kernel;
        unsigned int block, tpp;
        double ms;
        };
    std::vector<TuneSample> autotune();
    std::vector<TuneSample> last_tuning;
    uintptr_t stream_handle() const
        {
        return (uintptr_t)pdata->stream;
        }
    double sum_n_neigh();
    // restart the smallest-rebuild-period statistic (at each Simulation.run)
    void reset_build_stats();
    // captured step graphs and the neighbour-list buffer generation they were captured under
    size_t graph_count() const
        {
        return graphs.size();
        }
    uint64_t graph_generation() const
        {
        return graph_nlist_generation;
        }
    void drop_graphs(); // the captured step graphs are rebuilt at the next run

    private:
    void sort_particles();
    gb_step_one_args step_one_args(DevStatus* ds) const;
    gb_step_fuse fuse_args(DevStatus* ds) const;
    void enqueue_step_fused(cudaStream_t s);
    void enqueue_step_general(cudaStream_t s, uint64_t step);
    void run_chunk(unsigned int k);
    void run_npt(uint64_t nsteps);
    void npt_advance_barostat(uint64_t timestep);
    void npt_update_propagator();
    double npt_temperature() const;
    void checkpoint();
    void restore();
    cudaGraphExec_t graph_for(unsigned int k);
    void capture_step_conditional(cudaStream_t s, unsigned long long handle);

    DeviceArray<DevStatus> d_status;
    DeviceArray<char> d_step_scratch, d_thermo_scratch;
    static constexpr unsigned int BUSSI_RING = 1024; // >= the longest chunk
    DeviceArray<double> d_bussi_ring;                // (normal, 2*gamma) per timestep % RING
    DeviceArray<float> net_force, d_gamma;
    DeviceArray<float> ck_pos, ck_vel, ck_accel;
    DeviceArray<int32_t> ck_image;
    DeviceArray<DevStatus> ck_status;
    std::map<unsigned int, cudaGraphExec_t> graphs;
    uint64_t graph_sort_generation = ~0ull;
    uint64_t graph_nlist_generation = ~0ull; // NeighborList::alloc_generation of the graphs
    };

} // namespace gbe
