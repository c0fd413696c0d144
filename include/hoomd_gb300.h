/* hoomd_gb300.h -- C ABI of the GB300-native short-range MD step.
 *
 * One shared library (libhoomd_gb300.so) exports the kernel drivers of HOOMD-blue's short-range
 * MD hot path -- cell list, binned neighbour list, distance check, PotentialPair<Evaluator> force
 * loop, ConstantVolume/NVE integrator halves, thermodynamic reductions, Bussi factor, momentum
 * thermalisation and the space-filling-curve particle sort -- as extern "C" functions with POD
 * argument structs and plain device pointers. Each entry point names the reference kernel driver
 * it replaces (paths relative to the HOOMD-blue source tree).
 *
 * Conventions
 *  - All pointers named d_* (or documented as device) are device pointers owned by the caller.
 *  - Per-particle arrays keep HOOMD's FP32 layouts: positions float4 (x, y, z, type bits in w),
 *    velocities float4 (vx, vy, vz, mass), accelerations float3, images int3, forces float4
 *    (fx, fy, fz, energy), virials 6 x pitch floats (xx, xy, xz, yy, yz, zz).
 *  - Every call is ordered on `stream` (a cudaStream_t passed as void*; NULL = legacy default)
 *    and never synchronises the host. Functions return GB_OK or a gb_status error code and never
 *    throw across the boundary; gb_last_error() returns a message for the last failure on the
 *    calling host thread.
 *  - Device-side conditions (overflow, NaN, particle outside the box) are written to caller
 *    buffers, as the reference's m_conditions arrays are, for the host to read when it chooses.
 */
#ifndef HOOMD_GB300_H
#define HOOMD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gb_status
    {
    GB_OK = 0,
    GB_ERR_INVALID = 1,     /* bad argument (null pointer, zero size, unsupported option) */
    GB_ERR_CUDA = 2,        /* a CUDA launch or runtime call failed */
    GB_ERR_TOO_LARGE = 3,   /* size beyond a documented maximum */
    GB_ERR_UNSUPPORTED = 4  /* combination not implemented */
    } gb_status;

/* Simulation box at FP32, field for field the reference's BoxDim (hoomd/BoxDim.h:69-840). Build
 * it with gb_box_make so that lo, hi and Linv round exactly as BoxDim::setL does at FP32. */
typedef struct gb_box
    {
    float lo[3];
    float hi[3];
    float L[3];
    float Linv[3];
    float xy, xz, yz;
    uint32_t periodic[3];
    } gb_box;

/* BoxDim(Lx, Ly, Lz) + setTiltFactors + setPeriodic (hoomd/BoxDim.h:103-180), host only. */
/* sizeof of the argument structs, in this order: gb_box, gb_cell_list_args, gb_nlist_args,
 * gb_pair_args, gb_radial_param, gb_step_one_args, gb_step_fuse, gb_mlp_force_args, gb_replica,
 * gb_replica_batch. Writes min(n, 10) values and returns 10, so a binding can check its own
 * mirror of each struct before it passes one. */
unsigned int gb_abi_struct_sizes(size_t* out, unsigned int n);

int gb_box_make(const double L[3], double xy, double xz, double yz, const int periodic[3],
                gb_box* out);

/* Nearest plane distances (hoomd/BoxDim.h:552-567) and cell-grid dimensions
 * floor(npd / nominal_width), at least 1 (hoomd/CellList.cc:83-131), host only. */
int gb_cell_dims(const gb_box* box, unsigned int ndim, float nominal_width, unsigned int dim[3]);

const char* gb_last_error(void);
int gb_version(void);

/* ---------------------------------------------------------------------------------------------
 * Cell list. Replaces gpu_compute_cell_list (hoomd/CellListGPU.cuh:21-43, kernel
 * hoomd/CellListGPU.cu:42-170) with flag = particle index (NeighborListBinned.cc:25-28).
 * Slot layout: xyzf[cell * Nmax + slot] (Index2D(Nmax, ncell), hoomd/CellList.cc:241).
 * ------------------------------------------------------------------------------------------- */
typedef struct gb_cell_list_args
    {
    const float* d_pos;          /* float4[N] */
    unsigned int N;
    gb_box box;
    unsigned int dim[3];
    unsigned int Nmax;           /* slots per cell */
    unsigned int* d_cell_size;   /* [ncell], zeroed by the call */
    float* d_xyzf;               /* float4[ncell * Nmax]: x, y, z, particle index bits */
    unsigned int* d_cell_type;   /* optional [ncell * Nmax] particle type per slot (NULL = skip) */
    unsigned int* d_conditions;  /* [3]: needed Nmax on overflow, NaN index+1, out-of-box
                                    index+1 (max over offenders); the caller zeroes it */
    const uint32_t* d_gate;      /* optional: when non-NULL and *d_gate == 0 the call is a no-op
                                    on the device (rebuild decided on the GPU, no host sync) */
    int deterministic;           /* sort each cell's slots by particle index
                                    (nlist.Cell(deterministic=True), hoomd/CellListGPU.cu:478-540) */
    uint64_t* d_build_count;     /* optional: incremented once per (non-gated-off) call */
    /* optional, both or neither: the rebuild statistics of NeighborList::needsUpdating
     * (hoomd/md/NeighborList.cc:1388-1402, getSmallestRebuild :1428-1436). The step of a build
     * is *d_timestep + 1 (the step whose forces follow, the reference's needsUpdating(timestep +
     * 1)). d_build_steps[0] is the step of the last build (m_last_updated_tstep; UINT64_MAX
     * before the first) and d_build_steps[1] the smallest period between builds, capped at 99;
     * the caller sets it to 100 when the statistics start. */
    const uint64_t* d_timestep;
    uint64_t* d_build_steps;
    /* optional, with d_build_steps: dangerous builds. When check_dist is set, check_delay > 1 and
     * the step of the list build is exactly d_build_steps[0] + check_delay (the first check after the
     * delay found the list stale), *d_dangerous is incremented (hoomd/md/NeighborList.cc:
     * 1349-1356, 1405-1414). */
    uint64_t* d_dangerous;
    uint32_t check_delay;
    int check_dist;
    /* the caller has zeroed d_cell_size (gb_step_one_args.d_zero_words in the same step): the
       call does not zero it again, and the build statistics are kept by the binning launch */
    int counts_zeroed;
    } gb_cell_list_args;

int gb_cell_list_build(const gb_cell_list_args* args, void* stream);

/* Cell adjacency (hoomd/CellList.cc:346-402): per cell the (2r+1)^3 stencil (r = 1), wrapped,
 * sorted and deduplicated; computed on the device. width = 27 unless a dimension has < 3 cells.
 * d_adj must hold ncell * 27 entries. */
int gb_cell_adj_build(const unsigned int dim[3], unsigned int ndim, unsigned int* d_adj,
                      unsigned int* width_out, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Neighbour list. Replaces gpu_compute_nlist_binned (hoomd/md/NeighborListGPUBinned.cuh,
 * kernel hoomd/md/NeighborListGPUBinned.cu:52-298): full storage, dr^2 <= r_list^2 inclusive,
 * self and r_cut <= 0 pairs skipped, overflow recorded per type as the count needed. Unlike
 * the reference, d_n_neigh holds the stored count, min(found, Nmax[type]), so that a consumer
 * launched before the host has read the overflow condition never reads past a particle's list.
 * Layouts: with d_head_list non-NULL, neighbour k of particle i lives at
 * d_nlist[d_head_list[i] + k] (the reference's flat layout). With d_head_list NULL the list is
 * column-major with stride >= N: interleave 1 puts neighbour k at d_nlist[k * stride + i];
 * interleave 4 puts it at d_nlist[((k / 4) * stride + i) * 4 + k % 4], so one 16-byte load gives
 * a particle four consecutive neighbours and a warp reads 512 contiguous bytes.
 * ------------------------------------------------------------------------------------------- */
typedef struct gb_nlist_args
    {
    unsigned int* d_nlist;
    unsigned int* d_n_neigh;          /* [N] */
    float* d_last_pos;                /* optional float4[N]: positions at build (distance check) */
    unsigned int* d_conditions;       /* [ntypes]: max neighbours needed where Nmax overflowed */
    const uint64_t* d_head_list;      /* NULL = column-major */
    uint64_t stride;
    uint32_t interleave;              /* column-major only: 1 or 4 (0 means 1) */
    const unsigned int* d_Nmax;       /* [ntypes] capacity per particle type */
    const float* d_pos;               /* float4[N] */
    unsigned int N;
    const unsigned int* d_cell_size;
    const float* d_xyzf;
    const unsigned int* d_cell_type;  /* required when ntypes > 1 */
    const unsigned int* d_cell_adj;
    unsigned int dim[3];
    unsigned int Nmax_cell;
    unsigned int adj_width;
    gb_box box;
    const float* d_r_cut;             /* [ntypes^2] */
    const float* d_r_listsq;          /* [ntypes^2] (r_cut + r_buff)^2, 0 where r_cut <= 0 */
    unsigned int ntypes;
    const uint32_t* d_gate;           /* optional no-op gate, as for the cell list */
    /* threads per block of the tiled builds: 32, 64 or 128 (0 = 128), a warp per cell (the
       kernel parameters the reference's Autotuner varies, block size and threads per particle,
       hoomd/md/NeighborListGPUBinned.cc:39-44) */
    uint32_t block_size;
    uint64_t nlist_capacity;          /* words allocated at d_nlist, or 0 when unknown; below 2^32
                                         the tiled builds address slots with 32-bit offsets,
                                         else the warp-per-cell form runs */
    /* threads testing each own particle in the tiled build: 32 = candidate stream (a warp's
       lanes hold 32 candidates and test them against one own particle at a time; the default,
       0 means 32), 1 = one lane per own particle. Both give the same lists, entry for entry. */
    uint32_t threads_per_particle;
    } gb_nlist_args;

int gb_nlist_build_binned(const gb_nlist_args* args, void* stream);

/* Exclusions. Replaces gpu_nlist_filter (hoomd/md/NeighborListGPU.cu:140-260): removes from each
 * particle's list the indices in its exclusion row d_ex_list[i * ex_pitch + e], e < d_n_ex[i],
 * keeping the order of the rest, and lowers d_n_neigh[i]. Same layouts as gb_nlist_build_binned
 * (flat with d_head_list, column-major with stride and interleave 1 or 4). d_gate as above. */
int gb_nlist_filter(unsigned int* d_nlist, unsigned int* d_n_neigh, const uint64_t* d_head_list,
                    uint64_t stride, uint32_t interleave, unsigned int N,
                    const unsigned int* d_n_ex, const unsigned int* d_ex_list,
                    unsigned int ex_pitch, const uint32_t* d_gate, void* stream);

/* Rebuild check. Replaces gpu_nlist_needs_update_check_new (hoomd/md/NeighborListGPU.cu:42-83):
 * sets *d_result = checkn when any particle moved at least (r_list*lambda_min - r_cut)/2 since
 * the last build. */
int gb_nlist_needs_update(uint32_t* d_result, const float* d_last_pos, const float* d_pos,
                          unsigned int N, const gb_box* box, const float* d_rcut_max,
                          float r_buff, unsigned int ntypes, float lambda_min,
                          const float lambda[3], uint32_t checkn, void* stream);

/* Head list for the flat layout: head[i] = sum_{k<i} Nmax[type k]
 * (NeighborListGPU.cu:355-448). d_total must hold 1 + ceil(N/1024) elements: element 0
 * receives the total, the rest is the scan's block-sum scratch. */
int gb_nlist_head_list(uint64_t* d_head_list, uint64_t* d_total, const float* d_pos,
                       unsigned int N, const unsigned int* d_Nmax, unsigned int ntypes,
                       void* stream);

/* ---------------------------------------------------------------------------------------------
 * Pair forces. Replaces gpu_compute_pair_forces<Evaluator> (hoomd/md/PotentialPairGPU.cuh:
 * 44-98 pair_args_t, 140-404 kernel, 579-656 driver). shift_mode: 0 none, 1 shift, 2 xplor.
 * The evaluator parameter structs below are byte-for-byte the FP32 param_type of the reference
 * evaluators. threads_per_particle: flat head lists take 1-32 (0 = 8); plain column-major lists
 * take 1; the interleaved list takes 1, 4 or 8 lanes per particle (0 = by N: 8 up to 16,384
 * particles, 4 up to 65,536, else 1; virials and XPLOR use 1). block_size: the interleaved list
 * takes 128 or 256 threads (0 = 256), the others a multiple of 32 up to 1024 (0 = 256); these
 * are the kernel parameters the reference's Autotuner varies (hoomd/md/PotentialPairGPU.h:76-81).
 * ------------------------------------------------------------------------------------------- */
typedef struct gb_pair_args
    {
    float* d_force;                   /* float4[N]: fx, fy, fz, energy (half of each pair) */
    float* d_virial;                  /* 6 x virial_pitch, written when compute_virial */
    size_t virial_pitch;
    unsigned int N;
    const float* d_pos;
    const float* d_charge;            /* unused by LJ, Table, Example */
    gb_box box;
    const unsigned int* d_n_neigh;
    const unsigned int* d_nlist;
    const uint64_t* d_head_list;      /* NULL = column-major */
    uint64_t stride;
    uint32_t interleave;              /* column-major only: 1 or 4 (0 means 1), as gb_nlist_args */
    const float* d_rcutsq;            /* [ntypes^2] */
    const float* d_ronsq;             /* [ntypes^2], read when shift_mode == 2 */
    unsigned int ntypes;
    unsigned int shift_mode;
    unsigned int compute_virial;
    unsigned int block_size;          /* 0 = default */
    unsigned int threads_per_particle;
    } gb_pair_args;

/* EvaluatorPairLJ::param_type at FP32 (hoomd/md/EvaluatorPairLJ.h:99-155). */
typedef struct gb_lj_param
    {
    float sigma_6;
    float epsilon_x_4;
    } gb_lj_param;

/* EvaluatorPairTable::param_type (hoomd/md/EvaluatorPairTable.h:45-118). The tables of all type
 * pairs share one device array of bins: bin k of a pair is the float quad
 * (V[k], F[k], V[k+1], F[k+1]) with V[width] = F[width] = 0 (the reference's last-bin rule), so
 * an evaluation reads one 16-byte quad. `offset` is the pair's first bin, in quads.
 * gb_table_pack writes a pair's quads from its U and F arrays. `reserved` must be 0. */
typedef struct gb_table_param
    {
    float rmin;
    uint32_t width;
    uint32_t offset;
    uint32_t reserved;
    } gb_table_param;

/* Host helper: pack width points of U and F into width quads (4 * width floats) at out. */
int gb_table_pack(const double* U, const double* F, uint32_t width, float* out);

/* EvaluatorPairExample::param_type (example_plugins/pair_plugin/EvaluatorPairExample.h:30-60). */
typedef struct gb_example_param
    {
    float k;
    float sigma;
    } gb_example_param;

int gb_pair_forces_lj(const gb_pair_args* args, const gb_lj_param* d_params, void* stream);
int gb_pair_forces_table(const gb_pair_args* args, const gb_table_param* d_params,
                         const float* d_table, void* stream);
int gb_pair_forces_example(const gb_pair_args* args, const gb_example_param* d_params,
                           void* stream);

/* The other radial evaluators of the reference, one kernel family selected by `kind` (uniform per
 * force, so the switch does not diverge). Parameters per kind, in v[0..5], as the reference's
 * param_type keys (hoomd/md/pair/pair.py), r in the formulas below:
 *   GAUSS       epsilon, sigma            eps exp(-r^2 / 2 sigma^2)   (EvaluatorPairGauss.h)
 *   YUKAWA      epsilon, kappa            eps exp(-kappa r) / r        (EvaluatorPairYukawa.h)
 *   MORSE       D0, alpha, r0             D0 [e^{-2a(r-r0)} - 2 e^{-a(r-r0)}] (EvaluatorPairMorse.h)
 *   FORCE_SHIFTED_LJ  sigma, epsilon      LJ(r) + (r - r_cut) F_LJ(r_cut) (EvaluatorPairForceShiftedLJ.h)
 *   MIE         epsilon, sigma, n, m      (n/(n-m)) (n/m)^(m/(n-m)) eps [(s/r)^n - (s/r)^m] (EvaluatorPairMie.h)
 *   EXPANDED_MIE  epsilon, sigma, n, m, delta   Mie at r - delta  (EvaluatorPairExpandedMie.h)
 *   EXPANDED_LJ   sigma, epsilon, delta   LJ at r - delta              (EvaluatorPairExpandedLJ.h)
 *   BUCKINGHAM  A, rho, C                 A exp(-r/rho) - C / r^6      (EvaluatorPairBuckingham.h)
 *   LJ1208      sigma, epsilon            4 eps [(s/r)^12 - (s/r)^8]   (EvaluatorPairLJ1208.h)
 *   LJ0804      sigma, epsilon            4 eps [(s/r)^8 - (s/r)^4]    (EvaluatorPairLJ0804.h)
 *   LJ_GAUSS    epsilon, sigma, r0        1/r^12 - 2/r^6 - eps exp(-(r-r0)^2 / 2 sigma^2) (EvaluatorPairLJGauss.h)
 *   EXPANDED_GAUSS  epsilon, sigma, delta eps exp(-(r-delta)^2 / 2 sigma^2) (EvaluatorPairExpandedGaussian.h)
 *   OPP         C1, C2, eta1, eta2, k, phi  C1 r^-eta1 + C2 r^-eta2 cos(k r - phi) (EvaluatorPairOPP.h)
 *   TWF         sigma, epsilon, alpha     4 eps/alpha^2 [s^-6 - alpha s^-3], s = (r/sigma)^2 - 1 (EvaluatorPairTWF.h)
 *   DPD_CONSERVATIVE  A                   A (r_c - r) - A (r_c^2 - r^2) / (2 r_c)  (EvaluatorPairDPDThermoDPD.h:190-208)
 *   DLVO        kappa, Z, A, a1, a2       screened repulsion + sphere-sphere van der Waals (EvaluatorPairDLVO.h:120-169)
 *   FOURIER     a1, a2, a3, b1, b2, b3    1/r^12 + sum_n [a_n cos(n pi r / r_c) + b_n sin(n pi r / r_c)] / r^2 (EvaluatorPairFourier.h:135-180)
 *   MOLIERE     qi, qj, aF                qi qj / r (0.35 e^{-0.3 r/aF} + 0.55 e^{-1.2 r/aF} + 0.1 e^{-6 r/aF}) (EvaluatorPairMoliere.h:112-148)
 *   ZBL         qi, qj, aF                the four-exponential ZBL screening (EvaluatorPairZBL.h:95-123)
 *   REACTION_FIELD  epsilon, eps_rf       eps [1/r + (eps_rf - 1) / (2 eps_rf + 1) r^2 / r_c^3] (EvaluatorPairReactionField.h:122-151)
 *   EWALD       kappa, alpha              real-space Ewald term, erfc screening (EvaluatorPairEwald.h:121-148)
 * The forms are for unit charges; when args->d_charge is given, every pair's force and energy
 * is multiplied by q_i q_j (the reference's needsCharge evaluators: Ewald always,
 * ReactionField with use_charge).
 * Shift mode 1 subtracts the energy at r_cut; XPLOR smoothing as for LJ. DLVO, MOLIERE, ZBL and
 * REACTION_FIELD give zero force where the reference's evaluators return false (kappa, qi qj,
 * aF or epsilon zero). */
typedef enum gb_radial_kind
    {
    GB_RADIAL_GAUSS = 0,
    GB_RADIAL_YUKAWA = 1,
    GB_RADIAL_MORSE = 2,
    GB_RADIAL_FORCE_SHIFTED_LJ = 3,
    GB_RADIAL_MIE = 4,
    GB_RADIAL_EXPANDED_MIE = 5,
    GB_RADIAL_EXPANDED_LJ = 6,
    GB_RADIAL_BUCKINGHAM = 7,
    GB_RADIAL_LJ1208 = 8,
    GB_RADIAL_LJ0804 = 9,
    GB_RADIAL_LJ_GAUSS = 10,
    GB_RADIAL_EXPANDED_GAUSS = 11,
    GB_RADIAL_OPP = 12,
    GB_RADIAL_TWF = 13,
    GB_RADIAL_DPD_CONSERVATIVE = 14,
    GB_RADIAL_DLVO = 15,
    GB_RADIAL_FOURIER = 16,
    GB_RADIAL_MOLIERE = 17,
    GB_RADIAL_ZBL = 18,
    GB_RADIAL_REACTION_FIELD = 19,
    GB_RADIAL_EWALD = 20,
    GB_RADIAL_KINDS = 21
    } gb_radial_kind;

typedef struct gb_radial_param
    {
    float v[6];
    uint32_t kind;      /* gb_radial_kind, the same for every type pair of one force */
    float aux;          /* 0 (the kernels fill it per type pair: F(r_cut) of FORCE_SHIFTED_LJ,
                           the Mie prefactor, or r_cut) */
    } gb_radial_param;

int gb_pair_forces_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                          void* stream);

/* Energy between two sets of particles: replaces PotentialPair<E>::computeEnergyBetweenSets
 * (hoomd/md/PotentialPair.h:833-990, bound as computeEnergyBetweenSets and called by
 * hoomd/md/pair/pair.py compute_energy), which sums on the host over every tag of set 1 and
 * every tag of set 2. U = sum_i m1[i] (sum_j m2[j] V_ij(r) + m2[i] V_ii(0)) with the force's
 * shift / XPLOR mode, j over particle i's row of the full list in args plus its exclusion row
 * (the reference applies no exclusions; the list has the excluded pairs filtered out, so they
 * are added back, each distinct partner once). d_mult1[i] / d_mult2[i] count how often particle
 * index i's tag appears in set 1 / set 2 (duplicates and overlapping sets count as the
 * reference's double loop counts them; a tag in both sets adds the evaluator at r = 0, as
 * there). d_n_ex may be NULL (no exclusions). The forces and virial fields of args are not
 * used. d_partials receives gb_pair_energy_sets_blocks(N) doubles whose sum, in order, is U.
 * With args->d_charge set, the radial entry scales by q_i q_j. */
typedef struct gb_energy_sets
    {
    const uint32_t* d_mult1;       /* [N] occurrences of index i's tag in set 1 */
    const uint32_t* d_mult2;       /* [N] occurrences of index i's tag in set 2 */
    const unsigned int* d_n_ex;    /* [N] exclusion row lengths (as gb_nlist_filter), or NULL */
    const unsigned int* d_ex_list; /* [N * ex_pitch] excluded indices */
    unsigned int ex_pitch;
    } gb_energy_sets;

unsigned int gb_pair_energy_sets_blocks(unsigned int N);
int gb_pair_energy_sets_lj(const gb_pair_args* args, const gb_lj_param* d_params,
                           const gb_energy_sets* sets, double* d_partials, void* stream);
int gb_pair_energy_sets_table(const gb_pair_args* args, const gb_table_param* d_params,
                              const float* d_table, const gb_energy_sets* sets,
                              double* d_partials, void* stream);
int gb_pair_energy_sets_example(const gb_pair_args* args, const gb_example_param* d_params,
                                const gb_energy_sets* sets, double* d_partials, void* stream);
int gb_pair_energy_sets_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                               const gb_energy_sets* sets, double* d_partials, void* stream);

/* DPD thermostat pair forces (EvaluatorPairDPDThermoDPD.h:190-272, EvaluatorPairDPDThermoLJ.h:
 * 216-276, PotentialPairDPDThermo.h:160-240): a conservative part (DPD: A (1 - r/r_c); DPDLJ:
 * the LJ force with lj1 = 4 eps sigma^12, lj2 = 4 eps sigma^6), a drag
 * -gamma w(r)^2 (r_ij . v_ij) / r with w = 1 - r/r_c, and a random force
 * sqrt(6 gamma kT / dt) w(r) alpha with alpha uniform in [-1, 1] drawn from Philox with
 * Seed(22, timestep, seed), Counter(min(tag_i, tag_j), max(tag_i, tag_j)), so both particles of a
 * pair draw the same number. Energies and the virial use the conservative part only.
 * Column-major list interleaved by 4 (args->interleave == 4). d_vel: float4[N] velocities (mass in
 * w); d_tag: [N] tags. lj = 0: DPD (param a), lj = 1: DPDLJ (lj1, lj2; shift_mode 1 subtracts the
 * LJ energy at r_cut). */
typedef struct gb_dpd_param
    {
    float a;     /* DPD conservative amplitude A */
    float lj1;   /* DPDLJ: 4 eps sigma^12 */
    float lj2;   /* DPDLJ: 4 eps sigma^6 */
    float gamma; /* drag coefficient */
    } gb_dpd_param;

int gb_pair_forces_dpd(const gb_pair_args* args, const gb_dpd_param* d_params,
                       const float* d_vel, const uint32_t* d_tag, int lj, uint64_t timestep,
                       uint16_t seed, float dt, float kT, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Integrator halves. Replace gpu_nvt_rescale_step_one / _two
 * (hoomd/md/TwoStepConstantVolumeGPU.cu:35-89, 166-205; with scale 1 these are the NVE halves of
 * hoomd/md/TwoStepNVEGPU.cu:46-124, 383-453). The rescale factor is read on the device from
 * d_scale (a double, e.g. written by gb_bussi_factor) or taken as `scale` when d_scale is NULL.
 * ------------------------------------------------------------------------------------------- */
int gb_cv_step_one(float* d_pos, float* d_vel, const float* d_accel, int* d_image,
                   unsigned int N, const gb_box* box, float dt, float scale,
                   const double* d_scale, void* stream);
int gb_cv_step_two(float* d_vel, float* d_accel, const float* d_net_force, unsigned int N,
                   float dt, float scale, const double* d_scale, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Thermodynamic reductions in FP64. Replace gpu_compute_thermo_partial_sums / final_sums
 * (hoomd/md/ComputeThermoGPU.cu:46-120, 326-...), whose partial sums are in Scalar; here every
 * per-particle term is widened to double before it is summed, in a fixed order (deterministic).
 * d_out receives [0] translational KE, [1] potential energy, [2] W = sum(virial xx+yy+zz)/3
 * (0 when d_virial is NULL).
 * d_scratch is caller-provided global scratch of gb_thermo_scratch_bytes(N) bytes; its counter
 * word must be zero before the first call (cudaMemset once); the kernel leaves it zero.
 * ------------------------------------------------------------------------------------------- */
size_t gb_thermo_scratch_bytes(unsigned int N);
int gb_thermo_reduce(const float* d_vel, const float* d_force, const float* d_virial,
                     size_t virial_pitch, unsigned int N, void* d_scratch, double* d_out,
                     void* stream);

/* Allocation-free variant of gb_thermo_reduce; it has no counterpart in the reference. It is for
 * callers that cannot allocate device memory: a host that has given all device memory to its own
 * pool and forbids side allocations, or one that must not stall the GPU (cudaFree synchronises
 * the device), and so cannot pass the d_scratch buffer gb_thermo_reduce needs. Its scratch is a
 * fixed array inside the library (GB_NOALLOC_MAX_N particles' worth, 384.25 KiB), resident on
 * every GPU that loads the library until the process exits. N > GB_NOALLOC_MAX_N returns
 * GB_ERR_TOO_LARGE. The first call in each CUDA context (once per device; again after a
 * cudaDeviceReset or under another context) looks up the array's address with that context
 * current; make it before any stream capture. All calls share the array: calls that overlap on
 * the GPU race. Outputs as gb_thermo_reduce; no cudaMalloc or cudaFree is ever called. */
#define GB_NOALLOC_MAX_N 4194304u
int gb_thermo_reduce_noalloc(const float* d_vel, const float* d_force, const float* d_virial,
                             size_t virial_pitch, unsigned int N, double* d_out, void* stream);

/* Bussi stochastic velocity rescaling factor on the device (hoomd/md/Thermostat.h:357-446):
 * reads K = d_ke[0], draws with Philox4x32-10 key Seed(45, timestep, seed) and counter
 * instance_id, writes the factor (double) to d_factor. */
int gb_bussi_factor(const double* d_ke, double dof, double dt, double tau, double kT,
                    uint64_t timestep, uint16_t seed, uint32_t instance_id, double* d_factor,
                    void* stream);

/* ParticleGroup::thermalizeParticleMomenta for point particles (hoomd/ParticleGroup.cc:690-760):
 * per-particle Gaussian velocities (Philox key Seed(35, timestep, seed), counter = tag) and
 * removal of the centre-of-mass momentum (summed in double). d_scratch as for thermo. */
int gb_thermalize(float* d_vel, const uint32_t* d_tag, unsigned int N, double kT,
                  uint64_t timestep, uint16_t seed, unsigned int ndim, void* d_scratch,
                  void* stream);

/* Conditional graph nodes (GB300 design, no reference counterpart): inside a captured CUDA graph,
 * sets the value of the conditional node `handle` (a cudaGraphConditionalHandle created on that
 * graph) to (*d_flag != 0). The captured MD step uses it to run the cell-list and neighbour-list
 * build of a step only when the step's rebuild check raised the flag, instead of launching the
 * gated build kernels every step. */
int gb_graph_set_conditional(uint64_t handle, const uint32_t* d_flag, void* stream);

/* Advances the device step counter by one (the steps of methods whose second half is not the
 * fused pair step, which advances it itself), so the rebuild-check schedule and the rebuild
 * statistics see the current step. */
int gb_step_counter_advance(uint64_t* d_timestep, void* stream);

/* Snapshot transfer on the device: the per-particle loops of ParticleData::takeSnapshot
 * (hoomd/ParticleData.cc:1388-1617) and ParticleData::initializeFromSnapshot
 * (hoomd/ParticleData.cc:982-1379), which the reference runs on the host. Snapshot arrays are in
 * tag order and FP64 (positions and velocities 3 per particle, images 3 int32); the particle
 * arrays are in index order (positions float4 x, y, z, type bits; velocities float4 with the
 * mass; images int3; tags).
 * gb_snapshot_gather writes the tag-ordered arrays from the particle arrays.
 * gb_rtag writes rtag[tag[i]] = i (the reference's reverse-tag table).
 * gb_snapshot_scatter places tag t at index d_rtag[t] (d_rtag NULL: index t), wrapping the
 * position into the box with the image updated; d_in_charge may be NULL (charges left as they
 * are). A type id >= ntypes is not written: *d_err receives the smallest such tag (set *d_err to
 * 0xFFFFFFFF before the call). gb_snapshot_stage_bytes(N) is the size of one staging block that
 * holds every snapshot array of N particles, each section 256-byte aligned (pos, vel, mass,
 * charge, typeid, image, rtag). */
size_t gb_snapshot_stage_bytes(unsigned int N);
int gb_snapshot_gather(const float* d_pos, const float* d_vel, const int32_t* d_image,
                       const uint32_t* d_tag, unsigned int N, double* d_out_pos,
                       double* d_out_vel, double* d_out_mass, uint32_t* d_out_typeid,
                       int32_t* d_out_image, void* stream);
int gb_rtag(const uint32_t* d_tag, unsigned int N, uint32_t* d_rtag, void* stream);
int gb_snapshot_scatter(const double* d_in_pos, const double* d_in_vel, const double* d_in_mass,
                        const uint32_t* d_in_typeid, const int32_t* d_in_image,
                        const double* d_in_charge, const uint32_t* d_rtag, unsigned int N,
                        unsigned int ntypes, const gb_box* box, float* d_pos, float* d_vel,
                        int32_t* d_image, uint32_t* d_tag, float* d_charge, uint32_t* d_err,
                        void* stream);


/* ---------------------------------------------------------------------------------------------
 * Fused whole-step kernels (GB300 design; no single reference counterpart). One MD step of
 * IntegratorTwoStep::update (hoomd/md/IntegratorTwoStep.cc:51-139) for one ConstantVolume method
 * and one pair force runs as two kernels plus the rebuild kernels:
 *   gb_md_step_one      step one (gpu_nvt_rescale_step_one) + the rebuild check
 *                       (gpu_nlist_needs_update_check_new) in one pass over the particles;
 *   [gb_cell_list_build + gb_nlist_build_binned, gated on the device by the rebuild flag]
 *   gb_md_pair_step_*   pair forces + step two (gpu_nvt_rescale_step_two) + FP64 kinetic and
 *                       potential energy reductions + the Bussi factor for the next step.
 * No host synchronisation is needed between steps, so a run of steps can be captured into a
 * CUDA graph and replayed.
 * ------------------------------------------------------------------------------------------- */
typedef struct gb_step_one_args
    {
    float* d_pos;
    float* d_vel;
    const float* d_accel;       /* float3[N] */
    int* d_image;               /* int3[N] */
    unsigned int N;
    gb_box box;
    float dt;
    float scale;                /* used when d_scale is NULL */
    const double* d_scale;      /* device rescale factor (Bussi) or NULL */
    /* rebuild check, skipped when d_last_pos is NULL */
    const float* d_last_pos;    /* float4[N] positions at the last build */
    const float* d_rcut_max;    /* [ntypes] */
    float r_buff;
    uint32_t* d_rebuild;        /* set to 1 when any particle moved >= (r_buff)/2 */
    /* 0: TwoStepConstantVolume order (v += a dt/2, v *= s, x += v dt); 1: TwoStepNVE order
       (x += v dt + a dt^2/2, then v += a dt/2; hoomd/md/TwoStepNVEGPU.cu:68-98), which the
       Langevin method uses (hoomd/md/TwoStepLangevin.cc:57-81); scale is ignored */
    int nve_order;
    /* MTTK (Nose-Hoover) thermostat, hoomd/md/Thermostat.h:119-212 with the call order of
       hoomd/md/TwoStepConstantVolume.cc:7-80, 205-210: when d_mttk_state is given, step one scales
       the half-step velocities by exp(-xi dt/2) (not by scale / d_scale), reduces their kinetic
       energy in FP64, advances (xi, eta) with T = 2 KE / mttk_dof against mttk_kT, and writes
       exp(-xi dt/2) of the advanced xi to *d_mttk_scale2 for step two */
    double* d_mttk_state;       /* [2]: xi, eta */
    double* d_mttk_scale2;
    double mttk_dof, mttk_kT, mttk_tau;
    void* d_mttk_scratch;       /* gb_thermo_scratch_bytes(N), zeroed once before first use */
    /* DisplacementCapped (hoomd/md/TwoStepConstantVolume.cc:44-52): when > 0 (ConstantVolume
       order), velocities with |v| dt above this length are scaled down to it */
    float max_displacement;
    /* Brownian dynamics, TwoStepBD::integrateStepOne (hoomd/md/TwoStepBD.cc:47-151), instead of
       the velocity-Verlet half: x += (F + F_r) dt / gamma, F_r uniform of amplitude
       sqrt(6 gamma kT / dt) from Philox Seed(24, timestep, seed), Counter(tag); velocities drawn
       from NormalDistribution(sqrt(kT / m)) of the same stream, or set to F / gamma when
       noiseless (OverdampedViscous). Excludes nve_order and MTTK; scale is ignored. */
    int brownian;
    const float* d_bd_force;    /* float4[N] net force at the current positions */
    const uint32_t* d_tag;      /* [N] */
    const float* d_gamma;       /* [ntypes] */
    float bd_kT;
    uint32_t ndim;              /* 2: no random force or velocity along z */
    uint32_t seed;              /* low 16 bits */
    const uint64_t* d_timestep; /* current step on the device; NULL = use timestep */
    uint64_t timestep;
    int noiseless;
    /* Schedule of the rebuild check, NeighborList::shouldCheckDistance / needsUpdating
     * (hoomd/md/NeighborList.cc:1313-1403), applied when d_last_update is non-NULL (NULL: the
     * distance check every step, i.e. rebuild_check_delay = 1 with check_dist). The check is for
     * step T = *d_check_step + 1 (the step whose forces follow); *d_last_update is the step of
     * the last build (d_build_steps[0] of gb_cell_list_args). While T < last + check_delay nothing is checked. Otherwise the flag is
     * raised without a distance check when r_buff < 1e-6, or without check_dist when
     * check_delay is 0 or T == last + check_delay (check_delay > 1); in every other case the
     * distance check decides. */
    const uint64_t* d_check_step;
    const uint64_t* d_last_update;
    uint32_t check_delay;
    int check_dist;
    /* optional: n_zero_words words at d_zero_words are set to zero by the same launch (the cell
       counts of the build that may follow, gb_cell_list_args.counts_zeroed) */
    uint32_t* d_zero_words;
    uint32_t n_zero_words;
    } gb_step_one_args;

int gb_md_step_one(const gb_step_one_args* args, void* stream);

typedef struct gb_step_fuse
    {
    float* d_vel;               /* float4[N] in/out */
    float* d_accel;             /* float3[N] out */
    float dt;
    const double* d_scale2;     /* step-two rescale factor or NULL (= 1) */
    void* d_scratch;            /* gb_md_step_scratch_bytes(N); zeroed once before first use */
    double* d_thermo;           /* [3] out: translational KE, potential energy, W */
    int bussi;                  /* draw the next step's Bussi factor into d_factor */
    double dof, tau, kT;
    uint32_t seed;              /* low 16 bits used, as the reference's Seed */
    uint32_t instance_id;       /* tag of the first group member */
    uint64_t* d_timestep;       /* current step; incremented by one per call */
    double* d_factor;
    uint32_t* d_status;         /* bit 0 set: Bussi factor requested with zero kinetic energy */
    uint32_t* d_rebuild_reset;  /* optional: set to 0 once the step is complete (clears the
                                   rebuild flag that gated this step's neighbour-list build) */
    const double* d_bussi_ring; /* optional: pairs (normal, 2*gamma) drawn ahead by
                                   gb_bussi_draws, at index timestep % bussi_ring_size; NULL =
                                   draw in the kernel's last block */
    uint32_t bussi_ring_size;
    /* Langevin step two (hoomd/md/TwoStepLangevin.cc:206-290) instead of the rescaled one:
       drag -gamma v plus a uniform random force of amplitude sqrt(6 gamma kT / dt), drawn from
       Philox with Seed(25, timestep, seed), Counter(tag); excludes bussi and d_scale2 */
    int langevin;
    const uint32_t* d_tag;      /* [N] particle tag of each index */
    const float* d_pos;         /* float4[N] positions (type in w) */
    const float* d_gamma;       /* [ntypes] drag coefficients */
    float langevin_kT;
    uint32_t ndim;              /* 2: no random or drag force along z */
    double* d_reservoir;        /* optional: reservoir energy, reduced by dt * sum(F_bd . v) */
    /* Berendsen thermostat (hoomd/md/Thermostat.h:450-490): write the next step one's factor
       sqrt(1 + dt/tau (kT / T - 1)), T = 2 KE / dof, into d_factor; bit 1 of d_status when the
       kinetic energy is zero. Excludes bussi and langevin */
    int berendsen;
    /* Brownian dynamics has no second half: the epilogue writes the forces and the sums (KE of
       the velocities step one drew, PE) and leaves the velocities as they are */
    int brownian;
    } gb_step_fuse;

/* The Berendsen factor from a kinetic energy on the device (the first step of a run). */
int gb_berendsen_factor(const double* d_ke, double dof, double dt, double tau, double kT,
                        double* d_factor, uint32_t* d_status, void* stream);

/* One NormalDistribution<double>(sigma) draw (hoomd/RandomNumbers.h:346-372) from Philox with
 * Seed(id, timestep, seed), Counter(counter), into *d_out: the MTTK thermostat's
 * thermalize_dof (hoomd/md/Thermostat.h:273-300, id 28). */
int gb_normal_draw(uint8_t id, uint64_t timestep, uint16_t seed, uint32_t counter, double sigma,
                   double* d_out, void* stream);

/* Langevin step two on its own (the unfused path: several forces, the virial, the MLP
 * surrogate): a = (F_net + F_bd) / m, v += a dt/2 for all N particles at timestep *d_timestep
 * (incremented by one when the step is done), then the FP64 sums into d_thermo (KE, PE, 0) and,
 * when d_reservoir is given, *d_reservoir -= dt * sum(F_bd . v).
 * d_scratch: gb_md_step_scratch_bytes(N), zeroed once before first use. */
int gb_langevin_step_two(float* d_vel, float* d_accel, const float* d_net_force,
                         const float* d_pos, const uint32_t* d_tag, const float* d_gamma,
                         unsigned int N, float dt, float kT, uint32_t ndim, uint16_t seed,
                         uint64_t* d_timestep, void* d_scratch, double* d_thermo,
                         double* d_reservoir, void* stream);

/* Pre-draws the random numbers of the Bussi factor (hoomd/md/Thermostat.h:416-446) for timesteps
 * *d_timestep + 1 ... *d_timestep + count, one thread per timestep, into
 * d_ring[t % ring_size] as (normal, 2 * Gamma((dof - 1)/2, 1)). The draws depend only on the
 * timestep, seed, counter and dof, so the factor computed from them later equals the one drawn
 * at that step. count <= ring_size. */
int gb_bussi_draws(const uint64_t* d_timestep, unsigned int count, double dof, uint16_t seed,
                   uint32_t instance_id, double* d_ring, unsigned int ring_size, void* stream);

/* ConstantPressure halves (hoomd/md/TwoStepConstantPressure.cc:206-330, 587-640), translational
 * part. The propagators are upper-triangular 3x3 matrices given as (xx, xy, xz, yy, yz, zz).
 * Step one: v += dt/2 a; v = M_v v; v *= scale; r = M_r r; r += M_r,int v; wrap into new_box
 * (the box already scaled by M_r). Step two: a = F/m; v *= scale; v = M_v v; v += dt/2 a. */
int gb_npt_step_one(float* d_pos, float* d_vel, const float* d_accel, int* d_image,
                    unsigned int N, const gb_box* new_box, float dt, float scale,
                    const float* mat_exp_v, const float* mat_exp_r, const float* mat_exp_r_int,
                    void* stream);
int gb_npt_step_two(float* d_vel, float* d_accel, const float* d_net_force, unsigned int N,
                    float dt, float scale, const float* mat_exp_v, void* stream);

/* Kinetic and virial tensors for the pressure tensor (ComputeThermo::computeProperties,
 * hoomd/md/ComputeThermo.cc:76-290), summed in FP64 in a fixed order: d_out[0..5] =
 * sum m v_a v_b (xx, xy, xz, yy, yz, zz), d_out[6..11] = sum of the per-particle virial
 * (6 x virial_pitch, may be NULL), d_out[12] = sum of the force array's energies (may be NULL).
 * d_scratch: gb_thermo_tensor_scratch_bytes(N). */
size_t gb_thermo_tensor_scratch_bytes(unsigned int N);
int gb_thermo_tensor(const float* d_vel, const float* d_force, const float* d_virial,
                     size_t virial_pitch, unsigned int N, void* d_scratch, double* d_out,
                     void* stream);

/* Net force (hoomd/Integrator.cu:68-170 gpu_integrator_sum_net_force): d_net[i] = sum over the
 * n_forces force arrays (float4; energy in w), n_forces <= 8. */
int gb_sum_net_force(float* d_net, const float* const* h_force_ptrs, unsigned int n_forces,
                     unsigned int N, void* stream);

size_t gb_md_step_scratch_bytes(unsigned int N);
int gb_md_pair_step_lj(const gb_pair_args* args, const gb_lj_param* d_params,
                       const gb_step_fuse* fuse, void* stream);
int gb_md_pair_step_table(const gb_pair_args* args, const gb_table_param* d_params,
                          const float* d_table, const gb_step_fuse* fuse, void* stream);
int gb_md_pair_step_example(const gb_pair_args* args, const gb_example_param* d_params,
                            const gb_step_fuse* fuse, void* stream);
int gb_md_pair_step_radial(const gb_pair_args* args, const gb_radial_param* d_params,
                           const gb_step_fuse* fuse, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Space-filling-curve sort. Replaces SFCPackTunerGPU (hoomd/SFCPackTunerGPU.cu:26-160) and
 * SFCPackTuner::getSortedOrder3D / 2D (hoomd/SFCPackTuner.cc:289-651): particles binned on a
 * 2^grid_bits per side lattice of the box as the reference bins them ((unsigned)(f * grid) %
 * grid), ordered by their bin's position along the reference's Hilbert traversal
 * (generateTraversalOrder; in 2D, bins row by row), ties by old index -- the reference's order.
 * The reference's default grid is 256 = 2^8 (3D), 4096 = 2^12 (2D). d_order[new] = old index;
 * deterministic. d_scratch of gb_sfc_scratch_bytes[_dim](). gb_sfc_order is the 3D form.
 * gb_gather applies the order to one per-particle array (dst[i] = src[order[i]]; elements of
 * 4, 8, 12 or 16 bytes; dst and src must differ), as gpu_apply_sorted_order does.
 * ------------------------------------------------------------------------------------------- */
size_t gb_sfc_scratch_bytes(unsigned int N, int grid_bits);
int gb_sfc_order(const float* d_pos, unsigned int N, const gb_box* box, int grid_bits,
                 uint32_t* d_order, void* d_scratch, size_t scratch_bytes, void* stream);
size_t gb_sfc_scratch_bytes_dim(unsigned int N, int grid_bits, unsigned int ndim);
int gb_sfc_order_dim(const float* d_pos, unsigned int N, const gb_box* box, int grid_bits,
                     unsigned int ndim, uint32_t* d_order, void* d_scratch, size_t scratch_bytes,
                     void* stream);
int gb_gather(void* d_dst, const void* d_src, const uint32_t* d_order, unsigned int N,
              unsigned int elem_bytes, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Replica ensembles (GB300 design; the reference runs one Simulation per process, so a batch of
 * R systems is R separate runs of the path above: IntegratorTwoStep::update with
 * TwoStepConstantVolume + BussiThermostat, NeighborListGPUBinned and PotentialPairGPU<LJ>).
 * Many independent single-type LJ systems of uneven size advance in ONE persistent launch. Each
 * CTA takes the next replica from a device queue (the caller orders it, largest first) and runs
 * all of that replica's steps with block barriers only -- step one with the rebuild check, an
 * in-CTA cell list (counting sort, deterministic order) and neighbour-list build when the check
 * fires, then pair forces + step two + FP64 kinetic/potential energy sums + the Bussi factor for
 * the next step -- before it takes the next replica. No CTA ever waits for another.
 *
 * A replica's results do not depend on the launch shape: its neighbour order follows the
 * deterministic cell list, each particle sums its own forces, and the energy sums run over fixed
 * 32-particle chunks in a fixed order. block_size and grid_size can therefore be tuned on live
 * steps without changing any trajectory.
 *
 * Per-particle arrays are shared by all replicas: replica r owns elements [first, first + N).
 * Positions float4 (x, y, z, type bits = 0), velocities float4 (vx, vy, vz, mass),
 * accelerations float4 (ax, ay, az, 0), images int4 (ix, iy, iz, 0), forces float4 (fx, fy, fz,
 * energy), last-build positions float4. The neighbour list of replica r starts at word
 * nlist_offset of d_nlist: element k of its particle i is at word
 * nlist_offset + ((k / 4) * stride + i) * 4 + k % 4.
 * ------------------------------------------------------------------------------------------- */
#define GB_REPLICA_OVERFLOW 1u      /* the neighbour list needs `needed` > Nmax slots */
#define GB_REPLICA_NAN 2u           /* a position is NaN (hoomd/CellListGPU.cu:89-94) */
#define GB_REPLICA_OUTSIDE 4u       /* a particle left the box (hoomd/CellListGPU.cu:96-110) */
#define GB_REPLICA_ZERO_KE 8u       /* Bussi factor requested with zero kinetic energy */
#define GB_REPLICA_CONFIG 16u       /* the cell grid exceeds the launch's max_cells */
#define GB_REPLICA_MAX_BLOCK 1024u

typedef struct gb_replica
    {
    /* set by the caller */
    gb_box box;                 /* fully periodic; every perpendicular width >= 2 r_list */
    uint32_t N;
    uint32_t stride;            /* neighbour-list column stride: >= N, multiple of 32 */
    uint64_t first;             /* first particle in the shared arrays: multiple of 32 */
    uint64_t nlist_offset;      /* in uint32 words, multiple of 4 */
    uint32_t Nmax;              /* neighbour capacity per particle: multiple of 4 */
    uint32_t dim[3];            /* cell grid: width >= r_list / stencil in every direction */
    gb_lj_param lj;             /* EvaluatorPairLJ parameters of the one type pair */
    float r_cut;
    float r_buff;
    uint32_t shift_mode;        /* 0 none, 1 shift (hoomd/md/PotentialPair.h:255-341) */
    uint32_t bussi;             /* 1: ConstantVolume + Bussi; 0: NVE */
    uint32_t seed;              /* low 16 bits, as the reference's Seed */
    uint32_t stencil;           /* cells searched on each side of a particle's cell: 1 or 2 */
    double dt;                  /* rounded to float for the half steps, as a double for Bussi */
    double kT, tau, dof;
    uint64_t target;            /* advance until timestep == target */
    /* state: initialised by the caller (zeros, timestep, factor 1), then owned by the kernel */
    uint64_t timestep;
    double factor;              /* Bussi factor of the step that starts at `timestep` */
    double ke, pe;              /* translational kinetic and potential energy after the last step */
    uint64_t n_builds;
    uint32_t prepared;          /* forces and accelerations at `timestep` are current */
    uint32_t pending_build;     /* step one of the step at `timestep` is done; its neighbour
                                   list must be built before the step can finish */
    uint32_t status;            /* GB_REPLICA_* bits; the replica stops when any is set */
    uint32_t needed;            /* with GB_REPLICA_OVERFLOW: the neighbour count to fit */
    } gb_replica;

typedef struct gb_replica_batch
    {
    gb_replica* d_replicas;     /* [n_replicas], device */
    uint32_t n_replicas;
    const uint32_t* d_order;    /* [n_replicas] queue order (replica ids), device */
    uint32_t* d_queue;          /* two words, zero before the first launch; left zero */
    float* d_pos;
    float* d_vel;
    float* d_accel;
    int* d_image;
    float* d_force;
    float* d_last_pos;
    uint32_t* d_n_neigh;
    uint32_t* d_nlist;
    void* d_scratch;            /* gb_replica_scratch_bytes(total particle slots) */
    uint64_t n_slots;           /* length of the per-particle arrays (>= every first + N) */
    uint32_t max_cells;         /* largest dim[0] * dim[1] * dim[2] among the replicas */
    uint32_t block_size;        /* threads per CTA: multiple of 32, 64 ... 1024 */
    uint32_t grid_size;         /* persistent CTAs; 0 = every CTA that fits at once */
    uint64_t* d_phase_clocks;   /* optional [4 * n_replicas]: SM clock cycles the replica's CTA
                                   spent in step one, list builds, pair step, Bussi draws;
                                   accumulated (NULL = not recorded) */
    } gb_replica_batch;

size_t gb_replica_scratch_bytes(uint64_t n_slots);
/* Dynamic shared memory of one CTA; also the check that max_cells fits (0 = does not fit). */
size_t gb_replica_smem_bytes(uint32_t max_cells, uint32_t block_size);
/* CTAs of block_size threads resident per SM (0 = the shape cannot launch). */
int gb_replica_ctas_per_sm(uint32_t max_cells, uint32_t block_size);
int gb_replicas_run(const gb_replica_batch* batch, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Radial MLP surrogate of the Table pair potential (GB300 design; it stands in for
 * EvaluatorPairTable, hoomd/md/EvaluatorPairTable.h, on many type pairs at once). Per unordered
 * type pair p = (a <= b), index a*ntypes - a(a-1)/2 + (b - a), and distance r in [r_min, r_cut):
 *   phi_k(r) = exp(-gamma (r - mu_k)^2), mu_k = r_min + k h, h = (r_cut - r_min)/31,
 *              gamma = 1/(2 h^2), k = 0..31
 *   z1 = W1e E[p] + W1r phi + b1, h1 = silu(z1);  z2 = W2 h1 + b2, h2 = silu(z2);
 *   U = w3 . h2 + b3,  F(r) = -dU/dr (analytic, forward-mode through the same layers).
 * Parameters are one float array (offsets in floats; P = ntypes (ntypes + 1) / 2):
 *   W1e[64][16] @ 0, W1r[64][32] @ 1024, b1[64] @ 3072, W2[64][64] @ 3136, b2[64] @ 7232,
 *   w3[64] @ 7296, b3 @ 7360, E[P][16] @ 7424; gb_mlp_param_count(P) floats in all.
 * Inference (gb_mlp_prepare / gb_mlp_eval / gb_mlp_forces) runs the two 64-wide layers and their
 * derivative on BF16 tensor cores with FP32 accumulation: E, W1e, W1r, W2, w3 are rounded to
 * bfloat16; phi, dphi/dr, h1, dh1/dr enter the products as bfloat16 (act_split 0) or as the sum
 * of two bfloat16 numbers (act_split 1). Training (gb_mlp_loss_grad) evaluates the same function
 * in FP32 and returns the gradient of
 *   L = (1/B) sum_s [ (dU/dr_s + F_s)^2 + lam (U_s - U_s^target)^2 ]
 * with the rounding (quant = 0 none, 1 bfloat16, 2 two-term bfloat16) applied straight-through.
 * ------------------------------------------------------------------------------------------- */
#define GB_MLP_EMB 16u
#define GB_MLP_RBF 32u
#define GB_MLP_HID 64u

size_t gb_mlp_param_count(uint32_t n_pairs);
size_t gb_mlp_train_scratch_bytes(uint32_t batch);
/* d_grad (param_count floats) is overwritten; *d_loss (double) receives L. */
int gb_mlp_loss_grad(const float* d_theta, uint32_t n_pairs, float r_min, float r_cut,
                     const uint32_t* d_pair, const float* d_r, const float* d_U,
                     const float* d_F, uint32_t batch, float lam, int quant, float* d_grad,
                     double* d_loss, void* d_scratch, void* stream);
/* Adam (Kingma & Ba 2015) with bias correction; step counts from 1. */
int gb_mlp_adam(float* d_theta, const float* d_grad, float* d_m, float* d_v, size_t n, float lr,
                float beta1, float beta2, float eps, uint32_t step, void* stream);

/* Inference block: per-pair first-layer offsets C[p] = W1e E[p] + b1 (FP32) and the bfloat16
 * weights laid out as tensor-core operand fragments. */
size_t gb_mlp_infer_bytes(uint32_t n_pairs);
int gb_mlp_prepare(const float* d_theta, uint32_t n_pairs, void* d_infer, void* stream);
/* U and dU/dr of n samples (pair index, r) on the tensor-core path (tests). */
int gb_mlp_eval(const void* d_infer, uint32_t n_pairs, float r_min, float r_cut, int act_split,
                const uint32_t* d_pair, const float* d_r, uint32_t n, float* d_U, float* d_dU,
                void* stream);

/* Pair forces of the surrogate over a column-major interleaved-by-4 full neighbour list (the
 * layout of gb_nlist_build_binned with interleave 4): each unordered pair within
 * [r_min, r_cut) is evaluated once and its force added to both particles with atomics.
 * d_force (float4[N]: fx, fy, fz, energy) is overwritten. Orthorhombic or triclinic periodic
 * boxes. d_scratch: gb_mlp_forces_scratch_bytes(N, Nmax). */
typedef struct gb_mlp_force_args
    {
    float* d_force;
    const float* d_pos;               /* float4[N], type bits in w */
    unsigned int N;
    gb_box box;
    const unsigned int* d_n_neigh;
    const unsigned int* d_nlist;
    uint64_t stride;
    unsigned int Nmax;                /* capacity per particle (largest over types) */
    unsigned int ntypes;
    float r_min, r_cut;
    int act_split;
    const void* d_infer;
    void* d_scratch;
    /* 0: tcgen05 tiles of 128 pairs (operands in shared memory, FP32 accumulators in tensor
       memory, one CTA of 256 threads per tile, two per SM); 1: the mma.sync path (one warp per
       tile of 16 pairs, accumulators in registers). The tcgen05 path writes 1 to the second
       word of d_scratch when a wait for its products ran out (the forces are then incomplete). */
    int mma_sync;
    } gb_mlp_force_args;
size_t gb_mlp_forces_scratch_bytes(unsigned int N, unsigned int Nmax);
int gb_mlp_forces(const gb_mlp_force_args* args, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Pair-evaluator plugins. The reference's example_plugins/pair_plugin compiles an evaluator with
 * the reference's concept (EvaluatorPairExample.h: param_type, a three-argument constructor,
 * evalForceAndEnergy, ...) into its own module: PotentialPairExampleGPUKernel.cu explicitly
 * instantiates gpu_compute_pair_forces<Evaluator> (hoomd/md/PotentialPairGPU.cuh:579-656) and
 * module.cc calls export_PotentialPairGPU<Evaluator> (example_plugins/pair_plugin/module.cc:
 * 20-26). The headers under include/hoomd/ give those two files the same names here: the
 * instantiation compiles this library's pair kernels for the evaluator, and the export hands the
 * engine one gb_pair_plugin record. Every kernel call of the evaluator goes through its `call`
 * function with one gb_pair_plugin_call.
 * ------------------------------------------------------------------------------------------- */
typedef struct gb_pair_plugin_call
    {
    int op;                        /* 0: forces (+ virial if args->compute_virial), as
                                      gb_pair_forces_*; 1: the fused pair step, as
                                      gb_md_pair_step_*; 2: energy between sets, as
                                      gb_pair_energy_sets_* */
    const gb_pair_args* args;
    const gb_step_fuse* fuse;      /* op 1 */
    const gb_energy_sets* sets;    /* op 2 */
    double* d_partials;            /* op 2 */
    void* stream;
    int status;                    /* out: GB_OK or the gb_status of the failure */
    } gb_pair_plugin_call;

#define GB_PAIR_PLUGIN_ABI 1
typedef struct gb_pair_plugin
    {
    uint32_t abi;                  /* GB_PAIR_PLUGIN_ABI */
    uint32_t param_size;           /* sizeof(Evaluator::param_type) at FP32 */
    /* runs one call on the evaluator's kernels; d_params: ntypes^2 param_type records */
    int (*call)(gb_pair_plugin_call* call, const void* d_params);
    const char* name;              /* Evaluator::getName() */
    } gb_pair_plugin;

#ifdef __cplusplus
}
#endif

#endif /* HOOMD_GB300_H */
