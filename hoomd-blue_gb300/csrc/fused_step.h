// Conversion of the C-ABI gb_step_fuse into the pair kernel's epilogue arguments.
#pragma once

#include "pair_kernel.cuh"

namespace gb
{
// Scratch layout: [0, 256) counter word; [256, ...) 3 doubles per block of the pair kernel. The
// kernel may run up to 8 lanes per particle (small systems) in blocks of 128 or 256 threads, so
// room for 8 N threads in blocks of 128.
inline size_t step_scratch_bytes(unsigned int N)
    {
    return 256 + 3 * sizeof(double) * (size_t)div_up(8ull * (N > 0 ? N : 1), 128);
    }

inline int make_fuse_args(const gb_pair_args* a, const gb_step_fuse* f, FuseArgs& fz)
    {
    GB_REQUIRE(a && f, "fused step: null argument");
    GB_REQUIRE(f->d_vel && f->d_accel && f->d_scratch && f->d_thermo,
               "fused step: velocities, accelerations, scratch and thermo output are required");
    GB_REQUIRE(a->d_head_list == nullptr, "fused step: column-major neighbour list required");
    GB_REQUIRE(a->block_size == 0 || a->block_size == 128 || a->block_size == 256,
               "fused step: block size 128 or 256");
    GB_REQUIRE(!f->bussi || (f->d_timestep && f->d_factor && f->d_status),
               "fused step: Bussi needs timestep, factor and status buffers");
    fz.vel = reinterpret_cast<float4*>(f->d_vel);
    fz.accel = f->d_accel;
    fz.dt = f->dt;
    fz.d_scale2 = f->d_scale2;
    fz.counter = reinterpret_cast<unsigned int*>(f->d_scratch);
    fz.partials = reinterpret_cast<double*>(reinterpret_cast<char*>(f->d_scratch) + 256);
    fz.out = f->d_thermo;
    fz.bussi = f->bussi;
    fz.dof = f->dof;
    fz.tau = f->tau;
    fz.kT = f->kT;
    fz.dt_d = (double)f->dt;
    fz.seed = (uint16_t)f->seed;
    fz.instance_id = f->instance_id;
    fz.d_timestep = f->d_timestep;
    fz.d_factor = f->d_factor;
    fz.d_status = f->d_status;
    fz.d_rebuild_reset = f->d_rebuild_reset;
    GB_REQUIRE(!f->d_bussi_ring || f->bussi_ring_size > 0, "fused step: empty Bussi ring");
    fz.d_ring = reinterpret_cast<const double2*>(f->d_bussi_ring);
    fz.ring_size = f->bussi_ring_size;
    fz.langevin = f->langevin;
    if (f->langevin)
        {
        GB_REQUIRE(!f->bussi && !f->d_scale2, "fused step: Langevin excludes rescaling");
        GB_REQUIRE(f->d_tag && f->d_pos && f->d_gamma && f->d_timestep,
                   "fused step: Langevin needs tags, positions, drag coefficients and the "
                   "timestep");
        }
    fz.tag = f->d_tag;
    fz.pos = reinterpret_cast<const float4*>(f->d_pos);
    fz.gamma = f->d_gamma;
    fz.lkT = f->langevin_kT;
    fz.ndim = f->ndim ? f->ndim : 3u;
    fz.d_reservoir = f->d_reservoir;
    fz.berendsen = f->berendsen;
    fz.brownian = f->brownian;
    GB_REQUIRE(!f->brownian || (!f->bussi && !f->langevin && !f->berendsen && !f->d_scale2),
               "fused step: Brownian dynamics excludes the velocity-Verlet methods");
    GB_REQUIRE(!f->berendsen || (!f->bussi && !f->langevin && f->d_factor && f->d_status
                                 && f->tau > 0.0),
               "fused step: Berendsen needs the factor and status buffers and tau > 0, and "
               "excludes Bussi and Langevin");
    return GB_OK;
    }
} // namespace gb
