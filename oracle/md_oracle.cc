// ORACLE — test infrastructure only.
//
// A CPU restatement of HOOMD-blue 4.8.2's short-range MD step, written for this project and used
// only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the reference the
// GPU results are compared with or the timed CPU baseline. It is
// never linked into, loaded by or called from the product (hoomd-blue_gb300/). Every routine cites
// the reference file:line it follows (paths relative to the HOOMD-blue source tree).
//
// Pinning: the geometry and evaluator routines are checked bit-for-bit against the reference's own
// headers compiled in place (oracle/ref_shim.cc -> oracle/_ref/), and against the golden vectors of
// hoomd/md/pytest/forces_and_energies.json and hoomd/md/pytest/true_pair_list.json (copied into
// tests/golden/ by tests/golden/make_golden.py). Philox4x32-10 (third-party random123, absent
// from the reference checkout) is restated from Salmon et al., SC'11, and pinned by its published
// known-answer vectors; its stream parity with a built HOOMD cannot be checked here.
//
// Precision: every routine is templated on Real and exported as _f32 and _f64. Compile with
// -ffp-contract=off so that FP32 results are reproducible operation for operation.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{

// ------------------------------------------------------------------------------------------------
// Box geometry: hoomd/BoxDim.h
// ------------------------------------------------------------------------------------------------
template<class R> struct Box
    {
    R L[3], lo[3], hi[3], Linv[3];
    R xy, xz, yz;
    int periodic[3];

    // BoxDim(Lx,Ly,Lz) + setTiltFactors: hoomd/BoxDim.h:103-108 (setL at :170-180)
    void set(const double* b6, const int* per)
        {
        for (int d = 0; d < 3; d++)
            {
            L[d] = R(b6[d]);
            hi[d] = L[d] / R(2.0);
            lo[d] = -hi[d];
            Linv[d] = R(1.0) / L[d];
            periodic[d] = per ? (per[d] != 0) : 1;
            }
        if (L[2] == R(0.0))
            Linv[2] = 0;
        xy = R(b6[3]);
        xz = R(b6[4]);
        yz = R(b6[5]);
        }

    // Device form of minImage (rint), hoomd/BoxDim.h:322-341. This is the form the reference's
    // GPU kernels evaluate, and the one the GB300 kernels reproduce bit for bit.
    void min_image_rint(R& x, R& y, R& z) const
        {
        if (periodic[2])
            {
            R img = std::rint(z * Linv[2]);
            z -= L[2] * img;
            y -= L[2] * yz * img;
            x -= L[2] * xz * img;
            }
        if (periodic[1])
            {
            R img = std::rint(y * Linv[1]);
            y -= L[1] * img;
            x -= L[1] * xy * img;
            }
        if (periodic[0])
            {
            x -= L[0] * std::rint(x * Linv[0]);
            }
        }

    // Host form of minImage (branches), hoomd/BoxDim.h:342-389.
    void min_image_branch(R& x, R& y, R& z) const
        {
        if (periodic[2])
            {
            if (z >= hi[2])
                {
                z -= L[2];
                y -= L[2] * yz;
                x -= L[2] * xz;
                }
            else if (z < lo[2])
                {
                z += L[2];
                y += L[2] * yz;
                x += L[2] * xz;
                }
            }
        if (periodic[1])
            {
            if (y >= hi[1])
                {
                int i = int(y * Linv[1] + R(0.5));
                y -= R(i) * L[1];
                x -= R(i) * L[1] * xy;
                }
            else if (y < lo[1])
                {
                int i = int(-y * Linv[1] + R(0.5));
                y += R(i) * L[1];
                x += R(i) * L[1] * xy;
                }
            }
        if (periodic[0])
            {
            if (x >= hi[0])
                {
                int i = int(x * Linv[0] + R(0.5));
                x -= R(i) * L[0];
                }
            else if (x < lo[0])
                {
                int i = int(-x * Linv[0] + R(0.5));
                x += R(i) * L[0];
                }
            }
        }

    // hoomd/BoxDim.h:407-474 (wrap, no forced flags)
    void wrap(R& x, R& y, R& z, int& ix, int& iy, int& iz) const
        {
        R ox = (hi[0] + lo[0]) / R(2.0);
        R oy = (hi[1] + lo[1]) / R(2.0);
        R oz = (hi[2] + lo[2]) / R(2.0);
        (void)ox;
        if (!periodic[1])
            oy = 0;
        if (!periodic[2])
            oz = 0;
        if (periodic[0])
            {
            R tilt_x = (xz - xy * yz) * (z - oz) + xy * (y - oy);
            if (x >= hi[0] + tilt_x)
                {
                x -= L[0];
                ix++;
                }
            else if (x < lo[0] + tilt_x)
                {
                x += L[0];
                ix--;
                }
            }
        if (periodic[1])
            {
            R tilt_y = yz * (z - oz);
            if (y >= hi[1] + tilt_y)
                {
                y -= L[1];
                x -= L[1] * xy;
                iy++;
                }
            else if (y < lo[1] + tilt_y)
                {
                y += L[1];
                x += L[1] * xy;
                iy--;
                }
            }
        if (periodic[2])
            {
            if (z >= hi[2])
                {
                z -= L[2];
                y -= L[2] * yz;
                x -= L[2] * xz;
                iz++;
                }
            else if (z < lo[2])
                {
                z += L[2];
                y += L[2] * yz;
                x += L[2] * xz;
                iz--;
                }
            }
        }

    // hoomd/BoxDim.h:276-284 with ghost_width = 0 (the division by 1 + 0 is exact).
    void make_fraction(R x, R y, R z, R& fx, R& fy, R& fz) const
        {
        R dx = x - lo[0];
        R dy = y - lo[1];
        R dz = z - lo[2];
        dx -= (xz - yz * xy) * z + xy * y;
        dy -= yz * z;
        fx = dx * Linv[0];
        fy = dy * Linv[1];
        fz = dz * Linv[2];
        }

    // hoomd/BoxDim.h:552-567 (host form of fast::rsqrt is 1/sqrt)
    void nearest_plane_distance(R* d) const
        {
        d[0] = L[0] * (R(1.0) / std::sqrt(R(1.0) + xy * xy + (xy * yz - xz) * (xy * yz - xz)));
        d[1] = L[1] * (R(1.0) / std::sqrt(R(1.0) + yz * yz));
        d[2] = L[2];
        if (L[2] == R(0.0))
            d[2] = R(1.0);
        }
    };

template<class R> static inline uint32_t as_uint(R w)
    {
    // __scalar_as_int: the type/index bits stored in the w lane (hoomd/HOOMDMath.h)
    if (sizeof(R) == 4)
        {
        uint32_t u;
        float f = float(w);
        std::memcpy(&u, &f, 4);
        return u;
        }
    else
        {
        uint64_t u;
        double d = double(w);
        std::memcpy(&u, &d, 8);
        return uint32_t(u);
        }
    }

template<class R> static inline R from_uint(uint32_t u)
    {
    if (sizeof(R) == 4)
        {
        float f;
        std::memcpy(&f, &u, 4);
        return R(f);
        }
    else
        {
        uint64_t v = u;
        double d;
        std::memcpy(&d, &v, 8);
        return R(d);
        }
    }

// ------------------------------------------------------------------------------------------------
// Pair evaluators
// ------------------------------------------------------------------------------------------------

// hoomd/md/EvaluatorPairLJ.h:99-155 (param), :162-166 (lj1/lj2), :190-211 (evalForceAndEnergy)
template<class R> struct LJ
    {
    struct param_type
        {
        R sigma_6;
        R epsilon_x_4;
        };
    static param_type make_param(double sigma, double epsilon)
        {
        param_type p;
        R s = R(sigma);
        p.sigma_6 = s * s * s * s * s * s;
        p.epsilon_x_4 = R(4.0) * R(epsilon);
        return p;
        }
    R rsq, rcutsq, lj1, lj2;
    LJ(R rsq_, R rcutsq_, const param_type& p)
        : rsq(rsq_), rcutsq(rcutsq_), lj1(p.epsilon_x_4 * p.sigma_6 * p.sigma_6),
          lj2(p.epsilon_x_4 * p.sigma_6)
        {
        }
    bool eval(R& force_divr, R& pair_eng, bool energy_shift) const
        {
        if (rsq < rcutsq && lj1 != 0)
            {
            R r2inv = R(1.0) / rsq;
            R r6inv = r2inv * r2inv * r2inv;
            force_divr = r2inv * r6inv * (R(12.0) * lj1 * r6inv - R(6.0) * lj2);
            pair_eng = r6inv * (lj1 * r6inv - lj2);
            if (energy_shift)
                {
                R rcut2inv = R(1.0) / rcutsq;
                R rcut6inv = rcut2inv * rcut2inv * rcut2inv;
                pair_eng -= rcut6inv * (lj1 * rcut6inv - lj2);
                }
            return true;
            }
        return false;
        }
    // hoomd/md/EvaluatorPairLJ.h:213-248
    R lrc_energy() const
        {
        if (rcutsq == 0)
            return R(0.0);
        R rcut3inv = R(1.0) / std::pow(rcutsq, R(1.5));
        R rcut9inv = rcut3inv * rcut3inv * rcut3inv;
        return lj1 / R(9.0) * rcut9inv - lj2 / R(3.0) * rcut3inv;
        }
    R lrc_pressure() const
        {
        if (rcutsq == 0)
            return R(0.0);
        R rcut3inv = R(1.0) / std::pow(rcutsq, R(1.5));
        R rcut9inv = rcut3inv * rcut3inv * rcut3inv;
        return lj1 * R(4.0) / R(3.0) * rcut9inv - lj2 * R(2.0) * rcut3inv;
        }
    };

// hoomd/md/EvaluatorPairTable.h:45-118 (param), :151-194 (evalForceAndEnergy). Tables are views
// into one flat array; width = number of points; dr = (r_cut - r_min)/width.
template<class R> struct Table
    {
    struct param_type
        {
        R rmin;
        unsigned int width;
        const R* V;
        const R* F;
        };
    R rsq, rcutsq;
    const param_type& p;
    Table(R rsq_, R rcutsq_, const param_type& p_) : rsq(rsq_), rcutsq(rcutsq_), p(p_) { }
    bool eval(R& force_divr, R& pair_eng, bool) const
        {
        const unsigned int width = p.width;
        const R r = std::sqrt(rsq);
        if (rsq >= rcutsq || r < p.rmin)
            return false;
        const R rcut = std::sqrt(rcutsq);
        const R delta_r = (rcut - p.rmin) / static_cast<R>(width);
        const R value_f = (r - p.rmin) / delta_r;
        unsigned int value_i = static_cast<unsigned int>(std::floor(value_f));
        // The reference reads V_table[value_i] unguarded (EvaluatorPairTable.h:168-171); at FP32
        // r just below r_cut can round value_i up to width. Clamp so the oracle never reads past
        // the table; with value_i == width-1 the last-bin rule V1=F1=0 then applies.
        if (value_i >= width)
            value_i = width - 1;
        const R V0 = p.V[value_i];
        const R F0 = p.F[value_i];
        R V1 = 0, F1 = 0;
        if (value_i + 1 < width)
            {
            V1 = p.V[value_i + 1];
            F1 = p.F[value_i + 1];
            }
        const R f = value_f - R(value_i);
        const R V = V0 + f * (V1 - V0);
        const R F = F0 + f * (F1 - F0);
        if (rsq > R(0.0))
            force_divr = F / r;
        pair_eng = V;
        return true;
        }
    };

// example_plugins/pair_plugin/EvaluatorPairExample.h:82-142
template<class R> struct Example
    {
    struct param_type
        {
        R k;
        R sigma;
        };
    R rsq, rcutsq, k, sigma;
    Example(R rsq_, R rcutsq_, const param_type& p)
        : rsq(rsq_), rcutsq(rcutsq_), k(p.k), sigma(p.sigma)
        {
        }
    bool eval(R& force_divr, R& pair_eng, bool energy_shift) const
        {
        if (rsq < rcutsq)
            {
            R r = std::sqrt(rsq);
            R rinv = 1 / r;
            R overlap = sigma - r;
            force_divr = k * overlap * rinv;
            pair_eng = R(0.5) * k * overlap * overlap;
            if (energy_shift)
                {
                R rcut = std::sqrt(rcutsq);
                R cut_overlap = sigma - rcut;
                pair_eng -= R(0.5) * k * cut_overlap * cut_overlap;
                }
            return true;
            }
        return false;
        }
    };

// ------------------------------------------------------------------------------------------------
// Cell list: hoomd/CellList.cc
// ------------------------------------------------------------------------------------------------

// hoomd/CellList.cc:83-131 (no ghost layer on one rank; m_multiple = 1)
template<class R>
void cell_dims(const Box<R>& box, int ndim, R nominal_width, unsigned int* dim)
    {
    R Lp[3];
    box.nearest_plane_distance(Lp);
    for (int d = 0; d < 3; d++)
        dim[d] = (unsigned int)(Lp[d] / nominal_width);
    if (ndim == 2)
        dim[2] = 1;
    for (int d = 0; d < 3; d++)
        if (dim[d] == 0)
            dim[d] = 1;
    }

// hoomd/CellList.cc:346-402: per cell, the (2r+1)^3 stencil wrapped, sorted and deduplicated.
// Returns the row width W (adj holds W entries per cell, cell-major).
static unsigned int cell_adj(const unsigned int* dim, int ndim, int radius, unsigned int* adj)
    {
    unsigned int nu[3];
    for (int d = 0; d < 3; d++)
        nu[d] = dim[d] > unsigned(radius * 2 + 1) ? unsigned(radius * 2 + 1) : dim[d];
    unsigned int W = (ndim == 2) ? nu[0] * nu[1] : nu[0] * nu[1] * nu[2];
    std::vector<unsigned int> a;
    int mx = int(dim[0]), my = int(dim[1]), mz = int(dim[2]);
    for (int k = 0; k < mz; k++)
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++)
                {
                unsigned int cur = unsigned((k * my + j) * mx + i);
                a.clear();
                int r = radius, rk = (ndim == 2) ? 0 : radius;
                for (int nk = k - rk; nk <= k + rk; nk++)
                    for (int nj = j - r; nj <= j + r; nj++)
                        for (int ni = i - r; ni <= i + r; ni++)
                            {
                            int wi = ni % mx;
                            if (wi < 0)
                                wi += mx;
                            int wj = nj % my;
                            if (wj < 0)
                                wj += my;
                            int wk = nk % mz;
                            if (wk < 0)
                                wk += mz;
                            a.push_back(unsigned((wk * my + wj) * mx + wi));
                            }
                std::sort(a.begin(), a.end());
                a.erase(std::unique(a.begin(), a.end()), a.end());
                std::copy(a.begin(), a.end(), adj + size_t(cur) * W);
                }
    return W;
    }

// hoomd/CellList.cc:404-547 with xyzf flag = particle index (NeighborListBinned.cc:25-28).
// conditions[0] = overflow (max needed Nmax), [1] = NaN particle index+1, [2] = out-of-box index+1.
template<class R>
void cell_list(unsigned int N,
               const R* pos,
               const Box<R>& box,
               const unsigned int* dim,
               unsigned int Nmax,
               unsigned int* cell_size,
               R* xyzf,
               unsigned int* conditions)
    {
    const unsigned int ncell = dim[0] * dim[1] * dim[2];
    std::memset(cell_size, 0, sizeof(unsigned int) * ncell);
    conditions[0] = conditions[1] = conditions[2] = 0;
    for (unsigned int n = 0; n < N; n++)
        {
        R px = pos[4 * n], py = pos[4 * n + 1], pz = pos[4 * n + 2];
        if (std::isnan(px) || std::isnan(py) || std::isnan(pz))
            {
            conditions[1] = n + 1;
            continue;
            }
        R fx, fy, fz;
        box.make_fraction(px, py, pz, fx, fy, fz);
        int ib = (int)(fx * R(dim[0]));
        int jb = (int)(fy * R(dim[1]));
        int kb = (int)(fz * R(dim[2]));
        if ((fx < R(-0.00001) || fx >= R(1.00001)) || (fy < R(-0.00001) || fy >= R(1.00001))
            || (fz < R(-0.00001) || fz >= R(1.00001)))
            {
            conditions[2] = n + 1;
            continue;
            }
        if (ib == (int)dim[0] && box.periodic[0])
            ib = 0;
        if (jb == (int)dim[1] && box.periodic[1])
            jb = 0;
        if (kb == (int)dim[2] && box.periodic[2])
            kb = 0;
        if (ib < 0 || ib >= (int)dim[0] || jb < 0 || jb >= (int)dim[1] || kb < 0
            || kb >= (int)dim[2])
            {
            conditions[2] = n + 1;
            continue;
            }
        unsigned int bin = unsigned((kb * int(dim[1]) + jb) * int(dim[0]) + ib);
        unsigned int offset = cell_size[bin];
        if (offset < Nmax)
            {
            R* e = xyzf + 4 * (size_t(bin) * Nmax + offset);
            e[0] = px;
            e[1] = py;
            e[2] = pz;
            e[3] = from_uint<R>(n);
            }
        else
            {
            conditions[0] = std::max(conditions[0], offset + 1);
            }
        cell_size[bin]++;
        }
    }

// ------------------------------------------------------------------------------------------------
// Neighbor list: hoomd/md/NeighborListBinned.cc:36-179 (one build pass) with the rebuild policy
// of hoomd/md/NeighborList.cc.
// ------------------------------------------------------------------------------------------------
template<class R>
void nlist_binned(unsigned int N,
                  const R* pos,
                  const Box<R>& box,
                  unsigned int ntypes,
                  const R* r_cut,    // ntypes*ntypes
                  const R* r_listsq, // ntypes*ntypes
                  bool full,
                  const unsigned int* dim,
                  const unsigned int* cell_size,
                  const R* xyzf,
                  unsigned int Nmax_cell,
                  const unsigned int* adj,
                  unsigned int adj_w,
                  const unsigned int* Nmax, // per type
                  const uint64_t* head_list,
                  unsigned int* nlist,
                  unsigned int* n_neigh,
                  unsigned int* conditions, // per type
                  bool rint_min_image,
                  int nthreads = 1)
    {
    // each particle's list is built by one thread in the reference's order, so the result does
    // not depend on the thread count
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 512) num_threads(std::max(nthreads, 1))
#endif
    for (int i = 0; i < (int)N; i++)
        {
        unsigned int cur_n_neigh = 0;
        const R mx = pos[4 * i], my = pos[4 * i + 1], mz = pos[4 * i + 2];
        const unsigned int type_i = as_uint(pos[4 * i + 3]);
        const unsigned int Nmax_i = Nmax[type_i];
        const uint64_t head_i = head_list[i];
        R fx, fy, fz;
        box.make_fraction(mx, my, mz, fx, fy, fz);
        int ib = (int)(unsigned int)(fx * R(dim[0]));
        int jb = (int)(unsigned int)(fy * R(dim[1]));
        int kb = (int)(unsigned int)(fz * R(dim[2]));
        if (ib == (int)dim[0] && box.periodic[0])
            ib = 0;
        if (jb == (int)dim[1] && box.periodic[1])
            jb = 0;
        if (kb == (int)dim[2] && box.periodic[2])
            kb = 0;
        unsigned int my_cell = unsigned((kb * int(dim[1]) + jb) * int(dim[0]) + ib);
        for (unsigned int a = 0; a < adj_w; a++)
            {
            unsigned int nc = adj[size_t(my_cell) * adj_w + a];
            unsigned int size = cell_size[nc];
            for (unsigned int o = 0; o < size; o++)
                {
                const R* e = xyzf + 4 * (size_t(nc) * Nmax_cell + o);
                unsigned int j = as_uint(e[3]);
                unsigned int type_j = as_uint(pos[4 * j + 3]);
                R rc = r_cut[type_i * ntypes + type_j];
                bool excluded = ((i == (int)j) || (rc <= R(0.0)));
                if (excluded)
                    continue;
                R dx = mx - e[0], dy = my - e[1], dz = mz - e[2];
                if (rint_min_image)
                    box.min_image_rint(dx, dy, dz);
                else
                    box.min_image_branch(dx, dy, dz);
                R dr_sq = dx * dx + dy * dy + dz * dz;
                R rlsq = r_listsq[type_i * ntypes + type_j];
                if (dr_sq <= rlsq)
                    {
                    if (full || i < (int)j)
                        {
                        if (cur_n_neigh < Nmax_i)
                            nlist[head_i + cur_n_neigh] = j;
                        cur_n_neigh++;
                        }
                    }
                }
            }
        // overflow: the per-type condition is the largest count seen (one update per particle
        // instead of one per overflowing neighbour; the result is the same)
        if (cur_n_neigh > Nmax_i)
            {
#ifdef _OPENMP
#pragma omp critical(orc_nlist_cond)
#endif
            conditions[type_i] = std::max(conditions[type_i], cur_n_neigh);
            }
        n_neigh[i] = cur_n_neigh;
        }
    }

// ------------------------------------------------------------------------------------------------
// Pair force loop: hoomd/md/PotentialPair.h:587-794 (shift modes none=0, shift=1, xplor=2)
// ------------------------------------------------------------------------------------------------
template<class R, class E>
void pair_forces(unsigned int N,
                 const R* pos,
                 const Box<R>& box,
                 unsigned int ntypes,
                 const typename E::param_type* params,
                 const R* rcutsq,
                 const R* ronsq,
                 int shift_mode,
                 const unsigned int* n_neigh,
                 const unsigned int* nlist,
                 const uint64_t* head_list,
                 bool third_law,
                 bool compute_virial,
                 R* force,
                 R* virial, // 6 * N, SoA with pitch N
                 bool rint_min_image,
                 int nthreads,
                 int abs_terms = 0)
    {
    // abs_terms (full list only) accumulates magnitudes instead of the terms:
    //  1: of every term. The result bounds each sum's conditioning: a sum of n terms computed
    //     in a precision with unit roundoff u is within about n u times this of the exact sum.
    //  2: of the terms of the cut-off band only: pairs with |r^2 - r_cut^2| <= 1e-6 r_cut^2,
    //     evaluated just inside r_cut. Whether such a pair interacts turns on the last bits of
    //     r^2, which two correct FP32 evaluations may round differently; where the potential
    //     does not vanish at r_cut, one pair more or less moves the force by this much.
    const R band = R(1e-6);
    std::memset(force, 0, sizeof(R) * 4 * N);
    if (virial)
        std::memset(virial, 0, sizeof(R) * 6 * N);
    const size_t pitch = N;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(third_law ? 1 : std::max(nthreads, 1))
#endif
    for (int i = 0; i < (int)N; i++)
        {
        R pix = pos[4 * i], piy = pos[4 * i + 1], piz = pos[4 * i + 2];
        unsigned int typei = as_uint(pos[4 * i + 3]);
        R fx = 0, fy = 0, fz = 0, pei = 0;
        R vxx = 0, vxy = 0, vxz = 0, vyy = 0, vyz = 0, vzz = 0;
        const uint64_t myHead = head_list[i];
        const unsigned int size = n_neigh[i];
        for (unsigned int k = 0; k < size; k++)
            {
            unsigned int j = nlist[myHead + k];
            R dx = pix - pos[4 * j], dy = piy - pos[4 * j + 1], dz = piz - pos[4 * j + 2];
            unsigned int typej = as_uint(pos[4 * j + 3]);
            if (rint_min_image)
                box.min_image_rint(dx, dy, dz);
            else
                box.min_image_branch(dx, dy, dz);
            R rsq = dx * dx + dy * dy + dz * dz;
            unsigned int tp = typei * ntypes + typej;
            const typename E::param_type& param = params[tp];
            R rc2 = rcutsq[tp];
            R ro2 = R(0.0);
            if (shift_mode == 2)
                ro2 = ronsq[tp];
            bool energy_shift = false;
            if (shift_mode == 1)
                energy_shift = true;
            else if (shift_mode == 2)
                {
                if (ro2 > rc2)
                    energy_shift = true;
                }
            R force_divr = R(0.0);
            R pair_eng = R(0.0);
            if (abs_terms == 2)
                {
                using std::abs;
                if (!(abs(rsq - rc2) <= band * rc2))
                    continue;
                rsq = std::min(rsq, rc2 * (R(1) - band));
                }
            E eval(rsq, rc2, param);
            bool evaluated = eval.eval(force_divr, pair_eng, energy_shift);
            if (evaluated)
                {
                if (shift_mode == 2)
                    {
                    if (rsq >= ro2 && rsq < rc2)
                        {
                        R old_pair_eng = pair_eng;
                        R old_force_divr = force_divr;
                        R xplor_denom_inv = R(1.0) / ((rc2 - ro2) * (rc2 - ro2) * (rc2 - ro2));
                        R rsq_minus_r_cut_sq = rsq - rc2;
                        R s = rsq_minus_r_cut_sq * rsq_minus_r_cut_sq
                              * (rc2 + R(2.0) * rsq - R(3.0) * ro2) * xplor_denom_inv;
                        R ds_dr_divr = R(12.0) * (rsq - ro2) * rsq_minus_r_cut_sq * xplor_denom_inv;
                        pair_eng = old_pair_eng * s;
                        force_divr = s * old_force_divr - ds_dr_divr * old_pair_eng;
                        }
                    }
                R force_div2r = force_divr * R(0.5);
                if (abs_terms != 0)
                    {
                    using std::abs;
                    fx += abs(dx * force_divr);
                    fy += abs(dy * force_divr);
                    fz += abs(dz * force_divr);
                    pei += abs(pair_eng * R(0.5));
                    if (compute_virial)
                        {
                        vxx += abs(force_div2r * dx * dx);
                        vxy += abs(force_div2r * dx * dy);
                        vxz += abs(force_div2r * dx * dz);
                        vyy += abs(force_div2r * dy * dy);
                        vyz += abs(force_div2r * dy * dz);
                        vzz += abs(force_div2r * dz * dz);
                        }
                    continue;
                    }
                fx += dx * force_divr;
                fy += dy * force_divr;
                fz += dz * force_divr;
                pei += pair_eng * R(0.5);
                if (compute_virial)
                    {
                    vxx += force_div2r * dx * dx;
                    vxy += force_div2r * dx * dy;
                    vxz += force_div2r * dx * dz;
                    vyy += force_div2r * dy * dy;
                    vyz += force_div2r * dy * dz;
                    vzz += force_div2r * dz * dz;
                    }
                if (third_law && j < N)
                    {
                    force[4 * j] -= dx * force_divr;
                    force[4 * j + 1] -= dy * force_divr;
                    force[4 * j + 2] -= dz * force_divr;
                    force[4 * j + 3] += pair_eng * R(0.5);
                    if (compute_virial)
                        {
                        virial[0 * pitch + j] += force_div2r * dx * dx;
                        virial[1 * pitch + j] += force_div2r * dx * dy;
                        virial[2 * pitch + j] += force_div2r * dx * dz;
                        virial[3 * pitch + j] += force_div2r * dy * dy;
                        virial[4 * pitch + j] += force_div2r * dy * dz;
                        virial[5 * pitch + j] += force_div2r * dz * dz;
                        }
                    }
                }
            }
        force[4 * i] += fx;
        force[4 * i + 1] += fy;
        force[4 * i + 2] += fz;
        force[4 * i + 3] += pei;
        if (compute_virial)
            {
            virial[0 * pitch + i] += vxx;
            virial[1 * pitch + i] += vxy;
            virial[2 * pitch + i] += vxz;
            virial[3 * pitch + i] += vyy;
            virial[4 * pitch + i] += vyz;
            virial[5 * pitch + i] += vzz;
            }
        }
    }

// ------------------------------------------------------------------------------------------------
// Integrator halves: hoomd/md/TwoStepConstantVolume.cc:7-80 (one) and :213-261 (two);
// accelerations: hoomd/Integrator.cc:106-127.
// ------------------------------------------------------------------------------------------------
template<class R>
void cv_step_one(unsigned int N, R* pos, R* vel, const R* accel, int* image, const Box<R>& box,
                 R dt, R s, int nthreads = 1, R limit = R(0))
    {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(std::max(nthreads, 1))
#endif
    for (unsigned int j = 0; j < N; j++)
        {
        R vx = vel[4 * j], vy = vel[4 * j + 1], vz = vel[4 * j + 2];
        R px = pos[4 * j], py = pos[4 * j + 1], pz = pos[4 * j + 2];
        vx = vx + R(1.0 / 2.0) * accel[3 * j] * dt;
        vy = vy + R(1.0 / 2.0) * accel[3 * j + 1] * dt;
        vz = vz + R(1.0 / 2.0) * accel[3 * j + 2] * dt;
        vx *= s;
        vy *= s;
        vz *= s;
        if (limit > R(0))
            {
            // DisplacementCapped (hoomd/md/TwoStepConstantVolume.cc:44-52) with the step capped at
            // the limit as hoomd/md/methods/methods.py:583-598 documents: the reference's
            // expression divides by dt once more, which caps the step at limit / dt instead
            R len = std::sqrt(vx * vx + vy * vy + vz * vz) * dt;
            if (len > limit)
                {
                vx = vx / len * limit;
                vy = vy / len * limit;
                vz = vz / len * limit;
                }
            }
        px += dt * vx;
        py += dt * vy;
        pz += dt * vz;
        vel[4 * j] = vx;
        vel[4 * j + 1] = vy;
        vel[4 * j + 2] = vz;
        box.wrap(px, py, pz, image[3 * j], image[3 * j + 1], image[3 * j + 2]);
        pos[4 * j] = px;
        pos[4 * j + 1] = py;
        pos[4 * j + 2] = pz;
        }
    }

template<class R>
void cv_step_two(unsigned int N, R* vel, R* accel, const R* net_force, R dt, R s,
                 int nthreads = 1)
    {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(std::max(nthreads, 1))
#endif
    for (unsigned int j = 0; j < N; j++)
        {
        R vx = vel[4 * j], vy = vel[4 * j + 1], vz = vel[4 * j + 2];
        R m = vel[4 * j + 3];
        R minv = R(1.0) / m;
        R ax = net_force[4 * j] * minv, ay = net_force[4 * j + 1] * minv,
          az = net_force[4 * j + 2] * minv;
        vx *= s;
        vy *= s;
        vz *= s;
        vx += R(1.0 / 2.0) * dt * ax;
        vy += R(1.0 / 2.0) * dt * ay;
        vz += R(1.0 / 2.0) * dt * az;
        vel[4 * j] = vx;
        vel[4 * j + 1] = vy;
        vel[4 * j + 2] = vz;
        accel[3 * j] = ax;
        accel[3 * j + 1] = ay;
        accel[3 * j + 2] = az;
        }
    }

// hoomd/md/ComputeThermo.cc:119-131: translational KE accumulated in double.
template<class R> double kinetic_energy(unsigned int N, const R* vel)
    {
    double ke = 0.0;
    for (unsigned int j = 0; j < N; j++)
        ke += (double)vel[4 * j + 3]
              * ((double)vel[4 * j] * (double)vel[4 * j] + (double)vel[4 * j + 1] * (double)vel[4 * j + 1]
                 + (double)vel[4 * j + 2] * (double)vel[4 * j + 2]);
    return ke * 0.5;
    }

// ------------------------------------------------------------------------------------------------
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11), used through the wrappers of hoomd/RandomNumbers.h.
// ------------------------------------------------------------------------------------------------
static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo)
    {
    uint64_t p = uint64_t(a) * uint64_t(b);
    hi = uint32_t(p >> 32);
    lo = uint32_t(p);
    }

// Philox4x32 with 10 rounds: round function (c0,c1,c2,c3) -> (hi1^c1^k0, lo1, hi0^c3^k1, lo0)
// with multipliers M0=0xD2511F53, M1=0xCD9E8D57 on c0,c2 and Weyl key bumps 0x9E3779B9,0xBB67AE85.
static void philox4x32_10(const uint32_t in_ctr[4], const uint32_t in_key[2], uint32_t out[4])
    {
    uint32_t c[4] = {in_ctr[0], in_ctr[1], in_ctr[2], in_ctr[3]};
    uint32_t k[2] = {in_key[0], in_key[1]};
    for (int r = 0; r < 10; r++)
        {
        if (r > 0)
            {
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
            }
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c[0], hi0, lo0);
        mulhilo32(0xCD9E8D57u, c[2], hi1, lo1);
        uint32_t n0 = hi1 ^ c[1] ^ k[0];
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c[3] ^ k[1];
        uint32_t n3 = lo0;
        c[0] = n0;
        c[1] = n1;
        c[2] = n2;
        c[3] = n3;
        }
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
    out[3] = c[3];
    }

// hoomd/RandomNumbers.h:136-168 (Seed), :175-197 (Counter), :224-270 (generator: counter word 0
// increments after each draw)
struct RNG
    {
    uint32_t key[2];
    uint32_t ctr[4];
    RNG(uint8_t id, uint64_t timestep, uint16_t seed, uint32_t a, uint32_t b = 0, uint32_t c = 0,
        uint16_t d = 0)
        {
        key[0] = uint32_t(id) << 24 | uint32_t(seed) << 8
                 | uint32_t((timestep & 0x000000ff00000000ull) >> 32);
        key[1] = uint32_t(timestep & 0x00000000ffffffffull);
        ctr[0] = uint32_t(d) << 16;
        ctr[1] = c;
        ctr[2] = b;
        ctr[3] = a;
        }
    void next(uint32_t out[4])
        {
        philox4x32_10(ctr, key, out);
        ctr[0] += 1;
        }
    uint64_t u64()
        {
        uint32_t o[4];
        next(o);
        return uint64_t(o[0]) << 32 | o[1];
        }
    void two_u64(uint64_t& a, uint64_t& b)
        {
        uint32_t o[4];
        next(o);
        a = uint64_t(o[0]) << 32 | o[1];
        b = uint64_t(o[2]) << 32 | o[3];
        }
    };

// random123 uniform.hpp conversions (published algorithm): u01 maps an unsigned integer to
// (0,1] as in*2^-W + 2^-(W+1); uneg11 maps the signed reinterpretation to [-1,1].
template<class R> static inline R u01(uint64_t in)
    {
    const R factor = R(1.) / (R(18446744073709551615.0) + R(1.));
    const R halffactor = R(0.5) * factor;
    return R(in) * factor + halffactor;
    }
template<class R> static inline R uneg11(uint64_t in)
    {
    const R factor = R(1.) / (R(9223372036854775807.0) + R(1.));
    const R halffactor = R(0.5) * factor;
    return R(int64_t(in)) * factor + halffactor;
    }

// hoomd/RandomNumbers.h:346-402 (Box-Muller, one value per draw); host sincospi = sincos(pi*x)
template<class R> static R normal(RNG& rng, R sigma = R(1.0), R mu = R(0.0))
    {
    uint64_t u0, u1;
    rng.two_u64(u0, u1);
    R a = R(M_PI) * uneg11<R>(u0);
    R x = std::sin(a);
    R r = std::sqrt(R(-2.0) * std::log(u01<R>(u1)));
    x *= r;
    return x * sigma + mu;
    }

// hoomd/RandomNumbers.h:454-534 (Marsaglia-Tsang gamma with squeeze test)
template<class R> static R gamma(RNG& rng, R m_alpha, R m_b)
    {
    R alpha = m_alpha;
    if (m_alpha < R(1.0))
        alpha += R(1.0);
    R d = alpha - R(1. / 3.);
    R c = (R(1.0) / std::sqrt(d)) / R(3.);
    R v;
    while (1)
        {
        R x;
        do
            {
            x = normal<R>(rng);
            v = R(1.0) + c * x;
            } while (v <= R(0.));
        v = v * v * v;
        const R x2 = x * x;
        R u = u01<R>(rng.u64());
        if (u < R(1.0) - R(0.0331) * x2 * x2)
            break;
        if (std::log(u) < R(0.5) * x2 + d * (R(1.0) - v + std::log(v)))
            break;
        }
    v *= d * m_b;
    if (m_alpha < R(1.0))
        v *= std::pow(u01<R>(rng.u64()), R(1.0) / m_alpha);
    return v;
    }

// hoomd/md/Thermostat.h:357-391 (key: id 45, timestep, seed; counter: tag of the first group
// member) and :416-446 (compute_rescale_factor, all in double)
static double bussi_factor(double K, double dof, double dt, double tau, double set_T,
                           uint64_t timestep, uint16_t seed, uint32_t instance_id)
    {
    if (dt == 0.0 || dof == 0)
        return 1.0;
    RNG rng(45, timestep, seed, instance_id);
    double time_decay_factor = 0.0;
    if (tau != 0.0)
        time_decay_factor = std::exp(-dt / tau);
    double r_normal_one = normal<double>(rng);
    double r_gamma = 0.0;
    if (dof > 1.0)
        r_gamma = 2.0 * gamma<double>(rng, (dof - 1.0) / 2.0, 1.0);
    double v = set_T / 2.0 / K;
    double term1 = v * (1.0 - time_decay_factor) * (r_gamma + r_normal_one * r_normal_one);
    double term2 = 2.0 * r_normal_one * std::sqrt(v * (1.0 - time_decay_factor) * time_decay_factor);
    return std::sqrt(time_decay_factor + term1 + term2);
    }

// hoomd/ParticleGroup.cc:690-760: per-particle Gaussian velocities (RNG id 35, counter = tag) and
// removal of the centre-of-mass momentum. Point particles, no rigid bodies.
template<class R>
void thermalize(unsigned int N, R* vel, const unsigned int* tags, R kT, uint64_t timestep,
                uint16_t seed, int ndim)
    {
    R tpx = 0, tpy = 0, tpz = 0;
    for (unsigned int j = 0; j < N; j++)
        {
        RNG rng(35, timestep, seed, tags[j]);
        R mass = vel[4 * j + 3];
        R sigma = std::sqrt(kT / mass);
        vel[4 * j] = normal<R>(rng, sigma);
        vel[4 * j + 1] = normal<R>(rng, sigma);
        vel[4 * j + 2] = (ndim > 2) ? normal<R>(rng, sigma) : R(0);
        tpx += mass * vel[4 * j];
        tpy += mass * vel[4 * j + 1];
        tpz += mass * vel[4 * j + 2];
        }
    R cx = tpx / R(N), cy = tpy / R(N), cz = tpz / R(N);
    for (unsigned int j = 0; j < N; j++)
        {
        R mass = vel[4 * j + 3];
        vel[4 * j] = vel[4 * j] - cx / mass;
        vel[4 * j + 1] = vel[4 * j + 1] - cy / mass;
        if (ndim > 2)
            vel[4 * j + 2] = vel[4 * j + 2] - cz / mass;
        }
    }

// ------------------------------------------------------------------------------------------------
// Langevin dynamics, translational part. Step one in the TwoStepNVE order
// (hoomd/md/TwoStepLangevin.cc:57-81): x += v dt + (1/2) a dt^2, wrap, v += (1/2) a dt.
// Step two (hoomd/md/TwoStepLangevin.cc:206-292): three UniformDistribution<R>(-1, 1) draws from
// Seed(25, timestep, seed), Counter(tag); F_bd = r sqrt(6 gamma T / dt) - gamma v (z term zero in
// 2D); a = (F + F_bd) / m; v += (1/2) a dt; the reservoir tally sums F_bd . v in R
// (:290-292, :396-412). Returns that sum.
// ------------------------------------------------------------------------------------------------
template<class R>
void nve_step_one(unsigned int N, R* pos, R* vel, const R* accel, int* image, const Box<R>& box,
                  R dt, int nthreads = 1)
    {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(std::max(nthreads, 1))
#endif
    for (unsigned int j = 0; j < N; j++)
        {
        R dx = vel[4 * j] * dt + R(1.0 / 2.0) * accel[3 * j] * dt * dt;
        R dy = vel[4 * j + 1] * dt + R(1.0 / 2.0) * accel[3 * j + 1] * dt * dt;
        R dz = vel[4 * j + 2] * dt + R(1.0 / 2.0) * accel[3 * j + 2] * dt * dt;
        R px = pos[4 * j] + dx, py = pos[4 * j + 1] + dy, pz = pos[4 * j + 2] + dz;
        box.wrap(px, py, pz, image[3 * j], image[3 * j + 1], image[3 * j + 2]);
        pos[4 * j] = px;
        pos[4 * j + 1] = py;
        pos[4 * j + 2] = pz;
        vel[4 * j] += R(1.0 / 2.0) * accel[3 * j] * dt;
        vel[4 * j + 1] += R(1.0 / 2.0) * accel[3 * j + 1] * dt;
        vel[4 * j + 2] += R(1.0 / 2.0) * accel[3 * j + 2] * dt;
        }
    }

template<class R> static inline R uniform_m11(RNG& rng)
    {
    // hoomd/RandomNumbers.h:317-341: a + (b - a) * u01(draw)
    return R(-1) + R(2) * u01<R>(rng.u64());
    }

template<class R>
double langevin_step_two(unsigned int N, R* vel, R* accel, const R* pos, const unsigned int* tags,
                         const R* net_force, const R* gamma_t, R T, R dt, uint16_t seed,
                         uint64_t timestep, int ndim)
    {
    R bd_energy_transfer = 0;
    for (unsigned int j = 0; j < N; j++)
        {
        RNG rng(25, timestep, seed, tags[j]);
        R rx = uniform_m11<R>(rng);
        R ry = uniform_m11<R>(rng);
        R rz = uniform_m11<R>(rng);
        R gamma = gamma_t[as_uint(pos[4 * j + 3])];
        R coeff = std::sqrt(R(6.0) * gamma * T / dt);
        R bd_fx = rx * coeff - gamma * vel[4 * j];
        R bd_fy = ry * coeff - gamma * vel[4 * j + 1];
        R bd_fz = rz * coeff - gamma * vel[4 * j + 2];
        if (ndim < 3)
            bd_fz = R(0.0);
        R minv = R(1.0) / vel[4 * j + 3];
        accel[3 * j] = (net_force[4 * j] + bd_fx) * minv;
        accel[3 * j + 1] = (net_force[4 * j + 1] + bd_fy) * minv;
        accel[3 * j + 2] = (net_force[4 * j + 2] + bd_fz) * minv;
        vel[4 * j] += R(1.0 / 2.0) * accel[3 * j] * dt;
        vel[4 * j + 1] += R(1.0 / 2.0) * accel[3 * j + 1] * dt;
        vel[4 * j + 2] += R(1.0 / 2.0) * accel[3 * j + 2] * dt;
        bd_energy_transfer
            += bd_fx * vel[4 * j] + bd_fy * vel[4 * j + 1] + bd_fz * vel[4 * j + 2];
        }
    return double(bd_energy_transfer);
    }

// ------------------------------------------------------------------------------------------------
// Brownian dynamics, TwoStepBD::integrateStepOne (hoomd/md/TwoStepBD.cc:47-151), translational
// part: three UniformDistribution<R>(-1, 1) draws from Seed(24, timestep, seed), Counter(tag);
// x += (F + F_r) dt / gamma, F_r = r sqrt(6 gamma T / dt) (z zero in 2D); wrap; velocities from
// NormalDistribution<R>(sqrt(T / m)) of the same stream, or F / gamma when noiseless.
// ------------------------------------------------------------------------------------------------
template<class R>
void bd_step_one(unsigned int N, R* pos, R* vel, const R* force, int* image,
                 const unsigned int* tags, const R* gamma_t, const Box<R>& box, R T, R dt,
                 uint16_t seed, uint64_t timestep, int ndim, bool noiseless)
    {
    for (unsigned int j = 0; j < N; j++)
        {
        RNG rng(24, timestep, seed, tags[j]);
        R rx = uniform_m11<R>(rng);
        R ry = uniform_m11<R>(rng);
        R rz = uniform_m11<R>(rng);
        R gamma = gamma_t[as_uint(pos[4 * j + 3])];
        R coeff = std::sqrt(R(3.0) * R(2.0) * gamma * T / dt);
        if (noiseless)
            coeff = R(0.0);
        R frx = rx * coeff, fry = ry * coeff, frz = rz * coeff;
        if (ndim < 3)
            frz = R(0.0);
        R px = pos[4 * j] + (force[4 * j] + frx) * dt / gamma;
        R py = pos[4 * j + 1] + (force[4 * j + 1] + fry) * dt / gamma;
        R pz = pos[4 * j + 2] + (force[4 * j + 2] + frz) * dt / gamma;
        box.wrap(px, py, pz, image[3 * j], image[3 * j + 1], image[3 * j + 2]);
        pos[4 * j] = px;
        pos[4 * j + 1] = py;
        pos[4 * j + 2] = pz;
        if (noiseless)
            {
            vel[4 * j] = force[4 * j] / gamma;
            vel[4 * j + 1] = force[4 * j + 1] / gamma;
            vel[4 * j + 2] = ndim > 2 ? force[4 * j + 2] / gamma : R(0);
            }
        else
            {
            R sigma = std::sqrt(T / vel[4 * j + 3]);
            vel[4 * j] = normal<R>(rng, sigma);
            vel[4 * j + 1] = normal<R>(rng, sigma);
            vel[4 * j + 2] = ndim > 2 ? normal<R>(rng, sigma) : R(0);
            }
        }
    }

// ------------------------------------------------------------------------------------------------
// ConstantPressure halves, translational part (hoomd/md/TwoStepConstantPressure.cc:262-300 and
// :600-625): upper-triangular propagators (xx, xy, xz, yy, yz, zz) in R.
// ------------------------------------------------------------------------------------------------
template<class R> static inline void tri_apply(const R* m, R& x, R& y, R& z)
    {
    R nx = m[0] * x + m[1] * y + m[2] * z;
    R ny = m[3] * y + m[4] * z;
    R nz = m[5] * z;
    x = nx;
    y = ny;
    z = nz;
    }

template<class R>
void npt_step_one(unsigned int N, R* pos, R* vel, const R* accel, int* image,
                  const Box<R>& new_box, R dt, R s, const R* mv, const R* mr, const R* mri)
    {
    for (unsigned int j = 0; j < N; j++)
        {
        R vx = vel[4 * j], vy = vel[4 * j + 1], vz = vel[4 * j + 2];
        R px = pos[4 * j], py = pos[4 * j + 1], pz = pos[4 * j + 2];
        vx += dt / R(2.0) * accel[3 * j];
        vy += dt / R(2.0) * accel[3 * j + 1];
        vz += dt / R(2.0) * accel[3 * j + 2];
        tri_apply(mv, vx, vy, vz);
        vx *= s;
        vy *= s;
        vz *= s;
        tri_apply(mr, px, py, pz);
        R ix = vx, iy = vy, iz = vz;
        tri_apply(mri, ix, iy, iz);
        px += ix;
        py += iy;
        pz += iz;
        new_box.wrap(px, py, pz, image[3 * j], image[3 * j + 1], image[3 * j + 2]);
        pos[4 * j] = px;
        pos[4 * j + 1] = py;
        pos[4 * j + 2] = pz;
        vel[4 * j] = vx;
        vel[4 * j + 1] = vy;
        vel[4 * j + 2] = vz;
        }
    }

template<class R>
void npt_step_two(unsigned int N, R* vel, R* accel, const R* net_force, R dt, R s, const R* mv)
    {
    for (unsigned int j = 0; j < N; j++)
        {
        R minv = R(1.0) / vel[4 * j + 3];
        R ax = net_force[4 * j] * minv, ay = net_force[4 * j + 1] * minv,
          az = net_force[4 * j + 2] * minv;
        R vx = vel[4 * j] * s, vy = vel[4 * j + 1] * s, vz = vel[4 * j + 2] * s;
        tri_apply(mv, vx, vy, vz);
        vx += dt / R(2.0) * ax;
        vy += dt / R(2.0) * ay;
        vz += dt / R(2.0) * az;
        vel[4 * j] = vx;
        vel[4 * j + 1] = vy;
        vel[4 * j + 2] = vz;
        accel[3 * j] = ax;
        accel[3 * j + 1] = ay;
        accel[3 * j + 2] = az;
        }
    }

// ------------------------------------------------------------------------------------------------
// Particle sort: hoomd/SFCPackTuner.cc:289-486 (Hilbert traversal by recursion over octants with
// the walking tables and the eight permutation rules), :541-651 (getSortedOrder3D: bin with
// (unsigned)(f * grid) % grid, clamp, key = traversal position, sort (key, index) pairs) and
// :489-539 (getSortedOrder2D: key = row-major bin). Positions and fractions at the precision R.
// ------------------------------------------------------------------------------------------------
namespace sfc
{
const int istep[8] = {0, 0, 0, 0, 1, 1, 1, 1};
const int jstep[8] = {0, 0, 1, 1, 1, 1, 0, 0};
const int kstep[8] = {0, 1, 1, 0, 0, 1, 1, 0};
// child order of rule m: result[k] = in[perm[m][k]]
const int perm[8][8] = {{0, 3, 4, 7, 6, 5, 2, 1}, {0, 7, 6, 1, 2, 5, 4, 3},
                        {0, 7, 6, 1, 2, 5, 4, 3}, {2, 3, 0, 1, 6, 7, 4, 5},
                        {2, 3, 0, 1, 6, 7, 4, 5}, {4, 3, 2, 5, 6, 1, 0, 7},
                        {4, 3, 2, 5, 6, 1, 0, 7}, {6, 5, 2, 1, 0, 3, 4, 7}};

// appends the grid index i*M*M + j*M + k of every cell of the w-wide cube at (i, j, k) in
// traversal order
void traverse(int i, int j, int k, int w, int M, const unsigned int order[8],
              std::vector<unsigned int>& out)
    {
    if (w == 1)
        {
        out.push_back((unsigned int)(i * M * M + j * M + k));
        return;
        }
    w /= 2;
    for (int m = 0; m < 8; m++)
        {
        const unsigned int cur = order[m];
        unsigned int child[8];
        for (int q = 0; q < 8; q++)
            child[q] = order[perm[m][q]];
        traverse(i + w * istep[cur], j + w * jstep[cur], k + w * kstep[cur], w, M, child, out);
        }
    }
} // namespace sfc

template<class R>
void sfc_order(unsigned int N, const R* pos, const Box<R>& box, unsigned int grid, int ndim,
               unsigned int* order)
    {
    std::vector<unsigned int> rank;
    if (ndim == 3)
        {
        std::vector<unsigned int> seq;
        seq.reserve((size_t)grid * grid * grid);
        const unsigned int identity[8] = {0, 1, 2, 3, 4, 5, 6, 7};
        sfc::traverse(0, 0, 0, (int)grid, (int)grid, identity, seq);
        rank.assign(seq.size(), 0u);
        for (size_t n = 0; n < seq.size(); n++)
            rank[seq[n]] = (unsigned int)n;
        }
    std::vector<std::pair<unsigned int, unsigned int>> keys(N);
    for (unsigned int n = 0; n < N; n++)
        {
        R fx, fy, fz;
        box.make_fraction(pos[4 * n], pos[4 * n + 1], pos[4 * n + 2], fx, fy, fz);
        int ib = (int)((unsigned int)(fx * R(grid)) % grid);
        int jb = (int)((unsigned int)(fy * R(grid)) % grid);
        int kb = ndim == 3 ? (int)((unsigned int)(fz * R(grid)) % grid) : 0;
        ib = std::min(std::max(ib, 0), (int)grid - 1);
        jb = std::min(std::max(jb, 0), (int)grid - 1);
        kb = std::min(std::max(kb, 0), (int)grid - 1);
        const unsigned int key = ndim == 3
                                     ? rank[(size_t)ib * grid * grid + (size_t)jb * grid + kb]
                                     : (unsigned int)(ib * grid + jb);
        keys[n] = {key, n};
        }
    std::sort(keys.begin(), keys.end());
    for (unsigned int n = 0; n < N; n++)
        order[n] = keys[n].second;
    }

// ------------------------------------------------------------------------------------------------
// Whole-step runner: hoomd/md/IntegratorTwoStep.cc:51-139 (update), :226-298 (prepRun),
// hoomd/md/NeighborList.cc:363-435 (compute), :452-529 (updateRList), :1220-1289 (distanceCheck),
// :1325-1418 (needsUpdating, rebuild_check_delay = 1, check_dist = true), :1544-1617 (head list,
// overflow), hoomd/CellList.cc:133-200 (cell overflow retry). One ConstantVolume method on all
// particles, optional Bussi thermostat, LJ or Table pair force.
// ------------------------------------------------------------------------------------------------
template<class R> struct Sim
    {
    unsigned int N = 0, ntypes = 1;
    int ndim = 3;
    Box<R> box;
    std::vector<R> pos, vel, accel, force, virial, last_pos;
    std::vector<int> image;
    std::vector<unsigned int> tags;
    // pair force
    int kind = 0; // 0 = LJ, 1 = Table
    std::vector<typename LJ<R>::param_type> lj;
    std::vector<typename Table<R>::param_type> table;
    std::vector<R> table_data;
    std::vector<R> r_cut, rcutsq, ronsq, r_listsq, rcut_max;
    int shift_mode = 0;
    R r_buff = 0;
    bool full = false;
    int nthreads = 1;
    // neighbor list state
    std::vector<unsigned int> Nmax, nlist, n_neigh, nl_cond;
    std::vector<uint64_t> head_list;
    unsigned int dim[3] = {0, 0, 0};
    unsigned int Nmax_cell = 0;
    std::vector<unsigned int> cell_size, adj;
    unsigned int adj_w = 0;
    std::vector<R> xyzf;
    R last_L[3] = {0, 0, 0};
    bool force_update = true;
    uint64_t n_builds = 0;
    // rebuild-check schedule (nlist rebuild_check_delay, check_dist) and its counters: builds
    // decided by a check (the reference's num_builds), dangerous builds
    unsigned int check_delay = 1;
    bool dist_check = true;
    uint64_t last_updated = 0, n_updates = 0, n_dangerous = 0;
    // integrator
    R dt = 0;
    bool langevin = false;
    int thermostat = 0; // 0: none or Bussi (bussi flag), 2: Berendsen, 3: MTTK
    double xi = 0, eta = 0;
    std::vector<R> gamma;
    R langevin_T = 0;
    double reservoir = 0;
    bool bussi = false;
    double kT = 0, tau = 0;
    uint16_t seed = 0;
    uint64_t timestep = 0;
    bool prepared = false;
    std::string error;

    void update_rlist()
        {
        r_listsq.assign(ntypes * ntypes, 0);
        rcut_max.assign(ntypes, 0);
        for (unsigned int i = 0; i < ntypes; i++)
            {
            R m = 0;
            for (unsigned int j = 0; j < ntypes; j++)
                {
                R rc = r_cut[i * ntypes + j];
                if (rc > m)
                    m = rc;
                R rl = (rc > R(0.0)) ? rc + r_buff : R(0.0);
                r_listsq[i * ntypes + j] = rl * rl;
                }
            rcut_max[i] = m;
            }
        }

    R max_rcut() const
        {
        R m = 0;
        for (auto v : rcut_max)
            m = std::max(m, v);
        return m;
        }

    void build_head_list()
        {
        head_list.resize(N);
        uint64_t a = 0;
        for (unsigned int i = 0; i < N; i++)
            {
            head_list[i] = a;
            a += Nmax[as_uint(pos[4 * i + 3])];
            }
        if (nlist.size() < a)
            nlist.resize(a);
        }

    bool distance_check()
        {
        R Lg[3];
        box.nearest_plane_distance(Lg);
        R lam[3] = {Lg[0] / last_L[0], Lg[1] / last_L[1], Lg[2] / last_L[2]};
        R lmin = std::min(std::min(lam[0], lam[1]), lam[2]);
        int moved = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : moved) num_threads(std::max(nthreads, 1))
#endif
        for (unsigned int i = 0; i < N; i++)
            {
            unsigned int ti = as_uint(pos[4 * i + 3]);
            R old_rmin = rcut_max[ti];
            R rmax = old_rmin + r_buff;
            R delta_max = (rmax * lmin - old_rmin) / R(2.0);
            R maxsq = (delta_max > 0) ? delta_max * delta_max : 0;
            R dx = pos[4 * i] - lam[0] * last_pos[4 * i];
            R dy = pos[4 * i + 1] - lam[1] * last_pos[4 * i + 1];
            R dz = pos[4 * i + 2] - lam[2] * last_pos[4 * i + 2];
            box.min_image_rint(dx, dy, dz);
            if (dx * dx + dy * dy + dz * dz >= maxsq)
                moved = 1;
            }
        return moved != 0;
        }

    bool build()
        {
        // cell list sized to r_cut_max + r_buff (NeighborListBinned.cc:38-46)
        unsigned int d[3];
        cell_dims(box, ndim, max_rcut() + r_buff, d);
        if (d[0] != dim[0] || d[1] != dim[1] || d[2] != dim[2] || adj.empty())
            {
            dim[0] = d[0];
            dim[1] = d[1];
            dim[2] = d[2];
            unsigned int ncell = dim[0] * dim[1] * dim[2];
            Nmax_cell = std::max(1u, unsigned(std::ceil(double(N) / double(ncell))));
            adj.assign(size_t(27) * ncell, 0);
            adj_w = cell_adj(dim, ndim, 1, adj.data());
            }
        unsigned int ncell = dim[0] * dim[1] * dim[2];
        while (true)
            {
            cell_size.assign(ncell, 0);
            xyzf.assign(size_t(4) * ncell * Nmax_cell, 0);
            unsigned int cond[3];
            cell_list(N, pos.data(), box, dim, Nmax_cell, cell_size.data(), xyzf.data(), cond);
            if (cond[1])
                {
                error = "Particle with unique tag " + std::to_string(tags[cond[1] - 1])
                        + " has NaN for its position.";
                return false;
                }
            if (cond[2])
                {
                error = "Particle with unique tag " + std::to_string(tags[cond[2] - 1])
                        + " is no longer in the simulation box.";
                return false;
                }
            if (cond[0] > Nmax_cell)
                {
                Nmax_cell = cond[0];
                continue;
                }
            break;
            }
        while (true)
            {
            nl_cond.assign(ntypes, 0);
            nlist_binned(N, pos.data(), box, ntypes, r_cut.data(), r_listsq.data(), full, dim,
                         cell_size.data(), xyzf.data(), Nmax_cell, adj.data(), adj_w, Nmax.data(),
                         head_list.data(), nlist.data(), n_neigh.data(), nl_cond.data(), false,
                         nthreads);
            bool overflow = false;
            for (unsigned int t = 0; t < ntypes; t++)
                if (nl_cond[t] > Nmax[t])
                    {
                    Nmax[t] = (nl_cond[t] > 4) ? (nl_cond[t] + 3) & ~3u : 4;
                    overflow = true;
                    }
            if (!overflow)
                break;
            build_head_list();
            }
        for (unsigned int i = 0; i < N; i++)
            {
            last_pos[4 * i] = pos[4 * i];
            last_pos[4 * i + 1] = pos[4 * i + 1];
            last_pos[4 * i + 2] = pos[4 * i + 2];
            last_pos[4 * i + 3] = 0;
            }
        box.nearest_plane_distance(last_L);
        n_builds++;
        return true;
        }

    // NeighborList::shouldCheckDistance / needsUpdating (hoomd/md/NeighborList.cc:1313-1418) for
    // the forces of step T: a forced update builds at once; otherwise nothing is checked until
    // check_delay steps after the last build, the list is rebuilt without a check when r_buff is
    // tiny or (without dist_check) when the delay is 0 or just ran out, and the distance check
    // decides in every other case. A build at the first check after a delay > 1 is dangerous.
    bool needs_updating(uint64_t T)
        {
        if (force_update)
            {
            force_update = false;
            last_updated = T;
            return true;
            }
        if (T < last_updated + check_delay)
            return false;
        const bool dangerous = dist_check && check_delay > 1 && T == last_updated + check_delay;
        bool result;
        if (r_buff < R(1e-6)
            || (!dist_check
                && (check_delay == 0 || (check_delay > 1 && T == last_updated + check_delay))))
            result = true;
        else
            result = distance_check();
        if (result)
            {
            last_updated = T;
            n_updates++;
            if (dangerous)
                n_dangerous++;
            }
        return result;
        }

    bool compute_forces(uint64_t T)
        {
        if (force_update)
            build_head_list();
        const bool rebuild = needs_updating(T);
        if (rebuild)
            {
            // NeighborList::checkBoxSize (hoomd/md/NeighborList.cc:535-561)
            R npd[3];
            box.nearest_plane_distance(npd);
            R rmax = max_rcut() + r_buff;
            if ((box.periodic[0] && npd[0] <= rmax * R(2.0))
                || (box.periodic[1] && npd[1] <= rmax * R(2.0))
                || (ndim == 3 && box.periodic[2] && npd[2] <= rmax * R(2.0)))
                {
                error = "nlist: Simulation box is too small, the neighbor list is searching beyond "
                        "the minimum image";
                return false;
                }
            if (!build())
                return false;
            }
        if (kind == 0)
            pair_forces<R, LJ<R>>(N, pos.data(), box, ntypes, lj.data(), rcutsq.data(), ronsq.data(),
                                  shift_mode, n_neigh.data(), nlist.data(), head_list.data(), !full,
                                  false, force.data(), nullptr, false, nthreads);
        else
            pair_forces<R, Table<R>>(N, pos.data(), box, ntypes, table.data(), rcutsq.data(),
                                     ronsq.data(), 0, n_neigh.data(), nlist.data(),
                                     head_list.data(), !full, false, force.data(), nullptr, false,
                                     nthreads);
        return true;
        }

    bool prep_run()
        {
        if (!compute_forces(timestep))
            return false;
        for (unsigned int j = 0; j < N; j++)
            {
            R minv = R(1.0) / vel[4 * j + 3];
            accel[3 * j] = force[4 * j] * minv;
            accel[3 * j + 1] = force[4 * j + 1] * minv;
            accel[3 * j + 2] = force[4 * j + 2] * minv;
            }
        prepared = true;
        return true;
        }

    double dof() const
        {
        // IntegratorTwoStep::getTranslationalDOF: D*N - D for one momentum-conserving method on all
        // particles; D*N for Langevin (TwoStepLangevinBase::isMomentumConserving)
        return langevin ? double(ndim) * N : double(ndim) * N - double(ndim);
        }

    bool step()
        {
        if (langevin)
            {
            nve_step_one(N, pos.data(), vel.data(), accel.data(), image.data(), box, dt, nthreads);
            if (!compute_forces(timestep + 1))
                return false;
            const double e = langevin_step_two(N, vel.data(), accel.data(), pos.data(),
                                               tags.data(), force.data(), gamma.data(),
                                               langevin_T, dt, seed, timestep, ndim);
            reservoir -= e * double(dt);
            timestep++;
            return true;
            }
        if (thermostat == 2)
            {
            // BerendsenThermostat::getRescalingFactorsOne (hoomd/md/Thermostat.h:469-489)
            double K = kinetic_energy(N, vel.data());
            if (K == 0.0)
                {
                error = "Berendsen thermostat requires non-zero initial temperatures";
                return false;
                }
            double T_cur = 2.0 * K / dof();
            R s = R(std::sqrt(1.0 + double(dt) / tau * (kT / T_cur - 1.0)));
            cv_step_one(N, pos.data(), vel.data(), accel.data(), image.data(), box, dt, s,
                        nthreads);
            if (!compute_forces(timestep + 1))
                return false;
            cv_step_two(N, vel.data(), accel.data(), force.data(), dt, R(1.0), nthreads);
            timestep++;
            return true;
            }
        if (thermostat == 3)
            {
            // MTTKThermostat (hoomd/md/Thermostat.h:148-177) in TwoStepConstantVolume's order:
            // scale, advance (xi, eta) on the half-step temperature, forces, scale
            const double ddt = double(dt);
            R s1 = R(std::exp(-(1.0 / 2.0) * xi * ddt));
            cv_step_one(N, pos.data(), vel.data(), accel.data(), image.data(), box, dt, s1,
                        nthreads);
            double T_cur = 2.0 * kinetic_energy(N, vel.data()) / dof();
            double drive = (1.0 / 2.0) * ddt / tau / tau * (T_cur / kT - 1.0);
            double xi_prime = xi + drive;
            xi = xi_prime + drive;
            eta += xi_prime * ddt;
            if (!compute_forces(timestep + 1))
                return false;
            R s2 = R(std::exp(-(1.0 / 2.0) * xi * ddt));
            cv_step_two(N, vel.data(), accel.data(), force.data(), dt, s2, nthreads);
            timestep++;
            return true;
            }
        R s = R(1.0);
        if (bussi)
            {
            double K = kinetic_energy(N, vel.data());
            if (K == 0.0)
                {
                error = "Bussi thermostat requires non-zero initial momenta.";
                return false;
                }
            s = R(bussi_factor(K, dof(), double(dt), tau, kT, timestep, seed, tags[0]));
            }
        cv_step_one(N, pos.data(), vel.data(), accel.data(), image.data(), box, dt, s, nthreads);
        if (!compute_forces(timestep + 1))
            return false;
        cv_step_two(N, vel.data(), accel.data(), force.data(), dt, R(1.0), nthreads);
        timestep++;
        return true;
        }
    };

} // namespace orc

using namespace orc;

// ------------------------------------------------------------------------------------------------
// C ABI for ctypes (tests, smoke check, CPU baseline). Arrays are in the oracle's precision R;
// scalar parameters arrive in double and are rounded to R exactly as a HOOMD build with
// Scalar = R would round the Python-side values.
// ------------------------------------------------------------------------------------------------
#define ORC_EXPORT extern "C" __attribute__((visibility("default")))

#define ORC_GEOMETRY(SUF, R)                                                                      \
    ORC_EXPORT void orc_min_image_##SUF(int n, const double* b6, const int* per, R* v3,             \
                                        int use_rint)                                              \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        for (int i = 0; i < n; i++)                                                                \
            {                                                                                      \
            if (use_rint)                                                                          \
                box.min_image_rint(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]);                       \
            else                                                                                   \
                box.min_image_branch(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]);                     \
            }                                                                                      \
        }                                                                                          \
    ORC_EXPORT void orc_wrap_##SUF(int n, const double* b6, const int* per, R* v3, int* img3)      \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        for (int i = 0; i < n; i++)                                                                \
            box.wrap(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2], img3[3 * i], img3[3 * i + 1],        \
                     img3[3 * i + 2]);                                                             \
        }                                                                                          \
    ORC_EXPORT void orc_make_fraction_##SUF(int n, const double* b6, const int* per, R* v3)        \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        for (int i = 0; i < n; i++)                                                                \
            box.make_fraction(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2], v3[3 * i], v3[3 * i + 1],   \
                              v3[3 * i + 2]);                                                      \
        }                                                                                          \
    ORC_EXPORT void orc_nearest_plane_distance_##SUF(const double* b6, const int* per, R* out3)    \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        box.nearest_plane_distance(out3);                                                          \
        }                                                                                          \
    ORC_EXPORT void orc_cell_dims_##SUF(const double* b6, const int* per, int ndim,                \
                                        double nominal_width, unsigned int* dim3)                  \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        cell_dims<R>(box, ndim, R(nominal_width), dim3);                                           \
        }                                                                                          \
    ORC_EXPORT void orc_cell_list_##SUF(unsigned int N, const R* pos, const double* b6,            \
                                        const int* per, const unsigned int* dim3,                  \
                                        unsigned int Nmax, unsigned int* cell_size, R* xyzf,       \
                                        unsigned int* cond3)                                       \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        cell_list<R>(N, pos, box, dim3, Nmax, cell_size, xyzf, cond3);                             \
        }                                                                                          \
    ORC_EXPORT void orc_nlist_binned_##SUF(                                                        \
        unsigned int N, const R* pos, const double* b6, const int* per, unsigned int ntypes,      \
        const R* r_cut, const R* r_listsq, int full, const unsigned int* dim3,                     \
        const unsigned int* cell_size, const R* xyzf, unsigned int Nmax_cell,                      \
        const unsigned int* adj, unsigned int adj_w, const unsigned int* Nmax,                     \
        const uint64_t* head_list, unsigned int* nlist, unsigned int* n_neigh,                     \
        unsigned int* conditions, int rint_min_image, int nthreads)                                \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        nlist_binned<R>(N, pos, box, ntypes, r_cut, r_listsq, full != 0, dim3, cell_size, xyzf,    \
                        Nmax_cell, adj, adj_w, Nmax, head_list, nlist, n_neigh, conditions,        \
                        rint_min_image != 0, nthreads);                                            \
        }                                                                                          \
    ORC_EXPORT void orc_lj_eval_##SUF(int n, const double* rsq, double rcutsq, double sigma,       \
                                      double eps, int shift, R* fdivr, R* eng, int* evaluated)     \
        {                                                                                          \
        auto p = LJ<R>::make_param(sigma, eps);                                                    \
        for (int i = 0; i < n; i++)                                                                \
            {                                                                                      \
            LJ<R> e(R(rsq[i]), R(rcutsq), p);                                                      \
            R f = 0, u = 0;                                                                        \
            evaluated[i] = e.eval(f, u, shift != 0);                                               \
            fdivr[i] = f;                                                                          \
            eng[i] = u;                                                                            \
            }                                                                                      \
        }                                                                                          \
    ORC_EXPORT void orc_lj_lrc_##SUF(double rcutsq, double sigma, double eps, R* out2)             \
        {                                                                                          \
        auto p = LJ<R>::make_param(sigma, eps);                                                    \
        LJ<R> e(R(0), R(rcutsq), p);                                                               \
        out2[0] = e.lrc_energy();                                                                  \
        out2[1] = e.lrc_pressure();                                                                \
        }                                                                                          \
    ORC_EXPORT void orc_table_eval_##SUF(int n, const double* rsq, double rcutsq, double rmin,     \
                                         int width, const R* V, const R* F, R* fdivr, R* eng,      \
                                         int* evaluated)                                           \
        {                                                                                          \
        typename Table<R>::param_type p {R(rmin), unsigned(width), V, F};                          \
        for (int i = 0; i < n; i++)                                                                \
            {                                                                                      \
            Table<R> e(R(rsq[i]), R(rcutsq), p);                                                   \
            R f = 0, u = 0;                                                                        \
            evaluated[i] = e.eval(f, u, false);                                                    \
            fdivr[i] = f;                                                                          \
            eng[i] = u;                                                                            \
            }                                                                                      \
        }                                                                                          \
    ORC_EXPORT void orc_example_eval_##SUF(int n, const double* rsq, double rcutsq, double k,      \
                                           double sigma, int shift, R* fdivr, R* eng,              \
                                           int* evaluated)                                         \
        {                                                                                          \
        typename Example<R>::param_type p {R(k), R(sigma)};                                        \
        for (int i = 0; i < n; i++)                                                                \
            {                                                                                      \
            Example<R> e(R(rsq[i]), R(rcutsq), p);                                                 \
            R f = 0, u = 0;                                                                        \
            evaluated[i] = e.eval(f, u, shift != 0);                                               \
            fdivr[i] = f;                                                                          \
            eng[i] = u;                                                                            \
            }                                                                                      \
        }                                                                                          \
    /* kind: 0 = LJ (params: ntypes^2 x {sigma, epsilon}), 1 = Table (params: ntypes^2 x       \
       {r_min, width, offset} into tdata), 2 = Example (params: ntypes^2 x {k, sigma}) */          \
    ORC_EXPORT void orc_pair_forces_##SUF(                                                         \
        int kind, unsigned int N, const R* pos, const double* b6, const int* per,                 \
        unsigned int ntypes, const double* params, const R* tdata, const R* rcutsq,               \
        const R* ronsq, int shift_mode, const unsigned int* n_neigh, const unsigned int* nlist,   \
        const uint64_t* head_list, int third_law, int compute_virial, R* force, R* virial,        \
        int rint_min_image, int nthreads, int abs_terms)                                           \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        unsigned int np = ntypes * ntypes;                                                         \
        if (kind == 0)                                                                             \
            {                                                                                      \
            std::vector<typename LJ<R>::param_type> p(np);                                         \
            for (unsigned int t = 0; t < np; t++)                                                  \
                p[t] = LJ<R>::make_param(params[2 * t], params[2 * t + 1]);                        \
            pair_forces<R, LJ<R>>(N, pos, box, ntypes, p.data(), rcutsq, ronsq, shift_mode,        \
                                  n_neigh, nlist, head_list, third_law != 0, compute_virial != 0,  \
                                  force, virial, rint_min_image != 0, nthreads, abs_terms);   \
            }                                                                                      \
        else if (kind == 1)                                                                        \
            {                                                                                      \
            std::vector<typename Table<R>::param_type> p(np);                                      \
            for (unsigned int t = 0; t < np; t++)                                                  \
                {                                                                                  \
                unsigned int w = unsigned(params[3 * t + 1]);                                      \
                size_t off = size_t(params[3 * t + 2]);                                            \
                p[t] = typename Table<R>::param_type {R(params[3 * t]), w, tdata + off,            \
                                                      tdata + off + w};                            \
                }                                                                                  \
            pair_forces<R, Table<R>>(N, pos, box, ntypes, p.data(), rcutsq, ronsq, 0, n_neigh,     \
                                     nlist, head_list, third_law != 0, compute_virial != 0, force, \
                                     virial, rint_min_image != 0, nthreads, abs_terms);       \
            }                                                                                      \
        else                                                                                       \
            {                                                                                      \
            std::vector<typename Example<R>::param_type> p(np);                                    \
            for (unsigned int t = 0; t < np; t++)                                                  \
                p[t] = typename Example<R>::param_type {R(params[2 * t]), R(params[2 * t + 1])};   \
            pair_forces<R, Example<R>>(N, pos, box, ntypes, p.data(), rcutsq, ronsq, shift_mode,   \
                                       n_neigh, nlist, head_list, third_law != 0,                  \
                                       compute_virial != 0, force, virial, rint_min_image != 0,    \
                                       nthreads, abs_terms);                                  \
            }                                                                                      \
        }                                                                                          \
    ORC_EXPORT void orc_cv_step_one_##SUF(unsigned int N, R* pos, R* vel, const R* accel,          \
                                          int* image, const double* b6, const int* per, double dt, \
                                          double s)                                                \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        cv_step_one<R>(N, pos, vel, accel, image, box, R(dt), R(s));                               \
        }                                                                                          \
    ORC_EXPORT void orc_cv_step_two_##SUF(unsigned int N, R* vel, R* accel, const R* net_force,    \
                                          double dt, double s)                                     \
        {                                                                                          \
        cv_step_two<R>(N, vel, accel, net_force, R(dt), R(s));                                     \
        }                                                                                          \
    ORC_EXPORT double orc_kinetic_energy_##SUF(unsigned int N, const R* vel)                       \
        {                                                                                          \
        return kinetic_energy<R>(N, vel);                                                          \
        }                                                                                          \
    ORC_EXPORT void orc_thermalize_##SUF(unsigned int N, R* vel, const unsigned int* tags,         \
                                         double kT, uint64_t timestep, unsigned int seed,          \
                                         int ndim)                                                 \
        {                                                                                          \
        thermalize<R>(N, vel, tags, R(kT), timestep, uint16_t(seed), ndim);                        \
        }                                                                                          \
    ORC_EXPORT void* orc_sim_create_##SUF(                                                         \
        unsigned int N, const R* pos, const R* vel, const int* image, const unsigned int* tags,   \
        const double* b6, const int* per, int ndim, unsigned int ntypes, int kind,                \
        const double* params, const R* tdata, size_t tdata_len, const double* r_cut,              \
        int shift_mode, double r_buff, int full, double dt, int bussi, double kT, double tau,     \
        unsigned int seed, uint64_t timestep, int nthreads)                                       \
        {                                                                                          \
        auto* s = new Sim<R>();                                                                    \
        s->N = N;                                                                                  \
        s->ntypes = ntypes;                                                                        \
        s->ndim = ndim;                                                                            \
        s->box.set(b6, per);                                                                       \
        s->pos.assign(pos, pos + 4 * size_t(N));                                                   \
        s->vel.assign(vel, vel + 4 * size_t(N));                                                   \
        s->image.assign(image, image + 3 * size_t(N));                                             \
        s->tags.assign(tags, tags + N);                                                            \
        s->accel.assign(3 * size_t(N), 0);                                                         \
        s->force.assign(4 * size_t(N), 0);                                                         \
        s->last_pos.assign(4 * size_t(N), 0);                                                      \
        s->n_neigh.assign(N, 0);                                                                   \
        s->kind = kind;                                                                            \
        unsigned int np = ntypes * ntypes;                                                         \
        s->r_cut.resize(np);                                                                       \
        s->rcutsq.resize(np);                                                                      \
        s->ronsq.assign(np, 0);                                                                    \
        for (unsigned int t = 0; t < np; t++)                                                      \
            {                                                                                      \
            s->r_cut[t] = R(r_cut[t]);                                                             \
            s->rcutsq[t] = s->r_cut[t] * s->r_cut[t];                                              \
            }                                                                                      \
        if (kind == 0)                                                                             \
            {                                                                                      \
            s->lj.resize(np);                                                                      \
            for (unsigned int t = 0; t < np; t++)                                                  \
                s->lj[t] = LJ<R>::make_param(params[2 * t], params[2 * t + 1]);                    \
            }                                                                                      \
        else                                                                                       \
            {                                                                                      \
            s->table_data.assign(tdata, tdata + tdata_len);                                        \
            s->table.resize(np);                                                                   \
            for (unsigned int t = 0; t < np; t++)                                                  \
                {                                                                                  \
                unsigned int w = unsigned(params[3 * t + 1]);                                      \
                size_t off = size_t(params[3 * t + 2]);                                            \
                s->table[t] = typename Table<R>::param_type {R(params[3 * t]), w,                  \
                                                             s->table_data.data() + off,           \
                                                             s->table_data.data() + off + w};      \
                }                                                                                  \
            }                                                                                      \
        s->shift_mode = shift_mode;                                                                \
        s->r_buff = R(r_buff);                                                                     \
        s->full = full != 0;                                                                       \
        s->dt = R(dt);                                                                             \
        s->bussi = bussi != 0;                                                                     \
        s->kT = kT;                                                                                \
        s->tau = tau;                                                                              \
        s->seed = uint16_t(seed);                                                                  \
        s->timestep = timestep;                                                                    \
        s->nthreads = nthreads;                                                                    \
        s->Nmax.assign(ntypes, 4);                                                                 \
        s->update_rlist();                                                                         \
        return s;                                                                                  \
        }                                                                                          \
    ORC_EXPORT void orc_sim_set_langevin_##SUF(void* h, double kT, const double* gamma)            \
        {                                                                                          \
        auto* s = (Sim<R>*)h;                                                                      \
        s->langevin = true;                                                                        \
        s->bussi = false;                                                                          \
        s->langevin_T = R(kT);                                                                     \
        s->gamma.assign(s->ntypes, R(0));                                                          \
        for (unsigned int t = 0; t < s->ntypes; t++)                                               \
            s->gamma[t] = R(gamma[t]);                                                             \
        }                                                                                          \
    ORC_EXPORT void orc_sim_set_thermostat_##SUF(void* h, int kind, double kT, double tau,          \
                                                 double xi, double eta)                            \
        {                                                                                          \
        auto* s = (Sim<R>*)h;                                                                      \
        s->thermostat = kind;                                                                      \
        s->bussi = kind == 1;                                                                      \
        s->kT = kT;                                                                                \
        s->tau = tau;                                                                              \
        s->xi = xi;                                                                                \
        s->eta = eta;                                                                              \
        }                                                                                          \
    ORC_EXPORT void orc_sim_mttk_##SUF(void* h, double* out2)                                      \
        {                                                                                          \
        out2[0] = ((Sim<R>*)h)->xi;                                                                \
        out2[1] = ((Sim<R>*)h)->eta;                                                               \
        }                                                                                          \
    ORC_EXPORT double orc_sim_reservoir_##SUF(void* h)                                             \
        {                                                                                          \
        return ((Sim<R>*)h)->reservoir;                                                            \
        }                                                                                          \
    ORC_EXPORT void orc_cv_step_one_capped_##SUF(unsigned int N, R* pos, R* vel, const R* accel,   \
                                                 int* image, const double* b6, const int* per,     \
                                                 double dt, double s, double limit)                \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        cv_step_one<R>(N, pos, vel, accel, image, box, R(dt), R(s), 1, R(limit));                  \
        }                                                                                          \
    ORC_EXPORT void orc_bd_step_one_##SUF(unsigned int N, R* pos, R* vel, const R* force,          \
                                          int* image, const unsigned int* tags,                    \
                                          const double* gamma, unsigned int ntypes,                \
                                          const double* b6, const int* per, double kT, double dt,  \
                                          unsigned int seed, uint64_t timestep, int ndim,          \
                                          int noiseless)                                           \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        std::vector<R> g(ntypes);                                                                  \
        for (unsigned int t = 0; t < ntypes; t++)                                                  \
            g[t] = R(gamma[t]);                                                                    \
        bd_step_one<R>(N, pos, vel, force, image, tags, g.data(), box, R(kT), R(dt),               \
                       uint16_t(seed), timestep, ndim, noiseless != 0);                            \
        }                                                                                          \
    ORC_EXPORT void orc_npt_step_one_##SUF(unsigned int N, R* pos, R* vel, const R* accel,         \
                                           int* image, const double* b6, const int* per, double dt, \
                                           double s, const float* mv, const float* mr,             \
                                           const float* mri)                                       \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        R a[6], b[6], c[6];                                                                        \
        for (int k = 0; k < 6; k++)                                                                \
            {                                                                                      \
            a[k] = R(mv[k]);                                                                       \
            b[k] = R(mr[k]);                                                                       \
            c[k] = R(mri[k]);                                                                      \
            }                                                                                      \
        npt_step_one<R>(N, pos, vel, accel, image, box, R(dt), R(s), a, b, c);                     \
        }                                                                                          \
    ORC_EXPORT void orc_npt_step_two_##SUF(unsigned int N, R* vel, R* accel, const R* net_force,   \
                                           double dt, double s, const float* mv)                   \
        {                                                                                          \
        R a[6];                                                                                    \
        for (int k = 0; k < 6; k++)                                                                \
            a[k] = R(mv[k]);                                                                       \
        npt_step_two<R>(N, vel, accel, net_force, R(dt), R(s), a);                                 \
        }                                                                                          \
    ORC_EXPORT void orc_nve_step_one_##SUF(unsigned int N, R* pos, R* vel, const R* accel,         \
                                           int* image, const double* b6, const int* per,           \
                                           double dt)                                              \
        {                                                                                          \
        Box<R> box;                                                                                \
        box.set(b6, per);                                                                          \
        nve_step_one<R>(N, pos, vel, accel, image, box, R(dt));                                    \
        }                                                                                          \
    ORC_EXPORT double orc_langevin_step_two_##SUF(                                                 \
        unsigned int N, R* vel, R* accel, const R* pos, const unsigned int* tags,                  \
        const R* net_force, const double* gamma, unsigned int ntypes, double kT, double dt,        \
        unsigned int seed, uint64_t timestep, int ndim)                                            \
        {                                                                                          \
        std::vector<R> g(ntypes);                                                                  \
        for (unsigned int t = 0; t < ntypes; t++)                                                  \
            g[t] = R(gamma[t]);                                                                    \
        return langevin_step_two<R>(N, vel, accel, pos, tags, net_force, g.data(), R(kT), R(dt),   \
                                    uint16_t(seed), timestep, ndim);                               \
        }                                                                                          \
    ORC_EXPORT int orc_sim_run_##SUF(void* h, uint64_t nsteps)                                     \
        {                                                                                          \
        auto* s = (Sim<R>*)h;                                                                      \
        if (!s->prepared && !s->prep_run())                                                        \
            return -1;                                                                             \
        for (uint64_t k = 0; k < nsteps; k++)                                                      \
            if (!s->step())                                                                        \
                return -1;                                                                         \
        return 0;                                                                                  \
        }                                                                                          \
    ORC_EXPORT const char* orc_sim_error_##SUF(void* h)                                            \
        {                                                                                          \
        return ((Sim<R>*)h)->error.c_str();                                                        \
        }                                                                                          \
    ORC_EXPORT void orc_sim_get_##SUF(void* h, R* pos, R* vel, int* image, R* force, R* accel)     \
        {                                                                                          \
        auto* s = (Sim<R>*)h;                                                                      \
        size_t N = s->N;                                                                           \
        if (pos)                                                                                   \
            std::copy(s->pos.begin(), s->pos.end(), pos);                                          \
        if (vel)                                                                                   \
            std::copy(s->vel.begin(), s->vel.end(), vel);                                          \
        if (image)                                                                                 \
            std::copy(s->image.begin(), s->image.end(), image);                                    \
        if (force)                                                                                 \
            std::copy(s->force.begin(), s->force.begin() + 4 * N, force);                          \
        if (accel)                                                                                 \
            std::copy(s->accel.begin(), s->accel.end(), accel);                                    \
        }                                                                                          \
    ORC_EXPORT void orc_sim_set_check_##SUF(void* h, unsigned int delay, int dist_check)           \
        {                                                                                          \
        auto* s = (Sim<R>*)h;                                                                      \
        s->check_delay = delay;                                                                    \
        s->dist_check = dist_check != 0;                                                           \
        }                                                                                          \
    /* stats: [timestep, n_builds, sum n_neigh, kinetic energy, potential energy, checked builds,  \
       dangerous builds, step of the last build] */                                               \
    ORC_EXPORT void orc_sim_stats_##SUF(void* h, double* out5)                                     \
        {                                                                                          \
        auto* s = (Sim<R>*)h;                                                                      \
        double nn = 0, pe = 0;                                                                     \
        for (unsigned int i = 0; i < s->N; i++)                                                    \
            {                                                                                      \
            nn += s->n_neigh[i];                                                                   \
            pe += double(s->force[4 * i + 3]);                                                     \
            }                                                                                      \
        out5[0] = double(s->timestep);                                                             \
        out5[1] = double(s->n_builds);                                                             \
        out5[2] = nn;                                                                              \
        out5[3] = kinetic_energy<R>(s->N, s->vel.data());                                          \
        out5[4] = pe;                                                                              \
        out5[5] = double(s->n_updates);                                                            \
        out5[6] = double(s->n_dangerous);                                                          \
        out5[7] = double(s->last_updated);                                                         \
        }                                                                                          \
    ORC_EXPORT void orc_sim_destroy_##SUF(void* h)                                                 \
        {                                                                                          \
        delete (Sim<R>*)h;                                                                         \
        }

ORC_GEOMETRY(f32, float)
ORC_GEOMETRY(f64, double)

ORC_EXPORT void orc_sfc_order_f32(unsigned int N, const float* pos, const double* b6,
                                  const int* per, unsigned int grid, int ndim,
                                  unsigned int* order)
    {
    Box<float> box;
    box.set(b6, per);
    sfc_order<float>(N, pos, box, grid, ndim, order);
    }

ORC_EXPORT unsigned int orc_cell_adj(const unsigned int* dim3, int ndim, int radius,
                                     unsigned int* adj)
    {
    return cell_adj(dim3, ndim, radius, adj);
    }

ORC_EXPORT void orc_philox4x32_10(const uint32_t* ctr4, const uint32_t* key2, uint32_t* out4)
    {
    philox4x32_10(ctr4, key2, out4);
    }

ORC_EXPORT void orc_rng_seed_key(unsigned int id, uint64_t timestep, unsigned int seed,
                                 uint32_t* key2)
    {
    RNG r(uint8_t(id), timestep, uint16_t(seed), 0);
    key2[0] = r.key[0];
    key2[1] = r.key[1];
    }

ORC_EXPORT double orc_bussi_factor(double K, double dof, double dt, double tau, double kT,
                                   uint64_t timestep, unsigned int seed, unsigned int instance_id)
    {
    return bussi_factor(K, dof, dt, tau, kT, timestep, uint16_t(seed), instance_id);
    }

ORC_EXPORT void orc_normal_draws(unsigned int id, uint64_t timestep, unsigned int seed,
                                 unsigned int ctr_a, int n, double* out)
    {
    RNG rng(uint8_t(id), timestep, uint16_t(seed), ctr_a);
    for (int i = 0; i < n; i++)
        out[i] = normal<double>(rng);
    }

ORC_EXPORT void orc_gamma_draws(unsigned int id, uint64_t timestep, unsigned int seed,
                                unsigned int ctr_a, double alpha, int n, double* out)
    {
    RNG rng(uint8_t(id), timestep, uint16_t(seed), ctr_a);
    for (int i = 0; i < n; i++)
        out[i] = gamma<double>(rng, alpha, 1.0);
    }
