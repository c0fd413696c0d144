// ConstantPressure: the MTK barostat of TwoStepConstantPressure (hoomd/md/TwoStepConstantPressure.cc)
// with the MTTK thermostat or none, translational degrees of freedom. The box changes every
// step, so this method runs a host-driven loop: the barostat and thermostat variables advance
// on the host in FP64 from FP64 device reductions (kinetic and virial tensors), the particle
// halves run on the device (gb_npt_step_one / two), and the neighbour list is rebuilt for the
// new box each step (the reference's rebuild check scales the last positions by the box ratio;
// rebuilding every step gives the same pairs).
#include <cmath>
#include <stdexcept>

#include "engine.h"
#include "rng.cuh"

namespace gbe
{
namespace
{
// Taylor coefficients of sinh(x)/x, coth(x) - 1/x and 1/x^2 - 1/sinh(x)^2, as the reference's
// propagator uses them (hoomd/md/TwoStepConstantPressure.cc:14-37). The reference's fifth
// coefficient of coth(x) - 1/x is 1/93555 (the series has 2/93555); it is kept for parity (it
// weighs an x^9 term).
const double F_COEFF[6] = {1.0, 1.0 / 6.0, 1.0 / 120.0, 1.0 / 5040.0, 1.0 / 362880.0,
                           1.0 / 39916800.0};
const double G_COEFF[5] = {1.0 / 3.0, -1.0 / 45.0, 2.0 / 945.0, -1.0 / 4725.0, 1.0 / 93555.0};
const double H_COEFF[6] = {1.0 / 3.0, -1.0 / 15.0, 2.0 / 189.0, -1.0 / 675.0, 2.0 / 10395.0,
                           -1382.0 / 58046625.0};

enum
    {
    BARO_X = 1,
    BARO_Y = 2,
    BARO_Z = 4,
    BARO_XY = 8,
    BARO_XZ = 16,
    BARO_YZ = 32
    };
enum
    {
    COUPLE_NONE = 0,
    COUPLE_XY = 1,
    COUPLE_XZ = 2,
    COUPLE_YZ = 3,
    COUPLE_XYZ = 4
    };

// Standard normal draw (Box-Muller, one value per Philox block as hoomd/RandomNumbers.h:346-372)
double normal_host(gb::Philox& rng)
    {
    uint64_t u0, u1;
    rng.two_u64(u0, u1);
    const double a = gb::uneg11<double>(u0), b = gb::u01<double>(u1);
    return std::sin(M_PI * a) * std::sqrt(-2.0 * std::log(b));
    }
} // namespace

void Integrator::set_npt(const std::vector<double>& S, double tauS, int couple,
                         const std::vector<int>& box_dof, double gamma_)
    {
    if (S.size() != 6 || box_dof.size() != 6)
        throw std::invalid_argument("ConstantPressure: S and box_dof have six entries");
    if (!(tauS > 0.0))
        throw std::invalid_argument("ConstantPressure: tauS must be positive");
    if (couple < COUPLE_NONE || couple > COUPLE_XYZ)
        throw std::invalid_argument("ConstantPressure: invalid couple");
    if (bussi || berendsen || langevin || brownian)
        throw std::invalid_argument("ConstantPressure runs with the MTTK thermostat or none");
    for (int k = 0; k < 6; k++)
        npt_S[k] = S[k];
    npt_tauS = tauS;
    npt_couple = couple;
    npt_gamma = gamma_;
    const unsigned int bits[6] = {BARO_X, BARO_Y, BARO_Z, BARO_XY, BARO_XZ, BARO_YZ};
    npt_flags = 0;
    for (int k = 0; k < 6; k++)
        if (box_dof[k])
            npt_flags |= bits[k];
    if (pdata->ndim == 2)
        npt_flags &= ~(unsigned)(BARO_Z | BARO_XZ | BARO_YZ);
    npt = true;
    npt_tensor.clear();
    prepared = false;
    drop_graphs();
    }

std::vector<double> Integrator::barostat_dof()
    {
    return {nu[0], nu[1], nu[2], nu[3], nu[4], nu[5]};
    }

void Integrator::set_barostat_dof(const std::vector<double>& v)
    {
    if (v.size() != 6)
        throw std::length_error("barostat_dof must have length 6");
    for (int k = 0; k < 6; k++)
        nu[k] = v[k];
    }

// the thermostat's set point, or 1 without a thermostat (getTimestepTemperature)
double Integrator::npt_temperature() const
    {
    return mttk ? kT : 1.0;
    }

// TwoStepConstantPressure::getBarostatEnergy (:727-745)
double Integrator::barostat_energy()
    {
    const double d = pdata->ndim;
    const double W = (dof() + d) / d * npt_temperature() * npt_tauS * npt_tauS;
    return W * (nu[0] * nu[0] + nu[3] * nu[3] + nu[5] * nu[5] + nu[1] * nu[1] + nu[2] * nu[2]
                + nu[4] * nu[4])
           / 2.0;
    }

std::vector<double> Integrator::thermo_tensor()
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    DeviceArray<char> scratch;
    scratch.resize(gb_thermo_tensor_scratch_bytes(pd.N));
    DeviceArray<double> out;
    out.resize(13);
    std::vector<double> total(13, 0.0);
    for (size_t k = 0; k < forces.size(); k++)
        {
        PairForce& f = *forces[k];
        if (!f.virial_valid)
            f.compute(s, true);
        check(gb_thermo_tensor(pd.vel.get(), f.force.get(), f.virial.get(), pd.N, pd.N,
                               scratch.get(), out.get(), s),
              "gb_thermo_tensor");
        double h[13];
        out.download(h, 13, s);
        cuda_check(cudaStreamSynchronize(s), "thermo tensor");
        for (int t = 0; t < 13; t++)
            total[t] += (t < 6 && k > 0) ? 0.0 : h[t];
        const double V = f.box_volume();
        total[6] += f.tail_virial / V;
        total[9] += f.tail_virial / V;
        total[11] += f.tail_virial / V;
        total[12] += f.tail_energy / V;
        }
    return total;
    }

// TwoStepConstantPressure::advanceBarostat (:869-997) from the tensors of the last full step
void Integrator::npt_advance_barostat(uint64_t timestep)
    {
    ParticleData& pd = *pdata;
    const double d = pd.ndim;
    const double* b = pd.box6;
    const double V = pd.ndim == 2 ? b[0] * b[1] : b[0] * b[1] * b[2];
    const std::vector<double>& t = npt_tensor;
    // pressure tensor (kinetic + virial) / V; components xx, xy, xz, yy, yz, zz
    double P[6];
    for (int k = 0; k < 6; k++)
        P[k] = (t[k] + t[6 + k]) / V;
    const double Pxx = P[0], Pxy = P[1], Pxz = P[2], Pyy = P[3], Pyz = P[4], Pzz = P[5];
    const double T = npt_temperature();
    const double W = (dof() + d) / d * T * npt_tauS * npt_tauS;
    double mtk_term = 2.0 * (0.5 * (t[0] + t[3] + t[5]));
    mtk_term *= 0.5 * dt / dof() / W;
    // getRelevantCouplings (:133-171)
    int couple = npt_couple;
    if (!(npt_flags & BARO_X))
        {
        if (couple == COUPLE_XYZ)
            couple = COUPLE_YZ;
        if (couple == COUPLE_XY || couple == COUPLE_XZ)
            couple = COUPLE_NONE;
        }
    if (!(npt_flags & BARO_Y))
        {
        if (couple == COUPLE_XYZ)
            couple = COUPLE_XZ;
        if (couple == COUPLE_YZ || couple == COUPLE_XY)
            couple = COUPLE_NONE;
        }
    if (!(npt_flags & BARO_Z))
        {
        if (couple == COUPLE_XYZ)
            couple = COUPLE_XY;
        if (couple == COUPLE_YZ || couple == COUPLE_XZ)
            couple = COUPLE_NONE;
        }
    gb::Philox rng(46, timestep, pd.seed, 0u);
    double Pd[3], R[3];
    switch (couple)
        {
    case COUPLE_NONE:
        Pd[0] = Pxx;
        R[0] = normal_host(rng);
        Pd[1] = Pyy;
        R[1] = normal_host(rng);
        Pd[2] = Pzz;
        R[2] = normal_host(rng);
        break;
    case COUPLE_XY:
        Pd[0] = Pd[1] = 0.5 * (Pxx + Pyy);
        R[0] = R[1] = normal_host(rng);
        Pd[2] = Pzz;
        R[2] = normal_host(rng);
        break;
    case COUPLE_XZ:
        Pd[0] = Pd[2] = 0.5 * (Pxx + Pzz);
        R[0] = R[2] = normal_host(rng);
        Pd[1] = Pyy;
        R[1] = normal_host(rng);
        break;
    case COUPLE_YZ:
        Pd[0] = Pxx;
        R[0] = normal_host(rng);
        Pd[1] = Pd[2] = 0.5 * (Pyy + Pzz);
        R[1] = R[2] = normal_host(rng);
        break;
    default:
        Pd[0] = Pd[1] = Pd[2] = (Pxx + Pyy + Pzz) / 3.0;
        R[0] = R[1] = R[2] = normal_host(rng);
        break;
        }
    const double e = std::exp(-npt_gamma * dt / 2.0);
    const double coeff = std::sqrt(T * (1.0 - e * e) / W);
    const double k = 0.5 * dt * V / W;
    // S = (xx, yy, zz, yz, xz, xy); nu = (xx, xy, xz, yy, yz, zz)
    if (npt_flags & BARO_X)
        nu[0] = nu[0] * e + coeff * R[0] + k * (Pd[0] - npt_S[0]) + mtk_term;
    if (npt_flags & BARO_XY)
        {
        nu[1] = nu[1] * e + coeff * normal_host(rng);
        nu[1] += k * (Pxy - npt_S[5]);
        }
    if (npt_flags & BARO_XZ)
        {
        nu[2] = nu[2] * e + coeff * normal_host(rng);
        nu[2] += k * (Pxz - npt_S[4]);
        }
    if (npt_flags & BARO_Y)
        nu[3] = nu[3] * e + coeff * R[1] + k * (Pd[1] - npt_S[1]) + mtk_term;
    if (npt_flags & BARO_YZ)
        {
        nu[4] = nu[4] * e + coeff * normal_host(rng);
        nu[4] += k * (Pyz - npt_S[3]);
        }
    if (npt_flags & BARO_Z)
        nu[5] = nu[5] * e + coeff * R[2] + k * (Pd[2] - npt_S[2]) + mtk_term;
    }

// TwoStepConstantPressure::updatePropagator (:746-867): upper-triangular exponentials of the
// barostat matrix for the velocities (mat_v), positions (mat_r) and the integral of the
// positions' propagator (mat_ri), to second order in dt in the off-diagonal terms.
void Integrator::npt_update_propagator()
    {
    const double h = dt;
    const double nxx = nu[0], nxy = nu[1], nxz = nu[2], nyy = nu[3], nyz = nu[4], nzz = nu[5];
    const double vf[3] = {-0.25 * nxx, -0.25 * nyy, -0.25 * nzz};
    const double ev2[3] = {std::exp(2.0 * vf[0] * h), std::exp(2.0 * vf[1] * h),
                           std::exp(2.0 * vf[2] * h)};
    const double rf[3] = {0.5 * nxx, 0.5 * nyy, 0.5 * nzz};
    const double er[3] = {std::exp(0.5 * nxx * h), std::exp(0.5 * nyy * h),
                          std::exp(0.5 * nzz * h)};
    const double er2[3] = {std::exp(nxx * h), std::exp(nyy * h), std::exp(nzz * h)};
    double f_r[3] = {0, 0, 0}, g_r[3] = {0, 0, 0}, h_r[3] = {0, 0, 0};
    for (int a = 0; a < 3; a++)
        {
        const double x = rf[a] * h;
        double term = 1.0;
        for (int i = 0; i < 6; i++)
            {
            f_r[a] += F_COEFF[i] * term;
            term = term * x * x;
            }
        term = x;
        for (int i = 0; i < 5; i++)
            {
            g_r[a] += G_COEFF[i] * term;
            term = term * x * x;
            }
        term = 1.0;
        for (int i = 0; i < 6; i++)
            {
            h_r[a] += H_COEFF[i] * term;
            term = term * x * x;
            }
        }
    mat_v[0] = ev2[0];
    mat_v[1] = -h * 0.25 * nxy * (ev2[0] + ev2[1]);
    mat_v[2] = -h * 0.25 * nxz * (ev2[0] + ev2[2])
               + h * h * (1.0 / 32.0) * nxy * nyz * (ev2[0] + 2.0 * ev2[1] + ev2[2]);
    mat_v[3] = ev2[1];
    mat_v[4] = -h * 0.25 * nyz * (ev2[1] + ev2[2]);
    mat_v[5] = ev2[2];
    mat_r[0] = er2[0];
    mat_r[1] = h * 0.5 * nxy * (er2[0] + er2[1]);
    mat_r[2] = h * 0.5 * nxz * (er2[0] + er2[2])
               + h * h * (1.0 / 8.0) * nxy * nyz * (er2[0] + 2.0 * er2[1] + er2[2]);
    mat_r[3] = er2[1];
    mat_r[4] = h * 0.5 * nyz * (er2[1] + er2[2]);
    mat_r[5] = er2[2];
    double xz_fac[3];
    for (int a = 0; a < 3; a++)
        xz_fac[a] = (1.0 + g_r[a]) * (1.0 + g_r[a]) + h_r[a];
    mat_ri[0] = h * er[0] * f_r[0];
    mat_ri[1] = h * h * nxy * 0.25
                * (er[0] * f_r[0] * (1.0 + g_r[0]) + er[1] * f_r[1] * (1.0 + g_r[1]));
    mat_ri[2] = h * h * nxz * 0.25
                    * (er[0] * f_r[0] * (1.0 + g_r[0]) + er[2] * f_r[2] * (1.0 + g_r[2]))
                + h * h * h * nxy * nyz * (1.0 / 32.0)
                      * (er[0] * f_r[0] * xz_fac[0] + 2.0 * er[1] * f_r[1] * xz_fac[1]
                         + er[2] * f_r[2] * xz_fac[2]);
    mat_ri[3] = h * er[1] * f_r[1];
    mat_ri[4] = h * h * nyz * 0.25
                * (er[1] * f_r[1] * (1.0 + g_r[1]) + er[2] * f_r[2] * (1.0 + g_r[2]));
    mat_ri[5] = h * er[2] * f_r[2];
    }

// IntegratorTwoStep::update with TwoStepConstantPressure (:206-330 step one, :587-711 step two).
void Integrator::run_npt(uint64_t nsteps)
    {
    ParticleData& pd = *pdata;
    cudaStream_t s = pd.stream;
    if (npt_tensor.empty())
        npt_tensor = thermo_tensor();
    if (mttk && prepared)
        {
        const DevStatus st = read_status();
        mttk_host[0] = st.mttk[0];
        mttk_host[1] = st.mttk[1];
        }
    DeviceArray<double> ke_out;
    ke_out.resize(3);
    d_thermo_scratch.resize(gb_thermo_scratch_bytes(pd.N));
    const double ndof = dof();
    for (uint64_t step = 0; step < nsteps; step++)
        {
        const uint64_t t = pd.timestep;
        if (sort_period && t % sort_period == 0)
            {
            sort_particles();
            npt_tensor = thermo_tensor();
            }
        // step one
        npt_advance_barostat(t);
        double s1 = std::exp(-0.5 * dt * (nu[0] + nu[3] + nu[5]) / ndof);
        if (mttk)
            s1 *= std::exp(-0.5 * mttk_host[0] * dt);
        npt_update_propagator();
        // the box's lattice vectors under mat_r
        const double* b = pd.box6;
        double ax = b[0], bx = b[3] * b[1], by = b[1], cx = b[4] * b[2], cy = b[5] * b[2],
               cz = b[2];
        ax = mat_r[0] * ax;
        bx = mat_r[0] * bx + mat_r[1] * by;
        by = mat_r[3] * by;
        cx = mat_r[0] * cx + mat_r[1] * cy + mat_r[2] * cz;
        cy = mat_r[3] * cy + mat_r[4] * cz;
        cz = mat_r[5] * cz;
        double nb[6] = {ax, by, cz, bx / by, 0.0, 0.0};
        if (pd.ndim == 3)
            {
            nb[4] = cx / cz;
            nb[5] = cy / cz;
            }
        else
            nb[2] = b[2];
        pd.set_box(nb);
        float fv[6], fr[6], fri[6];
        for (int k = 0; k < 6; k++)
            {
            fv[k] = (float)mat_v[k];
            fr[k] = (float)mat_r[k];
            fri[k] = (float)mat_ri[k];
            }
        check(gb_npt_step_one(pd.pos.get(), pd.vel.get(), pd.accel.get(), pd.image.get(), pd.N,
                              &pd.box, (float)dt, (float)s1, fv, fr, fri, s),
              "gb_npt_step_one");
        if (mttk)
            {
            // MTTKThermostat::advanceThermostat on the half-step temperature (Thermostat.h:162-177)
            check(gb_thermo_reduce(pd.vel.get(), nullptr, nullptr, 0, pd.N,
                                   d_thermo_scratch.get(), ke_out.get(), s),
                  "thermo");
            double h[3];
            ke_out.download(h, 3, s);
            cuda_check(cudaStreamSynchronize(s), "thermo");
            const double T_cur = 2.0 * h[0] / ndof;
            const double drive = 0.5 * dt / tau / tau * (T_cur / kT - 1.0);
            const double xi_prime = mttk_host[0] + drive;
            mttk_host[0] = xi_prime + drive;
            mttk_host[1] += xi_prime * dt;
            }
        // forces at the new positions, in the new box, with the virial for the barostat
        nlist->dirty = true;
        nlist->build_sync();
        for (auto& f : forces)
            {
            f->force_timestep = t + 1;
            f->force_dt = (float)dt;
            f->compute(s, true);
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
        // step two
        double s2 = std::exp(-0.5 * dt * (nu[0] + nu[3] + nu[5]) / ndof);
        if (mttk)
            s2 *= std::exp(-0.5 * mttk_host[0] * dt);
        check(gb_npt_step_two(pd.vel.get(), pd.accel.get(), net, pd.N, (float)dt, (float)s2, fv,
                              s),
              "gb_npt_step_two");
        pd.timestep = t + 1;
        steps_run++;
        launch_count += 8 + forces.size();
        npt_tensor = thermo_tensor();
        npt_advance_barostat(t + 1);
        }
    // the device status follows the host state (timestep, thermostat) for later queries
    DevStatus st = read_status();
    st.timestep = pd.timestep;
    st.mttk[0] = mttk_host[0];
    st.mttk[1] = mttk_host[1];
    cuda_check(cudaMemcpyAsync(d_status.get(), &st, sizeof(st), cudaMemcpyHostToDevice, s),
               "status");
    cuda_check(cudaStreamSynchronize(s), "status");
    }

} // namespace gbe
