// Counter-based random numbers on the device, following the wrappers of hoomd/RandomNumbers.h
// around Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11; the random123 library is not part of
// the reference checkout, so the generator is written here from the published description), and
// the Bussi rescale factor of hoomd/md/Thermostat.h:416-446, all in double as the reference does.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
// host compilers: the generator and the uniform conversions are plain host code
#include <cuda_runtime.h>
#endif

namespace gb
{

struct Philox
    {
    uint32_t key[2];
    uint32_t ctr[4];

    // Seed (hoomd/RandomNumbers.h:136-168) + Counter(a, b, c, d) (:175-197)
    __host__ __device__ Philox(uint8_t id, uint64_t timestep, uint16_t seed, uint32_t a,
                               uint32_t b = 0, uint32_t c = 0, uint16_t d = 0)
        {
        key[0] = uint32_t(id) << 24 | uint32_t(seed) << 8
                 | uint32_t((timestep & 0x000000ff00000000ull) >> 32);
        key[1] = uint32_t(timestep & 0x00000000ffffffffull);
        ctr[0] = uint32_t(d) << 16;
        ctr[1] = c;
        ctr[2] = b;
        ctr[3] = a;
        }

    // Ten rounds of (c0,c1,c2,c3) -> (hi(M1*c2)^c1^k0, lo(M1*c2), hi(M0*c0)^c3^k1, lo(M0*c0)),
    // key bumped by the Weyl constants between rounds.
    __host__ __device__ void block(uint32_t out[4]) const
        {
        uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
        uint32_t k0 = key[0], k1 = key[1];
#pragma unroll
        for (int r = 0; r < 10; r++)
            {
            if (r > 0)
                {
                k0 += 0x9E3779B9u;
                k1 += 0xBB67AE85u;
                }
            const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
            const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
            const uint32_t n0 = uint32_t(p1 >> 32) ^ c1 ^ k0;
            const uint32_t n1 = uint32_t(p1);
            const uint32_t n2 = uint32_t(p0 >> 32) ^ c3 ^ k1;
            const uint32_t n3 = uint32_t(p0);
            c0 = n0;
            c1 = n1;
            c2 = n2;
            c3 = n3;
            }
        out[0] = c0;
        out[1] = c1;
        out[2] = c2;
        out[3] = c3;
        }

    // RandomGenerator::operator() (hoomd/RandomNumbers.h:264-270): draw, then bump counter word 0.
    __host__ __device__ void next(uint32_t out[4])
        {
        block(out);
        ctr[0] += 1;
        }
    __host__ __device__ uint64_t u64()
        {
        uint32_t o[4];
        next(o);
        return uint64_t(o[0]) << 32 | o[1];
        }
    __host__ __device__ void two_u64(uint64_t& a, uint64_t& b)
        {
        uint32_t o[4];
        next(o);
        a = uint64_t(o[0]) << 32 | o[1];
        b = uint64_t(o[2]) << 32 | o[3];
        }
    };

// Published random123 conversions: u01 -> (0,1], uneg11 -> [-1,1] (half-step offset).
template<class R> __host__ __device__ inline R u01(uint64_t in)
    {
    const R factor = R(1.) / (R(18446744073709551615.0) + R(1.));
    return R(in) * factor + R(0.5) * factor;
    }
template<class R> __host__ __device__ inline R uneg11(uint64_t in)
    {
    const R factor = R(1.) / (R(9223372036854775807.0) + R(1.));
    return R(int64_t(in)) * factor + R(0.5) * factor;
    }

// UniformDistribution<float>(-1, 1) (hoomd/RandomNumbers.h:317-341): a + width * u01(draw), one
// generator draw per value. The products by powers of two are exact, so contraction into a fused
// multiply-add cannot change the result.
__host__ __device__ inline float uniform_m11_f(Philox& rng)
    {
    return -1.0f + 2.0f * u01<float>(rng.u64());
    }

#ifdef __CUDACC__
// Box-Muller, one value per draw (hoomd/RandomNumbers.h:346-372).
__device__ inline double normal_d(Philox& rng)
    {
    uint64_t u0, u1;
    rng.two_u64(u0, u1);
    double s, c;
    sincospi(uneg11<double>(u0), &s, &c);
    const double r = sqrt(-2.0 * log(u01<double>(u1)));
    return s * r;
    }

__device__ inline float normal_f(Philox& rng)
    {
    uint64_t u0, u1;
    rng.two_u64(u0, u1);
    float s, c;
    sincospif(uneg11<float>(u0), &s, &c);
    const float r = sqrtf(-2.0f * logf(u01<float>(u1)));
    return s * r;
    }

// Marsaglia-Tsang gamma with squeeze test (hoomd/RandomNumbers.h:454-534). The rejection loop is
// bounded (acceptance is > 95% per iteration for alpha >= 1); after 64 rejections the last
// candidate is returned rather than spinning.
__device__ inline double gamma_d(Philox& rng, double shape, double scale)
    {
    // shape < 1: draw at shape + 1 and scale by U^(1/shape) (Marsaglia and Tsang, sect. 6)
    const double a = shape < 1.0 ? shape + 1.0 : shape;
    const double d = a - 1. / 3.;
    const double c = (1.0 / sqrt(d)) / 3.;
    double cube = 1.0;
    for (int it = 0; it < 64; it++)
        {
        double z;
        int tries = 0;
        do
            {
            z = normal_d(rng);
            cube = 1.0 + c * z;
            } while (cube <= 0. && ++tries < 64);
        cube = cube * cube * cube;
        const double z2 = z * z;
        const double u = u01<double>(rng.u64());
        if (u < 1.0 - 0.0331 * z2 * z2) // squeeze
            break;
        if (log(u) < 0.5 * z2 + d * (1.0 - cube + log(cube)))
            break;
        }
    double g = cube * d * scale;
    if (shape < 1.0)
        g *= pow(u01<double>(rng.u64()), 1.0 / shape);
    return g;
    }

// hoomd/md/Thermostat.h:357-391 (key id 45, counter = first member tag) and :416-446, split in
// two: the random draws of a timestep (one normal, then 2 * Gamma((dof-1)/2, 1)) depend only on
// the timestep, seed, counter and dof, so they can be drawn ahead for a run of steps, in
// parallel; the factor then needs only the kinetic energy and a few FP64 operations.
__device__ inline double2 bussi_draws_d(double dof, uint64_t timestep, uint16_t seed,
                                        uint32_t instance_id)
    {
    Philox rng(45, timestep, seed, instance_id);
    const double gauss = normal_d(rng);
    double chi2 = 0.0; // chi-squared with dof - 1 degrees of freedom, as 2 Gamma((dof - 1) / 2)
    if (dof > 1.0)
        chi2 = 2.0 * gamma_d(rng, (dof - 1.0) / 2.0, 1.0);
    return make_double2(gauss, chi2);
    }

// Bussi, Donadio and Parrinello (2007), eq. A7: with c = exp(-dt / tau) (0 for tau = 0) and
// w = kT / (2 K), alpha^2 = c + (1 - c) w (chi2 + g^2) + 2 g sqrt(c (1 - c) w).
__device__ inline double bussi_factor_from_draws(double K, double dof, double dt, double tau,
                                                 double set_T, double2 draws)
    {
    if (dt == 0.0 || dof == 0.0 || K <= 0.0)
        return 1.0;
    const double c = tau != 0.0 ? exp(-dt / tau) : 0.0;
    const double g = draws.x, chi2 = draws.y;
    const double w = set_T / 2.0 / K;
    const double stochastic = w * (1.0 - c) * (chi2 + g * g);
    const double cross = 2.0 * g * sqrt(w * (1.0 - c) * c);
    return sqrt(c + stochastic + cross);
    }

__device__ inline double bussi_factor_d(double K, double dof, double dt, double tau, double set_T,
                                        uint64_t timestep, uint16_t seed, uint32_t instance_id)
    {
    if (dt == 0.0 || dof == 0.0 || K <= 0.0)
        return 1.0;
    return bussi_factor_from_draws(K, dof, dt, tau, set_T,
                                   bussi_draws_d(dof, timestep, seed, instance_id));
    }

// BerendsenThermostat::getRescalingFactorsOne (hoomd/md/Thermostat.h:469-489), translational:
// sqrt(1 + dt / tau (kT / T - 1)) with T = 2 K / dof.
__device__ inline double berendsen_factor_d(double K, double dof, double dt, double tau, double kT)
    {
    const double T_cur = 2.0 * K / dof;
    return sqrt(1.0 + dt / tau * (kT / T_cur - 1.0));
    }

#endif // __CUDACC__

} // namespace gb
