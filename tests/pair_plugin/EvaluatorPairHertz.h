// A pair evaluator written to the reference's plugin concept
// (example_plugins/pair_plugin/EvaluatorPairExample.h): Hertzian soft-sphere contact,
// V(r) = epsilon (1 - r/sigma)^(5/2) for r < sigma. Test fixture for the plugin path: it is built
// as a plugin module and checked against the closed form on the GPU.

#ifndef __PAIR_EVALUATOR_HERTZ_H__
#define __PAIR_EVALUATOR_HERTZ_H__

#ifndef __HIPCC__
#include <string>
#endif

#include "hoomd/HOOMDMath.h"

#ifdef __HIPCC__
#define DEVICE __device__
#define HOSTDEVICE __host__ __device__
#else
#define DEVICE
#define HOSTDEVICE
#endif

namespace hoomd
    {
namespace md
    {

class EvaluatorPairHertz
    {
    public:
    struct param_type
        {
        Scalar epsilon; //!< contact energy scale
        Scalar sigma;   //!< contact diameter

        DEVICE void load_shared(char*& ptr, unsigned int& available_bytes) { }

        HOSTDEVICE void allocate_shared(char*& ptr, unsigned int& available_bytes) const { }

#ifdef ENABLE_HIP
        void set_memory_hint() const { }
#endif

#ifndef __HIPCC__
        param_type() : epsilon(0), sigma(1) { }

        param_type(pybind11::dict v, bool managed = false)
            {
            epsilon = v["epsilon"].cast<Scalar>();
            sigma = v["sigma"].cast<Scalar>();
            }

        pybind11::dict asDict()
            {
            pybind11::dict v;
            v["epsilon"] = epsilon;
            v["sigma"] = sigma;
            return v;
            }
#endif
        }
#if HOOMD_LONGREAL_SIZE == 32
        __attribute__((aligned(8)));
#else
        __attribute__((aligned(16)));
#endif

    DEVICE EvaluatorPairHertz(Scalar _rsq, Scalar _rcutsq, const param_type& _params)
        : rsq(_rsq), rcutsq(_rcutsq), epsilon(_params.epsilon), sigma(_params.sigma)
        {
        }

    DEVICE static bool needsCharge()
        {
        return false;
        }

    DEVICE void setCharge(Scalar qi, Scalar qj) { }

    //! force_divr = -(1/r) dV/dr = (5/2) (epsilon / sigma) (1 - r/sigma)^(3/2) / r
    DEVICE bool evalForceAndEnergy(Scalar& force_divr, Scalar& pair_eng, bool energy_shift)
        {
        if (rsq < rcutsq)
            {
            const Scalar r = fast::sqrt(rsq);
            const Scalar gap = Scalar(1.0) - r / sigma;
            if (gap <= Scalar(0.0))
                {
                force_divr = Scalar(0.0);
                pair_eng = Scalar(0.0);
                return true;
                }
            const Scalar root = fast::sqrt(gap);
            force_divr = Scalar(2.5) * epsilon / sigma * gap * root / r;
            pair_eng = epsilon * gap * gap * root;
            if (energy_shift)
                {
                const Scalar gap_c = Scalar(1.0) - fast::sqrt(rcutsq) / sigma;
                if (gap_c > Scalar(0.0))
                    pair_eng -= epsilon * gap_c * gap_c * fast::sqrt(gap_c);
                }
            return true;
            }
        return false;
        }

    DEVICE Scalar evalPressureLRCIntegral()
        {
        return 0;
        }

    DEVICE Scalar evalEnergyLRCIntegral()
        {
        return 0;
        }

#ifndef __HIPCC__
    static std::string getName()
        {
        return std::string("hertz");
        }

    std::string getShapeSpec() const
        {
        throw std::runtime_error("Shape definition not supported for this pair potential.");
        }
#endif

    protected:
    Scalar rsq;
    Scalar rcutsq;
    Scalar epsilon;
    Scalar sigma;
    };

    } // end namespace md
    } // end namespace hoomd

#endif // __PAIR_EVALUATOR_HERTZ_H__
