// Test infrastructure only (never shipped, never on the product path).
//
// Thin C wrapper around the reference's own header-only maths, compiled in place from the
// reference source tree by oracle/build.py into oracle/_ref/. It lets the CPU tests pin the
// oracle's restatement (oracle/md_oracle.cc) against the reference's unmodified code:
//   hoomd/BoxDim.h                       (minImage, wrap, makeFraction, getNearestPlaneDistance)
//   hoomd/md/EvaluatorPairLJ.h           (evalForceAndEnergy, LRC integrals)
//   hoomd/md/EvaluatorPairTable.h        (evalForceAndEnergy)
//   example_plugins/pair_plugin/EvaluatorPairExample.h
// Build once per precision: -DHOOMD_LONGREAL_SIZE=64 (reference default Scalar=double) and =32.

#include "hoomd/HOOMDMath.h"
#include "hoomd/BoxDim.h"
#include "hoomd/md/EvaluatorPairLJ.h"
#include "hoomd/md/EvaluatorPairTable.h"
#include "example_plugins/pair_plugin/EvaluatorPairExample.h"

using namespace hoomd;
using namespace hoomd::md;

static BoxDim make_box(const double* b6, const int* periodic)
    {
    const Scalar lx = Scalar(b6[0]), ly = Scalar(b6[1]), lz = Scalar(b6[2]);
    BoxDim box(lx, ly, lz);
    box.setTiltFactors(Scalar(b6[3]), Scalar(b6[4]), Scalar(b6[5]));
    box.setPeriodic(make_uchar3(periodic[0] != 0, periodic[1] != 0, periodic[2] != 0));
    return box;
    }

extern "C"
    {
    int ref_scalar_size()
        {
        return (int)sizeof(Scalar);
        }

    void ref_lj_eval(int n,
                     const double* rsq,
                     double rcutsq,
                     double sigma,
                     double epsilon,
                     int energy_shift,
                     double* force_divr,
                     double* pair_eng,
                     int* evaluated)
        {
        const Scalar s_sigma = Scalar(sigma), s_eps = Scalar(epsilon);
        EvaluatorPairLJ::param_type p(s_sigma, s_eps);
        for (int i = 0; i < n; i++)
            {
            EvaluatorPairLJ ev(Scalar(rsq[i]), Scalar(rcutsq), p);
            Scalar f = 0, e = 0;
            evaluated[i] = ev.evalForceAndEnergy(f, e, energy_shift != 0);
            force_divr[i] = f;
            pair_eng[i] = e;
            }
        }

    void ref_lj_lrc(double rcutsq, double sigma, double epsilon, double* out2)
        {
        const Scalar s_sigma = Scalar(sigma), s_eps = Scalar(epsilon);
        EvaluatorPairLJ::param_type p(s_sigma, s_eps);
        EvaluatorPairLJ ev(Scalar(0), Scalar(rcutsq), p);
        out2[0] = ev.evalEnergyLRCIntegral();
        out2[1] = ev.evalPressureLRCIntegral();
        }

    void ref_table_eval(int n,
                        const double* rsq,
                        double rcutsq,
                        double rmin,
                        int width,
                        const double* V,
                        const double* F,
                        double* force_divr,
                        double* pair_eng,
                        int* evaluated)
        {
        EvaluatorPairTable::param_type p;
        p.rmin = Scalar(rmin);
        p.V_table = ManagedArray<Scalar>(static_cast<unsigned int>(width), false);
        p.F_table = ManagedArray<Scalar>(static_cast<unsigned int>(width), false);
        for (int k = 0; k < width; k++)
            {
            p.V_table.get()[k] = Scalar(V[k]);
            p.F_table.get()[k] = Scalar(F[k]);
            }
        for (int i = 0; i < n; i++)
            {
            EvaluatorPairTable ev(Scalar(rsq[i]), Scalar(rcutsq), p);
            Scalar f = 0, e = 0;
            evaluated[i] = ev.evalForceAndEnergy(f, e, false);
            force_divr[i] = f;
            pair_eng[i] = e;
            }
        }

    void ref_example_eval(int n,
                          const double* rsq,
                          double rcutsq,
                          double k,
                          double sigma,
                          int energy_shift,
                          double* force_divr,
                          double* pair_eng,
                          int* evaluated)
        {
        EvaluatorPairExample::param_type p;
        p.k = Scalar(k);
        p.sigma = Scalar(sigma);
        for (int i = 0; i < n; i++)
            {
            EvaluatorPairExample ev(Scalar(rsq[i]), Scalar(rcutsq), p);
            Scalar f = 0, e = 0;
            evaluated[i] = ev.evalForceAndEnergy(f, e, energy_shift != 0);
            force_divr[i] = f;
            pair_eng[i] = e;
            }
        }

    // Host-side (branching) minimum image of n vectors, in place, as BoxDim::minImage.
    void ref_min_image(int n, const double* box6, const int* periodic, double* v3)
        {
        BoxDim box = make_box(box6, periodic);
        for (int i = 0; i < n; i++)
            {
            Scalar3 w = make_scalar3(Scalar(v3[3 * i]), Scalar(v3[3 * i + 1]), Scalar(v3[3 * i + 2]));
            w = box.minImage(w);
            v3[3 * i] = w.x;
            v3[3 * i + 1] = w.y;
            v3[3 * i + 2] = w.z;
            }
        }

    void ref_wrap(int n, const double* box6, const int* periodic, double* v3, int* img3)
        {
        BoxDim box = make_box(box6, periodic);
        for (int i = 0; i < n; i++)
            {
            Scalar3 w = make_scalar3(Scalar(v3[3 * i]), Scalar(v3[3 * i + 1]), Scalar(v3[3 * i + 2]));
            int3 img = make_int3(img3[3 * i], img3[3 * i + 1], img3[3 * i + 2]);
            box.wrap(w, img);
            v3[3 * i] = w.x;
            v3[3 * i + 1] = w.y;
            v3[3 * i + 2] = w.z;
            img3[3 * i] = img.x;
            img3[3 * i + 1] = img.y;
            img3[3 * i + 2] = img.z;
            }
        }

    void ref_make_fraction(int n, const double* box6, const int* periodic, double* v3)
        {
        BoxDim box = make_box(box6, periodic);
        for (int i = 0; i < n; i++)
            {
            Scalar3 w = make_scalar3(Scalar(v3[3 * i]), Scalar(v3[3 * i + 1]), Scalar(v3[3 * i + 2]));
            Scalar3 f = box.makeFraction(w);
            v3[3 * i] = f.x;
            v3[3 * i + 1] = f.y;
            v3[3 * i + 2] = f.z;
            }
        }

    void ref_nearest_plane_distance(const double* box6, const int* periodic, double* out3)
        {
        BoxDim box = make_box(box6, periodic);
        Scalar3 d = box.getNearestPlaneDistance();
        out3[0] = d.x;
        out3[1] = d.y;
        out3[2] = d.z;
        }
    }
