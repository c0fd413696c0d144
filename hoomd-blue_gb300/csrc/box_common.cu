// Host helpers of the C ABI: box construction, cell dimensions, error state, version.
#include <cmath>
#include <mutex>
#include <string>

#include "gb_host.h"

namespace gb
{
static thread_local std::string g_last_error;

void set_error(const std::string& msg)
    {
    g_last_error = msg;
    }

int num_sms()
    {
    static int n = 0;
    if (n == 0)
        {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0)
            n = 152;
        }
    return n;
    }
} // namespace gb

extern "C"
    {
    unsigned int gb_abi_struct_sizes(size_t* out, unsigned int n)
        {
        const size_t sizes[10] = {sizeof(gb_box),           sizeof(gb_cell_list_args),
                                  sizeof(gb_nlist_args),    sizeof(gb_pair_args),
                                  sizeof(gb_radial_param),  sizeof(gb_step_one_args),
                                  sizeof(gb_step_fuse),     sizeof(gb_mlp_force_args),
                                  sizeof(gb_replica),       sizeof(gb_replica_batch)};
        for (unsigned int k = 0; k < n && k < 10 && out; k++)
            out[k] = sizes[k];
        return 10;
        }

    const char* gb_last_error(void)
        {
        return gb::g_last_error.c_str();
        }

    int gb_version(void)
        {
        return 1;
        }

    // BoxDim(Lx,Ly,Lz) / setTiltFactors / setPeriodic at FP32 (hoomd/BoxDim.h:103-180): the
    // lengths are rounded to float first, then hi = L/2, lo = -hi, Linv = 1/L, all in float.
    int gb_box_make(const double L[3], double xy, double xz, double yz, const int periodic[3],
                    gb_box* out)
        {
        GB_REQUIRE(L && out, "gb_box_make: null argument");
        for (int d = 0; d < 3; d++)
            {
            volatile float l = (float)L[d];
            out->L[d] = l;
            out->hi[d] = l / 2.0f;
            out->lo[d] = -out->hi[d];
            out->Linv[d] = 1.0f / l;
            out->periodic[d] = periodic ? (periodic[d] != 0) : 1u;
            }
        if (out->L[2] == 0.0f)
            out->Linv[2] = 0.0f;
        out->xy = (float)xy;
        out->xz = (float)xz;
        out->yz = (float)yz;
        return GB_OK;
        }

    int gb_table_pack(const double* U, const double* F, uint32_t width, float* out)
        {
        GB_REQUIRE(U && F && out, "gb_table_pack: null argument");
        GB_REQUIRE(width > 0, "The length of V and F must not be zero.");
        for (uint32_t k = 0; k < width; k++)
            {
            out[4 * k + 0] = (float)U[k];
            out[4 * k + 1] = (float)F[k];
            out[4 * k + 2] = (k + 1 < width) ? (float)U[k + 1] : 0.0f;
            out[4 * k + 3] = (k + 1 < width) ? (float)F[k + 1] : 0.0f;
            }
        return GB_OK;
        }

    // hoomd/BoxDim.h:552-567 (host rsqrt = 1/sqrt) and hoomd/CellList.cc:83-131.
    int gb_cell_dims(const gb_box* box, unsigned int ndim, float nominal_width,
                     unsigned int dim[3])
        {
        GB_REQUIRE(box && dim, "gb_cell_dims: null argument");
        GB_REQUIRE(nominal_width > 0.0f, "Cell: cell width must be non-zero");
        volatile float a = box->xy * box->yz;
        volatile float b = a - box->xz;
        volatile float c = box->xy * box->xy;
        volatile float d1 = 1.0f + c;
        volatile float bb = b * b;
        volatile float d2 = d1 + bb;
        volatile float npx = box->L[0] * (1.0f / std::sqrt((float)d2));
        volatile float yzz = box->yz * box->yz;
        volatile float e1 = 1.0f + yzz;
        volatile float npy = box->L[1] * (1.0f / std::sqrt((float)e1));
        float npz = (box->L[2] == 0.0f) ? 1.0f : box->L[2];
        float np[3] = {npx, npy, npz};
        for (int k = 0; k < 3; k++)
            {
            volatile float q = np[k] / nominal_width;
            dim[k] = (unsigned int)q;
            }
        if (ndim == 2)
            dim[2] = 1;
        for (int k = 0; k < 3; k++)
            if (dim[k] == 0)
                dim[k] = 1;
        return GB_OK;
        }
    }
