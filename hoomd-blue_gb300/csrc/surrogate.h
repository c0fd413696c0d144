// Host side of the radial MLP surrogate of the Table potential: parameters, training on pair
// samples with the project's own kernels (gb_mlp_loss_grad + gb_mlp_adam), and the prepared
// inference block that PotentialPairGPU uses (gb_mlp_forces).
#pragma once

#include <cstdint>
#include <vector>

#include "engine.h"

namespace gbe
{

class MlpSurrogate
    {
    public:
    MlpSurrogate(unsigned int ntypes, double r_min, double r_cut, uint64_t seed);
    ~MlpSurrogate();
    MlpSurrogate(const MlpSurrogate&) = delete;
    MlpSurrogate& operator=(const MlpSurrogate&) = delete;

    unsigned int n_pairs() const
        {
        return ntypes * (ntypes + 1) / 2;
        }
    void set_params(const std::vector<float>& theta);
    std::vector<float> params();

    // training samples: type-pair index, r, target U and F = -dU/dr
    void set_samples(const std::vector<uint32_t>& pair, const std::vector<float>& r,
                     const std::vector<float>& U, const std::vector<float>& F);
    // Adam with a cosine learning-rate schedule from lr0 to lr_min over `steps`; minibatches are
    // consecutive slices of the samples, reshuffled every pass. Returns the loss every
    // `report` steps.
    std::vector<double> train(uint32_t steps, uint32_t batch, double lr0, double lr_min,
                              double lam, int quant, uint32_t report);
    double loss(uint32_t batch, double lam, int quant); // mean loss over the first batch
    // tensor-core evaluation of (U, dU/dr) for samples (tests, accuracy reports)
    void eval(const std::vector<uint32_t>& pair, const std::vector<float>& r,
              std::vector<float>& U, std::vector<float>& dU);

    const void* infer_block(); // prepared on demand after parameter changes
    unsigned int ntypes;
    float r_min, r_cut;
    int act_split = 1;
    int mma_sync = 0; // 0: tcgen05 tiles of 128 pairs, 1: mma.sync tiles of 16 pairs
    uint64_t train_steps = 0;
    double train_ms = 0.0;
    cudaStream_t stream = nullptr;

    private:
    void shuffle();

    uint64_t seed, rng_state;
    bool prepared = false;
    uint32_t adam_step = 0;
    size_t n_samples = 0;
    DeviceArray<float> d_theta, d_grad, d_m, d_v;
    DeviceArray<char> d_infer, d_scratch;
    DeviceArray<double> d_loss;
    DeviceArray<uint32_t> d_pair;
    DeviceArray<float> d_r, d_U, d_F;
    std::vector<uint32_t> h_pair;
    std::vector<float> h_r, h_U, h_F;
    };

} // namespace gbe
