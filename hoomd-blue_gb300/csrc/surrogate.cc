// Host side of the radial MLP surrogate (see surrogate.h).
#include "surrogate.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace gbe
{

static uint64_t splitmix(uint64_t& s)
    {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
    }

MlpSurrogate::MlpSurrogate(unsigned int ntypes_, double r_min_, double r_cut_, uint64_t seed_)
    : ntypes(ntypes_), r_min((float)r_min_), r_cut((float)r_cut_), seed(seed_), rng_state(seed_)
    {
    if (ntypes_ == 0)
        throw std::invalid_argument("the surrogate needs at least one particle type");
    if (!(r_cut_ > r_min_) || r_min_ < 0.0)
        throw std::invalid_argument("need 0 <= r_min < r_cut");
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
    const size_t n = gb_mlp_param_count(n_pairs());
    d_theta.resize(n);
    d_grad.resize(n);
    d_m.resize(n);
    d_v.resize(n);
    d_m.zero(stream);
    d_v.zero(stream);
    d_loss.resize(1);
    d_infer.resize(gb_mlp_infer_bytes(n_pairs()));
    // seeded initialisation: fan-in scaled uniform weights, N(0, 1) embeddings, zero biases
    std::vector<float> th(n, 0.0f);
    uint64_t s = seed_ * 0x9E3779B97F4A7C15ull + 12345;
    auto uni = [&]() { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); };
    auto fill = [&](size_t off, size_t cnt, double scale) {
        for (size_t k = 0; k < cnt; k++)
            th[off + k] = (float)((2.0 * uni() - 1.0) * scale);
    };
    fill(0, 1024, 1.0 / std::sqrt(48.0));
    fill(1024, 2048, 2.0 / std::sqrt(48.0));
    fill(3136, 4096, 2.0 / std::sqrt(64.0));
    fill(7296, 64, 1.0 / std::sqrt(64.0));
    for (size_t k = 7424; k < n; k += 2)
        {
        const double u1 = std::max(uni(), 1e-300), u2 = uni();
        const double rad = std::sqrt(-2.0 * std::log(u1));
        th[k] = (float)(rad * std::cos(6.283185307179586 * u2));
        if (k + 1 < n)
            th[k + 1] = (float)(rad * std::sin(6.283185307179586 * u2));
        }
    set_params(th);
    }

MlpSurrogate::~MlpSurrogate()
    {
    if (stream)
        {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
        }
    }

void MlpSurrogate::set_params(const std::vector<float>& th)
    {
    if (th.size() != d_theta.size())
        throw std::invalid_argument("parameter vector has the wrong length");
    d_theta.upload(th.data(), th.size(), stream);
    d_m.zero(stream);
    d_v.zero(stream);
    adam_step = 0;
    prepared = false;
    cuda_check(cudaStreamSynchronize(stream), "set params");
    }

std::vector<float> MlpSurrogate::params()
    {
    std::vector<float> th(d_theta.size());
    d_theta.download(th.data(), th.size(), stream);
    cuda_check(cudaStreamSynchronize(stream), "params");
    return th;
    }

void MlpSurrogate::set_samples(const std::vector<uint32_t>& pair, const std::vector<float>& r,
                               const std::vector<float>& U, const std::vector<float>& F)
    {
    const size_t n = pair.size();
    if (r.size() != n || U.size() != n || F.size() != n || n == 0)
        throw std::invalid_argument("sample arrays must be non-empty and of equal length");
    for (uint32_t p : pair)
        if (p >= n_pairs())
            throw std::invalid_argument("sample pair index out of range");
    h_pair = pair;
    h_r = r;
    h_U = U;
    h_F = F;
    n_samples = n;
    d_pair.resize(n);
    d_r.resize(n);
    d_U.resize(n);
    d_F.resize(n);
    shuffle();
    }

// Fisher-Yates over the host copy, then upload (one pass of minibatches per shuffle).
void MlpSurrogate::shuffle()
    {
    for (size_t k = n_samples; k > 1; k--)
        {
        const size_t j = (size_t)(splitmix(rng_state) % k);
        std::swap(h_pair[k - 1], h_pair[j]);
        std::swap(h_r[k - 1], h_r[j]);
        std::swap(h_U[k - 1], h_U[j]);
        std::swap(h_F[k - 1], h_F[j]);
        }
    d_pair.upload(h_pair.data(), n_samples, stream);
    d_r.upload(h_r.data(), n_samples, stream);
    d_U.upload(h_U.data(), n_samples, stream);
    d_F.upload(h_F.data(), n_samples, stream);
    }

std::vector<double> MlpSurrogate::train(uint32_t steps, uint32_t batch, double lr0,
                                        double lr_min, double lam, int quant, uint32_t report)
    {
    if (n_samples == 0)
        throw std::runtime_error("no training samples");
    batch = (uint32_t)std::min<size_t>(batch, n_samples);
    d_scratch.resize(gb_mlp_train_scratch_bytes(batch));
    std::vector<double> out;
    size_t cursor = 0;
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    cuda_check(cudaEventRecord(e0, stream), "event");
    for (uint32_t k = 0; k < steps; k++)
        {
        if (cursor + batch > n_samples)
            {
            shuffle();
            cursor = 0;
            }
        const double lr = lr_min + 0.5 * (lr0 - lr_min) * (1.0 + std::cos(3.141592653589793 * k / steps));
        check(gb_mlp_loss_grad(d_theta.get(), n_pairs(), r_min, r_cut, d_pair.get() + cursor,
                               d_r.get() + cursor, d_U.get() + cursor, d_F.get() + cursor, batch,
                               (float)lam, quant, d_grad.get(), d_loss.get(), d_scratch.get(),
                               stream),
              "gb_mlp_loss_grad");
        check(gb_mlp_adam(d_theta.get(), d_grad.get(), d_m.get(), d_v.get(), d_theta.size(),
                          (float)lr, 0.9f, 0.999f, 1e-8f, ++adam_step, stream),
              "gb_mlp_adam");
        cursor += batch;
        if (report && (k + 1) % report == 0)
            {
            double l = 0.0;
            d_loss.download(&l, 1, stream);
            cuda_check(cudaStreamSynchronize(stream), "loss");
            out.push_back(l);
            }
        }
    cuda_check(cudaEventRecord(e1, stream), "event");
    cuda_check(cudaEventSynchronize(e1), "event");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    train_ms += ms;
    train_steps += steps;
    prepared = false;
    return out;
    }

double MlpSurrogate::loss(uint32_t batch, double lam, int quant)
    {
    batch = (uint32_t)std::min<size_t>(batch, n_samples);
    d_scratch.resize(gb_mlp_train_scratch_bytes(batch));
    check(gb_mlp_loss_grad(d_theta.get(), n_pairs(), r_min, r_cut, d_pair.get(), d_r.get(),
                           d_U.get(), d_F.get(), batch, (float)lam, quant, d_grad.get(),
                           d_loss.get(), d_scratch.get(), stream),
          "gb_mlp_loss_grad");
    double l = 0.0;
    d_loss.download(&l, 1, stream);
    cuda_check(cudaStreamSynchronize(stream), "loss");
    return l;
    }

const void* MlpSurrogate::infer_block()
    {
    if (!prepared)
        {
        check(gb_mlp_prepare(d_theta.get(), n_pairs(), d_infer.get(), stream), "gb_mlp_prepare");
        cuda_check(cudaStreamSynchronize(stream), "prepare");
        prepared = true;
        }
    return d_infer.get();
    }

void MlpSurrogate::eval(const std::vector<uint32_t>& pair, const std::vector<float>& r,
                        std::vector<float>& U, std::vector<float>& dU)
    {
    const size_t n = pair.size();
    if (r.size() != n)
        throw std::invalid_argument("pair and r must have equal length");
    const void* inf = infer_block();
    DeviceArray<uint32_t> dp;
    DeviceArray<float> dr, dUo, ddU;
    dp.resize(std::max<size_t>(n, 1));
    dr.resize(std::max<size_t>(n, 1));
    dUo.resize(std::max<size_t>(n, 1));
    ddU.resize(std::max<size_t>(n, 1));
    dp.upload(pair.data(), n, stream);
    dr.upload(r.data(), n, stream);
    check(gb_mlp_eval(inf, n_pairs(), r_min, r_cut, act_split, dp.get(), dr.get(), (uint32_t)n,
                      dUo.get(), ddU.get(), stream),
          "gb_mlp_eval");
    U.resize(n);
    dU.resize(n);
    dUo.download(U.data(), n, stream);
    ddU.download(dU.data(), n, stream);
    cuda_check(cudaStreamSynchronize(stream), "eval");
    }

} // namespace gbe
