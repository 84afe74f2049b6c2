// Radiance-cache MLP on the 5th-generation tensor cores (host interface of mlp.cu).
//
// Network: 96 input features (85 used: 12-frequency sin/cos encoding of the position, direction,
// normal, roughness, diffuse and specular albedo; feature 85 is a constant 1) -> 5 hidden layers
// of 64 with ReLU -> 3 outputs with exp, no bias terms.  BF16 weights and activations, FP32
// accumulation, FP32 master weights and Adam state.  Parameters are the row-major [out][in]
// matrices W0 (64x96), W1..W4 (64x64), W5 (16x64, rows 3..15 stay zero), concatenated.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace lts {

constexpr int kMlpIn = 96, kMlpHidden = 64, kMlpOutPad = 16, kMlpOut = 3, kMlpLayers = 6;
constexpr int kMlpParams = 64 * 96 + 4 * 64 * 64 + 16 * 64;  // 23,552
// layer L: input width, (padded) output width, offset of W_L in the parameter vector
__host__ __device__ constexpr int mlp_in(int L) { return L == 0 ? 96 : 64; }
__host__ __device__ constexpr int mlp_out(int L) { return L == 5 ? 16 : 64; }
__host__ __device__ constexpr int mlp_offset(int L) { return L == 0 ? 0 : 6144 + 4096 * (L - 1); }

// Tensor-core product check: D = op(A) op(B) for the three operand arrangements the MLP uses
// (mode 0: K-major x K-major, 128x64 . (64x64)^T; mode 1: K-major x MN-major, 128x64 . 64x96;
// mode 2: MN-major x MN-major, (128x96)^T . 128x64 with M padded to 128).  Host buffers of bf16
// bits; D is 128 x 64 or 128 x 96 FP32.  swap exchanges the two byte offsets of MN-major
// descriptors (a layout check).
std::string umma_probe(int mode, int swap, const uint16_t* a, const uint16_t* b, float* d, uint32_t* d_err,
                       cudaStream_t s);

class Mlp {
   public:
    Mlp() = default;
    ~Mlp();
    Mlp(const Mlp&) = delete;
    Mlp& operator=(const Mlp&) = delete;

    // Allocates the parameters and Adam state and draws He-uniform weights from `seed`.
    std::string init(uint32_t seed, cudaStream_t s);
    std::string set_params(const float* host, cudaStream_t s);  // kMlpParams FP32 values
    std::string get_params(float* host, cudaStream_t s);

    // Inference (forward) uses an exponential moving average of the weights with this decay per
    // Adam step, training the weights themselves; 0: inference uses the weights.  The average
    // restarts from the weights at init / set_params.
    float ema = 0.0f;
    // out[r * out_stride + c] = network(features[r][96])_c for r = rows[i] (rows null: r = i),
    // i < n (device pointers; features are bf16 bits).
    // d_n (device, may be null): the row count to use, at most n (the grid is sized for n).
    std::string forward(const uint16_t* d_feat, int n, float* d_out, uint32_t* d_err, cudaStream_t s,
                        const int32_t* d_rows = nullptr, int out_stride = 3, const uint32_t* d_n = nullptr);
    // Gradient of the relative L2 loss mean((pred - t)^2 / (pred^2 + 0.01)) over the n samples
    // into the gradient buffer (zeroed first), the loss into *d_loss (device), then, if lr > 0,
    // one Adam step (beta 0.9 / 0.99, eps 1e-8) that also zeroes the gradient.
    std::string train_step(const uint16_t* d_feat, const float* d_target, int n, float lr, float* d_loss,
                           uint32_t* d_err, cudaStream_t s);
    std::string get_grad(float* host, cudaStream_t s);
    // One Adam step with the gradient buffer (zeroes it).
    std::string adam(float lr, cudaStream_t s);

    bool ready() const { return w32_ != nullptr; }
    float* scratch_loss() const { return loss_; }  // one device float for callers that drop the loss
    int steps = 0;

   private:
    float *w32_ = nullptr, *grad_ = nullptr, *m_ = nullptr, *v_ = nullptr, *loss_ = nullptr;
    uint16_t* w16_ = nullptr;
    float* e32_ = nullptr;  // weight average (inference), FP32 and BF16
    uint16_t* e16_ = nullptr;
    int blocks_train_ = 0, blocks_fwd_ = 0;
    std::string sync_bf16(cudaStream_t s);
};

// Bounded mbarrier waits of the tensor-core kernels: set the poll limit (<= 0: the default
// kSpinLimit); run one wait on an mbarrier phase that nothing completes, so that it runs out and
// sets DEV_ERR_MMA_TIMEOUT in *d_err (synchronises the stream).
std::string mlp_set_spin_limit(int limit);
std::string mlp_debug_mbar_timeout(uint32_t* d_err, cudaStream_t s);

}  // namespace lts
