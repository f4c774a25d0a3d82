// sph_mlp.cuh — the learned acceleration correction: a 32 -> 128 -> 128 -> 3
// MLP with GELU, BF16 weights and FP32 accumulation.
//
// Forward and backward run on the 5th-generation tensor cores: tcgen05.mma
// (kind::f16, BF16 operands from shared memory, FP32 accumulators in tensor
// memory), 128 particles per MMA tile; the elementwise parts and Adam run on
// the CUDA cores in FP32.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sph {
namespace mlp {

constexpr int kIn = 32;
constexpr int kHidden = 128;
constexpr int kOut = 3;
constexpr int kOutPad = 16;  // N of the last MMA (a multiple of 16 for M = 128)
constexpr int kTile = 128;   // particles per MMA tile (M)

// The forward pass's input tile: 128 rows of 32 normalised BF16 features in
// the tcgen05 no-swizzle K-major layout (8-row x 16-byte core matrices);
// x_tile_offset gives the byte offset of (row, 8-feature chunk) in a tile.
// Tiles of consecutive rows follow one another, kXTileBytes apart.
constexpr uint32_t kXTileBytes = kTile * kIn * 2;
__host__ __device__ constexpr uint32_t x_tile_offset(uint32_t row, uint32_t chunk) {
    return (row >> 3) * (kIn / 8u) * 128u + chunk * 128u + (row & 7u) * 16u;
}

// Offsets of the FP32 parameter vector (the layout the C ABI exposes):
// W1[128][32], b1[128], W2[128][128], b2[128], W3[3][128], b3[3].
constexpr int kW1 = 0;
constexpr int kB1 = kW1 + kHidden * kIn;
constexpr int kW2 = kB1 + kHidden;
constexpr int kB2 = kW2 + kHidden * kHidden;
constexpr int kW3 = kB2 + kHidden;
constexpr int kB3 = kW3 + kOut * kHidden;
constexpr int kParams = kB3 + kOut;

// Device view of a model for the forward kernel.
struct ModelView {
    const __nv_bfloat16* w1;  // [128][32]   row = output neuron, K contiguous
    const __nv_bfloat16* w2;  // [128][128]
    const __nv_bfloat16* w3;  // [16][128]   rows 3..15 zero
    const float* params;      // FP32 vector (biases read from here)
    const float* in_mean;     // [32] feature normalisation
    const float* in_inv_std;  // [32]
    const float* out_scale;   // [3]  output = network * scale
    uint32_t free_axes;       // bit a: each tank's mean correction along axis a is removed
};

// Activations kept for backward (may be null for inference).
struct ForwardSaves {
    float* z1;            // [n][128] pre-activation of layer 1
    float* z2;            // [n][128]
    __nv_bfloat16* x;     // [n][32]  normalised input as the MMA saw it
    __nv_bfloat16* h1;    // [n][128] GELU(z1) as BF16
    __nv_bfloat16* h2;    // [n][128]
    float* y;             // [n][4]   network output before scaling
};

// Tries of a bounded mbarrier wait before the forward pass gives up on its
// MMAs (sets *error_flag, drains, frees its tensor memory and returns).
constexpr uint32_t kWaitPolls = 1u << 22;

cudaError_t launch_forward(const ModelView& model, const float* features, uint32_t n, float* out_accel,
                           const ForwardSaves* saves, unsigned int* error_flag, cudaStream_t stream);
// Forward over ready input tiles (x_tiles: ceil(n / 128) tiles, as written by
// the learned step's features kernel); output as launch_forward, bit for bit.
// Warp-specialised: one persistent CTA per SM, two tiles in flight (TMEM
// columns, buffers and mbarriers per tile slot). programmatic: launched as a
// programmatic dependent of the kernel that writes the tiles, each CTA
// staging the weights and taking its tensor memory while that kernel ends.
cudaError_t launch_forward_tiles(const ModelView& model, const uint8_t* x_tiles, uint32_t n, float* out_accel,
                                 unsigned int* error_flag, cudaStream_t stream,
                                 bool programmatic = false);
// One CTA waits on an mbarrier (arrived at only when `arrive`) with at most
// `polls` tries; sets *error_flag when the wait gives up.
void launch_wait_selftest(uint32_t polls, int arrive, unsigned int* error_flag, cudaStream_t stream);

// Backward of the mean squared error on normalised targets on the tensor
// cores: dH1 = dZ2 W2 and the weight and bias gradients as tcgen05 products
// with FP32 accumulation (dY for W3, dZ2 and dZ1 rounded to BF16 on the way
// in), the elementwise parts in FP32. d_params receives the gradient of the
// FP32 parameter vector and loss (device, one float) the mean squared error;
// scratch holds backward_scratch_floats(n) floats. A tensor-core wait that
// gives up sets *error_flag.
size_t backward_scratch_floats(uint32_t n);
cudaError_t launch_backward(const ModelView& model, const ForwardSaves& saves, const float* targets, uint32_t n,
                            float* d_params, float* loss, float* scratch, unsigned int* error_flag,
                            cudaStream_t stream);

// Adam (src/gfx/neural_math.cpp:1177-1208) on the FP32 vector, then the
// BF16 weight copies are refreshed from it.
cudaError_t launch_adam(float* params, const float* grads, float* moments, uint32_t step, float lr, float beta1,
                        float beta2, float epsilon, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w3,
                        cudaStream_t stream);
// Refreshes the BF16 copies from the FP32 vector (round to nearest even).
cudaError_t launch_quantise(const float* params, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w3,
                            cudaStream_t stream);

// Sets the forward kernel's shared-memory limit; call once per device before
// any stream capture that contains a forward launch.
cudaError_t prepare_forward();
// max |erf of the forward pass - erff| over [-6, 6] as float bits in *out (pre-zeroed).
void launch_erf_selftest(uint32_t count, unsigned int* out, cudaStream_t stream);

}  // namespace mlp
}  // namespace sph

struct sph_mlp;
// The device view of a model (C++ only; the C ABI hands models around as
// opaque sph_mlp pointers).
bool sph_mlp_model_view(const sph_mlp* mlp, sph::mlp::ModelView* out);
