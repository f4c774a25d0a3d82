// sph_mlp.cu — the learned correction's MLP: tcgen05 forward, FP32 backward,
// Adam, and its C ABI (sph_mlp_* in include/sph_c.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/sph_c.h"
#include "sph_f32x2.cuh"
#include "sph_mlp.cuh"

namespace sph {
namespace mlp {

namespace {

// ---- tcgen05 / mbarrier helpers (inline PTX, sm_100-family) -----------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: no swizzle, K-major canonical layout of
// 8-row x 16-byte core matrices. lbo: byte stride between core matrices along
// K; sbo: byte stride between 8-row groups along M/N. Bits 46-47 hold the
// descriptor version (1 on sm_100-family tensor cores).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}

// Instruction descriptor of kind::f16: D = F32, A = B = BF16, both K-major,
// dense, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait: gives up after `polls` tries (each try_wait may itself
// suspend the thread for a short, hardware-chosen time) instead of hanging.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t polls) {
    for (uint32_t i = 0; i < polls; ++i) {
        if (mbar_try_wait(mbar, parity)) {
            return true;
        }
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global into shared memory, completing on `mbar` as transaction bytes.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(mbar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        v[k] = __uint_as_float(r[k]);
    }
}

// GELU(z) = z Phi(z) = 0.5 z (1 + erf(z / sqrt(2))) (Hendrycks & Gimpel 2016),
// with erf(z / sqrt(2)) taken as tanh(a z + b z^3), a = sqrt(2 / pi),
// b = 0.044715 a: the approximation that gives the paper its tanh form. Over
// [-6, 6] it is within 3.6e-4 of the exact erf (4.7e-4 in GELU), below the
// BF16 rounding (relative step 2^-8) that the activations get next.
constexpr float kGeluA = 0.7978845608028654f;   // sqrt(2 / pi)
constexpr float kGeluB = 0.0356774081363001f;   // 0.044715 sqrt(2 / pi)

// Derivative of that GELU (backward, FP32 with the accurate tanhf):
// 0.5 (1 + t) + 0.5 z (1 - t^2) (a + 3 b z^2), t = tanh(a z + b z^3).
__device__ __forceinline__ float gelu_grad(float z) {
    const float z2 = z * z;
    const float t = tanhf(z * fmaf(kGeluB, z2, kGeluA));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * fmaf(3.0f * kGeluB, z2, kGeluA);
}

// Byte offset of (row, 8-element chunk) in a K-major no-swizzle tile whose
// rows hold `k` BF16 elements.
__device__ __forceinline__ uint32_t tile_offset(uint32_t row, uint32_t chunk, uint32_t k) {
    return (row >> 3) * (k / 8u) * 128u + chunk * 128u + (row & 7u) * 16u;
}

constexpr uint32_t kSmemW1 = 0;
constexpr uint32_t kSmemW2 = kSmemW1 + kHidden * kIn * 2;        // 8 KB
constexpr uint32_t kSmemW3 = kSmemW2 + kHidden * kHidden * 2;    // +32 KB
constexpr uint32_t kSmemX = kSmemW3 + kOutPad * kHidden * 2;     // +4 KB
constexpr uint32_t kSmemH = kSmemX + kTile * kIn * 2;            // +8 KB
constexpr uint32_t kSmemBar = kSmemH + kTile * kHidden * 2;      // +32 KB
// Small FP32 vectors, staged once per CTA: b1, b2, input mean, input 1/std,
// b3 and the output scale (each padded to whole float4s).
constexpr uint32_t kVecB1 = 0;
constexpr uint32_t kVecB2 = kVecB1 + kHidden;
constexpr uint32_t kVecMean = kVecB2 + kHidden;
constexpr uint32_t kVecInvStd = kVecMean + kIn;
constexpr uint32_t kVecB3 = kVecInvStd + kIn;
constexpr uint32_t kVecScale = kVecB3 + 4;
constexpr uint32_t kVecFloats = kVecScale + 4;
constexpr uint32_t kSmemVec = kSmemBar + 64;
constexpr uint32_t kSmemBytes = kSmemVec + kVecFloats * 4;
static_assert(kXTileBytes == kTile * kIn * 2, "one input tile");
constexpr uint32_t kTmemCols = 128;

__device__ __forceinline__ void store_chunk(uint8_t* base, uint32_t offset, const float* v8) {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v8[0], v8[1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v8[2], v8[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v8[4], v8[5]);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(v8[6], v8[7]);
    uint4 q;
    q.x = *reinterpret_cast<uint32_t*>(&p0);
    q.y = *reinterpret_cast<uint32_t*>(&p1);
    q.z = *reinterpret_cast<uint32_t*>(&p2);
    q.w = *reinterpret_cast<uint32_t*>(&p3);
    *reinterpret_cast<uint4*>(base + offset) = q;
}

// The forward pass's tanh: the hardware's approximate tanh (one
// special-function op; maximum relative error about 2^-11).
__device__ __forceinline__ float tanh_approx(float x) {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// erf(x) as the forward pass evaluates it: tanh(a u + b u^3), u = sqrt(2) x.
__device__ __forceinline__ float erf_forward(float x) {
    const float u = x * 1.4142135623730951f;
    return tanh_approx(u * fmaf(kGeluB, u * u, kGeluA));
}

// z = v + bias and GELU(z) = 0.5 z + 0.5 z tanh(z (a + b z^2)) for two
// columns at a time on the packed FP32 pipe (sph_f32x2.cuh); z is returned for
// the training saves. Four issue slots and one special-function op per
// activation.
__device__ __forceinline__ void bias_gelu2(float v0, float v1, float b0, float b1, float& z0, float& z1, float& g0,
                                           float& g1) {
    const f32x2 z = add2(pack2(v0, v1), pack2(b0, b1));
    const f32x2 inner = fma2(mul2(z, z), pack2(kGeluB, kGeluB), pack2(kGeluA, kGeluA));
    float t0, t1;
    unpack2(mul2(z, inner), t0, t1);
    const f32x2 th = pack2(tanh_approx(t0), tanh_approx(t1));
    const f32x2 hz = mul2(pack2(0.5f, 0.5f), z);
    unpack2(fma2(hz, th, hz), g0, g1);
    unpack2(z, z0, z1);
}

// Twice GELU for two columns: z + z tanh(z (a + b z^2)), one multiply fewer
// than bias_gelu2; the layer that reads it takes its weights halved, which
// leaves every BF16 product, and so every sum, as it was (power-of-two
// scalings are exact).
__device__ __forceinline__ void bias_gelu2_twice(float v0, float v1, float b0, float b1, float& g0, float& g1) {
    const f32x2 z = add2(pack2(v0, v1), pack2(b0, b1));
    const f32x2 inner = fma2(mul2(z, z), pack2(kGeluB, kGeluB), pack2(kGeluA, kGeluA));
    float t0, t1;
    unpack2(mul2(z, inner), t0, t1);
    unpack2(fma2(z, pack2(tanh_approx(t0), tanh_approx(t1)), z), g0, g1);
}

// Halves eight BF16 values (exact for normal numbers).
__device__ __forceinline__ uint4 halve_bf16x8(uint4 q) {
    uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162*>(&w[i]);
        const float2 f = __bfloat1622float2(v);
        v = __floats2bfloat162_rn(0.5f * f.x, 0.5f * f.y);
        w[i] = *reinterpret_cast<uint32_t*>(&v);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

constexpr uint32_t kForwardThreads = 512;
constexpr uint32_t kGroups = kForwardThreads / 128;  // threads sharing one row's epilogue

// One CTA of 256 threads owns 128 TMEM columns and runs 128-particle tiles:
// X (normalised features, BF16) -> [MMA W1] -> +b1, GELU -> H1 (BF16) ->
// [MMA W2] -> +b2, GELU -> H2 -> [MMA W3] -> +b3 -> scaled output. Row r of a
// tile is TMEM lane r; warp w reads the lane quarter w % 4 and, for the hidden
// layers, the column group w / 4, so kGroups threads share each row's epilogue.
// One thread issues the MMAs; an mbarrier reports their completion. The
// input is FP32 features, normalised and rounded to BF16 here (the
// training forward and sph_mlp_forward; the learned step's own forward is
// mlp_forward_ws_kernel, over ready BF16 tiles).
template <bool kSave>
__global__ void __launch_bounds__(kForwardThreads, 2) mlp_forward_kernel(ModelView model,
                                                                         const float* __restrict__ features,
                                                                         uint32_t n, float* __restrict__ out,
                                                                         ForwardSaves saves,
                                                                         unsigned int* __restrict__ error_flag,
                                                                         uint32_t wait_polls) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kSmemBar);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kSmemBar + 8);
    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t quarter = warp & 3u;
    const uint32_t group = warp >> 2;
    const uint32_t local_row = quarter * 32u + (tid & 31u);

    // Weights into the canonical K-major layout (16-byte chunks).
    for (uint32_t c = tid; c < kHidden * (kIn / 8); c += blockDim.x) {
        uint32_t row = c / (kIn / 8);
        uint32_t chunk = c % (kIn / 8);
        *reinterpret_cast<uint4*>(smem + kSmemW1 + tile_offset(row, chunk, kIn)) =
            *reinterpret_cast<const uint4*>(model.w1 + row * kIn + chunk * 8);
    }
    for (uint32_t c = tid; c < kHidden * (kHidden / 8); c += blockDim.x) {
        uint32_t row = c / (kHidden / 8);
        uint32_t chunk = c % (kHidden / 8);
        *reinterpret_cast<uint4*>(smem + kSmemW2 + tile_offset(row, chunk, kHidden)) =
            *reinterpret_cast<const uint4*>(model.w2 + row * kHidden + chunk * 8);
    }
    for (uint32_t c = tid; c < kOutPad * (kHidden / 8); c += blockDim.x) {
        uint32_t row = c / (kHidden / 8);
        uint32_t chunk = c % (kHidden / 8);
        *reinterpret_cast<uint4*>(smem + kSmemW3 + tile_offset(row, chunk, kHidden)) =
            *reinterpret_cast<const uint4*>(model.w3 + row * kHidden + chunk * 8);
    }
    float* vec = reinterpret_cast<float*>(smem + kSmemVec);
    for (uint32_t i = tid; i < kVecFloats; i += blockDim.x) {
        float v = 0.0f;
        if (i < kVecB2) {
            v = model.params[kB1 + i];
        } else if (i < kVecMean) {
            v = model.params[kB2 + (i - kVecB2)];
        } else if (i < kVecInvStd) {
            v = model.in_mean[i - kVecMean];
        } else if (i < kVecB3) {
            v = model.in_inv_std[i - kVecInvStd];
        } else if (i < kVecScale) {
            v = i - kVecB3 < static_cast<uint32_t>(kOut) ? model.params[kB3 + (i - kVecB3)] : 0.0f;
        } else {
            v = i - kVecScale < static_cast<uint32_t>(kOut) ? model.out_scale[i - kVecScale] : 0.0f;
        }
        vec[i] = v;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_base = (quarter * 32u) << 16;
    const float* b1 = vec + kVecB1;
    const float* b2 = vec + kVecB2;
    const float* b3 = vec + kVecB3;
    const float* in_mean = vec + kVecMean;
    const float* in_inv_std = vec + kVecInvStd;
    const float* out_scale = vec + kVecScale;
    const uint32_t sX = smem_u32(smem + kSmemX);
    const uint32_t sH = smem_u32(smem + kSmemH);
    const uint32_t sW1 = smem_u32(smem + kSmemW1);
    const uint32_t sW2 = smem_u32(smem + kSmemW2);
    const uint32_t sW3 = smem_u32(smem + kSmemW3);
    constexpr uint32_t idesc_hidden = instr_desc(kTile, kHidden);
    constexpr uint32_t idesc_out = instr_desc(kTile, kOutPad);
    uint32_t parity = 0;
    bool failed = false;
    const uint32_t tiles = (n + kTile - 1) / kTile;

    // Each thread converts one 8-feature chunk of its row; the next tile's
    // chunk is loaded while this tile runs its three layers.
    static_assert((kIn / 8) / kGroups == 1, "one 8-feature chunk per thread");
    const uint32_t chunk = group;
    auto fetch = [&](uint32_t t, float4& a, float4& b) {
        const uint32_t r = t * kTile + local_row;
        if (t < tiles && r < n) {
            const float4* frow = reinterpret_cast<const float4*>(features + static_cast<size_t>(r) * kIn);
            a = __ldg(&frow[2 * chunk]);
            b = __ldg(&frow[2 * chunk + 1]);
        } else {
            a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            b = a;
        }
    };
    float4 next_a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 next_b = next_a;
    fetch(blockIdx.x, next_a, next_b);

    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const uint32_t row = tile * kTile + local_row;
        const bool valid = row < n;
        const uint32_t sXt = sX;
        const float4 a = next_a;
        const float4 b = next_b;
        fetch(tile + gridDim.x, next_a, next_b);
        {
            float v[8];
            const float raw[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) {
                uint32_t f = chunk * 8 + k;
                v[k] = valid ? (raw[k] - in_mean[f]) * in_inv_std[f] : 0.0f;
            }
            store_chunk(smem + kSmemX, tile_offset(local_row, chunk, kIn), v);
            if (kSave && valid) {
#pragma unroll
                for (uint32_t k = 0; k < 8; ++k) {
                    saves.x[static_cast<size_t>(row) * kIn + chunk * 8 + k] = __float2bfloat16_rn(v[k]);
                }
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();

        // ---- layer 1: [128 x 32] x [32 x 128] ----
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t k = 0; k < kIn / 16; ++k) {
                mma_bf16(tmem, smem_desc(sXt + k * 256u, 128u, (kIn / 8) * 128u),
                         smem_desc(sW1 + k * 256u, 128u, (kIn / 8) * 128u), idesc_hidden, k > 0 ? 1u : 0u);
            }
            mma_commit(mbar);
        }
        bool ok = mbar_wait(mbar, parity, wait_polls);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        parity ^= 1u;
        tc_fence_after();
#pragma unroll 1
        for (uint32_t j = 0; j < (kHidden / 16) / kGroups; ++j) {
            uint32_t c = group * ((kHidden / 16) / kGroups) + j;
            float v[16];
            tmem_load16(tmem + lane_base + c * 16u, v);
            float bias[16];
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                const float4 b4 = reinterpret_cast<const float4*>(b1 + c * 16)[q];
                bias[4 * q] = b4.x;
                bias[4 * q + 1] = b4.y;
                bias[4 * q + 2] = b4.z;
                bias[4 * q + 3] = b4.w;
            }
#pragma unroll
            for (uint32_t k = 0; k < 16; k += 2) {
                float z0, z1;
                bias_gelu2(v[k], v[k + 1], bias[k], bias[k + 1], z0, z1, v[k], v[k + 1]);
                if (kSave && valid) {
                    saves.z1[static_cast<size_t>(row) * kHidden + c * 16 + k] = z0;
                    saves.z1[static_cast<size_t>(row) * kHidden + c * 16 + k + 1] = z1;
                }
            }
            store_chunk(smem + kSmemH, tile_offset(local_row, 2 * c, kHidden), v);
            store_chunk(smem + kSmemH, tile_offset(local_row, 2 * c + 1, kHidden), v + 8);
            if (kSave && valid) {
#pragma unroll
                for (uint32_t k = 0; k < 16; ++k) {
                    saves.h1[static_cast<size_t>(row) * kHidden + c * 16 + k] = __float2bfloat16_rn(v[k]);
                }
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();

        // ---- layer 2: [128 x 128] x [128 x 128] ----
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t k = 0; k < kHidden / 16; ++k) {
                mma_bf16(tmem, smem_desc(sH + k * 256u, 128u, (kHidden / 8) * 128u),
                         smem_desc(sW2 + k * 256u, 128u, (kHidden / 8) * 128u), idesc_hidden, k > 0 ? 1u : 0u);
            }
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, parity, wait_polls);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        parity ^= 1u;
        tc_fence_after();
#pragma unroll 1
        for (uint32_t j = 0; j < (kHidden / 16) / kGroups; ++j) {
            uint32_t c = group * ((kHidden / 16) / kGroups) + j;
            float v[16];
            tmem_load16(tmem + lane_base + c * 16u, v);
            float bias[16];
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                const float4 b4 = reinterpret_cast<const float4*>(b2 + c * 16)[q];
                bias[4 * q] = b4.x;
                bias[4 * q + 1] = b4.y;
                bias[4 * q + 2] = b4.z;
                bias[4 * q + 3] = b4.w;
            }
#pragma unroll
            for (uint32_t k = 0; k < 16; k += 2) {
                float z0, z1;
                bias_gelu2(v[k], v[k + 1], bias[k], bias[k + 1], z0, z1, v[k], v[k + 1]);
                if (kSave && valid) {
                    saves.z2[static_cast<size_t>(row) * kHidden + c * 16 + k] = z0;
                    saves.z2[static_cast<size_t>(row) * kHidden + c * 16 + k + 1] = z1;
                }
            }
            store_chunk(smem + kSmemH, tile_offset(local_row, 2 * c, kHidden), v);
            store_chunk(smem + kSmemH, tile_offset(local_row, 2 * c + 1, kHidden), v + 8);
            if (kSave && valid) {
#pragma unroll
                for (uint32_t k = 0; k < 16; ++k) {
                    saves.h2[static_cast<size_t>(row) * kHidden + c * 16 + k] = __float2bfloat16_rn(v[k]);
                }
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();

        // ---- layer 3: [128 x 128] x [128 x 16] ----
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t k = 0; k < kHidden / 16; ++k) {
                mma_bf16(tmem, smem_desc(sH + k * 256u, 128u, (kHidden / 8) * 128u),
                         smem_desc(sW3 + k * 256u, 128u, (kHidden / 8) * 128u), idesc_out, k > 0 ? 1u : 0u);
            }
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, parity, wait_polls);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        parity ^= 1u;
        tc_fence_after();
        if (group == 0) {
            float v[16];
            tmem_load16(tmem + lane_base, v);
            if (valid) {
                float y0 = v[0] + b3[0];
                float y1 = v[1] + b3[1];
                float y2 = v[2] + b3[2];
                if (kSave) {
                    reinterpret_cast<float4*>(saves.y)[row] = make_float4(y0, y1, y2, 0.0f);
                }
                if (out != nullptr) {
                    reinterpret_cast<float4*>(out)[row] =
                        make_float4(y0 * out_scale[0], y1 * out_scale[1], y2 * out_scale[2], 0.0f);
                }
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) {
            atomicOr(error_flag, 1u);
        }
        // Let an MMA still in flight finish (bounded) before the columns go.
        mbar_wait(mbar, parity, wait_polls);
        tc_fence_before();
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// ---- warp-specialised forward, two tiles in flight ----------------------------
//
// The inference form over ready BF16 input tiles (the learned step's). One
// persistent CTA per SM: 16 epilogue warps and one issuing warp, two tile
// slots, each with its own 128 TMEM columns, X and H buffers and barriers.
// The issuing warp's first lane copies input tiles in and issues each
// layer's MMAs as soon as the slot's operands are ready; the epilogue warps
// take each finished layer (+bias, GELU, BF16 into H; the output at the end)
// and report back. While the tensor cores run one slot's layer the CUDA
// cores run the other slot's epilogue, and no step waits on a block-wide
// barrier:
//   issuer, per pair k and slot s: [done(s, k-1)] load -> L1 ; h1 -> next load, L2 ; h2 -> L3
//   epilogue warps:                mma -> E1 -> h1 ; mma -> E2 -> h2 ; mma -> E3 -> done
// Per tile the operations are mlp_forward_kernel's, so the output bits are
// the same.
constexpr uint32_t kPairW1 = 0;
constexpr uint32_t kPairW2 = kPairW1 + kHidden * kIn * 2;
constexpr uint32_t kPairW3 = kPairW2 + kHidden * kHidden * 2;
constexpr uint32_t kPairX = kPairW3 + kOutPad * kHidden * 2;        // two input tiles
constexpr uint32_t kPairHBytes = kTile * kHidden * 2;
constexpr uint32_t kPairH = kPairX + 2 * kXTileBytes;                // two hidden tiles
constexpr uint32_t kPairBar = kPairH + 2 * kPairHBytes;              // 10 barriers, TMEM address
constexpr uint32_t kPairVec = kPairBar + 128;
constexpr uint32_t kPairBytes = kPairVec + kVecFloats * 4;
constexpr uint32_t kPairTmemCols = 256;
constexpr uint32_t kEpilogueWarps = kForwardThreads / 32;            // 16
constexpr uint32_t kWsThreads = kForwardThreads + 32;                // + the issuing warp

// Weights into the canonical K-major layout (16-byte chunks) and the small
// FP32 vectors (b1, b2, input mean and 1/std, b3, output scale).
// half_w23: W2 and W3 halved (the epilogues then store twice GELU).
__device__ __forceinline__ void stage_model(const ModelView& model, uint8_t* smem, uint32_t w1, uint32_t w2, uint32_t w3,
                                            float* vec, uint32_t tid, uint32_t threads, bool half_w23) {
    for (uint32_t c = tid; c < kHidden * (kIn / 8); c += threads) {
        const uint32_t row = c / (kIn / 8);
        const uint32_t chunk = c % (kIn / 8);
        *reinterpret_cast<uint4*>(smem + w1 + tile_offset(row, chunk, kIn)) =
            *reinterpret_cast<const uint4*>(model.w1 + row * kIn + chunk * 8);
    }
    for (uint32_t c = tid; c < kHidden * (kHidden / 8); c += threads) {
        const uint32_t row = c / (kHidden / 8);
        const uint32_t chunk = c % (kHidden / 8);
        const uint4 q = *reinterpret_cast<const uint4*>(model.w2 + row * kHidden + chunk * 8);
        *reinterpret_cast<uint4*>(smem + w2 + tile_offset(row, chunk, kHidden)) = half_w23 ? halve_bf16x8(q) : q;
    }
    for (uint32_t c = tid; c < kOutPad * (kHidden / 8); c += threads) {
        const uint32_t row = c / (kHidden / 8);
        const uint32_t chunk = c % (kHidden / 8);
        const uint4 q = *reinterpret_cast<const uint4*>(model.w3 + row * kHidden + chunk * 8);
        *reinterpret_cast<uint4*>(smem + w3 + tile_offset(row, chunk, kHidden)) = half_w23 ? halve_bf16x8(q) : q;
    }
    for (uint32_t i = tid; i < kVecFloats; i += threads) {
        float v = 0.0f;
        if (i < kVecB2) {
            v = model.params[kB1 + i];
        } else if (i < kVecMean) {
            v = model.params[kB2 + (i - kVecB2)];
        } else if (i < kVecInvStd) {
            v = model.in_mean[i - kVecMean];
        } else if (i < kVecB3) {
            v = model.in_inv_std[i - kVecInvStd];
        } else if (i < kVecScale) {
            v = i - kVecB3 < static_cast<uint32_t>(kOut) ? model.params[kB3 + (i - kVecB3)] : 0.0f;
        } else {
            v = i - kVecScale < static_cast<uint32_t>(kOut) ? model.out_scale[i - kVecScale] : 0.0f;
        }
        vec[i] = v;
    }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

__global__ void __launch_bounds__(kWsThreads, 1) mlp_forward_ws_kernel(ModelView model,
                                                                       const uint8_t* __restrict__ x_tiles, uint32_t n,
                                                                       float* __restrict__ out,
                                                                       unsigned int* __restrict__ error_flag,
                                                                       uint32_t wait_polls) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kPairBar);
    uint64_t* load_bar = bars;      // [2] input tile landed (transaction bytes)
    uint64_t* mma_bar = bars + 2;   // [2] a layer's MMAs completed (three phases a pair)
    uint64_t* h1_bar = bars + 4;    // [2] epilogue 1 written (16 warp arrivals)
    uint64_t* h2_bar = bars + 6;    // [2] epilogue 2 written
    uint64_t* done_bar = bars + 8;  // [2] output read, the slot's columns free
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kPairBar + 80);
    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    float* vec = reinterpret_cast<float*>(smem + kPairVec);
    // A kernel launched programmatically after this one (the correction sums
    // or the finishing pass) may start once every CTA has started.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    stage_model(model, smem, kPairW1, kPairW2, kPairW3, vec, tid, blockDim.x, true);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kPairTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (uint32_t s = 0; s < 2; ++s) {
            mbar_init(&load_bar[s], 1);
            mbar_init(&mma_bar[s], 1);
            mbar_init(&h1_bar[s], kEpilogueWarps);
            mbar_init(&h2_bar[s], kEpilogueWarps);
            mbar_init(&done_bar[s], kEpilogueWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // Launched programmatically after the features pass, the CTA staged the
    // weights and took its tensor memory while that pass finished; the
    // input tiles are read only after its grid has ended.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t tiles = (n + kTile - 1) / kTile;
    const uint32_t pairs = (tiles + 1) / 2;
    bool failed = false;

    if (warp == kEpilogueWarps) {
        // ---- issuing warp (its first lane) ----
        if (lane == 0) {
            const uint32_t sW1 = smem_u32(smem + kPairW1);
            const uint32_t sW2 = smem_u32(smem + kPairW2);
            const uint32_t sW3 = smem_u32(smem + kPairW3);
            constexpr uint32_t idesc_hidden = instr_desc(kTile, kHidden);
            constexpr uint32_t idesc_out = instr_desc(kTile, kOutPad);
            uint32_t loads_issued[2] = {0, 0};
            uint32_t commits[2] = {0, 0};
            auto load_tile = [&](uint32_t s, uint32_t t) {
                bulk_load(smem + kPairX + s * kXTileBytes, x_tiles + static_cast<size_t>(t) * kXTileBytes,
                          kXTileBytes, &load_bar[s]);
                ++loads_issued[s];
            };
            auto layer = [&](uint32_t s, uint32_t a, uint32_t b, uint32_t k_row_bytes, uint32_t k_steps,
                             uint32_t idesc) {
                tc_fence_after();
                for (uint32_t k = 0; k < k_steps; ++k) {
                    mma_bf16(tmem + s * 128u, smem_desc(a + k * 256u, 128u, k_row_bytes),
                             smem_desc(b + k * 256u, 128u, k_row_bytes), idesc, k > 0 ? 1u : 0u);
                }
                mma_commit(&mma_bar[s]);
                ++commits[s];
            };
            if (blockIdx.x < pairs) {
                for (uint32_t s = 0; s < 2 && 2u * blockIdx.x + s < tiles; ++s) {
                    load_tile(s, 2u * blockIdx.x + s);
                }
            }
            uint32_t k = 0;
            for (uint32_t pair = blockIdx.x; pair < pairs && !failed; pair += gridDim.x, ++k) {
                const uint32_t slots = 2u * pair + 1u < tiles ? 2u : 1u;
                const uint32_t next = pair + gridDim.x;
                for (uint32_t s = 0; s < slots && !failed; ++s) {
                    // The slot's columns are free once the previous pair's output is read.
                    failed = (k > 0 && !mbar_wait(&done_bar[s], (k - 1u) & 1u, wait_polls)) ||
                             !mbar_wait(&load_bar[s], k & 1u, wait_polls);
                    if (!failed) {
                        layer(s, smem_u32(smem + kPairX + s * kXTileBytes), sW1, (kIn / 8) * 128u, kIn / 16,
                              idesc_hidden);
                    }
                }
                for (uint32_t s = 0; s < slots && !failed; ++s) {
                    failed = !mbar_wait(&h1_bar[s], k & 1u, wait_polls);
                    if (!failed) {
                        // Layer 1 of the slot is done (its epilogue waited for
                        // it), so its X buffer takes the next pair's tile.
                        if (next < pairs && 2u * next + s < tiles) {
                            load_tile(s, 2u * next + s);
                        }
                        layer(s, smem_u32(smem + kPairH + s * kPairHBytes), sW2, (kHidden / 8) * 128u, kHidden / 16,
                              idesc_hidden);
                    }
                }
                for (uint32_t s = 0; s < slots && !failed; ++s) {
                    failed = !mbar_wait(&h2_bar[s], k & 1u, wait_polls);
                    if (!failed) {
                        layer(s, smem_u32(smem + kPairH + s * kPairHBytes), sW3, (kHidden / 8) * 128u, kHidden / 16,
                              idesc_out);
                    }
                }
            }
            // Everything issued has completed before the columns and the
            // shared memory go (bounded waits; the last phase of each
            // barrier tells).
            for (uint32_t s = 0; s < 2; ++s) {
                if (commits[s] > 0) {
                    failed = !mbar_wait(&mma_bar[s], (commits[s] - 1u) & 1u, wait_polls) || failed;
                }
                if (loads_issued[s] > 0) {
                    failed = !mbar_wait(&load_bar[s], (loads_issued[s] - 1u) & 1u, wait_polls) || failed;
                }
            }
        }
    } else {
        // ---- epilogue warps ----
        const uint32_t quarter = warp & 3u;
        const uint32_t group = warp >> 2;
        const uint32_t local_row = quarter * 32u + lane;
        const uint32_t lane_base = (quarter * 32u) << 16;
        const float* b1 = vec + kVecB1;
        const float* b2 = vec + kVecB2;
        const float* b3 = vec + kVecB3;
        const float* out_scale = vec + kVecScale;
        // A warp decides together whether a wait completed, so that it
        // leaves the loop as a whole.
        auto wait_warp = [&](uint64_t* bar, uint32_t parity) -> bool {
            return __all_sync(0xFFFFFFFFu, mbar_wait(bar, parity, wait_polls));
        };
        auto report = [&](uint64_t* bar) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(bar);
            }
        };
        auto hidden = [&](uint32_t s, const float* bias_vec) {
            uint8_t* h = smem + kPairH + s * kPairHBytes;
            // The group's 32 columns: two 16-column TMEM loads, one wait.
            static_assert((kHidden / 16) / kGroups == 2, "two 16-column chunks per thread");
            const uint32_t c0 = group * 2u;
            uint32_t r[32];
            const uint32_t taddr = tmem + s * 128u + lane_base + c0 * 16u;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
                  "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                  "=r"(r[30]), "=r"(r[31])
                : "r"(taddr + 16u));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (uint32_t j = 0; j < 2; ++j) {
                const uint32_t c = c0 + j;
                float v[16];
#pragma unroll
                for (uint32_t q = 0; q < 16; ++q) {
                    v[q] = __uint_as_float(r[16 * j + q]);
                }
#pragma unroll
                for (uint32_t q = 0; q < 16; q += 4) {
                    const float4 b4 = reinterpret_cast<const float4*>(bias_vec + c * 16)[q / 4];
                    bias_gelu2_twice(v[q], v[q + 1], b4.x, b4.y, v[q], v[q + 1]);
                    bias_gelu2_twice(v[q + 2], v[q + 3], b4.z, b4.w, v[q + 2], v[q + 3]);
                }
                store_chunk(h, tile_offset(local_row, 2 * c, kHidden), v);
                store_chunk(h, tile_offset(local_row, 2 * c + 1, kHidden), v + 8);
            }
            // The next layer's MMAs read H through the async proxy.
            fence_async_smem();
        };
        uint32_t k = 0;
        for (uint32_t pair = blockIdx.x; pair < pairs && !failed; pair += gridDim.x, ++k) {
            const uint32_t slots = 2u * pair + 1u < tiles ? 2u : 1u;
            // mma_bar[s] completes three times a pair: phases 3k, 3k + 1, 3k + 2.
            for (uint32_t s = 0; s < slots && !failed; ++s) {
                failed = !wait_warp(&mma_bar[s], (3u * k) & 1u);
                if (!failed) {
                    tc_fence_after();
                    hidden(s, b1);
                    report(&h1_bar[s]);
                }
            }
            for (uint32_t s = 0; s < slots && !failed; ++s) {
                failed = !wait_warp(&mma_bar[s], (3u * k + 1u) & 1u);
                if (!failed) {
                    tc_fence_after();
                    hidden(s, b2);
                    report(&h2_bar[s]);
                }
            }
            for (uint32_t s = 0; s < slots && !failed; ++s) {
                failed = !wait_warp(&mma_bar[s], (3u * k + 2u) & 1u);
                if (!failed) {
                    tc_fence_after();
                    if (group == s) {
                        float v[16];
                        tmem_load16(tmem + s * 128u + lane_base, v);
                        const uint32_t row = (2u * pair + s) * kTile + local_row;
                        if (row < n && out != nullptr) {
                            const float y0 = v[0] + b3[0];
                            const float y1 = v[1] + b3[1];
                            const float y2 = v[2] + b3[2];
                            reinterpret_cast<float4*>(out)[row] =
                                make_float4(y0 * out_scale[0], y1 * out_scale[1], y2 * out_scale[2], 0.0f);
                        }
                    }
                    report(&done_bar[s]);
                }
            }
        }
    }
    tc_fence_before();
    if (__syncthreads_or(failed) && tid == 0) {
        atomicOr(error_flag, 1u);
    }
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPairTmemCols)
                     : "memory");
    }
}

// max |erf_forward(x) - erff(x)| over `count` points spread on [-6, 6] (as
// float bits in *out).
__global__ void erf_selftest_kernel(uint32_t count, unsigned int* out) {
    float worst = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        float x = -6.0f + 12.0f * (static_cast<float>(i) / static_cast<float>(count));
        worst = fmaxf(worst, fabsf(erf_forward(x) - erff(x)));
    }
    atomicMax(out, __float_as_uint(worst));
}

// The bounded wait on its own: one CTA waits on an mbarrier of one expected
// arrival, which thread 0 makes only when `arrive` is set, with a limit of
// `polls` tries, as the forward pass waits for its MMAs. No tensor-core work
// and no tensor memory are involved, so a wait that gives up leaves nothing
// in flight. A wait that gave up sets the error flag.
__global__ void wait_selftest_kernel(uint32_t polls, int arrive, unsigned int* error_flag) {
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) {
        mbar_init(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (arrive != 0 && threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&mbar)) : "memory");
    }
    const bool ok = mbar_wait(&mbar, 0, polls);
    if (!__syncthreads_and(ok) && threadIdx.x == 0) {
        atomicOr(error_flag, 1u);
    }
}

// ---- backward on the tensor cores ----------------------------------------------
//
// One persistent CTA per SM (512 threads, 512 TMEM columns) takes 128-row
// tiles of the batch. Per tile, on the CUDA cores: dY from the loss, dZ2 =
// (dY W3) * GELU'(z2) in FP32, rounded to BF16 into two shared-memory tiles,
// one K-major over hidden units (for dH1) and one transposed, K-major over
// the tile's rows (for dW2); the tile's H1, H2 and X rows are staged
// transposed the same way, each with an appended row of ones, so that the
// bias gradients come out of the same products. On the tensor cores
// (tcgen05 kind::f16, FP32 accumulation):
//   dH1[r][i]  = sum_c dZ2[r][c] W2[c][i]       (TMEM, per tile)
//   dW2[o][i]  += sum_r dZ2[r][o] H1[r][i]      (+ db2 in column 128)
//   dW3t[c][j] += sum_r H2[r][c] dY[r][j]
// then dZ1 = dH1 * GELU'(z1) (FP32, rounded to BF16, transposed) and
//   dW1[o][i]  += sum_r dZ1[r][o] X[r][i]       (+ db1 in column 32).
// The weight gradients stay in TMEM across all of a CTA's tiles; at the end
// each CTA writes one parameter-shaped partial, and partials are summed in CTA
// order (deterministic). db3 and the loss are summed on the CUDA cores in a
// fixed order. The BF16 roundings (dY for dW3, dZ2, dZ1) are those of the
// oracle's loss_and_grad(..., bf16_grads=True).

constexpr uint32_t kBwThreads = 512;
constexpr uint32_t kBwRows = 128;                              // K of the weight-gradient products
constexpr uint32_t kBwH1Rows = kHidden + 16;                   // h1 rows, a row of ones, padding
constexpr uint32_t kBwXRows = kIn + 16;                        // x rows, a row of ones, padding
constexpr uint32_t kBwW2T = 0;                                 // W2 transposed [i][c]
constexpr uint32_t kBwA = kBwW2T + kHidden * kHidden * 2;      // dZ2 [r][c], then dZ1 transposed [o][r]
constexpr uint32_t kBwT2 = kBwA + kBwRows * kHidden * 2;       // dZ2 transposed [o][r]
constexpr uint32_t kBwH1 = kBwT2 + kHidden * kBwRows * 2;      // H1 transposed + ones [i][r]
constexpr uint32_t kBwH2 = kBwH1 + kBwH1Rows * kBwRows * 2;    // H2 transposed [c][r]
constexpr uint32_t kBwDY = kBwH2 + kHidden * kBwRows * 2;      // dY transposed [j][r], rows 3..15 zero
constexpr uint32_t kBwX = kBwDY + kOutPad * kBwRows * 2;       // X transposed + ones [i][r]
constexpr uint32_t kBwW3 = kBwX + kBwXRows * kBwRows * 2;      // W3 as FP32 [3][128]
constexpr uint32_t kBwRed = kBwW3 + kOut * kHidden * 4;        // per-quarter sums: dY (3) and loss
constexpr uint32_t kBwBar = kBwRed + 64;
constexpr uint32_t kBwBytes = kBwBar + 16;
static_assert(kBwBytes <= 227u * 1024u, "one CTA's shared memory");
// TMEM columns of the accumulators (starts at multiples of 32).
constexpr uint32_t kBwColDH1 = 0;    // 128
constexpr uint32_t kBwColDW2 = 128;  // 144: dW2 (128), db2 (1), padding
constexpr uint32_t kBwColDW3 = 288;  // 16: dW3 transposed (3 used)
constexpr uint32_t kBwColDW1 = 320;  // 48: dW1 (32), db1 (1), padding
constexpr uint32_t kBwTmemCols = 512;

// Byte offset of element (row, k) in a K-major no-swizzle tile of `k_elems`
// BF16 elements a row.
__device__ __forceinline__ uint32_t elem_offset(uint32_t row, uint32_t k, uint32_t k_elems) {
    return tile_offset(row, k >> 3, k_elems) + (k & 7u) * 2u;
}

__device__ __forceinline__ void store_bf16(uint8_t* base, uint32_t offset, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + offset) = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(kBwThreads, 1) mlp_backward_tc_kernel(ModelView model, ForwardSaves saves,
                                                                        const float* __restrict__ targets, uint32_t n,
                                                                        float* __restrict__ partial,
                                                                        unsigned int* __restrict__ error_flag,
                                                                        uint32_t wait_polls) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kBwBar);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kBwBar + 8);
    float* w3f = reinterpret_cast<float*>(smem + kBwW3);
    float* red = reinterpret_cast<float*>(smem + kBwRed);
    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    const uint32_t quarter = warp & 3u;
    const uint32_t group = warp >> 2;  // 32 columns each
    const uint32_t local_row = quarter * 32u + lane;

    // Staged once: W2 transposed, W3 as FP32, the constant rows.
    for (uint32_t e = tid; e < kHidden * kHidden; e += blockDim.x) {
        const uint32_t c = e / kHidden;
        const uint32_t i = e % kHidden;
        *reinterpret_cast<__nv_bfloat16*>(smem + kBwW2T + elem_offset(i, c, kHidden)) = model.w2[e];
    }
    for (uint32_t e = tid; e < kOut * kHidden; e += blockDim.x) {
        w3f[e] = __bfloat162float(model.w3[e]);
    }
    for (uint32_t e = tid; e < 16u * kBwRows; e += blockDim.x) {
        const uint32_t extra = e / kBwRows;
        const uint32_t r = e % kBwRows;
        store_bf16(smem + kBwH1, elem_offset(kHidden + extra, r, kBwRows), extra == 0 ? 1.0f : 0.0f);
        store_bf16(smem + kBwX, elem_offset(kIn + extra, r, kBwRows), extra == 0 ? 1.0f : 0.0f);
        if (extra < kOutPad - kOut) {
            store_bf16(smem + kBwDY, elem_offset(kOut + extra, r, kBwRows), 0.0f);
        }
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kBwTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_base = (quarter * 32u) << 16;
    constexpr uint32_t idesc_dh1 = instr_desc(kTile, kHidden);
    constexpr uint32_t idesc_dw2 = instr_desc(kTile, kBwH1Rows);
    constexpr uint32_t idesc_dw3 = instr_desc(kTile, kOutPad);
    constexpr uint32_t idesc_dw1 = instr_desc(kTile, kBwXRows);
    const uint32_t sA = smem_u32(smem + kBwA);
    const uint32_t sT2 = smem_u32(smem + kBwT2);
    const uint32_t sH1 = smem_u32(smem + kBwH1);
    const uint32_t sH2 = smem_u32(smem + kBwH2);
    const uint32_t sDY = smem_u32(smem + kBwDY);
    const uint32_t sX = smem_u32(smem + kBwX);
    const uint32_t sW2T = smem_u32(smem + kBwW2T);
    constexpr uint32_t kSbo = (kBwRows / 8u) * 128u;  // K = 128 in every product
    const float inv = 2.0f / (static_cast<float>(n) * kOut);
    const uint32_t tiles = (n + kTile - 1) / kTile;
    uint32_t parity = 0;
    bool failed = false;
    bool first = true;
    float cta_dy[3] = {0.0f, 0.0f, 0.0f};  // thread 0: db3 of this CTA's rows
    float cta_loss = 0.0f;

    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const uint32_t row = tile * kTile + local_row;
        const bool valid = row < n;
        // dY and the row's squared error.
        float dy[3] = {0.0f, 0.0f, 0.0f};
        float err2 = 0.0f;
        if (valid) {
            const float4 y = reinterpret_cast<const float4*>(saves.y)[row];
            const float yv[3] = {y.x, y.y, y.z};
#pragma unroll
            for (uint32_t o = 0; o < kOut; ++o) {
                const float t = targets[static_cast<size_t>(row) * kOut + o] / model.out_scale[o];
                const float e = yv[o] - t;
                err2 += e * e;
                dy[o] = inv * e;
            }
        }
        if (group == 0) {
#pragma unroll
            for (uint32_t j = 0; j < kOut; ++j) {
                store_bf16(smem + kBwDY, elem_offset(j, local_row, kBwRows), dy[j]);
            }
            float sums[4] = {dy[0], dy[1], dy[2], err2};
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    sums[q] += __shfl_down_sync(0xFFFFFFFFu, sums[q], o);
                }
            }
            if (lane == 0) {
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) {
                    red[quarter * 4u + q] = sums[q];
                }
            }
        }
        // dZ2 for this thread's 32 columns, and the transposed H1 and H2 rows.
#pragma unroll 1
        for (uint32_t cc = 0; cc < 2; ++cc) {
            const uint32_t c0 = group * 32u + cc * 16u;
            float d[16];
#pragma unroll
            for (uint32_t k = 0; k < 16; ++k) {
                const uint32_t c = c0 + k;
                const float dh2 = dy[0] * w3f[c] + dy[1] * w3f[kHidden + c] + dy[2] * w3f[2 * kHidden + c];
                d[k] = valid ? dh2 * gelu_grad(saves.z2[static_cast<size_t>(row) * kHidden + c]) : 0.0f;
            }
            store_chunk(smem + kBwA, tile_offset(local_row, c0 / 8u, kHidden), d);
            store_chunk(smem + kBwA, tile_offset(local_row, c0 / 8u + 1u, kHidden), d + 8);
#pragma unroll
            for (uint32_t k = 0; k < 16; ++k) {
                store_bf16(smem + kBwT2, elem_offset(c0 + k, local_row, kBwRows), d[k]);
            }
            uint4 h1v[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
            uint4 h2v[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
            if (valid) {
                const uint4* h1row = reinterpret_cast<const uint4*>(saves.h1 + static_cast<size_t>(row) * kHidden + c0);
                const uint4* h2row = reinterpret_cast<const uint4*>(saves.h2 + static_cast<size_t>(row) * kHidden + c0);
                h1v[0] = h1row[0];
                h1v[1] = h1row[1];
                h2v[0] = h2row[0];
                h2v[1] = h2row[1];
            }
            const __nv_bfloat16* h1e = reinterpret_cast<const __nv_bfloat16*>(h1v);
            const __nv_bfloat16* h2e = reinterpret_cast<const __nv_bfloat16*>(h2v);
#pragma unroll
            for (uint32_t k = 0; k < 16; ++k) {
                *reinterpret_cast<__nv_bfloat16*>(smem + kBwH1 + elem_offset(c0 + k, local_row, kBwRows)) = h1e[k];
                *reinterpret_cast<__nv_bfloat16*>(smem + kBwH2 + elem_offset(c0 + k, local_row, kBwRows)) = h2e[k];
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t acc = first ? 0u : 1u;
#pragma unroll
            for (uint32_t k = 0; k < kHidden / 16; ++k) {
                mma_bf16(tmem + kBwColDH1, smem_desc(sA + k * 256u, 128u, (kHidden / 8) * 128u),
                         smem_desc(sW2T + k * 256u, 128u, (kHidden / 8) * 128u), idesc_dh1, k > 0 ? 1u : 0u);
            }
#pragma unroll
            for (uint32_t k = 0; k < kBwRows / 16; ++k) {
                mma_bf16(tmem + kBwColDW2, smem_desc(sT2 + k * 256u, 128u, kSbo), smem_desc(sH1 + k * 256u, 128u, kSbo),
                         idesc_dw2, k > 0 ? 1u : acc);
                mma_bf16(tmem + kBwColDW3, smem_desc(sH2 + k * 256u, 128u, kSbo), smem_desc(sDY + k * 256u, 128u, kSbo),
                         idesc_dw3, k > 0 ? 1u : acc);
            }
            mma_commit(mbar);
            // db3 and the loss of this tile, quarters in order.
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                cta_dy[0] += red[q * 4u];
                cta_dy[1] += red[q * 4u + 1u];
                cta_dy[2] += red[q * 4u + 2u];
                cta_loss += red[q * 4u + 3u];
            }
        }
        bool ok = mbar_wait(mbar, parity, wait_polls);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        parity ^= 1u;
        tc_fence_after();
        // dZ1 = dH1 * GELU'(z1), transposed into the A tile; the X rows.
#pragma unroll 1
        for (uint32_t cc = 0; cc < 2; ++cc) {
            const uint32_t c0 = group * 32u + cc * 16u;
            float v[16];
            tmem_load16(tmem + lane_base + kBwColDH1 + c0, v);
#pragma unroll
            for (uint32_t k = 0; k < 16; ++k) {
                const uint32_t i = c0 + k;
                const float d1 = valid ? v[k] * gelu_grad(saves.z1[static_cast<size_t>(row) * kHidden + i]) : 0.0f;
                store_bf16(smem + kBwA, elem_offset(i, local_row, kBwRows), d1);
            }
        }
        if (group == 0) {
            uint4 xv[4] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0),
                           make_uint4(0, 0, 0, 0)};
            if (valid) {
                const uint4* xrow = reinterpret_cast<const uint4*>(saves.x + static_cast<size_t>(row) * kIn);
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) {
                    xv[q] = xrow[q];
                }
            }
            const __nv_bfloat16* xe = reinterpret_cast<const __nv_bfloat16*>(xv);
#pragma unroll
            for (uint32_t i = 0; i < kIn; ++i) {
                *reinterpret_cast<__nv_bfloat16*>(smem + kBwX + elem_offset(i, local_row, kBwRows)) = xe[i];
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t k = 0; k < kBwRows / 16; ++k) {
                mma_bf16(tmem + kBwColDW1, smem_desc(sA + k * 256u, 128u, kSbo), smem_desc(sX + k * 256u, 128u, kSbo),
                         idesc_dw1, k > 0 ? 1u : (first ? 0u : 1u));
            }
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, parity, wait_polls);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        parity ^= 1u;
        tc_fence_after();
        first = false;
    }
    float* part = partial + static_cast<size_t>(blockIdx.x) * (kParams + 1);
    if (failed) {
        if (tid == 0) {
            atomicOr(error_flag, 1u);
        }
        // Let an MMA still in flight finish (bounded) before the columns go.
        mbar_wait(mbar, parity, wait_polls);
        tc_fence_before();
        __syncthreads();
    } else if (first) {
        // No tile for this CTA: a zero partial.
        for (uint32_t e = tid; e < kParams + 1; e += blockDim.x) {
            part[e] = 0.0f;
        }
    } else {
        // The accumulators: lane o of each product is output row o.
        const uint32_t o = local_row;
        for (uint32_t ch = group; ch < kBwH1Rows / 16u; ch += 4u) {
            float v[16];
            tmem_load16(tmem + lane_base + kBwColDW2 + ch * 16u, v);
#pragma unroll
            for (uint32_t k = 0; k < 16; ++k) {
                const uint32_t col = ch * 16u + k;
                if (col < kHidden) {
                    part[kW2 + o * kHidden + col] = v[k];
                } else if (col == kHidden) {
                    part[kB2 + o] = v[k];
                }
            }
        }
        if (group == 0) {
            float v[16];
            tmem_load16(tmem + lane_base + kBwColDW3, v);
#pragma unroll
            for (uint32_t j = 0; j < kOut; ++j) {
                part[kW3 + j * kHidden + o] = v[j];
            }
        }
        if (group < kBwXRows / 16u) {
            float v[16];
            tmem_load16(tmem + lane_base + kBwColDW1 + group * 16u, v);
#pragma unroll
            for (uint32_t k = 0; k < 16; ++k) {
                const uint32_t col = group * 16u + k;
                if (col < kIn) {
                    part[kW1 + o * kIn + col] = v[k];
                } else if (col == kIn) {
                    part[kB1 + o] = v[k];
                }
            }
        }
        if (tid == 0) {
            part[kB3] = cta_dy[0];
            part[kB3 + 1] = cta_dy[1];
            part[kB3 + 2] = cta_dy[2];
            part[kParams] = cta_loss / (static_cast<float>(n) * kOut);
        }
        tc_fence_before();
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBwTmemCols) : "memory");
    }
}

// grads[p] = sum over CTAs (in order) of the partials; loss likewise.
__global__ void reduce_partials_kernel(const float* __restrict__ partial, uint32_t ctas, float* __restrict__ grads,
                                       float* __restrict__ loss) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > static_cast<uint32_t>(kParams)) {
        return;
    }
    float s = 0.0f;
    for (uint32_t c = 0; c < ctas; ++c) {
        s += partial[static_cast<size_t>(c) * (kParams + 1) + p];
    }
    if (p < static_cast<uint32_t>(kParams)) {
        grads[p] = s;
    } else {
        *loss = s;
    }
}

__global__ void quantise_kernel(const float* __restrict__ params, __nv_bfloat16* __restrict__ w1,
                                __nv_bfloat16* __restrict__ w2, __nv_bfloat16* __restrict__ w3) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kHidden * kIn) {
        w1[i] = __float2bfloat16_rn(params[kW1 + i]);
    }
    if (i < kHidden * kHidden) {
        w2[i] = __float2bfloat16_rn(params[kW2 + i]);
    }
    if (i < kOutPad * kHidden) {
        w3[i] = i < kOut * kHidden ? __float2bfloat16_rn(params[kW3 + i]) : __float2bfloat16_rn(0.0f);
    }
}

// adamStep (src/gfx/neural_math.cpp:1188-1208), moments stored [first | second].
__global__ void adam_kernel(float* __restrict__ params, const float* __restrict__ grads, float* __restrict__ moments,
                            float lr, float beta1, float beta2, float epsilon, float first_correction,
                            float second_correction) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) {
        return;
    }
    float g = grads[i];
    float* first = moments;
    float* second = moments + kParams;
    first[i] = beta1 * first[i] + (1.0f - beta1) * g;
    second[i] = beta2 * second[i] + (1.0f - beta2) * g * g;
    float corrected_first = first[i] / first_correction;
    float corrected_second = second[i] / second_correction;
    params[i] -= lr * corrected_first / (sqrtf(corrected_second) + epsilon);
}

}  // namespace

cudaError_t launch_forward(const ModelView& model, const float* features, uint32_t n, float* out_accel,
                           const ForwardSaves* saves, unsigned int* error_flag, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    cudaError_t prepared = prepare_forward();
    if (prepared != cudaSuccess) {
        return prepared;
    }
    uint32_t tiles = (n + kTile - 1) / kTile;
    int device = 0;
    cudaGetDevice(&device);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t grid = std::min<uint32_t>(tiles, static_cast<uint32_t>(sms) * 2u);
    ForwardSaves none{};
    if (saves != nullptr) {
        mlp_forward_kernel<true><<<grid, kForwardThreads, kSmemBytes, stream>>>(model, features, n, out_accel,
                                                                                *saves, error_flag, kWaitPolls);
    } else {
        mlp_forward_kernel<false><<<grid, kForwardThreads, kSmemBytes, stream>>>(model, features, n, out_accel,
                                                                                 none, error_flag, kWaitPolls);
    }
    return cudaGetLastError();
}

cudaError_t launch_forward_tiles(const ModelView& model, const uint8_t* x_tiles, uint32_t n, float* out_accel,
                                 unsigned int* error_flag, cudaStream_t stream, bool programmatic) {
    if (n == 0) {
        return cudaSuccess;
    }
    cudaError_t prepared = prepare_forward();
    if (prepared != cudaSuccess) {
        return prepared;
    }
    uint32_t tiles = (n + kTile - 1) / kTile;
    int device = 0;
    cudaGetDevice(&device);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const uint32_t pairs = (tiles + 1) / 2;
    const uint32_t grid = std::min<uint32_t>(pairs, static_cast<uint32_t>(sms));
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kWsThreads);
    cfg.dynamicSmemBytes = kPairBytes;
    cfg.stream = stream;
    cfg.attrs = programmatic ? &attr : nullptr;
    cfg.numAttrs = programmatic ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, mlp_forward_ws_kernel, model, x_tiles, n, out_accel, error_flag, kWaitPolls);
}

void launch_wait_selftest(uint32_t polls, int arrive, unsigned int* error_flag, cudaStream_t stream) {
    wait_selftest_kernel<<<1, 128, 0, stream>>>(polls, arrive, error_flag);
}

void launch_erf_selftest(uint32_t count, unsigned int* out, cudaStream_t stream) {
    erf_selftest_kernel<<<152 * 4, 256, 0, stream>>>(count, out);
}

namespace {

// Kernel attributes are per device: which devices have had them set.
std::mutex g_attribute_guard;
uint64_t g_forward_ready = 0;
uint64_t g_backward_ready = 0;

// Runs `set` once per device (devices past 63 every time), under the guard.
template <typename Set>
cudaError_t once_per_device(uint64_t* ready, Set set) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) {
        return e;
    }
    std::lock_guard<std::mutex> lock(g_attribute_guard);
    if (device < 64 && (*ready >> device & 1u) != 0) {
        return cudaSuccess;
    }
    if ((e = set()) == cudaSuccess && device < 64) {
        *ready |= 1ull << device;
    }
    return e;
}

}  // namespace

cudaError_t prepare_forward() {
    return once_per_device(&g_forward_ready, [] {
        cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(kSmemBytes));
        if (e == cudaSuccess) {
            e = cudaFuncSetAttribute(mlp_forward_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(kSmemBytes));
        }
        if (e == cudaSuccess) {
            e = cudaFuncSetAttribute(mlp_forward_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(kPairBytes));
        }
        return e;
    });
}

size_t backward_scratch_floats(uint32_t n) {
    // One parameter-shaped partial (+ loss) per CTA; at most one CTA a tile.
    const size_t tiles = (static_cast<size_t>(n) + kTile - 1) / kTile;
    return (tiles == 0 ? 1 : tiles) * (kParams + 1);
}

cudaError_t launch_backward(const ModelView& model, const ForwardSaves& saves, const float* targets, uint32_t n,
                            float* d_params, float* loss, float* scratch, unsigned int* error_flag,
                            cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    cudaError_t attr = once_per_device(&g_backward_ready, [] {
        return cudaFuncSetAttribute(mlp_backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(kBwBytes));
    });
    if (attr != cudaSuccess) {
        return attr;
    }
    const uint32_t tiles = (n + kTile - 1) / kTile;
    int device = 0;
    cudaGetDevice(&device);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const uint32_t ctas = std::min<uint32_t>(tiles, static_cast<uint32_t>(sms));
    mlp_backward_tc_kernel<<<ctas, kBwThreads, kBwBytes, stream>>>(model, saves, targets, n, scratch, error_flag,
                                                                   kWaitPolls);
    reduce_partials_kernel<<<(kParams + 1 + 255) / 256, 256, 0, stream>>>(scratch, ctas, d_params, loss);
    return cudaGetLastError();
}

cudaError_t launch_quantise(const float* params, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w3,
                            cudaStream_t stream) {
    quantise_kernel<<<(kHidden * kHidden + 255) / 256, 256, 0, stream>>>(params, w1, w2, w3);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* params, const float* grads, float* moments, uint32_t step, float lr, float beta1,
                        float beta2, float epsilon, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w3,
                        cudaStream_t stream) {
    // adamCorrections (neural_math.cpp:1177-1186), step counted from 1.
    float first = 1.0F - std::pow(beta1, static_cast<float>(step));
    float second = 1.0F - std::pow(beta2, static_cast<float>(step));
    if (step == 0 || !(first > 0.0F) || !(second > 0.0F)) {
        return cudaSuccess;
    }
    adam_kernel<<<(kParams + 255) / 256, 256, 0, stream>>>(params, grads, moments, lr, beta1, beta2, epsilon, first,
                                                           second);
    return launch_quantise(params, w1, w2, w3, stream);
}

}  // namespace mlp
}  // namespace sph

// ---- C ABI --------------------------------------------------------------------


struct sph_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    float* params = nullptr;   // FP32 vector
    float* grads = nullptr;
    float* moments = nullptr;  // first | second
    __nv_bfloat16* w1 = nullptr;
    __nv_bfloat16* w2 = nullptr;
    __nv_bfloat16* w3 = nullptr;
    float* norm = nullptr;     // mean[32] | inv_std[32] | out_scale[3]
    float* loss = nullptr;
    unsigned int* error = nullptr;
    // Training buffers, grown to the largest batch.
    uint32_t capacity = 0;
    float* z1 = nullptr;
    float* z2 = nullptr;
    __nv_bfloat16* x = nullptr;
    __nv_bfloat16* h1 = nullptr;
    __nv_bfloat16* h2 = nullptr;
    float* y = nullptr;
    float* scratch = nullptr;
    uint32_t step = 0;
    float beta1 = 0.9F;
    float beta2 = 0.999F;
    float epsilon = 1e-8F;
    uint32_t free_axes = 0;
    std::string last_error;
};

namespace {

using sph::mlp::kHidden;
using sph::mlp::kIn;
using sph::mlp::kOut;
using sph::mlp::kOutPad;
using sph::mlp::kParams;

int mlp_fail(sph_mlp* m, cudaError_t e, const char* what) {
    if (m != nullptr) {
        m->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    }
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;
}

#define MLP_CUDA(m, call)                            \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) {                     \
            return mlp_fail((m), e_, #call);         \
        }                                            \
    } while (0)

sph::mlp::ModelView view(const sph_mlp* m) {
    sph::mlp::ModelView v;
    v.w1 = m->w1;
    v.w2 = m->w2;
    v.w3 = m->w3;
    v.params = m->params;
    v.in_mean = m->norm;
    v.in_inv_std = m->norm + kIn;
    v.out_scale = m->norm + 2 * kIn;
    v.free_axes = m->free_axes;
    return v;
}

uint64_t splitmix(uint64_t v) {
    v += 0x9E3779B97F4A7C15ULL;
    v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ULL;
    v = (v ^ (v >> 27)) * 0x94D049BB133111EBULL;
    return v ^ (v >> 31);
}

// Standard normal from two splitmix64 uniforms (Box-Muller).
float gaussian(uint64_t seed, uint64_t index) {
    double u1 = (static_cast<double>(splitmix(seed * 0x9E3779B97F4A7C15ULL + 2 * index) >> 11) + 1.0) * 0x1.0p-53;
    double u2 = static_cast<double>(splitmix(seed * 0x9E3779B97F4A7C15ULL + 2 * index + 1) >> 11) * 0x1.0p-53;
    return static_cast<float>(std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
}

int grow(sph_mlp* m, uint32_t n) {
    if (n <= m->capacity) {
        return SPH_OK;
    }
    void* bufs[] = {m->z1, m->z2, m->x, m->h1, m->h2, m->y, m->scratch};
    for (void* b : bufs) {
        if (b != nullptr) {
            cudaFree(b);
        }
    }
    size_t rows = n;
    MLP_CUDA(m, cudaMalloc(&m->z1, rows * kHidden * sizeof(float)));
    MLP_CUDA(m, cudaMalloc(&m->z2, rows * kHidden * sizeof(float)));
    MLP_CUDA(m, cudaMalloc(&m->x, rows * kIn * sizeof(__nv_bfloat16)));
    MLP_CUDA(m, cudaMalloc(&m->h1, rows * kHidden * sizeof(__nv_bfloat16)));
    MLP_CUDA(m, cudaMalloc(&m->h2, rows * kHidden * sizeof(__nv_bfloat16)));
    MLP_CUDA(m, cudaMalloc(&m->y, rows * 4 * sizeof(float)));
    MLP_CUDA(m, cudaMalloc(&m->scratch, sph::mlp::backward_scratch_floats(n) * sizeof(float)));
    m->capacity = n;
    return SPH_OK;
}

int gradients(sph_mlp* m, const void* features, const void* targets, uint32_t n) {
    int status = grow(m, n);
    if (status != SPH_OK) {
        return status;
    }
    sph::mlp::ForwardSaves saves{m->z1, m->z2, m->x, m->h1, m->h2, m->y};
    sph::mlp::ModelView v = view(m);
    MLP_CUDA(m, cudaMemsetAsync(m->error, 0, sizeof(unsigned int), m->stream));
    MLP_CUDA(m, sph::mlp::launch_forward(v, static_cast<const float*>(features), n, nullptr, &saves, m->error,
                                         m->stream));
    MLP_CUDA(m, sph::mlp::launch_backward(v, saves, static_cast<const float*>(targets), n, m->grads, m->loss,
                                          m->scratch, m->error, m->stream));
    return SPH_OK;
}

int check_error_flag(sph_mlp* m) {
    unsigned int flag = 0;
    MLP_CUDA(m, cudaMemcpyAsync(&flag, m->error, sizeof(flag), cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    if (flag != 0) {
        m->last_error = "tensor-core completion wait timed out";
        return SPH_ERR_TIMEOUT;
    }
    return SPH_OK;
}

}  // namespace

bool sph_mlp_model_view(const sph_mlp* m, sph::mlp::ModelView* out) {
    if (m == nullptr || out == nullptr) {
        return false;
    }
    *out = view(m);
    return true;
}

extern "C" {

int sph_mlp_create(int device, uint64_t seed, sph_mlp** out) {
    if (out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
        cudaGetLastError();
        return SPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= devices) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    sph_mlp* m = new (std::nothrow) sph_mlp();
    if (m == nullptr) {
        return SPH_ERR_OUT_OF_MEMORY;
    }
    m->device = device;
    auto cleanup = [&](int status) {
        sph_mlp_destroy(m);
        return status;
    };
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&m->params, kParams * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->grads, kParams * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->moments, 2 * kParams * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->w1, kHidden * kIn * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&m->w2, kHidden * kHidden * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&m->w3, kOutPad * kHidden * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&m->norm, (2 * kIn + kOut + 1) * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->loss, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->error, sizeof(unsigned int)) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(SPH_ERR_OUT_OF_MEMORY);
    }
    // He-normal weights (std sqrt(2 / fan_in)), zero biases; the last layer is
    // scaled down so an untrained model starts near "no correction".
    std::vector<float> p(kParams, 0.0F);
    uint64_t stream_id = 0;
    auto fill = [&](int offset, int count, int fan_in, float extra) {
        float deviation = std::sqrt(2.0F / static_cast<float>(fan_in)) * extra;
        for (int i = 0; i < count; ++i) {
            p[offset + i] = deviation * gaussian(seed + stream_id, static_cast<uint64_t>(i));
        }
        ++stream_id;
    };
    fill(sph::mlp::kW1, kHidden * kIn, kIn, 1.0F);
    fill(sph::mlp::kW2, kHidden * kHidden, kHidden, 1.0F);
    fill(sph::mlp::kW3, kOut * kHidden, kHidden, 0.1F);
    std::vector<float> norm(2 * kIn + kOut + 1, 0.0F);
    for (int i = 0; i < kIn; ++i) {
        norm[kIn + i] = 1.0F;
    }
    for (int o = 0; o < kOut; ++o) {
        norm[2 * kIn + o] = 1.0F;
    }
    if (cudaMemcpy(m->params, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->norm, norm.data(), norm.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->moments, 0, 2 * kParams * sizeof(float)) != cudaSuccess ||
        sph::mlp::launch_quantise(m->params, m->w1, m->w2, m->w3, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(SPH_ERR_CUDA);
    }
    *out = m;
    return SPH_OK;
}

int sph_mlp_destroy(sph_mlp* m) {
    if (m == nullptr) {
        return SPH_OK;
    }
    cudaSetDevice(m->device);
    void* bufs[] = {m->params, m->grads, m->moments, m->w1, m->w2, m->w3, m->norm, m->loss, m->error,
                    m->z1,     m->z2,    m->x,       m->h1, m->h2, m->y,  m->scratch};
    for (void* b : bufs) {
        if (b != nullptr) {
            cudaFree(b);
        }
    }
    if (m->stream != nullptr) {
        cudaStreamDestroy(m->stream);
    }
    delete m;
    return SPH_OK;
}

const char* sph_mlp_last_error(const sph_mlp* m) { return m == nullptr ? "" : m->last_error.c_str(); }

int sph_mlp_get_params(sph_mlp* m, float* params) {
    if (m == nullptr || params == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    MLP_CUDA(m, cudaMemcpy(params, m->params, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    return SPH_OK;
}

int sph_mlp_set_params(sph_mlp* m, const float* params) {
    if (m == nullptr || params == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < kParams; ++i) {
        if (!std::isfinite(params[i])) {
            return SPH_ERR_NONFINITE;
        }
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaMemcpyAsync(m->params, params, kParams * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MLP_CUDA(m, sph::mlp::launch_quantise(m->params, m->w1, m->w2, m->w3, m->stream));
    MLP_CUDA(m, cudaMemsetAsync(m->moments, 0, 2 * kParams * sizeof(float), m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    m->step = 0;
    return SPH_OK;
}

int sph_mlp_set_normalisation(sph_mlp* m, const float* feature_mean, const float* feature_std,
                              const float* output_scale) {
    if (m == nullptr || feature_mean == nullptr || feature_std == nullptr || output_scale == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::vector<float> norm(2 * kIn + kOut + 1, 0.0F);
    for (int i = 0; i < kIn; ++i) {
        if (!(feature_std[i] > 0.0F) || !std::isfinite(feature_mean[i])) {
            return SPH_ERR_INVALID_ARGUMENT;
        }
        norm[i] = feature_mean[i];
        norm[kIn + i] = 1.0F / feature_std[i];
    }
    for (int o = 0; o < kOut; ++o) {
        if (!(output_scale[o] > 0.0F)) {
            return SPH_ERR_INVALID_ARGUMENT;
        }
        norm[2 * kIn + o] = output_scale[o];
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaMemcpy(m->norm, norm.data(), norm.size() * sizeof(float), cudaMemcpyHostToDevice));
    return SPH_OK;
}

int sph_mlp_get_normalisation(sph_mlp* m, float* feature_mean, float* feature_std, float* output_scale) {
    if (m == nullptr || feature_mean == nullptr || feature_std == nullptr || output_scale == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::vector<float> norm(2 * kIn + kOut + 1);
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaMemcpy(norm.data(), m->norm, norm.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int i = 0; i < kIn; ++i) {
        feature_mean[i] = norm[i];
        feature_std[i] = 1.0F / norm[kIn + i];
    }
    for (int o = 0; o < kOut; ++o) {
        output_scale[o] = norm[2 * kIn + o];
    }
    return SPH_OK;
}

int sph_mlp_forward(sph_mlp* m, const void* features, uint32_t count, void* accel, void* stream) {
    if (m == nullptr || (count > 0 && (features == nullptr || accel == nullptr))) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    cudaStream_t s = stream != nullptr ? static_cast<cudaStream_t>(stream) : m->stream;
    MLP_CUDA(m, cudaMemsetAsync(m->error, 0, sizeof(unsigned int), s));
    MLP_CUDA(m, sph::mlp::launch_forward(view(m), static_cast<const float*>(features), count,
                                         static_cast<float*>(accel), nullptr, m->error, s));
    if (stream == nullptr) {
        return check_error_flag(m);
    }
    return SPH_OK;
}

int sph_mlp_gradients(sph_mlp* m, const void* features, const void* targets, uint32_t count, float* grads,
                      float* loss) {
    if (m == nullptr || features == nullptr || targets == nullptr || count == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    int status = gradients(m, features, targets, count);
    if (status != SPH_OK) {
        return status;
    }
    status = check_error_flag(m);
    if (status != SPH_OK) {
        return status;
    }
    if (grads != nullptr) {
        MLP_CUDA(m, cudaMemcpy(grads, m->grads, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    }
    if (loss != nullptr) {
        MLP_CUDA(m, cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    }
    return SPH_OK;
}

int sph_mlp_set_adam(sph_mlp* m, float beta1, float beta2, float epsilon) {
    if (m == nullptr || !(beta1 >= 0.0F && beta1 < 1.0F) || !(beta2 >= 0.0F && beta2 < 1.0F) || !(epsilon > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    m->beta1 = beta1;
    m->beta2 = beta2;
    m->epsilon = epsilon;
    return SPH_OK;
}

int sph_mlp_set_net_force_free(sph_mlp* m, uint32_t axes) {
    if (m == nullptr || axes > 7u) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    m->free_axes = axes;
    return SPH_OK;
}

int sph_mlp_train_step(sph_mlp* m, const void* features, const void* targets, uint32_t count, float learning_rate,
                       float* loss) {
    if (m == nullptr || features == nullptr || targets == nullptr || count == 0 || !(learning_rate > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    int status = gradients(m, features, targets, count);
    if (status != SPH_OK) {
        return status;
    }
    m->step += 1;
    MLP_CUDA(m, sph::mlp::launch_adam(m->params, m->grads, m->moments, m->step, learning_rate, m->beta1, m->beta2,
                                      m->epsilon, m->w1, m->w2, m->w3, m->stream));
    if (loss != nullptr) {
        MLP_CUDA(m, cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    }
    return check_error_flag(m);
}

int sph_mlp_apply_gradients(sph_mlp* m, const float* grads, float learning_rate) {
    if (m == nullptr || grads == nullptr || !(learning_rate > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaMemcpyAsync(m->grads, grads, kParams * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    m->step += 1;
    MLP_CUDA(m, sph::mlp::launch_adam(m->params, m->grads, m->moments, m->step, learning_rate, m->beta1, m->beta2,
                                      m->epsilon, m->w1, m->w2, m->w3, m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    return check_error_flag(m);
}

int sph_mlp_selftest_wait(sph_mlp* m, uint32_t polls, int arrive) {
    if (m == nullptr || polls == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaMemsetAsync(m->error, 0, sizeof(unsigned int), m->stream));
    sph::mlp::launch_wait_selftest(polls, arrive, m->error, m->stream);
    MLP_CUDA(m, cudaGetLastError());
    const int status = check_error_flag(m);
    MLP_CUDA(m, cudaMemsetAsync(m->error, 0, sizeof(unsigned int), m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    return status;
}

int sph_mlp_selftest_erf(sph_mlp* m, uint32_t count, float* max_abs_error) {
    if (m == nullptr || max_abs_error == nullptr || count == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    MLP_CUDA(m, cudaSetDevice(m->device));
    MLP_CUDA(m, cudaMemsetAsync(m->error, 0, sizeof(unsigned int), m->stream));
    sph::mlp::launch_erf_selftest(count, m->error, m->stream);
    unsigned int bits = 0;
    MLP_CUDA(m, cudaMemcpyAsync(&bits, m->error, sizeof(bits), cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(m, cudaStreamSynchronize(m->stream));
    std::memcpy(max_abs_error, &bits, sizeof(float));
    MLP_CUDA(m, cudaMemsetAsync(m->error, 0, sizeof(unsigned int), m->stream));
    return SPH_OK;
}

int sph_mlp_stream(sph_mlp* m, void** stream) {
    if (m == nullptr || stream == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *stream = static_cast<void*>(m->stream);
    return SPH_OK;
}

}  // extern "C"
