// Training kernels of the learned Kepler start: a 4 -> 64 -> 64 -> 1 MLP with
// SiLU activations, bf16 weights in the forward pass and FP32 accumulation,
// mean-squared error against log(converged root / plain first guess).
//
// FP32 master parameters live in one flat array (layout below).  Each step:
//   k_round_bf16  : bf16 copy of the master weights (what inference uses);
//   k_mlp_grad    : forward + backward of a mini-batch, one sample per thread,
//                   block-level reductions of the weight gradients in shared
//                   memory (dW2 = dZ2^T H1 as a 64x64x128 product per block),
//                   then one atomicAdd per parameter per block;
//   k_adam        : Adam update of the master parameters.
// Samples whose target is NaN (solver failures) carry no loss.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tg_common.cuh"

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace tg {

constexpr int IN = 4, H = 64, B = 128;       // features, hidden, samples/block
// flat parameter layout (fp32 masters and their gradients)
constexpr int OFF_W1 = 0;                    // H x IN
constexpr int OFF_B1 = OFF_W1 + H * IN;      // H
constexpr int OFF_W2 = OFF_B1 + H;           // H x H
constexpr int OFF_B2 = OFF_W2 + H * H;       // H
constexpr int OFF_W3 = OFF_B2 + H;           // H
constexpr int OFF_B3 = OFF_W3 + H;           // 1
constexpr int N_PARAM = OFF_B3 + 1;

__device__ __forceinline__ float sig(float x) { return 1.0f / (1.0f + __expf(-x)); }

// bf16 rounding of the weights; biases stay fp32.
__global__ void k_round_bf16(const float *p, __nv_bfloat16 *w1,
                             __nv_bfloat16 *w2, __nv_bfloat16 *w3, float *rw)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N_PARAM;
         t += gridDim.x * blockDim.x) {
        const float v = p[t];
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        float r = v;
        if (t < OFF_B1) { w1[t - OFF_W1] = b; r = __bfloat162float(b); }
        else if (t >= OFF_W2 && t < OFF_B2) { w2[t - OFF_W2] = b; r = __bfloat162float(b); }
        else if (t >= OFF_W3 && t < OFF_B3) { w3[t - OFF_W3] = b; r = __bfloat162float(b); }
        rw[t] = r;     // the values the forward pass multiplies with
    }
}

struct GradSmem {
    float w1[H * IN], b1[H], w2[H * H], b2[H], w3[H], b3;
    float norm[8];
    float h1[B][H + 1];        // activations of layer 1 (post SiLU)
    float d2[B][H + 1];        // z2, then dL/dz2
    float d1[B][H + 1];        // dL/dz1
    float x[B][IN];
    float g[B];                // dL/dy
};

// Forward + backward of samples [blockIdx.x*B, +B); gradients summed into
// grad[N_PARAM], squared error into *loss.  rw: bf16-rounded parameters.
__global__ void __launch_bounds__(B)
k_mlp_grad(const float *rw, const float *norm, const float *X, const float *Y,
           uint64_t n, float scale, float *grad, float *loss)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GradSmem &S = *reinterpret_cast<GradSmem *>(smem_raw);
    const int t = threadIdx.x;
    for (int k = t; k < H * H; k += B) {
        S.w2[k] = rw[OFF_W2 + k];
        if (k < H * IN) S.w1[k] = rw[OFF_W1 + k];
        if (k < H) {
            S.b1[k] = rw[OFF_B1 + k];
            S.b2[k] = rw[OFF_B2 + k];
            S.w3[k] = rw[OFF_W3 + k];
        }
        if (k < 8) S.norm[k] = norm[k];
    }
    if (t == 0) S.b3 = rw[OFF_B3];
    __syncthreads();

    const uint64_t s = (uint64_t)blockIdx.x * B + t;
    float tgt = s < n ? Y[s] : 0.0f;
    const bool valid = s < n && tgt == tgt;
    float x[IN];
    for (int k = 0; k < IN; ++k) {
        const float raw = s < n ? X[4 * s + k] : 0.0f;
        x[k] = (raw - S.norm[k]) * S.norm[4 + k];
        S.x[t][k] = valid ? x[k] : 0.0f;
    }
    // forward
    float z1[H];
#pragma unroll
    for (int o = 0; o < H; ++o) {
        float a = S.b1[o];
#pragma unroll
        for (int k = 0; k < IN; ++k) a = fmaf(S.w1[o * IN + k], x[k], a);
        z1[o] = a;
        S.h1[t][o] = a * sig(a);
    }
    float y = S.b3;
    for (int o = 0; o < H; ++o) {
        float a = S.b2[o];
#pragma unroll 16
        for (int k = 0; k < H; ++k) a = fmaf(S.w2[o * H + k], S.h1[t][k], a);
        S.d2[t][o] = a;
        y = fmaf(S.w3[o], a * sig(a), y);
    }
    const float err = valid ? (y - tgt) : 0.0f;
    const float g = 2.0f * err * scale;
    S.g[t] = g;
    if (valid) atomicAdd(loss, err * err);
    // dL/dz2 = g w3 silu'(z2)
    for (int o = 0; o < H; ++o) {
        const float z = S.d2[t][o];
        const float sg = sig(z);
        S.d2[t][o] = g * S.w3[o] * (sg * (1.0f + z * (1.0f - sg)));
    }
    // dL/dz1 = (W2^T dz2) silu'(z1)
#pragma unroll
    for (int k = 0; k < H; ++k) {
        float a = 0.0f;
        for (int o = 0; o < H; ++o) a = fmaf(S.w2[o * H + k], S.d2[t][o], a);
        const float sg = sig(z1[k]);
        S.d1[t][k] = a * (sg * (1.0f + z1[k] * (1.0f - sg)));
    }
    __syncthreads();
    // block reductions over the B samples
    for (int q = t; q < H * H; q += B) {           // dW2[o][k] = sum d2[.,o] h1[.,k]
        const int o = q / H, k = q % H;
        float a = 0.0f;
        for (int r = 0; r < B; ++r) a = fmaf(S.d2[r][o], S.h1[r][k], a);
        atomicAdd(&grad[OFF_W2 + q], a);
    }
    for (int q = t; q < H * IN; q += B) {          // dW1[o][k] = sum d1[.,o] x[.,k]
        const int o = q / IN, k = q % IN;
        float a = 0.0f;
        for (int r = 0; r < B; ++r) a = fmaf(S.d1[r][o], S.x[r][k], a);
        atomicAdd(&grad[OFF_W1 + q], a);
    }
    if (t < H) {                                   // bias gradients
        float a1 = 0.0f, a2 = 0.0f;
        for (int r = 0; r < B; ++r) {
            a1 += S.d1[r][t];
            a2 += S.d2[r][t];
        }
        atomicAdd(&grad[OFF_B1 + t], a1);
        atomicAdd(&grad[OFF_B2 + t], a2);
    }
    // dw3[o] = sum g * silu(z2[o]): z2 was overwritten, recompute from h1
    if (t < H) {
        float a = 0.0f;
        for (int r = 0; r < B; ++r) {
            float z = S.b2[t];
            for (int k = 0; k < H; ++k) z = fmaf(S.w2[t * H + k], S.h1[r][k], z);
            a = fmaf(S.g[r], z * sig(z), a);
        }
        atomicAdd(&grad[OFF_W3 + t], a);
    }
    if (t == 0) {
        float a = 0.0f;
        for (int r = 0; r < B; ++r) a += S.g[r];
        atomicAdd(&grad[OFF_B3], a);
    }
}

__global__ void k_adam(float *p, float *m, float *v, float *grad, float lr,
                       float b1, float b2, float c1, float c2, float eps)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N_PARAM;
         t += gridDim.x * blockDim.x) {
        const float g = grad[t];
        const float mt = b1 * m[t] + (1.0f - b1) * g;
        const float vt = b2 * v[t] + (1.0f - b2) * g * g;
        m[t] = mt;
        v[t] = vt;
        p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
        grad[t] = 0.0f;
    }
}

}  // namespace tg

using namespace tg;

// ===========================================================================
// C-ABI (no counterpart in the reference).  All pointers are DEVICE pointers.
// ===========================================================================

TG_EXPORT int tupan_gb300_mlp_param_count(void) { return N_PARAM; }

// bf16 copies of the weights (w1 64x4, w2 64x64, w3 64) and the rounded
// parameter vector rw (fp32 values actually used by the forward pass).
TG_EXPORT int tupan_gb300_mlp_round(const float *params, void *w1, void *w2,
                                    void *w3, float *rw, void *stream)
{
    k_round_bf16<<<32, 256, 0, (cudaStream_t)stream>>>(
        params, (__nv_bfloat16 *)w1, (__nv_bfloat16 *)w2,
        (__nv_bfloat16 *)w3, rw);
    g_launch_count += 1;
    return cudaGetLastError() == cudaSuccess ? ST_OK : ST_CUDA;
}

// Adds the gradient of scale * sum (y - target)^2 over n samples (X: n x 4
// raw features, Y: n targets) to grad, and the sum of squared errors to
// *loss.  rw: rounded parameters (tupan_gb300_mlp_round); norm: mean[4],
// 1/std[4].
TG_EXPORT int tupan_gb300_mlp_grad(const float *rw, const float *norm,
                                   const float *X, const float *Y, uint64_t n,
                                   float scale, float *grad, float *loss,
                                   void *stream)
{
    if (n == 0) return ST_OK;
    static bool attr = false;
    const size_t smem = sizeof(GradSmem);
    if (!attr) {
        if (cudaFuncSetAttribute(k_mlp_grad,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return ST_CUDA;
        attr = true;
    }
    const unsigned blocks = (unsigned)((n + B - 1) / B);
    k_mlp_grad<<<blocks, B, smem, (cudaStream_t)stream>>>(rw, norm, X, Y, n,
                                                          scale, grad, loss);
    g_launch_count += 1;
    return cudaGetLastError() == cudaSuccess ? ST_OK : ST_CUDA;
}

// One Adam step on the fp32 master parameters; zeroes grad.  step >= 1.
TG_EXPORT int tupan_gb300_mlp_adam(float *params, float *m, float *v,
                                   float *grad, float lr, int step,
                                   void *stream)
{
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)step);
    const float c2 = 1.0f - powf(b2, (float)step);
    k_adam<<<32, 256, 0, (cudaStream_t)stream>>>(params, m, v, grad, lr, b1,
                                                 b2, c1, c2, 1e-8f);
    g_launch_count += 1;
    return cudaGetLastError() == cudaSuccess ? ST_OK : ST_CUDA;
}
