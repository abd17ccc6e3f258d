// ivr_mlp.cu -- the learned empty-space predictor's support kernels: Adam on
// the FP32 parameters and the BF16 operand copies, the per-macrocell
// histograms, features and exact bounds it learns from, the TF knots and
// calibration.  The network itself -- training (forward and backward),
// inference and a TF's learned grid -- runs on the tcgen05 tensor cores
// (ivr_mlp_tc.cu).
#include <cuda_bf16.h>
#include <float.h>
#include <stdint.h>
#include <string.h>

#include "ivr_internal.h"
#include "ivr_mlp.h"

namespace ivr {
namespace {

using bf16 = __nv_bfloat16;
constexpr int F = kMlpIn;      // 32 (26 features, zero padded)
constexpr int H = kMlpHidden;  // 64

// Adam on the FP32 master parameters, then the BF16 operand copies
// c12 (nullable): the bias corrections c1, c2 read from device memory
// instead of the arguments (a launch that a CUDA graph replays every epoch)
__global__ void mlp_adam_kernel(float *p, float *m, float *v, const float *gr, int np, float lr, float beta1,
                                float beta2, float eps, float c1, float c2, const float *c12, bf16 *w1t, bf16 *w2t,
                                bf16 *w2)
{
    if (c12) {
        c1 = c12[0];
        c2 = c12[1];
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        float gi = gr[i];
        if (i >= kOffW1 + kMlpFeatures * H && i < kOffW1 + F * H) gi = 0.0f;  // padding inputs
        const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
        const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void mlp_pack_kernel(const float *p, bf16 *w1t, bf16 *w2t, bf16 *w2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F * H + H * H; i += gridDim.x * blockDim.x) {
        if (i < F * H) {
            const int f = i / H, u = i % H;  // W1[f][u]
            w1t[u * F + f] = __float2bfloat16(p[kOffW1 + i]);
        } else {
            const int j = i - F * H, a = j / H, b = j % H;  // W2[a][b]
            const bf16 v = __float2bfloat16(p[kOffW2 + j]);
            w2[j] = v;
            w2t[b * H + a] = v;
        }
    }
}

// Per-cell 8-bin histogram of a brick's voxels over the volume range
// [vmin, vmax], cells as in the macrocell grid (`cell` voxels plus the +1
// layer).
__global__ void cell_hist_kernel(const void *data, int dtype, int nx, int ny, int nz, int cell, int mcx, int mcy,
                                 float vmin, float vmax, float *hist)
{
    const int cid = blockIdx.x;
    const int cx = cid % mcx, cy = (cid / mcx) % mcy, cz = cid / (mcx * mcy);
    const int x0 = cx * cell, y0 = cy * cell, z0 = cz * cell;
    const int ex = min(x0 + cell, nx - 1) - x0 + 1, ey = min(y0 + cell, ny - 1) - y0 + 1,
              ez = min(z0 + cell, nz - 1) - z0 + 1;
    __shared__ int sh[8];
    if (threadIdx.x < 8) sh[threadIdx.x] = 0;
    __syncthreads();
    const float scale = vmax > vmin ? 8.0f / (vmax - vmin) : 0.0f;
    int local[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int tot = ex * ey * ez;
    for (int q = threadIdx.x; q < tot; q += blockDim.x) {
        const int x = q % ex, r = q / ex, y = r % ey, z = r / ey;
        const long long o = ((long long) (z0 + z) * ny + (y0 + y)) * nx + (x0 + x);
        float v;
        if (dtype == IVR_U8) v = (float) __ldg((const uint8_t *) data + o);
        else if (dtype == IVR_U16) v = (float) __ldg((const uint16_t *) data + o);
        else v = __ldg((const float *) data + o);
        const int b = min(max((int) ((v - vmin) * scale), 0), 7);
        local[b]++;
    }
    for (int b = 0; b < 8; b++)
        if (local[b]) atomicAdd(&sh[b], local[b]);
    __syncthreads();
    if (threadIdx.x < 8) hist[cid * 8 + threadIdx.x] = (float) sh[threadIdx.x] / (float) tot;
}

// Features of every cell of a brick for one TF (bf16 rows of kMlpIn) and, if
// targets != null, the exact post-TF maximum opacity of the cell: the largest
// LUT opacity among the entries its samples can index (the index range of
// the exact empty-cell test, so a bound of 0 is exactly a transparent cell).
__global__ void cell_features_kernel(const float *mc, const float *hist, int ncell, float vmin, float vmax,
                                     const float *knots, const float4 *lut, int lut_n, int lut_off, float lut_scale,
                                     bf16 *X, float *targets)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        const float lo = mc[2 * c], hi = mc[2 * c + 1];
        const float inv = vmax > vmin ? 1.0f / (vmax - vmin) : 0.0f;
        bf16 *x = X + (long long) c * kMlpIn;
        x[0] = __float2bfloat16((lo - vmin) * inv);
        x[1] = __float2bfloat16((hi - vmin) * inv);
        for (int b = 0; b < 8; b++) x[2 + b] = __float2bfloat16(hist[c * 8 + b]);
        for (int k = 0; k < 16; k++) x[10 + k] = __float2bfloat16(knots[k]);
        for (int k = kMlpFeatures; k < kMlpIn; k++) x[k] = __float2bfloat16(0.0f);
        if (targets) {
            int a = min(max((int) (lo * lut_scale) - 1 - lut_off, 0), lut_n - 1);
            int b = min(max((int) (hi * lut_scale) + 1 - lut_off, 0), lut_n - 1);
            float m = 0.0f;
            for (int i = a; i <= b; i++) m = fmaxf(m, lut[i].w);
            targets[c] = m;
        }
    }
}

// The TF's 16-knot encoding, on 16 knots evenly spaced over the LUT's
// entries (entry k (n-1)/15, the knots of a piecewise-linear TF of 16
// knots): feature k < 15 is the largest opacity between knots k and k + 1,
// both included, and feature 15 the largest opacity of the whole LUT.  A
// cell is transparent when every interval its index range overlaps is zero,
// which the network can read off these and the cell's min and max.  One
// warp per feature.
__global__ void tf_knots_kernel(const float4 *lut, int lut_n, float *knots)
{
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= kMlpKnots) return;
    const int last = kMlpKnots - 1;
    const int a = k < last ? k * (lut_n - 1) / last : 0;
    const int b = k < last ? ((k + 1) * (lut_n - 1) + last - 1) / last : lut_n - 1;
    float m = 0.0f;
    for (int i = a + lane; i <= b; i += 32) m = fmaxf(m, lut[i].w);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) knots[k] = m;
}

// order-preserving float <-> int keys for atomicMax
__device__ __forceinline__ int float_key(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

// calibration: out_key = max over rows with T > 0 of key(-y); counts[0] =
// rows with T <= 0; counts[1] = those with y + margin <= 0
__global__ void calibrate_kernel(const float *y, const float *T, long long n, float margin, int *out_key,
                                 unsigned long long *counts)
{
    int key = float_key(-FLT_MAX);
    unsigned long long zeros = 0, skipped = 0;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        if (T[i] > 0.0f) {
            key = max(key, float_key(-y[i]));
        } else {
            zeros++;
            skipped += y[i] + margin <= 0.0f;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        key = max(key, __shfl_xor_sync(0xffffffffu, key, o));
        zeros += __shfl_xor_sync(0xffffffffu, zeros, o);
        skipped += __shfl_xor_sync(0xffffffffu, skipped, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out_key, key);
        atomicAdd(counts, zeros);
        atomicAdd(counts + 1, skipped);
    }
}

int grid_of(long long n, int threads)
{
    long long g = (n + threads - 1) / threads;
    return (int) (g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

}  // namespace

void mlp_adam_corrections(long long step, float *c1, float *c2)
{
    *c1 = 1.0f - powf(0.9f, (float) step);
    *c2 = 1.0f - powf(0.999f, (float) step);
}

cudaError_t mlp_adam(float *p, float *m, float *v, const float *grad, float lr, int step, const float *c12,
                     void *w1t, void *w2t, void *w2, cudaStream_t s)
{
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.0f, c2 = 1.0f;
    if (!c12) mlp_adam_corrections(step, &c1, &c2);
    mlp_adam_kernel<<<grid_of(kMlpParams, 256), 256, 0, s>>>(p, m, v, grad, kMlpParams, lr, b1, b2, 1e-8f, c1, c2,
                                                             c12, (bf16 *) w1t, (bf16 *) w2t, (bf16 *) w2);
    mlp_pack_kernel<<<grid_of(F * H + H * H, 256), 256, 0, s>>>(p, (bf16 *) w1t, (bf16 *) w2t, (bf16 *) w2);
    return cudaGetLastError();
}

cudaError_t mlp_pack(const float *p, void *w1t, void *w2t, void *w2, cudaStream_t s)
{
    mlp_pack_kernel<<<grid_of(F * H + H * H, 256), 256, 0, s>>>(p, (bf16 *) w1t, (bf16 *) w2t, (bf16 *) w2);
    return cudaGetLastError();
}

cudaError_t mlp_cell_hist(const void *data, int dtype, int nx, int ny, int nz, int cell, int mcx, int mcy, int mcz,
                          float vmin, float vmax, float *hist, cudaStream_t s)
{
    cell_hist_kernel<<<mcx * mcy * mcz, 128, 0, s>>>(data, dtype, nx, ny, nz, cell, mcx, mcy, vmin, vmax, hist);
    return cudaGetLastError();
}

cudaError_t mlp_cell_features(const float *mc, const float *hist, int ncell, float vmin, float vmax,
                              const float *knots_dev, const float4 *lut, int lut_n, int lut_off, float lut_scale,
                              void *X, float *targets, cudaStream_t s)
{
    cell_features_kernel<<<grid_of(ncell, 128), 128, 0, s>>>(mc, hist, ncell, vmin, vmax, knots_dev, lut, lut_n,
                                                             lut_off, lut_scale, (bf16 *) X, targets);
    return cudaGetLastError();
}

cudaError_t mlp_tf_knots(const float4 *lut, int lut_n, float *knots, cudaStream_t s)
{
    tf_knots_kernel<<<1, 32 * kMlpKnots, 0, s>>>(lut, lut_n, knots);
    return cudaGetLastError();
}

cudaError_t mlp_calibrate(const float *y, const float *T, long long n, float margin, int *key,
                          unsigned long long *counts, cudaStream_t s)
{
    calibrate_kernel<<<grid_of(n, 256), 256, 0, s>>>(y, T, n, margin, key, counts);
    return cudaGetLastError();
}

int mlp_key_of(float f)
{
    int i;
    memcpy(&i, &f, sizeof(i));
    return i >= 0 ? i : i ^ 0x7fffffff;
}

float mlp_key_value(int key)
{
    const int i = key >= 0 ? key : key ^ 0x7fffffff;
    float f;
    memcpy(&f, &i, sizeof(f));
    return f;
}

}  // namespace ivr
