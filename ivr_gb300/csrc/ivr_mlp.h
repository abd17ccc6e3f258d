// ivr_mlp.h -- the learned empty-space predictor's parameter layout and
// kernel entry points.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>

namespace ivr {

// cudaFuncSetAttribute(kernel, MaxDynamicSharedMemorySize, bytes) once per
// device: the attribute belongs to the current device's context, so a flag
// per device (bit dev of done) rather than one per process.
template <typename K>
inline cudaError_t set_dynamic_smem_once(K kernel, int bytes, std::atomic<unsigned long long> &done)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return e;
}

constexpr int kMlpFeatures = 26;  // min, max, 8-bin histogram, 16 TF knots
constexpr int kMlpIn = 32;        // padded input width
constexpr int kMlpHidden = 64;
constexpr int kMlpKnots = 16;

// FP32 master parameters, one flat array: W1[in][hidden] (rows >= 26 are
// padding and stay zero), b1, W2[hidden][hidden], b2, w3, b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpIn * kMlpHidden;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden;
constexpr int kMlpParams = kOffB3 + 1;
// parameters that are not padding: 26*64 + 64 + 64*64 + 64 + 64 + 1 = 5953

// device view of the weights the kernels read
struct MlpDev {
    const void *w1t;  // bf16 [hidden][in]
    const void *w2t;  // bf16 [hidden out][hidden in]
    const void *w2;   // bf16 [hidden in][hidden out]
    const float *b1, *b2, *w3, *b3;
    int *status;      // inference: kMlpTcTimeout when a tensor-core wait ran out (else untouched)
};
constexpr int kMlpTcTimeout = 1;

// inference: y for rows 0..n of X, on the tcgen05 tensor cores (ivr_mlp_tc.cu);
// a wait that runs out records kMlpTcTimeout in *w.status
cudaError_t mlp_forward(const MlpDev &w, const void *X, long long n, float *y, cudaStream_t s);
// forward + backward over rows idx[0..n) (idx null: rows 0..n) on tcgen05,
// gradients added into grad, loss into *loss; targets <= 0 are one-sided
// (gamma) (ivr_mlp_tc.cu)
cudaError_t mlp_train_step(const MlpDev &w, const void *X, const float *T, const int *idx, long long n,
                           long long n_total, float wneg, float gamma, float *grad, float *loss, cudaStream_t s);
// Adam step `step` (1-based) on the FP32 parameters, then the BF16 copies;
// with c12 the step's bias corrections (mlp_adam_corrections) are read from
// device memory instead
cudaError_t mlp_adam(float *p, float *m, float *v, const float *grad, float lr, int step, const float *c12,
                     void *w1t, void *w2t, void *w2, cudaStream_t s);
void mlp_adam_corrections(long long step, float *c1, float *c2);
cudaError_t mlp_pack(const float *p, void *w1t, void *w2t, void *w2, cudaStream_t s);
cudaError_t mlp_cell_hist(const void *data, int dtype, int nx, int ny, int nz, int cell, int mcx, int mcy, int mcz,
                          float vmin, float vmax, float *hist, cudaStream_t s);
cudaError_t mlp_cell_features(const float *mc, const float *hist, int ncell, float vmin, float vmax,
                              const float *knots_dev, const float4 *lut, int lut_n, int lut_off, float lut_scale,
                              void *X, float *targets, cudaStream_t s);
cudaError_t mlp_tf_knots(const float4 *lut, int lut_n, float *knots, cudaStream_t s);
// One brick's learned grid for one TF, in one launch: each cell's features
// (as mlp_cell_features writes them), the network (as mlp_forward runs it)
// and the transparent flag (kDistCap / 0) of y + margin <= 0; with certify
// a cell the exact test (mc, nzprefix, LUT index rule) finds opaque stays
// opaque.  stats (nullable): += cells, exactly transparent, called
// transparent, false skips.  Cells a block could not finish (a tensor-core
// wait ran out: *w.status) are left opaque.
struct MlpGridArgs {
    const float *mc;        // per cell: min, max
    const float *hist;      // per cell: 8 bins
    const float *knots;     // the TF's 16 knots
    int ncell;
    float vmin, vmax, margin;
    const int *nzprefix;    // count of nonzero-opacity LUT entries below each index
    int lut_n, lut_off;
    float lut_scale;
    int certify;
    uint8_t *dist;          // out: kDistCap or 0 per cell
    unsigned long long *stats;
};
cudaError_t mlp_learned_grid_tc(const MlpDev &w, const MlpGridArgs &g, cudaStream_t s);
// *key (initialised to the key of -FLT_MAX) = key of the largest -y over
// rows with T > 0; counts[0] += rows with T <= 0, counts[1] += those with
// y + margin <= 0
cudaError_t mlp_calibrate(const float *y, const float *T, long long n, float margin, int *key,
                          unsigned long long *counts, cudaStream_t s);
float mlp_key_value(int key);
int mlp_key_of(float f);

}  // namespace ivr
