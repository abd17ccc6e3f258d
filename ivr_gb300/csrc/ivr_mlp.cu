// ivr_mlp.cu -- the learned empty-space predictor: a 26 -> 64 -> 64 -> 1 MLP
// (BF16 weights and activations, FP32 accumulation) on the tensor cores with
// mma.sync.m16n8k16 for its training step (forward + backward in one kernel
// per 128-row tile, weight gradients accumulated in FP32), Adam, and the
// per-macrocell features and targets it learns from.  Inference runs on the
// tcgen05 tensor cores (ivr_mlp_tc.cu).
//
// Fragment layouts of mma.m16n8k16 (row.col, bf16 -> f32), per lane with
// g = lane / 4 and t = lane % 4:
//   A (16x16, row-major):  a0 = A[g][2t..2t+1],   a1 = A[g+8][2t..2t+1],
//                          a2 = A[g][2t+8..+9],   a3 = A[g+8][2t+8..+9]
//   B (16x8, stored n-major as Bt[n][k]): b0 = Bt[g][2t..2t+1], b1 = Bt[g][2t+8..+9]
//   C (16x8, f32):         c0 = C[g][2t], c1 = C[g][2t+1], c2 = C[g+8][2t], c3 = C[g+8][2t+1]
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
constexpr int R = 128;         // rows per block (4 warps x 32)
constexpr int LDX = F + 8;     // padded row strides (bank-conflict free fragment loads)
constexpr int LDH = H + 8;
constexpr int LDR = R + 8;

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

__device__ __forceinline__ void load_a(uint32_t (&a)[4], const bf16 *A, int ld, int row0, int k0)
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    a[0] = ld32(A + (row0 + g) * ld + k0 + 2 * t);
    a[1] = ld32(A + (row0 + g + 8) * ld + k0 + 2 * t);
    a[2] = ld32(A + (row0 + g) * ld + k0 + 2 * t + 8);
    a[3] = ld32(A + (row0 + g + 8) * ld + k0 + 2 * t + 8);
}

__device__ __forceinline__ void load_b(uint32_t (&b)[2], const bf16 *Bt, int ld, int n0, int k0)
{
    const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    b[0] = ld32(Bt + (n0 + g) * ld + k0 + 2 * t);
    b[1] = ld32(Bt + (n0 + g) * ld + k0 + 2 * t + 8);
}

// shared layout of the forward pass
struct FwdSmem {
    bf16 X[R * LDX];
    bf16 H1[R * LDH];
    bf16 W1t[H * LDX];  // [out][in]
    bf16 W2t[H * LDH];  // [out][in]
    float b1[H], b2[H], w3[H];
};
// extra for the backward pass
struct BwdSmem {
    FwdSmem f;
    bf16 Xt[F * LDR];   // [feature][row]
    bf16 H1t[H * LDR];  // [unit][row]
    bf16 D2[R * LDH];   // dL/dh2 [row][unit]
    bf16 D2t[H * LDR];  // [unit][row]
    bf16 D1t[H * LDR];  // dL/dh1 [unit][row]
    bf16 W2[H * LDH];   // [in][out]
    float red[8];
};

// loads the weights and the block's rows into shared memory
template <bool TRANSPOSED>
__device__ void load_tile(FwdSmem &s, bf16 *Xt, const MlpDev &w, const bf16 *X, const int *idx, long long row0,
                          long long n)
{
    const bf16 *w1t = (const bf16 *) w.w1t, *w2t = (const bf16 *) w.w2t;
    for (int i = threadIdx.x; i < H * F; i += blockDim.x) s.W1t[(i / F) * LDX + i % F] = w1t[i];
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) s.W2t[(i / H) * LDH + i % H] = w2t[i];
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        s.b1[i] = w.b1[i];
        s.b2[i] = w.b2[i];
        s.w3[i] = w.w3[i];
    }
    for (int i = threadIdx.x; i < R * F; i += blockDim.x) {
        const int r = i / F, c = i % F;
        bf16 v = __float2bfloat16(0.0f);
        if (row0 + r < n) v = X[(idx ? (long long) idx[row0 + r] : row0 + r) * F + c];
        s.X[r * LDX + c] = v;
        if (TRANSPOSED) Xt[c * LDR + r] = v;
    }
}

// layer 1 (X W1 + b1, relu) and layer 2 (H1 W2 + b2, relu) for the warp's 32
// rows; h2 stays in registers in C-fragment layout, H1 goes to shared memory
template <bool TRANSPOSED>
__device__ void forward_rows(FwdSmem &s, bf16 *H1t, float (&h2)[2][8][4])
{
    const int warp = threadIdx.x >> 5, g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
    const int rbase = warp * 32;
    {
        float acc[2][8][4] = {};
        for (int mt = 0; mt < 2; mt++)
            for (int ks = 0; ks < F / 16; ks++) {
                uint32_t a[4];
                load_a(a, s.X, LDX, rbase + 16 * mt, 16 * ks);
                for (int nt = 0; nt < 8; nt++) {
                    uint32_t b[2];
                    load_b(b, s.W1t, LDX, 8 * nt, 16 * ks);
                    mma16816(acc[mt][nt], a, b);
                }
            }
        for (int mt = 0; mt < 2; mt++)
            for (int nt = 0; nt < 8; nt++)
                for (int c = 0; c < 4; c++) {
                    const int row = rbase + 16 * mt + g + (c >> 1) * 8, col = 8 * nt + 2 * t + (c & 1);
                    const bf16 v = __float2bfloat16(fmaxf(acc[mt][nt][c] + s.b1[col], 0.0f));
                    s.H1[row * LDH + col] = v;
                    if (TRANSPOSED) H1t[col * LDR + row] = v;
                }
    }
    __syncwarp();
    for (int mt = 0; mt < 2; mt++)
        for (int nt = 0; nt < 8; nt++)
            for (int c = 0; c < 4; c++) h2[mt][nt][c] = 0.0f;
    for (int mt = 0; mt < 2; mt++)
        for (int ks = 0; ks < H / 16; ks++) {
            uint32_t a[4];
            load_a(a, s.H1, LDH, rbase + 16 * mt, 16 * ks);
            for (int nt = 0; nt < 8; nt++) {
                uint32_t b[2];
                load_b(b, s.W2t, LDH, 8 * nt, 16 * ks);
                mma16816(h2[mt][nt], a, b);
            }
        }
    for (int mt = 0; mt < 2; mt++)
        for (int nt = 0; nt < 8; nt++)
            for (int c = 0; c < 4; c++) {
                const int col = 8 * nt + 2 * t + (c & 1);
                h2[mt][nt][c] = fmaxf(h2[mt][nt][c] + s.b2[col], 0.0f);
            }
}

// layer 3: y for rows (g, g+8) of each m-tile, summed over the group's 4 lanes
__device__ void output_rows(const FwdSmem &s, const float (&h2)[2][8][4], float b3, float (&y)[2][2])
{
    const int t = threadIdx.x & 3;
    for (int mt = 0; mt < 2; mt++)
        for (int hi = 0; hi < 2; hi++) {
            float p = 0.0f;
            for (int nt = 0; nt < 8; nt++)
                for (int c = 0; c < 2; c++) p = fmaf(h2[mt][nt][hi * 2 + c], s.w3[8 * nt + 2 * t + c], p);
            p += __shfl_xor_sync(0xffffffffu, p, 1);
            p += __shfl_xor_sync(0xffffffffu, p, 2);
            y[mt][hi] = p + b3;
        }
}

// Forward and backward of one 128-row tile of rows idx[0..n) (or 0..n).
// Per row, with bound T: T > 0 costs wt * (y - T)^2, wt = wneg when y < T
// and 1 otherwise; T <= 0 (a transparent cell) costs max(y + gamma, 0)^2.
// Loss = sum / n_total.  Gradients are added into grad (FP32).
__global__ void __launch_bounds__(R) mlp_train_kernel(MlpDev w, const bf16 *X, const float *T, const int *idx,
                                                      long long n, long long n_total, float wneg, float gamma,
                                                      float *grad, float *loss)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BwdSmem &s = *reinterpret_cast<BwdSmem *>(smem_raw);
    const long long row0 = (long long) blockIdx.x * R;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int rbase = warp * 32;
    load_tile<true>(s.f, s.Xt, w, X, idx, row0, n);
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) s.W2[(i / H) * LDH + i % H] = ((const bf16 *) w.w2)[i];
    __syncthreads();
    float h2[2][8][4];
    forward_rows<true>(s.f, s.H1t, h2);
    float y[2][2];
    output_rows(s.f, h2, *w.b3, y);

    // dL/dy, loss, and the layer-3 gradients
    float dy[2][2], lsum = 0.0f, db3 = 0.0f;
    for (int mt = 0; mt < 2; mt++)
        for (int hi = 0; hi < 2; hi++) {
            const long long row = row0 + rbase + 16 * mt + g + 8 * hi;
            float d = 0.0f;
            if (row < n) {
                const float tv = T[idx ? (long long) idx[row] : row];
                float r, wt = 1.0f;
                if (tv > 0.0f) {
                    r = y[mt][hi] - tv;
                    if (r < 0.0f) wt = wneg;
                } else {
                    r = fmaxf(y[mt][hi] + gamma, 0.0f);
                }
                if (t == 0) lsum += wt * r * r / (float) n_total;
                d = 2.0f * wt * r / (float) n_total;
            }
            dy[mt][hi] = d;
            if (t == 0) db3 += d;
        }
    float *gW1 = grad + kOffW1, *gb1 = grad + kOffB1, *gW2 = grad + kOffW2, *gb2 = grad + kOffB2,
          *gw3 = grad + kOffW3, *gb3 = grad + kOffB3;
    // dw3[col] = sum_rows dy * h2 ; dh2 = dy * w3 * relu'(h2) ; db2 = sum dh2
    for (int nt = 0; nt < 8; nt++)
        for (int c = 0; c < 2; c++) {
            const int col = 8 * nt + 2 * t + c;
            float pw = 0.0f, pb = 0.0f;
            for (int mt = 0; mt < 2; mt++)
                for (int hi = 0; hi < 2; hi++) {
                    const float hv = h2[mt][nt][hi * 2 + c];
                    pw = fmaf(dy[mt][hi], hv, pw);
                    const float d2 = hv > 0.0f ? dy[mt][hi] * s.f.w3[col] : 0.0f;
                    pb += d2;
                    const int row = rbase + 16 * mt + g + 8 * hi;
                    const bf16 b = __float2bfloat16(d2);
                    s.D2[row * LDH + col] = b;
                    s.D2t[col * LDR + row] = b;
                }
            // sum over the 8 groups of the warp (lanes with equal t)
            for (int o = 4; o < 32; o <<= 1) {
                pw += __shfl_xor_sync(0xffffffffu, pw, o);
                pb += __shfl_xor_sync(0xffffffffu, pb, o);
            }
            if (g == 0) {
                atomicAdd(gw3 + col, pw);
                atomicAdd(gb2 + col, pb);
            }
        }
    for (int o = 1; o < 32; o <<= 1) {
        lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        db3 += __shfl_xor_sync(0xffffffffu, db3, o);
    }
    if (lane == 0) {
        atomicAdd(gb3, db3);
        atomicAdd(loss, lsum);
    }
    __syncthreads();

    // dW2[i][o] = sum_r H1t[i][r] D2t[o][r]: warp w owns rows i in [16w, 16w+16)
    {
        float acc[8][4] = {};
        for (int ks = 0; ks < R / 16; ks++) {
            uint32_t a[4];
            load_a(a, s.H1t, LDR, 16 * warp, 16 * ks);
            for (int nt = 0; nt < 8; nt++) {
                uint32_t b[2];
                load_b(b, s.D2t, LDR, 8 * nt, 16 * ks);
                mma16816(acc[nt], a, b);
            }
        }
        for (int nt = 0; nt < 8; nt++)
            for (int c = 0; c < 4; c++)
                atomicAdd(gW2 + (16 * warp + g + (c >> 1) * 8) * H + 8 * nt + 2 * t + (c & 1), acc[nt][c]);
    }
    // dh1[r][i] = sum_o D2[r][o] W2[i][o] * relu'(h1)
    {
        float acc[2][8][4] = {};
        for (int mt = 0; mt < 2; mt++)
            for (int ks = 0; ks < H / 16; ks++) {
                uint32_t a[4];
                load_a(a, s.D2, LDH, rbase + 16 * mt, 16 * ks);
                for (int nt = 0; nt < 8; nt++) {
                    uint32_t b[2];
                    load_b(b, s.W2, LDH, 8 * nt, 16 * ks);
                    mma16816(acc[mt][nt], a, b);
                }
            }
        for (int nt = 0; nt < 8; nt++)
            for (int c2 = 0; c2 < 2; c2++) {
                const int col = 8 * nt + 2 * t + c2;
                float pb = 0.0f;
                for (int mt = 0; mt < 2; mt++)
                    for (int hi = 0; hi < 2; hi++) {
                        const int row = rbase + 16 * mt + g + 8 * hi;
                        const float h1 = __bfloat162float(s.f.H1[row * LDH + col]);
                        const float d1 = h1 > 0.0f ? acc[mt][nt][hi * 2 + c2] : 0.0f;
                        pb += d1;
                        s.D1t[col * LDR + row] = __float2bfloat16(d1);
                    }
                for (int o = 4; o < 32; o <<= 1) pb += __shfl_xor_sync(0xffffffffu, pb, o);
                if (g == 0) atomicAdd(gb1 + col, pb);
            }
    }
    __syncthreads();
    // dW1[f][i] = sum_r Xt[f][r] D1t[i][r]: warp w owns columns i in [16w, 16w+16)
    {
        float acc[2][2][4] = {};
        for (int ks = 0; ks < R / 16; ks++)
            for (int mt = 0; mt < 2; mt++) {
                uint32_t a[4];
                load_a(a, s.Xt, LDR, 16 * mt, 16 * ks);
                for (int j = 0; j < 2; j++) {
                    uint32_t b[2];
                    load_b(b, s.D1t, LDR, 8 * (2 * warp + j), 16 * ks);
                    mma16816(acc[mt][j], a, b);
                }
            }
        for (int mt = 0; mt < 2; mt++)
            for (int j = 0; j < 2; j++)
                for (int c = 0; c < 4; c++)
                    atomicAdd(gW1 + (16 * mt + g + (c >> 1) * 8) * H + 8 * (2 * warp + j) + 2 * t + (c & 1),
                              acc[mt][j][c]);
    }
}

// Adam on the FP32 master parameters, then the BF16 operand copies
__global__ void mlp_adam_kernel(float *p, float *m, float *v, const float *gr, int np, float lr, float beta1,
                                float beta2, float eps, float c1, float c2, bf16 *w1t, bf16 *w2t, bf16 *w2)
{
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

// The TF's 16-knot encoding: knot k is the largest LUT opacity over the
// entries that values in the k-th sixteenth of [vmin, vmax] index (the same
// index rule as the bounds).  One warp per knot.
__global__ void tf_knots_kernel(const float4 *lut, int lut_n, int lut_off, float lut_scale, float vmin, float vmax,
                                float *knots)
{
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= kMlpKnots) return;
    const float r = vmax - vmin;
    const float lo = vmin + r * (float) k / (float) kMlpKnots, hi = vmin + r * (float) (k + 1) / (float) kMlpKnots;
    const int a = min(max((int) (lo * lut_scale) - 1 - lut_off, 0), lut_n - 1);
    const int b = min(max((int) (hi * lut_scale) + 1 - lut_off, 0), lut_n - 1);
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

size_t mlp_forward_smem() { return sizeof(FwdSmem); }
size_t mlp_train_smem() { return sizeof(BwdSmem); }

cudaError_t mlp_forward(const MlpDev &w, const void *X, long long n, float *y, cudaStream_t s)
{
    return mlp_forward_tc(w, X, n, y, w.status, s);
}

cudaError_t mlp_train_step(const MlpDev &w, const void *X, const float *T, const int *idx, long long n,
                           long long n_total, float wneg, float gamma, float *grad, float *loss, cudaStream_t s)
{
    static std::atomic<unsigned long long> attr{0};
    cudaError_t e = set_dynamic_smem_once(mlp_train_kernel, (int) sizeof(BwdSmem), attr);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    mlp_train_kernel<<<(unsigned) ((n + R - 1) / R), R, sizeof(BwdSmem), s>>>(w, (const bf16 *) X, T, idx, n,
                                                                              n_total, wneg, gamma, grad, loss);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float *p, float *m, float *v, const float *grad, float lr, int step, void *w1t, void *w2t,
                     void *w2, cudaStream_t s)
{
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float) step), c2 = 1.0f - powf(b2, (float) step);
    mlp_adam_kernel<<<grid_of(kMlpParams, 256), 256, 0, s>>>(p, m, v, grad, kMlpParams, lr, b1, b2, 1e-8f, c1, c2,
                                                             (bf16 *) w1t, (bf16 *) w2t, (bf16 *) w2);
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

cudaError_t mlp_tf_knots(const float4 *lut, int lut_n, int lut_off, float lut_scale, float vmin, float vmax,
                         float *knots, cudaStream_t s)
{
    tf_knots_kernel<<<1, 32 * kMlpKnots, 0, s>>>(lut, lut_n, lut_off, lut_scale, vmin, vmax, knots);
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
