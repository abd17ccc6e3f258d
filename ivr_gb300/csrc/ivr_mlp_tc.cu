// ivr_mlp_tc.cu -- the learned empty-space predictor on the 5th-generation
// tensor cores (tcgen05): inference, a TF's learned grid, and the training
// step (forward and backward).  Inference: a 128-row tile of features X
// [128 x 32] times W1 [32 x 64] and the hidden layer H1 [128 x 64] times W2
// [64 x 64], BF16 operands in shared memory, FP32 accumulators in tensor
// memory (TMEM), one elected thread issuing the MMAs, an mbarrier signalled
// by tcgen05.commit, and the epilogues (bias, ReLU, the last layer's dot
// product) on the accumulators read back with tcgen05.ld: TMEM lane r holds
// tile row r, so every thread finishes its own row.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, the K-adjacent ones 128 bytes apart (the
// descriptor's leading byte offset) and the row-adjacent ones SBO bytes
// apart (the stride byte offset: K/8 core matrices of 128 bytes).  Element
// (r, k) of such a tile lies at (r/8)*SBO + (k/8)*128 + (r%8)*16 + (k%8)*2.
//
// Every wait is bounded; a wait that runs out records kMlpTcTimeout in
// *status, waits (bounded) for the MMAs in flight, frees the tile's TMEM and
// leaves the rows (or the tile's gradients) unwritten; the caller turns the
// status into an error.
#include <cuda_bf16.h>
#include <stdint.h>

#include "ivr_internal.h"
#include "ivr_mlp.h"

namespace ivr {
namespace {

using bf16 = __nv_bfloat16;
constexpr int kIn = kMlpIn;       // 32
constexpr int kHid = kMlpHidden;  // 64
constexpr int kRows = 128;        // M of one MMA tile, one row per thread
constexpr int kSbo1 = (kIn / 8) * 128;   // 512: X and W1 tiles (K = 32)
constexpr int kSbo2 = (kHid / 8) * 128;  // 1024: H1 and W2 tiles (K = 64)
constexpr uint32_t kTmemCols = 128;      // D1 in columns 0-63, D2 in 64-127
constexpr long long kWaitLimit = 1ll << 24;

struct TcSmem {
    alignas(128) unsigned char x[kRows * kIn * 2];   // 8 KB, A of layer 1
    alignas(128) unsigned char w1[kHid * kIn * 2];   // 4 KB, B of layer 1 (W1t: n x k)
    alignas(128) unsigned char h1[kRows * kHid * 2]; // 16 KB, A of layer 2
    alignas(128) unsigned char w2[kHid * kHid * 2];  // 8 KB, B of layer 2 (W2t: n x k)
    float b1[kHid], b2[kHid], w3[kHid];
    unsigned long long mbar;
    uint32_t tmem;
};
// dynamic shared memory asked per block: above TcSmem, so that at most four
// blocks share an SM and their 4 x 128 TMEM columns fit its 512
constexpr size_t kTcSmemBytes = 56 * 1024;
static_assert(sizeof(TcSmem) <= kTcSmemBytes, "smem");

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

__device__ __forceinline__ int kmajor_off(int r, int k, int sbo) { return (r >> 3) * sbo + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2; }

// shared-memory matrix descriptor: start, leading byte offset (K-adjacent
// core matrices), stride byte offset (row-adjacent), descriptor version 1,
// no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t) ((saddr >> 4) & 0x3fffu) | ((uint64_t) ((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t) ((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (n >> 3) << 17) | ((uint32_t) (m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// bounded wait for phase `parity` of the mbarrier; false when it ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    for (long long it = 0; it < kWaitLimit; it++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// A ROWS x K BF16 matrix, row-major in global memory, into a canonical
// K-major tile: 16-byte chunks (8 elements of a row), all of a thread's
// loads issued before its stores (the trip count is a constant).
template <int ROWS, int K>
__device__ __forceinline__ void stage_kmajor(unsigned char *dst, const void *src, int sbo)
{
    constexpr int kChunks = ROWS * (K / 8), kPer = kChunks / kRows;
    static_assert(kChunks % kRows == 0, "whole chunks per thread");
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; j++) v[j] = __ldg(s4 + threadIdx.x + j * kRows);
#pragma unroll
    for (int j = 0; j < kPer; j++) {
        const int i = threadIdx.x + j * kRows;
        *reinterpret_cast<uint4 *>(dst + kmajor_off(i / (K / 8), 8 * (i % (K / 8)), sbo)) = v[j];
    }
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    const bf16 lo = __float2bfloat16(a), hi = __float2bfloat16(b);
    return (uint32_t) __bfloat16_as_ushort(lo) | ((uint32_t) __bfloat16_as_ushort(hi) << 16);
}

// GRID: the rows are the cells of g (features built here, flags written
// instead of y); otherwise rows of X in, y out.
template <bool GRID>
__global__ void __launch_bounds__(kRows) mlp_tc_kernel(MlpDev w, const bf16 *X, long long n, float *y, int *status,
                                                        MlpGridArgs g)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem &s = *reinterpret_cast<TcSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights and biases, once per block, in the operand layouts
    const bf16 *w1t = (const bf16 *) w.w1t, *w2t = (const bf16 *) w.w2t;
    stage_kmajor<kHid, kIn>(s.w1, w1t, kSbo1);
    stage_kmajor<kHid, kHid>(s.w2, w2t, kSbo2);
    for (int i = tid; i < kHid; i += kRows) {
        s.b1[i] = w.b1[i];
        s.b2[i] = w.b2[i];
        s.w3[i] = w.w3[i];
    }
    const uint32_t mbar = smem_addr(&s.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s.tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t lane_addr = tmem + ((uint32_t) (warp * 32) << 16);  // this warp's 32 TMEM lanes
    const float b3 = *w.b3;
    constexpr uint32_t idesc = idesc_bf16(kRows, kHid);
    const uint32_t sx = smem_addr(s.x), sw1 = smem_addr(s.w1), sh1 = smem_addr(s.h1), sw2 = smem_addr(s.w2);
    uint32_t phase = 0;
    bool ok = true;
    const long long ntiles = (n + kRows - 1) / kRows;
    // GRID: the TF's knots (the same for every cell) and the cell counts
    float knot[kMlpKnots];
    if (GRID)
#pragma unroll
        for (int k = 0; k < kMlpKnots; k++) knot[k] = g.knots[k];
    const float inv = g.vmax > g.vmin ? 1.0f / (g.vmax - g.vmin) : 0.0f;
    unsigned ncells = 0, nexact = 0, nlearned = 0, nfalse = 0;
    long long tile = blockIdx.x;
    for (; tile < ntiles && ok; tile += gridDim.x) {
        const long long row = tile * kRows + tid;
        // this thread's feature row, 4 x 16 bytes, zero past n
        uint4 xr[4] = {};
        float lo = 0.0f, hi = 0.0f;
        if (row < n) {
            if (GRID) {
                // the row mlp_cell_features writes: min and max normalised, 8 bins,
                // 16 knots, zero padding
                lo = g.mc[2 * row];
                hi = g.mc[2 * row + 1];
                const float4 h0 = reinterpret_cast<const float4 *>(g.hist + row * 8)[0];
                const float4 h1 = reinterpret_cast<const float4 *>(g.hist + row * 8)[1];
                xr[0] = make_uint4(pack2((lo - g.vmin) * inv, (hi - g.vmin) * inv), pack2(h0.x, h0.y),
                                   pack2(h0.z, h0.w), pack2(h1.x, h1.y));
                xr[1] = make_uint4(pack2(h1.z, h1.w), pack2(knot[0], knot[1]), pack2(knot[2], knot[3]),
                                   pack2(knot[4], knot[5]));
                xr[2] = make_uint4(pack2(knot[6], knot[7]), pack2(knot[8], knot[9]), pack2(knot[10], knot[11]),
                                   pack2(knot[12], knot[13]));
                xr[3] = make_uint4(pack2(knot[14], knot[15]), 0u, 0u, 0u);
            } else {
                const uint4 *src = reinterpret_cast<const uint4 *>(X + row * kIn);
#pragma unroll
                for (int q = 0; q < 4; q++) xr[q] = src[q];
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) *reinterpret_cast<uint4 *>(s.x + kmajor_off(tid, 8 * q, kSbo1)) = xr[q];
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // layer 1: D1 = X W1 (K = 32: two MMAs of K = 16)
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kIn / 16; ks++)
                mma_bf16(tmem, sdesc(sx + ks * 256, 128, kSbo1), sdesc(sw1 + ks * 256, 128, kSbo1), idesc, ks);
            mma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        fence_after();
        // epilogue 1: H1 = bf16(relu(D1 + b1)), row tid, into layer 2's A
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float d[16];
            tmem_ld16(lane_addr + (uint32_t) c0, d);
#pragma unroll
            for (int half = 0; half < 2; half++) {
                uint4 v;
                const int c = c0 + 8 * half;
                v.x = pack2(fmaxf(d[8 * half + 0] + s.b1[c + 0], 0.0f), fmaxf(d[8 * half + 1] + s.b1[c + 1], 0.0f));
                v.y = pack2(fmaxf(d[8 * half + 2] + s.b1[c + 2], 0.0f), fmaxf(d[8 * half + 3] + s.b1[c + 3], 0.0f));
                v.z = pack2(fmaxf(d[8 * half + 4] + s.b1[c + 4], 0.0f), fmaxf(d[8 * half + 5] + s.b1[c + 5], 0.0f));
                v.w = pack2(fmaxf(d[8 * half + 6] + s.b1[c + 6], 0.0f), fmaxf(d[8 * half + 7] + s.b1[c + 7], 0.0f));
                *reinterpret_cast<uint4 *>(s.h1 + kmajor_off(tid, c, kSbo2)) = v;
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // layer 2: D2 = H1 W2 (K = 64: four MMAs), columns 64-127
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ks++)
                mma_bf16(tmem + kHid, sdesc(sh1 + ks * 256, 128, kSbo2), sdesc(sw2 + ks * 256, 128, kSbo2), idesc,
                         ks);
            mma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        fence_after();
        // epilogue 2: y = relu(D2 + b2) . w3 + b3
        float acc = 0.0f;
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float d[16];
            tmem_ld16(lane_addr + (uint32_t) (kHid + c0), d);
#pragma unroll
            for (int i = 0; i < 16; i++) acc = fmaf(fmaxf(d[i] + s.b2[c0 + i], 0.0f), s.w3[c0 + i], acc);
        }
        if (row < n) {
            const float yv = acc + b3;
            if (GRID) {
                // learned transparency, certified by the exact empty-cell test
                const bool learned = yv + g.margin <= 0.0f;
                const int a = min(max((int) (lo * g.lut_scale) - 1 - g.lut_off, 0), g.lut_n - 1);
                const int b = min(max((int) (hi * g.lut_scale) + 1 - g.lut_off, 0), g.lut_n - 1);
                const bool exact = (g.nzprefix[b + 1] - g.nzprefix[a]) == 0;
                g.dist[row] = (learned && (exact || !g.certify)) ? (uint8_t) kDistCap : 0;
                ncells++;
                nexact += exact;
                nlearned += learned;
                nfalse += learned && !exact;
            } else {
                y[row] = yv;
            }
        }
        fence_before();
        __syncthreads();  // s.x, s.h1 and the accumulators are rewritten by the next tile
        fence_after();
    }
    if (!ok) {
        if (tid == 0 && status) atomicExch(status, kMlpTcTimeout);
        mbar_wait(mbar, phase);  // the MMAs in flight, if any (bounded)
        if (GRID)  // the cells this block did not finish stay opaque
            for (; tile < ntiles; tile += gridDim.x) {
                const long long row = tile * kRows + tid;
                if (row < n) g.dist[row] = 0;
            }
    }
    if (GRID && g.stats) {
        for (int o = 16; o > 0; o >>= 1) {
            ncells += __shfl_xor_sync(0xffffffffu, ncells, o);
            nexact += __shfl_xor_sync(0xffffffffu, nexact, o);
            nlearned += __shfl_xor_sync(0xffffffffu, nlearned, o);
            nfalse += __shfl_xor_sync(0xffffffffu, nfalse, o);
        }
        if ((tid & 31) == 0 && ncells) {
            atomicAdd(g.stats, (unsigned long long) ncells);
            atomicAdd(g.stats + 1, (unsigned long long) nexact);
            atomicAdd(g.stats + 2, (unsigned long long) nlearned);
            if (nfalse) atomicAdd(g.stats + 3, (unsigned long long) nfalse);
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---------------------------------------------------------------------------
// Training: forward and backward of one 128-row tile on tcgen05.  Thread t
// owns row t (its TMEM lane); the weight gradients are GEMMs over the rows,
// dW2 = H1^T D2 and dW1 = X^T D1, computed with the rows as K (the
// transposed operands written into K-major tiles of their own, the unused
// rows of the 128-row A tiles zero), and dH1 = D2 W2^T with the hidden units
// as K.  TMEM columns: D1 (then dH1) 0-63, D2 64-127, dW2 128-191,
// dW1 192-255.  Loss and rounding points follow the mma.sync kernel's: BF16
// operands (X, W, H1, D2, D1), FP32 accumulation, FP32 h2 and biases.
constexpr int kSboR = (kRows / 8) * 128;  // 2048: tiles whose K is the 128 rows
constexpr uint32_t kTrainCols = 256;
constexpr uint32_t kColD1 = 0, kColD2 = 64, kColG2 = 128, kColG1 = 192;

struct TrainSmem {
    alignas(128) unsigned char x[kRows * kIn * 2];      // A of D1: rows x features
    alignas(128) unsigned char w1[kHid * kIn * 2];      // B of D1: W1t, hidden x features
    alignas(128) unsigned char h1[kRows * kHid * 2];    // A of D2: rows x hidden
    alignas(128) unsigned char w2t[kHid * kHid * 2];    // B of D2: W2t, out x in
    alignas(128) unsigned char d2[kRows * kHid * 2];    // A of dH1: rows x out
    alignas(128) unsigned char w2[kHid * kHid * 2];     // B of dH1: W2, in x out
    alignas(128) unsigned char h1t[kRows * kRows * 2];  // A of dW2: hidden (rows 64-127 zero) x rows
    alignas(128) unsigned char d2t[kHid * kRows * 2];   // B of dW2: out x rows
    alignas(128) unsigned char xt[kRows * kRows * 2];   // A of dW1: features (rows 32-127 zero) x rows
    alignas(128) unsigned char d1t[kHid * kRows * 2];   // B of dW1: hidden x rows
    float b1[kHid], b2[kHid], w3[kHid];
    float gb1[kHid], gb2[kHid], gw3[kHid];
    float lsum, db3;
    unsigned long long mbar;
    uint32_t tmem;
};
constexpr size_t kTrainSmemBytes = sizeof(TrainSmem) + 128;  // + alignment slack of the dynamic base

__device__ __forceinline__ void st_bf16(unsigned char *tile, int r, int k, int sbo, float v)
{
    *reinterpret_cast<bf16 *>(tile + kmajor_off(r, k, sbo)) = __float2bfloat16(v);
}

// sum over the warp, added to *dst in shared memory by lane 0
__device__ __forceinline__ void warp_add(float v, float *dst)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd_block(dst, v);
}

// Column sums over the warp's 32 rows of v[0..63] (one row per lane), added
// to dst[0..63] in shared memory.  A transposing butterfly: at each step a
// lane keeps half of its columns and adds its partner's values of them, so
// lane l ends with the sums of columns 2l and 2l+1 after 32 + 16 + 8 + 4 + 2
// shuffles (one reduction per column would take 5 each).
__device__ __forceinline__ void warp_col_sums64(float (&v)[64], float *dst)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int m = 16, len = 32; m >= 1; m >>= 1, len >>= 1) {
        const bool up = (lane & m) != 0;  // keep the upper half of the current columns
#pragma unroll
        for (int i = 0; i < len; i++) {
            const float lo = v[i], hi = v[i + len];
            const float other = __shfl_xor_sync(0xffffffffu, up ? lo : hi, m);
            v[i] = (up ? hi : lo) + other;
        }
    }
    atomicAdd_block(dst + 2 * lane, v[0]);
    atomicAdd_block(dst + 2 * lane + 1, v[1]);
}

__global__ void __launch_bounds__(kRows) mlp_train_tc_kernel(MlpDev w, const bf16 *X, const float *T,
                                                              const int *idx, long long n, long long n_total,
                                                              float wneg, float gamma, float *grad, float *loss)
{
    extern __shared__ unsigned char smem_raw[];
    TrainSmem &s = *reinterpret_cast<TrainSmem *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t) 127);
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights in their operand layouts, biases, zeroed sums and padding rows
    const bf16 *w1t = (const bf16 *) w.w1t, *w2t = (const bf16 *) w.w2t, *w2 = (const bf16 *) w.w2;
    stage_kmajor<kHid, kIn>(s.w1, w1t, kSbo1);
    stage_kmajor<kHid, kHid>(s.w2t, w2t, kSbo2);
    stage_kmajor<kHid, kHid>(s.w2, w2, kSbo2);
    for (int i = tid; i < kHid; i += kRows) {
        s.b1[i] = w.b1[i];
        s.b2[i] = w.b2[i];
        s.w3[i] = w.w3[i];
        s.gb1[i] = s.gb2[i] = s.gw3[i] = 0.0f;
    }
    if (tid == 0) s.lsum = s.db3 = 0.0f;
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    for (int i = tid; i < (8 * kSboR) / 16; i += kRows)  // h1t rows 64-127
        reinterpret_cast<uint4 *>(s.h1t + 8 * kSboR)[i] = z4;
    for (int i = tid; i < (12 * kSboR) / 16; i += kRows)  // xt rows 32-127
        reinterpret_cast<uint4 *>(s.xt + 4 * kSboR)[i] = z4;
    // this thread's row: features (zero past n) and target
    const long long row = (long long) blockIdx.x * kRows + tid;
    const bool valid = row < n;
    const long long src = valid ? (idx ? (long long) idx[row] : row) : 0;
    uint4 xr[4] = {};
    if (valid) {
        const uint4 *p = reinterpret_cast<const uint4 *>(X + src * kIn);
#pragma unroll
        for (int q = 0; q < 4; q++) xr[q] = p[q];
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        *reinterpret_cast<uint4 *>(s.x + kmajor_off(tid, 8 * q, kSbo1)) = xr[q];
        const uint32_t u[4] = {xr[q].x, xr[q].y, xr[q].z, xr[q].w};
#pragma unroll
        for (int e = 0; e < 8; e++)
            *reinterpret_cast<uint16_t *>(s.xt + kmajor_off(8 * q + e, tid, kSboR)) =
                (uint16_t) (u[e >> 1] >> (16 * (e & 1)));
    }
    const float tv = valid ? T[src] : 0.0f;
    const uint32_t mbar = smem_addr(&s.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s.tmem)),
                     "r"(kTrainCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t lane_addr = tmem + ((uint32_t) (warp * 32) << 16);
    constexpr uint32_t idesc = idesc_bf16(kRows, kHid);
    const uint32_t sx = smem_addr(s.x), sw1 = smem_addr(s.w1), sh1 = smem_addr(s.h1), sw2t = smem_addr(s.w2t),
                   sd2 = smem_addr(s.d2), sw2 = smem_addr(s.w2), sh1t = smem_addr(s.h1t), sd2t = smem_addr(s.d2t),
                   sxt = smem_addr(s.xt), sd1t = smem_addr(s.d1t);
    uint32_t phase = 0;
    bool ok = true;
    do {
        // layer 1: D1 = X W1
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kIn / 16; ks++)
                mma_bf16(tmem + kColD1, sdesc(sx + ks * 256, 128, kSbo1), sdesc(sw1 + ks * 256, 128, kSbo1), idesc,
                         ks);
            mma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        fence_after();
        // H1 = bf16(relu(D1 + b1)): row-major for layer 2, transposed for dW2
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float d[16];
            tmem_ld16(lane_addr + kColD1 + (uint32_t) c0, d);
#pragma unroll
            for (int half = 0; half < 2; half++) {
                float h[8];
#pragma unroll
                for (int e = 0; e < 8; e++) h[e] = fmaxf(d[8 * half + e] + s.b1[c0 + 8 * half + e], 0.0f);
                *reinterpret_cast<uint4 *>(s.h1 + kmajor_off(tid, c0 + 8 * half, kSbo2)) =
                    make_uint4(pack2(h[0], h[1]), pack2(h[2], h[3]), pack2(h[4], h[5]), pack2(h[6], h[7]));
#pragma unroll
                for (int e = 0; e < 8; e++) st_bf16(s.h1t, c0 + 8 * half + e, tid, kSboR, h[e]);
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // layer 2: D2 = H1 W2
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ks++)
                mma_bf16(tmem + kColD2, sdesc(sh1 + ks * 256, 128, kSbo2), sdesc(sw2t + ks * 256, 128, kSbo2),
                         idesc, ks);
            mma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        fence_after();
        // y = relu(D2 + b2) . w3 + b3, the row's loss and dL/dy
        float y = 0.0f;
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float d[16];
            tmem_ld16(lane_addr + kColD2 + (uint32_t) c0, d);
#pragma unroll
            for (int i = 0; i < 16; i++) y = fmaf(fmaxf(d[i] + s.b2[c0 + i], 0.0f), s.w3[c0 + i], y);
        }
        y += *w.b3;
        float dy = 0.0f, l = 0.0f;
        if (valid) {
            float r, wt = 1.0f;
            if (tv > 0.0f) {
                r = y - tv;
                if (r < 0.0f) wt = wneg;
            } else {
                r = fmaxf(y + gamma, 0.0f);
            }
            l = wt * r * r / (float) n_total;
            dy = 2.0f * wt * r / (float) n_total;
        }
        warp_add(l, &s.lsum);
        warp_add(dy, &s.db3);
        // dw3 = sum dy h2; d2 = dy w3 relu'(h2); db2 = sum d2; D2 in BF16,
        // row-major for dH1 and transposed for dW2
        {
            float v[64];
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float d[16];
                tmem_ld16(lane_addr + kColD2 + (uint32_t) c0, d);
#pragma unroll
                for (int i = 0; i < 16; i++) v[c0 + i] = dy * fmaxf(d[i] + s.b2[c0 + i], 0.0f);
            }
            warp_col_sums64(v, s.gw3);
        }
        {
            float v[64];
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float d[16];
                tmem_ld16(lane_addr + kColD2 + (uint32_t) c0, d);
#pragma unroll
                for (int half = 0; half < 2; half++) {
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const int c = c0 + 8 * half + e;
                        const float h2 = fmaxf(d[8 * half + e] + s.b2[c], 0.0f);
                        v[c] = h2 > 0.0f ? dy * s.w3[c] : 0.0f;
                        st_bf16(s.d2t, c, tid, kSboR, v[c]);
                    }
                    const int c = c0 + 8 * half;
                    *reinterpret_cast<uint4 *>(s.d2 + kmajor_off(tid, c, kSbo2)) =
                        make_uint4(pack2(v[c], v[c + 1]), pack2(v[c + 2], v[c + 3]), pack2(v[c + 4], v[c + 5]),
                                   pack2(v[c + 6], v[c + 7]));
                }
            }
            warp_col_sums64(v, s.gb2);
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // dH1 = D2 W2^T (over the units) and dW2 = H1^T D2 (over the rows)
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ks++)
                mma_bf16(tmem + kColD1, sdesc(sd2 + ks * 256, 128, kSbo2), sdesc(sw2 + ks * 256, 128, kSbo2), idesc,
                         ks);
#pragma unroll
            for (int ks = 0; ks < kRows / 16; ks++)
                mma_bf16(tmem + kColG2, sdesc(sh1t + ks * 256, 128, kSboR), sdesc(sd2t + ks * 256, 128, kSboR),
                         idesc, ks);
            mma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        fence_after();
        // d1 = dH1 relu'(h1); db1 = sum d1; D1 in BF16, transposed for dW1
        {
            float v[64];
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float d[16];
                tmem_ld16(lane_addr + kColD1 + (uint32_t) c0, d);
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    // the row's 8 BF16 h1 values of these columns, one 16-byte load
                    const uint4 hq = *reinterpret_cast<const uint4 *>(s.h1 + kmajor_off(tid, c0 + 8 * half, kSbo2));
                    const uint32_t hw[4] = {hq.x, hq.y, hq.z, hq.w};
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const int c = c0 + 8 * half + e;
                        const float h1 = __uint_as_float((hw[e >> 1] >> (16 * (e & 1))) << 16);
                        v[c] = h1 > 0.0f ? d[8 * half + e] : 0.0f;
                        st_bf16(s.d1t, c, tid, kSboR, v[c]);
                    }
                }
            }
            warp_col_sums64(v, s.gb1);
        }
        // dW2 rows (units in) are TMEM lanes 0-63: warps 0 and 1
        if (warp < 2)
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float d[16];
                tmem_ld16(lane_addr + kColG2 + (uint32_t) c0, d);
#pragma unroll
                for (int i = 0; i < 16; i++) atomicAdd(grad + kOffW2 + tid * kHid + c0 + i, d[i]);
            }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // dW1 = X^T D1 (over the rows)
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kRows / 16; ks++)
                mma_bf16(tmem + kColG1, sdesc(sxt + ks * 256, 128, kSboR), sdesc(sd1t + ks * 256, 128, kSboR),
                         idesc, ks);
            mma_commit(mbar);
        }
        ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        if (!ok) break;
        phase ^= 1u;
        fence_after();
        // dW1 rows (features) are TMEM lanes 0-31: warp 0
        if (warp == 0)
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float d[16];
                tmem_ld16(lane_addr + kColG1 + (uint32_t) c0, d);
#pragma unroll
                for (int i = 0; i < 16; i++) atomicAdd(grad + kOffW1 + tid * kHid + c0 + i, d[i]);
            }
        __syncthreads();
        if (tid < kHid) {
            atomicAdd(grad + kOffB1 + tid, s.gb1[tid]);
            atomicAdd(grad + kOffB2 + tid, s.gb2[tid]);
            atomicAdd(grad + kOffW3 + tid, s.gw3[tid]);
        }
        if (tid == 0) {
            atomicAdd(grad + kOffB3, s.db3);
            atomicAdd(loss, s.lsum);
        }
    } while (false);
    if (!ok) {
        if (tid == 0 && w.status) atomicExch(w.status, kMlpTcTimeout);
        mbar_wait(mbar, phase);  // the MMAs in flight, if any (bounded)
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTrainCols) : "memory");
}

}  // namespace

namespace {

template <bool GRID>
cudaError_t launch_tc(const MlpDev &w, const void *X, long long n, float *y, const MlpGridArgs &g, cudaStream_t s)
{
    static std::atomic<unsigned long long> attr{0};
    cudaError_t e = set_dynamic_smem_once(mlp_tc_kernel<GRID>, (int) kTcSmemBytes, attr);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (n + kRows - 1) / kRows;
    const long long grid = tiles < 2ll * sms ? tiles : 2ll * sms;
    mlp_tc_kernel<GRID><<<(unsigned) grid, kRows, kTcSmemBytes, s>>>(w, (const bf16 *) X, n, y, w.status, g);
    return cudaGetLastError();
}

}  // namespace

cudaError_t mlp_forward(const MlpDev &w, const void *X, long long n, float *y, cudaStream_t s)
{
    return launch_tc<false>(w, X, n, y, MlpGridArgs{}, s);
}

cudaError_t mlp_learned_grid_tc(const MlpDev &w, const MlpGridArgs &g, cudaStream_t s)
{
    return launch_tc<true>(w, nullptr, g.ncell, nullptr, g, s);
}

cudaError_t mlp_train_step(const MlpDev &w, const void *X, const float *T, const int *idx, long long n,
                           long long n_total, float wneg, float gamma, float *grad, float *loss, cudaStream_t s)
{
    static std::atomic<unsigned long long> attr{0};
    cudaError_t e = set_dynamic_smem_once(mlp_train_tc_kernel, (int) kTrainSmemBytes, attr);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    mlp_train_tc_kernel<<<(unsigned) ((n + kRows - 1) / kRows), kRows, kTrainSmemBytes, s>>>(
        w, (const bf16 *) X, T, idx, n, n_total, wneg, gamma, grad, loss);
    return cudaGetLastError();
}

}  // namespace ivr
