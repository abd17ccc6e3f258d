// ivr_kernels.cu -- the kernels around the march: byte swap, brick gather,
// min/max + histogram (initvolluts), macrocell min/max and per-TF empty
// flags, sort-last compositing (compositetiles) and RGBA8 quantisation.
// Compiled with -fmad=false like the march.
#include <float.h>
#include <stdint.h>

#include <algorithm>

#include <mutex>

#include "ivr_internal.h"

namespace ivr {
namespace {

constexpr int kSms = 152;

int grid_for(long long n, int threads, int per_sm = 8)
{
    long long g = (n + threads - 1) / threads;
    long long cap = (long long) kSms * per_sm;
    return (int) (g < cap ? (g < 1 ? 1 : g) : cap);
}

template <typename T> __device__ __forceinline__ float tof(T v) { return (float) v; }

__device__ __forceinline__ float load_any(const void *p, int dtype, long long i)
{
    switch (dtype) {
    case IVR_U8: return (float) __ldg(reinterpret_cast<const uint8_t *>(p) + i);
    case IVR_U16: return (float) __ldg(reinterpret_cast<const uint16_t *>(p) + i);
    default: return __ldg(reinterpret_cast<const float *>(p) + i);
    }
}

__global__ void byteswap16_kernel(uint16_t *p, long long n)
{
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        p[i] = (uint16_t) ((p[i] >> 8) | (p[i] << 8));
}

// BYTESWAP_FP (sysutil.h:121-133): byte order reversed
__global__ void byteswap32_kernel(uint32_t *p, long long n)
{
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        p[i] = __byte_perm(p[i], 0, 0x0123);
}

// readfromfile (main.c:1254-1265): brick [sz..sz+ld) x [sy..sy+lh) x
// [sx..sx+lw) of the global volume into a dense [ld][lh][lw] array.
template <typename T>
__global__ void gather_kernel(const T *__restrict__ src, int gw, int gh, T *__restrict__ dst, int sx, int sy,
                              int sz, int lw, int lh, long long n)
{
    for (long long o = blockIdx.x * (long long) blockDim.x + threadIdx.x; o < n; o += (long long) gridDim.x * blockDim.x) {
        int x = (int) (o % lw);
        long long r = o / lw;
        int y = (int) (r % lh);
        int z = (int) (r / lh);
        dst[o] = src[((long long) (sz + z) * gh + (sy + y)) * gw + (sx + x)];
    }
}

__global__ void minmax_kernel(const void *data, int dtype, long long n, float *partial)
{
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        float v = load_any(data, dtype, i);
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ float slo[32], shi[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { slo[w] = lo; shi[w] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int) (blockDim.x >> 5); k++) { lo = fminf(lo, slo[k]); hi = fmaxf(hi, shi[k]); }
        partial[2 * blockIdx.x] = lo;
        partial[2 * blockIdx.x + 1] = hi;
    }
}

// histogram (mathutil.c:459-467): bin (int)(v - min); privatised in shared
// memory when the bins fit.
constexpr int kSmemBins = 12288;
__global__ void hist_smem_kernel(const void *data, int dtype, long long n, float mn, int hsize, int *hist)
{
    __shared__ int sh[kSmemBins];
    for (int b = threadIdx.x; b < hsize; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        int b = (int) (load_any(data, dtype, i) - mn);
        if (b >= 0 && b < hsize) atomicAdd(&sh[b], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < hsize; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], sh[b]);
}
__global__ void hist_global_kernel(const void *data, int dtype, long long n, float mn, int hsize, int *hist)
{
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        int b = (int) (load_any(data, dtype, i) - mn);
        if (b >= 0 && b < hsize) atomicAdd(&hist[b], 1);
    }
}

// Macrocell min/max: with edge `cell`, cell (cx,cy,cz) spans voxels
// [c*cell, min(c*cell+cell, n-1)] per axis -- its voxel cells plus the +1
// layer a trilinear sample in the cell also reads.  One block per cell.
__global__ void macrocell_kernel(const void *data, int dtype, int nx, int ny, int nz, int cell, float *mc, int mcx,
                                 int mcy)
{
    const int cid = blockIdx.x;
    const int cx = cid % mcx, cy = (cid / mcx) % mcy, cz = cid / (mcx * mcy);
    const int x0 = cx * cell, y0 = cy * cell, z0 = cz * cell;
    const int x1 = min(x0 + cell, nx - 1), y1 = min(y0 + cell, ny - 1), z1 = min(z0 + cell, nz - 1);
    const int ex = x1 - x0 + 1, ey = y1 - y0 + 1, ez = z1 - z0 + 1;
    float lo = FLT_MAX, hi = -FLT_MAX;
    const int tot = ex * ey * ez;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        int x = t % ex, r = t / ex;
        int y = r % ey, z = r / ey;
        float v = load_any(data, dtype, ((long long) (z0 + z) * ny + (y0 + y)) * nx + (x0 + x));
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ float slo[32], shi[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { slo[w] = lo; shi[w] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int) (blockDim.x >> 5); k++) { lo = fminf(lo, slo[k]); hi = fmaxf(hi, shi[k]); }
        mc[2 * cid] = lo;
        mc[2 * cid + 1] = hi;
    }
}

// A cell is transparent when no LUT entry its samples can index has
// non-zero opacity.  Samples lie in [min, max] of the cell's voxels up to
// rounding, so the index range is widened by one on each side.
// nzprefix[i] = number of entries in [0, i) with non-zero opacity.
// Writes kDistCap for a transparent cell and 0 for the others.  In the same
// pass (opac non-null), the tile cost estimate's input: 255 sqrt(mean LUT
// opacity over the entries the cell's voxel range [min, max] indexes); the
// square root keeps small opacities apart; aprefix[i] = sum of the
// opacities of entries [0, i).
__global__ void empty_kernel(const float *mc, int ncell, const int *nzprefix, const double *aprefix, int lut_n,
                             int lut_off, float lut_scale, uint8_t *dist, uint8_t *opac)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        const int i0 = (int) (mc[2 * c] * lut_scale) - lut_off, i1 = (int) (mc[2 * c + 1] * lut_scale) - lut_off;
        const int lo = min(max(i0 - 1, 0), lut_n - 1);
        const int hi = min(max(i1 + 1, 0), lut_n - 1);
        dist[c] = (nzprefix[hi + 1] - nzprefix[lo]) == 0 ? (uint8_t) kDistCap : 0;
        if (opac) {
            const int a = min(max(i0, 0), lut_n - 1);
            const int b = min(max(i1, a), lut_n - 1);
            const double mean = (aprefix[b + 1] - aprefix[a]) / (double) (b - a + 1);
            const float q = sqrtf(fminf(fmaxf((float) mean, 0.0f), 1.0f)) * 255.0f + 0.5f;
            opac[c] = (uint8_t) min((int) q, 255);
        }
    }
}

// The Chebyshev distance (in cells) from each transparent cell to the
// nearest opaque one, capped: d = min(cap, max(|dx|, |dy|, |dz|) to the
// nearest cell with flag 0), 0 for opaque cells; cells outside the grid are
// not opaque (a ray there has left the brick).  Every cell within d-1 of a
// cell with d >= 1 is then transparent.  The L-infinity distance separates
// by axis: with g0 = 0 (opaque) or cap (transparent) and, along each axis
// in turn, g(p) = min over |k| <= cap of max(|k|, g(p + k)), three passes
// give the distance exactly (a minimum over the cells of the window of the
// largest per-axis offset; anything farther than the cap is the cap).
//
// One pass over the lines along `axis` (0 = x, 1 = y, 2 = z), in place: a
// block takes `lines` neighbouring lines whole (32, fewer for very long
// lines; neighbours along x for the y and z passes, along y for the x
// pass), so that its loads and stores coalesce, stages them in shared
// memory and writes them back once all are read.
constexpr int kDistLines = 32;
__global__ void dist_axis_kernel(uint8_t *dist, int mcx, int mcy, int mcz, int axis, int lines)
{
    extern __shared__ uint8_t tile[];  // [L][lines + 1]
    const int P = lines + 1;
    const int L = axis == 0 ? mcx : axis == 1 ? mcy : mcz;
    const long long slab = (long long) mcx * mcy;
    const long long stride = axis == 0 ? 1 : axis == 1 ? mcx : slab;
    // this block's group of lines: the first line's base and the distance
    // between neighbouring lines; nl lines are in the grid
    const int across = axis == 0 ? mcy : mcx;  // lines of a group run along this dimension
    const int groups_across = (across + lines - 1) / lines;
    const long long g = blockIdx.x;
    const int outer = (int) (g / groups_across), first = (int) (g % groups_across) * lines;
    const int nl = min(lines, across - first);
    long long base;
    long long step;
    if (axis == 0) {  // rows (y, z): outer = z, lines along y
        base = ((long long) outer * mcy + first) * mcx;
        step = mcx;
    } else if (axis == 1) {  // columns (x, z): outer = z, lines along x
        base = (long long) outer * slab + first;
        step = 1;
    } else {  // pillars (x, y): outer = y, lines along x
        base = (long long) outer * mcx + first;
        step = 1;
    }
    const int n = L * nl;
    // element e of the group: line l, position p (the x pass walks a row's
    // bytes with neighbouring threads, the others neighbouring lines); four
    // loads in flight per thread before their stores
    constexpr int U = 4;
    for (int e0 = threadIdx.x; e0 < n; e0 += U * blockDim.x) {
        uint8_t v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int e = e0 + u * blockDim.x;
            const int l = axis == 0 ? e / L : e % nl, p = axis == 0 ? e % L : e / nl;
            v[u] = e < n ? dist[base + l * step + p * stride] : 0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int e = e0 + u * blockDim.x;
            const int l = axis == 0 ? e / L : e % nl, p = axis == 0 ? e % L : e / nl;
            if (e < n) tile[p * P + l] = v[u];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int l = axis == 0 ? e / L : e % nl, p = axis == 0 ? e % L : e / nl;
        int m = tile[p * P + l];
        for (int k = 1; k < m; k++) {  // only offsets below the current minimum can lower it
            if (p - k >= 0) m = min(m, max(k, (int) tile[(p - k) * P + l]));
            if (p + k < L) m = min(m, max(k, (int) tile[(p + k) * P + l]));
        }
        dist[base + l * step + p * stride] = (uint8_t) m;
    }
}

// compositetiles (main.c:1203-1218)
__global__ void composite_kernel(float4 *dst, const float4 *__restrict__ src, int num, long long npix)
{
    for (long long p = blockIdx.x * (long long) blockDim.x + threadIdx.x; p < npix; p += (long long) gridDim.x * blockDim.x) {
        float4 d = dst[p];
        for (int k = num - 1; k >= 0; k--) {
            float4 s = __ldg(src + (long long) k * npix + p);
            d.z = s.z + (1.0f - s.w) * d.z;
            d.y = s.y + (1.0f - s.w) * d.y;
            d.x = s.x + (1.0f - s.w) * d.x;
            d.w = s.w + (1.0f - s.w) * d.w;
        }
        dst[p] = d;
    }
}

// (uint8)(v*255 + 0.5) for v clamped to [0,1], computed exactly in integers
// (see q8 in ivr_march.cu).
__device__ __forceinline__ unsigned q8k(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 1.0f) return 255u;
    unsigned bits = __float_as_uint(v);
    int e = (int) (bits >> 23);
    if (e == 0) return 0u;
    unsigned long long m = (bits & 0x7fffffu) | 0x800000u;
    int s = 150 - e;
    if (s >= 34) return 0u;
    return (unsigned) ((255ull * m + (1ull << (s - 1))) >> s);
}

__global__ void quantize_kernel(const float *__restrict__ in, uint8_t *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        out[i] = (uint8_t) q8k(in[i]);
}

// ---- allocation-free histogram ---------------------------------------------
// Scratch of ivr_volume_histogram_noalloc: min/max partials, the reduced
// min/max and up to kNoAllocMaxBins bins, in one static device array that
// every GPU loading this library holds until the process exits.
struct NoAllocScratch {
    float partial[2 * kSms * 4];
    float minmax[2];
    int hist[kNoAllocMaxBins];
};
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

__global__ void minmax_final_kernel(const float *partial, int nparts, float *minmax)
{
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        lo = fminf(lo, partial[2 * i]);
        hi = fmaxf(hi, partial[2 * i + 1]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ float slo[32], shi[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { slo[w] = lo; shi[w] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int) (blockDim.x >> 5); k++) { lo = fminf(lo, slo[k]); hi = fmaxf(hi, shi[k]); }
        minmax[0] = lo;
        minmax[1] = hi;
    }
}

// the histogram of hist_*_kernel with the minimum read from device memory
__global__ void hist_devmin_kernel(const void *data, int dtype, long long n, const float *minmax, int hsize,
                                   int *hist)
{
    __shared__ int sh[kSmemBins];
    const float mn = minmax[0];
    const bool priv = hsize <= kSmemBins;
    if (priv) {
        for (int b = threadIdx.x; b < hsize; b += blockDim.x) sh[b] = 0;
        __syncthreads();
    }
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        int b = (int) (load_any(data, dtype, i) - mn);
        if (b >= 0 && b < hsize) atomicAdd(priv ? &sh[b] : &hist[b], 1);
    }
    if (priv) {
        __syncthreads();
        for (int b = threadIdx.x; b < hsize; b += blockDim.x)
            if (sh[b]) atomicAdd(&hist[b], sh[b]);
    }
}

}  // namespace

// Device address of the static scratch on the current device.  Resolved
// once per device with cudaGetSymbolAddress (the first call on a device
// loads this module there if it is not loaded yet).
static cudaError_t noalloc_scratch(NoAllocScratch **out)
{
    static std::mutex mu;
    static void *ptrs[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        ptrs[dev] = p;
    }
    *out = static_cast<NoAllocScratch *>(ptrs[dev]);
    return cudaSuccess;
}

cudaError_t noalloc_histogram(const void *data, int dtype, long long n, int hsize, int *hist_host,
                              float *minmax_host, cudaStream_t s)
{
    NoAllocScratch *sc = nullptr;
    cudaError_t e = noalloc_scratch(&sc);
    if (e != cudaSuccess) return e;
    const int parts = kSms * 4;
    minmax_kernel<<<parts, 256, 0, s>>>(data, dtype, n, sc->partial);
    minmax_final_kernel<<<1, 1024, 0, s>>>(sc->partial, parts, sc->minmax);
    if ((e = cudaMemsetAsync(sc->hist, 0, sizeof(int) * (size_t) hsize, s)) != cudaSuccess) return e;
    hist_devmin_kernel<<<grid_for(n, 512, 2), 512, 0, s>>>(data, dtype, n, sc->minmax, hsize, sc->hist);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(hist_host, sc->hist, sizeof(int) * (size_t) hsize, cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(minmax_host, sc->minmax, 2 * sizeof(float), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    return cudaStreamSynchronize(s);
}

size_t dtype_size(int dtype) { return dtype == IVR_U8 ? 1 : dtype == IVR_U16 ? 2 : 4; }

int minmax_parts() { return kSms * 4; }

cudaError_t launch_byteswap(void *data, long long n, int elem, cudaStream_t s)
{
    if (n <= 0 || elem == 1) return cudaSuccess;
    if (elem == 2) byteswap16_kernel<<<grid_for(n, 256), 256, 0, s>>>((uint16_t *) data, n);
    else byteswap32_kernel<<<grid_for(n, 256), 256, 0, s>>>((uint32_t *) data, n);
    return cudaGetLastError();
}

cudaError_t launch_gather_brick(const void *src, int gw, int gh, int gd, void *dst, int sx, int sy, int sz, int lw,
                                int lh, int ld, int elem, cudaStream_t s)
{
    (void) gd;
    long long n = (long long) lw * lh * ld;
    int g = grid_for(n, 256);
    if (elem == 1) gather_kernel<uint8_t><<<g, 256, 0, s>>>((const uint8_t *) src, gw, gh, (uint8_t *) dst, sx, sy, sz, lw, lh, n);
    else if (elem == 2) gather_kernel<uint16_t><<<g, 256, 0, s>>>((const uint16_t *) src, gw, gh, (uint16_t *) dst, sx, sy, sz, lw, lh, n);
    else gather_kernel<uint32_t><<<g, 256, 0, s>>>((const uint32_t *) src, gw, gh, (uint32_t *) dst, sx, sy, sz, lw, lh, n);
    return cudaGetLastError();
}

cudaError_t launch_minmax(const void *data, int dtype, long long n, float *partial, int nparts, cudaStream_t s)
{
    minmax_kernel<<<nparts, 256, 0, s>>>(data, dtype, n, partial);
    return cudaGetLastError();
}

cudaError_t launch_histogram(const void *data, int dtype, long long n, float mn, int hsize, int *hist, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int) * (size_t) hsize, s);
    if (e != cudaSuccess) return e;
    if (hsize <= kSmemBins) hist_smem_kernel<<<grid_for(n, 512, 2), 512, 0, s>>>(data, dtype, n, mn, hsize, hist);
    else hist_global_kernel<<<grid_for(n, 256), 256, 0, s>>>(data, dtype, n, mn, hsize, hist);
    return cudaGetLastError();
}

cudaError_t launch_macrocells(const void *data, int dtype, int nx, int ny, int nz, int cell, float *mc, int mcx,
                              int mcy, int mcz, cudaStream_t s)
{
    macrocell_kernel<<<mcx * mcy * mcz, 128, 0, s>>>(data, dtype, nx, ny, nz, cell, mc, mcx, mcy);
    return cudaGetLastError();
}

cudaError_t launch_empty_flags(const float *mc, int mcx, int mcy, int mcz, const int *nzprefix, const double *aprefix,
                               int lut_n, int lut_off, float lut_scale, uint8_t *empty, uint8_t *opac, cudaStream_t s)
{
    const int ncell = mcx * mcy * mcz;
    empty_kernel<<<grid_for(ncell, 256), 256, 0, s>>>(mc, ncell, nzprefix, aprefix, lut_n, lut_off, lut_scale, empty,
                                                      opac);
    return launch_dist_transform(empty, mcx, mcy, mcz, s);
}

cudaError_t launch_dist_transform(uint8_t *dist, int mcx, int mcy, int mcz, cudaStream_t s)
{
    if (mcx <= 0 || mcy <= 0 || mcz <= 0) return cudaSuccess;
    const int dims[3] = {mcx, mcy, mcz};
    for (int axis = 0; axis < 3; axis++) {
        const int L = dims[axis];
        if (L == 1) continue;  // a line of one cell keeps its flag
        // 32 lines a block up to 1489 cells a line, fewer above
        const int lines = std::min(kDistLines, 48 * 1024 / L - 1);
        if (lines < 1) return cudaErrorInvalidValue;  // a line of more than 24576 macrocells
        const size_t smem = (size_t) L * (lines + 1);
        const int across = axis == 0 ? mcy : mcx, outer = axis == 2 ? mcy : mcz;
        const long long groups = (long long) outer * ((across + lines - 1) / lines);
        dist_axis_kernel<<<(unsigned) groups, 256, smem, s>>>(dist, mcx, mcy, mcz, axis, lines);
    }
    return cudaGetLastError();
}

// Per-voxel gradient (gradient3d, restated as intended): per axis a halved
// central difference inside and a halved one-sided difference on the
// faces, times the unit spacing; w = |(x, y, z)| as mag3f computes it.
template <typename T>
__device__ __forceinline__ float grad_axis(const T *v, long long o, int c, int n, long long stride)
{
    if (c == 0) return ((float) v[o + stride] - (float) v[o]) / 2.0f * 1.0f;
    if (c == n - 1) return ((float) v[o] - (float) v[o - stride]) / 2.0f * 1.0f;
    return ((float) v[o + stride] - (float) v[o - stride]) / 2.0f * 1.0f;
}

template <typename T>
__global__ void gradient_kernel(const T *vol, int w, int h, int d, float4 *out)
{
    const long long n = (long long) w * h * d;
    for (long long o = blockIdx.x * (long long) blockDim.x + threadIdx.x; o < n;
         o += (long long) gridDim.x * blockDim.x) {
        const int j = (int) (o % w);
        const long long r = o / w;
        const int i = (int) (r % h), k = (int) (r / h);
        const float x = grad_axis(vol, o, j, w, 1);
        const float y = grad_axis(vol, o, i, h, w);
        const float z = grad_axis(vol, o, k, d, (long long) w * h);
        out[o] = make_float4(x, y, z, sqrtf(x * x + y * y + z * z));
    }
}

cudaError_t launch_gradient(const void *data, int dtype, int w, int h, int d, float4 *out, cudaStream_t s)
{
    const long long n = (long long) w * h * d;
    const int grid = grid_for(n, 256);
    switch (dtype) {
    case IVR_U8: gradient_kernel<<<grid, 256, 0, s>>>((const uint8_t *) data, w, h, d, out); break;
    case IVR_U16: gradient_kernel<<<grid, 256, 0, s>>>((const uint16_t *) data, w, h, d, out); break;
    case IVR_F32: gradient_kernel<<<grid, 256, 0, s>>>((const float *) data, w, h, d, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T, typename V>
__global__ void quad_kernel(const T *src, int nx, int ny, int nz, V *dst)
{
    const long long qx = nx - 1, qy = ny - 1, n = qx * qy * nz;
    for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < n;
         e += (long long) gridDim.x * blockDim.x) {
        const long long j = e % qx, r = e / qx, i = r % qy, k = r / qy;
        const T *p = src + (k * ny + i) * nx + j;
        V v;
        v.x = p[0];
        v.y = p[1];
        v.z = p[nx];
        v.w = p[nx + 1];
        if constexpr (sizeof(T) == sizeof(float)) {
            if (kQuadDelta) {  // the sampler's x-lerp differences, rounded as it rounds them
                v.y = p[1] - p[0];
                v.w = p[nx + 1] - p[nx];
            }
        }
        dst[e] = v;
    }
}

size_t quad_bytes(int dtype, int nx, int ny, int nz)
{
    return (size_t) (nx - 1) * (ny - 1) * nz * 4 * dtype_size(dtype);
}

cudaError_t launch_quads(const void *data, int dtype, int nx, int ny, int nz, void *quad, cudaStream_t s)
{
    const long long n = (long long) (nx - 1) * (ny - 1) * nz;
    const int grid = grid_for(n, 256);
    switch (dtype) {
    case IVR_U8: quad_kernel<<<grid, 256, 0, s>>>((const uint8_t *) data, nx, ny, nz, (uchar4 *) quad); break;
    case IVR_U16: quad_kernel<<<grid, 256, 0, s>>>((const uint16_t *) data, nx, ny, nz, (ushort4 *) quad); break;
    case IVR_F32: quad_kernel<<<grid, 256, 0, s>>>((const float *) data, nx, ny, nz, (float4 *) quad); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_composite(float *dst, const float *src, int num, long long npix, cudaStream_t s)
{
    composite_kernel<<<grid_for(npix, 256), 256, 0, s>>>((float4 *) dst, (const float4 *) src, num, npix);
    return cudaGetLastError();
}

cudaError_t launch_quantize(const float *in, uint8_t *out, long long n, cudaStream_t s)
{
    quantize_kernel<<<grid_for(n, 256), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

}  // namespace ivr
