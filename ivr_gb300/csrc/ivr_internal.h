// ivr_internal.h -- structures shared by the host code and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ivr_gpu.h"

namespace ivr {

constexpr int kMaxBricks = IVR_MAX_BRICKS;
constexpr int kCell = 16;  // default macrocell edge in voxels (ivr_volume_set_macrocell)
constexpr int kMinCell = 4, kMaxCell = 32;  // the edges a volume may use: powers of two
#ifndef IVR_DIST_CAP
#define IVR_DIST_CAP 8
#endif
constexpr int kDistCap = IVR_DIST_CAP;  // largest transparent radius stored per macrocell
// f32 corner-packed copies hold each row pair as (v0, v1 - v0): the
// sampler's x lerp fmaf(fx, v1 - v0, v0) then takes no subtraction, and
// the difference is the same IEEE subtraction the sampler would make, so
// every sample is bitwise unchanged.  (u8/u16 differences do not fit their
// lanes.)  IVR_QUAD_DELTA=0 stores the voxels themselves.
#ifndef IVR_QUAD_DELTA
#define IVR_QUAD_DELTA 1
#endif
constexpr bool kQuadDelta = IVR_QUAD_DELTA != 0;

// One brick as the march kernels see it.  Geometry follows the reference's
// per-rank AABB (main.c:552-618): bmin and w/h/d from the brick's world
// extent, nx/ny/nz the local array dims including the halo.
struct DevBrick {
    const void *data;       // [nz][ny][nx] of the volume's dtype
    int nx, ny, nz;
    float bminx, bminy, bminz;
    float w, h, d;          // aabb.w/h/d
    float icx, icy, icz;    // CONFIG: core voxels per world unit
    float mcwx, mcwy, mcwz; // CONFIG: world size of one macrocell
    float vwx, vwy, vwz;    // CONFIG: world size of one voxel, 1 / ic
    int cshift;             // log2 of the macrocell edge in voxels
    float dconst[6];        // clip-plane constants of this brick
    int istrt, istop, jstrt, jstop;  // pixel rect (createlocalimage)
    float dir0x, dir0y, dir0z;       // REF: ray direction at (istrt, jstrt)
    const uint8_t *empty;   // per macrocell: 0 = some sample there can be
                            // opaque; r >= 1 = every cell within r-1 cells
                            // (Chebyshev) is transparent; or null
    int mcx, mcy, mcz;      // macrocell grid dims
    uint8_t *touched;       // census only: cells an executed sample read
    const void *quad;       // corner-packed copy or null: element (j, i, k),
                            // j < nx-1, i < ny-1, holds the voxels (j, i),
                            // (j+1, i), (j, i+1), (j+1, i+1) of slab k (f32
                            // with kQuadDelta: the second of each pair as
                            // its difference from the first)
    const uint8_t *opac;    // per macrocell: 255 sqrt(mean LUT opacity over
                            // its value range) -- the tile cost estimate's
                            // input; or null
};

// Learned-skip judge words of a view (device).  maxdiff and warps_done (the
// compare launch's blocks done) are per-frame scratch the compare launch
// clears after use; fail is the last frame's verdict (the fallback launch's
// gate); the rest are running totals.
struct JudgeWords {
    int maxdiff;
    int warps_done;
    int fail;
    int worst;                      // largest difference seen
    unsigned long long frames;      // frames judged
    unsigned long long fallbacks;   // frames re-rendered with the exact grid
    unsigned long long pixels;      // pixels compared
    unsigned long long exact_frames;  // judged launches that found their learned
                                      // grid marked wrong and used the exact one
};

// Everything one launch needs, passed by value as a __grid_constant__.
struct FrameDesc {
    int vw, vh;              // viewport
    int nb;                  // bricks
    int preset, tf_mode, dtype;
    float origx, origy, origz;
    float incrix, incriy, incriz;
    float incrjx, incrjy, incrjz;
    float ctm[9];            // CONFIG ray directions: ctm * (u, v, 5)
    float left, bottom, du, dv, eyen;
    float step;              // REF: ray-parameter step; CONFIG: world step
    int max_samples;         // 0 = unbounded
    float term_alpha;
    float alpha;             // opacity scale (STATE.alpha)
    const float4 *lut;
    int lut_n, lut_off;
    float lut_scale;
    float gdconst[6];        // CONFIG: the clipped global box
    int out_x, out_y, out_w, out_h;  // output window in viewport pixels
    int single;              // >= 0: render only this brick (no compositing)
    unsigned long long *counters;    // [0] executed samples, [1] lattice
                                     // points (census) -- nullable
    int census;              // 1: count lattice points of every brick and
                             // mark touched cells (diagnostic launch)
    unsigned long long *tickets;     // CONFIG: tile ticket counter (view-owned)
    unsigned long long ticket_base;  // its value when this launch starts
    const int *gate;                 // CONFIG: if set, render only when
                                     // *gate != 0 (the judge's fallback)
    // CONFIG learned skipping (judge null: none): tiles whose index is
    // judge_phase modulo judge_stride are marched again with the exact
    // grids and compared; see JudgeWords
    JudgeWords *judge;
    int *judge_reject;               // set to 1 when the frame fails (host-mapped)
    int *learned_bad;                // nonzero: the learned grid is wrong,
                                     // render with the exact grids
    int judge_stride, judge_phase, judge_tol;
    uchar4 *judge8;                  // the judged tiles' exact re-march, 32 pixels each
    const int *perm;                 // CONFIG: ticket n renders tile perm[n] (null: n)
    int order[kMaxBricks];   // near -> far
    DevBrick b[kMaxBricks];
    const uint8_t *exact[kMaxBricks];  // the exact grids (judged launches)
};

// kernel parameters are limited to 32764 bytes
static_assert(sizeof(FrameDesc) <= 32000, "FrameDesc too large for a kernel parameter");

// One frame of a batched launch (device copy).
struct BatchItem {
    float4 *out32;
    uchar4 *out8;
    long long tile0;   // first global tile number of this frame
    int tiles_x;       // warp tiles per output row
    int pad;
    FrameDesc f;
};
struct BatchHeader {
    int nitems;
    int pad;
    long long total_tiles;
};
constexpr int kBatchVariants = 6;  // warp tile 8x4 / 4x8 / 16x2, with and without PAIR

// Host-side brick record (device array + geometry that does not depend on
// the view).
struct HostBrick {
    int lw, lh, ld;     // local dims incl. halo
    int cw, ch, cd;     // core dims
    int sx, sy, sz;     // start index in the global volume
    int col, row, slab;
    float bminx, bminy, bminz, bmaxx, bmaxy, bmaxz;
    float w, h, d;
    void *data;         // device
    bool owns;          // false when it aliases the full volume
    float *mc_minmax;   // device [mcz][mcy][mcx][2]
    int mcx, mcy, mcz;
    int cell;           // macrocell edge in voxels (a power of two)
    void *quad;         // device corner-packed copy (DevBrick::quad) or null
};

size_t dtype_size(int dtype);

// kernels (ivr_kernels.cu)
cudaError_t launch_byteswap(void *data, long long n, int elem, cudaStream_t s);
cudaError_t launch_gather_brick(const void *src, int gw, int gh, int gd, void *dst, int sx, int sy, int sz,
                                int lw, int lh, int ld, int elem, cudaStream_t s);
cudaError_t launch_minmax(const void *data, int dtype, long long n, float *partial, int nparts, cudaStream_t s);
cudaError_t launch_histogram(const void *data, int dtype, long long n, float mn, int hsize, int *hist,
                             cudaStream_t s);
cudaError_t launch_macrocells(const void *data, int dtype, int nx, int ny, int nz, int cell, float *mc, int mcx,
                              int mcy, int mcz, cudaStream_t s);
// a TF's exact grid: the empty-cell flags, then the distance transform; with
// opac, each cell's 255 sqrt(mean LUT opacity over its value range) as well
// (DevBrick::opac, the tile cost estimate's input)
cudaError_t launch_empty_flags(const float *mc, int mcx, int mcy, int mcz, const int *nzprefix, const double *aprefix,
                               int lut_n, int lut_off, float lut_scale, uint8_t *empty, uint8_t *opac, cudaStream_t s);
// per-voxel gradient (gx, gy, gz, |g|) of a w x h x d volume into out
cudaError_t launch_gradient(const void *data, int dtype, int w, int h, int d, float4 *out, cudaStream_t s);
// corner-packed copy of an nx x ny x nz brick: (nx-1)(ny-1)nz four-voxel
// elements of 4 * sizeof(dtype) bytes
size_t quad_bytes(int dtype, int nx, int ny, int nz);
cudaError_t launch_quads(const void *data, int dtype, int nx, int ny, int nz, void *quad, cudaStream_t s);
cudaError_t launch_composite(float *dst, const float *src, int num, long long npix, cudaStream_t s);
cudaError_t launch_quantize(const float *in, uint8_t *out, long long n, cudaStream_t s);
int minmax_parts();

// allocation-free histogram (ivr_volume_histogram_noalloc): min/max and
// hsize <= kNoAllocMaxBins bins of n voxels, scratch in a static device array
constexpr int kNoAllocMaxBins = 65536;
cudaError_t noalloc_histogram(const void *data, int dtype, long long n, int hsize, int *hist_host,
                              float *minmax_host, cudaStream_t s);

// march (ivr_march.cu)
// *tickets: how many tile tickets the launch takes from f.tickets (a
// persistent CONFIG launch takes each tile once and each warp fails once).
cudaError_t launch_march(const FrameDesc &f, float4 *out32, uchar4 *out8, cudaStream_t s, long long *tickets);
// the sampler alone on brick f.b[0] (sample-rate roofline): every thread
// takes `steps` samples; *samples = threads * steps; out holds one float4 per
// thread (sample_peak_threads())
// 3D textures of the sample-rate roofline's brick (point and hardware
// filtered); scale turns the filtered fetch back into volume units
struct SamplerTex {
    cudaTextureObject_t point, linear;
    float scale;
};
// the sampler roofline through an ivr_sampler_layout: samples/s launch into
// out (when set) and the largest sample error against the exact sampler
// into *err as float bits (when set)
cudaError_t launch_sample_peak(const FrameDesc &f, int layout, const SamplerTex &tex, int steps, float4 *out,
                               long long *samples, unsigned *err, cudaStream_t s);
int sample_peak_threads();
// the verdict of a learned-skip frame rendered by a judged launch of f
cudaError_t launch_judge_compare(const FrameDesc &f, const uchar4 *out8, const float4 *out32, cudaStream_t s);
// bytes of f.judge8 a judged launch of f writes
long long judge_scratch_bytes(const FrameDesc &f);
// the CONFIG tile order of f, costliest first, into perm (ntiles ints) with
// key (ntiles bytes) and counts (128 ints) as scratch
cudaError_t launch_tile_order(const FrameDesc &f, uint8_t *key, int *counts, int *perm, cudaStream_t s);
// the capped distance transform of a flag grid (kDistCap or 0 per cell), in place
cudaError_t launch_dist_transform(uint8_t *dist, int mcx, int mcy, int mcz, cudaStream_t s);
// batched CONFIG frames of one volume dtype; *ticket must be zero at launch
cudaError_t launch_batch(int dtype, int variant, const BatchHeader *hdr, const BatchItem *items,
                         unsigned long long *ticket, cudaStream_t s);
int batch_variant_tile_w(int variant);

}  // namespace ivr
