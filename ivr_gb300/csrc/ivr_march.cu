// ivr_march.cu -- the per-ray march: ray setup, slab test, sample lattice,
// trilinear reconstruction, transfer function, brick compositing, RGBA
// stores.  One thread per ray; a warp covers an 8x4 screen tile.
//
// Compiled with -fmad=false: every float multiply and add is rounded on its
// own, as in the reference's C, unless written as fmaf() here.  With IEEE
// division and square root (no fast-math) the REF preset reproduces the
// reference's arithmetic operation for operation.
#include <float.h>
#include <stdint.h>

#include <atomic>

#include "ivr_internal.h"

namespace ivr {
namespace {

constexpr int kBlockX = 16;  // pixels per block: 2x2 warps of 8x4
constexpr int kBlockY = 8;
constexpr int kThreads = 128;
#ifndef IVR_CFG_PAIR
#define IVR_CFG_PAIR 1  // two CONFIG samples per loop iteration
#endif
constexpr bool kPair = IVR_CFG_PAIR != 0;
// The second sample of a PAIR iteration reuses the first's corner-packed
// cell when both lie in it (for u8 and u16 volumes; IVR_CELL_REUSE=0 turns
// it off).  Measured on GB300: learned_1024 (u16) +4%; for f32 (16-byte
// elements, twice the registers per cell) the plain march lost 4% and the
// skipping march nothing, and keeping the last cell across iterations as
// well cost more in spills than it saved (sorted_brick_512 -8%).
#ifndef IVR_CELL_REUSE
#define IVR_CELL_REUSE 1
#endif
template <int DT> __host__ __device__ constexpr bool cell_reuse() { return IVR_CELL_REUSE != 0 && DT != IVR_F32; }
// Likewise its LUT entry when both samples index the same one (every dtype;
// IVR_LUT_REUSE=0 turns it off): +1-2% on learned_1024 and the plain march.
// A copy of the LUT in each block's shared memory instead of reads through
// L1 was 2-4% slower.
#ifndef IVR_LUT_REUSE
#define IVR_LUT_REUSE 1
#endif
constexpr bool kLutReuse = IVR_LUT_REUSE != 0;
// Resident blocks per SM each kernel is compiled for.  More warps hide more
// gather latency; past 8 blocks (64 registers) the compiler spills a little,
// and measured on GB300 the occupancy still wins: 9 blocks (56 registers)
// for the single-frame march, 9 (56) for the batched kernel, which reads
// its frames from global memory (835 -> 1017 Gsamples/s from 6 blocks).
#ifndef IVR_CFG_BLOCKS_PER_SM
#define IVR_CFG_BLOCKS_PER_SM 9
#endif
constexpr int kCfgBlocksPerSm = IVR_CFG_BLOCKS_PER_SM;
// judged launches (learned skipping) hold the exact march's state as well
#ifndef IVR_JUDGE_BLOCKS_PER_SM
#define IVR_JUDGE_BLOCKS_PER_SM 8
#endif
constexpr int kJudgeBlocksPerSm = IVR_JUDGE_BLOCKS_PER_SM;
#ifndef IVR_BATCH_BLOCKS_PER_SM
#define IVR_BATCH_BLOCKS_PER_SM 9
#endif
constexpr int kBatchBlocksPerSm = IVR_BATCH_BLOCKS_PER_SM;

template <int DT> struct VoxT;
template <> struct VoxT<IVR_U8> { using T = uint8_t; using V4 = uchar4; };
template <> struct VoxT<IVR_U16> { using T = uint16_t; using V4 = ushort4; };
template <> struct VoxT<IVR_F32> { using T = float; using V4 = float4; };

template <int DT>
__device__ __forceinline__ float vload(const void *p, long long i)
{
    return (float) __ldg(reinterpret_cast<const typename VoxT<DT>::T *>(p) + i);
}

// getrayintersect (ray.c:276-318).  All six planes are visited: once
// tin >= tout no later plane can make it a hit, so skipping the reference's
// early loop exit changes nothing.
// numer = d - n.o and denom = n.d for face p (normals of aabb.facenormals,
// main.c:611-613), evaluated as dot3f does.
__device__ __forceinline__ void plane_eval(int p, float dc, float ox, float oy, float oz, float dx, float dy,
                                           float dz, float &numer, float &denom)
{
    const int axis = p >> 1;
    const float nrm = (p & 1) ? 1.0f : -1.0f;
    const float nx = axis == 0 ? nrm : 0.0f, ny = axis == 1 ? nrm : 0.0f, nz = axis == 2 ? nrm : 0.0f;
    numer = dc - (nx * ox + ny * oy + nz * oz);
    denom = nx * dx + ny * dy + nz * dz;
}

__device__ __forceinline__ bool ray_box(const float *dc, float ox, float oy, float oz, float dx, float dy,
                                        float dz, float &tin, float &tout)
{
    tin = -FLT_MAX;
    tout = FLT_MAX;
#pragma unroll
    for (int p = 0; p < 6; p++) {
        float numer, denom;
        plane_eval(p, dc[p], ox, oy, oz, dx, dy, dz, numer, denom);
        if (tin < tout) {
            if (denom == 0.0f) {
                if (numer < 0.0f) tin = tout + 1.0f;
            } else {
                float thit = numer / denom;
                if (denom > 0.0f) tout = fminf(tout, thit);
                else tin = fmaxf(tin, thit);
            }
        }
    }
    return tin < tout && (tin > 0.0f || tout > 0.0f);
}

// The CONFIG slab test: ray_box's planes and visiting order, with each hit
// parameter taken as +-numer times the ray's reciprocal direction component
// (id*) instead of a division -- the CONFIG lattice's own definition; the
// REF preset keeps the reference's division.  For the axis-aligned normals
// numer = d -+ o and denom = +-d exactly, so only the rounding of the hit
// parameters differs from ray_box.
__device__ __forceinline__ bool ray_box_cfg(const float *dc, float ox, float oy, float oz, float dx, float dy,
                                            float dz, float idx, float idy, float idz, float &tin, float &tout)
{
    tin = -FLT_MAX;
    tout = FLT_MAX;
#pragma unroll
    for (int p = 0; p < 6; p++) {
        const int axis = p >> 1;
        const bool pos = (p & 1) != 0;
        const float o = axis == 0 ? ox : axis == 1 ? oy : oz;
        const float d = axis == 0 ? dx : axis == 1 ? dy : dz;
        const float id = axis == 0 ? idx : axis == 1 ? idy : idz;
        const float numer = pos ? dc[p] - o : dc[p] + o;
        if (tin < tout) {
            if (d == 0.0f) {
                if (numer < 0.0f) tin = tout + 1.0f;
            } else {
                const float thit = (pos ? numer : -numer) * id;
                if (pos ? d > 0.0f : d < 0.0f) tout = fminf(tout, thit);
                else tin = fmaxf(tin, thit);
            }
        }
    }
    return tin < tout && (tin > 0.0f || tout > 0.0f);
}

// getlinearsample (ray.c:87-181, non-BGQ branch), quirks included: the
// weights are scaled by the cell size squared, and the x weight blends the
// +1 row (y) neighbour.  x + fabs(min.x) is a double sum in the reference,
// which rounds to the same float as this float sum.
template <int DT>
__device__ __forceinline__ float sample_ref(const DevBrick &b, float x, float y, float z)
{
    const int vw = b.nx, vh = b.ny, vd = b.nz;
    float ratio = (x - b.bminx) / b.w;
    int j = (int) ((float) vw * ratio);
    ratio = (y - b.bminy) / b.h;
    int i = (int) ((float) vh * ratio);
    ratio = (z - b.bminz) / b.d;
    int k = (int) ((float) vd * ratio);
    i = min(i, vh - 2);
    j = min(j, vw - 2);
    k = min(k, vd - 2);
    i = max(i, 0);  // no lower clamp in the reference; guards memory only
    j = max(j, 0);
    k = max(k, 0);
    const long long row = vw, slab = (long long) vw * vh;
    const long long p = k * slab + i * row + j;
    float v000 = vload<DT>(b.data, p);
    float v100 = vload<DT>(b.data, p + row);
    float v010 = vload<DT>(b.data, p + 1);
    float v001 = vload<DT>(b.data, p + slab);
    float v101 = vload<DT>(b.data, p + row + slab);
    float v011 = vload<DT>(b.data, p + 1 + slab);
    float v110 = vload<DT>(b.data, p + row + 1);
    float v111 = vload<DT>(b.data, p + row + 1 + slab);
    float xp = x + fabsf(b.bminx), yp = y + fabsf(b.bminy), zp = z + fabsf(b.bminz);
    float x0 = ((float) j * b.w) / (float) vw;
    float y0 = ((float) i * b.h) / (float) vh;
    float z0 = ((float) k * b.d) / (float) vd;
    float xd = (fabsf(xp - x0) * b.w) / (float) vw;
    float yd = (fabsf(yp - y0) * b.h) / (float) vh;
    float zd = (fabsf(zp - z0) * b.d) / (float) vd;
    float c00 = v000 * (1.0f - xd) + v100 * xd;
    float c10 = v010 * (1.0f - xd) + v110 * xd;
    float c01 = v001 * (1.0f - xd) + v101 * xd;
    float c11 = v011 * (1.0f - xd) + v111 * xd;
    float c0 = c00 * (1.0f - yd) + c10 * yd;
    float c1 = c01 * (1.0f - yd) + c11 * yd;
    return c0 * (1.0f - zd) + c1 * zd;
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }

// CONFIG sampler: trilinear with voxel values at cell corners (the
// reference's index convention; the halo sits on the high side), clamp to
// edge, at a position (ux, uy, uz) in the brick's voxel coordinates (voxel
// (j, i, k) at u = (j, i, k)).  Split in two so that the march's macrocell
// check can use the cell coordinates of the sample it is about to take.
struct CellPos {
    int j, i, k;         // voxel cell, clamped to [0, n-2]
    float fx, fy, fz;    // position in it, [0, 1]
};

__device__ __forceinline__ CellPos cell_cfg(const DevBrick &b, float ux, float uy, float uz)
{
    const int nx = b.nx, ny = b.ny, nz = b.nz;
    // clamp to edge: the coordinate to [0, n-1], the cell to [0, n-2]; then
    // the fraction u - floor(u) is exact and lies in [0, 1] (this gives the
    // same cell and fraction as clamping the cell and then the fraction)
    ux = fminf(fmaxf(ux, 0.0f), (float) (nx - 1));
    uy = fminf(fmaxf(uy, 0.0f), (float) (ny - 1));
    uz = fminf(fmaxf(uz, 0.0f), (float) (nz - 1));
    CellPos c;
    c.j = min(__float2int_rd(ux), nx - 2);
    c.i = min(__float2int_rd(uy), ny - 2);
    c.k = min(__float2int_rd(uz), nz - 2);
    c.fx = ux - (float) c.j;
    c.fy = uy - (float) c.i;
    c.fz = uz - (float) c.k;
    return c;
}

// Packed integer voxels without conversion instructions (which run on a
// narrow pipe; eight per sample made the u8/u16 corner-packed sampler
// conversion-bound): a u8 or u16 lane placed in the low mantissa bits under
// the exponent of 2^23 is the float 2^23 + v, exactly.  lerp23 is lerpf on
// two such values: B - A is b - a and A - 2^23 is a, both exact, so the
// result is lerpf(a, b, t) bit for bit.  (For the brick's own voxels, one
// load each, the conversion is cheaper than the permute and the offset.)
__device__ __forceinline__ float off23(unsigned v, unsigned sel)
{
    return __int_as_float(__byte_perm(v, 0x4B000000u, sel));
}
__device__ __forceinline__ float lerp23(float A, float B, float t) { return fmaf(t, B - A, A - 8388608.0f); }
// byte_perm selectors: u8 lane n of a word, u16 half n of a word, each with
// 0x4B in the top byte and zeros between
constexpr unsigned kU8Lane0 = 0x7540u, kU8Lane1 = 0x7541u, kU8Lane2 = 0x7542u, kU8Lane3 = 0x7543u;
constexpr unsigned kU16Half0 = 0x7410u, kU16Half1 = 0x7432u;

template <int DT>
__device__ __forceinline__ float fetch_cfg(const DevBrick &b, const CellPos &c)
{
    const int nx = b.nx, ny = b.ny;
    const int j = c.j, i = c.i, k = c.k;
    const float fx = c.fx, fy = c.fy, fz = c.fz;
    float c00, c10, c01, c11;
    if (b.quad) {
        // corner-packed copy: the cell's 8 voxels in two vector loads
        using V = typename VoxT<DT>::V4;
        const unsigned qx = (unsigned) nx - 1u, qs = qx * ((unsigned) ny - 1u);
        const V *e = reinterpret_cast<const V *>(b.quad) + ((unsigned) k * qs + (unsigned) i * qx + (unsigned) j);
        if (DT == IVR_U8) {
            // one word per element: lanes (j, i), (j+1, i), (j, i+1), (j+1, i+1)
            const unsigned lo = __ldg(reinterpret_cast<const unsigned *>(e));
            const unsigned hi = __ldg(reinterpret_cast<const unsigned *>(e + qs));
            c00 = lerp23(off23(lo, kU8Lane0), off23(lo, kU8Lane1), fx);
            c10 = lerp23(off23(lo, kU8Lane2), off23(lo, kU8Lane3), fx);
            c01 = lerp23(off23(hi, kU8Lane0), off23(hi, kU8Lane1), fx);
            c11 = lerp23(off23(hi, kU8Lane2), off23(hi, kU8Lane3), fx);
        } else if (DT == IVR_U16) {
            // two words per element, two lanes each
            const uint2 lo = __ldg(reinterpret_cast<const uint2 *>(e));
            const uint2 hi = __ldg(reinterpret_cast<const uint2 *>(e + qs));
            c00 = lerp23(off23(lo.x, kU16Half0), off23(lo.x, kU16Half1), fx);
            c10 = lerp23(off23(lo.y, kU16Half0), off23(lo.y, kU16Half1), fx);
            c01 = lerp23(off23(hi.x, kU16Half0), off23(hi.x, kU16Half1), fx);
            c11 = lerp23(off23(hi.y, kU16Half0), off23(hi.y, kU16Half1), fx);
        } else if (kQuadDelta) {
            // (v0, v1 - v0) pairs: the x lerps without their subtraction
            const V lo = __ldg(e), hi = __ldg(e + qs);
            c00 = fmaf(fx, (float) lo.y, (float) lo.x);
            c10 = fmaf(fx, (float) lo.w, (float) lo.z);
            c01 = fmaf(fx, (float) hi.y, (float) hi.x);
            c11 = fmaf(fx, (float) hi.w, (float) hi.z);
        } else {
            const V lo = __ldg(e), hi = __ldg(e + qs);
            c00 = lerpf((float) lo.x, (float) lo.y, fx);
            c10 = lerpf((float) lo.z, (float) lo.w, fx);
            c01 = lerpf((float) hi.x, (float) hi.y, fx);
            c11 = lerpf((float) hi.z, (float) hi.w, fx);
        }
    } else {
        // one pointer to the cell's low corner (a brick holds fewer than
        // 2^32 voxels, checked at load, so its offset fits 32 bits); the
        // other corners are whole rows (nx) and slabs (nx*ny) away, the +1
        // neighbours an immediate offset
        using T = typename VoxT<DT>::T;
        const unsigned sz = (unsigned) nx * (unsigned) ny;
        const T *q0 = reinterpret_cast<const T *>(b.data) + ((unsigned) k * sz + (unsigned) i * (unsigned) nx + (unsigned) j);
        const T *q1 = q0 + nx, *q2 = q0 + sz, *q3 = q2 + nx;
        c00 = lerpf((float) __ldg(q0), (float) __ldg(q0 + 1), fx);
        c10 = lerpf((float) __ldg(q1), (float) __ldg(q1 + 1), fx);
        c01 = lerpf((float) __ldg(q2), (float) __ldg(q2 + 1), fx);
        c11 = lerpf((float) __ldg(q3), (float) __ldg(q3 + 1), fx);
    }
    float c0 = lerpf(c00, c10, fy);
    float c1 = lerpf(c01, c11, fy);
    return lerpf(c0, c1, fz);
}

template <int DT>
__device__ __forceinline__ float sample_cfg(const DevBrick &b, float ux, float uy, float uz)
{
    return fetch_cfg<DT>(b, cell_cfg(b, ux, uy, uz));
}

// One voxel cell of a corner-packed copy as loaded: the two elements (slab
// k and k+1), each holding the cell's four voxels of that slab.  A ray
// stepping half a voxel takes its next sample in the same cell about half
// the time; the march keeps the last cell it loaded, with its element
// offset as the key, and loads again only when the cell changes.  The
// values are the same voxels, so every sample is bitwise unchanged.
template <int DT> struct QuadCell;
template <> struct QuadCell<IVR_U8> { unsigned lo, hi; };
template <> struct QuadCell<IVR_U16> { uint2 lo, hi; };
template <> struct QuadCell<IVR_F32> { float4 lo, hi; };

// element offset of cell c in the corner-packed copy (unique per cell)
__device__ __forceinline__ unsigned quad_key(const DevBrick &b, const CellPos &c)
{
    const unsigned qx = (unsigned) b.nx - 1u, qs = qx * ((unsigned) b.ny - 1u);
    return (unsigned) c.k * qs + (unsigned) c.i * qx + (unsigned) c.j;
}

template <int DT>
__device__ __forceinline__ QuadCell<DT> quad_load(const DevBrick &b, unsigned key)
{
    using E = decltype(QuadCell<DT>::lo);
    const unsigned qs = ((unsigned) b.nx - 1u) * ((unsigned) b.ny - 1u);
    const E *e = reinterpret_cast<const E *>(b.quad) + key;
    QuadCell<DT> q;
    q.lo = __ldg(e);
    q.hi = __ldg(e + qs);
    return q;
}

// fetch_cfg's corner-packed interpolation on a loaded cell
template <int DT>
__device__ __forceinline__ float quad_interp(const QuadCell<DT> &q, const CellPos &c)
{
    float c00, c10, c01, c11;
    if constexpr (DT == IVR_U8) {
        c00 = lerp23(off23(q.lo, kU8Lane0), off23(q.lo, kU8Lane1), c.fx);
        c10 = lerp23(off23(q.lo, kU8Lane2), off23(q.lo, kU8Lane3), c.fx);
        c01 = lerp23(off23(q.hi, kU8Lane0), off23(q.hi, kU8Lane1), c.fx);
        c11 = lerp23(off23(q.hi, kU8Lane2), off23(q.hi, kU8Lane3), c.fx);
    } else if constexpr (DT == IVR_U16) {
        c00 = lerp23(off23(q.lo.x, kU16Half0), off23(q.lo.x, kU16Half1), c.fx);
        c10 = lerp23(off23(q.lo.y, kU16Half0), off23(q.lo.y, kU16Half1), c.fx);
        c01 = lerp23(off23(q.hi.x, kU16Half0), off23(q.hi.x, kU16Half1), c.fx);
        c11 = lerp23(off23(q.hi.y, kU16Half0), off23(q.hi.y, kU16Half1), c.fx);
    } else if (kQuadDelta) {
        c00 = fmaf(c.fx, q.lo.y, q.lo.x);
        c10 = fmaf(c.fx, q.lo.w, q.lo.z);
        c01 = fmaf(c.fx, q.hi.y, q.hi.x);
        c11 = fmaf(c.fx, q.hi.w, q.hi.z);
    } else {
        c00 = lerpf(q.lo.x, q.lo.y, c.fx);
        c10 = lerpf(q.lo.z, q.lo.w, c.fx);
        c01 = lerpf(q.hi.x, q.hi.y, c.fx);
        c11 = lerpf(q.hi.z, q.hi.w, c.fx);
    }
    const float c0 = lerpf(c00, c10, c.fy);
    const float c1 = lerpf(c01, c11, c.fy);
    return lerpf(c0, c1, c.fz);
}

// A ray's CONFIG lattice in a brick's voxel coordinates: lattice index i
// samples u_i = fmaf(i, s, base) per axis, with s = (d * ic) * dt and
// base = fmaf(d * ic, t0, (o - bmin) * ic) -- the point o + t_i d, t_i =
// t0 + i dt, mapped by the brick's world-to-voxel scaling ic.  Three fmaf
// per sample instead of the lattice parameter, the world point and its
// mapping.
struct VoxLattice {
    float sx, sy, sz;
    float bx, by, bz;
};

__device__ __forceinline__ VoxLattice vox_lattice(const DevBrick &b, float ox, float oy, float oz, float dx,
                                                  float dy, float dz, float t0, float dt)
{
    const float ux = dx * b.icx, uy = dy * b.icy, uz = dz * b.icz;
    VoxLattice L;
    L.sx = ux * dt;
    L.sy = uy * dt;
    L.sz = uz * dt;
    L.bx = fmaf(ux, t0, (ox - b.bminx) * b.icx);
    L.by = fmaf(uy, t0, (oy - b.bminy) * b.icy);
    L.bz = fmaf(uz, t0, (oz - b.bminz) * b.icz);
    return L;
}

__device__ __forceinline__ float4 lut_at(const FrameDesc &f, int idx)
{
    idx = min(max(idx, 0), f.lut_n - 1);
    return __ldg(f.lut + idx);
}

// raycast (ray.c:59-85) + getsamplesonray (ray.c:239-273) + one transfer
// function of transferfuncs.c:24-199.  Samples are computed in the order the
// transfer function consumes them (ascending or descending) instead of
// being stored.  Returns (r, g, b, a).
template <int DT, int TF>
__device__ float4 raycast_ref(const FrameDesc &f, const DevBrick &b, float dx, float dy, float dz,
                              unsigned long long &nexec)
{
    float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float tin, tout;
    if (!ray_box(b.dconst, f.origx, f.origy, f.origz, dx, dy, dz, tin, tout)) return c;
    const float dt = f.step;
    int iend = (int) (1.0f + (tout - tin) / dt + 0.5f);
    if (f.max_samples > 0 && iend > f.max_samples) iend = f.max_samples;
    if (iend <= 0) return c;
    nexec += (unsigned long long) iend;
    const float ox = f.origx, oy = f.origy, oz = f.origz;
    const float myalpha = f.alpha;
    auto sample = [&](int i) {
        float t = tin + ((float) i * dt);
        return sample_ref<DT>(b, dx * t + ox, dy * t + oy, dz * t + oz);
    };
    if (TF == IVR_TF_MED) {  // transferfuncs.c:24-68
        for (int i = 0; i < iend; ++i) {
            float4 e = lut_at(f, (int) sample(i) - f.lut_off);
            c.z = ((double) e.z < 0.8) ? fmaxf(e.z, c.z) : c.z;
            c.y = ((double) e.y < 0.8) ? fmaxf(e.y, c.y) : c.y;
            c.x = ((double) e.x < 0.8) ? fmaxf(e.x, c.x) : c.x;
            c.w = e.w * myalpha;
        }
    } else if (TF == IVR_TF_BLEND) {  // transferfuncs.c:70-83 (no lutoffset)
        for (int i = 0; i < iend; ++i) {
            float4 e = lut_at(f, (int) sample(i));
            float al = e.w;
            c.z = al * e.z + (1.0f - al) * c.z;
            c.y = al * e.y + (1.0f - al) * c.y;
            c.x = al * e.x + (1.0f - al) * c.x;
            c.w = al * myalpha;
        }
    } else if (TF == IVR_TF_SEISMIC2 || TF == IVR_TF_CHEM) {  // transferfuncs.c:109-168
        for (int i = iend - 1; i >= 0; i--) {
            int idx = (int) sample(i) - f.lut_off;
            if (idx < 0) idx = 0;
            if (TF == IVR_TF_SEISMIC2 && idx > f.lut_n - 1) idx = f.lut_n - 1;
            float4 e = lut_at(f, idx);
            float al = e.w * myalpha;
            float oma = 1.0f - al;
            c.z = oma * c.z + al * e.z;
            c.y = oma * c.y + al * e.y;
            c.x = oma * c.x + al * e.x;
            c.w = al + oma * c.w;
            if (c.w > 1.0f) c.w = 1.0f;
        }
    } else if (TF == IVR_TF_RGBBLEND) {  // transferfuncs.c:170-200
        for (int i = iend - 1; i >= 0; i--) {
            unsigned u = __float_as_uint(sample(i));
            float r = 1.0f / 255.0f * (float) ((u >> 24) & 0xff);
            float g = 1.0f / 255.0f * (float) ((u >> 16) & 0xff);
            float bl = 1.0f / 255.0f * (float) ((u >> 8) & 0xff);
            float al = myalpha;
            float oma = 1.0f - al;
            c.z = oma * c.z + al * bl;
            c.y = oma * c.y + al * g;
            c.x = oma * c.x + al * r;
            c.w = al + oma * c.w;
            if (c.w > 1.0f) c.w = 1.0f;
        }
    } else {  // IVR_TF_SEISMIC, transferfuncs.c:86-107
        for (int i = 0; i < iend; ++i) {
            float4 e = lut_at(f, (int) sample(i) - f.lut_off);
            c.z = ((double) e.z > 0.65 && e.z < 1.0f) ? 0.6f : c.z;
            c.y = ((double) e.y > 0.65 && e.y < 1.0f) ? 0.0f : c.y;
            c.x = ((double) e.x > 0.65 && e.x < 1.0f) ? 0.0f : c.x;
            c.z = ((double) e.z > 0.5 && e.z < 0.65f) ? 0.9f : c.z;
            c.y = ((double) e.y > 0.5 && e.y < 0.65f) ? 0.9f : c.y;
            c.x = ((double) e.x > 0.5 && e.x < 0.65f) ? 0.9f : c.x;
            c.z = ((double) e.z > 0.3 && e.z < 0.5f) ? 0.0f : c.z;
            c.y = ((double) e.y > 0.3 && e.y < 0.5f) ? 0.0f : c.y;
            c.x = ((double) e.x > 0.3 && e.x < 0.5f) ? 0.6f : c.x;
            c.w = 1.0f * myalpha;
        }
    }
    return c;
}

// compositetiles (main.c:1206-1215): d = s + (1 - s.a) * d
__device__ __forceinline__ float4 over(float4 s, float4 d)
{
    d.z = s.z + (1.0f - s.w) * d.z;
    d.y = s.y + (1.0f - s.w) * d.y;
    d.x = s.x + (1.0f - s.w) * d.x;
    d.w = s.w + (1.0f - s.w) * d.w;
    return d;
}

// (uint8)(v*255 + 0.5) for v in [0,1], exact: for v = m * 2^(e-150) the
// value is floor((255 m + 2^(s-1)) / 2^s) with s = 150 - e.
__device__ __forceinline__ unsigned q8(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 1.0f) return 255u;
    unsigned bits = __float_as_uint(v);
    int e = (int) (bits >> 23);
    if (e == 0) return 0u;  // subnormal: far below 1/510
    unsigned long long m = (bits & 0x7fffffu) | 0x800000u;
    int s = 150 - e;
    if (s >= 34) return 0u;
    return (unsigned) ((255ull * m + (1ull << (s - 1))) >> s);
}

__device__ __forceinline__ bool in_rect(const DevBrick &b, int i, int j)
{
    return i >= b.istrt && i < b.istop && j >= b.jstrt && j < b.jstop;
}

// CONFIG lattice: t_i = fmaf(i, dt, t0).
__device__ __forceinline__ float cfg_t(float t0, float dt, int i) { return fmaf((float) i, dt, t0); }
// First lattice index i >= 0 with t_i >= a.  The estimate is exact up to
// rounding, so the fix-up loops run a step or two; they are bounded anyway.
constexpr int kMaxLattice = 1 << 24;
__device__ __forceinline__ int cfg_first_ge(float t0, float dt, float idt, float a)
{
    if (!(a > t0)) return 0;
    float q = (a - t0) * idt;  // an estimate: the loops below make it exact
    int i = q < (float) kMaxLattice ? (int) q : kMaxLattice;
    for (int it = 0; it < 64 && i > 0 && cfg_t(t0, dt, i - 1) >= a; it++) i--;
    for (int it = 0; it < 64 && i < kMaxLattice && cfg_t(t0, dt, i) < a; it++) i++;
    return i;
}


// One brick of the CONFIG march: samples tin_k <= t_i < tout_k of the ray's
// lattice, front-to-back into acc.  One loop iteration takes one lattice
// index (two with PAIR) for every lane, so the lanes of a warp stay in step.
// With a macrocell grid a lane checks the cell of its sample (by the same
// index arithmetic the sampler uses) only when it passes the exit of the last
// opaque cell it checked.  A transparent cube's samples are stepped over to
// just past its exit (or to two samples before it, where rounding at a face
// leaves the last one in doubt), and successive cubes are leapt within the
// same iteration; each skipped sample lies in a transparent cell, so it would
// have had zero opacity and left acc unchanged.  An opaque cell's samples are
// taken up to one past its exit without further checks.  Every sample that is
// taken is computed exactly as without skipping.
template <int DT, bool SKIP, bool CENSUS, bool PAIR>
__device__ void march_cfg(const FrameDesc &f, const DevBrick &b, const uint8_t *empty, float dx, float dy, float dz,
                          float idx, float idy, float idz, float t0, float dt, float idt, float4 &acc, bool &done,
                          unsigned long long &nexec, unsigned long long &nlat)
{
    float tin, tout;
    if (!ray_box_cfg(b.dconst, f.origx, f.origy, f.origz, dx, dy, dz, idx, idy, idz, tin, tout)) return;
    const int i0 = cfg_first_ge(t0, dt, idt, tin);
    const int i1 = cfg_first_ge(t0, dt, idt, tout);
    if (CENSUS) {
        nlat += (unsigned long long) max(i1 - i0, 0);
        if (done) return;
    }
    const float opac = f.alpha, term = f.term_alpha;
    const VoxLattice L = vox_lattice(b, f.origx, f.origy, f.origz, dx, dy, dz, t0, dt);
    // lattice steps per voxel (about 1 / L.s), for the exits of transparent
    // cubes
    const float isx = idx * idt * b.vwx, isy = idy * idt * b.vwy, isz = idz * idt * b.vwz;
    int icheck = i0;  // next lattice index whose cell must be checked
    for (int i = i0; i < i1; i++) {
        float fi = (float) i;
        CellPos c0 = cell_cfg(b, fmaf(fi, L.sx, L.bx), fmaf(fi, L.sy, L.by), fmaf(fi, L.sz, L.bz));
        // A lane leaps over transparent cubes within one iteration, until
        // its sample lies in an opaque cell (or the brick ends), so that it
        // samples beside the lanes that did not leap.  Every leap moves i
        // forward and an opaque check leaves the loop, so it ends.
        if (SKIP && i >= icheck) for (;;) {
            // the sample's macrocell: its voxel cell (the sampler's own index
            // arithmetic) over the macrocell edge (cells are never negative:
            // the sampler clamps them)
            const int cs = b.cshift, edge = 1 << cs;
            const int cj = c0.j >> cs, ci = c0.i >> cs, ck = c0.k >> cs;
            // r >= 1: the cube of cells within r-1 of this one is transparent
            const int r = empty[(ck * b.mcy + ci) * b.mcx + cj];
            const int rr = max(r, 1);
            // the voxel plane of the face through which the ray leaves that
            // cube (or this one opaque cell), per axis, and the lattice index
            // of the exit; approximate, the margins absorb its rounding
            const float fx = (float) ((L.sx > 0.0f ? cj + rr : cj - rr + 1) * edge);
            const float fy = (float) ((L.sy > 0.0f ? ci + rr : ci - rr + 1) * edge);
            const float fz = (float) ((L.sz > 0.0f ? ck + rr : ck - rr + 1) * edge);
            const float qx = L.sx != 0.0f ? (fx - L.bx) * isx : FLT_MAX;
            const float qy = L.sy != 0.0f ? (fy - L.by) * isy : FLT_MAX;
            const float qz = L.sz != 0.0f ? (fz - L.bz) * isz : FLT_MAX;
            const float q = fminf(fmaxf(fminf(qx, fminf(qy, qz)), 0.0f), (float) kMaxLattice);
            const int iexit = (int) q;  // last lattice index at or before the exit
            if (r != 0) {
                // Leap.  Sample positions are monotone in the lattice index
                // along each axis and sample i lies in the cube, so when the
                // last one before the exit (iexit) is still short of every
                // exit face, so is every sample up to it: all are in the
                // transparent cube, and the march resumes just past the
                // exit.  Otherwise (rounding at a face) it resumes two
                // samples earlier, where the next check looks again.
                const float fe = (float) iexit;
                const float ex = fmaf(fe, L.sx, L.bx), ey = fmaf(fe, L.sy, L.by), ez = fmaf(fe, L.sz, L.bz);
                const bool inside = (L.sx > 0.0f ? ex < fx : L.sx < 0.0f ? ex >= fx : true) &&
                                    (L.sy > 0.0f ? ey < fy : L.sy < 0.0f ? ey >= fy : true) &&
                                    (L.sz > 0.0f ? ez < fz : L.sz < 0.0f ? ez >= fz : true);
                i = max(i, inside ? iexit : iexit - 2) + 1;  // iexit + 1 or iexit - 1
                if (i >= i1) break;
                fi = (float) i;
                c0 = cell_cfg(b, fmaf(fi, L.sx, L.bx), fmaf(fi, L.sy, L.by), fmaf(fi, L.sz, L.bz));
                continue;
            }
            icheck = iexit + 1;
            break;
        }
        if (SKIP && i >= i1) break;
        // PAIR: two samples per iteration, both samples' loads in flight
        // before either is composited.  The second is only composited when
        // it comes before the next cell check and the first did not end the
        // ray; sample_cfg clamps its indices, so computing it is always safe.
        if (PAIR && !CENSUS) {
            const int lim = SKIP ? min(i1, icheck) : i1;
            const float f1 = fi + 1.0f;  // (float) (i + 1): i < 2^24
            float s0, s1;
            if (cell_reuse<DT>() && b.quad) {
                const CellPos c1 = cell_cfg(b, fmaf(f1, L.sx, L.bx), fmaf(f1, L.sy, L.by), fmaf(f1, L.sz, L.bz));
                const unsigned k0 = quad_key(b, c0), k1 = quad_key(b, c1);
                const QuadCell<DT> q0 = quad_load<DT>(b, k0);
                QuadCell<DT> q1 = q0;
                if (k1 != k0) q1 = quad_load<DT>(b, k1);
                s0 = quad_interp<DT>(q0, c0);
                s1 = quad_interp<DT>(q1, c1);
            } else {
                s0 = fetch_cfg<DT>(b, c0);
                s1 = sample_cfg<DT>(b, fmaf(f1, L.sx, L.bx), fmaf(f1, L.sy, L.by), fmaf(f1, L.sz, L.bz));
            }
            const int x0 = (int) (s0 * f.lut_scale) - f.lut_off, x1 = (int) (s1 * f.lut_scale) - f.lut_off;
            const float4 e0 = lut_at(f, x0);
            float4 e1 = e0;
            if (!kLutReuse || x1 != x0) e1 = lut_at(f, x1);  // the same entry: no second load
            float wgt = (1.0f - acc.w) * (e0.w * opac);
            acc.x = fmaf(wgt, e0.x, acc.x);
            acc.y = fmaf(wgt, e0.y, acc.y);
            acc.z = fmaf(wgt, e0.z, acc.z);
            acc.w = acc.w + wgt;
            if (acc.w >= term) {
                done = true;
                return;
            }
            if (i + 1 < lim) {
                wgt = (1.0f - acc.w) * (e1.w * opac);
                acc.x = fmaf(wgt, e1.x, acc.x);
                acc.y = fmaf(wgt, e1.y, acc.y);
                acc.z = fmaf(wgt, e1.z, acc.z);
                acc.w = acc.w + wgt;
                if (acc.w >= term) {
                    done = true;
                    return;
                }
                i++;
            }
            continue;
        }
        const float s = fetch_cfg<DT>(b, c0);
        if (CENSUS) {
            nexec++;
            b.touched[((long long) (c0.k >> b.cshift) * b.mcy + (c0.i >> b.cshift)) * b.mcx + (c0.j >> b.cshift)] = 1;
        }
        const float4 e = lut_at(f, (int) (s * f.lut_scale) - f.lut_off);
        const float al = e.w * opac;
        const float wgt = (1.0f - acc.w) * al;
        acc.x = fmaf(wgt, e.x, acc.x);
        acc.y = fmaf(wgt, e.y, acc.y);
        acc.z = fmaf(wgt, e.z, acc.z);
        acc.w = acc.w + wgt;
        if (acc.w >= term) {
            done = true;
            return;
        }
    }
}

__device__ __forceinline__ void count_exec(const FrameDesc &f, unsigned long long nexec,
                                           unsigned long long nlat = 0)
{
    if (f.counters == nullptr) return;
    // every lane of the warp reaches here (out-of-range pixels store
    // nothing but still count zero)
    for (int o = 16; o > 0; o >>= 1) {
        nexec += __shfl_xor_sync(0xffffffffu, nexec, o);
        nlat += __shfl_xor_sync(0xffffffffu, nlat, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(f.counters, nexec);
        if (nlat) atomicAdd(f.counters + 1, nlat);
    }
}

__device__ __forceinline__ void pixel_of(const FrameDesc &f, int &i, int &j, int &oi, int &oj)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    oj = blockIdx.x * kBlockX + (warp & 1) * 8 + (lane & 7);
    oi = blockIdx.y * kBlockY + (warp >> 1) * 4 + (lane >> 3);
    j = f.out_x + oj;
    i = f.out_y + oi;
}

template <int DT, int TF>
__global__ void __launch_bounds__(kThreads) march_ref_kernel(const __grid_constant__ FrameDesc f, float4 *out32,
                                                             uchar4 *out8)
{
    int i, j, oi, oj;
    pixel_of(f, i, j, oi, oj);
    const bool inside = oj < f.out_w && oi < f.out_h;
    float4 d = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    unsigned long long nexec = 0;
    if (inside && i < f.vh && j < f.vw) {
        // far -> near over of per-brick colours; each brick casts its own ray
        // with the sequential column increments of createlocalimage
        // (main.c:986-999)
        for (int s = f.nb - 1; s >= 0; s--) {
            const int k = f.order[s];
            if (f.single >= 0 && k != f.single) continue;
            const DevBrick &b = f.b[k];
            if (!in_rect(b, i, j)) continue;
            const float fi = (float) (i - b.istrt);
            float dx = b.dir0x + f.incrix * fi, dy = b.dir0y + f.incriy * fi, dz = b.dir0z + f.incriz * fi;
            for (int c = b.jstrt; c <= j; c++) {
                dx += f.incrjx;
                dy += f.incrjy;
                dz += f.incrjz;
            }
            float4 cs = raycast_ref<DT, TF>(f, b, dx, dy, dz, nexec);
            d = over(cs, d);
        }
    }
    if (inside) {
        const long long o = (long long) oi * f.out_w + oj;
        if (out32) out32[o] = d;
        if (out8) out8[o] = make_uchar4(q8(d.x), q8(d.y), q8(d.z), q8(d.w));
    }
    count_exec(f, nexec);
}

// One CONFIG ray: pixel (i, j) of the viewport, all bricks front to back,
// skipping by the bricks' grids, or by the exact grids f.exact when exact.
template <int DT, bool SKIP, bool CENSUS, bool PAIR>
__device__ __forceinline__ float4 ray_cfg(const FrameDesc &f, int i, int j, unsigned long long &nexec,
                                          unsigned long long &nlat, bool exact = false)
{
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool any = false;
    for (int k = 0; k < f.nb; k++) any |= in_rect(f.b[k], i, j);
    if (!any) return acc;
    // ctm * (u, v, 5) at the pixel centre
    const float u = f.left + ((float) j + 0.5f) * f.du;
    const float v = f.bottom + ((float) i + 0.5f) * f.dv;
    const float dx = f.ctm[0] * u + f.ctm[1] * v + f.ctm[2] * f.eyen;
    const float dy = f.ctm[3] * u + f.ctm[4] * v + f.ctm[5] * f.eyen;
    const float dz = f.ctm[6] * u + f.ctm[7] * v + f.ctm[8] * f.eyen;
    const float idx = 1.0f / dx, idy = 1.0f / dy, idz = 1.0f / dz;
    float tin, tout;
    if (!ray_box_cfg(f.gdconst, f.origx, f.origy, f.origz, dx, dy, dz, idx, idy, idz, tin, tout)) return acc;
    const float t0 = tin > 0.0f ? tin : 0.0f;
    const float len = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
    const float dt = f.step / len;
    bool done = !(dt > 0.0f);
    const float idt = 1.0f / dt;
    for (int s = 0; s < f.nb && (CENSUS || !done); s++) {
        const int k = f.order[s];
        if (f.single >= 0 && k != f.single) continue;
        const DevBrick &b = f.b[k];
        if (!in_rect(b, i, j)) continue;
        const uint8_t *empty = exact ? f.exact[k] : b.empty;
        if (SKIP && empty != nullptr)
            march_cfg<DT, true, CENSUS, PAIR>(f, b, empty, dx, dy, dz, idx, idy, idz, t0, dt, idt, acc, done, nexec,
                                              nlat);
        else
            march_cfg<DT, false, CENSUS, PAIR>(f, b, empty, dx, dy, dz, idx, idy, idz, t0, dt, idt, acc, done, nexec,
                                               nlat);
    }
    return acc;
}

// One pixel of the output window (ow, oh) = (oj, oi).
template <int DT, bool SKIP, bool CENSUS, bool PAIR>
__device__ __forceinline__ float4 pixel_cfg(const FrameDesc &f, int oi, int oj, float4 *out32, uchar4 *out8,
                                            unsigned long long &nexec, unsigned long long &nlat, bool exact = false)
{
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (oj >= f.out_w || oi >= f.out_h) return acc;
    const int j = f.out_x + oj, i = f.out_y + oi;
    if (i < f.vh && j < f.vw) acc = ray_cfg<DT, SKIP, CENSUS, PAIR>(f, i, j, nexec, nlat, exact);
    const long long o = (long long) oi * f.out_w + oj;
    if (out32) out32[o] = acc;
    if (out8) out8[o] = make_uchar4(q8(acc.x), q8(acc.y), q8(acc.z), q8(acc.w));
    return acc;
}

// Estimated cost of one CONFIG ray, in samples: a walk over the bricks'
// macrocell grids front to back, cell by cell, with no volume reads.  A
// transparent cube (the grid's distance field) costs one step, as the
// march's leap over it does; an opaque cell costs the lattice points it
// holds, and its mean LUT opacity (b.opac) lowers the ray's estimated
// transmittance, so that the walk stops about where early termination
// would.  Only the order of tiles depends on it, never a pixel.
__device__ float ray_cost(const FrameDesc &f, int i, int j)
{
    bool any = false;
    for (int k = 0; k < f.nb; k++) any |= in_rect(f.b[k], i, j);
    if (!any) return 0.0f;
    const float u = f.left + ((float) j + 0.5f) * f.du;
    const float v = f.bottom + ((float) i + 0.5f) * f.dv;
    const float dx = f.ctm[0] * u + f.ctm[1] * v + f.ctm[2] * f.eyen;
    const float dy = f.ctm[3] * u + f.ctm[4] * v + f.ctm[5] * f.eyen;
    const float dz = f.ctm[6] * u + f.ctm[7] * v + f.ctm[8] * f.eyen;
    const float idx = 1.0f / dx, idy = 1.0f / dy, idz = 1.0f / dz;
    float tin, tout;
    if (!ray_box_cfg(f.gdconst, f.origx, f.origy, f.origz, dx, dy, dz, idx, idy, idz, tin, tout)) return 0.0f;
    const float t0 = tin > 0.0f ? tin : 0.0f;
    const float dt = f.step / sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
    if (!(dt > 0.0f)) return 0.0f;
    const float idt = 1.0f / dt;
    const float ox = f.origx, oy = f.origy, oz = f.origz;
    // log2 of the transmittance where the march stops
    const float lstop = f.term_alpha < 1.0f ? __log2f(1.0f - f.term_alpha) : -FLT_MAX;
    float lt = 0.0f, cost = 0.0f;
    for (int s = 0; s < f.nb; s++) {
        const int k = f.order[s];
        if (f.single >= 0 && k != f.single) continue;
        const DevBrick &b = f.b[k];
        if (!in_rect(b, i, j)) continue;
        float ta, tb;
        if (!ray_box_cfg(b.dconst, ox, oy, oz, dx, dy, dz, idx, idy, idz, ta, tb)) continue;
        float t = fmaxf(ta, t0);
        if (b.empty == nullptr || b.opac == nullptr) {
            cost += fmaxf(tb - t, 0.0f) * idt;
            continue;
        }
        for (int it = 0; it < 4096 && t < tb; it++) {
            // the cell a quarter step past t (the march's index arithmetic)
            const float tm = fmaf(0.25f, dt, t);
            const int cj = min(max((int) floorf((fmaf(dx, tm, ox) - b.bminx) * b.icx), 0), b.nx - 2) >> b.cshift;
            const int ci = min(max((int) floorf((fmaf(dy, tm, oy) - b.bminy) * b.icy), 0), b.ny - 2) >> b.cshift;
            const int ck = min(max((int) floorf((fmaf(dz, tm, oz) - b.bminz) * b.icz), 0), b.nz - 2) >> b.cshift;
            const long long c = ((long long) ck * b.mcy + ci) * b.mcx + cj;
            const int r = b.empty[c];
            const int oq = b.opac[c];
            const int rr = max(r, 1);
            const float tx = dx > 0.0f ? (fmaf((float) (cj + rr), b.mcwx, b.bminx) - ox) * idx
                             : dx < 0.0f ? (fmaf((float) (cj - rr + 1), b.mcwx, b.bminx) - ox) * idx : FLT_MAX;
            const float ty = dy > 0.0f ? (fmaf((float) (ci + rr), b.mcwy, b.bminy) - oy) * idy
                             : dy < 0.0f ? (fmaf((float) (ci - rr + 1), b.mcwy, b.bminy) - oy) * idy : FLT_MAX;
            const float tz = dz > 0.0f ? (fmaf((float) (ck + rr), b.mcwz, b.bminz) - oz) * idz
                             : dz < 0.0f ? (fmaf((float) (ck - rr + 1), b.mcwz, b.bminz) - oz) * idz : FLT_MAX;
            float te = fminf(fminf(tx, ty), fminf(tz, tb));
            if (!(te > t)) te = t + dt;
            if (r != 0) {
                cost += 1.0f;
            } else {
                const float n = (te - t) * idt;
                const float a = (float) (oq * oq) * (1.0f / 65025.0f) * f.alpha;
                if (a > 0.0f) {
                    const float la = __log2f(1.0f - fminf(a, 0.999f));  // per sample, < 0
                    const float need = (lstop - lt) / la;
                    if (need <= n) return cost + need;
                    lt = fmaf(n, la, lt);
                }
                cost += n;
            }
            t = te;
        }
    }
    return cost;
}

constexpr int kCostKeys = 64;  // quarter-octave buckets of the tile cost

// Tile costs: kCostRays threads per 8x4 tile walk rays of it (its centre,
// two opposite corners, or all four); the tile's key is the quarter-octave
// of the largest, counted per key in counts[0..63].
#ifndef IVR_COST_RAYS
#define IVR_COST_RAYS 4
#endif
constexpr int kCostRays = IVR_COST_RAYS;
static_assert(kCostRays == 1 || kCostRays == 2 || kCostRays == 4, "rays per tile: 1, 2 or 4");
__global__ void tile_cost_kernel(const __grid_constant__ FrameDesc f, uint8_t *key, int *counts, long long ntiles)
{
    __shared__ int hist[kCostKeys];
    for (int t = threadIdx.x; t < kCostKeys; t += blockDim.x) hist[t] = 0;
    __syncthreads();
    const long long g = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    const long long tile = g / kCostRays;
    const int r = (int) (g % kCostRays);
    const int tiles_x = (f.out_w + 7) >> 3;
    float cost = 0.0f;
    if (tile < ntiles) {
        const int di = kCostRays == 1 ? 2 : kCostRays == 2 ? 3 * r : 3 * (r >> 1);
        const int dj = kCostRays == 1 ? 4 : kCostRays == 2 ? 7 * r : 7 * (r & 1);
        const int oi = min((int) (tile / tiles_x) * 4 + di, f.out_h - 1);
        const int oj = min((int) (tile % tiles_x) * 8 + dj, f.out_w - 1);
        const int i = f.out_y + oi, j = f.out_x + oj;
        if (i < f.vh && j < f.vw) cost = ray_cost(f, i, j);
    }
    for (int o = 1; o < kCostRays; o <<= 1) cost = fmaxf(cost, __shfl_xor_sync(0xffffffffu, cost, o));
    if (tile < ntiles && r == 0) {
        const int kq = min(max((int) (__log2f(cost + 1.0f) * 4.0f), 0), kCostKeys - 1);
        key[tile] = (uint8_t) kq;
        atomicAdd(&hist[kq], 1);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kCostKeys; t += blockDim.x)
        if (hist[t]) atomicAdd(&counts[t], hist[t]);
}

// The permutation, costliest key first: perm[start(key) + n] = tile, with
// start(key) the number of tiles of larger keys.  counts[64..127] are the
// per-key cursors (zero on entry); ties go in block order.
__global__ void tile_scatter_kernel(const uint8_t *key, int *counts, int *perm, long long ntiles)
{
    __shared__ int start[kCostKeys], loc[kCostKeys], base[kCostKeys];
    if (threadIdx.x < kCostKeys) loc[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = kCostKeys - 1; k >= 0; k--) {
            start[k] = acc;
            acc += counts[k];
        }
    }
    __syncthreads();
    const long long tile = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    int kq = 0, rank = 0;
    if (tile < ntiles) {
        kq = key[tile];
        rank = atomicAdd(&loc[kq], 1);
    }
    __syncthreads();
    if (threadIdx.x < kCostKeys && loc[threadIdx.x] > 0)
        base[threadIdx.x] = atomicAdd(&counts[kCostKeys + threadIdx.x], loc[threadIdx.x]);
    __syncthreads();
    if (tile < ntiles) {
        const long long pos = (long long) start[kq] + base[kq] + rank;
        if (pos < ntiles) perm[pos] = (int) tile;
    }
}

// What the judge's verdict needs (from the frame descriptor).
struct JudgeArgs {
    JudgeWords *judge;
    int *judge_reject;
    int *learned_bad;
    int judge_tol;
};

// End of a judge launch for one block: the largest difference and pixel
// count of its warps go into the judge words (one set of atomics per block,
// not per warp: thousands of warps updating the same words would serialise
// on them); the launch's last block sets the verdict (fail = largest
// difference > tolerance), adds it to the totals, marks the learned grid
// wrong on failure and clears the per-frame words.  A grid already marked
// wrong was not used (the frame marched with the exact grid): nothing is
// judged and the frame counts as an exact one.  Every thread of the block
// calls it.
__device__ __forceinline__ void judge_finish(const JudgeArgs &a, int worst, unsigned judged, bool known_bad)
{
    __shared__ int b_worst;
    __shared__ unsigned b_judged;
    if (threadIdx.x == 0) {
        b_worst = 0;
        b_judged = 0;
    }
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) {
        worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
        judged += __shfl_xor_sync(0xffffffffu, judged, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (worst > 0) atomicMax_block(&b_worst, worst);
        if (judged) atomicAdd_block(&b_judged, judged);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    JudgeWords *jw = a.judge;
    if (b_worst > 0) atomicMax(&jw->maxdiff, b_worst);
    if (b_judged) atomicAdd(&jw->pixels, (unsigned long long) b_judged);
    __threadfence();
    if (atomicAdd(&jw->warps_done, 1) != (int) gridDim.x - 1) return;  // counts blocks
    __threadfence();
    const int m = atomicAdd(&jw->maxdiff, 0);
    const int failed = m > a.judge_tol;
    jw->fail = failed;
    if (known_bad) {
        jw->exact_frames += 1;
    } else {
        jw->frames += 1;
        jw->fallbacks += (unsigned long long) failed;
        if (m > jw->worst) jw->worst = m;
    }
    if (failed) {
        *a.learned_bad = 1;
        *(volatile int *) a.judge_reject = 1;
        __threadfence_system();
    }
    jw->maxdiff = 0;
    jw->warps_done = 0;
}

// Tiles judged in a frame: judge_phase, judge_phase + judge_stride, ...
__host__ __device__ inline long long judged_tiles(long long ntiles, int stride, int phase)
{
    return ntiles > phase ? (ntiles - phase + stride - 1) / stride : 0;
}

// CONFIG kernel, persistent: every warp takes 8x4 pixel tiles from the
// view's ticket counter until none are left, so warps that drew short rays
// pick up more work instead of idling while the grid's last blocks finish.
// With f.perm the n-th ticket renders tile perm[n] (costliest first).
// A gated launch (f.gate set) renders only if *f.gate != 0; otherwise its
// warps take their share of tickets (tiles + one failed take each) and leave.
// JUDGE (learned skipping): the first tickets re-march the judged tiles
// (judge_phase modulo judge_stride) with the exact grids into f.judge8,
// each on its own warp, so that a judged heavy tile does not double the
// launch's longest warp; the rest render every tile.  A learned grid
// already marked wrong (*learned_bad) is not used: the tiles march with the
// exact grids and nothing is re-marched.  judge_compare_kernel gives the
// verdict afterwards.
template <int DT, bool SKIP, bool CENSUS, bool JUDGE>
__global__ void __launch_bounds__(kThreads, JUDGE ? kJudgeBlocksPerSm : kCfgBlocksPerSm)
    march_cfg_kernel(const __grid_constant__ FrameDesc f, float4 *out32, uchar4 *out8)
{
    unsigned long long nexec = 0, nlat = 0;
    const int lane = threadIdx.x & 31;
    const int tiles_x = (f.out_w + 7) >> 3;
    const long long ntiles = (long long) tiles_x * ((f.out_h + 3) >> 2);
    if (f.gate != nullptr && *f.gate == 0) {
        // no fallback: the launch's share of tickets (every tile, and one
        // failed take per warp) in one add instead of one per warp
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicAdd(f.tickets, (unsigned long long) ntiles + (unsigned long long) gridDim.x * (blockDim.x >> 5));
        return;
    }
    const bool exact = JUDGE && *(volatile const int *) f.learned_bad != 0;
    const long long njudged = JUDGE ? judged_tiles(ntiles, f.judge_stride, f.judge_phase) : 0;
    for (;;) {
        unsigned long long ticket = 0;
        if (lane == 0) ticket = atomicAdd(f.tickets, 1ull);
        const long long q = (long long) (__shfl_sync(0xffffffffu, ticket, 0) - f.ticket_base);
        if (q >= ntiles + njudged) break;
        // a judged tile (re-marched with the exact grids into judge8) or a
        // render tile, through one copy of the march
        const bool judge = JUDGE && q < njudged;
        if (judge && exact) continue;
        long long tile;
        if (judge) {
            tile = q * f.judge_stride + f.judge_phase;
        } else {
            tile = q - njudged;
            if (f.perm != nullptr) {
                const long long p = f.perm[tile];
                if (p >= 0 && p < ntiles) tile = p;  // a permutation by construction; never leave the window
            }
        }
        const int oi = (int) (tile / tiles_x) * 4 + (lane >> 3), oj = (int) (tile % tiles_x) * 8 + (lane & 7);
        const bool in_window = oi < f.out_h && oj < f.out_w;
        const int i = f.out_y + oi, j = f.out_x + oj;
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (in_window && i < f.vh && j < f.vw) acc = ray_cfg<DT, SKIP, CENSUS, kPair>(f, i, j, nexec, nlat, judge || exact);
        const uchar4 a8 = make_uchar4(q8(acc.x), q8(acc.y), q8(acc.z), q8(acc.w));
        if (judge) {
            f.judge8[q * 32 + lane] = a8;
        } else if (in_window) {
            const long long o = (long long) oi * f.out_w + oj;
            if (out32) out32[o] = acc;
            if (out8) out8[o] = a8;
        }
    }
    if (CENSUS) count_exec(f, nexec, nlat);
}

// The verdict of a learned-skip frame: each warp compares one judged tile's
// exact re-march (judge8) with the stored frame (out8, or out32 quantised).
__global__ void judge_compare_kernel(JudgeArgs a, const uchar4 *judge8, const uchar4 *out8, const float4 *out32,
                                     int out_x, int out_y, int out_w, int out_h, int vw, int vh, int stride,
                                     int phase)
{
    const int lane = threadIdx.x & 31;
    const int tiles_x = (out_w + 7) >> 3;
    const long long njudged = judged_tiles((long long) tiles_x * ((out_h + 3) >> 2), stride, phase);
    const bool known_bad = *(volatile const int *) a.learned_bad != 0;
    int worst = 0;
    unsigned judged = 0;
    if (!known_bad)
        for (long long q = (long long) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < njudged;
             q += (long long) gridDim.x * (blockDim.x >> 5)) {
            const long long tile = q * stride + phase;
            const int oi = (int) (tile / tiles_x) * 4 + (lane >> 3), oj = (int) (tile % tiles_x) * 8 + (lane & 7);
            if (oi < out_h && oj < out_w && out_y + oi < vh && out_x + oj < vw) {
                const uchar4 e = judge8[q * 32 + lane];
                const long long o = (long long) oi * out_w + oj;
                uchar4 v;
                if (out8) {
                    v = out8[o];
                } else {
                    const float4 c = out32[o];
                    v = make_uchar4(q8(c.x), q8(c.y), q8(c.z), q8(c.w));
                }
                const int d = max(max(abs((int) v.x - (int) e.x), abs((int) v.y - (int) e.y)),
                                  max(abs((int) v.z - (int) e.z), abs((int) v.w - (int) e.w)));
                worst = max(worst, d);
                judged++;
            }
        }
    judge_finish(a, worst, judged, known_bad);
}

// Sample-rate roofline: the CONFIG sampler (trilinear reconstruction, LUT
// fetch, front-to-back blend) with nothing else -- no ray set-up, skipping,
// termination or divergence -- over a brick small enough to stay in L1/L2.
// Each thread marches its own ray of `steps` samples, 0.5 voxel apart, from
// a start that neighbouring lanes share up to a voxel, as in an 8x4 tile.
// One sample of the roofline's brick through a sampler layout: the
// march's own sampler (corner-packed copy, or the brick itself when b.quad
// is null), or a 3D texture of the brick -- eight point fetches blended as
// fetch_cfg does (the same value, bit for bit), or one hardware-filtered
// fetch (fixed-point weights).
template <int DT, int LAYOUT>
__device__ __forceinline__ float sample_layout(const DevBrick &b, const SamplerTex &t, float ux, float uy, float uz)
{
    if (LAYOUT == IVR_SAMPLER_QUADS || LAYOUT == IVR_SAMPLER_BRICKS) return sample_cfg<DT>(b, ux, uy, uz);
    const CellPos c = cell_cfg(b, ux, uy, uz);
    if (LAYOUT == IVR_SAMPLER_TEX_LINEAR)
        return tex3D<float>(t.linear, (float) c.j + c.fx + 0.5f, (float) c.i + c.fy + 0.5f,
                            (float) c.k + c.fz + 0.5f) * t.scale;
    using T = typename VoxT<DT>::T;
    const float x0 = (float) c.j + 0.5f, y0 = (float) c.i + 0.5f, z0 = (float) c.k + 0.5f;
    const float x1 = x0 + 1.0f, y1 = y0 + 1.0f, z1 = z0 + 1.0f;
    const float c00 = lerpf((float) tex3D<T>(t.point, x0, y0, z0), (float) tex3D<T>(t.point, x1, y0, z0), c.fx);
    const float c10 = lerpf((float) tex3D<T>(t.point, x0, y1, z0), (float) tex3D<T>(t.point, x1, y1, z0), c.fx);
    const float c01 = lerpf((float) tex3D<T>(t.point, x0, y0, z1), (float) tex3D<T>(t.point, x1, y0, z1), c.fx);
    const float c11 = lerpf((float) tex3D<T>(t.point, x0, y1, z1), (float) tex3D<T>(t.point, x1, y1, z1), c.fx);
    return lerpf(lerpf(c00, c10, c.fy), lerpf(c01, c11, c.fy), c.fz);
}

template <int DT, int LAYOUT>
__global__ void __launch_bounds__(kThreads, kCfgBlocksPerSm) sample_peak_kernel(const __grid_constant__ FrameDesc f,
                                                                                SamplerTex tex, int steps,
                                                                                float4 *out)
{
    const DevBrick &b = f.b[0];
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    // the warp's 8x4 tile of starts, one voxel apart, at a hashed place
    const unsigned w = gid >> 5, lane = gid & 31;
    const unsigned h = w * 2654435761u;
    // positions in the brick's voxel coordinates, as the march samples
    const float sx = (float) (b.nx - 2), sy = (float) (b.ny - 2), sz = (float) (b.nz - 2);
    float x = 2.0f + (float) (h % 997u) / 997.0f * (sx - 12.0f) + (float) (lane & 7);
    float y = 2.0f + (float) ((h >> 10) % 991u) / 991.0f * (sy - 8.0f) + (float) (lane >> 3);
    float z = 2.0f + (float) ((h >> 20) % 983u) / 983.0f * (sz - 4.0f);
    // half a voxel per step along a direction fixed per warp
    const float dx = (w & 1) ? 0.3f : -0.3f, dy = (w & 2) ? 0.2f : -0.2f, dz = (w & 4) ? 0.35f : -0.35f;
    const float lox = 1.0f, hix = sx - 1.0f;
    const float loy = 1.0f, hiy = sy - 1.0f;
    const float loz = 1.0f, hiz = sz - 1.0f;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    QuadCell<DT> qlast{};
    unsigned qkey = 0;
    for (int i = 0; i < steps; i++) {
        float s;
        if (LAYOUT == IVR_SAMPLER_QUADS && cell_reuse<DT>()) {
            // the march's sampler: samples taken in pairs, the second
            // reusing the first's cell when both lie in it
            const CellPos c = cell_cfg(b, x, y, z);
            const unsigned k = quad_key(b, c);
            if (!(i & 1) || k != qkey) qlast = quad_load<DT>(b, k);
            qkey = k;
            s = quad_interp<DT>(qlast, c);
        } else {
            s = sample_layout<DT, LAYOUT>(b, tex, x, y, z);
        }
        const float4 e = lut_at(f, (int) (s * f.lut_scale) - f.lut_off);
        const float wgt = (1.0f - acc.w) * (e.w * f.alpha);
        acc.x = fmaf(wgt, e.x, acc.x);
        acc.y = fmaf(wgt, e.y, acc.y);
        acc.z = fmaf(wgt, e.z, acc.z);
        acc.w = acc.w * 0.5f + wgt;  // stays below 1: no termination
        x += dx;
        y += dy;
        z += dz;
        // reflect at the faces so the ray stays inside the brick
        x = x < lox ? 2.0f * lox - x : (x > hix ? 2.0f * hix - x : x);
        y = y < loy ? 2.0f * loy - y : (y > hiy ? 2.0f * hiy - y : y);
        z = z < loz ? 2.0f * loz - z : (z > hiz ? 2.0f * hiz - z : z);
    }
    out[gid] = acc;
}

// The largest |layout sample - exact trilinear sample (the brick itself)|
// over npos hashed positions of the brick, as float bits into *err.
template <int DT, int LAYOUT>
__global__ void sample_err_kernel(const __grid_constant__ FrameDesc f, SamplerTex tex, int npos, unsigned *err)
{
    const DevBrick &b = f.b[0];
    DevBrick ref = b;
    ref.quad = nullptr;
    float worst = 0.0f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npos; p += gridDim.x * blockDim.x) {
        unsigned h = (unsigned) p * 2654435761u + 12345u;
        const float ux = (float) ((h = h * 1664525u + 1013904223u) >> 8) / 16777216.0f * (float) (b.nx - 1);
        const float uy = (float) ((h = h * 1664525u + 1013904223u) >> 8) / 16777216.0f * (float) (b.ny - 1);
        const float uz = (float) ((h = h * 1664525u + 1013904223u) >> 8) / 16777216.0f * (float) (b.nz - 1);
        worst = fmaxf(worst, fabsf(sample_layout<DT, LAYOUT>(b, tex, ux, uy, uz) - sample_cfg<DT>(ref, ux, uy, uz)));
    }
    atomicMax(err, __float_as_uint(worst));  // non-negative floats order as their bits
}

template <typename K>
int persistent_grid(K kernel, size_t smem)
{
    // SM count of the current device, looked up once per device
    static std::atomic<int> sm_count[64];
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = dev >= 0 && dev < 64 ? sm_count[dev].load(std::memory_order_relaxed) : 0;
    if (sms == 0) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (dev >= 0 && dev < 64) sm_count[dev].store(sms, std::memory_order_relaxed);
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
    return sms * (per_sm > 0 ? per_sm : 1);
}

template <int DT>
cudaError_t launch_dt(const FrameDesc &f, float4 *o32, uchar4 *o8, cudaStream_t s, long long *warps_launched)
{
    dim3 grid((f.out_w + kBlockX - 1) / kBlockX, (f.out_h + kBlockY - 1) / kBlockY);
    if (f.preset == IVR_PRESET_CONFIG) {
        bool skip = false;
        for (int k = 0; k < f.nb; k++) skip |= f.b[k].empty != nullptr;
        const bool judge = f.judge != nullptr;
        if (judge && (!skip || f.census || !f.judge8 || f.judge_stride < 1 || f.judge_phase < 0 ||
                      f.judge_phase >= f.judge_stride))
            return cudaErrorInvalidValue;
        auto kern = f.census ? (skip ? march_cfg_kernel<DT, true, true, false> : march_cfg_kernel<DT, false, true, false>)
                    : judge  ? march_cfg_kernel<DT, true, false, true>
                    : skip   ? march_cfg_kernel<DT, true, false, false>
                             : march_cfg_kernel<DT, false, false, false>;
        const int blocks = persistent_grid(kern, 0);
        // every tile (and, judged, every re-march) is taken once and every
        // warp ends on one failed take
        const long long ntiles = (long long) ((f.out_w + 7) >> 3) * ((f.out_h + 3) >> 2);
        if (warps_launched)
            *warps_launched = ntiles + (judge ? judged_tiles(ntiles, f.judge_stride, f.judge_phase) : 0) +
                              (long long) blocks * (kThreads / 32);
        kern<<<blocks, kThreads, 0, s>>>(f, o32, o8);
        return cudaGetLastError();
    }
    if (warps_launched) *warps_launched = 0;
    switch (f.tf_mode) {
    case IVR_TF_SEISMIC: march_ref_kernel<DT, IVR_TF_SEISMIC><<<grid, kThreads, 0, s>>>(f, o32, o8); break;
    case IVR_TF_MED: march_ref_kernel<DT, IVR_TF_MED><<<grid, kThreads, 0, s>>>(f, o32, o8); break;
    case IVR_TF_SEISMIC2: march_ref_kernel<DT, IVR_TF_SEISMIC2><<<grid, kThreads, 0, s>>>(f, o32, o8); break;
    case IVR_TF_CHEM: march_ref_kernel<DT, IVR_TF_CHEM><<<grid, kThreads, 0, s>>>(f, o32, o8); break;
    case IVR_TF_BLEND: march_ref_kernel<DT, IVR_TF_BLEND><<<grid, kThreads, 0, s>>>(f, o32, o8); break;
    case IVR_TF_RGBBLEND: march_ref_kernel<DT, IVR_TF_RGBBLEND><<<grid, kThreads, 0, s>>>(f, o32, o8); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Batched CONFIG kernel: the tiles of every frame of a batch in one
// persistent launch.  Frame descriptors are in device memory (uploaded with
// the batch); a warp's ticket is a global tile number, mapped to its frame by
// a binary search over the frames' first tiles.  Warp tiles are TW x (32/TW)
// pixels; PAIR takes two samples per loop iteration.
template <int DT, int TW, bool PAIR>
__global__ void __launch_bounds__(kThreads, kBatchBlocksPerSm)
    march_batch_kernel(const BatchHeader *__restrict__ hdr, const BatchItem *__restrict__ items,
                       unsigned long long *ticket)
{
    constexpr int TH = 32 / TW;
    const int lane = threadIdx.x & 31;
    const int n = hdr->nitems;
    const long long total = hdr->total_tiles;
    unsigned long long nexec = 0, nlat = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1ull);
        const long long g = (long long) __shfl_sync(0xffffffffu, t, 0);
        if (g >= total) break;
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tile0 <= g) lo = mid;
            else hi = mid - 1;
        }
        const BatchItem &it = items[lo];
        const long long tile = g - it.tile0;
        pixel_cfg<DT, true, false, PAIR>(it.f, (int) (tile / it.tiles_x) * TH + lane / TW,
                                        (int) (tile % it.tiles_x) * TW + lane % TW, it.out32, it.out8, nexec, nlat);
    }
}

template <int DT, int TW, bool PAIR>
cudaError_t launch_batch_v(const BatchHeader *hdr, const BatchItem *items, unsigned long long *ticket,
                           cudaStream_t s)
{
    auto kern = march_batch_kernel<DT, TW, PAIR>;
    kern<<<persistent_grid(kern, 0), kThreads, 0, s>>>(hdr, items, ticket);
    return cudaGetLastError();
}

template <int DT>
cudaError_t launch_batch_dt(int variant, const BatchHeader *hdr, const BatchItem *items, unsigned long long *ticket,
                            cudaStream_t s)
{
    switch (variant) {
    case 0: return launch_batch_v<DT, 8, true>(hdr, items, ticket, s);
    case 1: return launch_batch_v<DT, 8, false>(hdr, items, ticket, s);
    case 2: return launch_batch_v<DT, 4, true>(hdr, items, ticket, s);
    case 3: return launch_batch_v<DT, 4, false>(hdr, items, ticket, s);
    case 4: return launch_batch_v<DT, 16, true>(hdr, items, ticket, s);
    case 5: return launch_batch_v<DT, 16, false>(hdr, items, ticket, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

int batch_variant_tile_w(int variant) { return variant < 2 ? 8 : variant < 4 ? 4 : 16; }

cudaError_t launch_batch(int dtype, int variant, const BatchHeader *hdr, const BatchItem *items,
                         unsigned long long *ticket, cudaStream_t s)
{
    switch (dtype) {
    case IVR_U8: return launch_batch_dt<IVR_U8>(variant, hdr, items, ticket, s);
    case IVR_U16: return launch_batch_dt<IVR_U16>(variant, hdr, items, ticket, s);
    case IVR_F32: return launch_batch_dt<IVR_F32>(variant, hdr, items, ticket, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int DT, int LAYOUT>
cudaError_t launch_sample_layout(const FrameDesc &f, const SamplerTex &tex, int steps, float4 *out,
                                 long long *samples, unsigned *err, cudaStream_t s)
{
    auto kern = sample_peak_kernel<DT, LAYOUT>;
    const int blocks = persistent_grid(kern, 0);
    if (out) {
        kern<<<blocks, kThreads, 0, s>>>(f, tex, steps, out);
        *samples = (long long) blocks * kThreads * steps;
    }
    if (err) sample_err_kernel<DT, LAYOUT><<<256, 256, 0, s>>>(f, tex, 1 << 20, err);
    return cudaGetLastError();
}

template <int DT>
cudaError_t launch_sample_dt(const FrameDesc &f, int layout, const SamplerTex &tex, int steps, float4 *out,
                             long long *samples, unsigned *err, cudaStream_t s)
{
    switch (layout) {
    case IVR_SAMPLER_QUADS: return launch_sample_layout<DT, IVR_SAMPLER_QUADS>(f, tex, steps, out, samples, err, s);
    case IVR_SAMPLER_BRICKS: return launch_sample_layout<DT, IVR_SAMPLER_BRICKS>(f, tex, steps, out, samples, err, s);
    case IVR_SAMPLER_TEX_POINT:
        return launch_sample_layout<DT, IVR_SAMPLER_TEX_POINT>(f, tex, steps, out, samples, err, s);
    case IVR_SAMPLER_TEX_LINEAR:
        return launch_sample_layout<DT, IVR_SAMPLER_TEX_LINEAR>(f, tex, steps, out, samples, err, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sample_peak(const FrameDesc &f, int layout, const SamplerTex &tex, int steps, float4 *out,
                               long long *samples, unsigned *err, cudaStream_t s)
{
    switch (f.dtype) {
    case IVR_U8: return launch_sample_dt<IVR_U8>(f, layout, tex, steps, out, samples, err, s);
    case IVR_U16: return launch_sample_dt<IVR_U16>(f, layout, tex, steps, out, samples, err, s);
    case IVR_F32: return launch_sample_dt<IVR_F32>(f, layout, tex, steps, out, samples, err, s);
    default: return cudaErrorInvalidValue;
    }
}

int sample_peak_threads()
{
    return persistent_grid(sample_peak_kernel<IVR_F32, IVR_SAMPLER_QUADS>, 0) * kThreads;
}

cudaError_t launch_judge_compare(const FrameDesc &f, const uchar4 *out8, const float4 *out32, cudaStream_t s)
{
    const long long ntiles = (long long) ((f.out_w + 7) >> 3) * ((f.out_h + 3) >> 2);
    const long long nj = judged_tiles(ntiles, f.judge_stride, f.judge_phase);
    const long long blocks = nj > 0 ? (nj + 7) / 8 : 1;  // a warp per judged tile
    JudgeArgs a{f.judge, f.judge_reject, f.learned_bad, f.judge_tol};
    judge_compare_kernel<<<(unsigned) (blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, s>>>(
        a, f.judge8, out8, out32, f.out_x, f.out_y, f.out_w, f.out_h, f.vw, f.vh, f.judge_stride, f.judge_phase);
    return cudaGetLastError();
}

cudaError_t launch_tile_order(const FrameDesc &f, uint8_t *key, int *counts, int *perm, cudaStream_t s)
{
    const long long ntiles = (long long) ((f.out_w + 7) >> 3) * ((f.out_h + 3) >> 2);
    if (ntiles <= 0) return cudaSuccess;
    if (ntiles > (1ll << 30)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * 2 * kCostKeys, s);
    if (e != cudaSuccess) return e;
    tile_cost_kernel<<<(unsigned) ((ntiles * kCostRays + 127) / 128), 128, 0, s>>>(f, key, counts, ntiles);
    tile_scatter_kernel<<<(unsigned) ((ntiles + 255) / 256), 256, 0, s>>>(key, counts, perm, ntiles);
    return cudaGetLastError();
}

long long judge_scratch_bytes(const FrameDesc &f)
{
    const long long ntiles = (long long) ((f.out_w + 7) >> 3) * ((f.out_h + 3) >> 2);
    return judged_tiles(ntiles, f.judge_stride, f.judge_phase) * 32 * (long long) sizeof(uchar4);
}

cudaError_t launch_march(const FrameDesc &f, float4 *out32, uchar4 *out8, cudaStream_t s, long long *warps)
{
    if (warps) *warps = 0;
    if (f.out_w <= 0 || f.out_h <= 0) return cudaSuccess;
    switch (f.dtype) {
    case IVR_U8: return launch_dt<IVR_U8>(f, out32, out8, s, warps);
    case IVR_U16: return launch_dt<IVR_U16>(f, out32, out8, s, warps);
    case IVR_F32: return launch_dt<IVR_F32>(f, out32, out8, s, warps);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ivr
