/*
 * ivr_oracle.c -- O2: CPU restatement of the iVR ray-casting hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (tests/, smoke(),
 * bench.py's CPU baseline).  The product never links or calls it.
 *
 * Every function cites the reference code it restates.  In the REF preset
 * the order and precision of every floating-point operation follows the
 * reference as gcc compiles it with -ffp-contract=off (float arithmetic,
 * double only where the reference promotes), so the output is bitwise equal
 * to the reference rebuilt from source; tests pin that.  The CONFIG preset
 * is this project's benchmark semantics; the CUDA kernels compute it with the
 * same operations (explicit fmaf where fused).
 */
#include "ivr_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;
typedef struct { float r, g, b, a; } c4;

/* ---------------------------------------------------------------- math --
 * mathutil.c:28-32 dot3f, :34-38 dot4f, :40-47 cross3f, :103-113
 * normalize3f, :129-149 mat3fxvec3f, :150-171 mat3fxmat3f, :172-196
 * mat4fxmat4f, :197-219 mat4fxvec4f.  Left-to-right sums of rounded
 * products. */
static float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float dot4(v4 a, v4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static v3 cross3(v3 a, v3 b)
{
    v3 c = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return c;
}
static v3 norm3(v3 a)
{
    float m = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    v3 r = {a.x / m, a.y / m, a.z / m};
    return r;
}
static v3 m3v(float m[3][3], v3 v)
{
    v3 r;
    v3 r0 = {m[0][0], m[0][1], m[0][2]}, r1 = {m[1][0], m[1][1], m[1][2]}, r2 = {m[2][0], m[2][1], m[2][2]};
    r.x = dot3(r0, v); r.y = dot3(r1, v); r.z = dot3(r2, v);
    return r;
}
static void m3m(float io[3][3], float in[3][3])
{
    float t[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            v3 row = {io[i][0], io[i][1], io[i][2]}, col = {in[0][j], in[1][j], in[2][j]};
            t[i][j] = dot3(row, col);
        }
    memcpy(io, t, sizeof(t));
}
static void m4m(float io[4][4], float in[4][4])
{
    float t[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            v4 row = {io[i][0], io[i][1], io[i][2], io[i][3]}, col = {in[0][j], in[1][j], in[2][j], in[3][j]};
            t[i][j] = dot4(row, col);
        }
    memcpy(io, t, sizeof(t));
}
static v4 m4v(float m[4][4], v4 v)
{
    v4 r;
    float t[4];
    for (int j = 0; j < 4; j++) {
        v4 row = {m[j][0], m[j][1], m[j][2], m[j][3]};
        t[j] = dot4(row, v);
    }
    r.x = t[0]; r.y = t[1]; r.z = t[2]; r.w = t[3];
    return r;
}
/* GL column-major -> row-major (mathutil.h:212-233 setmvm/setpm) */
static void from_gl(float m[4][4], const float cm[16])
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) m[r][c] = cm[c * 4 + r];
}

/* --------------------------------------------------------------- scene --
 * View state that is common to every brick (camera, viewport, ray frame). */
typedef struct {
    float vwm[3][3];
    float mvm[4][4], pm[4][4], vpm[4][4];
    v3 cam_e, cam_r;
    float vpx, vpy, vpw, vph;   /* WINDOW x,y,w,h (floats) */
    int vw, vh;
    float left, right, bottom, top;
    float du, dv;
    float ctm[3][3];            /* transpose(mvm3) * vwm (buildray) */
    v3 orig, incri, incrj;
} view_t;

typedef struct {
    int lw, lh, ld;          /* local dims incl. halo (volume.localdims) */
    int cw, ch, cd;          /* core dims, before the halo is added */
    int sx, sy, sz;          /* startindex */
    int col, row, slab;
    v3 bmin, bmax;           /* aabb.min / aabb.max */
    float w, h, d;           /* aabb.w/h/d */
    float dconst[6];
    float wc[6];             /* wincoord x,y,z,w,h,d */
    int istrt, istop, jstrt, jstop;
    v3 dir0;                 /* buildray direction at (istrt, jstrt) */
    v3 invcell;              /* CONFIG: core voxels per world unit */
    float *data;             /* float copy, [ld][lh][lw] */
    unsigned char *empty;    /* CONFIG skip: transparent macrocells */
    int mcx, mcy, mcz;
} brick_t;

static const v3 k_normals[6] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};

static float vox(const void *p, int dtype, long long i)
{
    switch (dtype) {
    case ORC_U8: return (float) ((const uint8_t *) p)[i];
    case ORC_U16: return (float) ((const uint16_t *) p)[i];
    default: return ((const float *) p)[i];
    }
}

/* initcamera (main.c:428-500) and the frame's view calls (main.c:226-232):
 * setviewport (mathutil.h:147-163), setmvm/setpm, setfrustum, then buildray's
 * brick-independent part (mathutil.c:1115-1154). */
static void view_setup(const orc_scene *sc, view_t *v)
{
    memset(v, 0, sizeof(*v));
    v3 n = {0.0f, 0.0f, -1.0f}, up = {0.0f, 1.0f, 0.0f};
    v3 cv = norm3(up);
    v3 cu = cross3(n, cv);
    v->vwm[0][0] = cu.x; v->vwm[0][1] = cv.x; v->vwm[0][2] = n.x;
    v->vwm[1][0] = cu.y; v->vwm[1][1] = cv.y; v->vwm[1][2] = n.y;
    v->vwm[2][0] = cu.z; v->vwm[2][1] = cv.z; v->vwm[2][2] = n.z;
    v->cam_e.x = 0.0f; v->cam_e.y = 0.0f; v->cam_e.z = -5.0f;
    v->cam_r.x = v->cam_r.y = v->cam_r.z = 0.0f;

    int tilex = sc->state.winwidth / sc->tilew, tiley = sc->state.winheight / sc->tileh;
    v->vpw = (float) (tilex * sc->tilew);
    v->vph = (float) (tiley * sc->tileh);
    v->vpx = 0.0f; v->vpy = 0.0f;
    int w = (int) v->vpw, h = (int) v->vph, x = 0, y = 0;
    v->vw = w; v->vh = h;
    memset(v->vpm, 0, sizeof(v->vpm));
    v->vpm[0][0] = w / 2.0f; v->vpm[0][3] = (x + w) / 2.0f;
    v->vpm[1][1] = h / 2.0f; v->vpm[1][3] = (y + h) / 2.0f;
    v->vpm[2][2] = 0.5f; v->vpm[2][3] = 0.5f;
    v->vpm[3][3] = 1.0f;

    from_gl(v->mvm, sc->state.mvm);
    from_gl(v->pm, sc->state.pm);
    v->left = sc->state.vv[0]; v->right = sc->state.vv[1];
    v->bottom = sc->state.vv[2]; v->top = sc->state.vv[3];
    v->du = (v->right - v->left) / v->vpw;
    v->dv = (v->top - v->bottom) / v->vph;

    /* buildray, brick-independent part */
    v3 ii = {0.0f, v->dv, 0.0f}, jj = {v->du, 0.0f, 0.0f};
    v3 trans = {v->mvm[0][3], v->mvm[1][3], 0.0f};
    v3 eye = m3v(v->vwm, v->cam_e);
    eye.x = eye.x + v->cam_r.x; eye.y = eye.y + v->cam_r.y; eye.z = eye.z + v->cam_r.z;
    v3 o = {eye.x - trans.x, eye.y - trans.y, eye.z - trans.z};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v->ctm[i][j] = v->mvm[j][i];
    v->orig = m3v(v->ctm, o);
    m3m(v->ctm, v->vwm);
    v->incri = m3v(v->ctm, ii);
    v->incrj = m3v(v->ctm, jj);
}

/* getlocalbrick (utils.c:332-388) + initvolbbox (main.c:505-624) +
 * setplaneconst (ray.c:44-51) + updatevolbbox (mathutil.c:948-1018) +
 * createlocalimage's rect and first ray (main.c:950-981). */
static void brick_setup(const orc_scene *sc, const view_t *v, int rank, brick_t *b)
{
    memset(b, 0, sizeof(*b));
    int gw = sc->gw, gh = sc->gh, gd = sc->gd;
    int py = sc->procdims[0], px = sc->procdims[1], pz = sc->procdims[2];
    int mx = gw > gh ? gw : gh;
    mx = mx > gd ? mx : gd;
    float maxdim = (float) mx;
    float invdim = 1.0f / maxdim;
    v3 sf = {(float) gw * invdim, (float) gh * invdim, (float) gd * invdim};

    b->slab = rank / (py * px);
    b->row = (rank / px) % py;
    b->col = rank % px;

    int lw = gw / px, lh = gh / py, ld = gd / pz;
    int rw = gw % (lw * px), rh = gh % (lh * py), rd = gd % (ld * pz);
    b->sx = b->col * lw; b->sy = b->row * lh; b->sz = b->slab * ld;
    if (b->col == px - 1) lw += rw;
    if (b->row == py - 1) lh += rh;
    if (b->slab == pz - 1) ld += rd;
    b->cw = lw; b->ch = lh; b->cd = ld;

    v3 range = {sf.x * 2.0f, sf.y * 2.0f, sf.z * 2.0f};
    v3 ratio = {(float) lw / (float) gw, (float) lh / (float) gh, (float) ld / (float) gd};
    float bw = 2.0f * sf.x * ratio.x, bh = 2.0f * sf.y * ratio.y, bd = 2.0f * sf.z * ratio.z;
    v3 rs = {(float) b->sx / (float) gw, (float) b->sy / (float) gh, (float) b->sz / (float) gd};
    float bx = -sf.x + range.x * rs.x, by = -sf.y + range.y * rs.y, bz = -sf.z + range.z * rs.z;

    b->lw = (b->col == px - 1) ? lw : lw + sc->overlap;
    b->lh = (b->row == py - 1) ? lh : lh + sc->overlap;
    b->ld = (b->slab == pz - 1) ? ld : ld + sc->overlap;

    /* the 8 vertices are the corners {bx, bx+bw} x {by, by+bh} x {bz, bz+bd} */
    float x1 = bx + bw, y1 = by + bh, z1 = bz + bd;
    b->bmin.x = fminf(bx, x1); b->bmax.x = fmaxf(bx, x1);
    b->bmin.y = fminf(by, y1); b->bmax.y = fmaxf(by, y1);
    b->bmin.z = fminf(bz, z1); b->bmax.z = fmaxf(bz, z1);
    b->w = b->bmax.x - b->bmin.x; b->h = b->bmax.y - b->bmin.y; b->d = b->bmax.z - b->bmin.z;

    float pz0[6] = {b->bmin.x * -1.0f, b->bmax.x * 1.0f, b->bmin.y * -1.0f,
                    b->bmax.y * 1.0f, b->bmin.z * -1.0f, b->bmax.z * 1.0f};
    for (int i = 0; i < 6; i++)
        b->dconst[i] = (sc->state.newconst[i] < pz0[i]) ? sc->state.newconst[i] : pz0[i];

    /* updatevolbbox */
    float ctm[4][4];
    memcpy(ctm, v->pm, sizeof(ctm));
    float mv[4][4];
    memcpy(mv, v->mvm, sizeof(mv));
    m4m(ctm, mv);
    v3 wmin = {FLT_MAX, FLT_MAX, FLT_MAX}, wmax = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int c = 0; c < 8; c++) {
        v4 vert = {(c & 1) ? x1 : bx, (c & 2) ? y1 : by, (c & 4) ? z1 : bz, 1.0f};
        v4 pc = m4v(ctm, vert);
        float w = pc.w;
        v4 ndc = {pc.x / w, pc.y / w, pc.z / w, 1.0f};
        float vp[4][4];
        memcpy(vp, v->vpm, sizeof(vp));
        v4 win = m4v(vp, ndc);
        wmin.x = fminf(wmin.x, win.x); wmin.y = fminf(wmin.y, win.y); wmin.z = fminf(wmin.z, win.z);
        wmax.x = fmaxf(wmax.x, win.x); wmax.y = fmaxf(wmax.y, win.y); wmax.z = fmaxf(wmax.z, win.z);
    }
    float xe = v->vpx + v->vpw, ye = v->vpy + v->vph;
    wmin.x = (wmin.x < v->vpx) ? v->vpx : wmin.x;
    wmax.x = (wmax.x > xe) ? xe : wmax.x;
    wmin.x = (wmin.x > xe) ? xe : wmin.x;
    wmax.x = (wmax.x < v->vpx) ? v->vpx : wmax.x;
    wmin.y = (wmin.y < v->vpy) ? v->vpy : wmin.y;
    wmax.y = (wmax.y > ye) ? ye : wmax.y;
    wmin.y = (wmin.y > ye) ? ye : wmin.y;
    wmax.y = (wmax.y < v->vpy) ? v->vpy : wmax.y;
    b->wc[0] = wmin.x; b->wc[1] = wmin.y; b->wc[2] = wmax.z;
    b->wc[3] = wmax.x - wmin.x; b->wc[4] = wmax.y - wmin.y;
    b->wc[5] = (wmax.z + wmin.z) / 2.0f;

    /* createlocalimage: rect and the first ray of the rect */
    b->istrt = (int) (b->wc[1] - 0.5f);
    b->istop = (int) (b->wc[1] + b->wc[4] + 1.0f);
    b->jstrt = (int) (b->wc[0] - 0.5f);
    b->jstop = (int) (b->wc[0] + b->wc[3] + 1.0f);
    float vv = v->bottom + b->istrt * v->dv + v->dv / 2.0f;
    float uu = v->left + b->jstrt * v->du - v->du / 2.0f;
    v3 d = {uu, vv, -v->cam_e.z};
    float ctm3[3][3];
    memcpy(ctm3, v->ctm, sizeof(ctm3));
    b->dir0 = m3v(ctm3, d);

    b->invcell.x = (float) b->cw / b->w;
    b->invcell.y = (float) b->ch / b->h;
    b->invcell.z = (float) b->cd / b->d;
}

/* readfromfile (main.c:1220-1269): brick sub-array of the global volume. */
static void brick_load(const orc_scene *sc, brick_t *b)
{
    size_t n = (size_t) b->lw * b->lh * b->ld;
    b->data = (float *) malloc(sizeof(float) * n);
    for (int z = 0; z < b->ld; z++)
        for (int y = 0; y < b->lh; y++)
            for (int x = 0; x < b->lw; x++) {
                long long src = ((long long) (b->sz + z) * sc->gh + (b->sy + y)) * sc->gw + (b->sx + x);
                b->data[((size_t) z * b->lh + y) * b->lw + x] = vox(sc->data, sc->dtype, src);
            }
}

/* getrayintersect (ray.c:276-318): slab test against the 6 clip planes. */
static int ray_box(const float dconst[6], v3 o, v3 d, float *tin, float *tout)
{
    *tin = -FLT_MAX;
    *tout = FLT_MAX;
    int i = 0;
    while (i < 6 && *tin < *tout) {
        float numer = dconst[i] - dot3(k_normals[i], o);
        float denom = dot3(k_normals[i], d);
        if (denom == 0.0f) {
            if (numer < 0.0f) *tin = *tout + 1.0f;
        } else {
            float thit = numer / denom;
            if (denom > 0.0f) *tout = fminf(*tout, thit);
            else *tin = fmaxf(*tin, thit);
        }
        i++;
    }
    if (*tin < *tout) {
        if (*tin > 0.0f) return 1;
        if (*tout > 0.0f) return 1;
    }
    return 0;
}

/* The CONFIG slab test: ray_box's planes and order, each hit parameter
 * +-numer times the reciprocal direction component (the CONFIG lattice's
 * definition; REF keeps the reference's division).  With the axis-aligned
 * normals numer = d -+ o and denom = +-d exactly. */
static int ray_box_cfg(const float dconst[6], v3 o, v3 d, v3 id, float *tin, float *tout)
{
    *tin = -FLT_MAX;
    *tout = FLT_MAX;
    for (int p = 0; p < 6 && *tin < *tout; p++) {
        int axis = p >> 1, pos = p & 1;
        float oa = axis == 0 ? o.x : axis == 1 ? o.y : o.z;
        float da = axis == 0 ? d.x : axis == 1 ? d.y : d.z;
        float ia = axis == 0 ? id.x : axis == 1 ? id.y : id.z;
        float numer = pos ? dconst[p] - oa : dconst[p] + oa;
        if (da == 0.0f) {
            if (numer < 0.0f) *tin = *tout + 1.0f;
        } else {
            float thit = (pos ? numer : -numer) * ia;
            if (pos ? da > 0.0f : da < 0.0f) *tout = fminf(*tout, thit);
            else *tin = fmaxf(*tin, thit);
        }
    }
    if (*tin < *tout) {
        if (*tin > 0.0f) return 1;
        if (*tout > 0.0f) return 1;
    }
    return 0;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* getlinearsample, non-BGQ branch (ray.c:87-181), quirks included:
 * weights scale by the cell size squared and the x weight blends the +1 row
 * (y) neighbour.  xp = x + fabs(min.x) is evaluated in double by the
 * reference and rounded to float; for a sum of two floats that double
 * rounding equals the single float rounding (53 >= 2*24+2). */
static float sample_ref(const brick_t *b, float x, float y, float z)
{
    int vw = b->lw, vh = b->lh, vd = b->ld;
    float ratio = (x - b->bmin.x) / b->w;
    int j = (int) ((float) vw * ratio);
    ratio = (y - b->bmin.y) / b->h;
    int i = (int) ((float) vh * ratio);
    ratio = (z - b->bmin.z) / b->d;
    int k = (int) ((float) vd * ratio);
    i = (i > vh - 2) ? vh - 2 : i;
    j = (j > vw - 2) ? vw - 2 : j;
    k = (k > vd - 2) ? vd - 2 : k;
    /* the reference has no lower clamp; indices stay >= 0 for samples inside
     * the box, and the clamp below only guards memory */
    i = i < 0 ? 0 : i; j = j < 0 ? 0 : j; k = k < 0 ? 0 : k;
    const float *D = b->data;
#define V(I, J, K) D[(((size_t) (K) * vh) + (I)) * vw + (J)]
    float v000 = V(i, j, k), v100 = V(i + 1, j, k), v010 = V(i, j + 1, k), v001 = V(i, j, k + 1);
    float v101 = V(i + 1, j, k + 1), v011 = V(i, j + 1, k + 1), v110 = V(i + 1, j + 1, k), v111 = V(i + 1, j + 1, k + 1);
#undef V
    float xp = x + fabsf(b->bmin.x), yp = y + fabsf(b->bmin.y), zp = z + fabsf(b->bmin.z);
    float x0 = ((float) j * b->w) / (float) vw;
    float y0 = ((float) i * b->h) / (float) vh;
    float z0 = ((float) k * b->d) / (float) vd;
    float xd = (fabsf(xp - x0) * b->w) / (float) vw;
    float yd = (fabsf(yp - y0) * b->h) / (float) vh;
    float zd = (fabsf(zp - z0) * b->d) / (float) vd;
    float c00 = v000 * (1.0f - xd) + v100 * xd;
    float c10 = v010 * (1.0f - xd) + v110 * xd;
    float c01 = v001 * (1.0f - xd) + v101 * xd;
    float c11 = v011 * (1.0f - xd) + v111 * xd;
    float c0 = c00 * (1.0f - yd) + c10 * yd;
    float c1 = c01 * (1.0f - yd) + c11 * yd;
    return c0 * (1.0f - zd) + c1 * zd;
}

/* CONFIG sampler: true trilinear, voxel values at cell corners (the
 * reference's index convention, utils.c halo on the high side), clamp to
 * edge, at (ux, uy, uz) in the brick's voxel coordinates (voxel (j, i, k)
 * at u = (j, i, k)).  lerp(a,b,t) = fmaf(t, b-a, a). */
static float lerpf_(float a, float b, float t) { return fmaf(t, b - a, a); }
static float sample_cfg(const brick_t *b, float ux, float uy, float uz)
{
    int nx = b->lw, ny = b->lh, nz = b->ld;
    int j = clampi((int) floorf(ux), 0, nx - 2);
    int i = clampi((int) floorf(uy), 0, ny - 2);
    int k = clampi((int) floorf(uz), 0, nz - 2);
    float fx = fminf(fmaxf(ux - (float) j, 0.0f), 1.0f);
    float fy = fminf(fmaxf(uy - (float) i, 0.0f), 1.0f);
    float fz = fminf(fmaxf(uz - (float) k, 0.0f), 1.0f);
    const float *D = b->data;
    size_t p = ((size_t) k * ny + i) * nx + j;
    size_t sy = (size_t) nx, sz = (size_t) nx * ny;
    float c00 = lerpf_(D[p], D[p + 1], fx);
    float c10 = lerpf_(D[p + sy], D[p + sy + 1], fx);
    float c01 = lerpf_(D[p + sz], D[p + sz + 1], fx);
    float c11 = lerpf_(D[p + sz + sy], D[p + sz + sy + 1], fx);
    float c0 = lerpf_(c00, c10, fy);
    float c1 = lerpf_(c01, c11, fy);
    return lerpf_(c0, c1, fz);
}

/* ------------------------------------------------------- REF ray cast --
 * raycast (ray.c:59-85) + getsamplesonray (ray.c:239-273) + the transfer
 * functions of transferfuncs.c:24-199.  Samples are recomputed in the
 * order each transfer function consumes them instead of being stored. */
typedef struct {
    const c4 *lut;
    int n, off;
    float alpha;
} tf_t;

static c4 lutat(const tf_t *t, int idx) { return t->lut[clampi(idx, 0, t->n - 1)]; }

static c4 raycast_ref(const orc_scene *sc, const brick_t *b, v3 o, v3 d, const tf_t *tf,
                      long long *nalg, long long *nexec)
{
    c4 c = {0.0f, 0.0f, 0.0f, 0.0f};
    float tin, tout;
    if (!ray_box(b->dconst, o, d, &tin, &tout)) return c;
    float dt = sc->step;
    int iend = (int) (1.0f + (tout - tin) / dt + 0.5f);
    if (sc->max_samples > 0 && iend > sc->max_samples) iend = sc->max_samples;
    if (iend <= 0) return c;
    *nalg += iend;
    *nexec += iend;
#define SAMPLE(I) ({ float t_ = tin + ((float) (I) * dt); \
        sample_ref(b, d.x * t_ + o.x, d.y * t_ + o.y, d.z * t_ + o.z); })
    float myalpha = tf->alpha;
    switch (sc->tf_mode) {
    case ORC_TF_MED: /* transferfuncs.c:24-68 */
        for (int i = 0; i < iend; ++i) {
            c4 e = lutat(tf, (int) SAMPLE(i) - tf->off);
            c.b = ((double) e.b < 0.8) ? fmaxf(e.b, c.b) : c.b;
            c.g = ((double) e.g < 0.8) ? fmaxf(e.g, c.g) : c.g;
            c.r = ((double) e.r < 0.8) ? fmaxf(e.r, c.r) : c.r;
            c.a = e.a * myalpha;
        }
        break;
    case ORC_TF_BLEND: /* transferfuncs.c:70-83: no lutoffset */
        for (int i = 0; i < iend; ++i) {
            c4 e = lutat(tf, (int) SAMPLE(i));
            float al = e.a;
            c.b = al * e.b + (1.0f - al) * c.b;
            c.g = al * e.g + (1.0f - al) * c.g;
            c.r = al * e.r + (1.0f - al) * c.r;
            c.a = al * myalpha;
        }
        break;
    case ORC_TF_SEISMIC2: /* transferfuncs.c:109-136 */
    case ORC_TF_CHEM:     /* transferfuncs.c:137-168 */
        for (int i = iend - 1; i >= 0; i--) {
            int idx = (int) SAMPLE(i) - tf->off;
            if (idx < 0) idx = 0;
            if (sc->tf_mode == ORC_TF_SEISMIC2 && idx > tf->n - 1) idx = tf->n - 1;
            c4 e = lutat(tf, idx);
            float al = e.a * myalpha;
            float oma = 1.0f - al;
            c.b = oma * c.b + al * e.b;
            c.g = oma * c.g + al * e.g;
            c.r = oma * c.r + al * e.r;
            c.a = al + oma * c.a;
            if (c.a > 1.0f) c.a = 1.0f;
        }
        break;
    case ORC_TF_RGBBLEND: /* transferfuncs.c:170-200 */
        for (int i = iend - 1; i >= 0; i--) {
            float s = SAMPLE(i);
            uint32_t u;
            memcpy(&u, &s, 4);
            float r = 1.0f / 255.0f * (float) ((u >> 24) & 0xff);
            float g = 1.0f / 255.0f * (float) ((u >> 16) & 0xff);
            float bl = 1.0f / 255.0f * (float) ((u >> 8) & 0xff);
            float al = myalpha;
            float oma = 1.0f - al;
            c.b = oma * c.b + al * bl;
            c.g = oma * c.g + al * g;
            c.r = oma * c.r + al * r;
            c.a = al + oma * c.a;
            if (c.a > 1.0f) c.a = 1.0f;
        }
        break;
    default: /* ORC_TF_SEISMIC, transferfuncs.c:86-107 */
        for (int i = 0; i < iend; ++i) {
            c4 e = lutat(tf, (int) SAMPLE(i) - tf->off);
            c.b = ((double) e.b > 0.65 && e.b < 1.0f) ? 0.6f : c.b;
            c.g = ((double) e.g > 0.65 && e.g < 1.0f) ? 0.0f : c.g;
            c.r = ((double) e.r > 0.65 && e.r < 1.0f) ? 0.0f : c.r;
            c.b = ((double) e.b > 0.5 && e.b < 0.65f) ? 0.9f : c.b;
            c.g = ((double) e.g > 0.5 && e.g < 0.65f) ? 0.9f : c.g;
            c.r = ((double) e.r > 0.5 && e.r < 0.65f) ? 0.9f : c.r;
            c.b = ((double) e.b > 0.3 && e.b < 0.5f) ? 0.0f : c.b;
            c.g = ((double) e.g > 0.3 && e.g < 0.5f) ? 0.0f : c.g;
            c.r = ((double) e.r > 0.3 && e.r < 0.5f) ? 0.6f : c.r;
            c.a = 1.0f * myalpha;
        }
        break;
    }
#undef SAMPLE
    return c;
}

/* ---------------------------------------------------- CONFIG ray cast --
 * One lattice per ray, t_i = fmaf(i, dt, t0) from the entry into the
 * clipped global box (t0 >= 0); brick k owns the samples with
 * tin_k <= t_i < tout_k.  Front-to-back premultiplied accumulation. */
static float cfg_t(float t0, float dt, int i) { return fmaf((float) i, dt, t0); }
#define CFG_MAX_LATTICE (1 << 24)
static int cfg_first_ge(float t0, float dt, float a)
{
    if (!(a > t0)) return 0;
    float q = (a - t0) / dt;
    int i = q < (float) CFG_MAX_LATTICE ? (int) q : CFG_MAX_LATTICE;
    for (int it = 0; it < 64 && i > 0 && cfg_t(t0, dt, i - 1) >= a; it++) i--;
    for (int it = 0; it < 64 && i < CFG_MAX_LATTICE && cfg_t(t0, dt, i) < a; it++) i++;
    return i;
}

typedef struct { float r, g, b, a; int done; } acc_t;

#define MC 16
/* Transparent-cell flags of one brick for a LUT: cell c spans local voxels
 * [c*16, min(c*16+16, n-1)] per axis; it is transparent when no LUT entry
 * between (int)(min*scale)-1 and (int)(max*scale)+1 (less the offset) has
 * non-zero opacity. */
static void brick_empty(brick_t *b, const orc_scene *sc)
{
    b->mcx = (b->lw - 2) / MC + 1;
    b->mcy = (b->lh - 2) / MC + 1;
    b->mcz = (b->ld - 2) / MC + 1;
    b->empty = (unsigned char *) malloc((size_t) b->mcx * b->mcy * b->mcz);
    int n = sc->lut_n;
    int *pre = (int *) calloc((size_t) n + 1, sizeof(int));
    for (int i = 0; i < n; i++) pre[i + 1] = pre[i] + (sc->lut[4 * i + 3] != 0.0f);
    for (int cz = 0; cz < b->mcz; cz++)
        for (int cy = 0; cy < b->mcy; cy++)
            for (int cx = 0; cx < b->mcx; cx++) {
                float lo = FLT_MAX, hi = -FLT_MAX;
                int x1 = cx * MC + MC < b->lw - 1 ? cx * MC + MC : b->lw - 1;
                int y1 = cy * MC + MC < b->lh - 1 ? cy * MC + MC : b->lh - 1;
                int z1 = cz * MC + MC < b->ld - 1 ? cz * MC + MC : b->ld - 1;
                for (int z = cz * MC; z <= z1; z++)
                    for (int y = cy * MC; y <= y1; y++)
                        for (int x = cx * MC; x <= x1; x++) {
                            float v = b->data[((size_t) z * b->lh + y) * b->lw + x];
                            lo = fminf(lo, v);
                            hi = fmaxf(hi, v);
                        }
                int a = clampi((int) (lo * sc->lut_scale) - 1 - sc->lut_offset, 0, n - 1);
                int c = clampi((int) (hi * sc->lut_scale) + 1 - sc->lut_offset, 0, n - 1);
                b->empty[((size_t) cz * b->mcy + cy) * b->mcx + cx] =
                    (sc->state.alpha == 0.0f || pre[c + 1] - pre[a] == 0) ? 1 : 0;
            }
    free(pre);
}

static void march_cfg(const orc_scene *sc, const brick_t *b, v3 o, v3 d, float t0, float dt,
                      const tf_t *tf, acc_t *acc, long long *nalg, long long *nexec)
{
    float tin, tout;
    v3 id = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    if (!ray_box_cfg(b->dconst, o, d, id, &tin, &tout)) return;
    int i0 = cfg_first_ge(t0, dt, tin);
    int i1 = cfg_first_ge(t0, dt, tout);
    if (i1 <= i0) return;
    *nalg += i1 - i0;
    if (acc->done) return;
    /* the lattice in the brick's voxel coordinates: index i samples
     * u_i = fmaf(i, s, base) per axis, s = (d ic) dt, base = fmaf(d ic, t0,
     * (o - bmin) ic) -- the point o + t_i d mapped by the brick's
     * world-to-voxel scaling ic */
    v3 du = {d.x * b->invcell.x, d.y * b->invcell.y, d.z * b->invcell.z};
    v3 st = {du.x * dt, du.y * dt, du.z * dt};
    v3 base = {fmaf(du.x, t0, (o.x - b->bmin.x) * b->invcell.x), fmaf(du.y, t0, (o.y - b->bmin.y) * b->invcell.y),
               fmaf(du.z, t0, (o.z - b->bmin.z) * b->invcell.z)};
    for (int i = i0; i < i1; i++) {
        float ux = fmaf((float) i, st.x, base.x), uy = fmaf((float) i, st.y, base.y),
              uz = fmaf((float) i, st.z, base.z);
        if (b->empty) {
            int cj = clampi((int) floorf(ux), 0, b->lw - 2) / MC;
            int ci = clampi((int) floorf(uy), 0, b->lh - 2) / MC;
            int ck = clampi((int) floorf(uz), 0, b->ld - 2) / MC;
            if (b->empty[((size_t) ck * b->mcy + ci) * b->mcx + cj]) {
                /* lattice index of the exit through the cell's voxel faces
                 * (in double); leap to one before it, so rounding never
                 * steps over a sample outside the cell */
                double qx = st.x > 0.0f ? ((double) ((cj + 1) * MC) - base.x) / st.x
                          : (st.x < 0.0f ? ((double) (cj * MC) - base.x) / st.x : 1e30);
                double qy = st.y > 0.0f ? ((double) ((ci + 1) * MC) - base.y) / st.y
                          : (st.y < 0.0f ? ((double) (ci * MC) - base.y) / st.y : 1e30);
                double qz = st.z > 0.0f ? ((double) ((ck + 1) * MC) - base.z) / st.z
                          : (st.z < 0.0f ? ((double) (ck * MC) - base.z) / st.z : 1e30);
                double q = fmin(qx, fmin(qy, qz));
                int inext = (q < (double) CFG_MAX_LATTICE ? (int) q : CFG_MAX_LATTICE) - 1;
                if (inext > i) i = (inext < i1 ? inext : i1) - 1;
                continue;
            }
        }
        float s = sample_cfg(b, ux, uy, uz);
        (*nexec)++;
        int idx = (int) (s * sc->lut_scale) - tf->off;
        c4 e = lutat(tf, idx);
        float al = e.a * tf->alpha;
        float wgt = (1.0f - acc->a) * al;
        acc->r = fmaf(wgt, e.r, acc->r);
        acc->g = fmaf(wgt, e.g, acc->g);
        acc->b = fmaf(wgt, e.b, acc->b);
        acc->a = acc->a + wgt;
        if (acc->a >= sc->term_alpha) { acc->done = 1; return; }
    }
}

/* CONFIG direction for pixel (i, j): ctm * (u_j, v_i, 5), pixel centres. */
static v3 cfg_dir(const view_t *v, int i, int j)
{
    float uu = v->left + ((float) j + 0.5f) * v->du;
    float vv = v->bottom + ((float) i + 0.5f) * v->dv;
    v3 d = {uu, vv, -v->cam_e.z};
    float ctm3[3][3];
    memcpy(ctm3, v->ctm, sizeof(ctm3));
    return m3v(ctm3, d);
}

/* sortboxlist (utils.c:175-199): Hoare quicksort on the centre depth with
 * the middle element as pivot.  Restated step for step because ties must
 * resolve to the same permutation. */
typedef struct { float d; int rank; } box_t;
static void sort_boxes(int l, int r, box_t *bl)
{
    int i = l, j = r;
    box_t mid = bl[(l + r) / 2], tmp;
    do {
        while (bl[i].d < mid.d) i++;
        while (bl[j].d > mid.d) j--;
        if (i <= j) {
            tmp = bl[i]; bl[i] = bl[j]; bl[j] = tmp;
            i++; j--;
        }
    } while (i <= j);
    if (l < j) sort_boxes(l, j, bl);
    if (i < r) sort_boxes(i, r, bl);
}

/* Exact front-to-back order for a regular brick grid: sort by the eye's
 * distance to each brick's interval along z, then y, then x. */
static float axis_dist(float e, float lo, float hi)
{
    if (e < lo) return lo - e;
    if (e > hi) return e - hi;
    return 0.0f;
}
static void order_axis(const brick_t *bs, int K, v3 eye, int *order)
{
    for (int k = 0; k < K; k++) order[k] = k;
    for (int a = 1; a < K; a++) { /* insertion sort: stable */
        int x = order[a], p = a - 1;
        const brick_t *bx = &bs[x];
        float kz = axis_dist(eye.z, bx->bmin.z, bx->bmax.z), ky = axis_dist(eye.y, bx->bmin.y, bx->bmax.y),
              kx = axis_dist(eye.x, bx->bmin.x, bx->bmax.x);
        while (p >= 0) {
            const brick_t *bp = &bs[order[p]];
            float pz = axis_dist(eye.z, bp->bmin.z, bp->bmax.z), py = axis_dist(eye.y, bp->bmin.y, bp->bmax.y),
                  px = axis_dist(eye.x, bp->bmin.x, bp->bmax.x);
            int greater = (pz > kz) || (pz == kz && (py > ky || (py == ky && px > kx)));
            if (!greater) break;
            order[p + 1] = order[p];
            p--;
        }
        order[p + 1] = x;
    }
}

static int in_rect(const brick_t *b, int i, int j)
{
    return i >= b->istrt && i < b->istop && j >= b->jstrt && j < b->jstop;
}

/* compositetiles (main.c:1203-1218) per pixel: d = s + (1 - s.a) * d */
static void over(float *d, const float *s)
{
    d[2] = s[2] + (1.0f - s[3]) * d[2];
    d[1] = s[1] + (1.0f - s[3]) * d[1];
    d[0] = s[0] + (1.0f - s[3]) * d[0];
    d[3] = s[3] + (1.0f - s[3]) * d[3];
}

struct orc_prepared {
    int K;
    float *data[ORC_MAX_BRICKS];
};

orc_prepared *orc_prepare(const orc_scene *sc)
{
    int K = sc->procdims[0] * sc->procdims[1] * sc->procdims[2];
    if (K < 1 || K > ORC_MAX_BRICKS) return NULL;
    orc_prepared *p = (orc_prepared *) calloc(1, sizeof(orc_prepared));
    view_t v;
    view_setup(sc, &v);
    p->K = K;
    for (int k = 0; k < K; k++) {
        brick_t b;
        brick_setup(sc, &v, k, &b);
        brick_load(sc, &b);
        p->data[k] = b.data;
    }
    return p;
}

void orc_prepared_free(orc_prepared *p)
{
    if (!p) return;
    for (int k = 0; k < p->K; k++) free(p->data[k]);
    free(p);
}

int orc_render(const orc_scene *sc, int nthreads, float *rgba32, unsigned char *rgba8,
               float *bricks, orc_stats *st)
{
    return orc_render_prepared(sc, NULL, nthreads, rgba32, rgba8, bricks, st);
}

int orc_render_prepared(const orc_scene *sc, const orc_prepared *prep, int nthreads, float *rgba32,
                        unsigned char *rgba8, float *bricks, orc_stats *st)
{
    int K = sc->procdims[0] * sc->procdims[1] * sc->procdims[2];
    if (K < 1 || K > ORC_MAX_BRICKS) return -1;
    if (sc->gw < 2 || sc->gh < 2 || sc->gd < 2 || sc->tilew < 1 || sc->tileh < 1) return -2;
    if (sc->tf_mode != ORC_TF_RGBBLEND && (!sc->lut || sc->lut_n < 1)) return -3;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    view_t v;
    view_setup(sc, &v);
    int vw = v.vw, vh = v.vh;
    if (vw < 1 || vh < 1) return -4;
    brick_t *bs = (brick_t *) calloc((size_t) K, sizeof(brick_t));
    if (prep && prep->K != K) { free(bs); return -5; }
    for (int k = 0; k < K; k++) {
        brick_setup(sc, &v, k, &bs[k]);
        if (prep) bs[k].data = prep->data[k];
        else brick_load(sc, &bs[k]);
        if (sc->skip && sc->preset == ORC_PRESET_CONFIG) brick_empty(&bs[k], sc);
    }
    int order[ORC_MAX_BRICKS];
    if (sc->order == ORC_ORDER_AXIS) {
        order_axis(bs, K, v.orig, order);
    } else {
        box_t bl[ORC_MAX_BRICKS];
        for (int k = 0; k < K; k++) { bl[k].d = bs[k].wc[5]; bl[k].rank = k; }
        sort_boxes(0, K - 1, bl);
        for (int k = 0; k < K; k++) order[k] = bl[k].rank;
    }
    tf_t tf = {(const c4 *) sc->lut, sc->lut_n, sc->lut_offset, sc->state.alpha};
    int r0 = sc->row0 > 0 ? sc->row0 : 0;
    int r1 = (sc->row1 > 0 && sc->row1 < vh) ? sc->row1 : vh;

    /* global box for the CONFIG lattice anchor */
    float gdconst[6];
    float step_world = 0.0f;
    if (sc->preset == ORC_PRESET_CONFIG) {
        int mx = sc->gw > sc->gh ? sc->gw : sc->gh;
        mx = mx > sc->gd ? mx : sc->gd;
        float invdim = 1.0f / (float) mx;
        float s3[3] = {(float) sc->gw * invdim, (float) sc->gh * invdim, (float) sc->gd * invdim};
        for (int a = 0; a < 3; a++) {
            float lo = -s3[a], hi = s3[a];
            float p0 = lo * -1.0f, p1 = hi * 1.0f;
            gdconst[2 * a] = sc->state.newconst[2 * a] < p0 ? sc->state.newconst[2 * a] : p0;
            gdconst[2 * a + 1] = sc->state.newconst[2 * a + 1] < p1 ? sc->state.newconst[2 * a + 1] : p1;
        }
        step_world = sc->step * (2.0f / (float) mx);
    }

    long long nalg = 0, nexec = 0;
    size_t npix = (size_t) vw * vh;
    float *img = (float *) calloc(npix * 4, sizeof(float));
    if (bricks) memset(bricks, 0, sizeof(float) * 4 * npix * (size_t) K);

#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nalg, nexec)
    for (int i = r0; i < r1; i++) {
        if (sc->preset == ORC_PRESET_REF) {
            /* far -> near over of per-brick colours; each brick casts its own
             * rays with the sequential direction increments of
             * createlocalimage (main.c:984-1008) */
            for (int s = K - 1; s >= 0; s--) {
                const brick_t *b = &bs[order[s]];
                if (i < b->istrt || i >= b->istop) continue;
                v3 d;
                d.x = b->dir0.x + v.incri.x * (float) (i - b->istrt);
                d.y = b->dir0.y + v.incri.y * (float) (i - b->istrt);
                d.z = b->dir0.z + v.incri.z * (float) (i - b->istrt);
                for (int j = b->jstrt; j < b->jstop; j++) {
                    d.x += v.incrj.x; d.y += v.incrj.y; d.z += v.incrj.z;
                    if (j < 0 || j >= vw) continue;
                    c4 c = raycast_ref(sc, b, v.orig, d, &tf, &nalg, &nexec);
                    float cs[4] = {c.r, c.g, c.b, c.a};
                    size_t p = ((size_t) i * vw + j) * 4;
                    over(img + p, cs);
                    if (bricks) memcpy(bricks + (size_t) order[s] * npix * 4 + p, cs, sizeof(cs));
                }
            }
        } else {
            for (int j = 0; j < vw; j++) {
                int any = 0;
                for (int k = 0; k < K; k++) any |= in_rect(&bs[k], i, j);
                if (!any) continue;
                v3 d = cfg_dir(&v, i, j);
                v3 id = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
                float tin, tout;
                if (!ray_box_cfg(gdconst, v.orig, d, id, &tin, &tout)) continue;
                float t0 = tin > 0.0f ? tin : 0.0f;
                float len = sqrtf(fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x)));
                float dt = step_world / len;
                acc_t acc = {0.0f, 0.0f, 0.0f, 0.0f, !(dt > 0.0f)};
                size_t p = ((size_t) i * vw + j) * 4;
                for (int s = 0; s < K; s++) {
                    const brick_t *b = &bs[order[s]];
                    if (!in_rect(b, i, j)) continue;
                    if (bricks) {
                        acc_t one = {0.0f, 0.0f, 0.0f, 0.0f, 0};
                        long long na = 0, ne = 0;
                        march_cfg(sc, b, v.orig, d, t0, dt, &tf, &one, &na, &ne);
                        float cs[4] = {one.r, one.g, one.b, one.a};
                        memcpy(bricks + (size_t) order[s] * npix * 4 + p, cs, sizeof(cs));
                    }
                    march_cfg(sc, b, v.orig, d, t0, dt, &tf, &acc, &nalg, &nexec);
                }
                img[p + 0] = acc.r; img[p + 1] = acc.g; img[p + 2] = acc.b; img[p + 3] = acc.a;
            }
        }
    }

    if (rgba32) memcpy(rgba32, img, sizeof(float) * 4 * npix);
    if (rgba8) orc_quantize(img, rgba8, (long long) npix * 4);
    if (st) {
        st->samples_alg = nalg;
        st->samples_exec = nexec;
        st->vw = vw; st->vh = vh; st->nbricks = K;
        for (int k = 0; k < K; k++) {
            memcpy(st->wincoord[k], bs[k].wc, sizeof(bs[k].wc));
            st->order[k] = order[k];
            st->rect[k][0] = bs[k].istrt; st->rect[k][1] = bs[k].istop;
            st->rect[k][2] = bs[k].jstrt; st->rect[k][3] = bs[k].jstop;
        }
    }
    free(img);
    for (int k = 0; k < K; k++) {
        if (!prep) free(bs[k].data);
        free(bs[k].empty);
    }
    free(bs);
    return K;
}

void orc_composite(float *dst, const float *sub, const int *order, int num, int npix)
{
    for (int s = num - 1; s >= 0; s--) {
        const float *src = sub + (size_t) order[s] * npix * 4;
        for (int p = 0; p < npix; p++) over(dst + (size_t) p * 4, src + (size_t) p * 4);
    }
}

void orc_quantize(const float *in, unsigned char *out, long long n)
{
    for (long long i = 0; i < n; i++) {
        float v = in[i];
        if (!(v > 0.0f)) out[i] = 0;
        else if (v >= 1.0f) out[i] = 255;
        else out[i] = (unsigned char) (int) ((double) v * 255.0 + 0.5);
    }
}

/* ------------------------------------------------------------ colormaps --
 * colormap.c:21-181.  Double arithmetic where the reference mixes double
 * constants in.  rainbowcolormap adds to entries it never initialises
 * (colormap.c:65-76); here they start at zero. */
void orc_colormap(int type, float *lut, int hsize, float histmin, float histmax)
{
    c4 *L = (c4 *) lut;
    switch (type) {
    case 0: /* basecolormap */
        for (int i = 0; i < hsize; i++) {
            float c = (float) (i + histmin) / histmax;
            L[i].b = L[i].g = L[i].r = c;
            if (c > 0.8) { L[i].r = 0.7f; L[i].g = 0.75f; L[i].b = (float) 0.46; L[i].a = (float) 0.07; }
            if (c < 0.3) { L[i].b = (float) 0.6; L[i].a = (float) 0.01; }
            if (c > 0.3 && c < 0.6) { L[i].r = (float) 0.6; L[i].a = (float) 0.01; }
            if (c > 0.6 && c < 0.8) { L[i].r = (float) 0.6; L[i].g = (float) 0.6; L[i].a = (float) 0.005; }
        }
        break;
    case 1: { /* rainbowcolormap */
        memset(L, 0, sizeof(c4) * (size_t) hsize);
        L[0].b = 1.0f; L[0].g = 0.0f; L[0].r = 0.0f;
        float dr = 1.0f / hsize, db = -dr;
        for (int i = 0; i < hsize; i++) { L[i].r += dr; L[i].b += db; L[i].a = 1.0f; }
        break;
    }
    case 2: { /* medcolormap */
        float parm[4] = {(float) 0.04, (float) 0.9, (float) 0.9, (float) 0.8};
        for (int i = 0; i < hsize; i++) {
            float x = i / (float) (hsize - 1) * 4096.0f, a, y1, y2;
            if ((0 <= x) && (x <= 484)) {
                L[i].r = (float) 0.1; L[i].g = (float) 0.1; L[i].b = (float) 0.1; L[i].a = (float) (0.1 * parm[0]);
            } else if ((484 < x) && (x <= 545)) {
                a = (float) ((x - 484.0) / (545.0 - 484.0));
                y1 = (float) ((1.0 - a) * parm[0]); y2 = (float) (a * parm[1]);
                L[i].r = (float) (0.6 * y1 + 0.8 * y2); L[i].g = (float) (0.6 * y1 + 0.7 * y2);
                L[i].b = (float) (0.8 * y1 + 0.0 * y2); L[i].a = (float) (0.1 * y1 + 0.03125 * y2);
            } else if ((545 < x) && (x <= 726)) {
                L[i].r = (float) 0.8; L[i].g = (float) 0.7; L[i].b = 0.0f; L[i].a = (float) (0.03125 * parm[1]);
            } else if ((726 < x) && (x <= 819)) {
                a = (float) ((x - 726.0) / (819.0 - 726.0));
                y1 = (float) ((1.0 - a) * parm[1]); y2 = (float) (a * parm[2]);
                L[i].r = (float) (0.8 * y1 + 0.2 * y2); L[i].g = (float) (0.7 * y1 + 0.0 * y2);
                L[i].b = (float) (0.0 * y1 + 0.0 * y2); L[i].a = (float) (0.03125 * y1 + 0.1875 * y2);
            } else if ((819 < x) && (x <= 883)) {
                L[i].r = (float) 0.2; L[i].g = 0.0f; L[i].b = 0.0f; L[i].a = (float) (0.1875 * parm[2]);
            } else if ((883 < x) && (x <= 1535)) {
                a = (float) ((x - 883.0) / (1535.0 - 883.0));
                y1 = (float) ((1.0 - a) * parm[2]); y2 = (float) (a * parm[3]);
                L[i].r = (float) (0.2 * y1 + 1.0 * y2); L[i].g = (float) (0.0 * y1 + 1.0 * y2);
                L[i].b = (float) (0.0 * y1 + 0.9 * y2); L[i].a = (float) (0.1875 * y1 + 0.75 * y2);
            } else if (1535 < x) {
                L[i].r = 1.0f; L[i].g = 1.0f; L[i].b = (float) 0.9; L[i].a = (float) (0.75 * parm[3]);
            }
        }
        break;
    }
    case 3: { /* seismiccolormap with mathutil.h:42-59 lerp */
        float er[3] = {1.0f, 1.0f, 0.0f}, eg[3] = {0.0f, 1.0f, 0.0f}, eb[3] = {0.0f, 1.0f, 1.0f};
        float s0[3] = {1.0f, 0.5f * hsize, (float) hsize};
        float *ends[3] = {er, eg, eb};
        for (int ch = 0; ch < 3; ch++) {
            float *v1 = ends[ch];
            float inc1 = (v1[1] - v1[0]) / (s0[1] - s0[0]);
            float inc2 = (v1[2] - v1[1]) / (s0[2] - s0[1]);
            for (int i = 1; i <= hsize; i++) {
                float val;
                if ((i >= s0[0]) && (i <= s0[1])) val = v1[0] + i * inc1;
                else if ((i >= s0[1]) && (i <= s0[2])) val = v1[1] + (i - s0[1]) * inc2;
                else continue;
                if (ch == 0) L[i - 1].r = val;
                else if (ch == 1) L[i - 1].g = val;
                else L[i - 1].b = val;
            }
        }
        for (int i = 0; i < hsize; i++) L[i].a = 1.0f;
        break;
    }
    case 4: /* jetcolormap */
        for (int i = 0; i < hsize; i++) {
            float i4 = (4.0f * i) / hsize;
            L[i].r = (float) fmin(fmax(fmin(i4 - 1.5, -i4 + 4.5), 0.0f), 1.0f);
            L[i].g = (float) fmin(fmax(fmin(i4 - 0.5, -i4 + 3.5), 0.0f), 1.0f);
            L[i].b = (float) fmin(fmax(fmin(i4 + 0.5, -i4 + 2.5), 0.0f), 1.0f);
            L[i].a = 1.0f;
        }
        break;
    default: /* nomap */
        break;
    }
}

/* histogram (mathutil.c:444-470): min/max, hsize = (int)(max-min+1),
 * bin = (int)(v - min). */
int orc_minmax(const void *data, int dtype, long long n, float *mn, float *mx)
{
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (long long i = 0; i < n; i++) {
        float v = vox(data, dtype, i);
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
    }
    *mn = lo;
    *mx = hi;
    return (int) ((hi - lo) + 1);
}

void orc_histogram(const void *data, int dtype, long long n, float mn, int hsize, int *hist)
{
    memset(hist, 0, sizeof(int) * (size_t) hsize);
    for (long long i = 0; i < n; i++) {
        int b = (int) (vox(data, dtype, i) - mn);
        if (b >= 0 && b < hsize) hist[b]++;
    }
}

void orc_macrocells(const float *vol, int w, int h, int d, int cell, float *cmin, float *cmax)
{
    int cx = (w + cell - 1) / cell, cy = (h + cell - 1) / cell, cz = (d + cell - 1) / cell;
    for (int kz = 0; kz < cz; kz++)
        for (int ky = 0; ky < cy; ky++)
            for (int kx = 0; kx < cx; kx++) {
                float lo = FLT_MAX, hi = -FLT_MAX;
                int z1 = (kz + 1) * cell, y1 = (ky + 1) * cell, x1 = (kx + 1) * cell;
                z1 = z1 < d - 1 ? z1 : d - 1; y1 = y1 < h - 1 ? y1 : h - 1; x1 = x1 < w - 1 ? x1 : w - 1;
                for (int z = kz * cell; z <= z1; z++)
                    for (int y = ky * cell; y <= y1; y++)
                        for (int x = kx * cell; x <= x1; x++) {
                            float v = vol[((size_t) z * h + y) * w + x];
                            lo = fminf(lo, v);
                            hi = fmaxf(hi, v);
                        }
                size_t c = ((size_t) kz * cy + ky) * cx + kx;
                cmin[c] = lo;
                cmax[c] = hi;
            }
}

/* gradient3d (mathutil.c:242-325) with grad() (mathutil.c:326-337) and the
 * index map maptoffset3d (mathutil.h:139-143): per voxel (row i, column j,
 * slab k) x from columns, y from rows, z from slabs; a central difference
 * halved inside, (V(1) - V(0)) / 2 and (V(n-1) - V(n-2)) / 2 on the faces
 * (the reference's face formulas), then times the unit spacing, and
 * w = mag3f(x, y, z) (mathutil.c:233-236).  Restated as intended: the
 * reference writes every voxel to offset i*j*k, takes the k = p-1 face from
 * k-1 and k-2, and leaves edges and corners unwritten; here every voxel gets
 * the per-axis rule at its own offset. */
static float grad_axis(const float *v, long long o, int c, int n, long long stride)
{
    if (c == 0) return (v[o + stride] - v[o]) / 2.0f * 1.0f;
    if (c == n - 1) return (v[o] - v[o - stride]) / 2.0f * 1.0f;
    return (v[o + stride] - v[o - stride]) / 2.0f * 1.0f;
}

void orc_gradient(const float *vol, int w, int h, int d, float *out)
{
    for (int k = 0; k < d; k++)
        for (int i = 0; i < h; i++)
            for (int j = 0; j < w; j++) {
                const long long o = ((long long) k * h + i) * w + j;
                const float x = grad_axis(vol, o, j, w, 1);
                const float y = grad_axis(vol, o, i, h, w);
                const float z = grad_axis(vol, o, k, d, (long long) w * h);
                out[4 * o + 0] = x;
                out[4 * o + 1] = y;
                out[4 * o + 2] = z;
                out[4 * o + 3] = sqrtf(x * x + y * y + z * z);
            }
}
