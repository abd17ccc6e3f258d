// ivr_frame.cpp -- host-side frame geometry: brick decomposition, camera,
// viewport, ray frame, projected brick rectangles and composite order.
//
// This is the set-up half of the reference's per-frame path.  Its float
// arithmetic is evaluated in the reference's order (compiled with
// -ffp-contract=off, no excess precision), because the kernels consume
// these numbers and the REF preset is bit-compatible with the reference.
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <tuple>

#include "ivr_frame.h"

namespace ivr {
namespace {

struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

// mathutil.c:28-38 dot3f/dot4f: left-to-right sums of rounded products
float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float dot4(V4 a, V4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

V3 mul3(const float m[3][3], V3 v)  // mat3fxvec3f (mathutil.c:129-149)
{
    V3 r0 = {m[0][0], m[0][1], m[0][2]}, r1 = {m[1][0], m[1][1], m[1][2]}, r2 = {m[2][0], m[2][1], m[2][2]};
    return V3{dot3(r0, v), dot3(r1, v), dot3(r2, v)};
}

void mul33(float io[3][3], const float in[3][3])  // mat3fxmat3f (mathutil.c:150-171)
{
    float t[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t[i][j] = dot3(V3{io[i][0], io[i][1], io[i][2]}, V3{in[0][j], in[1][j], in[2][j]});
    memcpy(io, t, sizeof(t));
}

void mul44(float io[4][4], const float in[4][4])  // mat4fxmat4f (mathutil.c:172-196)
{
    float t[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            t[i][j] = dot4(V4{io[i][0], io[i][1], io[i][2], io[i][3]}, V4{in[0][j], in[1][j], in[2][j], in[3][j]});
    memcpy(io, t, sizeof(t));
}

V4 mul4(const float m[4][4], V4 v)  // mat4fxvec4f (mathutil.c:197-219)
{
    float t[4];
    for (int j = 0; j < 4; j++) t[j] = dot4(V4{m[j][0], m[j][1], m[j][2], m[j][3]}, v);
    return V4{t[0], t[1], t[2], t[3]};
}

void gl_to_rows(float m[4][4], const float cm[16])  // setmvm/setpm (mathutil.h:212-233)
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) m[r][c] = cm[c * 4 + r];
}

float axis_gap(float e, float lo, float hi) { return e < lo ? lo - e : (e > hi ? e - hi : 0.0f); }

}  // namespace

// getlocalbrick (utils.c:332-388) and the AABB of initvolbbox
// (main.c:505-608) for brick `rank`; rank order is slab-major, then row,
// then column (main.c:536-546).
void brick_geometry(int gw, int gh, int gd, int py, int px, int pz, int overlap, int rank, HostBrick &b)
{
    int mx = std::max(gw, std::max(gh, gd));
    float maxdim = (float) mx;
    float invdim = 1.0f / maxdim;
    float sfx = (float) gw * invdim, sfy = (float) gh * invdim, sfz = (float) gd * invdim;
    b.slab = rank / (py * px);
    b.row = (rank / px) % py;
    b.col = rank % px;
    int lw = gw / px, lh = gh / py, ld = gd / pz;
    int rw = gw % (lw * px), rh = gh % (lh * py), rd = gd % (ld * pz);
    b.sx = b.col * lw;
    b.sy = b.row * lh;
    b.sz = b.slab * ld;
    if (b.col == px - 1) lw += rw;
    if (b.row == py - 1) lh += rh;
    if (b.slab == pz - 1) ld += rd;
    b.cw = lw;
    b.ch = lh;
    b.cd = ld;
    float rangex = sfx * 2.0f, rangey = sfy * 2.0f, rangez = sfz * 2.0f;
    float bw = 2.0f * sfx * ((float) lw / (float) gw);
    float bh = 2.0f * sfy * ((float) lh / (float) gh);
    float bd = 2.0f * sfz * ((float) ld / (float) gd);
    float bx = -sfx + rangex * ((float) b.sx / (float) gw);
    float by = -sfy + rangey * ((float) b.sy / (float) gh);
    float bz = -sfz + rangez * ((float) b.sz / (float) gd);
    b.lw = (b.col == px - 1) ? lw : lw + overlap;
    b.lh = (b.row == py - 1) ? lh : lh + overlap;
    b.ld = (b.slab == pz - 1) ? ld : ld + overlap;
    // the AABB's 8 vertices are {bx, bx+bw} x {by, by+bh} x {bz, bz+bd}
    float x1 = bx + bw, y1 = by + bh, z1 = bz + bd;
    b.bminx = fminf(bx, x1); b.bmaxx = fmaxf(bx, x1);
    b.bminy = fminf(by, y1); b.bmaxy = fmaxf(by, y1);
    b.bminz = fminf(bz, z1); b.bmaxz = fmaxf(bz, z1);
    b.w = b.bmaxx - b.bminx;
    b.h = b.bmaxy - b.bminy;
    b.d = b.bmaxz - b.bminz;
}

int build_frame(int gw, int gh, int gd, int dtype, const HostBrick *bricks, int nb, const ivr_state &st,
                const ivr_render_params &p, FrameDesc &f, ivr_frame_info &info)
{
    memset(&f, 0, sizeof(f));
    memset(&info, 0, sizeof(info));
    if (p.tilew < 1 || p.tileh < 1 || st.winwidth < 1 || st.winheight < 1) return IVR_ERR_INVALID;
    if (nb < 1 || nb > kMaxBricks) return IVR_ERR_INVALID;

    // initcamera (main.c:428-500): n = (0,0,-1), v = normalize(0,1,0),
    // u = n x v, e = (0,0,-5), r = 0; vwm columns u, v, n (setvwm)
    V3 n{0.0f, 0.0f, -1.0f}, up{0.0f, 1.0f, 0.0f};
    float mag = sqrtf(up.x * up.x + up.y * up.y + up.z * up.z);
    V3 cv{up.x / mag, up.y / mag, up.z / mag};
    V3 cu{n.y * cv.z - n.z * cv.y, n.z * cv.x - n.x * cv.z, n.x * cv.y - n.y * cv.x};
    float vwm[3][3] = {{cu.x, cv.x, n.x}, {cu.y, cv.y, n.y}, {cu.z, cv.z, n.z}};
    V3 cam_e{0.0f, 0.0f, -5.0f}, cam_r{0.0f, 0.0f, 0.0f};

    // setviewport (mathutil.h:147-163) with x = y = 0
    int tilex = st.winwidth / p.tilew, tiley = st.winheight / p.tileh;
    float vpw = (float) (tilex * p.tilew), vph = (float) (tiley * p.tileh), vpx = 0.0f, vpy = 0.0f;
    int w = (int) vpw, h = (int) vph;
    if (w < 1 || h < 1) return IVR_ERR_INVALID;
    float vpm[4][4] = {{0}};
    vpm[0][0] = w / 2.0f; vpm[0][3] = (0 + w) / 2.0f;
    vpm[1][1] = h / 2.0f; vpm[1][3] = (0 + h) / 2.0f;
    vpm[2][2] = 0.5f; vpm[2][3] = 0.5f;
    vpm[3][3] = 1.0f;

    float mvm[4][4], pm[4][4];
    gl_to_rows(mvm, st.mvm);
    gl_to_rows(pm, st.pm);
    float left = st.vv[0], right = st.vv[1], bottom = st.vv[2], top = st.vv[3];

    // createlocalimage (main.c:950-951)
    float du = (right - left) / vpw;
    float dv = (top - bottom) / vph;

    // buildray (mathutil.c:1115-1154), brick-independent part
    V3 ii{0.0f, dv, 0.0f}, jj{du, 0.0f, 0.0f};
    V3 trans{mvm[0][3], mvm[1][3], 0.0f};
    V3 eye = mul3(vwm, cam_e);
    eye = V3{eye.x + cam_r.x, eye.y + cam_r.y, eye.z + cam_r.z};
    V3 o{eye.x - trans.x, eye.y - trans.y, eye.z - trans.z};
    float ctm[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) ctm[i][j] = mvm[j][i];
    V3 orig = mul3(ctm, o);
    mul33(ctm, vwm);
    V3 incri = mul3(ctm, ii), incrj = mul3(ctm, jj);

    // updatevolbbox (mathutil.c:948-1018): ctm = pm * mvm
    float pmv[4][4];
    memcpy(pmv, pm, sizeof(pmv));
    mul44(pmv, mvm);

    f.vw = w;
    f.vh = h;
    f.nb = nb;
    f.preset = p.preset;
    f.dtype = dtype;
    f.origx = orig.x; f.origy = orig.y; f.origz = orig.z;
    f.incrix = incri.x; f.incriy = incri.y; f.incriz = incri.z;
    f.incrjx = incrj.x; f.incrjy = incrj.y; f.incrjz = incrj.z;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) f.ctm[i * 3 + j] = ctm[i][j];
    f.left = left; f.bottom = bottom; f.du = du; f.dv = dv;
    f.eyen = -cam_e.z;
    f.max_samples = p.max_samples;
    f.term_alpha = p.term_alpha;
    f.alpha = st.alpha;
    f.single = -1;
    info.vw = w;
    info.vh = h;
    info.nbricks = nb;

    for (int k = 0; k < nb; k++) {
        const HostBrick &hb = bricks[k];
        DevBrick &b = f.b[k];
        b.data = hb.data;
        b.quad = hb.quad;
        b.nx = hb.lw; b.ny = hb.lh; b.nz = hb.ld;
        b.bminx = hb.bminx; b.bminy = hb.bminy; b.bminz = hb.bminz;
        b.w = hb.w; b.h = hb.h; b.d = hb.d;
        b.icx = (float) hb.cw / hb.w;
        b.icy = (float) hb.ch / hb.h;
        b.icz = (float) hb.cd / hb.d;
        b.mcx = hb.mcx; b.mcy = hb.mcy; b.mcz = hb.mcz;
        b.mcwx = (float) hb.cell / b.icx;
        b.mcwy = (float) hb.cell / b.icy;
        b.mcwz = (float) hb.cell / b.icz;
        b.vwx = 1.0f / b.icx;
        b.vwy = 1.0f / b.icy;
        b.vwz = 1.0f / b.icz;
        b.cshift = 0;
        while ((1 << b.cshift) < hb.cell) b.cshift++;
        // pzero (main.c:616-618) and setplaneconst (ray.c:44-51)
        float pz0[6] = {hb.bminx * -1.0f, hb.bmaxx * 1.0f, hb.bminy * -1.0f,
                        hb.bmaxy * 1.0f, hb.bminz * -1.0f, hb.bmaxz * 1.0f};
        for (int i = 0; i < 6; i++) b.dconst[i] = (st.newconst[i] < pz0[i]) ? st.newconst[i] : pz0[i];

        // project the 8 vertices to window coordinates
        float wminx = FLT_MAX, wminy = FLT_MAX, wminz = FLT_MAX;
        float wmaxx = -FLT_MAX, wmaxy = -FLT_MAX, wmaxz = -FLT_MAX;
        for (int c = 0; c < 8; c++) {
            V4 vert{(c & 1) ? hb.bmaxx : hb.bminx, (c & 2) ? hb.bmaxy : hb.bminy, (c & 4) ? hb.bmaxz : hb.bminz, 1.0f};
            // the reference's vertices are bx+bw etc.; bmax holds that sum
            V4 pc = mul4(pmv, vert);
            float ww = pc.w;
            V4 ndc{pc.x / ww, pc.y / ww, pc.z / ww, 1.0f};
            V4 win = mul4(vpm, ndc);
            wminx = fminf(wminx, win.x); wminy = fminf(wminy, win.y); wminz = fminf(wminz, win.z);
            wmaxx = fmaxf(wmaxx, win.x); wmaxy = fmaxf(wmaxy, win.y); wmaxz = fmaxf(wmaxz, win.z);
        }
        float xe = vpx + vpw, ye = vpy + vph;
        wminx = (wminx < vpx) ? vpx : wminx;
        wmaxx = (wmaxx > xe) ? xe : wmaxx;
        wminx = (wminx > xe) ? xe : wminx;
        wmaxx = (wmaxx < vpx) ? vpx : wmaxx;
        wminy = (wminy < vpy) ? vpy : wminy;
        wmaxy = (wmaxy > ye) ? ye : wmaxy;
        wminy = (wminy > ye) ? ye : wminy;
        wmaxy = (wmaxy < vpy) ? vpy : wmaxy;
        float wc[6] = {wminx, wminy, wmaxz, wmaxx - wminx, wmaxy - wminy, (wmaxz + wminz) / 2.0f};
        memcpy(info.wincoord[k], wc, sizeof(wc));

        // createlocalimage rect and first ray (main.c:959-981); the rect is
        // clamped to the viewport here (the reference writes one row and
        // column past it, main.c:959-962)
        int istrt = (int) (wc[1] - 0.5f), istop = (int) (wc[1] + wc[4] + 1.0f);
        int jstrt = (int) (wc[0] - 0.5f), jstop = (int) (wc[0] + wc[3] + 1.0f);
        info.rect[k][0] = istrt; info.rect[k][1] = istop; info.rect[k][2] = jstrt; info.rect[k][3] = jstop;
        b.istrt = istrt; b.istop = std::min(istop, h);
        b.jstrt = jstrt; b.jstop = std::min(jstop, w);
        float vv = bottom + istrt * dv + dv / 2.0f;
        float uu = left + jstrt * du - du / 2.0f;
        V3 d0 = mul3(ctm, V3{uu, vv, -cam_e.z});
        b.dir0x = d0.x; b.dir0y = d0.y; b.dir0z = d0.z;
    }

    // composite order, near -> far
    int order[kMaxBricks];
    if (p.order == IVR_ORDER_AXIS) {
        // exact for a regular grid: by the eye's distance to each brick's
        // interval along z, then y, then x (stable)
        for (int k = 0; k < nb; k++) order[k] = k;
        auto key = [&](int k) {
            const HostBrick &hb = bricks[k];
            return std::make_tuple(axis_gap(orig.z, hb.bminz, hb.bmaxz), axis_gap(orig.y, hb.bminy, hb.bmaxy),
                                   axis_gap(orig.x, hb.bminx, hb.bmaxx));
        };
        std::stable_sort(order, order + nb, [&](int a, int b) { return key(a) < key(b); });
    } else {
        // sortboxlist (utils.c:175-199): Hoare partition, middle pivot, on
        // the centre depth; the same steps give the same order for ties
        struct Box { float d; int rank; } bl[kMaxBricks];
        for (int k = 0; k < nb; k++) bl[k] = Box{info.wincoord[k][5], k};
        struct Sorter {
            static void run(Box *a, int l, int r)
            {
                int i = l, j = r;
                Box mid = a[(l + r) / 2];
                do {
                    while (a[i].d < mid.d) i++;
                    while (a[j].d > mid.d) j--;
                    if (i <= j) {
                        Box t = a[i]; a[i] = a[j]; a[j] = t;
                        i++; j--;
                    }
                } while (i <= j);
                if (l < j) run(a, l, j);
                if (i < r) run(a, i, r);
            }
        };
        Sorter::run(bl, 0, nb - 1);
        for (int k = 0; k < nb; k++) order[k] = bl[k].rank;
    }
    for (int k = 0; k < nb; k++) { f.order[k] = order[k]; info.order[k] = order[k]; }

    if (p.preset == IVR_PRESET_CONFIG) {
        // one lattice per ray, anchored on the clipped global box
        float sf[3] = {(float) gw / (float) std::max(gw, std::max(gh, gd)), 0, 0};
        int mx = std::max(gw, std::max(gh, gd));
        float invdim = 1.0f / (float) mx;
        sf[0] = (float) gw * invdim;
        sf[1] = (float) gh * invdim;
        sf[2] = (float) gd * invdim;
        for (int a = 0; a < 3; a++) {
            float p0 = -sf[a] * -1.0f, p1 = sf[a] * 1.0f;
            f.gdconst[2 * a] = st.newconst[2 * a] < p0 ? st.newconst[2 * a] : p0;
            f.gdconst[2 * a + 1] = st.newconst[2 * a + 1] < p1 ? st.newconst[2 * a + 1] : p1;
        }
        f.step = p.step * (2.0f / (float) mx);
    } else {
        f.step = p.step;
    }
    return IVR_OK;
}

}  // namespace ivr
