// ivr_colormap.cpp -- the reference's LUT builders (colormap.c:21-181),
// evaluated with the reference's float/double mix so the tables match it
// bit for bit.  Entries a builder leaves unset stay zero (rainbowcolormap
// reads uninitialised memory in the reference, colormap.c:65-76).
#include <math.h>
#include <string.h>

#include "ivr_frame.h"

namespace ivr {
namespace {

struct Rgba { float r, g, b, a; };

void base(Rgba *L, int n, float hmin, float hmax)  // colormap.c:24-60
{
    for (int i = 0; i < n; i++) {
        const float c = (float) (i + hmin) / hmax;
        L[i].r = L[i].g = L[i].b = c;
        if (c > 0.8) { L[i].r = 0.7f; L[i].g = 0.75f; L[i].b = (float) 0.46; L[i].a = (float) 0.07; }
        if (c < 0.3) { L[i].b = (float) 0.6; L[i].a = (float) 0.01; }
        if (c > 0.3 && c < 0.6) { L[i].r = (float) 0.6; L[i].a = (float) 0.01; }
        if (c > 0.6 && c < 0.8) { L[i].r = (float) 0.6; L[i].g = (float) 0.6; L[i].a = (float) 0.005; }
    }
}

void rainbow(Rgba *L, int n)  // colormap.c:62-77
{
    L[0].b = 1.0f;
    L[0].g = 0.0f;
    L[0].r = 0.0f;
    const float dr = 1.0f / n, db = -dr;
    for (int i = 0; i < n; i++) {
        L[i].r += dr;
        L[i].b += db;
        L[i].a = 1.0f;
    }
}

// one piece of medcolormap: a blend between two tissue classes
void med_blend(Rgba &e, float x, double x0, double x1, float p0, float p1, const double c0[4], const double c1[4])
{
    const float a = (float) ((x - x0) / (x1 - x0));
    const float y1 = (float) ((1.0 - a) * p0), y2 = (float) (a * p1);
    e.r = (float) (c0[0] * y1 + c1[0] * y2);
    e.g = (float) (c0[1] * y1 + c1[1] * y2);
    e.b = (float) (c0[2] * y1 + c1[2] * y2);
    e.a = (float) (c0[3] * y1 + c1[3] * y2);
}

void medical(Rgba *L, int n)  // colormap.c:79-138
{
    const float parm[4] = {(float) 0.04, (float) 0.9, (float) 0.9, (float) 0.8};
    static const double air[4] = {0.6, 0.6, 0.8, 0.1}, fat[4] = {0.8, 0.7, 0.0, 0.03125},
                        tissue[4] = {0.2, 0.0, 0.0, 0.1875}, bone[4] = {1.0, 1.0, 0.9, 0.75};
    for (int i = 0; i < n; i++) {
        const float x = i / (float) (n - 1) * 4096.0f;
        Rgba &e = L[i];
        if (0 <= x && x <= 484) {
            e.r = e.g = e.b = (float) 0.1;
            e.a = (float) (0.1 * parm[0]);
        } else if (484 < x && x <= 545) {
            med_blend(e, x, 484.0, 545.0, parm[0], parm[1], air, fat);
        } else if (545 < x && x <= 726) {
            e.r = (float) 0.8; e.g = (float) 0.7; e.b = 0.0f;
            e.a = (float) (0.03125 * parm[1]);
        } else if (726 < x && x <= 819) {
            med_blend(e, x, 726.0, 819.0, parm[1], parm[2], fat, tissue);
        } else if (819 < x && x <= 883) {
            e.r = (float) 0.2; e.g = 0.0f; e.b = 0.0f;
            e.a = (float) (0.1875 * parm[2]);
        } else if (883 < x && x <= 1535) {
            med_blend(e, x, 883.0, 1535.0, parm[2], parm[3], tissue, bone);
        } else if (1535 < x) {
            e.r = 1.0f; e.g = 1.0f; e.b = (float) 0.9;
            e.a = (float) (0.75 * parm[3]);
        }
    }
}

// seismiccolormap (colormap.c:139-169) with the two-segment lerp of
// mathutil.h:42-59: knots at 1, n/2 and n
void seismic(Rgba *L, int n)
{
    const float knot[3] = {1.0f, 0.5f * n, (float) n};
    const float ends[3][3] = {{1.0f, 1.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 1.0f, 1.0f}};
    for (int ch = 0; ch < 3; ch++) {
        const float *v = ends[ch];
        const float inc1 = (v[1] - v[0]) / (knot[1] - knot[0]);
        const float inc2 = (v[2] - v[1]) / (knot[2] - knot[1]);
        for (int i = 1; i <= n; i++) {
            float val;
            if (i >= knot[0] && i <= knot[1]) val = v[0] + i * inc1;
            else if (i >= knot[1] && i <= knot[2]) val = v[1] + (i - knot[1]) * inc2;
            else continue;
            float *dst = ch == 0 ? &L[i - 1].r : ch == 1 ? &L[i - 1].g : &L[i - 1].b;
            *dst = val;
        }
    }
    for (int i = 0; i < n; i++) L[i].a = 1.0f;
}

void jet(Rgba *L, int n)  // colormap.c:171-181
{
    for (int i = 0; i < n; i++) {
        const float i4 = (4.0f * i) / n;
        L[i].r = (float) fmin(fmax(fmin(i4 - 1.5, -i4 + 4.5), 0.0f), 1.0f);
        L[i].g = (float) fmin(fmax(fmin(i4 - 0.5, -i4 + 3.5), 0.0f), 1.0f);
        L[i].b = (float) fmin(fmax(fmin(i4 + 0.5, -i4 + 2.5), 0.0f), 1.0f);
        L[i].a = 1.0f;
    }
}

}  // namespace

void build_colormap(int type, float *rgba, int hsize, float histmin, float histmax)
{
    Rgba *L = reinterpret_cast<Rgba *>(rgba);
    memset(L, 0, sizeof(Rgba) * (size_t) hsize);
    switch (type) {
    case IVR_CM_BASE: base(L, hsize, histmin, histmax); break;
    case IVR_CM_RAINBOW: rainbow(L, hsize); break;
    case IVR_CM_MEDICAL: medical(L, hsize); break;
    case IVR_CM_SEISMIC: seismic(L, hsize); break;
    case IVR_CM_JET: jet(L, hsize); break;
    default: break;  // nomap
    }
}

}  // namespace ivr
