/*
 * ref_driver.c -- test harness that drives the REFERENCE iVR C code (O1).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
 * reference's own sources (ray.c, transferfuncs.c, colormap.c, mathutil.c,
 * utils.c, connection.c and main.c renamed to ivr_ref_main) into
 * oracle/_ref/libivr_ref.so by oracle/Makefile.  Nothing in the product
 * links or loads it; only tests/ and the fixture generator do.
 *
 * It reproduces, in one process, what the MPI build of iVR does for one
 * steered frame:
 *   init()                        main.c:282-351 (done piecewise below)
 *   per-frame view setup          main.c:226-233
 *   createlocalimage(rank)        main.c:937-1026, once per brick/rank
 *   sortboxlist + compositetiles  main.c:762, main.c:1203-1218
 * The MPI pieces are emulated:
 *   - bricks: initvolattrs(args, r) + readfromfile() per rank r
 *     (main.c:387, main.c:687 -> main.c:1220);
 *   - LUT: the global min/max/hsize merge of initvolluts' MPI branch
 *     (main.c:1113-1179) is computed from the whole volume with the
 *     reference's histogram() and colormap builders; maxlutindx = hsize-1
 *     as in that branch (main.c:1159);
 *   - compositing: whole frames, bricks in sortboxlist order, composited
 *     with the reference's compositetiles (far -> near).
 * colorbuf is padded past its end because createlocalimage can write one
 * row and one column past the viewport (main.c:959-962).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "ray.h"
#include "colormap.h"

/* globals owned by the reference's main.c */
extern color4f *colorbuf;
extern color4f *lut;
extern float *initbuffer;
extern int lutoffset;
extern int maxlutindx;
extern float pzero[6];
extern STATE mystate;
extern FRUSTUM viewvolume, frustum;
extern WINDOW viewport;

/* reference functions without a header declaration */
int endianness(void);
void initcamera(void);
void initvolattrs(CMDARGS, int);
int readvoldata(char *);
void initcolbufs(int);
void createlocalimage(int);
int compositetiles(float *, float *, int, int, int);
void readfromfile(char *, float *, int *, int *, int *);
float BYTESWAP_FP(float);

typedef struct {
    int width, height, depth;  /* global volume dims (x, y, z) */
    int dataendian;            /* argv[5]; 1 = little-endian file on x86/arm */
    int colormap;              /* argv[6]; -1 = inject lut below */
    int xfer;                  /* argv[7] */
    int procdims[3];           /* argv[8..10]: rows (y), cols (x), slabs (z) */
    int tilew, tileh;          /* argv[11..12] */
    int winwidth, winheight;   /* STATE.winwidth/winheight */
    float alpha;               /* STATE.alpha */
    float newconst[6];         /* STATE.newconst */
    float vv[4];               /* STATE.vv */
    float mvm[16];             /* STATE.mvm (GL column-major) */
    float pm[16];              /* STATE.pm  (GL column-major) */
    const float *inj_lut;      /* RGBA rows when colormap == -1 */
    int inj_n;
    int inj_offset;
} ref_frame;

/* Output: out_rgba = composited frame [vh][vw][4]; out_bricks (nullable) =
 * per-brick sub-images [K][vh][vw][4] in rank order; out_info (nullable) =
 * per rank: wincoord x,y,z,w,h,d, sorted position, istrt-ish unused.
 * Returns K on success, negative on failure. */
int ref_render(const char *volpath, const ref_frame *f, int nthreads,
               float *out_rgba, float *out_bricks, float *out_info,
               float *out_lut, int *out_lutinfo, int *out_vpdims)
{
    CMDARGS a;
    memset(&a, 0, sizeof(a));
    strncpy(a.filename, volpath, sizeof(a.filename) - 1);
    a.width = f->width; a.height = f->height; a.depth = f->depth;
    a.dataendian = f->dataendian;
    a.colormap = f->colormap;
    a.xfer = f->xfer;
    a.procdims[0] = f->procdims[0]; a.procdims[1] = f->procdims[1]; a.procdims[2] = f->procdims[2];
    a.tilewid = f->tilew; a.tilehgt = f->tileh;

    if (nthreads > 0) omp_set_num_threads(nthreads);

    int K = a.procdims[0] * a.procdims[1] * a.procdims[2];
    AABB *boxes = (AABB *) calloc((size_t) K, sizeof(AABB));
    float *images = NULL;
    int vw = 0, vh = 0;

    for (int r = 0; r < K; r++) {
        memset(&volume, 0, sizeof(volume));
        memset(&aabb, 0, sizeof(aabb));
        /* init(): window + camera (main.c:295-310) */
        viewport.tilewid = a.tilewid;
        viewport.tilehgt = a.tilehgt;
        viewport.tilex = WINDOWWIDTH / viewport.tilewid;
        viewport.tiley = WINDOWHEIGHT / viewport.tilehgt;
        viewport.w = viewport.tilex * viewport.tilewid;
        viewport.h = viewport.tiley * viewport.tilehgt;
        initcamera();
        setviewport(&viewport, 0, 0, viewport.w, viewport.h);
        initvolattrs(a, r);

        if (K == 1) {
            if (readvoldata(a.filename) < 0) return -1;
        } else {
            int gd[3] = {volume.globaldims.h, volume.globaldims.w, volume.globaldims.d};
            int ld[3] = {volume.localdims.h, volume.localdims.w, volume.localdims.d};
            int si[3] = {volume.startindex.y, volume.startindex.x, volume.startindex.z};
            long long n = (long long) ld[0] * ld[1] * ld[2];
            volume.data.f = (float *) malloc(sizeof(float) * n);
            readfromfile(a.filename, volume.data.f, gd, ld, si);
            if (volume.byteswap)
                for (long long i = 0; i < n; i++) volume.data.f[i] = BYTESWAP_FP(volume.data.f[i]);
        }

        if (r == 0) {
            initcolormap(a.colormap);
            if (a.colormap != -1) {
                /* global histogram / min / max over the whole volume, as the
                 * MPI merge in initvolluts yields (main.c:1113-1179) */
                long long n = (long long) a.width * a.height * a.depth;
                float *full = (float *) malloc(sizeof(float) * n);
                FILE *fp = fopen(a.filename, "rb");
                if (!fp) return -2;
                if (fread(full, sizeof(float), (size_t) n, fp) != (size_t) n) return -3;
                fclose(fp);
                if (volume.byteswap)
                    for (long long i = 0; i < n; i++) full[i] = BYTESWAP_FP(full[i]);
                int *hist = NULL;
                float mn, mx;
                histogram(&hist, full, &mn, &mx, a.width, a.height, a.depth);
                int hsize = (int) ((mx - mn) + 1);
                lut = (color4f *) calloc((size_t) hsize, sizeof(color4f));
                maxlutindx = hsize - 1;
                colormap(lut, hist, hsize, mn, mx);
                lutoffset = (int) (mn + 0.5);
                free(hist);
                free(full);
            } else {
                lut = (color4f *) malloc(sizeof(color4f) * (size_t) f->inj_n);
                memcpy(lut, f->inj_lut, sizeof(color4f) * (size_t) f->inj_n);
                maxlutindx = f->inj_n - 1;
                lutoffset = f->inj_offset;
            }
            if (out_lutinfo) { out_lutinfo[0] = maxlutindx + 1; out_lutinfo[1] = lutoffset; }
            if (out_lut && lut) memcpy(out_lut, lut, sizeof(color4f) * (size_t) (maxlutindx + 1));
        }
        inittransferfunc(a.xfer);
        initsamplefunc(LINEAR);

        /* one steered frame (main.c:212, main.c:226-233) */
        winwidth = f->winwidth; winheight = f->winheight;
        mystate.winwidth = f->winwidth; mystate.winheight = f->winheight;
        mystate.alpha = f->alpha;
        memcpy(mystate.newconst, f->newconst, sizeof(mystate.newconst));
        memcpy(mystate.vv, f->vv, sizeof(mystate.vv));
        memcpy(mystate.mvm, f->mvm, sizeof(mystate.mvm));
        memcpy(mystate.pm, f->pm, sizeof(mystate.pm));
        float planeconst[6] = {pzero[0], pzero[1], pzero[2], pzero[3], pzero[4], pzero[5]};
        setviewport(&viewport, 0, 0, winwidth, winheight);
        setplaneconst(planeconst, mystate.newconst);
        setmvm(mvm, mystate.mvm);
        setpm(pm, mystate.pm);
        setfrustum(&viewvolume, mystate.vv);
        updatevolbbox();
        initcolbufs(r);

        vw = (int) viewport.w; vh = (int) viewport.h;
        /* pad: rows istrt..h and columns up to w are written (main.c:959-962) */
        free(colorbuf);
        colorbuf = (color4f *) calloc((size_t) (vw * (vh + 2) + 2), sizeof(color4f));

        createlocalimage(r);

        if (!images) images = (float *) calloc((size_t) K * vw * vh * 4, sizeof(float));
        memcpy(images + (size_t) r * vw * vh * 4, colorbuf, sizeof(float) * 4 * (size_t) vw * vh);
        if (out_bricks) memcpy(out_bricks + (size_t) r * vw * vh * 4, colorbuf, sizeof(float) * 4 * (size_t) vw * vh);

        boxes[r].wincoord = aabb.wincoord;
        boxes[r].rank = r;
        if (out_info) {
            out_info[r * 8 + 0] = aabb.wincoord.x;
            out_info[r * 8 + 1] = aabb.wincoord.y;
            out_info[r * 8 + 2] = aabb.wincoord.z;
            out_info[r * 8 + 3] = aabb.wincoord.w;
            out_info[r * 8 + 4] = aabb.wincoord.h;
            out_info[r * 8 + 5] = aabb.wincoord.d;
        }
        free(volume.data.f);
        volume.data.f = NULL;
    }

    sortboxlist(0, K - 1, boxes);
    if (out_info)
        for (int s = 0; s < K; s++) out_info[boxes[s].rank * 8 + 6] = (float) s;

    /* rcolorbuf in near -> far order, composited far -> near onto a zeroed
     * tile buffer (main.c:904-907) */
    size_t px = (size_t) vw * vh * 4;
    float *rcolor = (float *) malloc(sizeof(float) * px * (size_t) K);
    for (int s = 0; s < K; s++)
        memcpy(rcolor + (size_t) s * px, images + (size_t) boxes[s].rank * px, sizeof(float) * px);
    memset(out_rgba, 0, sizeof(float) * px);
    compositetiles(out_rgba, rcolor, K, vw, vh);
    if (out_vpdims) { out_vpdims[0] = vw; out_vpdims[1] = vh; }

    free(rcolor);
    free(images);
    free(boxes);
    free(colorbuf); colorbuf = NULL;
    free(initbuffer); initbuffer = NULL;
    free(lut); lut = NULL;
    return K;
}

/* The reference's RGBA8 quantisation rule (main.c:1404), applied to a
 * float buffer, for the fixture generator. */
void ref_quantize(const float *in, unsigned char *out, long long n)
{
    for (long long i = 0; i < n; i++) out[i] = (unsigned char) (in[i] * 255.0 + 0.5f);
}

/* Exposes the reference's colormap builders for LUT parity tests. */
void ref_colormap(int type, float *out_rgba, int hsize, float histmin, float histmax)
{
    int *hist = (int *) calloc((size_t) hsize, sizeof(int));
    initcolormap(type);
    colormap((color4f *) out_rgba, hist, hsize, histmin, histmax);
    free(hist);
}
