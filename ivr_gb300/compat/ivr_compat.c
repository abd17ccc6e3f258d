/*
 * ivr_compat.c -- the reference's hot-path function names over the GB300
 * library (declared in include/ivr_compat.h).
 *
 * The reference's frame path lives in process globals set by a fixed call
 * sequence (main.c:282-351 at start-up, main.c:226-248 per steered frame).
 * This file keeps the same globals and functions and maps each call onto
 * the handle API of libivr_gpu.so: one context, one volume with all its
 * bricks resident, one transfer function and one view, all held here.
 * Everything is the REF preset, so the frames are the reference's bit for
 * bit.  No CUDA header is needed: device buffers come from the library
 * (ivr_device_alloc) and move with ivr_copy.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ivr_compat.h"

/* ---- the reference's globals (main.c:63-105) --------------------------- */
ivr_state mystate;
ivr_window viewport;
ivr_matrix4f mvm, pm;
ivr_frustum viewvolume;
float pzero[6] = {1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.0f};
int winwidth = 1280, winheight = 720;  /* WINDOWWIDTH, WINDOWHEIGHT (types.h:23-24) */
int lutoffset, maxlutindx;
ivr_color4f *lut = NULL;
ivr_color4f *colorbuf = NULL;
unsigned char *tiffimage = NULL;

/* ---- what this layer holds ---------------------------------------------- */
static ivr_ctx *g_ctx;
static ivr_volume *g_vol;
static ivr_tf *g_tf;
static ivr_view *g_view;
static int g_dims[3];             /* w, h, d */
static int g_procdims[3] = {1, 1, 1};
static int g_endian = 1;          /* argv[5]: 1 = the file is little endian */
static int g_colormap = -1, g_xfer = 0;
static float g_plane[6], g_newconst[6];
static int g_view_ok;
static ivr_color4f *g_lut_owned;  /* the LUT initvolluts allocated */
static ivr_color4f *g_lut_sent;   /* the LUT the library holds, to notice direct edits */
static int g_lut_sent_n = -1, g_lut_sent_off, g_lut_sent_mode = -1;
static float *g_dev32;            /* one RGBA32 frame on the device */
static unsigned char *g_dev8;     /* one RGBA8 frame on the device */
static size_t g_dev32_bytes, g_dev8_bytes;
static char g_err[512];

static int fail(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return -1;
}

/* a library status: 0, or -1 with its message */
static int lib(int rc, const char *what)
{
    if (rc == IVR_OK) return 0;
    return fail("%s: %s", what, g_ctx ? ivr_last_error(g_ctx) : "no context");
}

const char *ivr_compat_last_error(void) { return g_err; }

static int ensure_ctx(void)
{
    if (g_ctx) return 0;
    const char *dev = getenv("IVR_DEVICE");
    if (ivr_create(dev ? atoi(dev) : 0, 0, &g_ctx) != IVR_OK) {
        g_ctx = NULL;
        return fail("ivr_create failed (no usable GPU?)");
    }
    if (lib(ivr_tf_create(g_ctx, &g_tf), "ivr_tf_create")) return -1;
    return lib(ivr_view_create(g_ctx, &g_view), "ivr_view_create");
}

/* device buffers grow to the largest frame asked for */
static int ensure_dev(size_t bytes32, size_t bytes8)
{
    if (bytes32 > g_dev32_bytes) {
        if (g_dev32) ivr_device_free(g_ctx, g_dev32, g_dev32_bytes);
        g_dev32 = NULL;
        g_dev32_bytes = 0;
        if (lib(ivr_device_alloc(g_ctx, bytes32, (void **) &g_dev32), "frame buffer")) return -1;
        g_dev32_bytes = bytes32;
    }
    if (bytes8 > g_dev8_bytes) {
        if (g_dev8) ivr_device_free(g_ctx, g_dev8, g_dev8_bytes);
        g_dev8 = NULL;
        g_dev8_bytes = 0;
        if (lib(ivr_device_alloc(g_ctx, bytes8, (void **) &g_dev8), "frame buffer")) return -1;
        g_dev8_bytes = bytes8;
    }
    return 0;
}

/* ---- start-up ------------------------------------------------------------ */

/* initvolattrs (main.c:387-426): the volume's dimensions, file byte order
 * and brick grid, then initvolbbox. */
void initvolattrs(ivr_cmdargs args, int rank)
{
    g_dims[0] = args.width;
    g_dims[1] = args.height;
    g_dims[2] = args.depth;
    g_endian = args.dataendian;
    for (int i = 0; i < 3; i++) g_procdims[i] = args.procdims[i] > 0 ? args.procdims[i] : 1;
    initvolbbox(rank);
}

/* initvolbbox (main.c:505-624): the box [-s, s] with s = dims / maxdim, its
 * plane constants in pzero, and setplaneconst(pzero, pzero).  One process
 * holds every brick, so the box is the whole volume's for every rank. */
int initvolbbox(int rank)
{
    (void) rank;
    int m = g_dims[0];
    if (g_dims[1] > m) m = g_dims[1];
    if (g_dims[2] > m) m = g_dims[2];
    if (m < 1) return fail("volume dimensions %d x %d x %d", g_dims[0], g_dims[1], g_dims[2]);
    const float inv = 1.0f / (float) m;
    const float s[3] = {(float) g_dims[0] * inv, (float) g_dims[1] * inv, (float) g_dims[2] * inv};
    for (int a = 0; a < 3; a++) pzero[2 * a] = pzero[2 * a + 1] = s[a];
    setplaneconst(pzero, pzero);
    return 0;
}

/* readvoldata (main.c:629-706): the raw float32 volume file, byte-swapped
 * when its byte order differs from the host's, split into the brick grid
 * with a one-voxel overlap (getlocalbrick, utils.c:332-388). */
int readvoldata(char *filename)
{
    if (ensure_ctx()) return -1;
    if (g_vol) {
        ivr_volume_free(g_vol);
        g_vol = NULL;
    }
    g_view_ok = 0;
    if (lib(ivr_volume_load_file(g_ctx, filename, g_dims[0], g_dims[1], g_dims[2], IVR_F32, g_endian, &g_vol),
            "readvoldata"))
        return -1;
    if (g_procdims[0] * g_procdims[1] * g_procdims[2] > 1 &&
        lib(ivr_bricks_setup(g_vol, g_procdims[0], g_procdims[1], g_procdims[2], 1), "brick set-up"))
        return -1;
    return 0;
}

/* initcolormap (colormap.c:183-206): which LUT builder initvolluts uses;
 * unknown ids are nomap. */
void initcolormap(int type) { g_colormap = type >= 0 && type <= 4 ? type : -1; }

/* inittransferfunc (transferfuncs.c:201-226): ids 0-5, unknown ids are
 * SEISMIC (the reference's default case). */
void inittransferfunc(int xfer) { g_xfer = xfer >= 0 && xfer <= 5 ? xfer : 0; }

/* initsamplefunc (ray.c:485-501): the reference hard-wires LINEAR
 * (main.c:345), the only sampler here. */
void initsamplefunc(int type) { (void) type; }

/* initvolluts (main.c:1075-1200): histogram of the whole volume, colormap
 * over its range, lutoffset = (int)(min + 0.5), maxlutindx = hsize - 1;
 * the LUT is also copied to the `lut` global. */
int initvolluts(void)
{
    if (!g_vol) return fail("initvolluts before readvoldata");
    if (lib(ivr_tf_set_colormap(g_tf, g_vol, g_colormap, g_xfer), "initvolluts")) return -1;
    int n = 0, off = 0;
    if (lib(ivr_tf_get_lut(g_tf, NULL, 0, &n, &off), "initvolluts")) return -1;
    ivr_color4f *t = (ivr_color4f *) malloc(sizeof(ivr_color4f) * (size_t) (n > 0 ? n : 1));
    if (!t) return fail("initvolluts: out of host memory");
    if (lib(ivr_tf_get_lut(g_tf, (float *) t, n, NULL, NULL), "initvolluts")) {
        free(t);
        return -1;
    }
    if (g_lut_owned) free(g_lut_owned);
    g_lut_owned = lut = t;
    lutoffset = off;
    maxlutindx = n - 1;
    free(g_lut_sent);
    g_lut_sent = (ivr_color4f *) malloc(sizeof(ivr_color4f) * (size_t) (n > 0 ? n : 1));
    if (g_lut_sent) memcpy(g_lut_sent, t, sizeof(ivr_color4f) * (size_t) n);
    g_lut_sent_n = g_lut_sent ? n : -1;
    g_lut_sent_off = off;
    g_lut_sent_mode = g_xfer;
    return 0;
}

/* initcolbufs (main.c:357-384): colorbuf (and tiffimage) for the viewport,
 * zeroed. */
void initcolbufs(int rank)
{
    (void) rank;
    size_t vpsize = (size_t) viewport.w * (size_t) viewport.h;
    free(colorbuf);
    colorbuf = (ivr_color4f *) calloc(vpsize ? vpsize : 1, sizeof(ivr_color4f));
    free(tiffimage);
    tiffimage = (unsigned char *) calloc(vpsize ? vpsize * 4 : 1, 1);
}

/* init (main.c:282-351): the start-up sequence of the reference's server. */
int init(ivr_cmdargs args, int rank)
{
    viewport.tilewid = args.tilewid > 0 ? args.tilewid : 1;
    viewport.tilehgt = args.tilehgt > 0 ? args.tilehgt : 1;
    setviewport(&viewport, 0, 0, winwidth, winheight);
    initvolattrs(args, rank);
    if (readvoldata(args.filename) < 0) return -1;
    initcolormap(args.colormap);
    inittransferfunc(args.xfer);
    if (args.colormap != -1 && initvolluts() < 0) return -1;
    initcolbufs(rank);
    initsamplefunc(1);
    return 0;
}

/* ---- per frame ----------------------------------------------------------- */

/* setplaneconst (ray.c:44-51): the clip planes are min(planeconst, newconst);
 * kept here and applied by updatevolbbox. */
void setplaneconst(float *planeconst, float *newconst)
{
    for (int i = 0; i < 6; i++) {
        g_plane[i] = planeconst[i];
        g_newconst[i] = newconst[i];
    }
}

/* updatevolbbox (mathutil.c:948-1018): the frame's geometry from the
 * globals the steering loop set (viewport, mvm, pm, viewvolume, mystate) and
 * the clip planes; the library derives the rays, every brick's window
 * rectangle and the composite order from it. */
void updatevolbbox(void)
{
    g_view_ok = 0;
    if (!g_vol) {
        fail("updatevolbbox before readvoldata");
        return;
    }
    ivr_state st;
    memset(&st, 0, sizeof st);
    st.winwidth = (int) viewport.w;
    st.winheight = (int) viewport.h;
    st.alpha = mystate.alpha;
    /* a newconst at or beyond the box leaves the box's own plane: the
     * library takes min(box, newconst) per brick, as each rank's dconst is */
    for (int i = 0; i < 6; i++) st.newconst[i] = g_newconst[i] < g_plane[i] ? g_newconst[i] : 1.0e30f;
    st.vv[0] = viewvolume.left;
    st.vv[1] = viewvolume.right;
    st.vv[2] = viewvolume.bottom;
    st.vv[3] = viewvolume.top;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            st.mvm[4 * c + r] = mvm[r][c];
            st.pm[4 * c + r] = pm[r][c];
        }
    ivr_render_params p;
    ivr_params_ref(&p);
    p.tilew = viewport.tilewid > 0 ? viewport.tilewid : 1;
    p.tileh = viewport.tilehgt > 0 ? viewport.tilehgt : 1;
    if (lib(ivr_set_view(g_view, g_vol, &st, &p), "updatevolbbox")) return;
    g_view_ok = 1;
}

/* the `lut` global into the library when it differs from what it holds (a
 * caller may set lut/lutoffset/maxlutindx itself, main.c:64-65,80) */
static int sync_lut(void)
{
    if (!lut) return fail("no LUT: initvolluts, or set lut, lutoffset and maxlutindx");
    const int n = maxlutindx + 1;
    if (n < 1) return fail("maxlutindx %d", maxlutindx);
    if (n == g_lut_sent_n && lutoffset == g_lut_sent_off && g_xfer == g_lut_sent_mode &&
        memcmp(lut, g_lut_sent, sizeof(ivr_color4f) * (size_t) n) == 0)
        return 0;
    if (lib(ivr_tf_set_lut(g_tf, (const float *) lut, n, lutoffset, 1.0f, g_xfer), "LUT")) return -1;
    free(g_lut_sent);
    g_lut_sent = (ivr_color4f *) malloc(sizeof(ivr_color4f) * (size_t) n);
    if (g_lut_sent) memcpy(g_lut_sent, lut, sizeof(ivr_color4f) * (size_t) n);
    g_lut_sent_n = g_lut_sent ? n : -1;
    g_lut_sent_off = lutoffset;
    g_lut_sent_mode = g_xfer;
    return 0;
}

static int frame_ready(size_t *npix)
{
    if (!g_view_ok) return fail("no frame: updatevolbbox did not succeed");
    if (sync_lut()) return -1;
    ivr_frame_info fi;
    if (lib(ivr_view_info(g_view, &fi), "view info")) return -1;
    if (fi.vw != (int) viewport.w || fi.vh != (int) viewport.h)
        return fail("viewport %gx%g differs from the frame's %dx%d", viewport.w, viewport.h, fi.vw, fi.vh);
    if (!colorbuf || !tiffimage) return fail("no colour buffers: initcolbufs");
    *npix = (size_t) fi.vw * (size_t) fi.vh;
    return ensure_dev(*npix * 16, *npix * 4);
}

/* createlocalimage (main.c:937-1026): brick `rank`'s sub-image over the
 * viewport into colorbuf, zero outside its window rectangle. */
void createlocalimage(int rank)
{
    size_t npix;
    if (frame_ready(&npix)) return;
    if (lib(ivr_render_brick(g_view, g_tf, rank, g_dev32, NULL), "createlocalimage")) return;
    if (lib(ivr_copy(g_ctx, colorbuf, g_dev32, npix * 16, NULL), "createlocalimage")) return;
    lib(ivr_stream_wait(g_ctx, NULL), "createlocalimage");
}

/* compositelocalimage (main.c:708-934) with the gather of writetomemory
 * (main.c:1333-1417): every brick composited far to near in sortboxlist
 * order; the whole frame lands in colorbuf, and its RGBA8 (main.c:1404) in
 * the library's frame buffer for writetomemory. */
int compositelocalimage(void)
{
    size_t npix;
    if (frame_ready(&npix)) return -1;
    if (lib(ivr_render(g_view, g_tf, g_dev32, g_dev8, NULL), "compositelocalimage")) return -1;
    if (lib(ivr_copy(g_ctx, colorbuf, g_dev32, npix * 16, NULL), "compositelocalimage")) return -1;
    return lib(ivr_stream_wait(g_ctx, NULL), "compositelocalimage");
}

/* writetomemory (main.c:1333-1417): the composited frame as RGBA8 in
 * tiffimage, (uint8)(v * 255 + 0.5) per channel. */
int writetomemory(int rank, int a)
{
    (void) rank;
    (void) a;
    size_t npix;
    if (frame_ready(&npix)) return -1;
    if (lib(ivr_copy(g_ctx, g_dev32, colorbuf, npix * 16, NULL), "writetomemory")) return -1;
    if (lib(ivr_quantize(g_ctx, g_dev32, g_dev8, (long long) npix * 4, NULL), "writetomemory")) return -1;
    if (lib(ivr_copy(g_ctx, tiffimage, g_dev8, npix * 4, NULL), "writetomemory")) return -1;
    return lib(ivr_stream_wait(g_ctx, NULL), "writetomemory");
}

/* compositetiles (main.c:1203-1218): num w*h sub-images of rcolorbuf
 * composited onto tilebuf, d = s + (1 - s.a) * d, in host memory. */
int compositetiles(float *tilebuf, float *rcolorbuf, int num, int w, int h)
{
    if (num <= 0) return 0;
    if (!tilebuf || !rcolorbuf || w < 1 || h < 1) return fail("compositetiles arguments");
    if (ensure_ctx()) return -1;
    const size_t one = (size_t) w * (size_t) h * 16;
    float *dt = NULL, *ds = NULL;
    int rc = lib(ivr_device_alloc(g_ctx, one, (void **) &dt), "compositetiles");
    if (!rc) rc = lib(ivr_device_alloc(g_ctx, one * (size_t) num, (void **) &ds), "compositetiles");
    if (!rc) rc = lib(ivr_copy(g_ctx, dt, tilebuf, one, NULL), "compositetiles");
    if (!rc) rc = lib(ivr_copy(g_ctx, ds, rcolorbuf, one * (size_t) num, NULL), "compositetiles");
    if (!rc) rc = lib(ivr_composite(g_ctx, dt, ds, num, w, h, NULL), "compositetiles");
    if (!rc) rc = lib(ivr_copy(g_ctx, tilebuf, dt, one, NULL), "compositetiles");
    if (!rc) rc = lib(ivr_stream_wait(g_ctx, NULL), "compositetiles");
    if (ds) ivr_device_free(g_ctx, ds, one * (size_t) num);
    if (dt) ivr_device_free(g_ctx, dt, one);
    return rc;
}

/* freeall (main.c:267-278) */
void freeall(void)
{
    if (g_dev32) ivr_device_free(g_ctx, g_dev32, g_dev32_bytes);
    if (g_dev8) ivr_device_free(g_ctx, g_dev8, g_dev8_bytes);
    g_dev32 = NULL;
    g_dev8 = NULL;
    g_dev32_bytes = g_dev8_bytes = 0;
    if (g_view) ivr_view_free(g_view);
    if (g_tf) ivr_tf_free(g_tf);
    if (g_vol) ivr_volume_free(g_vol);
    if (g_ctx) ivr_destroy(g_ctx);
    g_view = NULL;
    g_tf = NULL;
    g_vol = NULL;
    g_ctx = NULL;
    g_view_ok = 0;
    if (lut == g_lut_owned) lut = NULL;
    free(g_lut_owned);
    g_lut_owned = NULL;
    free(g_lut_sent);
    g_lut_sent = NULL;
    g_lut_sent_n = -1;
    free(colorbuf);
    colorbuf = NULL;
    free(tiffimage);
    tiffimage = NULL;
}
