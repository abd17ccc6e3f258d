/*
 * ivr_compat.h -- the reference's own names for the hot path, over the GB300
 * library (libivr_compat.so, which links libivr_gpu.so).
 *
 * The reference's frame path is a set of C functions that talk through
 * process globals (main.c:63-105, mathutil.h:17-30).  This layer exports the
 * same functions, with the same signatures and record layouts, and the same
 * globals, so that the reference's steered frame loop (main.c:226-248)
 *
 *     float planeconst[6] = {pzero[0], ..., pzero[5]};
 *     setviewport(&viewport, 0, 0, winwidth, winheight);
 *     setplaneconst(planeconst, mystate.newconst);
 *     setmvm(mvm, mystate.mvm);
 *     setpm(pm, mystate.pm);
 *     setfrustum(&viewvolume, mystate.vv);
 *     updatevolbbox();
 *     initcolbufs(rank);
 *     createlocalimage(rank);
 *     compositelocalimage();
 *
 * runs on one GPU unchanged.  What replaces what:
 *
 *   ray.c, transferfuncs.c, colormap.c        this library (the GPU march)
 *   main.c: init, initvolattrs, initvolbbox,   this library; link main.c
 *     readvoldata, initvolluts, initcolbufs,     without these definitions
 *     createlocalimage, compositelocalimage,     (they are the hot path it
 *     compositetiles, writetomemory, freeall     replaces)
 *   mathutil.c: updatevolbbox                  this library
 *   mathutil.h: setviewport, setmvm, setpm,    unchanged: the reference's static
 *     setfrustum (static inline)                 inlines, or the ones below
 *
 * One process holds every brick (no MPI): createlocalimage(rank) renders
 * brick `rank`'s sub-image into colorbuf, as that rank would;
 * compositelocalimage() leaves the whole composited frame in colorbuf (what
 * the reference's tile exchange and gather assemble, main.c:708-934,
 * 1333-1417); writetomemory() quantises it into tiffimage (main.c:1404).
 * Sampling is the reference's own (the REF preset: step 0.001, 256-sample
 * cap, getlinearsample, centre-depth brick order), bit for bit.
 *
 * Globals: this library defines the ones below.  A program that defines
 * them itself (main.c does) keeps its own definitions -- they have the same
 * layout -- and this library reads and writes those.  A LUT set directly in
 * `lut`, `lutoffset` and `maxlutindx` (colormap -1, no initvolluts) is used
 * by the next render.  Failures print nothing and exit nothing: the calls
 * that return int return -1, and ivr_compat_last_error() has the message.
 */
#ifndef IVR_COMPAT_H
#define IVR_COMPAT_H

#include "ivr_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Records with the reference's layouts (types.h, connection.h). */
typedef struct { float r, g, b, a; } ivr_color4f;           /* color4f, types.h:115-117 */
typedef struct {                                            /* CMDARGS, types.h:128-141 */
    char filename[80];
    int width, height, depth;
    int xfer, colormap, dataendian;
    int procdims[3];                                        /* rows, columns, slabs */
    int tilewid, tilehgt;
    float angle;
    float axis[3];
} ivr_cmdargs;
typedef struct {                                            /* WINDOW, types.h:204-211 */
    int tilex, tiley;
    int tilewid, tilehgt;
    float x, y, w, h;
} ivr_window;
typedef struct {                                            /* FRUSTUM, types.h:195-202 */
    float left, right, top, bottom, near_, far_;
} ivr_frustum;
typedef float ivr_matrix4f[4][4];                           /* matrix4f, types.h:110 */

/* Globals (main.c:63-105). */
extern ivr_state mystate;          /* STATE (connection.h:9-18) */
extern ivr_window viewport;
extern ivr_matrix4f mvm, pm;
extern ivr_frustum viewvolume;
extern float pzero[6];             /* the volume box's plane constants (initvolbbox) */
extern int winwidth, winheight;
extern int lutoffset, maxlutindx;
extern ivr_color4f *lut;           /* maxlutindx + 1 entries */
extern ivr_color4f *colorbuf;      /* viewport.w * viewport.h, rows bottom-up */
extern unsigned char *tiffimage;   /* viewport.w * viewport.h * 4 (RGBA8) */

/* main.c */
int init(ivr_cmdargs args, int rank);                       /* main.c:282 */
void initvolattrs(ivr_cmdargs args, int rank);              /* main.c:387 */
int initvolbbox(int rank);                                  /* main.c:505 */
int readvoldata(char *filename);                            /* main.c:629 */
int initvolluts(void);                                      /* main.c:1075 */
void initcolbufs(int rank);                                 /* main.c:357 */
void createlocalimage(int rank);                            /* main.c:937 */
int compositelocalimage(void);                              /* main.c:708 */
int compositetiles(float *tilebuf, float *rcolorbuf, int num, int w, int h); /* main.c:1203 */
int writetomemory(int rank, int a);                         /* main.c:1333 */
void freeall(void);                                         /* main.c:267 */
/* ray.c, transferfuncs.c, colormap.c, mathutil.c */
void setplaneconst(float *planeconst, float *newconst);     /* ray.c:44 */
void initsamplefunc(int type);                              /* ray.c:485 (LINEAR only) */
void inittransferfunc(int xfer);                            /* transferfuncs.c:201 */
void initcolormap(int type);                                /* colormap.c:183 */
void updatevolbbox(void);                                   /* mathutil.c:948 */

/* No counterpart in the reference: the message of the last failure. */
const char *ivr_compat_last_error(void);

/* The static inline setters of mathutil.h:147-233, for callers that do not
 * include the reference's mathutil.h. */
#ifndef IBM_Ray_Caster_mathutil_h
static inline void setviewport(ivr_window *v, int x, int y, int w, int h)
{
    v->tilex = w / v->tilewid;
    v->tiley = h / v->tilehgt;
    v->w = (float) (v->tilex * v->tilewid);
    v->h = (float) (v->tiley * v->tilehgt);
    v->x = (float) x;
    v->y = (float) y;
}
static inline void setfrustum(ivr_frustum *f, float *vv)
{
    f->left = vv[0];
    f->right = vv[1];
    f->bottom = vv[2];
    f->top = vv[3];
}
/* GL column-major in, row-major [r][c] out */
static inline void setmvm(ivr_matrix4f m, float cm[16])
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) m[r][c] = cm[4 * c + r];
}
static inline void setpm(ivr_matrix4f m, float cm[16])
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) m[r][c] = cm[4 * c + r];
}
#endif

#ifdef __cplusplus
}
#endif
#endif
