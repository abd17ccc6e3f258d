/*
 * ivr_oracle.h -- O2: CPU restatement of the iVR ray-casting hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA path is
 * compared against (tests/, __graft_entry__.smoke(), bench.py's CPU
 * baseline).  The product never links, loads or calls it.
 *
 * Two presets:
 *   ORC_PRESET_REF     bit-faithful to the reference's C code (ray.c,
 *                      transferfuncs.c, main.c createlocalimage/compositetiles,
 *                      mathutil.c buildray/updatevolbbox, utils.c
 *                      getlocalbrick/sortboxlist), quirks included;
 *                      pinned bitwise against the reference built from source.
 *   ORC_PRESET_CONFIG  the benchmark semantics: true trilinear, one global
 *                      sample lattice per ray (step in voxels), no sample cap,
 *                      front-to-back compositing with early termination,
 *                      exact per-axis brick order.
 */
#ifndef IVR_ORACLE_H
#define IVR_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* The steering STATE record (connection.h:9-18), 184 bytes. */
typedef struct {
    int finish, winwidth, winheight;
    float alpha;
    float newconst[6];
    float vv[4];
    float mvm[16];
    float pm[16];
} orc_state;

enum { ORC_U8 = 0, ORC_U16 = 1, ORC_F32 = 2 };
enum { ORC_PRESET_REF = 0, ORC_PRESET_CONFIG = 1 };
/* ids 0-5 follow transferfuncs.h:8-13; 6 is the front-to-back LUT mode */
enum { ORC_TF_SEISMIC = 0, ORC_TF_MED = 1, ORC_TF_SEISMIC2 = 2, ORC_TF_CHEM = 3,
       ORC_TF_BLEND = 4, ORC_TF_RGBBLEND = 5, ORC_TF_F2B = 6 };
enum { ORC_ORDER_CENTER = 0, ORC_ORDER_AXIS = 1 };

#define ORC_MAX_BRICKS 64

typedef struct {
    const void *data;      /* global volume, x fastest: ((k*h)+i)*w + j */
    int dtype;             /* ORC_U8 / ORC_U16 / ORC_F32 */
    int gw, gh, gd;        /* global dims */
    int procdims[3];       /* rows (y), cols (x), slabs (z) -- argv[8..10] */
    int overlap;           /* halo on the high side of inner bricks (1) */
    orc_state state;
    int tilew, tileh;      /* viewport is rounded down to these */
    const float *lut;      /* RGBA rows */
    int lut_n;
    int lut_offset;
    float lut_scale;       /* CONFIG only: index = (int)(s*scale) - offset */
    int tf_mode;
    int preset;
    float step;            /* REF: ray-parameter step (0.001); CONFIG: voxels */
    int max_samples;       /* REF: 256; CONFIG: 0 = unbounded */
    float term_alpha;      /* CONFIG: stop at A >= term_alpha (> 1 = never) */
    int order;             /* ORC_ORDER_* */
    int row0, row1;        /* render rows [row0,row1); row1 <= 0 = all */
    int skip;              /* CONFIG: step over 16^3 macrocells whose samples
                              all have zero opacity (must not change output) */
} orc_scene;

typedef struct {
    long long samples_alg;   /* lattice points (no cap, no termination) */
    long long samples_exec;  /* samples actually taken */
    int vw, vh, nbricks;
    float wincoord[ORC_MAX_BRICKS][6];
    int order[ORC_MAX_BRICKS];     /* composite order, near -> far */
    int rect[ORC_MAX_BRICKS][4];   /* istrt, istop, jstrt, jstop */
} orc_stats;

/* Render one frame.  rgba32 = [vh][vw][4] (nullable), rgba8 = [vh][vw][4]
 * (nullable), bricks = [K][vh][vw][4] per-brick sub-images (nullable).
 * Returns the brick count, or a negative error. */
int orc_render(const orc_scene *sc, int nthreads, float *rgba32,
               unsigned char *rgba8, float *bricks, orc_stats *st);

/* Brick arrays of a scene's volume, extracted once (the reference reads
 * its brick at start-up, main.c:316); orc_render_prepared reuses them for
 * any view of the same volume and brick grid. */
typedef struct orc_prepared orc_prepared;
orc_prepared *orc_prepare(const orc_scene *sc);
void orc_prepared_free(orc_prepared *p);
int orc_render_prepared(const orc_scene *sc, const orc_prepared *p, int nthreads, float *rgba32,
                        unsigned char *rgba8, float *bricks, orc_stats *st);

/* Premultiplied over, far -> near, in the given near->far order
 * (compositetiles, main.c:1203-1218). */
void orc_composite(float *dst, const float *subimages, const int *order,
                   int num, int npix);

/* RGBA8 rule of writetomemory (main.c:1404), clamped to [0,1] first. */
void orc_quantize(const float *in, unsigned char *out, long long n);

/* LUT builders (colormap.c) and histogram (mathutil.c:444-470). */
void orc_colormap(int type, float *rgba, int hsize, float histmin, float histmax);
int orc_minmax(const void *data, int dtype, long long n, float *mn, float *mx);
void orc_histogram(const void *data, int dtype, long long n, float mn, int hsize, int *hist);

/* Macrocell min/max over cells of `cell` voxels plus the +1 boundary layer
 * (what a trilinear sample in the cell can read). */
/* per-voxel gradient (gx, gy, gz, |g|) of a [d][h][w] float volume */
void orc_gradient(const float *vol, int w, int h, int d, float *out);
void orc_macrocells(const float *vol, int w, int h, int d, int cell,
                    float *cmin, float *cmax);

#ifdef __cplusplus
}
#endif
#endif
