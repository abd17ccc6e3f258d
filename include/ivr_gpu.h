/*
 * ivr_gpu.h -- C ABI of the GB300 (sm_103a) iVR ray-casting hot path.
 *
 * Drop-in for the reference's per-frame path.  The reference keeps all state
 * in process globals (main.c:63-105) and selects variants through function
 * pointers (ray.h:25, transferfuncs.h:22, colormap.h:22); here the same steps
 * are explicit calls on opaque handles:
 *
 *   reference                                   this ABI
 *   -----------------------------------------   ------------------------------
 *   readvoldata / readfromfile (main.c:629,     ivr_volume_load, ivr_volume_load_file
 *     main.c:1220), byteswap (main.c:695-703)
 *   initvolattrs / initvolbbox / getlocalbrick  ivr_bricks_setup
 *     (main.c:387, main.c:505, utils.c:332)
 *   setviewport / setplaneconst / setmvm /      ivr_set_view (takes the 184-byte
 *     setpm / setfrustum / updatevolbbox          STATE of connection.h:9-18)
 *     (mathutil.h:147-233, ray.c:44,
 *      mathutil.c:948)
 *   initcolormap / initvolluts /                ivr_tf_set_colormap, ivr_tf_set_lut
 *     inittransferfunc (colormap.c:183,
 *     main.c:1075, transferfuncs.c:201)
 *   createlocalimage (main.c:937)               ivr_render_brick (one brick), and
 *     + compositelocalimage (main.c:708)        ivr_render / ivr_render_tile (all
 *     + compositetiles (main.c:1203)              bricks, composited on device)
 *   compositetiles (main.c:1203)                ivr_composite
 *   writetomemory RGBA8 rule (main.c:1404)      ivr_quantize (and fused in ivr_render)
 *
 * Conventions.  Every call returns an int status: IVR_OK (0) or a negative
 * IVR_ERR_*; nothing calls exit() or assert().  ivr_last_error() gives the
 * message of the last failure on a context.  Buffers named *_dev are device
 * pointers; device work is queued on the caller's stream (a cudaStream_t
 * passed as void*, NULL = the legacy default stream).  Handles are not
 * thread-safe: use one context per host thread, or serialise calls.  A view
 * owns the work counter of its launches: launches of one view must be
 * ordered (one stream); use one view per stream for concurrent frames.
 * ivr_create, ivr_destroy, ivr_device_alloc, ivr_host_alloc, the volume
 * loads, ivr_volume_gradient and ivr_volume_set_macrocell make the
 * context's device current (cudaSetDevice) and leave it current; the other
 * calls work on the current device, which must be the context's.
 * Images are [h][w] rows of RGBA, row 0 at the bottom (GL raster order).
 */
#ifndef IVR_GPU_H
#define IVR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IVR_OK 0
#define IVR_ERR_INVALID (-1)     /* bad argument or handle */
#define IVR_ERR_CUDA (-2)        /* a CUDA call failed */
#define IVR_ERR_NOMEM (-3)       /* allocation refused by the HBM budget or by CUDA */
#define IVR_ERR_IO (-4)          /* volume file missing or short */
#define IVR_ERR_UNSUPPORTED (-5) /* a valid request the library does not serve */
#define IVR_ERR_TIMEOUT (-6)     /* a bounded device wait gave up */

typedef struct ivr_ctx ivr_ctx;
typedef struct ivr_volume ivr_volume;
typedef struct ivr_tf ivr_tf;
typedef struct ivr_view ivr_view;

/* STATE (connection.h:9-18): the steering message, GL column-major
 * matrices, 184 bytes. */
typedef struct ivr_state {
    int finish, winwidth, winheight;
    float alpha;        /* opacity scale (mystate.alpha) */
    float newconst[6];  /* clip plane constants; min()'d with the box (ray.c:44) */
    float vv[4];        /* view-plane extents l, r, b, t (getfrustum) */
    float mvm[16];
    float pm[16];
} ivr_state;

typedef enum { IVR_U8 = 0, IVR_U16 = 1, IVR_F32 = 2 } ivr_dtype;

/* Transfer functions: ids 0-5 are the reference's (transferfuncs.h:8-13);
 * IVR_TF_F2B is front-to-back premultiplied compositing with early
 * termination (the CONFIG preset). */
typedef enum {
    IVR_TF_SEISMIC = 0, IVR_TF_MED = 1, IVR_TF_SEISMIC2 = 2, IVR_TF_CHEM = 3,
    IVR_TF_BLEND = 4, IVR_TF_RGBBLEND = 5, IVR_TF_F2B = 6
} ivr_tf_mode;

/* Colormap ids (colormap.h:15-20). */
typedef enum { IVR_CM_BASE = 0, IVR_CM_RAINBOW = 1, IVR_CM_MEDICAL = 2, IVR_CM_SEISMIC = 3,
               IVR_CM_JET = 4, IVR_CM_NOMAP = -1 } ivr_colormap;

typedef enum { IVR_PRESET_REF = 0, IVR_PRESET_CONFIG = 1 } ivr_preset;
typedef enum { IVR_ORDER_CENTER = 0, IVR_ORDER_AXIS = 1 } ivr_order;
/* IVR_SKIP_GRID: the exact macrocell grid (never changes the image).
 * IVR_SKIP_LEARNED: the grid the volume's learned predictor gives
 * (ivr_volume_set_mlp), every frame judged against the exact grid. */
typedef enum { IVR_SKIP_NONE = 0, IVR_SKIP_GRID = 1, IVR_SKIP_LEARNED = 2 } ivr_skip;
/* The order in which a CONFIG launch hands its 8x4 pixel tiles to warps.
 * IVR_TILES_COST (with a skipping grid): costliest first, by an estimate
 * from a walk of each tile's corner rays over the macrocell grid, so that the
 * launch does not end on a long tile drawn late.  The order never changes
 * a pixel. */
typedef enum { IVR_TILES_RASTER = 0, IVR_TILES_COST = 1 } ivr_tile_order;

/* How a frame is sampled.
 * REF: the reference's sampling exactly (ray.c): ray-parameter step 0.001,
 *   256-sample cap, its trilinear formula, per-brick lattices, centre-depth
 *   brick order (sortboxlist), transfer function ids 0-5.
 * CONFIG: true trilinear, one sample lattice per ray with `step` in voxels,
 *   no cap, front-to-back compositing stopping at A >= term_alpha, exact
 *   per-axis brick order. */
typedef struct ivr_render_params {
    int preset;        /* ivr_preset */
    float step;        /* REF: ray-parameter step; CONFIG: voxels */
    int max_samples;   /* per ray and brick; 0 = unbounded */
    float term_alpha;  /* early termination threshold (> 1 disables) */
    int order;         /* ivr_order */
    int skip;          /* ivr_skip */
    int tilew, tileh;  /* viewport rounded down to multiples (argv[11..12]) */
    int judge_stride;  /* IVR_SKIP_LEARNED: judge 1 in judge_stride 8x4 tiles, rotating */
    int judge_tol;     /* IVR_SKIP_LEARNED: largest 8-bit channel difference accepted */
    int tile_order;    /* ivr_tile_order (CONFIG) */
} ivr_render_params;

/* Per-frame geometry ivr_set_view computed, for callers that composite or
 * tile themselves (the fields of compositelocalimage's bookkeeping). */
#define IVR_MAX_BRICKS 64
typedef struct ivr_frame_info {
    int vw, vh;                        /* viewport after tile rounding */
    int nbricks;
    int order[IVR_MAX_BRICKS];         /* composite order, near -> far */
    float wincoord[IVR_MAX_BRICKS][6]; /* x, y, z, w, h, d (updatevolbbox) */
    int rect[IVR_MAX_BRICKS][4];       /* istrt, istop, jstrt, jstop */
} ivr_frame_info;

/* --- context ----------------------------------------------------------- */
void ivr_params_ref(ivr_render_params *p);     /* REF defaults */
void ivr_params_config(ivr_render_params *p);  /* CONFIG defaults */
int ivr_create(int device, size_t hbm_budget_bytes, ivr_ctx **out); /* budget 0 = no limit */
int ivr_destroy(ivr_ctx *ctx);
const char *ivr_last_error(const ivr_ctx *ctx);
int ivr_mem_used(const ivr_ctx *ctx, size_t *bytes);

/* Device memory counted against the context's HBM budget (for callers'
 * output buffers); free with the same size. */
int ivr_device_alloc(ivr_ctx *ctx, size_t bytes, void **ptr);
int ivr_device_free(ivr_ctx *ctx, void *ptr, size_t bytes);
/* Page-locked host memory (not counted against the budget), for frame
 * buffers the device copies into directly: ivr_server requests whose
 * rgba8_host lies in it skip the server's staging copy. */
int ivr_host_alloc(ivr_ctx *ctx, size_t bytes, void **ptr);
int ivr_host_free(ivr_ctx *ctx, void *ptr);  /* ctx may be NULL (no message then) */

/* --- volume load / brick setup (readvoldata, readfromfile, initvolbbox) -- */
/* Copies a host volume (x fastest, [d][h][w]) to the device.  byteswap != 0
 * reverses the bytes of every element (main.c:695-703 for f32). */
int ivr_volume_load(ivr_ctx *ctx, const void *host, int w, int h, int d, int dtype,
                    int byteswap, ivr_volume **out);
/* Reads a raw volume file.  file_little_endian follows argv[5] of the
 * reference: the data are byte-swapped when it differs from the host. */
int ivr_volume_load_file(ivr_ctx *ctx, const char *path, int w, int h, int d, int dtype,
                         int file_little_endian, ivr_volume **out);
int ivr_volume_free(ivr_volume *vol);
/* Splits the volume into py x px x pz bricks (rows, columns, slabs as
 * argv[8..10]) with `overlap` halo voxels on the high side of inner bricks
 * (getlocalbrick).  Each brick becomes its own device array.  The default
 * after load is one brick. */
int ivr_bricks_setup(ivr_volume *vol, int py, int px, int pz, int overlap);
/* Per-voxel gradient, as gradient3d (mathutil.c:242-325, built under
 * -DGRAD at main.c:1181-1196) intends it: grad4_dev receives w*h*d float4
 * (gx, gy, gz, |g|) in the volume's [d][h][w] order; per axis a central
 * difference halved inside and (V(1)-V(0))/2, (V(n-1)-V(n-2))/2 on the
 * faces.  The reference's own code writes every voxel to offset i*j*k,
 * takes its last z face from the two slabs before it and leaves edges and
 * corners unwritten; those are fixed here.  Queued on `stream`. */
int ivr_volume_gradient(ivr_volume *vol, float *grad4_dev, void *stream);
/* Corner-packed brick copies (no counterpart in the reference; on by
 * default).  Each brick gets a second copy in which element (j, i, k) holds
 * the four voxels (j, i), (j+1, i), (j, i+1), (j+1, i+1) of slab k (f32:
 * the second of each pair as its difference from the first), so a
 * trilinear sample of the CONFIG march is two vector loads instead of eight
 * gathers.  It costs 4x the brick's bytes of HBM; a copy that does not fit
 * the budget is left out and the march reads the brick itself.  The images
 * are the same either way.  Switching rebuilds the bricks. */
int ivr_volume_set_quads(ivr_volume *vol, int on);
int ivr_volume_quad_bytes(const ivr_volume *vol, size_t *bytes);  /* bytes held by the copies */
/* Macrocell edge of the CONFIG empty-space skipping grids, in voxels: a
 * power of two in [4, 32], 16 by default (no counterpart in the reference,
 * which has no skipping).  Smaller cells hug the transparent regions more
 * closely, so fewer samples are taken, at the price of more cell crossings
 * and of grids 8x larger per halving.  The images are the same for every
 * edge.  Switching rebuilds the bricks and drops the volume's per-TF grids;
 * views set on the volume derive their frames again on their next render.
 * A predictor attached with ivr_volume_set_mlp stays attached: its grids are
 * built from the new cells (certified and judged as before), but it predicts
 * best on the cell size it was trained on. */
int ivr_volume_set_macrocell(ivr_volume *vol, int cell);
int ivr_volume_macrocell(const ivr_volume *vol, int *cell);
/* min, max and the histogram of mathutil.c:444-470 (hist may be NULL;
 * otherwise it holds hsize = (int)(max-min+1) bins). */
int ivr_volume_minmax(ivr_volume *vol, float *mn, float *mx);
int ivr_volume_histogram(ivr_volume *vol, int *hist, int hsize);
/* The same min, max and histogram without allocating any device memory.
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc/cudaFree where they compute a LUT: a steering
 * server whose HBM budget is fully given to resident volumes (an allocation
 * there fails or evicts a volume), and a frame loop that renders on other
 * streams meanwhile (cudaFree waits for the whole device, stalling them).
 * Its scratch is one static device array (about 261 KiB) that every GPU
 * loading this library holds until the process exits, so hsize is limited
 * to 65536 bins (IVR_ERR_INVALID above that).  The first call on a device
 * looks up that array's address with cudaGetSymbolAddress (and loads the
 * library's kernels there if they are not loaded yet); make that first call
 * before any stream capture.  Calls share the array and it keeps the last
 * call's contents (the bins are cleared at the start of each call): calls
 * that overlap on the GPU -- on two streams or from two threads -- race.
 * The work is queued on `stream`; the call then copies the results into the
 * caller's host arrays and waits for `stream` before it returns.  The
 * volume's device is current during the call; the caller's current device
 * is restored before it returns. */
int ivr_volume_histogram_noalloc(ivr_volume *vol, int *hist, int hsize, float *mn, float *mx, void *stream);

/* --- transfer function (initcolormap, initvolluts, inittransferfunc) ---- */
int ivr_tf_create(ivr_ctx *ctx, ivr_tf **out);
int ivr_tf_free(ivr_tf *tf);
/* Direct LUT injection: n RGBA rows; index = (int)(sample*scale) - offset
 * (scale must be 1 outside IVR_TF_F2B). */
int ivr_tf_set_lut(ivr_tf *tf, const float *rgba, int n, int lut_offset, float lut_scale, int mode);
/* The reference's LUT path: histogram + colormap builder over the volume's
 * global range, lutoffset = (int)(min + 0.5), maxlutindx = hsize - 1. */
int ivr_tf_set_colormap(ivr_tf *tf, ivr_volume *vol, int colormap, int mode);
int ivr_tf_get_lut(const ivr_tf *tf, float *rgba, int n, int *lut_n, int *lut_offset);

/* --- view (setviewport ... updatevolbbox) ------------------------------ */
int ivr_view_create(ivr_ctx *ctx, ivr_view **out);
int ivr_view_free(ivr_view *view);
int ivr_set_view(ivr_view *view, ivr_volume *vol, const ivr_state *state, const ivr_render_params *p);
int ivr_view_info(const ivr_view *view, ivr_frame_info *info);

/* --- render (createlocalimage + compositelocalimage + writetomemory) ---- */
/* Full viewport, all bricks composited.  rgba32_dev: [vh][vw] float4
 * (nullable); rgba8_dev: [vh][vw] uchar4 (nullable). */
int ivr_render(ivr_view *view, ivr_tf *tf, float *rgba32_dev, uint8_t *rgba8_dev, void *stream);
/* One screen tile [x,x+w) x [y,y+h) of the viewport into [h][w] buffers. */
int ivr_render_tile(ivr_view *view, ivr_tf *tf, int x, int y, int w, int h,
                    float *rgba32_dev, uint8_t *rgba8_dev, void *stream);
/* One brick's sub-image over the whole viewport, zero outside its rect
 * (createlocalimage(rank)). */
int ivr_render_brick(ivr_view *view, ivr_tf *tf, int brick, float *rgba32_dev, void *stream);
/* End to end: STATE from host memory in, RGBA8 frame to host memory out;
 * waits for the frame.  Page-locked output (cudaHostAlloc, or registered)
 * is written by the launch itself; pageable output goes through a device
 * buffer and a copy. */
int ivr_render_host(ivr_view *view, ivr_volume *vol, ivr_tf *tf, const ivr_state *state,
                    const ivr_render_params *p, uint8_t *rgba8_host, void *stream);

/* Work census of one CONFIG frame (a diagnostic launch, not for timing):
 * lattice = sample points of the plain method (every brick, no skipping, no
 * termination) -- the unit of Gsamples/s; executed = samples actually
 * taken; touched_bytes = bytes of the macrocells an executed sample read,
 * the frame's compulsory volume traffic. */
int ivr_census(ivr_view *view, ivr_tf *tf, unsigned long long *lattice, unsigned long long *executed,
               unsigned long long *touched_bytes, void *stream);

/* --- batches: many frames in one persistent launch ---------------------- */
/* A batch holds up to max_frames CONFIG frames (each a set view, a TF and
 * its output buffers) of volumes with one dtype; ivr_batch_render renders
 * them all in one persistent launch (warps take tiles of every frame from
 * one queue).  With use_graph the launch is captured into a CUDA graph on
 * first use and replayed after that.  Each frame is bitwise the frame
 * ivr_render gives for the same view and TF.  The batch's staging memory is
 * reused: ivr_batch_clear/ivr_batch_add wait until the last render has
 * started reading it. */
typedef struct ivr_batch ivr_batch;
int ivr_batch_create(ivr_ctx *ctx, int max_frames, ivr_batch **out);
int ivr_batch_free(ivr_batch *batch);
int ivr_batch_clear(ivr_batch *batch);
int ivr_batch_add(ivr_batch *batch, ivr_view *view, ivr_tf *tf, float *rgba32_dev, uint8_t *rgba8_dev);
int ivr_batch_render(ivr_batch *batch, int use_graph, void *stream);
/* Times every kernel variant (warp tiles 8x4, 4x8, 16x2; one or two
 * samples per loop iteration) on the filled batch and keeps the fastest.
 * variant (nullable) receives its index, ms_per_variant (nullable, 6 floats)
 * the timings. */
int ivr_batch_autotune(ivr_batch *batch, void *stream, int *variant, float *ms_per_variant);
int ivr_batch_set_variant(ivr_batch *batch, int variant);

/* --- steering server: continuous batching over resident volumes ---------
 * Replaces the ivrserver/relay frame path (main.c:206-250,
 * myserver.c:133-165).  Clients submit requests at any time; a scheduler
 * thread keeps `slots` batches in flight, each on its own stream.  The
 * frames' device memory is one output pool of slots * arena_bytes taken from
 * the context's HBM budget at creation.  A free slot takes the queued
 * requests in arrival order, of any volume dtype, while their RGBA8 outputs
 * fit the pool's largest free range (the HBM admission rule), and renders
 * them (CONFIG preset; one batched launch per dtype among them); requests
 * arriving meanwhile, or not fitting the free memory yet, wait and are
 * admitted as slots and pool memory free up.  Only a frame larger than the
 * whole pool is refused (IVR_ERR_NOMEM).  Every frame equals ivr_render of
 * the same view and TF.  While a server runs, its context is used by the
 * server's threads: make no other calls on that context until
 * ivr_server_destroy. */
typedef struct ivr_server ivr_server;
typedef struct ivr_server_config {
    int slots;              /* batches in flight (streams), 1..16 */
    int max_batch_frames;   /* frames per batch */
    size_t arena_bytes;     /* RGBA8 output memory per slot: the pool is slots * arena_bytes */
    int poll_us;            /* scheduler wake-up interval when idle */
    float step;             /* CONFIG sampling of every request */
    float term_alpha;
    int tilew, tileh;
    int variant;            /* batch kernel variant (ivr_batch_set_variant) */
} ivr_server_config;
typedef struct ivr_request {
    int volume;               /* id from ivr_server_add_volume */
    int tf;                   /* id from ivr_server_add_tf */
    ivr_state state;          /* the steering STATE: view, window, opacity, clip */
    uint8_t *rgba8_host;      /* viewport RGBA8, written before completion (page-locked
                                 memory, e.g. from ivr_host_alloc, is written directly) */
    unsigned long long tag;   /* the caller's id, returned in the completion */
} ivr_request;
typedef struct ivr_completion {
    unsigned long long tag;
    int status;               /* IVR_OK, IVR_ERR_NOMEM (frame larger than the output pool), ... */
    int vw, vh;
    double t_queue;           /* seconds from submit to the start of its batch */
    double t_total;           /* seconds from submit to the frame in host memory */
} ivr_completion;
void ivr_server_config_default(ivr_server_config *cfg);
int ivr_server_create(ivr_ctx *ctx, const ivr_server_config *cfg, ivr_server **out);
int ivr_server_destroy(ivr_server *server);  /* finishes every queued request first */
int ivr_server_add_volume(ivr_server *server, ivr_volume *vol, int dtype, int *id);
/* registers a transfer function (copied; a TF edit is a new id) */
int ivr_server_add_tf(ivr_server *server, const float *rgba, int n, int lut_offset, float lut_scale, int *id);
int ivr_server_submit(ivr_server *server, const ivr_request *req);
/* up to max completions, waiting up to wait_ms for the first */
int ivr_server_poll(ivr_server *server, ivr_completion *out, int max, int *n, int wait_ms);
int ivr_server_stats(ivr_server *server, long long *completed, long long *rejected, long long *batches, int *queued);
/* seconds: summed device time of the batches, and the scheduler's time
 * forming/launching batches and copying frames out */
int ivr_server_times(ivr_server *server, double *gpu_s, double *dispatch_s, double *finish_s);
/* Steering front end on 127.0.0.1:port (0 = any): per connection, a
 * 184-byte STATE (finish, winwidth, winheight in network byte order,
 * connection.c:167-200) is answered with the viewport's RGBA8 bytes
 * (connection.c:203-215), rendering `volume` with `tf`; finish != 0 or a
 * disconnect ends the connection. */
int ivr_server_listen(ivr_server *server, int port, int volume, int tf, int *bound_port);

/* --- learned empty-space skipping ---------------------------------------
 * No counterpart in the reference, which samples every lattice point.  A
 * small MLP predicts, per macrocell and transfer function, an upper bound on
 * the cell's post-TF opacity, so the skipping grid of a new TF comes from
 * one batched inference.
 *   inputs (26, zero padded to 32, BF16): the cell's min and max normalised
 *     to the volume's range, its 8-bin value histogram (fractions), and the
 *     TF's 16-knot encoding on 16 knots evenly spaced over the LUT's entries
 *     (entry k (n-1)/15): the largest opacity between knots k and k + 1 for
 *     k < 15, and the largest opacity of the LUT;
 *   network: 26 -> 64 -> 64 -> 1, ReLU, BF16 weights and activations, FP32
 *     accumulation on the tcgen05 tensor cores with accumulators in tensor
 *     memory (training, inference, and the grid of a TF in one launch);
 *   target: the exact bound the plain grid uses, the largest LUT opacity
 *     over the index range of the cell's values.  A cell whose bound is 0
 *     costs only when y > -IVR_MLP_TRANSPARENT; otherwise the loss is
 *     w * (y - target)^2 with w = wneg for y < target, 1 above;
 *   grid: a cell is transparent when y + margin <= 0.
 * A view with skip = IVR_SKIP_LEARNED renders with that grid and, in the
 * same launch, marches a rotating 1/judge_stride of its 8x4 tiles again
 * with the exact grid (on warps of their own); a compare kernel sets the
 * verdict: when some 8-bit channel differs by more than judge_tol, the frame
 * is re-rendered with the exact grid by a launch gated on the verdict (the
 * decision stays on the device) and the TF's learned grid is not used
 * again. */
typedef struct ivr_mlp ivr_mlp;
#define IVR_MLP_PARAMS 6337       /* W1[32][64] (rows 26-31 zero), b1[64], W2[64][64], b2[64], w3[64], b3 */
#define IVR_MLP_IN 32             /* feature row width (BF16) */
#define IVR_MLP_TRANSPARENT 0.5f  /* training code of a zero bound: y <= -0.5 costs nothing */
typedef struct ivr_judge_stats {
    unsigned long long frames;       /* frames judged */
    unsigned long long fallbacks;    /* judged frames above tolerance, re-rendered with the exact grid */
    unsigned long long pixels;       /* pixels compared */
    int worst;                       /* largest 8-bit difference seen */
    int pad;
    unsigned long long exact_frames; /* learned-skip frames rendered with the exact grid because a
                                        judged frame had already found their learned grid wrong */
} ivr_judge_stats;
int ivr_mlp_create(ivr_ctx *ctx, unsigned long long seed, ivr_mlp **out);  /* He-initialised */
int ivr_mlp_free(ivr_mlp *mlp);
int ivr_mlp_get_params(const ivr_mlp *mlp, float *params);  /* IVR_MLP_PARAMS floats */
int ivr_mlp_set_params(ivr_mlp *mlp, const float *params);
/* the parameters as a small binary file (magic, count, little-endian floats) */
int ivr_mlp_save(const ivr_mlp *mlp, const char *path);
int ivr_mlp_load(ivr_mlp *mlp, const char *path);
/* Features ([n][IVR_MLP_IN] BF16) and exact bounds ([n] floats, nullable) of
 * every macrocell of every brick of vol (brick order, cells x fastest) for
 * tf; n = cells, at most cap. */
int ivr_mlp_features(ivr_mlp *mlp, ivr_volume *vol, ivr_tf *tf, uint16_t *x_dev, float *bound_dev, long long cap,
                     long long *n, void *stream);
int ivr_mlp_forward(ivr_mlp *mlp, const uint16_t *x_dev, long long n, float *y_dev, void *stream);
/* Training loss over n rows and its gradient (grad_dev: IVR_MLP_PARAMS
 * floats, loss_dev: one float; both overwritten). */
int ivr_mlp_gradient(ivr_mlp *mlp, const uint16_t *x_dev, const float *bound_dev, long long n, float wneg,
                     float *grad_dev, float *loss_dev, void *stream);
/* The training set: every macrocell of vol under tf, appended. */
int ivr_mlp_add_samples(ivr_mlp *mlp, ivr_volume *vol, ivr_tf *tf, long long *total);
int ivr_mlp_clear_samples(ivr_mlp *mlp);
/* Adam over shuffled mini-batches of batch_rows; loss_per_epoch (nullable)
 * receives the mean batch loss of each epoch. */
int ivr_mlp_train(ivr_mlp *mlp, int epochs, int batch_rows, float lr, float wneg, float *loss_per_epoch);
/* The smallest margin with y + margin > 0 for every training sample whose
 * bound is above 0, plus slack; recall = the fraction of zero-bound samples
 * that margin leaves transparent. */
int ivr_mlp_calibrate(ivr_mlp *mlp, float slack, float *margin, float *recall);
/* Attaches a predictor and its margin to the volume (NULL detaches); the
 * volume's learned grids are dropped.  The predictor must outlive the
 * attachment; changing its parameters later invalidates the grids too.
 * certify != 0: each learned grid is checked cell by cell against the exact
 * empty-cell test as it is built, and a false skip (a cell called
 * transparent whose LUT range holds a nonzero opacity) is kept opaque.
 * With certify = 0 only the per-frame image judge guards the frames. */
int ivr_volume_set_mlp(ivr_volume *vol, ivr_mlp *mlp, float margin, int certify);
/* Counts over the learned grids built since ivr_volume_set_mlp (waits):
 * stats[0] cells, [1] exactly transparent cells, [2] cells the predictor
 * called transparent, [3] false skips among them. */
int ivr_volume_learned_stats(ivr_volume *vol, unsigned long long *stats);
/* The skipping grid that frames of the given skip mode (IVR_SKIP_GRID or
 * IVR_SKIP_LEARNED) use for tf, built if needed, for one brick: per
 * macrocell (x fastest, dims[0] x dims[1] x dims[2] cells) 0 where a sample
 * can be opaque, else r >= 1 = every cell within r - 1 cells (Chebyshev) is
 * transparent, capped (at 8 unless built otherwise).  Copies it into host memory cells (capacity n
 * bytes) and waits; with cells = NULL only dims is filled. */
int ivr_volume_skip_grid(ivr_volume *vol, ivr_tf *tf, int skip, int brick, uint8_t *cells, long long n, int *dims);
/* The judge's totals over the view's learned-skip frames (waits for them). */
int ivr_view_judge_stats(ivr_view *view, ivr_judge_stats *stats);

/* --- measurement -------------------------------------------------------- */
/* The sample-rate roofline of the CONFIG march (no counterpart in the
 * reference): the sampler alone -- trilinear reconstruction from the
 * corner-packed layout, LUT fetch, front-to-back blend, no ray set-up,
 * skipping or divergence -- on a 64^3 brick of `dtype` that stays in cache,
 * every resident thread marching its own ray.  Samples per second / 1e9
 * (waits for the timing). */
int ivr_sample_peak(ivr_ctx *ctx, int dtype, double *gsamples_per_s, void *stream);
/* The same roofline through other layouts of the brick, for comparison:
 * the march reads the corner-packed copies (QUADS) or the bricks themselves
 * (BRICKS); TEX_POINT reads a 3D texture with eight point fetches and the
 * same blend (the same value, bit for bit); TEX_LINEAR takes one
 * hardware-filtered texture fetch, whose fixed-point weights make it
 * inexact.  max_abs_err (nullable): the largest |sample - exact trilinear
 * sample| over 2^20 hashed positions, in volume units. */
typedef enum { IVR_SAMPLER_QUADS = 0, IVR_SAMPLER_BRICKS = 1, IVR_SAMPLER_TEX_POINT = 2,
               IVR_SAMPLER_TEX_LINEAR = 3 } ivr_sampler_layout;
int ivr_sample_peak_layout(ivr_ctx *ctx, int dtype, int layout, double *gsamples_per_s, double *max_abs_err,
                           void *stream);

/* --- compositing and output -------------------------------------------- */
/* compositetiles (main.c:1203-1218): num sub-images of w*h RGBA floats in
 * near -> far order, composited far -> near onto tilebuf with
 * d = s + (1 - s.a) * d. */
int ivr_composite(ivr_ctx *ctx, float *tilebuf_dev, const float *rcolorbuf_dev, int num,
                  int w, int h, void *stream);
/* (uint8)(clamp(v,0,1) * 255 + 0.5) per float (main.c:1404). */
int ivr_quantize(ivr_ctx *ctx, const float *in_dev, uint8_t *out_dev, long long n, void *stream);

/* --- host plumbing (no counterpart in the reference, whose buffers are all
 * host memory) ------------------------------------------------------------
 * For C callers that hold no CUDA headers: a copy of `bytes` between any
 * two of host and device memory, queued on `stream`, and a wait for
 * everything queued on `stream`. */
int ivr_copy(ivr_ctx *ctx, void *dst, const void *src, size_t bytes, void *stream);
int ivr_stream_wait(ivr_ctx *ctx, void *stream);

#ifdef __cplusplus
}
#endif
#endif
