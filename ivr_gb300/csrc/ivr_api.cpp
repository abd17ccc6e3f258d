// ivr_api.cpp -- the C ABI (include/ivr_gpu.h): handles, device memory
// under an HBM budget, volume load and brick set-up, transfer functions,
// views and render calls.
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ivr_handles.h"

namespace ivr {

int fail(ivr_ctx *c, int code, const char *fmt, ...)
{
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_fail(ivr_ctx *c, cudaError_t e, const char *what)
{
    return fail(c, IVR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int dev_alloc(ivr_ctx *c, size_t bytes, void **p)
{
    *p = nullptr;
    if (bytes == 0) return IVR_OK;
    if (c->budget && c->used + bytes > c->budget)
        return fail(c, IVR_ERR_NOMEM, "HBM budget: %zu + %zu bytes exceeds %zu", c->used, bytes, c->budget);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(c, IVR_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    c->used += bytes;
    return IVR_OK;
}

void dev_free(ivr_ctx *c, void *p, size_t bytes)
{
    if (!p) return;
    cudaFree(p);
    c->used -= bytes;
}

void *host_mapping(void *p, size_t n)
{
    if (!p || n == 0) return nullptr;
    cudaPointerAttributes a, z;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&z, (char *) p + n - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || z.type != cudaMemoryTypeHost || !a.devicePointer || !z.devicePointer)
        return nullptr;
    if ((char *) z.devicePointer - (char *) a.devicePointer != (ptrdiff_t) (n - 1)) return nullptr;
    return a.devicePointer;
}

size_t brick_bytes(const ivr_volume *v, const HostBrick &b)
{
    return (size_t) b.lw * b.lh * b.ld * dtype_size(v->dtype);
}

}  // namespace ivr

namespace {

using namespace ivr;

void delete_grid(ivr_volume *v, ivr_volume::TfGrid *g)
{
    for (size_t k = 0; k < g->dist.size(); k++)
        if (g->dist[k]) dev_free(v->ctx, g->dist[k], mc_cells(v->bricks[k]));
    for (size_t k = 0; k < g->opac.size(); k++)
        if (g->opac[k]) dev_free(v->ctx, g->opac[k], mc_cells(v->bricks[k]));
    if (g->ev) cudaEventDestroy(g->ev);
    if (g->built) cudaEventDestroy(g->built);
    if (g->h_reject) cudaFreeHost(g->h_reject);
    if (g->d_bad) dev_free(v->ctx, g->d_bad, sizeof(int));
    delete g;
}

}  // namespace

void ivr::drop_learned_grids(ivr_volume *v)
{
    if (v->grids.empty()) return;
    cudaDeviceSynchronize();
    std::vector<ivr_volume::TfGrid *> keep;
    for (auto *g : v->grids)
        if (g->learned) delete_grid(v, g);
        else keep.push_back(g);
    v->grids.swap(keep);
}

namespace {

void free_grids(ivr_volume *v)
{
    if (!v->grids.empty()) cudaDeviceSynchronize();
    for (auto *g : v->grids) delete_grid(v, g);
    v->grids.clear();
}

void free_bricks(ivr_volume *v)
{
    free_grids(v);
    learned_release(v);
    for (auto &b : v->bricks) {
        if (b.owns) dev_free(v->ctx, b.data, brick_bytes(v, b));
        dev_free(v->ctx, b.mc_minmax, mc_cells(b) * 2 * sizeof(float));
        if (b.quad) dev_free(v->ctx, b.quad, quad_bytes(v->dtype, b.lw, b.lh, b.ld));
    }
    v->bricks.clear();
}

// macrocell grid over a brick's local voxels (cells of the volume's edge,
// +1 layer)
int build_macrocells(ivr_volume *v, HostBrick &b)
{
    b.cell = v->cell;
    b.mcx = (b.lw - 2) / b.cell + 1;
    b.mcy = (b.lh - 2) / b.cell + 1;
    b.mcz = (b.ld - 2) / b.cell + 1;
    int rc = dev_alloc(v->ctx, mc_cells(b) * 2 * sizeof(float), (void **) &b.mc_minmax);
    if (rc) return rc;
    CK(v->ctx, launch_macrocells(b.data, v->dtype, b.lw, b.lh, b.ld, b.cell, b.mc_minmax, b.mcx, b.mcy, b.mcz, 0));
    return IVR_OK;
}

int setup_bricks(ivr_volume *v, int py, int px, int pz, int overlap)
{
    ivr_ctx *c = v->ctx;
    if (py < 1 || px < 1 || pz < 1 || py * px * pz > kMaxBricks || overlap < 0 || overlap > 1)
        return fail(c, IVR_ERR_INVALID, "brick grid %dx%dx%d (overlap %d) not supported", py, px, pz, overlap);
    if (v->w / px < 2 || v->h / py < 2 || v->d / pz < 2)
        return fail(c, IVR_ERR_INVALID, "bricks of %dx%dx%d voxels are too thin", v->w / px, v->h / py, v->d / pz);
    free_bricks(v);
    v->layout++;
    int K = py * px * pz;
    v->bricks.resize(K);
    for (int r = 0; r < K; r++) {
        HostBrick &b = v->bricks[r];
        memset(&b, 0, sizeof(b));
        brick_geometry(v->w, v->h, v->d, py, px, pz, overlap, r, b);
        if (K == 1) {
            b.data = v->d_full;
            b.owns = false;
        } else {
            int rc = dev_alloc(c, brick_bytes(v, b), &b.data);
            if (rc) { free_bricks(v); return rc; }
            b.owns = true;
            CK(c, launch_gather_brick(v->d_full, v->w, v->h, v->d, b.data, b.sx, b.sy, b.sz, b.lw, b.lh, b.ld,
                                      (int) dtype_size(v->dtype), 0));
        }
        int rc = build_macrocells(v, b);
        if (rc) { free_bricks(v); return rc; }
        if (v->quads) {
            // the corner-packed copy is an accelerator: without room for it
            // the march reads the brick itself
            const size_t qb = quad_bytes(v->dtype, b.lw, b.lh, b.ld);
            const std::string err = c->err;
            if (dev_alloc(c, qb, &b.quad) == IVR_OK)
                CK(c, launch_quads(b.data, v->dtype, b.lw, b.lh, b.ld, b.quad, 0));
            else
                c->err = err;
        }
    }
    CK(c, cudaDeviceSynchronize());
    v->py = py; v->px = px; v->pz = pz; v->overlap = overlap;
    return IVR_OK;
}

int valid_params(ivr_ctx *c, const ivr_render_params *p)
{
    if (!p) return fail(c, IVR_ERR_INVALID, "null render params");
    if (p->preset != IVR_PRESET_REF && p->preset != IVR_PRESET_CONFIG)
        return fail(c, IVR_ERR_INVALID, "unknown preset %d", p->preset);
    // bounds that keep every ray's sample count finite and modest
    if (p->preset == IVR_PRESET_REF) {
        if (!(p->step >= 1.0e-5f && p->step <= 1.0f)) return fail(c, IVR_ERR_INVALID, "REF step must be in [1e-5, 1]");
        if (p->max_samples < 1 || p->max_samples > 65536)
            return fail(c, IVR_ERR_INVALID, "REF max_samples must be in [1, 65536]");
    } else {
        if (!(p->step >= 0.01f && p->step <= 64.0f)) return fail(c, IVR_ERR_INVALID, "step must be in [0.01, 64] voxels");
        if (p->max_samples != 0) return fail(c, IVR_ERR_UNSUPPORTED, "CONFIG samples are not capped");
    }
    if (p->tilew < 1 || p->tileh < 1) return fail(c, IVR_ERR_INVALID, "tile size must be >= 1");
    if (p->skip < IVR_SKIP_NONE || p->skip > IVR_SKIP_LEARNED) return fail(c, IVR_ERR_INVALID, "unknown skip %d", p->skip);
    if (p->skip == IVR_SKIP_LEARNED) {
        if (p->preset != IVR_PRESET_CONFIG) return fail(c, IVR_ERR_UNSUPPORTED, "learned skipping needs the CONFIG preset");
        if (p->judge_stride < 1 || p->judge_stride > (1 << 20))
            return fail(c, IVR_ERR_INVALID, "judge_stride must be in [1, 2^20]");
        if (p->judge_tol < 0 || p->judge_tol > 255) return fail(c, IVR_ERR_INVALID, "judge_tol must be in [0, 255]");
    }
    if (p->tile_order != IVR_TILES_RASTER && p->tile_order != IVR_TILES_COST)
        return fail(c, IVR_ERR_INVALID, "unknown tile_order %d", p->tile_order);
    return IVR_OK;
}

// The per-brick distance fields of the volume for a TF, built on `s` when
// the TF (or a zero opacity scale) is new to the volume: the exact fields, or
// with `learned` the attached predictor's.  Up to kMaxTfGrids are kept;
// beyond that the least recently used one not read by frames since
// `protect_from` is rebuilt in place once the last launch that read it has
// finished (its event), or a new one is added when every grid is protected.
int tf_grid(ivr_volume *v, const ivr_tf *tf, bool zero_alpha, bool learned, cudaStream_t s,
            unsigned long long protect_from, ivr_volume::TfGrid **out, bool *built = nullptr)
{
    if (built) *built = false;
    ivr_ctx *c = v->ctx;
    if (learned && !v->mlp) return fail(c, IVR_ERR_INVALID, "IVR_SKIP_LEARNED: no predictor attached to the volume");
    const unsigned mser = learned ? mlp_serial(v->mlp) : 0;
    const unsigned long long now = ++c->grid_clock;
    for (auto *g : v->grids)
        if (g->serial == tf->serial && g->zero_alpha == (int) zero_alpha && g->learned == (int) learned &&
            g->mlp_serial == mser) {
            g->last_use = now;
            *out = g;
            return IVR_OK;
        }
    ivr_volume::TfGrid *g = nullptr;
    if (v->grids.size() >= kMaxTfGrids)
        for (auto *h : v->grids)
            if (h->last_use < protect_from && (!g || h->last_use < g->last_use)) g = h;
    if (g) {
        CK(c, cudaEventSynchronize(g->ev));
    } else {
        g = new ivr_volume::TfGrid();
        g->dist.assign(v->bricks.size(), nullptr);
        g->opac.assign(v->bricks.size(), nullptr);
        int rc = IVR_OK;
        if (cudaEventCreateWithFlags(&g->ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&g->built, cudaEventDisableTiming) != cudaSuccess ||
            cudaHostAlloc((void **) &g->h_reject, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer((void **) &g->d_reject, g->h_reject, 0) != cudaSuccess) {
            cudaGetLastError();
            rc = IVR_ERR_CUDA;
        }
        if (rc == IVR_OK) rc = dev_alloc(c, sizeof(int), (void **) &g->d_bad);
        for (size_t k = 0; k < v->bricks.size() && rc == IVR_OK; k++) {
            rc = dev_alloc(c, mc_cells(v->bricks[k]), (void **) &g->dist[k]);
            if (rc == IVR_OK) rc = dev_alloc(c, mc_cells(v->bricks[k]), (void **) &g->opac[k]);
        }
        if (rc) {
            delete_grid(v, g);
            return rc == IVR_ERR_CUDA ? fail(c, rc, "events for a distance field") : rc;
        }
        v->grids.push_back(g);
    }
    g->serial = tf->serial;
    g->zero_alpha = (int) zero_alpha;
    g->learned = (int) learned;
    g->mlp_serial = mser;
    g->last_use = now;
    g->rejected = false;
    *(volatile int *) g->h_reject = 0;  // no launch that reads it is pending
    CK(c, cudaMemsetAsync(g->d_bad, 0, sizeof(int), s));
    // cell opacities (the tile order's input): an exact grid's only; learned
    // frames use those of their TF's exact grid
    if (zero_alpha) {
        for (size_t k = 0; k < v->bricks.size(); k++) {
            CK(c, cudaMemsetAsync(g->opac[k], 0, mc_cells(v->bricks[k]), s));
            CK(c, cudaMemsetAsync(g->dist[k], kDistCap, mc_cells(v->bricks[k]), s));
        }
    } else if (learned) {
        int rc = learned_fields(v, tf, g->dist, s);
        if (rc) {
            g->serial = 0;  // unusable; rebuilt on next use
            g->last_use = 0;
            return rc;
        }
    } else {
        for (size_t k = 0; k < v->bricks.size(); k++) {
            const HostBrick &b = v->bricks[k];
            CK(c, launch_empty_flags(b.mc_minmax, b.mcx, b.mcy, b.mcz, tf->d_nzprefix, tf->d_aprefix, tf->n, tf->off,
                                     tf->scale, g->dist[k], g->opac[k], s));
        }
    }
    CK(c, cudaEventRecord(g->ev, s));
    CK(c, cudaEventRecord(g->built, s));
    *out = g;
    if (built) *built = true;
    return IVR_OK;
}

// A learned grid the judge rejected is replaced by the exact one.  The host
// reads the mapped verdict word without waiting: a verdict that has not
// arrived yet only means one more judged frame.
bool learned_rejected(ivr_volume::TfGrid *g)
{
    if (!g->rejected) g->rejected = *(volatile int *) g->h_reject != 0;
    return g->rejected;
}

// Fills everything of a launch's frame descriptor that depends on the TF,
// the output window and the skipping grid.
int frame_for(ivr_view *view, ivr_tf *tf, int x, int y, int w, int h, int single, cudaStream_t s, FrameDesc &f,
              ivr_volume::TfGrid **grid, unsigned long long protect_from = ~0ull, bool *built = nullptr,
              ivr_volume::TfGrid **exact = nullptr)
{
    if (built) *built = false;
    *grid = nullptr;
    if (exact) *exact = nullptr;
    ivr_ctx *c = view->ctx;
    if (!view->valid) return fail(c, IVR_ERR_INVALID, "ivr_set_view has not succeeded on this view");
    if (!tf) return fail(c, IVR_ERR_INVALID, "null transfer function");
    if (tf->mode != IVR_TF_RGBBLEND && tf->n < 1) return fail(c, IVR_ERR_INVALID, "transfer function has no LUT");
    const bool f2b = tf->mode == IVR_TF_F2B;
    if ((view->p.preset == IVR_PRESET_CONFIG) != f2b)
        return fail(c, IVR_ERR_UNSUPPORTED, "CONFIG preset needs IVR_TF_F2B and REF needs ids 0-5 (got %d)", tf->mode);
    if (view->layout != view->vol->layout) {
        // the volume's bricks were rebuilt (ivr_bricks_setup, corner-packed
        // copies or macrocell edge switched) since ivr_set_view: derive the
        // frame again from the view's STATE and parameters
        ivr_volume *vol = view->vol;
        int rc = build_frame(vol->w, vol->h, vol->d, vol->dtype, vol->bricks.data(), (int) vol->bricks.size(),
                             view->st, view->p, view->f, view->info);
        if (rc) {
            view->valid = false;
            return fail(c, rc, "view set-up failed after the volume's bricks changed");
        }
        view->layout = vol->layout;
    }
    if (x < 0 || y < 0 || w < 1 || h < 1 || x + w > view->info.vw || y + h > view->info.vh)
        return fail(c, IVR_ERR_INVALID, "tile %d,%d %dx%d outside the %dx%d viewport", x, y, w, h, view->info.vw,
                    view->info.vh);
    f = view->f;
    f.tf_mode = tf->mode;
    f.lut = tf->d_lut;
    f.lut_n = tf->n;
    f.lut_off = tf->off;
    f.lut_scale = tf->scale;
    f.out_x = x; f.out_y = y; f.out_w = w; f.out_h = h;
    f.single = single;
    f.counters = nullptr;
    f.gate = nullptr;
    f.judge = nullptr;
    f.judge_reject = nullptr;
    f.learned_bad = nullptr;
    f.judge8 = nullptr;
    f.perm = nullptr;
    if (view->p.skip != IVR_SKIP_NONE && view->p.preset == IVR_PRESET_CONFIG) {
        // a learned grid comes with the exact one (the judge's and the
        // fallback's), unless the judge has rejected it: then only the exact
        const bool zero_alpha = !(f.alpha != 0.0f);
        bool learned = view->p.skip == IVR_SKIP_LEARNED && !zero_alpha;
        if (learned && !exact)
            return fail(view->ctx, IVR_ERR_UNSUPPORTED, "IVR_SKIP_LEARNED frames render through ivr_render*");
        // the exact grid first: its cell opacities (the tile order's input,
        // the same for both grids of a TF) serve the learned frames too
        ivr_volume::TfGrid *eg = nullptr;
        bool ebuilt = false;
        int rc = tf_grid(view->vol, tf, zero_alpha, false, s, protect_from, &eg, &ebuilt);
        if (rc) return rc;
        ivr_volume::TfGrid *lg = nullptr;
        if (learned) {
            rc = tf_grid(view->vol, tf, false, true, s, protect_from, &lg, built);
            if (rc) return rc;
            learned = !learned_rejected(lg);
        }
        if (built) *built |= ebuilt;
        *grid = learned ? lg : eg;
        if (learned) *exact = eg;
        for (int k = 0; k < f.nb; k++) {
            f.b[k].empty = (*grid)->dist[k];
            f.b[k].opac = eg->opac[k];
        }
    }
    return IVR_OK;
}

// One CONFIG/REF launch of f on the view's ticket counter.
int launch_view(ivr_view *view, FrameDesc &f, float *o32, uint8_t *o8, cudaStream_t s)
{
    ivr_ctx *c = view->ctx;
    if (view->tickets_dirty) {
        CK(c, cudaMemsetAsync(view->d_tickets, 0, sizeof(unsigned long long), s));
        view->ticket_base = 0;
        view->tickets_dirty = false;
    }
    f.tickets = view->d_tickets;
    f.ticket_base = view->ticket_base;
    long long used = 0;
    cudaError_t e = launch_march(f, (float4 *) o32, (uchar4 *) o8, s, &used);
    if (e != cudaSuccess) {
        view->tickets_dirty = true;
        return cuda_fail(c, e, "march launch");
    }
    view->ticket_base += (unsigned long long) used;
    return IVR_OK;
}

// IVR_TILES_COST: the launch's tile permutation, costliest first, into the
// view's next slot (grown to the window's tile count); sets f.perm and
// returns the slot.  Built on the view's order stream after the launches
// that last read the slot and after the builds of the grid and of the exact
// grid (whose cell opacities it reads), so it overlaps the tail of the
// frame before (in a stream capture: on s itself).
int order_tiles(ivr_view *view, FrameDesc &f, const ivr_volume::TfGrid *grid, const ivr_volume::TfGrid *exact,
                cudaStream_t s, int *slot)
{
    ivr_ctx *c = view->ctx;
    const long long ntiles = (long long) ((f.out_w + 7) >> 3) * ((f.out_h + 3) >> 2);
    if (!view->order_stream) {
        // all or nothing: the stream is set only once its slots are complete
        cudaStream_t os = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&os, cudaStreamNonBlocking);
        for (auto &o : view->tiles) {
            if (e == cudaSuccess && !o.done) e = cudaEventCreateWithFlags(&o.done, cudaEventDisableTiming);
            if (e == cudaSuccess && !o.used) e = cudaEventCreateWithFlags(&o.used, cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            if (os) cudaStreamDestroy(os);
            return cuda_fail(c, e, "tile order stream and events");
        }
        for (auto &o : view->tiles)
            if (!o.counts) {
                int rc = dev_alloc(c, sizeof(int) * 128, (void **) &o.counts);
                if (rc) {
                    cudaStreamDestroy(os);
                    return rc;
                }
            }
        view->order_stream = os;
    }
    if (view->tile_cap < ntiles) {
        for (auto &o : view->tiles) {  // cudaFree waits for the launches that read them
            dev_free(c, o.perm, sizeof(int) * (size_t) view->tile_cap);
            dev_free(c, o.key, (size_t) view->tile_cap);
            o.perm = nullptr;
            o.key = nullptr;
        }
        view->tile_cap = 0;
        for (auto &o : view->tiles) {
            int rc = dev_alloc(c, sizeof(int) * (size_t) ntiles, (void **) &o.perm);
            if (rc == IVR_OK) rc = dev_alloc(c, (size_t) ntiles, (void **) &o.key);
            if (rc) {
                for (auto &q : view->tiles) {
                    dev_free(c, q.perm, q.perm ? sizeof(int) * (size_t) ntiles : 0);
                    dev_free(c, q.key, q.key ? (size_t) ntiles : 0);
                    q.perm = nullptr;
                    q.key = nullptr;
                }
                return rc;
            }
        }
        view->tile_cap = ntiles;
    }
    *slot = view->tile_slot;
    view->tile_slot ^= 1;
    ivr_view::TileOrder &o = view->tiles[*slot];
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(c, cudaStreamIsCapturing(s, &cap));
    cudaStream_t os = cap == cudaStreamCaptureStatusNone ? view->order_stream : s;
    if (os != s) {
        if (o.used_recorded) CK(c, cudaStreamWaitEvent(os, o.used, 0));
        CK(c, cudaStreamWaitEvent(os, grid->built, 0));
        if (exact) CK(c, cudaStreamWaitEvent(os, exact->built, 0));  // its cell opacities
    }
    CK(c, launch_tile_order(f, o.key, o.counts, o.perm, os));
    if (os != s) {
        CK(c, cudaEventRecord(o.done, os));
        CK(c, cudaStreamWaitEvent(s, o.done, 0));
    }
    f.perm = o.perm;
    return IVR_OK;
}

int render_window(ivr_view *view, ivr_tf *tf, int x, int y, int w, int h, int single, float *o32, uint8_t *o8,
                  void *stream, std::vector<uint8_t *> *touched = nullptr)
{
    ivr_ctx *c = view ? view->ctx : nullptr;
    if (!view) return fail(c, IVR_ERR_INVALID, "null view");
    cudaStream_t s = (cudaStream_t) stream;
    FrameDesc f;
    ivr_volume::TfGrid *grid = nullptr, *exact = nullptr;
    int rc = frame_for(view, tf, x, y, w, h, single, s, f, &grid, c->grid_clock + 1, nullptr, &exact);
    if (rc) return rc;
    if (touched) {
        f.counters = c->d_counters;  // census launches count
        f.census = 1;
        for (int k = 0; k < f.nb; k++) f.b[k].touched = (*touched)[k];
    }
    // a learned-skip frame: judged in the same launch (a rotating
    // 1/judge_stride of its tiles marched again with the exact grid), then
    // re-rendered with the exact grid by a launch gated on the verdict
    const bool judged = exact && !touched && (o32 || o8);
    if (judged) {
        f.judge = (JudgeWords *) view->d_judge;
        f.judge_reject = grid->d_reject;
        f.learned_bad = grid->d_bad;
        f.judge_stride = view->p.judge_stride;
        f.judge_phase = (int) (view->judge_frame++ % (unsigned long long) view->p.judge_stride);
        f.judge_tol = view->p.judge_tol;
        for (int k = 0; k < f.nb; k++) f.exact[k] = exact->dist[k];
        const size_t need = (size_t) std::max(judge_scratch_bytes(f), (long long) sizeof(uchar4));
        if (view->judge_bytes < need) {
            dev_free(c, view->d_judge8, view->judge_bytes);
            view->d_judge8 = nullptr;
            view->judge_bytes = 0;
            rc = dev_alloc(c, need, (void **) &view->d_judge8);
            if (rc) return rc;
            view->judge_bytes = need;
        }
        f.judge8 = view->d_judge8;
    }
    int slot = -1;
    if (!touched && grid && view->p.tile_order == IVR_TILES_COST) {
        rc = order_tiles(view, f, grid, exact, s, &slot);
        if (rc) return rc;
    }
    rc = launch_view(view, f, o32, o8, s);
    if (rc == IVR_OK && judged) {
        const cudaError_t je = launch_judge_compare(f, (const uchar4 *) o8, (const float4 *) o32, s);
        if (je != cudaSuccess) rc = cuda_fail(c, je, "judge compare launch");
        FrameDesc ff = f;
        ff.judge = nullptr;
        for (int k = 0; k < ff.nb; k++) ff.b[k].empty = exact->dist[k];
        ff.gate = &((JudgeWords *) view->d_judge)->fail;
        if (rc == IVR_OK) rc = launch_view(view, ff, o32, o8, s);
    }
    if (slot >= 0) {  // the slot's readers, whether or not they launched
        CK(c, cudaEventRecord(view->tiles[slot].used, s));
        view->tiles[slot].used_recorded = true;
    }
    if (rc) return rc;
    if (grid) CK(c, cudaEventRecord(grid->ev, s));
    if (exact) CK(c, cudaEventRecord(exact->ev, s));
    return IVR_OK;
}

}  // namespace

extern "C" {

void ivr_params_ref(ivr_render_params *p)
{
    if (!p) return;
    p->preset = IVR_PRESET_REF;
    p->step = 0.001f;  // DELTASAMPLE (types.h:17)
    p->max_samples = 256;  // MAXVOLUMESAMPLES * 4 (ray.c:61)
    p->term_alpha = 2.0f;
    p->order = IVR_ORDER_CENTER;
    p->skip = IVR_SKIP_NONE;
    p->tilew = 1;
    p->tileh = 1;
    p->judge_stride = 16;
    p->judge_tol = 1;
    p->tile_order = IVR_TILES_RASTER;
}

void ivr_params_config(ivr_render_params *p)
{
    if (!p) return;
    p->preset = IVR_PRESET_CONFIG;
    p->step = 0.5f;
    p->max_samples = 0;
    p->term_alpha = 0.99f;
    p->order = IVR_ORDER_AXIS;
    p->skip = IVR_SKIP_GRID;
    p->tilew = 1;
    p->tileh = 1;
    p->judge_stride = 16;
    p->judge_tol = 1;
    p->tile_order = IVR_TILES_COST;
}

int ivr_create(int device, size_t budget, ivr_ctx **out)
{
    if (!out) return IVR_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return IVR_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return IVR_ERR_CUDA;
    ivr_ctx *c = new ivr_ctx();
    c->device = device;
    c->budget = budget;
    if (dev_alloc(c, sizeof(unsigned long long) * 4, (void **) &c->d_counters) ||
        dev_alloc(c, sizeof(float) * 2 * minmax_parts(), (void **) &c->d_partial)) {
        ivr_destroy(c);
        return IVR_ERR_NOMEM;
    }
    cudaMemset(c->d_counters, 0, sizeof(unsigned long long) * 4);
    *out = c;
    return IVR_OK;
}

int ivr_destroy(ivr_ctx *c)
{
    if (!c) return IVR_ERR_INVALID;
    cudaSetDevice(c->device);
    dev_free(c, c->d_counters, sizeof(unsigned long long) * 4);
    dev_free(c, c->d_partial, sizeof(float) * 2 * minmax_parts());
    dev_free(c, c->d_frame8, c->frame8_bytes);
    delete c;
    return IVR_OK;
}

const char *ivr_last_error(const ivr_ctx *c) { return c ? c->err.c_str() : "null context"; }

int ivr_mem_used(const ivr_ctx *c, size_t *bytes)
{
    if (!c || !bytes) return IVR_ERR_INVALID;
    *bytes = c->used;
    return IVR_OK;
}

int ivr_device_alloc(ivr_ctx *c, size_t bytes, void **ptr)
{
    if (!c || !ptr) return IVR_ERR_INVALID;
    CK(c, cudaSetDevice(c->device));
    return dev_alloc(c, bytes, ptr);
}

int ivr_device_free(ivr_ctx *c, void *ptr, size_t bytes)
{
    if (!c) return IVR_ERR_INVALID;
    dev_free(c, ptr, bytes);
    return IVR_OK;
}

int ivr_host_alloc(ivr_ctx *c, size_t bytes, void **ptr)
{
    if (!c || !ptr || bytes == 0) return c ? fail(c, IVR_ERR_INVALID, "bad host allocation") : IVR_ERR_INVALID;
    *ptr = nullptr;
    CK(c, cudaSetDevice(c->device));
    if (cudaHostAlloc(ptr, bytes, cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(c, IVR_ERR_NOMEM, "cudaHostAlloc(%zu) failed", bytes);
    }
    return IVR_OK;
}

int ivr_host_free(ivr_ctx *c, void *ptr)
{
    if (!ptr) return IVR_OK;
    const cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return c ? cuda_fail(c, e, "cudaFreeHost") : IVR_ERR_CUDA;
    return IVR_OK;
}

int ivr_volume_load(ivr_ctx *c, const void *host, int w, int h, int d, int dtype, int byteswap, ivr_volume **out)
{
    if (!c || !out) return IVR_ERR_INVALID;
    *out = nullptr;
    if (!host) return fail(c, IVR_ERR_INVALID, "null volume data");
    if (w < 2 || h < 2 || d < 2) return fail(c, IVR_ERR_INVALID, "volume %dx%dx%d: every dimension must be >= 2", w, h, d);
    if (dtype != IVR_U8 && dtype != IVR_U16 && dtype != IVR_F32) return fail(c, IVR_ERR_INVALID, "dtype %d", dtype);
    // the kernels index a brick with 32-bit voxel offsets
    if ((long long) w * h * d >= (1LL << 32)) return fail(c, IVR_ERR_UNSUPPORTED, "volume of 2^32 or more voxels");
    CK(c, cudaSetDevice(c->device));
    ivr_volume *v = new ivr_volume();
    v->ctx = c;
    v->w = w; v->h = h; v->d = d; v->dtype = dtype;
    v->full_bytes = (size_t) w * h * d * dtype_size(dtype);
    int rc = dev_alloc(c, v->full_bytes, &v->d_full);
    if (rc) { delete v; return rc; }
    cudaError_t e = cudaMemcpy(v->d_full, host, v->full_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && byteswap) e = launch_byteswap(v->d_full, (long long) w * h * d, (int) dtype_size(dtype), 0);
    if (e != cudaSuccess) {
        ivr_volume_free(v);
        return cuda_fail(c, e, "volume upload");
    }
    rc = setup_bricks(v, 1, 1, 1, 0);
    if (rc) { ivr_volume_free(v); return rc; }
    *out = v;
    return IVR_OK;
}

// Streams a raw file to the device: the file is read in chunks into two
// page-locked staging buffers in turn, each chunk's upload overlapping the
// next chunk's read; the byte swap runs on the device afterwards.
static int stream_file(ivr_ctx *c, FILE *fp, const char *path, void *dst, size_t bytes)
{
    const size_t chunk = std::min(bytes, (size_t) 64 << 20);
    void *stage[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaStream_t st = nullptr;
    bool used[2] = {false, false};
    int rc = IVR_OK;
    for (int k = 0; k < 2 && rc == IVR_OK; k++)
        if (cudaHostAlloc(&stage[k], chunk, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming) != cudaSuccess)
            rc = fail(c, IVR_ERR_NOMEM, "page-locked staging of %zu bytes", chunk);
    if (rc == IVR_OK && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        rc = fail(c, IVR_ERR_CUDA, "upload stream");
    size_t off = 0;
    for (int k = 0; rc == IVR_OK && off < bytes; k ^= 1) {
        const size_t n = std::min(chunk, bytes - off);
        if (used[k] && cudaEventSynchronize(ev[k]) != cudaSuccess) {
            rc = fail(c, IVR_ERR_CUDA, "upload of %s", path);
            break;
        }
        const size_t got = fread(stage[k], 1, n, fp);
        if (got != n) {
            rc = fail(c, IVR_ERR_IO, "%s: read %zu of %zu bytes", path, off + got, bytes);
            break;
        }
        if (cudaMemcpyAsync((char *) dst + off, stage[k], n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaEventRecord(ev[k], st) != cudaSuccess) {
            rc = fail(c, IVR_ERR_CUDA, "upload of %s", path);
            break;
        }
        used[k] = true;
        off += n;
    }
    if (st && cudaStreamSynchronize(st) != cudaSuccess && rc == IVR_OK) rc = fail(c, IVR_ERR_CUDA, "upload of %s", path);
    if (st) cudaStreamDestroy(st);
    for (int k = 0; k < 2; k++) {
        if (ev[k]) cudaEventDestroy(ev[k]);
        if (stage[k]) cudaFreeHost(stage[k]);
    }
    cudaGetLastError();
    return rc;
}

int ivr_volume_load_file(ivr_ctx *c, const char *path, int w, int h, int d, int dtype, int file_little_endian,
                         ivr_volume **out)
{
    if (!c || !out) return IVR_ERR_INVALID;
    *out = nullptr;
    if (!path) return fail(c, IVR_ERR_INVALID, "null path");
    if (w < 2 || h < 2 || d < 2 || (dtype != IVR_U8 && dtype != IVR_U16 && dtype != IVR_F32))
        return fail(c, IVR_ERR_INVALID, "bad volume shape or dtype");
    if ((long long) w * h * d >= (1LL << 32)) return fail(c, IVR_ERR_UNSUPPORTED, "volume of 2^32 or more voxels");
    const size_t bytes = (size_t) w * h * d * dtype_size(dtype);
    CK(c, cudaSetDevice(c->device));
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(c, IVR_ERR_IO, "cannot open %s", path);
    setvbuf(fp, nullptr, _IONBF, 0);  // chunks go straight into the staging buffers
    ivr_volume *v = new ivr_volume();
    v->ctx = c;
    v->w = w; v->h = h; v->d = d; v->dtype = dtype;
    v->full_bytes = bytes;
    int rc = dev_alloc(c, bytes, &v->d_full);
    if (rc == IVR_OK) rc = stream_file(c, fp, path, v->d_full, bytes);
    fclose(fp);
    const uint16_t probe = 1;
    const bool host_little = *(const unsigned char *) &probe == 1;
    if (rc == IVR_OK && (file_little_endian != 0) != host_little) {
        const cudaError_t e = launch_byteswap(v->d_full, (long long) w * h * d, (int) dtype_size(dtype), 0);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "byte swap");
    }
    if (rc == IVR_OK) rc = setup_bricks(v, 1, 1, 1, 0);
    if (rc) {
        const std::string err = c->err;
        ivr_volume_free(v);
        c->err = err;
        return rc;
    }
    *out = v;
    return IVR_OK;
}

int ivr_volume_free(ivr_volume *v)
{
    if (!v) return IVR_ERR_INVALID;
    free_bricks(v);
    dev_free(v->ctx, v->d_lstats, 4 * sizeof(unsigned long long));
    dev_free(v->ctx, v->d_full, v->full_bytes);
    delete v;
    return IVR_OK;
}

int ivr_volume_skip_grid(ivr_volume *v, ivr_tf *tf, int skip, int brick, uint8_t *cells, long long n, int *dims)
{
    if (!v) return IVR_ERR_INVALID;
    ivr_ctx *c = v->ctx;
    if (!tf) return fail(c, IVR_ERR_INVALID, "null transfer function");
    if (skip != IVR_SKIP_GRID && skip != IVR_SKIP_LEARNED)
        return fail(c, IVR_ERR_INVALID, "skip %d: the grids are IVR_SKIP_GRID's and IVR_SKIP_LEARNED's", skip);
    if (brick < 0 || brick >= (int) v->bricks.size())
        return fail(c, IVR_ERR_INVALID, "brick %d of %d", brick, (int) v->bricks.size());
    const HostBrick &b = v->bricks[brick];
    if (dims) {
        dims[0] = b.mcx;
        dims[1] = b.mcy;
        dims[2] = b.mcz;
    }
    if (!cells) return IVR_OK;
    const long long ncell = (long long) mc_cells(b);
    if (n < ncell) return fail(c, IVR_ERR_INVALID, "%lld bytes for a grid of %lld cells", n, ncell);
    ivr_volume::TfGrid *g = nullptr;
    int rc = tf_grid(v, tf, false, skip == IVR_SKIP_LEARNED, 0, c->grid_clock + 1, &g);
    if (rc) return rc;
    CK(c, cudaEventSynchronize(g->built));
    CK(c, cudaMemcpy(cells, g->dist[brick], (size_t) ncell, cudaMemcpyDeviceToHost));
    return IVR_OK;
}

int ivr_bricks_setup(ivr_volume *v, int py, int px, int pz, int overlap)
{
    if (!v) return IVR_ERR_INVALID;
    return setup_bricks(v, py, px, pz, overlap);
}

int ivr_volume_gradient(ivr_volume *v, float *grad4_dev, void *stream)
{
    if (!v) return IVR_ERR_INVALID;
    if (!grad4_dev) return fail(v->ctx, IVR_ERR_INVALID, "null gradient output");
    CK(v->ctx, cudaSetDevice(v->ctx->device));
    CK(v->ctx, launch_gradient(v->d_full, v->dtype, v->w, v->h, v->d, (float4 *) grad4_dev, (cudaStream_t) stream));
    return IVR_OK;
}

int ivr_volume_set_quads(ivr_volume *v, int on)
{
    if (!v) return IVR_ERR_INVALID;
    if (v->quads == (on != 0)) return IVR_OK;
    v->quads = on != 0;
    return setup_bricks(v, v->py, v->px, v->pz, v->overlap);  // rebuilt with or without the copies
}

int ivr_volume_set_macrocell(ivr_volume *v, int cell)
{
    if (!v) return IVR_ERR_INVALID;
    if (cell < kMinCell || cell > kMaxCell || (cell & (cell - 1)) != 0)
        return fail(v->ctx, IVR_ERR_INVALID, "macrocell edge %d: a power of two in [%d, %d]", cell, kMinCell, kMaxCell);
    if (v->cell == cell) return IVR_OK;
    CK(v->ctx, cudaSetDevice(v->ctx->device));
    v->cell = cell;
    return setup_bricks(v, v->py, v->px, v->pz, v->overlap);  // grids rebuilt on the new cells
}

int ivr_volume_macrocell(const ivr_volume *v, int *cell)
{
    if (!v || !cell) return IVR_ERR_INVALID;
    *cell = v->cell;
    return IVR_OK;
}

int ivr_volume_quad_bytes(const ivr_volume *v, size_t *bytes)
{
    if (!v || !bytes) return IVR_ERR_INVALID;
    size_t n = 0;
    for (const auto &b : v->bricks)
        if (b.quad) n += quad_bytes(v->dtype, b.lw, b.lh, b.ld);
    *bytes = n;
    return IVR_OK;
}

int ivr_volume_minmax(ivr_volume *v, float *mn, float *mx)
{
    if (!v || !mn || !mx) return v ? fail(v->ctx, IVR_ERR_INVALID, "null output") : IVR_ERR_INVALID;
    ivr_ctx *c = v->ctx;
    if (!v->have_minmax) {
        int parts = minmax_parts();
        CK(c, launch_minmax(v->d_full, v->dtype, (long long) v->w * v->h * v->d, c->d_partial, parts, 0));
        std::vector<float> h(2 * parts);
        CK(c, cudaMemcpy(h.data(), c->d_partial, sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
        float lo = FLT_MAX, hi = -FLT_MAX;
        for (int i = 0; i < parts; i++) {
            lo = fminf(lo, h[2 * i]);
            hi = fmaxf(hi, h[2 * i + 1]);
        }
        v->vmin = lo;
        v->vmax = hi;
        v->have_minmax = true;
    }
    *mn = v->vmin;
    *mx = v->vmax;
    return IVR_OK;
}

int ivr_volume_histogram(ivr_volume *v, int *hist, int hsize)
{
    if (!v || !hist || hsize < 1) return v ? fail(v->ctx, IVR_ERR_INVALID, "bad histogram output") : IVR_ERR_INVALID;
    ivr_ctx *c = v->ctx;
    float mn, mx;
    int rc = ivr_volume_minmax(v, &mn, &mx);
    if (rc) return rc;
    int *d_hist = nullptr;
    rc = dev_alloc(c, sizeof(int) * (size_t) hsize, (void **) &d_hist);
    if (rc) return rc;
    cudaError_t e = launch_histogram(v->d_full, v->dtype, (long long) v->w * v->h * v->d, mn, hsize, d_hist, 0);
    if (e == cudaSuccess) e = cudaMemcpy(hist, d_hist, sizeof(int) * (size_t) hsize, cudaMemcpyDeviceToHost);
    dev_free(c, d_hist, sizeof(int) * (size_t) hsize);
    if (e != cudaSuccess) return cuda_fail(c, e, "histogram");
    return IVR_OK;
}

int ivr_volume_histogram_noalloc(ivr_volume *v, int *hist, int hsize, float *mn, float *mx, void *stream)
{
    if (!v) return IVR_ERR_INVALID;
    ivr_ctx *c = v->ctx;
    if (!hist || !mn || !mx) return fail(c, IVR_ERR_INVALID, "null output");
    if (hsize < 1 || hsize > kNoAllocMaxBins)
        return fail(c, IVR_ERR_INVALID, "hsize %d is outside [1, %d], the bins the allocation-free histogram holds",
                    hsize, kNoAllocMaxBins);
    // the volume's device is made current for the call and the caller's
    // current device is put back afterwards, whatever the outcome
    int prev = -1;
    CK(c, cudaGetDevice(&prev));
    CK(c, cudaSetDevice(c->device));
    float mm[2];
    cudaError_t e = noalloc_histogram(v->d_full, v->dtype, (long long) v->w * v->h * v->d, hsize, hist, mm,
                                      (cudaStream_t) stream);
    cudaError_t r = cudaSetDevice(prev);
    CK(c, e);
    CK(c, r);
    *mn = mm[0];
    *mx = mm[1];
    return IVR_OK;
}

int ivr_tf_create(ivr_ctx *c, ivr_tf **out)
{
    if (!c || !out) return IVR_ERR_INVALID;
    ivr_tf *t = new ivr_tf();
    t->ctx = c;
    *out = t;
    return IVR_OK;
}

int ivr_tf_free(ivr_tf *t)
{
    if (!t) return IVR_ERR_INVALID;
    dev_free(t->ctx, t->d_lut, sizeof(float4) * (size_t) t->cap);
    dev_free(t->ctx, t->d_nzprefix, sizeof(int) * (size_t) (t->cap + 1));
    dev_free(t->ctx, t->d_aprefix, sizeof(double) * (size_t) (t->cap + 1));
    delete t;
    return IVR_OK;
}

int ivr_tf_set_lut(ivr_tf *t, const float *rgba, int n, int off, float scale, int mode)
{
    if (!t) return IVR_ERR_INVALID;
    ivr_ctx *c = t->ctx;
    if (mode < IVR_TF_SEISMIC || mode > IVR_TF_F2B) return fail(c, IVR_ERR_INVALID, "transfer function mode %d", mode);
    if (mode != IVR_TF_RGBBLEND && (!rgba || n < 1)) return fail(c, IVR_ERR_INVALID, "empty LUT");
    if (n > (1 << 24)) return fail(c, IVR_ERR_UNSUPPORTED, "LUT of %d entries", n);
    if (mode != IVR_TF_F2B && scale != 1.0f) return fail(c, IVR_ERR_INVALID, "lut_scale applies to IVR_TF_F2B only");
    if (!(scale > 0.0f)) return fail(c, IVR_ERR_INVALID, "lut_scale must be > 0");
    if (n > t->cap) {
        dev_free(c, t->d_lut, sizeof(float4) * (size_t) t->cap);
        dev_free(c, t->d_nzprefix, sizeof(int) * (size_t) (t->cap + 1));
        dev_free(c, t->d_aprefix, sizeof(double) * (size_t) (t->cap + 1));
        t->d_lut = nullptr;
        t->d_nzprefix = nullptr;
        t->d_aprefix = nullptr;
        t->cap = 0;
        int rc = dev_alloc(c, sizeof(float4) * (size_t) n, (void **) &t->d_lut);
        if (rc) return rc;
        rc = dev_alloc(c, sizeof(int) * (size_t) (n + 1), (void **) &t->d_nzprefix);
        if (rc) return rc;
        rc = dev_alloc(c, sizeof(double) * (size_t) (n + 1), (void **) &t->d_aprefix);
        if (rc) return rc;
        t->cap = n;
    }
    t->n = n;
    t->off = off;
    t->scale = scale;
    t->mode = mode;
    if (n > 0) {
        t->host.assign(rgba, rgba + 4 * (size_t) n);
        std::vector<int> pre((size_t) n + 1, 0);
        std::vector<double> apre((size_t) n + 1, 0.0);
        for (int i = 0; i < n; i++) {
            pre[i + 1] = pre[i] + (rgba[4 * i + 3] != 0.0f ? 1 : 0);
            apre[i + 1] = apre[i] + (double) rgba[4 * i + 3];
        }
        CK(c, cudaMemcpy(t->d_lut, rgba, sizeof(float4) * (size_t) n, cudaMemcpyHostToDevice));
        CK(c, cudaMemcpy(t->d_nzprefix, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice));
        CK(c, cudaMemcpy(t->d_aprefix, apre.data(), sizeof(double) * apre.size(), cudaMemcpyHostToDevice));
    }
    t->serial = ++c->tf_serial;
    return IVR_OK;
}

int ivr_tf_set_colormap(ivr_tf *t, ivr_volume *v, int colormap, int mode)
{
    if (!t || !v) return IVR_ERR_INVALID;
    ivr_ctx *c = t->ctx;
    float mn, mx;
    int rc = ivr_volume_minmax(v, &mn, &mx);
    if (rc) return rc;
    // initvolluts (main.c:1093, 1142, 1158-1179)
    float span = (mx - mn) + 1;
    if (!(span < (float) (1 << 24))) return fail(c, IVR_ERR_UNSUPPORTED, "value range %g needs too large a LUT", span);
    int hsize = (int) span;
    std::vector<float> lut(4 * (size_t) hsize);
    build_colormap(colormap, lut.data(), hsize, mn, mx);
    int off = (int) (mn + 0.5);
    return ivr_tf_set_lut(t, lut.data(), hsize, off, 1.0f, mode);
}

int ivr_tf_get_lut(const ivr_tf *t, float *rgba, int n, int *lut_n, int *lut_off)
{
    if (!t) return IVR_ERR_INVALID;
    if (lut_n) *lut_n = t->n;
    if (lut_off) *lut_off = t->off;
    if (rgba) {
        int m = n < t->n ? n : t->n;
        memcpy(rgba, t->host.data(), sizeof(float) * 4 * (size_t) m);
    }
    return IVR_OK;
}

int ivr_view_create(ivr_ctx *c, ivr_view **out)
{
    if (!c || !out) return IVR_ERR_INVALID;
    ivr_view *v = new ivr_view();
    v->ctx = c;
    int rc = dev_alloc(c, sizeof(unsigned long long), (void **) &v->d_tickets);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(JudgeWords), (void **) &v->d_judge);
    if (rc == IVR_OK && cudaMemset(v->d_judge, 0, sizeof(JudgeWords)) != cudaSuccess) rc = fail(c, IVR_ERR_CUDA, "judge words");
    if (rc) {
        ivr_view_free(v);
        return rc;
    }
    *out = v;
    return IVR_OK;
}

int ivr_view_free(ivr_view *v)
{
    if (!v) return IVR_ERR_INVALID;
    dev_free(v->ctx, v->d_tickets, sizeof(unsigned long long));
    dev_free(v->ctx, v->d_judge, sizeof(JudgeWords));
    dev_free(v->ctx, v->d_judge8, v->judge_bytes);
    for (auto &o : v->tiles) {
        dev_free(v->ctx, o.perm, sizeof(int) * (size_t) v->tile_cap);
        dev_free(v->ctx, o.key, (size_t) v->tile_cap);
        dev_free(v->ctx, o.counts, sizeof(int) * 128);
        if (o.done) cudaEventDestroy(o.done);
        if (o.used) cudaEventDestroy(o.used);
    }
    if (v->order_stream) {
        cudaStreamSynchronize(v->order_stream);
        cudaStreamDestroy(v->order_stream);
    }
    delete v;
    return IVR_OK;
}

int ivr_view_judge_stats(ivr_view *v, ivr_judge_stats *st)
{
    if (!v || !st) return v ? fail(v->ctx, IVR_ERR_INVALID, "null stats") : IVR_ERR_INVALID;
    JudgeWords jw;
    CK(v->ctx, cudaDeviceSynchronize());
    CK(v->ctx, cudaMemcpy(&jw, v->d_judge, sizeof(jw), cudaMemcpyDeviceToHost));
    memset(st, 0, sizeof(*st));
    st->frames = jw.frames;
    st->fallbacks = jw.fallbacks;
    st->pixels = jw.pixels;
    st->worst = jw.worst;
    st->exact_frames = jw.exact_frames;
    return IVR_OK;
}

int ivr_set_view(ivr_view *view, ivr_volume *vol, const ivr_state *st, const ivr_render_params *p)
{
    if (!view) return IVR_ERR_INVALID;
    ivr_ctx *c = view->ctx;
    view->valid = false;
    if (!vol || !st) return fail(c, IVR_ERR_INVALID, "null volume or state");
    int rc = valid_params(c, p);
    if (rc) return rc;
    rc = build_frame(vol->w, vol->h, vol->d, vol->dtype, vol->bricks.data(), (int) vol->bricks.size(), *st, *p,
                     view->f, view->info);
    if (rc) return fail(c, rc, "view set-up failed (window %dx%d, tile %dx%d)", st->winwidth, st->winheight,
                        p->tilew, p->tileh);
    view->vol = vol;
    view->layout = vol->layout;
    view->p = *p;
    view->st = *st;
    view->valid = true;
    return IVR_OK;
}

int ivr_view_info(const ivr_view *view, ivr_frame_info *info)
{
    if (!view || !info || !view->valid) return IVR_ERR_INVALID;
    *info = view->info;
    return IVR_OK;
}

int ivr_render(ivr_view *view, ivr_tf *tf, float *o32, uint8_t *o8, void *stream)
{
    if (!view) return IVR_ERR_INVALID;
    return render_window(view, tf, 0, 0, view->info.vw, view->info.vh, -1, o32, o8, stream);
}

int ivr_render_tile(ivr_view *view, ivr_tf *tf, int x, int y, int w, int h, float *o32, uint8_t *o8, void *stream)
{
    return render_window(view, tf, x, y, w, h, -1, o32, o8, stream);
}

int ivr_render_brick(ivr_view *view, ivr_tf *tf, int brick, float *o32, void *stream)
{
    if (!view) return IVR_ERR_INVALID;
    if (brick < 0 || brick >= view->info.nbricks) return fail(view->ctx, IVR_ERR_INVALID, "brick %d", brick);
    return render_window(view, tf, 0, 0, view->info.vw, view->info.vh, brick, o32, nullptr, stream);
}

int ivr_render_host(ivr_view *view, ivr_volume *vol, ivr_tf *tf, const ivr_state *st, const ivr_render_params *p,
                    uint8_t *host8, void *stream)
{
    if (!view || !host8) return view ? fail(view->ctx, IVR_ERR_INVALID, "null output") : IVR_ERR_INVALID;
    ivr_ctx *c = view->ctx;
    int rc = ivr_set_view(view, vol, st, p);
    if (rc) return rc;
    size_t bytes = (size_t) view->info.vw * view->info.vh * 4;
    // page-locked output: the launch stores the frame there itself
    if (void *direct = host_mapping(host8, bytes)) {
        rc = ivr_render(view, tf, nullptr, (uint8_t *) direct, stream);
        if (rc) return rc;
        CK(c, cudaStreamSynchronize((cudaStream_t) stream));
        return IVR_OK;
    }
    if (bytes > c->frame8_bytes) {
        dev_free(c, c->d_frame8, c->frame8_bytes);
        c->d_frame8 = nullptr;
        c->frame8_bytes = 0;
        rc = dev_alloc(c, bytes, (void **) &c->d_frame8);
        if (rc) return rc;
        c->frame8_bytes = bytes;
    }
    rc = ivr_render(view, tf, nullptr, (uint8_t *) c->d_frame8, stream);
    if (rc) return rc;
    CK(c, cudaMemcpyAsync(host8, c->d_frame8, bytes, cudaMemcpyDeviceToHost, (cudaStream_t) stream));
    CK(c, cudaStreamSynchronize((cudaStream_t) stream));
    return IVR_OK;
}

int ivr_census(ivr_view *view, ivr_tf *tf, unsigned long long *lattice, unsigned long long *executed,
               unsigned long long *touched_bytes, void *stream)
{
    if (!view) return IVR_ERR_INVALID;
    ivr_ctx *c = view->ctx;
    if (!view->valid) return fail(c, IVR_ERR_INVALID, "ivr_set_view has not succeeded on this view");
    if (view->p.preset != IVR_PRESET_CONFIG) return fail(c, IVR_ERR_UNSUPPORTED, "census needs the CONFIG preset");
    ivr_volume *vol = view->vol;
    std::vector<uint8_t *> touched(vol->bricks.size(), nullptr);
    int rc = IVR_OK;
    for (size_t k = 0; k < touched.size() && rc == IVR_OK; k++) {
        rc = dev_alloc(c, mc_cells(vol->bricks[k]), (void **) &touched[k]);
        if (rc == IVR_OK && cudaMemset(touched[k], 0, mc_cells(vol->bricks[k])) != cudaSuccess) rc = IVR_ERR_CUDA;
    }
    unsigned long long cnt[2] = {0, 0};
    size_t bytes = 0;
    if (rc == IVR_OK && cudaMemset(c->d_counters, 0, sizeof(unsigned long long) * 4) != cudaSuccess) rc = IVR_ERR_CUDA;
    if (rc == IVR_OK) rc = render_window(view, tf, 0, 0, view->info.vw, view->info.vh, -1, nullptr, nullptr, stream, &touched);
    if (rc == IVR_OK && cudaStreamSynchronize((cudaStream_t) stream) != cudaSuccess) rc = IVR_ERR_CUDA;
    if (rc == IVR_OK && cudaMemcpy(cnt, c->d_counters, sizeof(cnt), cudaMemcpyDeviceToHost) != cudaSuccess) rc = IVR_ERR_CUDA;
    for (size_t k = 0; k < touched.size() && rc == IVR_OK; k++) {
        const HostBrick &b = vol->bricks[k];
        std::vector<uint8_t> h(mc_cells(b));
        if (cudaMemcpy(h.data(), touched[k], h.size(), cudaMemcpyDeviceToHost) != cudaSuccess) { rc = IVR_ERR_CUDA; break; }
        for (int cz = 0; cz < b.mcz; cz++)
            for (int cy = 0; cy < b.mcy; cy++)
                for (int cx = 0; cx < b.mcx; cx++)
                    if (h[((size_t) cz * b.mcy + cy) * b.mcx + cx])
                        bytes += (size_t) std::min(b.cell, b.lw - cx * b.cell) *
                                 std::min(b.cell, b.lh - cy * b.cell) * std::min(b.cell, b.ld - cz * b.cell) *
                                 dtype_size(vol->dtype);
    }
    for (size_t k = 0; k < touched.size(); k++)
        if (touched[k]) dev_free(c, touched[k], mc_cells(vol->bricks[k]));
    cudaMemset(c->d_counters, 0, sizeof(unsigned long long) * 4);
    if (rc == IVR_ERR_CUDA) return fail(c, rc, "census launch failed");
    if (rc) return rc;
    if (lattice) *lattice = cnt[1];
    if (executed) *executed = cnt[0];
    if (touched_bytes) *touched_bytes = bytes;
    return IVR_OK;
}

// --- batches -----------------------------------------------------------
namespace {
size_t batch_bytes(int cap) { return sizeof(BatchHeader) + sizeof(BatchItem) * (size_t) cap; }
BatchHeader *batch_hdr(ivr_batch *b) { return (BatchHeader *) b->h_buf; }
BatchItem *batch_items(ivr_batch *b) { return (BatchItem *) ((char *) b->h_buf + sizeof(BatchHeader)); }

int batch_wait(ivr_batch *b)
{
    if (b->pending) {
        CK(b->ctx, cudaEventSynchronize(b->done));
        b->pending = false;
    }
    return IVR_OK;
}

// tile numbering for the batch's warp-tile width
void batch_layout(ivr_batch *b)
{
    const int tw = batch_variant_tile_w(b->variant), th = 32 / tw;
    long long t = 0;
    BatchItem *it = batch_items(b);
    for (int i = 0; i < b->n; i++) {
        it[i].tile0 = t;
        it[i].tiles_x = (it[i].f.out_w + tw - 1) / tw;
        t += (long long) it[i].tiles_x * ((it[i].f.out_h + th - 1) / th);
    }
    batch_hdr(b)->nitems = b->n;
    batch_hdr(b)->total_tiles = t;
}

int batch_launch(ivr_batch *b, cudaStream_t s, bool graph)
{
    ivr_ctx *c = b->ctx;
    if (!graph) {
        CK(c, cudaMemsetAsync(b->d_ticket, 0, sizeof(unsigned long long), s));
        CK(c, cudaMemcpyAsync(b->d_buf, b->h_buf, batch_bytes(b->n), cudaMemcpyHostToDevice, s));
        CK(c, launch_batch(b->dtype, b->variant, (const BatchHeader *) b->d_buf,
                           (const BatchItem *) ((char *) b->d_buf + sizeof(BatchHeader)), b->d_ticket, s));
        return IVR_OK;
    }
    const int v = b->variant;
    if (!b->graph[v]) {
        // capture once: ticket reset, descriptor upload (the whole staging
        // area, so any later batch of up to cap frames replays unchanged),
        // the persistent launch
        cudaStream_t cs;
        CK(c, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->d_ticket, 0, sizeof(unsigned long long), cs);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_buf, b->h_buf, batch_bytes(b->cap), cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess)
            e = launch_batch(b->dtype, v, (const BatchHeader *) b->d_buf,
                             (const BatchItem *) ((char *) b->d_buf + sizeof(BatchHeader)), b->d_ticket, cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[v], g, 0);
        if (e2 == cudaSuccess) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) {
            b->graph[v] = nullptr;
            return cuda_fail(c, e, "batch graph capture");
        }
    }
    CK(c, cudaGraphLaunch(b->graph[v], s));
    return IVR_OK;
}
}  // namespace

int ivr_batch_create(ivr_ctx *c, int max_frames, ivr_batch **out)
{
    if (!c || !out) return IVR_ERR_INVALID;
    *out = nullptr;
    if (max_frames < 1 || max_frames > 4096) return fail(c, IVR_ERR_INVALID, "batch capacity %d", max_frames);
    ivr_batch *b = new ivr_batch();
    b->ctx = c;
    b->cap = max_frames;
    b->buf_bytes = batch_bytes(max_frames);
    cudaError_t e = cudaMallocHost(&b->h_buf, b->buf_bytes);
    if (e != cudaSuccess) {
        delete b;
        return fail(c, IVR_ERR_NOMEM, "pinned staging for %d frames: %s", max_frames, cudaGetErrorString(e));
    }
    memset(b->h_buf, 0, b->buf_bytes);
    int rc = dev_alloc(c, b->buf_bytes, &b->d_buf);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(unsigned long long), (void **) &b->d_ticket);
    if (rc == IVR_OK && cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess) rc = IVR_ERR_CUDA;
    if (rc) {
        ivr_batch_free(b);
        return rc;
    }
    *out = b;
    return IVR_OK;
}

int ivr_batch_free(ivr_batch *b)
{
    if (!b) return IVR_ERR_INVALID;
    batch_wait(b);
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    if (b->done) cudaEventDestroy(b->done);
    dev_free(b->ctx, b->d_buf, b->buf_bytes);
    dev_free(b->ctx, b->d_ticket, sizeof(unsigned long long));
    if (b->h_buf) cudaFreeHost(b->h_buf);
    delete b;
    return IVR_OK;
}

int ivr_batch_clear(ivr_batch *b)
{
    if (!b) return IVR_ERR_INVALID;
    int rc = batch_wait(b);
    if (rc) return rc;
    b->n = 0;
    b->dtype = -1;
    b->grids.clear();
    b->clock0 = b->ctx->grid_clock + 1;
    return IVR_OK;
}

int ivr_batch_add(ivr_batch *b, ivr_view *view, ivr_tf *tf, float *rgba32_dev, uint8_t *rgba8_dev)
{
    if (!b) return IVR_ERR_INVALID;
    ivr_ctx *c = b->ctx;
    if (!view || view->ctx != c) return fail(c, IVR_ERR_INVALID, "view missing or from another context");
    if (!view->valid) return fail(c, IVR_ERR_INVALID, "ivr_set_view has not succeeded on this view");
    if (view->p.preset != IVR_PRESET_CONFIG) return fail(c, IVR_ERR_UNSUPPORTED, "batches render the CONFIG preset");
    if (b->n == b->cap) return fail(c, IVR_ERR_INVALID, "batch is full (%d frames)", b->cap);
    if (b->dtype >= 0 && view->vol->dtype != b->dtype)
        return fail(c, IVR_ERR_INVALID, "one batch renders volumes of one dtype");
    int rc = batch_wait(b);
    if (rc) return rc;
    BatchItem &it = batch_items(b)[b->n];
    // the frame descriptor; a TF new to the volume has its distance field
    // built here on the legacy stream, and ivr_batch_render makes its stream
    // wait for that build on the device
    bool built = false;
    ivr_volume::TfGrid *grid = nullptr;
    if (b->n == 0) b->clock0 = c->grid_clock + 1;
    rc = frame_for(view, tf, 0, 0, view->info.vw, view->info.vh, -1, 0, it.f, &grid, b->clock0, &built);
    if (rc) return rc;
    (void) built;  // the render's stream waits for the build on the device
    if (grid) b->grids.push_back(grid);
    it.out32 = (float4 *) rgba32_dev;
    it.out8 = (uchar4 *) rgba8_dev;
    b->dtype = view->vol->dtype;
    b->n++;
    return IVR_OK;
}

int ivr_batch_render(ivr_batch *b, int use_graph, void *stream)
{
    if (!b) return IVR_ERR_INVALID;
    if (b->n == 0) return IVR_OK;
    batch_layout(b);
    for (auto *g : b->grids) CK(b->ctx, cudaStreamWaitEvent((cudaStream_t) stream, g->built, 0));
    int rc = batch_launch(b, (cudaStream_t) stream, use_graph != 0);
    if (rc) return rc;
    for (auto *g : b->grids) CK(b->ctx, cudaEventRecord(g->ev, (cudaStream_t) stream));
    CK(b->ctx, cudaEventRecord(b->done, (cudaStream_t) stream));
    b->pending = true;
    return IVR_OK;
}

int ivr_batch_autotune(ivr_batch *b, void *stream, int *variant, float *ms_per_variant)
{
    if (!b) return IVR_ERR_INVALID;
    ivr_ctx *c = b->ctx;
    if (b->n == 0) return fail(c, IVR_ERR_INVALID, "autotune needs a filled batch");
    cudaStream_t s = (cudaStream_t) stream;
    for (auto *g : b->grids) CK(c, cudaStreamWaitEvent(s, g->built, 0));
    cudaEvent_t e0, e1;
    CK(c, cudaEventCreate(&e0));
    CK(c, cudaEventCreate(&e1));
    int best = 0;
    float best_ms = 0.0f;
    for (int v = 0; v < kBatchVariants; v++) {
        b->variant = v;
        int rc = batch_wait(b);
        batch_layout(b);
        if (rc == IVR_OK) rc = batch_launch(b, s, false);  // warm-up
        if (rc == IVR_OK && cudaEventRecord(e0, s) != cudaSuccess) rc = IVR_ERR_CUDA;
        for (int r = 0; r < 3 && rc == IVR_OK; r++) rc = batch_launch(b, s, false);
        if (rc == IVR_OK && cudaEventRecord(e1, s) != cudaSuccess) rc = IVR_ERR_CUDA;
        float ms = 0.0f;
        if (rc == IVR_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            rc = IVR_ERR_CUDA;
        if (rc) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc == IVR_ERR_CUDA ? fail(c, rc, "autotune timing failed") : rc;
        }
        ms /= 3.0f;
        if (ms_per_variant) ms_per_variant[v] = ms;
        if (v == 0 || ms < best_ms) {
            best = v;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->variant = best;
    if (variant) *variant = best;
    return IVR_OK;
}

int ivr_batch_set_variant(ivr_batch *b, int variant)
{
    if (!b) return IVR_ERR_INVALID;
    if (variant < 0 || variant >= kBatchVariants) return fail(b->ctx, IVR_ERR_INVALID, "variant %d", variant);
    b->variant = variant;
    return IVR_OK;
}

int ivr_sample_peak(ivr_ctx *c, int dtype, double *gsamples_per_s, void *stream)
{
    return ivr_sample_peak_layout(c, dtype, IVR_SAMPLER_QUADS, gsamples_per_s, nullptr, stream);
}

int ivr_sample_peak_layout(ivr_ctx *c, int dtype, int layout, double *gsamples_per_s, double *max_abs_err,
                           void *stream)
{
    if (!c || !gsamples_per_s) return c ? fail(c, IVR_ERR_INVALID, "null output") : IVR_ERR_INVALID;
    if (dtype < IVR_U8 || dtype > IVR_F32) return fail(c, IVR_ERR_INVALID, "unknown dtype %d", dtype);
    if (layout < IVR_SAMPLER_QUADS || layout > IVR_SAMPLER_TEX_LINEAR)
        return fail(c, IVR_ERR_INVALID, "unknown sampler layout %d", layout);
    cudaStream_t s = (cudaStream_t) stream;
    // a 64^3 brick of pseudo-random values over the LUT's range, a 256-entry
    // ramp LUT, world units = voxels
    const int n = 64;
    const size_t nvox = (size_t) n * n * n, esz = dtype_size(dtype);
    std::vector<unsigned char> host(nvox * esz);
    unsigned r = 12345u;
    for (size_t i = 0; i < nvox; i++) {
        r = r * 1664525u + 1013904223u;
        const float v = (float) (r >> 8) / 16777216.0f;
        if (dtype == IVR_U8) host[i] = (unsigned char) (v * 255.0f);
        else if (dtype == IVR_U16) { const uint16_t u = (uint16_t) (v * 65535.0f); memcpy(&host[2 * i], &u, 2); }
        else { const float f = v * 255.0f; memcpy(&host[4 * i], &f, 4); }
    }
    std::vector<float4> lut(256);
    for (int i = 0; i < 256; i++) lut[i] = make_float4(i / 255.0f, 0.5f, 1.0f - i / 255.0f, 0.02f * (i / 255.0f));
    const int threads = sample_peak_threads();
    void *d_vol = nullptr, *d_lut = nullptr, *d_out = nullptr, *d_quad = nullptr, *d_err = nullptr;
    const bool quads = layout == IVR_SAMPLER_QUADS, tex = layout >= IVR_SAMPLER_TEX_POINT;
    const size_t qb = quads ? quad_bytes(dtype, n, n, n) : 0;
    int rc = dev_alloc(c, nvox * esz, &d_vol);
    if (rc == IVR_OK && quads) rc = dev_alloc(c, qb, &d_quad);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(float4) * 256, &d_lut);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(float4) * (size_t) threads, &d_out);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(unsigned), &d_err);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaArray_t arr = nullptr;
    SamplerTex st{0, 0, 1.0f};
    if (rc == IVR_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        rc = fail(c, IVR_ERR_CUDA, "events");
    if (rc == IVR_OK) {
        FrameDesc f{};
        f.dtype = dtype;
        f.nb = 1;
        f.alpha = 1.0f;
        f.lut = (const float4 *) d_lut;
        f.lut_n = 256;
        f.lut_scale = dtype == IVR_U16 ? 256.0f / 65536.0f : 1.0f;
        DevBrick &b = f.b[0];
        b.data = d_vol;
        b.quad = d_quad;  // null: the sampler reads the brick itself
        b.nx = b.ny = b.nz = n;
        b.icx = b.icy = b.icz = 1.0f;
        b.vwx = b.vwy = b.vwz = 1.0f;
        b.cshift = 4;
        const int steps = 4096;
        long long samples = 0;
        float ms = 0.0f;
        cudaError_t e = cudaMemcpy(d_vol, host.data(), host.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && quads) e = launch_quads(d_vol, dtype, n, n, n, d_quad, s);
        if (e == cudaSuccess && tex) {
            // the brick as a 3D array; element reads for the point fetches,
            // filtered reads (normalised for integer types) for the other
            const cudaChannelFormatDesc cd = dtype == IVR_U8    ? cudaCreateChannelDesc<unsigned char>()
                                             : dtype == IVR_U16 ? cudaCreateChannelDesc<unsigned short>()
                                                                : cudaCreateChannelDesc<float>();
            e = cudaMalloc3DArray(&arr, &cd, make_cudaExtent(n, n, n));
            cudaMemcpy3DParms cp = {};
            cp.srcPtr = make_cudaPitchedPtr(d_vol, n * esz, n, n);
            cp.dstArray = arr;
            cp.extent = make_cudaExtent(n, n, n);
            cp.kind = cudaMemcpyDeviceToDevice;
            if (e == cudaSuccess) e = cudaMemcpy3D(&cp);
            cudaResourceDesc rd = {};
            rd.resType = cudaResourceTypeArray;
            rd.res.array.array = arr;
            cudaTextureDesc td = {};
            td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
            td.normalizedCoords = 0;
            td.filterMode = cudaFilterModePoint;
            td.readMode = cudaReadModeElementType;
            if (e == cudaSuccess) e = cudaCreateTextureObject(&st.point, &rd, &td, nullptr);
            td.filterMode = cudaFilterModeLinear;
            td.readMode = dtype == IVR_F32 ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
            st.scale = dtype == IVR_U8 ? 255.0f : dtype == IVR_U16 ? 65535.0f : 1.0f;
            if (e == cudaSuccess) e = cudaCreateTextureObject(&st.linear, &rd, &td, nullptr);
        }
        if (e == cudaSuccess) e = cudaMemcpy(d_lut, lut.data(), sizeof(float4) * 256, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)  // warm-up
            e = launch_sample_peak(f, layout, st, steps, (float4 *) d_out, &samples, nullptr, s);
        if (e == cudaSuccess) e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) e = launch_sample_peak(f, layout, st, steps, (float4 *) d_out, &samples, nullptr, s);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        unsigned err_bits = 0;
        if (max_abs_err) {
            if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(unsigned), s);
            if (e == cudaSuccess) e = launch_sample_peak(f, layout, st, 0, nullptr, &samples, (unsigned *) d_err, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&err_bits, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
        if (e != cudaSuccess) {
            rc = cuda_fail(c, e, "sample-rate roofline");
        } else {
            *gsamples_per_s = (double) samples / (ms * 1e-3) / 1e9;
            if (max_abs_err) {
                float v;
                memcpy(&v, &err_bits, sizeof(v));
                *max_abs_err = v;
            }
        }
    }
    if (st.point) cudaDestroyTextureObject(st.point);
    if (st.linear) cudaDestroyTextureObject(st.linear);
    if (arr) cudaFreeArray(arr);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dev_free(c, d_vol, nvox * esz);
    dev_free(c, d_quad, qb);
    dev_free(c, d_lut, sizeof(float4) * 256);
    dev_free(c, d_out, sizeof(float4) * (size_t) threads);
    dev_free(c, d_err, sizeof(unsigned));
    return rc;
}

int ivr_composite(ivr_ctx *c, float *tilebuf, const float *rcolorbuf, int num, int w, int h, void *stream)
{
    if (!c) return IVR_ERR_INVALID;
    if (!tilebuf || (num > 0 && !rcolorbuf) || num < 0 || w < 0 || h < 0)
        return fail(c, IVR_ERR_INVALID, "bad composite arguments");
    if (num == 0 || w == 0 || h == 0) return IVR_OK;
    CK(c, launch_composite(tilebuf, rcolorbuf, num, (long long) w * h, (cudaStream_t) stream));
    return IVR_OK;
}

int ivr_quantize(ivr_ctx *c, const float *in, uint8_t *out, long long n, void *stream)
{
    if (!c) return IVR_ERR_INVALID;
    if (n < 0 || (n > 0 && (!in || !out))) return fail(c, IVR_ERR_INVALID, "bad quantize arguments");
    if (n == 0) return IVR_OK;
    CK(c, launch_quantize(in, out, n, (cudaStream_t) stream));
    return IVR_OK;
}

int ivr_copy(ivr_ctx *c, void *dst, const void *src, size_t bytes, void *stream)
{
    if (!c) return IVR_ERR_INVALID;
    if (bytes > 0 && (!dst || !src)) return fail(c, IVR_ERR_INVALID, "null copy buffer");
    if (bytes == 0) return IVR_OK;
    CK(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t) stream));
    return IVR_OK;
}

int ivr_stream_wait(ivr_ctx *c, void *stream)
{
    if (!c) return IVR_ERR_INVALID;
    CK(c, cudaStreamSynchronize((cudaStream_t) stream));
    return IVR_OK;
}

}  // extern "C"
