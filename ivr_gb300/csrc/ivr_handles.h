// ivr_handles.h -- the opaque handles of the C ABI and the host helpers the
// API translation units share.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "ivr_frame.h"

struct ivr_ctx {
    int device = 0;
    size_t budget = 0;   // 0 = unlimited
    size_t used = 0;
    std::string err;
    unsigned long long *d_counters = nullptr;
    float *d_partial = nullptr;  // min/max partials
    uchar4 *d_frame8 = nullptr;  // ivr_render_host staging
    size_t frame8_bytes = 0;
    unsigned tf_serial = 0;
    unsigned long long grid_clock = 0;  // recency of the per-TF distance fields
};

struct ivr_volume {
    ivr_ctx *ctx = nullptr;
    int w = 0, h = 0, d = 0, dtype = 0;
    void *d_full = nullptr;
    size_t full_bytes = 0;
    std::vector<ivr::HostBrick> bricks;
    int py = 1, px = 1, pz = 1, overlap = 0;
    bool quads = true;  // keep corner-packed copies of the bricks (HostBrick::quad)
    int cell = ivr::kCell;  // macrocell edge in voxels (ivr_volume_set_macrocell)
    unsigned layout = 0;    // counts brick rebuilds: views set before one re-derive their frame
    bool have_minmax = false;
    float vmin = 0.0f, vmax = 0.0f;
    // macrocell distance fields, one set per transfer function in use
    // (keyed by TF serial, whether the opacity scale is zero and whether the
    // transparent cells are the exact ones or the learned predictor's)
    struct TfGrid {
        unsigned serial;
        int zero_alpha;
        int learned;
        unsigned mlp_serial;          // learned: the predictor's parameter version
        unsigned long long last_use;  // ctx grid_clock
        std::vector<uint8_t *> dist;  // per brick
        std::vector<uint8_t *> opac;  // per brick: DevBrick::opac (the exact rule's)
        cudaEvent_t ev;               // after the last launch that read it
        cudaEvent_t built;            // after its build
        // learned grids: d_bad (device) is nonzero once a judged frame was
        // above the tolerance; launches read it and render with the exact
        // grid.  h_reject (host-mapped, device address d_reject) is set with
        // it so the host can stop using the grid.
        int *d_bad;
        int *h_reject;
        int *d_reject;
        bool rejected;                // host has seen it: render with the exact grid
    };
    std::vector<TfGrid *> grids;
    // learned skipping: the attached predictor, its margin, and per brick the
    // 8-bin value histogram of every macrocell (built on first use)
    ivr_mlp *mlp = nullptr;
    float mlp_margin = 0.0f;
    bool mlp_certify = true;
    unsigned long long *d_lstats = nullptr;  // learned-grid cell counts (ivr_volume_learned_stats)
    std::vector<float *> cell_hist;
};
constexpr size_t kMaxTfGrids = 128;

struct ivr_tf {
    ivr_ctx *ctx = nullptr;
    int n = 0, off = 0, mode = IVR_TF_SEISMIC;
    float scale = 1.0f;
    float4 *d_lut = nullptr;
    int *d_nzprefix = nullptr;
    double *d_aprefix = nullptr;  // prefix sums of the entries' opacities
    int cap = 0;
    std::vector<float> host;
    unsigned serial = 0;
};

struct ivr_view {
    ivr_ctx *ctx = nullptr;
    ivr_volume *vol = nullptr;
    unsigned long long *d_tickets = nullptr;  // tile tickets of CONFIG launches
    unsigned long long ticket_base = 0;
    bool tickets_dirty = true;
    ivr_render_params p{};
    ivr_state st{};
    bool valid = false;
    unsigned layout = 0;   // the volume's brick layout the frame was derived for
    ivr::FrameDesc f{};
    ivr_frame_info info{};
    // learned-skip judge: the per-frame verdict words and running totals,
    // and the scratch of the judged tiles' exact re-march
    int *d_judge = nullptr;                 // ivr::JudgeWords
    uchar4 *d_judge8 = nullptr;
    size_t judge_bytes = 0;
    unsigned long long judge_frame = 0;     // rotates the sampled tiles
    // IVR_TILES_COST: two slots of the tile permutation and its scratch
    // (tile_cap tiles each), used by alternate frames.  A frame's order is
    // built on order_stream, so that it runs in the tail of the launch
    // before it; `used` follows the launches that read the slot.
    struct TileOrder {
        int *perm = nullptr;
        uint8_t *key = nullptr;
        int *counts = nullptr;          // 128 ints
        cudaEvent_t done = nullptr;     // the permutation is written
        cudaEvent_t used = nullptr;     // its readers are done (when recorded)
        bool used_recorded = false;
    };
    TileOrder tiles[2];
    int tile_slot = 0;
    long long tile_cap = 0;
    cudaStream_t order_stream = nullptr;
};

struct ivr_batch {
    ivr_ctx *ctx = nullptr;
    int cap = 0, n = 0, dtype = -1;
    int variant = 0;
    void *h_buf = nullptr;  // pinned: BatchHeader then cap BatchItems
    void *d_buf = nullptr;
    size_t buf_bytes = 0;
    unsigned long long *d_ticket = nullptr;
    cudaEvent_t done = nullptr;  // after the last render: the staging may be refilled
    bool pending = false;
    cudaGraphExec_t graph[ivr::kBatchVariants] = {};
    cudaStream_t graph_stream[ivr::kBatchVariants] = {};
    std::vector<ivr_volume::TfGrid *> grids;  // read by the frames in the batch
    unsigned long long clock0 = 0;           // grid_clock when it was cleared
};

namespace ivr {

// records the message in the context and returns code
int fail(ivr_ctx *c, int code, const char *fmt, ...);
int cuda_fail(ivr_ctx *c, cudaError_t e, const char *what);

#define CK(ctx, call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return ivr::cuda_fail((ctx), e_, #call); \
    } while (0)

// device memory counted against the context's HBM budget
int dev_alloc(ivr_ctx *c, size_t bytes, void **p);
void dev_free(ivr_ctx *c, void *p, size_t bytes);

size_t brick_bytes(const ivr_volume *v, const HostBrick &b);
// the device address of n bytes of page-locked host memory at p mapped as
// one range, or null (pageable memory, or not one mapping)
void *host_mapping(void *p, size_t n);
inline size_t mc_cells(const HostBrick &b) { return (size_t) b.mcx * b.mcy * b.mcz; }

// learned skipping (ivr_learn.cpp): the predictor's parameter version
// (changes whenever its parameters do)
unsigned mlp_serial(const ivr_mlp *m);
// writes the learned distance field of every brick of v for tf into dist
// on s (certified cell by cell when the volume asks for that)
int learned_fields(ivr_volume *v, const ivr_tf *tf, const std::vector<uint8_t *> &dist, cudaStream_t s);
// frees the per-cell histograms (volume freed or re-bricked)
void learned_release(ivr_volume *v);
// drops the volume's learned grids (waits for the device)
void drop_learned_grids(ivr_volume *v);

}  // namespace ivr
