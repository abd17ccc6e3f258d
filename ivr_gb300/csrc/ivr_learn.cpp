// ivr_learn.cpp -- learned empty-space skipping: the predictor handle, its
// training set and training loop (Adam over shuffled mini-batches, every
// step on the device), the margin calibration, and the learned distance
// fields the march reads.
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <random>
#include <vector>

#include "ivr_handles.h"
#include "ivr_mlp.h"

using namespace ivr;

struct ivr_mlp {
    ivr_ctx *ctx = nullptr;
    unsigned long long seed = 0;
    unsigned serial = 0;            // parameter version
    float *d_p = nullptr;           // FP32 master parameters
    float *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr;  // Adam moments, gradient
    void *d_w1t = nullptr, *d_w2t = nullptr, *d_w2 = nullptr;  // BF16 operand copies
    int step = 0;                   // Adam steps taken
    // training set: features, bounds, predictions (calibration), shuffle
    uint16_t *d_X = nullptr;
    float *d_T = nullptr, *d_Y = nullptr;
    long long n = 0, cap = 0;
    int *d_idx = nullptr;
    float *d_loss = nullptr;
    long long loss_cap = 0;
    float *d_knots = nullptr;  // the knots of the TF whose learned grid is being built
    int *d_key = nullptr;
    int *d_status = nullptr;  // tensor-core status word (kMlpTcTimeout): training, inference, grids
    unsigned long long *d_counts = nullptr;
    cudaEvent_t scratch_ev = nullptr;  // after the last use of d_knots
};

namespace {

constexpr size_t kParamBytes = sizeof(float) * kMlpParams;
constexpr size_t kBf16Bytes = 2;
constexpr char kMagic[8] = {'I', 'V', 'R', 'M', 'L', 'P', '0', '1'};

MlpDev dev_of(const ivr_mlp *m)
{
    MlpDev w;
    w.w1t = m->d_w1t;
    w.w2t = m->d_w2t;
    w.w2 = m->d_w2;
    w.b1 = m->d_p + kOffB1;
    w.b2 = m->d_p + kOffB2;
    w.w3 = m->d_p + kOffW3;
    w.b3 = m->d_p + kOffB3;
    w.status = m->d_status;
    return w;
}

// new parameters: padding rows of W1 cleared, BF16 copies packed, Adam reset
int upload(ivr_mlp *m, std::vector<float> p)
{
    for (int f = kMlpFeatures; f < kMlpIn; f++)
        for (int u = 0; u < kMlpHidden; u++) p[kOffW1 + f * kMlpHidden + u] = 0.0f;
    ivr_ctx *c = m->ctx;
    CK(c, cudaMemcpy(m->d_p, p.data(), kParamBytes, cudaMemcpyHostToDevice));
    CK(c, cudaMemset(m->d_m, 0, kParamBytes));
    CK(c, cudaMemset(m->d_v, 0, kParamBytes));
    CK(c, mlp_pack(m->d_p, m->d_w1t, m->d_w2t, m->d_w2, 0));
    CK(c, cudaDeviceSynchronize());
    m->step = 0;
    m->serial++;
    return IVR_OK;
}

// grows a device array to hold `need` elements of `elem` bytes, keeping the
// first `keep` elements
int grow(ivr_ctx *c, void **p, long long *cap, long long need, size_t elem, long long keep)
{
    if (need <= *cap) return IVR_OK;
    long long nc = std::max(need, *cap * 2);
    void *q = nullptr;
    int rc = dev_alloc(c, (size_t) nc * elem, &q);
    if (rc) return rc;
    if (keep > 0) CK(c, cudaMemcpy(q, *p, (size_t) keep * elem, cudaMemcpyDeviceToDevice));
    dev_free(c, *p, (size_t) *cap * elem);
    *p = q;
    *cap = nc;
    return IVR_OK;
}

long long volume_cells(const ivr_volume *v)
{
    long long n = 0;
    for (const auto &b : v->bricks) n += (long long) mc_cells(b);
    return n;
}

// the volume's range and the per-cell histograms of every brick
int ensure_cell_hist(ivr_volume *v, cudaStream_t s)
{
    if (!v->cell_hist.empty()) return IVR_OK;
    float mn, mx;
    int rc = ivr_volume_minmax(v, &mn, &mx);
    if (rc) return rc;
    std::vector<float *> h(v->bricks.size(), nullptr);
    for (size_t k = 0; k < v->bricks.size() && rc == IVR_OK; k++) {
        const HostBrick &b = v->bricks[k];
        rc = dev_alloc(v->ctx, mc_cells(b) * 8 * sizeof(float), (void **) &h[k]);
        if (rc == IVR_OK && mlp_cell_hist(b.data, v->dtype, b.lw, b.lh, b.ld, b.cell, b.mcx, b.mcy, b.mcz, mn, mx, h[k], s) !=
                                cudaSuccess)
            rc = fail(v->ctx, IVR_ERR_CUDA, "cell histogram launch");
    }
    if (rc) {
        for (size_t k = 0; k < h.size(); k++)
            if (h[k]) dev_free(v->ctx, h[k], mc_cells(v->bricks[k]) * 8 * sizeof(float));
        return rc;
    }
    v->cell_hist = h;
    return IVR_OK;
}

int check_tf(ivr_ctx *c, const ivr_tf *tf)
{
    if (!tf) return fail(c, IVR_ERR_INVALID, "null transfer function");
    if (tf->n < 1 || !tf->d_lut) return fail(c, IVR_ERR_INVALID, "transfer function has no LUT");
    return IVR_OK;
}

// features (and bounds) of every cell of every brick, rows from X (and T)
int features(ivr_mlp *m, ivr_volume *v, const ivr_tf *tf, uint16_t *X, float *T, cudaStream_t s)
{
    ivr_ctx *c = m->ctx;
    int rc = ensure_cell_hist(v, s);
    if (rc) return rc;
    CK(c, mlp_tf_knots(tf->d_lut, tf->n, m->d_knots, s));
    long long off = 0;
    for (size_t k = 0; k < v->bricks.size(); k++) {
        const HostBrick &b = v->bricks[k];
        const int ncell = (int) mc_cells(b);
        CK(c, mlp_cell_features(b.mc_minmax, v->cell_hist[k], ncell, v->vmin, v->vmax, m->d_knots, tf->d_lut, tf->n,
                                tf->off, tf->scale, X + off * kMlpIn, T ? T + off : nullptr, s));
        off += ncell;
    }
    return IVR_OK;
}

}  // namespace

namespace {

// splitmix64: the training order's random stream (seeded per predictor)
struct SplitMix {
    uint64_t x;
    uint64_t next()
    {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    // uniform in [0, bound), bound < 2^32: the multiply-shift reduction with
    // rejection of the biased low range (Lemire)
    uint32_t below(uint32_t bound)
    {
        uint64_t m = (next() >> 32) * (uint64_t) bound;
        uint32_t lo = (uint32_t) m;
        if (lo < bound) {
            const uint32_t t = (uint32_t) (-bound) % bound;
            while (lo < t) {
                m = (next() >> 32) * (uint64_t) bound;
                lo = (uint32_t) m;
            }
        }
        return (uint32_t) (m >> 32);
    }
};

// Fisher-Yates over a[0..n)
void shuffle_rows(int *a, size_t n, SplitMix &rng)
{
    for (size_t i = n; i > 1; i--) {
        const size_t j = rng.below((uint32_t) i);
        std::swap(a[i - 1], a[j]);
    }
}

}  // namespace

unsigned ivr::mlp_serial(const ivr_mlp *m) { return m->serial; }

void ivr::learned_release(ivr_volume *v)
{
    for (size_t k = 0; k < v->cell_hist.size(); k++)
        if (v->cell_hist[k]) dev_free(v->ctx, v->cell_hist[k], mc_cells(v->bricks[k]) * 8 * sizeof(float));
    v->cell_hist.clear();
}

// Per brick: one launch for the features, the network and the certified
// flags, then the distance transform.  The predictor's knot scratch is
// shared by every volume it is attached to, so builds are ordered on the
// device through its event.
int ivr::learned_fields(ivr_volume *v, const ivr_tf *tf, const std::vector<uint8_t *> &dist, cudaStream_t s)
{
    ivr_mlp *m = v->mlp;
    ivr_ctx *c = v->ctx;
    int rc = check_tf(c, tf);
    if (rc) return rc;
    rc = ensure_cell_hist(v, s);
    if (rc) return rc;
    CK(c, cudaStreamWaitEvent(s, m->scratch_ev, 0));
    CK(c, mlp_tf_knots(tf->d_lut, tf->n, m->d_knots, s));
    const MlpDev w = dev_of(m);
    for (size_t k = 0; k < v->bricks.size(); k++) {
        const HostBrick &b = v->bricks[k];
        MlpGridArgs g{};
        g.mc = b.mc_minmax;
        g.hist = v->cell_hist[k];
        g.knots = m->d_knots;
        g.ncell = (int) mc_cells(b);
        g.vmin = v->vmin;
        g.vmax = v->vmax;
        g.margin = v->mlp_margin;
        g.nzprefix = tf->d_nzprefix;
        g.lut_n = tf->n;
        g.lut_off = tf->off;
        g.lut_scale = tf->scale;
        g.certify = v->mlp_certify ? 1 : 0;
        g.dist = dist[k];
        g.stats = v->d_lstats;
        CK(c, mlp_learned_grid_tc(w, g, s));
        CK(c, launch_dist_transform(dist[k], b.mcx, b.mcy, b.mcz, s));
    }
    CK(c, cudaEventRecord(m->scratch_ev, s));
    return IVR_OK;
}

extern "C" {

int ivr_mlp_free(ivr_mlp *m)
{
    if (!m) return IVR_ERR_INVALID;
    ivr_ctx *c = m->ctx;
    cudaDeviceSynchronize();
    dev_free(c, m->d_p, kParamBytes);
    dev_free(c, m->d_m, kParamBytes);
    dev_free(c, m->d_v, kParamBytes);
    dev_free(c, m->d_grad, kParamBytes);
    dev_free(c, m->d_w1t, (size_t) kMlpHidden * kMlpIn * kBf16Bytes);
    dev_free(c, m->d_w2t, (size_t) kMlpHidden * kMlpHidden * kBf16Bytes);
    dev_free(c, m->d_w2, (size_t) kMlpHidden * kMlpHidden * kBf16Bytes);
    dev_free(c, m->d_X, (size_t) m->cap * kMlpIn * kBf16Bytes);
    dev_free(c, m->d_T, (size_t) m->cap * sizeof(float));
    dev_free(c, m->d_Y, (size_t) m->cap * sizeof(float));
    dev_free(c, m->d_idx, (size_t) m->cap * sizeof(int));
    dev_free(c, m->d_loss, (size_t) m->loss_cap * sizeof(float));
    dev_free(c, m->d_knots, kMlpKnots * sizeof(float));
    dev_free(c, m->d_key, sizeof(int));
    dev_free(c, m->d_status, sizeof(int));
    dev_free(c, m->d_counts, 2 * sizeof(unsigned long long));
    if (m->scratch_ev) cudaEventDestroy(m->scratch_ev);
    delete m;
    return IVR_OK;
}

int ivr_mlp_create(ivr_ctx *c, unsigned long long seed, ivr_mlp **out)
{
    if (!c || !out) return IVR_ERR_INVALID;
    *out = nullptr;
    ivr_mlp *m = new ivr_mlp();
    m->ctx = c;
    m->seed = seed;
    int rc = IVR_OK;
    void **bufs[] = {(void **) &m->d_p, (void **) &m->d_m, (void **) &m->d_v, (void **) &m->d_grad};
    for (void **b : bufs)
        if (rc == IVR_OK) rc = dev_alloc(c, kParamBytes, b);
    if (rc == IVR_OK) rc = dev_alloc(c, (size_t) kMlpHidden * kMlpIn * kBf16Bytes, &m->d_w1t);
    if (rc == IVR_OK) rc = dev_alloc(c, (size_t) kMlpHidden * kMlpHidden * kBf16Bytes, &m->d_w2t);
    if (rc == IVR_OK) rc = dev_alloc(c, (size_t) kMlpHidden * kMlpHidden * kBf16Bytes, &m->d_w2);
    if (rc == IVR_OK) rc = dev_alloc(c, kMlpKnots * sizeof(float), (void **) &m->d_knots);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(int), (void **) &m->d_key);
    if (rc == IVR_OK) rc = dev_alloc(c, sizeof(int), (void **) &m->d_status);
    if (rc == IVR_OK && cudaMemset(m->d_status, 0, sizeof(int)) != cudaSuccess)
        rc = fail(c, IVR_ERR_CUDA, "predictor status");
    if (rc == IVR_OK) rc = dev_alloc(c, 2 * sizeof(unsigned long long), (void **) &m->d_counts);
    if (rc == IVR_OK && cudaEventCreateWithFlags(&m->scratch_ev, cudaEventDisableTiming) != cudaSuccess)
        rc = fail(c, IVR_ERR_CUDA, "predictor event");
    if (rc == IVR_OK) {
        // He initialisation of the weights, zero biases
        std::mt19937_64 rng(seed);
        std::vector<float> p(kMlpParams, 0.0f);
        std::normal_distribution<float> n1(0.0f, sqrtf(2.0f / kMlpFeatures)), n2(0.0f, sqrtf(2.0f / kMlpHidden)),
            n3(0.0f, sqrtf(1.0f / kMlpHidden));
        for (int f = 0; f < kMlpFeatures; f++)
            for (int u = 0; u < kMlpHidden; u++) p[kOffW1 + f * kMlpHidden + u] = n1(rng);
        for (int i = 0; i < kMlpHidden * kMlpHidden; i++) p[kOffW2 + i] = n2(rng);
        for (int i = 0; i < kMlpHidden; i++) p[kOffW3 + i] = n3(rng);
        rc = upload(m, p);
    }
    if (rc) {
        ivr_mlp_free(m);
        return rc;
    }
    *out = m;
    return IVR_OK;
}

int ivr_mlp_get_params(const ivr_mlp *m, float *params)
{
    if (!m || !params) return m ? fail(m->ctx, IVR_ERR_INVALID, "null output") : IVR_ERR_INVALID;
    CK(m->ctx, cudaDeviceSynchronize());
    CK(m->ctx, cudaMemcpy(params, m->d_p, kParamBytes, cudaMemcpyDeviceToHost));
    return IVR_OK;
}

int ivr_mlp_set_params(ivr_mlp *m, const float *params)
{
    if (!m || !params) return m ? fail(m->ctx, IVR_ERR_INVALID, "null parameters") : IVR_ERR_INVALID;
    for (int i = 0; i < kMlpParams; i++)
        if (!isfinite(params[i])) return fail(m->ctx, IVR_ERR_INVALID, "parameter %d is not finite", i);
    CK(m->ctx, cudaDeviceSynchronize());
    return upload(m, std::vector<float>(params, params + kMlpParams));
}

int ivr_mlp_save(const ivr_mlp *m, const char *path)
{
    if (!m || !path) return m ? fail(m->ctx, IVR_ERR_INVALID, "null path") : IVR_ERR_INVALID;
    std::vector<float> p(kMlpParams);
    int rc = ivr_mlp_get_params(m, p.data());
    if (rc) return rc;
    FILE *f = fopen(path, "wb");
    if (!f) return fail(m->ctx, IVR_ERR_IO, "cannot write %s", path);
    // little-endian on disk whatever the host
    std::vector<unsigned char> buf(sizeof(kMagic) + 4 + 4 * (size_t) kMlpParams);
    memcpy(buf.data(), kMagic, sizeof(kMagic));
    const uint32_t cnt = kMlpParams;
    for (int b = 0; b < 4; b++) buf[8 + b] = (unsigned char) (cnt >> (8 * b));
    for (int i = 0; i < kMlpParams; i++) {
        uint32_t u;
        memcpy(&u, &p[i], 4);
        for (int b = 0; b < 4; b++) buf[12 + 4 * (size_t) i + b] = (unsigned char) (u >> (8 * b));
    }
    const size_t wrote = fwrite(buf.data(), 1, buf.size(), f);
    const int closed = fclose(f);
    if (wrote != buf.size() || closed != 0) return fail(m->ctx, IVR_ERR_IO, "short write to %s", path);
    return IVR_OK;
}

int ivr_mlp_load(ivr_mlp *m, const char *path)
{
    if (!m || !path) return m ? fail(m->ctx, IVR_ERR_INVALID, "null path") : IVR_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(m->ctx, IVR_ERR_IO, "cannot open %s", path);
    std::vector<unsigned char> buf(sizeof(kMagic) + 4 + 4 * (size_t) kMlpParams);
    const size_t got = fread(buf.data(), 1, buf.size(), f);
    fclose(f);
    if (got != buf.size() || memcmp(buf.data(), kMagic, sizeof(kMagic)) != 0)
        return fail(m->ctx, IVR_ERR_IO, "%s is not a predictor file", path);
    uint32_t cnt = 0;
    for (int b = 0; b < 4; b++) cnt |= (uint32_t) buf[8 + b] << (8 * b);
    if (cnt != (uint32_t) kMlpParams) return fail(m->ctx, IVR_ERR_IO, "%s holds %u parameters, not %d", path, cnt, kMlpParams);
    std::vector<float> p(kMlpParams);
    for (int i = 0; i < kMlpParams; i++) {
        uint32_t u = 0;
        for (int b = 0; b < 4; b++) u |= (uint32_t) buf[12 + 4 * (size_t) i + b] << (8 * b);
        memcpy(&p[i], &u, 4);
    }
    return ivr_mlp_set_params(m, p.data());
}

int ivr_mlp_features(ivr_mlp *m, ivr_volume *v, ivr_tf *tf, uint16_t *x_dev, float *bound_dev, long long cap,
                     long long *n, void *stream)
{
    if (!m) return IVR_ERR_INVALID;
    ivr_ctx *c = m->ctx;
    if (!v || v->ctx != c || !x_dev || !n) return fail(c, IVR_ERR_INVALID, "bad volume or output");
    int rc = check_tf(c, tf);
    if (rc) return rc;
    const long long cells = volume_cells(v);
    *n = cells;
    if (cells > cap) return fail(c, IVR_ERR_INVALID, "%lld cells do not fit %lld rows", cells, cap);
    CK(c, cudaStreamWaitEvent((cudaStream_t) stream, m->scratch_ev, 0));
    rc = features(m, v, tf, x_dev, bound_dev, (cudaStream_t) stream);
    if (rc) return rc;
    CK(c, cudaEventRecord(m->scratch_ev, (cudaStream_t) stream));
    return IVR_OK;
}

int ivr_mlp_forward(ivr_mlp *m, const uint16_t *x_dev, long long n, float *y_dev, void *stream)
{
    if (!m) return IVR_ERR_INVALID;
    if (n < 0 || (n > 0 && (!x_dev || !y_dev))) return fail(m->ctx, IVR_ERR_INVALID, "bad rows");
    CK(m->ctx, mlp_forward(dev_of(m), x_dev, n, y_dev, (cudaStream_t) stream));
    return IVR_OK;
}

int ivr_mlp_gradient(ivr_mlp *m, const uint16_t *x_dev, const float *bound_dev, long long n, float wneg,
                     float *grad_dev, float *loss_dev, void *stream)
{
    if (!m) return IVR_ERR_INVALID;
    ivr_ctx *c = m->ctx;
    if (n < 1 || !x_dev || !bound_dev || !grad_dev || !loss_dev) return fail(c, IVR_ERR_INVALID, "bad rows or outputs");
    if (!(wneg > 0.0f && wneg < 1e6f)) return fail(c, IVR_ERR_INVALID, "wneg must be in (0, 1e6)");
    cudaStream_t s = (cudaStream_t) stream;
    CK(c, cudaMemsetAsync(grad_dev, 0, kParamBytes, s));
    CK(c, cudaMemsetAsync(loss_dev, 0, sizeof(float), s));
    CK(c, mlp_train_step(dev_of(m), x_dev, bound_dev, nullptr, n, n, wneg, IVR_MLP_TRANSPARENT, grad_dev, loss_dev, s));
    return IVR_OK;
}

int ivr_mlp_add_samples(ivr_mlp *m, ivr_volume *v, ivr_tf *tf, long long *total)
{
    if (!m) return IVR_ERR_INVALID;
    ivr_ctx *c = m->ctx;
    if (!v || v->ctx != c) return fail(c, IVR_ERR_INVALID, "volume missing or from another context");
    int rc = check_tf(c, tf);
    if (rc) return rc;
    const long long cells = volume_cells(v);
    if (m->n + cells > (long long) 0x7fffffff) return fail(c, IVR_ERR_INVALID, "training set above 2^31 rows");
    CK(c, cudaDeviceSynchronize());
    if (m->n + cells > m->cap) {
        // all four arrays move to the new capacity together, or none does
        const long long nc = std::max(m->n + cells, m->cap * 2);
        void *x = nullptr, *t = nullptr, *y = nullptr, *ix = nullptr;
        rc = dev_alloc(c, (size_t) nc * kMlpIn * kBf16Bytes, &x);
        if (rc == IVR_OK) rc = dev_alloc(c, (size_t) nc * sizeof(float), &t);
        if (rc == IVR_OK) rc = dev_alloc(c, (size_t) nc * sizeof(float), &y);
        if (rc == IVR_OK) rc = dev_alloc(c, (size_t) nc * sizeof(int), &ix);
        if (rc == IVR_OK && m->n > 0 &&
            (cudaMemcpy(x, m->d_X, (size_t) m->n * kMlpIn * kBf16Bytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
             cudaMemcpy(t, m->d_T, (size_t) m->n * sizeof(float), cudaMemcpyDeviceToDevice) != cudaSuccess))
            rc = fail(c, IVR_ERR_CUDA, "copying the training set");
        if (rc) {
            dev_free(c, x, (size_t) nc * kMlpIn * kBf16Bytes);
            dev_free(c, t, (size_t) nc * sizeof(float));
            dev_free(c, y, (size_t) nc * sizeof(float));
            dev_free(c, ix, (size_t) nc * sizeof(int));
            return rc;
        }
        dev_free(c, m->d_X, (size_t) m->cap * kMlpIn * kBf16Bytes);
        dev_free(c, m->d_T, (size_t) m->cap * sizeof(float));
        dev_free(c, m->d_Y, (size_t) m->cap * sizeof(float));
        dev_free(c, m->d_idx, (size_t) m->cap * sizeof(int));
        m->d_X = (uint16_t *) x;
        m->d_T = (float *) t;
        m->d_Y = (float *) y;
        m->d_idx = (int *) ix;
        m->cap = nc;
    }
    rc = features(m, v, tf, m->d_X + m->n * kMlpIn, m->d_T + m->n, 0);
    if (rc) return rc;
    CK(c, cudaDeviceSynchronize());
    m->n += cells;
    if (total) *total = m->n;
    return IVR_OK;
}

int ivr_mlp_clear_samples(ivr_mlp *m)
{
    if (!m) return IVR_ERR_INVALID;
    m->n = 0;
    return IVR_OK;
}

int ivr_mlp_train(ivr_mlp *m, int epochs, int batch_rows, float lr, float wneg, float *loss_per_epoch)
{
    if (!m) return IVR_ERR_INVALID;
    ivr_ctx *c = m->ctx;
    if (m->n < 1) return fail(c, IVR_ERR_INVALID, "empty training set");
    if (epochs < 1 || epochs > 100000) return fail(c, IVR_ERR_INVALID, "epochs must be in [1, 100000]");
    if (batch_rows < 1 || batch_rows > (1 << 24)) return fail(c, IVR_ERR_INVALID, "batch_rows must be in [1, 2^24]");
    if (!(lr > 0.0f && lr < 1.0f)) return fail(c, IVR_ERR_INVALID, "lr must be in (0, 1)");
    if (!(wneg > 0.0f && wneg < 1e6f)) return fail(c, IVR_ERR_INVALID, "wneg must be in (0, 1e6)");
    const long long nb = (m->n + batch_rows - 1) / batch_rows;
    int rc = grow(c, (void **) &m->d_loss, &m->loss_cap, nb, sizeof(float), 0);
    if (rc) return rc;
    // the Adam bias corrections of an epoch's steps, device-resident so that
    // one captured epoch replays with each epoch's values
    float *d_c12 = nullptr;
    rc = dev_alloc(c, sizeof(float) * 2 * (size_t) nb, (void **) &d_c12);
    if (rc) return rc;
    struct Graph {
        cudaStream_t s = nullptr;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t x = nullptr;
        ~Graph()
        {
            if (x) cudaGraphExecDestroy(x);
            if (g) cudaGraphDestroy(g);
            if (s) cudaStreamDestroy(s);
        }
    } gr;
    auto done = [&](int code) {
        dev_free(c, d_c12, sizeof(float) * 2 * (size_t) nb);
        return code;
    };
    const MlpDev w = dev_of(m);
    // the epochs' row orders in two page-locked buffers (the host shuffles
    // the next epoch's while the device trains on the current one), and the
    // epoch's bias corrections and losses in page-locked memory too, so that
    // no copy of an epoch waits for the host or the host for the device
    // before the shuffle is done
    const size_t n = (size_t) m->n;
    int *order[2] = {nullptr, nullptr};
    float *c12 = nullptr, *losses = nullptr;
    struct Pinned {
        void *p[4];
        ~Pinned()
        {
            for (void *q : p)
                if (q) cudaFreeHost(q);
        }
    } pinned{};
    SplitMix rng{m->seed ^ 0x9e3779b97f4a7c15ull};
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaHostAlloc(&pinned.p[0], sizeof(int) * n, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&pinned.p[1], sizeof(int) * n, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&pinned.p[2], sizeof(float) * 2 * (size_t) nb, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&pinned.p[3], sizeof(float) * (size_t) nb, 0);
    if (e != cudaSuccess) return done(cuda_fail(c, e, "training order buffers"));
    order[0] = (int *) pinned.p[0];
    order[1] = (int *) pinned.p[1];
    c12 = (float *) pinned.p[2];
    losses = (float *) pinned.p[3];
    for (size_t i = 0; i < n; i++) order[0][i] = (int) i;
    shuffle_rows(order[0], n, rng);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&gr.s, cudaStreamNonBlocking);
    // the kernels' shared-memory attributes, set outside the capture
    if (e == cudaSuccess) e = mlp_train_step(w, m->d_X, m->d_T, m->d_idx, 0, 1, wneg, IVR_MLP_TRANSPARENT, m->d_grad,
                                             m->d_loss, gr.s);
    // one epoch's mini-batches: gradient reset, training step, Adam (a
    // launch-bound loop of 3 x nb launches, captured once)
    if (e == cudaSuccess) e = cudaStreamBeginCapture(gr.s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t ce = cudaSuccess;
        for (long long b = 0; b < nb && ce == cudaSuccess; b++) {
            const long long r0 = b * batch_rows, rows = std::min<long long>(batch_rows, m->n - r0);
            ce = cudaMemsetAsync(m->d_grad, 0, kParamBytes, gr.s);
            if (ce == cudaSuccess)
                ce = mlp_train_step(w, m->d_X, m->d_T, m->d_idx + r0, rows, rows, wneg, IVR_MLP_TRANSPARENT, m->d_grad,
                                    m->d_loss + b, gr.s);
            if (ce == cudaSuccess)
                ce = mlp_adam(m->d_p, m->d_m, m->d_v, m->d_grad, lr, 0, d_c12 + 2 * b, m->d_w1t, m->d_w2t, m->d_w2,
                              gr.s);
        }
        e = cudaStreamEndCapture(gr.s, &gr.g);
        if (e == cudaSuccess) e = ce;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&gr.x, gr.g, 0);
    if (e != cudaSuccess) return done(cuda_fail(c, e, "training graph"));
    for (int ep = 0; ep < epochs; ep++) {
        const int cur = ep & 1;
        for (long long b = 0; b < nb; b++) mlp_adam_corrections(m->step + b + 1, &c12[2 * b], &c12[2 * b + 1]);
        e = cudaMemcpyAsync(m->d_idx, order[cur], sizeof(int) * n, cudaMemcpyHostToDevice, gr.s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_c12, c12, sizeof(float) * 2 * (size_t) nb, cudaMemcpyHostToDevice, gr.s);
        if (e == cudaSuccess) e = cudaMemsetAsync(m->d_loss, 0, sizeof(float) * (size_t) nb, gr.s);
        if (e == cudaSuccess) e = cudaGraphLaunch(gr.x, gr.s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(losses, m->d_loss, sizeof(float) * (size_t) nb, cudaMemcpyDeviceToHost, gr.s);
        if (e == cudaSuccess && ep + 1 < epochs) {  // the next epoch's order, meanwhile
            memcpy(order[cur ^ 1], order[cur], sizeof(int) * n);
            shuffle_rows(order[cur ^ 1], n, rng);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(gr.s);  // c12 and the order buffers are rewritten next
        if (e != cudaSuccess) return done(cuda_fail(c, e, "training epoch"));
        m->step += (int) nb;
        if (loss_per_epoch) {
            double sum = 0.0;
            for (long long b = 0; b < nb; b++) sum += losses[b];
            loss_per_epoch[ep] = (float) (sum / (double) nb);
        }
    }
    m->serial++;
    int status = 0;
    e = cudaMemcpy(&status, m->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return done(cuda_fail(c, e, "training status"));
    if (status != 0) {
        cudaMemset(m->d_status, 0, sizeof(int));
        return done(fail(c, IVR_ERR_TIMEOUT, "a tensor-core wait of the training step ran out; the parameters are suspect"));
    }
    return done(IVR_OK);
}

int ivr_mlp_calibrate(ivr_mlp *m, float slack, float *margin, float *recall)
{
    if (!m) return IVR_ERR_INVALID;
    ivr_ctx *c = m->ctx;
    if (m->n < 1) return fail(c, IVR_ERR_INVALID, "empty training set");
    if (!(slack >= 0.0f && slack < 1e3f) || !margin) return fail(c, IVR_ERR_INVALID, "bad slack or output");
    CK(c, mlp_forward(dev_of(m), m->d_X, m->n, m->d_Y, 0));
    int key = mlp_key_of(-FLT_MAX);
    unsigned long long counts[2] = {0, 0};
    CK(c, cudaMemcpy(m->d_key, &key, sizeof(int), cudaMemcpyHostToDevice));
    CK(c, cudaMemset(m->d_counts, 0, sizeof(counts)));
    CK(c, mlp_calibrate(m->d_Y, m->d_T, m->n, 0.0f, m->d_key, m->d_counts, 0));
    CK(c, cudaMemcpy(&key, m->d_key, sizeof(int), cudaMemcpyDeviceToHost));
    const float worst = mlp_key_value(key);  // largest -y of a sample with a bound above 0
    const float mg = std::max(worst, 0.0f) + slack;
    CK(c, cudaMemset(m->d_counts, 0, sizeof(counts)));
    CK(c, mlp_calibrate(m->d_Y, m->d_T, m->n, mg, m->d_key, m->d_counts, 0));
    CK(c, cudaMemcpy(counts, m->d_counts, sizeof(counts), cudaMemcpyDeviceToHost));
    int status = 0;
    CK(c, cudaMemcpy(&status, m->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status != 0) {
        cudaMemset(m->d_status, 0, sizeof(int));
        return fail(c, IVR_ERR_TIMEOUT, "a tensor-core wait of the predictor's inference ran out");
    }
    *margin = mg;
    if (recall) *recall = counts[0] ? (float) ((double) counts[1] / (double) counts[0]) : 0.0f;
    return IVR_OK;
}

int ivr_volume_set_mlp(ivr_volume *v, ivr_mlp *m, float margin, int certify)
{
    if (!v) return IVR_ERR_INVALID;
    if (m && m->ctx != v->ctx) return fail(v->ctx, IVR_ERR_INVALID, "predictor from another context");
    if (!(margin >= 0.0f && margin < 1e3f)) return fail(v->ctx, IVR_ERR_INVALID, "margin must be in [0, 1000)");
    drop_learned_grids(v);
    if (!v->d_lstats) {
        int rc = dev_alloc(v->ctx, 4 * sizeof(unsigned long long), (void **) &v->d_lstats);
        if (rc) return rc;
    }
    CK(v->ctx, cudaMemset(v->d_lstats, 0, 4 * sizeof(unsigned long long)));
    v->mlp = m;
    v->mlp_margin = margin;
    v->mlp_certify = certify != 0;
    return IVR_OK;
}

int ivr_volume_learned_stats(ivr_volume *v, unsigned long long *stats)
{
    if (!v || !stats) return v ? fail(v->ctx, IVR_ERR_INVALID, "null output") : IVR_ERR_INVALID;
    memset(stats, 0, 4 * sizeof(unsigned long long));
    if (!v->d_lstats) return IVR_OK;
    CK(v->ctx, cudaDeviceSynchronize());
    CK(v->ctx, cudaMemcpy(stats, v->d_lstats, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    return IVR_OK;
}

}  // extern "C"
