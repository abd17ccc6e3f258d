// ivr_server.cpp -- the steering server: continuous batching of render
// requests over resident volumes.
//
// Replaces the reference's frame path of ivrserver + relay
// (main.c:206-250, myserver.c:133-165): instead of one client whose STATE is
// broadcast to MPI ranks and answered with one frame, many clients submit
// requests (a resident volume, a STATE, a transfer function, an RGBA8 output
// buffer) at any time.  A scheduler thread keeps several batch slots in
// flight, each on its own stream.  The frames' device memory is one output
// pool taken from the context's HBM budget at start (slots x arena_bytes):
// whenever a slot is free it takes the queued requests, in arrival order and
// of any volume dtype, whose RGBA8 outputs fit the largest free range of the
// pool -- the HBM admission rule -- renders them (one persistent batched
// launch per dtype), copies the frames back and records completion times.
// Requests that arrive while slots are busy, or that do not fit the free
// memory yet, wait in the queue and are admitted as slots and pool memory
// free up, so batches overlap on the device; only a frame larger than the
// whole pool is refused.
//
// The optional TCP front end speaks the reference's steering protocol: a
// client sends the 184-byte STATE (finish, winwidth, winheight in network
// byte order, connection.c:167-200) and receives the viewport as RGBA8
// (connection.c:203-215).
#include <arpa/inet.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <sys/socket.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <future>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ivr_gpu.h"

namespace {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    ivr_request r;
    ivr_volume *vol;  // r.volume's handle and dtype, resolved under the lock at submit
    int dtype;
    double t_submit;
    int vw, vh;
    size_t bytes;
    bool direct;  // the output buffer is page-locked: the frame is copied straight into it
    std::shared_ptr<std::promise<int>> notify;  // front-end requests
    ivr_completion c;
};

struct Slot {
    cudaStream_t stream = nullptr;
    size_t base = 0, span = 0;  // its batch's range of the output pool (span 0: none)
    std::vector<ivr_view *> views;
    ivr_batch *batch[3] = {nullptr, nullptr, nullptr};  // per dtype
    cudaEvent_t ev = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;  // timing of the batch's device work
    bool busy = false;     // launched, or frames not yet copied out
    bool copying = false;  // handed to the completion thread
    std::vector<Req> reqs;
    std::vector<size_t> offs;
    double t_start = 0.0;
};

struct PendingTf {
    int id;
    std::vector<float> lut;
    int n, off;
    float scale;
};

}  // namespace

struct ivr_server {
    ivr_ctx *ctx = nullptr;
    int device = 0;
    ivr_server_config cfg{};
    ivr_render_params params{};
    std::vector<ivr_volume *> vols;
    std::vector<int> vol_dtype;
    std::vector<ivr_tf *> tfs;  // materialised on the scheduler thread
    std::deque<PendingTf> pending_tfs;
    int next_tf = 0;
    std::deque<Req> queue;
    std::deque<ivr_completion> done;
    std::vector<Slot> slots;
    // the output pool: device RGBA8 frames of the batches in flight and
    // their page-locked host staging, at the same offsets; ranges = the
    // [offset, offset + bytes) the slots hold, under mu
    void *pool = nullptr;
    void *pool_pinned = nullptr;
    size_t pool_bytes = 0;
    std::vector<std::pair<size_t, size_t>> ranges;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread sched, copier;
    bool stop = false;
    std::deque<Slot *> to_copy;  // finished slots for the completion thread
    std::condition_variable cv_copy;
    bool copier_stop = false;
    std::atomic<long long> completed{0}, rejected{0}, batches{0};
    double gpu_s = 0.0;       // summed device time of the batches
    double dispatch_s = 0.0;  // scheduler time spent forming and launching batches
    double finish_s = 0.0;    // scheduler time spent copying frames out
    // TCP front end
    int listen_fd = -1;
    std::thread acceptor;
    std::vector<std::thread> conns;
    std::vector<int> conn_fds;  // open client sockets (under mu), shut down by ivr_server_destroy
    std::atomic<bool> net_stop{false};
    int net_tf = 0;
    int net_volume = 0;
    std::atomic<unsigned long long> net_tag{1ull << 62};
    std::string err;
};

namespace {

int viewport_dim(int win, int tile) { return (win / tile) * tile; }

// The output pool's free ranges, between the held ones (sorted by offset).
// Under s->mu.  largest_free: the longest; first_fit: the offset of the
// first at least `need` long, or pool_bytes when none is.
size_t largest_free(const ivr_server *s)
{
    size_t at = 0, best = 0;
    for (const auto &r : s->ranges) {
        if (r.first > at) best = std::max(best, r.first - at);
        at = std::max(at, r.first + r.second);
    }
    return std::max(best, s->pool_bytes > at ? s->pool_bytes - at : 0);
}

size_t first_fit(const ivr_server *s, size_t need)
{
    size_t at = 0;
    for (const auto &r : s->ranges) {
        if (r.first >= at + need) return at;
        at = std::max(at, r.first + r.second);
    }
    return s->pool_bytes >= at + need ? at : s->pool_bytes;
}

void hold_range(ivr_server *s, Slot &sl, size_t off, size_t bytes)
{
    auto it = s->ranges.begin();
    while (it != s->ranges.end() && it->first < off) ++it;
    s->ranges.insert(it, {off, bytes});
    sl.base = off;
    sl.span = bytes;
}

void release_range(ivr_server *s, Slot &sl)
{
    if (sl.span == 0) return;
    for (auto it = s->ranges.begin(); it != s->ranges.end(); ++it)
        if (it->first == sl.base && it->second == sl.span) {
            s->ranges.erase(it);
            break;
        }
    sl.base = sl.span = 0;
}

void complete(ivr_server *s, Req &q, int status, double t_start)
{
    q.c.tag = q.r.tag;
    q.c.status = status;
    q.c.vw = q.vw;
    q.c.vh = q.vh;
    q.c.t_queue = t_start > 0.0 ? t_start - q.t_submit : 0.0;
    q.c.t_total = now_s() - q.t_submit;
    if (status == IVR_OK) s->completed++;
    else s->rejected++;
    if (q.notify) {
        q.notify->set_value(status);
        return;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    s->done.push_back(q.c);
    s->cv_done.notify_all();
}

// copies a finished slot's frames out and frees the slot
void finish_slot(ivr_server *s, Slot &sl)
{
    const double t = now_s();
    float ms = 0.0f;
    const double batch_s = cudaEventElapsedTime(&ms, sl.t0, sl.t1) == cudaSuccess ? ms / 1000.0 : 0.0;
    for (size_t i = 0; i < sl.reqs.size(); i++) {
        Req &q = sl.reqs[i];
        if (!q.direct) memcpy(q.r.rgba8_host, (char *) s->pool_pinned + sl.base + sl.offs[i], q.bytes);
        complete(s, q, IVR_OK, sl.t_start);
    }
    sl.reqs.clear();
    sl.offs.clear();
    std::lock_guard<std::mutex> lock(s->mu);
    release_range(s, sl);
    sl.busy = false;
    s->gpu_s += batch_s;  // read under the same lock by ivr_server_times
    s->finish_s += now_s() - t;
}

// completion thread: copies finished slots' frames to the callers' buffers
// (the scheduler keeps launching meanwhile) and then frees the slot
void copier(ivr_server *s)
{
    for (;;) {
        Slot *sl = nullptr;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_copy.wait(lock, [&] { return s->copier_stop || !s->to_copy.empty(); });
            if (s->to_copy.empty()) return;
            sl = s->to_copy.front();
            s->to_copy.pop_front();
        }
        finish_slot(s, *sl);
        {
            std::lock_guard<std::mutex> lock(s->mu);
            sl->copying = false;
        }
        s->cv_work.notify_one();
    }
}

void materialise_tfs(ivr_server *s)
{
    std::deque<PendingTf> todo;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        todo.swap(s->pending_tfs);
    }
    for (auto &p : todo) {
        ivr_tf *tf = nullptr;
        int rc = ivr_tf_create(s->ctx, &tf);
        if (rc == IVR_OK) rc = ivr_tf_set_lut(tf, p.lut.data(), p.n, p.off, p.scale, IVR_TF_F2B);
        if ((int) s->tfs.size() <= p.id) s->tfs.resize(p.id + 1, nullptr);
        s->tfs[p.id] = rc == IVR_OK ? tf : nullptr;
        if (rc != IVR_OK && tf) ivr_tf_free(tf);
    }
}

// takes the queued requests that fit a free slot and the free output
// memory, and launches them
bool dispatch(ivr_server *s, Slot &sl)
{
    std::vector<Req> take, never;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->queue.empty()) return false;
        const size_t room = largest_free(s);
        size_t used = 0;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int) take.size() < s->cfg.max_batch_frames;) {
            if (it->bytes > s->pool_bytes) {  // larger than the whole pool: never admitted
                never.push_back(*it);
                it = s->queue.erase(it);
                continue;
            }
            if (used + it->bytes > room) break;  // arrival order: wait for memory to free up
            used += it->bytes;
            take.push_back(*it);
            it = s->queue.erase(it);
        }
        if (!take.empty()) hold_range(s, sl, first_fit(s, used), used);
    }
    for (auto &q : never) complete(s, q, IVR_ERR_NOMEM, 0.0);
    if (take.empty()) return !never.empty();
    sl.t_start = now_s();
    for (auto &q : take)
        if (q.r.tf >= (int) s->tfs.size() || (q.r.tf >= 0 && !s->tfs[q.r.tf])) {
            materialise_tfs(s);  // registered after the last pass
            break;
        }
    char *const dev = (char *) s->pool + sl.base;
    size_t off = 0;
    std::vector<Req> ok;
    cudaEventRecord(sl.t0, sl.stream);
    int rc = IVR_OK;
    // one batched launch per volume dtype among the requests taken
    for (int dtype = IVR_U8; dtype <= IVR_F32 && rc == IVR_OK; dtype++) {
        ivr_batch *&b = sl.batch[dtype];
        size_t nd = 0;
        for (auto &q : take) nd += q.dtype == dtype;
        if (nd == 0) continue;
        if (!b) {
            if (ivr_batch_create(s->ctx, s->cfg.max_batch_frames, &b) != IVR_OK) b = nullptr;
            else ivr_batch_set_variant(b, s->cfg.variant);
        }
        if (b) ivr_batch_clear(b);
        size_t added = 0;
        for (auto &q : take) {
            if (q.dtype != dtype) continue;
            ivr_view *view = sl.views[ok.size()];
            ivr_tf *tf = (q.r.tf >= 0 && q.r.tf < (int) s->tfs.size()) ? s->tfs[q.r.tf] : nullptr;
            int qrc = b ? IVR_OK : IVR_ERR_NOMEM;
            if (qrc == IVR_OK && !tf) qrc = IVR_ERR_INVALID;
            if (qrc == IVR_OK) qrc = ivr_set_view(view, q.vol, &q.r.state, &s->params);
            if (qrc == IVR_OK) qrc = ivr_batch_add(b, view, tf, nullptr, (uint8_t *) dev + off);
            if (qrc != IVR_OK) {
                complete(s, q, qrc, sl.t_start);
                continue;
            }
            sl.offs.push_back(off);
            off += q.bytes;
            ok.push_back(q);
            added++;
        }
        if (added) rc = ivr_batch_render(b, 1, sl.stream);
    }
    if (ok.empty()) {
        std::lock_guard<std::mutex> lock(s->mu);
        release_range(s, sl);
        return true;
    }
    if (rc == IVR_OK) cudaEventRecord(sl.t1, sl.stream);
    // frames for page-locked buffers go straight there; the others through
    // the pool's staging, one copy per run of consecutive staged frames
    for (size_t i = 0; i < ok.size() && rc == IVR_OK;) {
        const size_t o = sl.offs[i];
        if (ok[i].direct) {
            if (cudaMemcpyAsync(ok[i].r.rgba8_host, dev + o, ok[i].bytes, cudaMemcpyDeviceToHost, sl.stream) !=
                cudaSuccess)
                rc = IVR_ERR_CUDA;
            i++;
            continue;
        }
        size_t j = i, end = o;
        while (j < ok.size() && !ok[j].direct) end = sl.offs[j] + ok[j].bytes, j++;
        if (cudaMemcpyAsync((char *) s->pool_pinned + sl.base + o, dev + o, end - o, cudaMemcpyDeviceToHost,
                            sl.stream) != cudaSuccess)
            rc = IVR_ERR_CUDA;
        i = j;
    }
    if (rc == IVR_OK && cudaEventRecord(sl.ev, sl.stream) != cudaSuccess) rc = IVR_ERR_CUDA;
    if (rc != IVR_OK) {
        // nothing of this batch may still write the range it releases
        cudaStreamSynchronize(sl.stream);
        for (auto &q : ok) complete(s, q, rc, sl.t_start);
        sl.offs.clear();
        std::lock_guard<std::mutex> lock(s->mu);
        release_range(s, sl);
        return true;
    }
    sl.reqs = std::move(ok);
    {
        std::lock_guard<std::mutex> lock(s->mu);
        sl.busy = true;
    }
    s->batches++;
    return true;
}

void scheduler(ivr_server *s)
{
    cudaSetDevice(s->device);
    for (;;) {
        bool did = false;
        for (auto &sl : s->slots) {
            bool hand = false;
            {
                std::lock_guard<std::mutex> lock(s->mu);
                hand = sl.busy && !sl.copying && cudaEventQuery(sl.ev) == cudaSuccess;
                if (hand) {
                    sl.copying = true;
                    s->to_copy.push_back(&sl);
                }
            }
            if (hand) {
                s->cv_copy.notify_one();
                did = true;
            }
        }
        materialise_tfs(s);
        for (auto &sl : s->slots) {
            bool idle;
            {
                std::lock_guard<std::mutex> lock(s->mu);
                idle = !sl.busy;
            }
            if (idle) {
                const double t = now_s();
                const bool d = dispatch(s, sl);
                if (d) {
                    std::lock_guard<std::mutex> lock(s->mu);
                    s->dispatch_s += now_s() - t;
                }
                did |= d;
            }
        }
        std::unique_lock<std::mutex> lock(s->mu);
        if (s->stop) {
            bool busy = false;
            for (auto &sl : s->slots) busy |= sl.busy;
            if (!busy && s->queue.empty()) break;
        }
        if (!did) s->cv_work.wait_for(lock, std::chrono::microseconds(s->cfg.poll_us));
    }
}

// Both ends of [p, p + n) in page-locked host memory (cudaHostAlloc or
// cudaHostRegister): the device can copy into it directly.
bool page_locked(const void *p, size_t n)
{
    for (const char *q : {(const char *) p, (const char *) p + n - 1}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

int submit_req(ivr_server *s, const ivr_request *r, std::shared_ptr<std::promise<int>> notify)
{
    if (r->volume < 0 || !r->rgba8_host) return IVR_ERR_INVALID;
    Req q;
    q.r = *r;
    q.t_submit = now_s();
    q.vw = viewport_dim(r->state.winwidth, s->params.tilew);
    q.vh = viewport_dim(r->state.winheight, s->params.tileh);
    if (q.vw < 1 || q.vh < 1) return IVR_ERR_INVALID;
    q.bytes = (size_t) q.vw * q.vh * 4;
    q.direct = page_locked(r->rgba8_host, q.bytes);
    q.notify = std::move(notify);
    memset(&q.c, 0, sizeof(q.c));
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->stop || r->volume >= (int) s->vols.size()) return IVR_ERR_INVALID;
        q.vol = s->vols[r->volume];
        q.dtype = s->vol_dtype[r->volume];
        s->queue.push_back(q);
    }
    s->cv_work.notify_one();
    return IVR_OK;
}

bool recv_all(int fd, void *buf, size_t n)
{
    char *p = (char *) buf;
    while (n > 0) {
        ssize_t r = recv(fd, p, n, 0);
        if (r <= 0) return false;
        p += r;
        n -= (size_t) r;
    }
    return true;
}

bool send_all(int fd, const void *buf, size_t n)
{
    const char *p = (const char *) buf;
    while (n > 0) {
        ssize_t r = send(fd, p, n, MSG_NOSIGNAL);
        if (r <= 0) return false;
        p += r;
        n -= (size_t) r;
    }
    return true;
}

// one steering client: STATE in, frame out, until finish or disconnect
void serve_conn(ivr_server *s, int fd)
{
    int one = 1;
    setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &one, sizeof(one));
    std::vector<uint8_t> frame;
    for (;;) {
        ivr_state st;
        if (!recv_all(fd, &st, sizeof(st))) break;  // short read or disconnect
        st.finish = (int) ntohl((uint32_t) st.finish);
        st.winwidth = (int) ntohl((uint32_t) st.winwidth);
        st.winheight = (int) ntohl((uint32_t) st.winheight);
        if (st.finish) break;
        ivr_request r;
        memset(&r, 0, sizeof(r));
        r.volume = s->net_volume;
        r.tf = s->net_tf;
        r.state = st;
        r.tag = s->net_tag++;
        const int vw = viewport_dim(st.winwidth, s->params.tilew), vh = viewport_dim(st.winheight, s->params.tileh);
        if (vw < 1 || vh < 1 || (long long) vw * vh > (1LL << 26)) break;
        frame.resize((size_t) vw * vh * 4);
        r.rgba8_host = frame.data();
        auto p = std::make_shared<std::promise<int>>();
        auto fut = p->get_future();
        if (submit_req(s, &r, p) != IVR_OK) break;
        if (fut.get() != IVR_OK) break;
        if (!send_all(fd, frame.data(), frame.size())) break;
    }
    {
        // untracked first, so that ivr_server_destroy never shuts down a
        // descriptor number that has been reused
        std::lock_guard<std::mutex> lock(s->mu);
        for (size_t i = 0; i < s->conn_fds.size(); i++)
            if (s->conn_fds[i] == fd) {
                s->conn_fds.erase(s->conn_fds.begin() + (long) i);
                break;
            }
    }
    close(fd);
}

void accept_loop(ivr_server *s)
{
    while (!s->net_stop) {
        int fd = accept(s->listen_fd, nullptr, nullptr);
        if (fd < 0) {
            if (s->net_stop) break;
            continue;
        }
        std::lock_guard<std::mutex> lock(s->mu);
        s->conn_fds.push_back(fd);
        s->conns.emplace_back(serve_conn, s, fd);
    }
}

}  // namespace

extern "C" {

void ivr_server_config_default(ivr_server_config *c)
{
    if (!c) return;
    c->slots = 4;
    c->max_batch_frames = 64;
    c->arena_bytes = (size_t) 96 << 20;
    c->poll_us = 100;
    c->step = 0.5f;
    c->term_alpha = 0.99f;
    c->tilew = 1;
    c->tileh = 1;
    c->variant = 1;  // 8x4 warp tiles, one sample per iteration
}

int ivr_server_create(ivr_ctx *ctx, const ivr_server_config *cfg, ivr_server **out)
{
    if (!ctx || !out) return IVR_ERR_INVALID;
    *out = nullptr;
    ivr_server_config c;
    ivr_server_config_default(&c);
    if (cfg) c = *cfg;
    if (c.slots < 1 || c.slots > 16 || c.max_batch_frames < 1 || c.max_batch_frames > 1024 || c.arena_bytes < 4 ||
        c.poll_us < 1)
        return IVR_ERR_INVALID;
    ivr_server *s = new ivr_server();
    s->ctx = ctx;
    s->cfg = c;
    cudaGetDevice(&s->device);  // the context's device (current after ivr_create)
    ivr_params_config(&s->params);
    s->params.step = c.step;
    s->params.term_alpha = c.term_alpha;
    s->params.tilew = c.tilew;
    s->params.tileh = c.tileh;
    s->slots.resize(c.slots);
    int rc = IVR_OK;
    // the output pool comes out of the context's HBM budget
    s->pool_bytes = c.arena_bytes * (size_t) c.slots;
    if (cudaMallocHost(&s->pool_pinned, s->pool_bytes) != cudaSuccess) {
        s->pool_pinned = nullptr;
        rc = IVR_ERR_NOMEM;
    }
    if (rc == IVR_OK && (rc = ivr_device_alloc(ctx, s->pool_bytes, &s->pool)) != IVR_OK) s->pool = nullptr;
    for (auto &sl : s->slots) {
        if (rc != IVR_OK) break;
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreate(&sl.t0) != cudaSuccess || cudaEventCreate(&sl.t1) != cudaSuccess) {
            rc = IVR_ERR_CUDA;
            break;
        }
        sl.views.resize(c.max_batch_frames, nullptr);
        for (auto &v : sl.views)
            if ((rc = ivr_view_create(ctx, &v)) != IVR_OK) break;
        if (rc) break;
    }
    if (rc != IVR_OK) {
        ivr_server_destroy(s);
        return rc;
    }
    s->sched = std::thread(scheduler, s);
    s->copier = std::thread(copier, s);
    *out = s;
    return IVR_OK;
}

int ivr_server_add_volume(ivr_server *s, ivr_volume *vol, int dtype, int *id)
{
    if (!s || !vol || !id || dtype < IVR_U8 || dtype > IVR_F32) return IVR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    if (!s->queue.empty()) return IVR_ERR_INVALID;  // volumes are registered before serving
    s->vols.push_back(vol);
    s->vol_dtype.push_back(dtype);
    *id = (int) s->vols.size() - 1;
    return IVR_OK;
}

int ivr_server_add_tf(ivr_server *s, const float *rgba, int n, int lut_offset, float lut_scale, int *id)
{
    if (!s || !rgba || n < 1 || n > (1 << 24) || !id || !(lut_scale > 0.0f)) return IVR_ERR_INVALID;
    PendingTf p;
    p.lut.assign(rgba, rgba + 4 * (size_t) n);
    p.n = n;
    p.off = lut_offset;
    p.scale = lut_scale;
    std::lock_guard<std::mutex> lock(s->mu);
    p.id = s->next_tf++;
    *id = p.id;
    s->pending_tfs.push_back(std::move(p));
    s->cv_work.notify_one();
    return IVR_OK;
}

int ivr_server_submit(ivr_server *s, const ivr_request *r)
{
    if (!s || !r) return IVR_ERR_INVALID;
    return submit_req(s, r, nullptr);
}

int ivr_server_poll(ivr_server *s, ivr_completion *out, int max, int *n, int wait_ms)
{
    if (!s || !out || !n || max < 1) return IVR_ERR_INVALID;
    std::unique_lock<std::mutex> lock(s->mu);
    if (s->done.empty() && wait_ms > 0)
        s->cv_done.wait_for(lock, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
    int k = 0;
    while (k < max && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *n = k;
    return IVR_OK;
}

int ivr_server_stats(ivr_server *s, long long *completed, long long *rejected, long long *batches, int *queued)
{
    if (!s) return IVR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    if (completed) *completed = s->completed;
    if (rejected) *rejected = s->rejected;
    if (batches) *batches = s->batches;
    if (queued) *queued = (int) s->queue.size();
    return IVR_OK;
}

int ivr_server_times(ivr_server *s, double *gpu_s, double *dispatch_s, double *finish_s)
{
    if (!s) return IVR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    if (gpu_s) *gpu_s = s->gpu_s;
    if (dispatch_s) *dispatch_s = s->dispatch_s;
    if (finish_s) *finish_s = s->finish_s;
    return IVR_OK;
}

int ivr_server_listen(ivr_server *s, int port, int volume, int tf, int *bound_port)
{
    if (!s || s->listen_fd >= 0 || volume < 0) return IVR_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (volume >= (int) s->vols.size()) return IVR_ERR_INVALID;
    }
    int fd = socket(AF_INET, SOCK_STREAM, 0);
    if (fd < 0) return IVR_ERR_IO;
    int one = 1;
    setsockopt(fd, SOL_SOCKET, SO_REUSEADDR, &one, sizeof(one));
    sockaddr_in a;
    memset(&a, 0, sizeof(a));
    a.sin_family = AF_INET;
    a.sin_addr.s_addr = htonl(INADDR_LOOPBACK);
    a.sin_port = htons((uint16_t) port);
    socklen_t len = sizeof(a);
    if (bind(fd, (sockaddr *) &a, sizeof(a)) != 0 || listen(fd, 64) != 0 ||
        getsockname(fd, (sockaddr *) &a, &len) != 0) {
        close(fd);
        return IVR_ERR_IO;
    }
    s->listen_fd = fd;
    s->net_volume = volume;
    s->net_tf = tf;
    if (bound_port) *bound_port = ntohs(a.sin_port);
    s->acceptor = std::thread(accept_loop, s);
    return IVR_OK;
}

int ivr_server_destroy(ivr_server *s)
{
    if (!s) return IVR_ERR_INVALID;
    if (s->listen_fd >= 0) {
        s->net_stop = true;
        shutdown(s->listen_fd, SHUT_RDWR);
        close(s->listen_fd);
        if (s->acceptor.joinable()) s->acceptor.join();
    }
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->sched.joinable()) s->sched.join();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->copier_stop = true;
    }
    s->cv_copy.notify_all();
    if (s->copier.joinable()) s->copier.join();
    std::vector<std::thread> conns;
    {
        // the queue is drained: wake connections waiting for a client's next
        // STATE, so that they end
        std::lock_guard<std::mutex> lock(s->mu);
        for (int fd : s->conn_fds) shutdown(fd, SHUT_RDWR);
        conns.swap(s->conns);
    }
    for (auto &t : conns)
        if (t.joinable()) t.join();
    for (auto &sl : s->slots) {
        for (auto *b : sl.batch)
            if (b) ivr_batch_free(b);
        for (auto *v : sl.views)
            if (v) ivr_view_free(v);
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.t0) cudaEventDestroy(sl.t0);
        if (sl.t1) cudaEventDestroy(sl.t1);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    if (s->pool) ivr_device_free(s->ctx, s->pool, s->pool_bytes);
    if (s->pool_pinned) cudaFreeHost(s->pool_pinned);
    for (auto *tf : s->tfs)
        if (tf) ivr_tf_free(tf);
    delete s;
    return IVR_OK;
}

}  // extern "C"
