// asv_server.cpp -- request pool on one GPU (include/asv.h, "serving").
//
// Clip requests wait in one FIFO; a worker thread per slot takes the first
// request it can admit (slot 0 only small clips when there are two or more
// slots): one of its own shape (its context keeps the device
// layout and the captured graph, no new memory), or one whose memory fits
// the free part of the HBM budget after the worker drops its current layout.
// Each slot's context runs on its own CUDA streams, so admitted requests
// overlap on the device; small clips run on a higher-priority stream than
// large ones, and streaming windows on the device's highest priority, so the
// block scheduler serves them first when the GPU is shared; the contexts
// launch the JFA with one block per tile, so no pass holds the SMs for its
// whole length and the priorities act between tiles.  A streaming
// session owns a resident streaming context and a worker that runs its
// windows in submission order.
#include "asv.h"
#include "asv_internal.h"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    asv_request r{};
    Clock::time_point t_submit, t_start, t_done;
    asv_status status = ASV_OK;
    bool done = false;
    int done_frames = 0;
    size_t bytes = 0;
};

struct Slot {
    asv_ctx *ctx = nullptr;
    int W = 0, H = 0, D = 0, K = 0;
    size_t bytes = 0;
    cudaStream_t small = nullptr, large = nullptr;   // priority streams for the two request classes
};

struct Session {
    asv_ctx *ctx = nullptr;
    size_t bytes = 0;
    std::deque<long long> q;
    std::thread th;
    cudaStream_t st = nullptr;                       // highest priority: windows are real-time
};

// clips up to this many voxels run on the slot's higher-priority stream, so
// their blocks are scheduled ahead of those of large clips sharing the GPU
const long long kSmallClipVoxels = 4LL << 20;

} // namespace

struct asv_server {
    asv_config cfg{};
    size_t budget = 0, used = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<long long> queue;
    std::map<long long, std::unique_ptr<Req>> reqs;
    std::vector<Slot> slots;
    std::vector<std::thread> workers;
    std::vector<std::unique_ptr<Session>> sessions;
    long long next_id = 1, submitted = 0, completed = 0, failed = 0;
    int running = 0;
    int prio_hi = 0;                  // greatest stream priority of the device
    bool stop = false;
};

static double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

static bool is_small(const asv_request &r) { return (long long)r.W * r.H * r.D <= kSmallClipVoxels; }

// with two or more slots, slot 0 serves small clips only: they are half of
// a typical mix but a few per cent of its GPU time, and would otherwise
// wait behind bursts of large clips holding every slot
static bool small_only(const asv_server *s, int w) { return w == 0 && s->slots.size() >= 2; }

// first queued request slot w can take; extra = new bytes it would need.  A
// request of the slot's own shape among the next few is preferred (no
// re-layout), then the first that fits the budget.
static bool pick(asv_server *s, int w, long long *id, size_t *extra)
{
    Slot &sl = s->slots[w];
    const bool small = small_only(s, w);
    size_t look = s->slots.size();
    for (auto it = s->queue.begin(); it != s->queue.end() && look; ++it, --look) {
        const asv_request &r = s->reqs[*it]->r;
        if (sl.ctx && r.W == sl.W && r.H == sl.H && r.D == sl.D && r.K == sl.K) {
            *id = *it; *extra = 0; s->queue.erase(it); return true;
        }
    }
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        Req &q = *s->reqs[*it];
        if (small && !is_small(q.r)) continue;
        size_t need = q.bytes;
        size_t freed = sl.bytes;
        if (!s->budget || s->used - freed + need <= s->budget) {
            *id = *it; *extra = need; s->queue.erase(it); return true;
        }
    }
    return false;
}

// the head request does not fit in the free part of the budget
static bool head_blocked(asv_server *s)
{
    if (!s->budget || s->queue.empty()) return false;
    return s->used + s->reqs[s->queue.front()]->bytes > s->budget;
}

static size_t held_by_slots(const asv_server *s)
{
    size_t b = 0;
    for (const Slot &sl : s->slots) b += sl.ctx ? sl.bytes + 1 : 0;
    return b;
}

static void worker(asv_server *s, int w)
{
    std::unique_lock<std::mutex> lk(s->mu);
    Slot &sl = s->slots[w];
    while (true) {
        long long id = 0;
        size_t extra = 0;
        while (!pick(s, w, &id, &extra)) {
            if (s->stop) return;
            if (!s->queue.empty() && sl.ctx && (!small_only(s, w) || head_blocked(s))) {
                // a queued request cannot be admitted and this slot's layout is
                // not wanted: give its memory back so the request can fit (the
                // small-clip slot keeps its layout unless the budget blocks)
                asv_ctx *c = sl.ctx;
                sl.ctx = nullptr;
                sl.W = sl.H = sl.D = sl.K = 0;
                lk.unlock();
                asv_destroy(c);
                lk.lock();
                s->used -= sl.bytes;
                sl.bytes = 0;
                s->cv_work.notify_all();
                continue;
            }
            if (!s->queue.empty() && s->running == 0 && held_by_slots(s) == 0) {
                // nothing runs and no slot holds memory: the head request can
                // never fit next to the open streaming sessions
                Req &q = *s->reqs[s->queue.front()];
                s->queue.pop_front();
                q.status = ASV_ERR_OVER_BUDGET;
                q.done = true;
                q.t_start = q.t_done = Clock::now();
                s->completed++;
                s->failed++;
                s->cv_done.notify_all();
                continue;
            }
            s->cv_work.wait(lk);
        }
        Req &q = *s->reqs[id];
        if (extra) {                    // the slot changes shape: account the new layout
            s->used = s->used - sl.bytes + extra;
            sl.bytes = extra;
        }
        s->running++;
        q.t_start = Clock::now();
        lk.unlock();
        asv_status st = ASV_OK;
        if (!sl.ctx) {
            asv_config c = s->cfg;
            c.stream = sl.large;
            st = asv_create(&c, &sl.ctx);
        }
        if (st == ASV_OK) {
            const asv_request &r = q.r;
            asv::set_stream(sl.ctx, is_small(r) ? sl.small : sl.large);
            st = asv_segment_clip(sl.ctx, r.rgb, r.fwd, r.bwd, r.W, r.H, r.D, r.K, r.labels_out);
            if (st == ASV_OK) { sl.W = r.W; sl.H = r.H; sl.D = r.D; sl.K = r.K; }
            else { sl.W = sl.H = sl.D = sl.K = 0; }
        }
        size_t held = asv::ctx_bytes(sl.ctx);
        lk.lock();
        s->used = s->used - sl.bytes + held;   // the estimate becomes what the context holds
        sl.bytes = held;
        q.status = st;
        q.done = true;
        q.t_done = Clock::now();
        s->running--;
        s->completed++;
        if (st != ASV_OK) s->failed++;
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

// A session's windows run in submission order.  Each window's frames are
// fed to the context's copy stream (asv_stream_feed), and so are those of
// the next queued window before this one is pushed, so that upload runs
// while this window computes.  A window whose feed is refused (e.g. the
// staging does not fit the budget) goes through asv_stream_push instead.
static void session_worker(asv_server *s, Session *ss)
{
    std::unique_lock<std::mutex> lk(s->mu);
    long long fed = -1;                        // the last request whose window is fed
    while (true) {
        s->cv_work.wait(lk, [&] { return s->stop || !ss->q.empty(); });
        if (ss->q.empty()) return;
        long long id = ss->q.front();
        ss->q.pop_front();
        Req &q = *s->reqs[id];
        const long long nid = ss->q.empty() ? -1 : ss->q.front();
        const Req *nq = nid >= 0 ? s->reqs[nid].get() : nullptr;   // alive until it is done
        s->running++;
        q.t_start = Clock::now();
        lk.unlock();
        const bool fed_this = fed == id || asv_stream_feed(ss->ctx, q.r.rgb, q.r.fwd, q.r.bwd) == ASV_OK;
        if (fed_this && nq && asv_stream_feed(ss->ctx, nq->r.rgb, nq->r.fwd, nq->r.bwd) == ASV_OK) fed = nid;
        int done = 0;
        asv_status st = fed_this ? asv_stream_push_fed(ss->ctx, q.r.labels_out, &done)
                                 : asv_stream_push(ss->ctx, q.r.rgb, q.r.fwd, q.r.bwd, q.r.labels_out, &done);
        lk.lock();
        q.status = st;
        q.done_frames = done;
        q.done = true;
        q.t_done = Clock::now();
        s->running--;
        s->completed++;
        if (st != ASV_OK) s->failed++;
        s->cv_done.notify_all();
    }
}

extern "C" {

asv_status asv_server_create(const asv_config *cfg, int max_slots, size_t hbm_budget, asv_server **out)
{
    if (!out || max_slots < 1 || max_slots > 256) return ASV_ERR_BAD_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return ASV_ERR_NO_DEVICE; }
    asv_server *s = new asv_server();
    if (cfg) s->cfg = *cfg; else asv_config_default(&s->cfg);
    s->cfg.stream = nullptr;          // every slot gets its own streams
    s->cfg.jfa_tile_blocks = 1;       // JFA blocks retire per tile: priorities can act between them
    s->budget = hbm_budget;
    s->slots.resize(max_slots);
    cudaSetDevice(s->cfg.device);
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    s->prio_hi = greatest;
    const int mid = (least + greatest) / 2;
    for (auto &sl : s->slots) {
        if (cudaStreamCreateWithPriority(&sl.small, cudaStreamNonBlocking, mid) != cudaSuccess ||
            cudaStreamCreateWithPriority(&sl.large, cudaStreamNonBlocking, least) != cudaSuccess) {
            cudaGetLastError();
            for (auto &t : s->slots) {
                if (t.small) cudaStreamDestroy(t.small);
                if (t.large) cudaStreamDestroy(t.large);
            }
            delete s;
            return ASV_ERR_CUDA;
        }
    }
    for (int w = 0; w < max_slots; w++) s->workers.emplace_back(worker, s, w);
    *out = s;
    return ASV_OK;
}

asv_status asv_server_destroy(asv_server *s)
{
    if (!s) return ASV_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    for (auto &ss : s->sessions) if (ss->th.joinable()) ss->th.join();
    {
        // requests no worker took end with ASV_ERR_STATE
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &kv : s->reqs)
            if (!kv.second->done) { kv.second->status = ASV_ERR_STATE; kv.second->done = true; }
        s->cv_done.notify_all();
    }
    for (auto &sl : s->slots) if (sl.ctx) asv_destroy(sl.ctx);
    for (auto &ss : s->sessions) if (ss->ctx) asv_destroy(ss->ctx);
    for (auto &sl : s->slots) {
        cudaStreamDestroy(sl.small);
        cudaStreamDestroy(sl.large);
    }
    for (auto &ss : s->sessions) if (ss->st) cudaStreamDestroy(ss->st);
    delete s;
    return ASV_OK;
}

asv_status asv_server_open_session(asv_server *s, int W, int H, int D_all, int K_video, int seeds_num_100,
                                   int block_size, int *session)
{
    if (!s || !session) return ASV_ERR_BAD_ARG;
    auto ss = std::make_unique<Session>();
    cudaSetDevice(s->cfg.device);
    if (cudaStreamCreateWithPriority(&ss->st, cudaStreamNonBlocking, s->prio_hi) != cudaSuccess) {
        cudaGetLastError();
        return ASV_ERR_CUDA;
    }
    asv_config c = s->cfg;
    c.use_graph = 0;
    c.stream = ss->st;
    asv_status st = asv_create(&c, &ss->ctx);
    if (st != ASV_OK) { cudaStreamDestroy(ss->st); return st; }
    st = asv_stream_begin(ss->ctx, W, H, D_all, K_video, seeds_num_100, block_size);
    if (st != ASV_OK) { asv_destroy(ss->ctx); cudaStreamDestroy(ss->st); return st; }
    ss->bytes = asv::ctx_bytes(ss->ctx);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->budget && s->used + ss->bytes > s->budget) {
        asv_destroy(ss->ctx);
        cudaStreamDestroy(ss->st);
        return ASV_ERR_OVER_BUDGET;
    }
    s->used += ss->bytes;
    Session *raw = ss.get();
    s->sessions.push_back(std::move(ss));
    raw->th = std::thread(session_worker, s, raw);
    *session = (int)s->sessions.size() - 1;
    return ASV_OK;
}

asv_status asv_server_submit(asv_server *s, const asv_request *req, long long *id)
{
    if (!s || !req || !id) return ASV_ERR_BAD_ARG;
    if (!req->rgb || !req->labels_out || (!req->fwd) != (!req->bwd)) return ASV_ERR_BAD_ARG;
    auto q = std::make_unique<Req>();
    q->r = *req;
    q->t_submit = Clock::now();
    if (req->kind == ASV_REQ_CLIP) {
        q->bytes = asv_clip_bytes(req->W, req->H, req->D, req->K);
        if (!q->bytes) return ASV_ERR_BAD_ARG;
        if (s->budget && q->bytes > s->budget) return ASV_ERR_OVER_BUDGET;
    } else if (req->kind != ASV_REQ_WINDOW) {
        return ASV_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (req->kind == ASV_REQ_WINDOW && (req->session < 0 || req->session >= (int)s->sessions.size()))
        return ASV_ERR_BAD_ARG;
    long long k = s->next_id++;
    s->reqs[k] = std::move(q);
    if (req->kind == ASV_REQ_CLIP) s->queue.push_back(k);
    else s->sessions[req->session]->q.push_back(k);
    s->submitted++;
    *id = k;
    s->cv_work.notify_all();
    return ASV_OK;
}

asv_status asv_server_wait(asv_server *s, long long id, double *latency_ms, double *queue_ms,
                           int *done_frames)
{
    if (!s) return ASV_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return ASV_ERR_BAD_ARG;
    Req &q = *it->second;
    s->cv_done.wait(lk, [&] { return q.done; });
    if (latency_ms) *latency_ms = ms_between(q.t_submit, q.t_done);
    if (queue_ms) *queue_ms = ms_between(q.t_submit, q.t_start);
    if (done_frames) *done_frames = q.done_frames;
    return q.status;
}

asv_status asv_server_poll(asv_server *s, long long id, int *done)
{
    if (!s || !done) return ASV_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return ASV_ERR_BAD_ARG;
    *done = it->second->done ? 1 : 0;
    return ASV_OK;
}

asv_status asv_server_get_stats(asv_server *s, asv_server_stats *st)
{
    if (!s || !st) return ASV_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->failed = s->failed;
    st->queued = (long long)s->queue.size();
    for (auto &ss : s->sessions) st->queued += (long long)ss->q.size();
    st->running = s->running;
    st->bytes_in_use = s->used;
    st->budget = s->budget;
    st->slots = (int)s->slots.size();
    st->sessions = (int)s->sessions.size();
    return ASV_OK;
}

} // extern "C"
