// server.cu — request server for concurrent SLAM sessions with continuous
// batching.  No counterpart in the reference, which runs one session
// (FullSystem/src/System.cpp:43-65 drives Tracking::GrabImageRGBD per frame).
//
// Clients submit frames (host RGB + depth) for their session at any time;
// each frame is copied into the session's pinned input ring.  One worker
// thread runs the loop:
//   1. completed frames (session event done) become results, with their
//      latency from submission to completion;
//   2. every session with a queued frame and none in flight takes it;
//   3. a taken frame starts at once on its session's stream: input copy and
//      the first half of the frame (pyramids, raycast, model pyramid; a
//      captured graph);
//   4. whenever fewer than two batched Gauss-Newton launches are pending on
//      the server's GN stream, every session whose first half is queued joins
//      one batched launch; the second halves (pose update, fusion, frame
//      state to the host) follow on the session streams.
//      With gn_per_session set, a taken frame instead gets its own GN launch
//      (a one-session batch of a fixed CTA share) and its second half on its
//      session's stream as soon as its share fits: frames take the GPU in the
//      order their first halves were launched, and the shares of the GN
//      launches that may be running never exceed the co-resident CTAs, so
//      every cooperative grid can be resident at once.  No session waits for
//      others to gather.
// Frames that arrive while others are on the GPU start at once and their
// work overlaps with the running batch; under load the batches grow.  Each session keeps
// its map, pyramids and buffers device resident; a session is admitted only
// if its estimated device footprint fits the free HBM minus a reserve.
//
// A session's computations are the same alone and in any batch: it takes a
// fixed CTA count in the batched launch and folds only its own rows.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "yas_session.h"

using namespace yas;

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct QueuedFrame {
    int slot;                   // input ring slot
    long long index;            // frame number within the session
    Clock::time_point arrival;  // submission time
};

struct ServedSession {
    int id = -1;
    yas_session *s = nullptr;
    int w = 0, h = 0;
    int ring = 0;
    uint8_t *rgb = nullptr;    // pinned, ring * w * h * 3
    uint16_t *depth = nullptr; // pinned, ring * w * h
    std::vector<bool> slot_used;
    std::deque<QueuedFrame> queue;
    bool in_flight = false;
    bool awaiting_gn = false;  // first half launched, GN not yet dispatched
    QueuedFrame cur{};
    cudaEvent_t ev_pre = nullptr, ev_done = nullptr;
    GNBatchItem *d_own = nullptr;  // gn_per_session: the session's descriptor per frame parity
    GNBatchItem *h_own = nullptr;  // pinned source of d_own, written once per parity
    bool own_ready[2] = {false, false};
    int own_ctas = 0, own_pix = 0;
    cudaEvent_t ev_gn = nullptr;  // after the session's own GN launch
    bool gn_running = false;      // its share counts against the co-resident CTAs
    long long submitted = 0, completed = 0;
    bool closing = false;
    bool suspended = false;  // map swapped out to host memory; frames wait in the queue
};

// Device footprint of a session with this configuration (map, pyramids,
// tracker scratch, raycaster and frame buffers), for admission.
size_t session_bytes_estimate(const yas_session_config &c) {
    const size_t vbytes = c.map.voxel_format == YAS_VOXEL_F32 ? 8 : 4;
    const size_t map = (size_t)c.map.hash_slots * 16 + (size_t)c.map.max_blocks * (12 + 512 * vbytes);
    size_t P = 0;
    for (int l = 0; l < std::max(1, c.num_levels); ++l) P += (size_t)(c.width >> l) * (c.height >> l);
    const size_t P0 = (size_t)c.width * c.height;
    const size_t pyramids = 88 * P;                       // two frame sets + gradients
    const size_t frame = P0 * (16 + 4 + 16 + 4 + 3 + 2 + 4); // residuals, staging, vmap, depth, inputs
    return map + pyramids + frame + (8u << 20);            // + tracker rows, graphs, small buffers
}

}  // namespace

struct yas_server {
    yas_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::vector<ServedSession *> sessions;  // by id; nullptr once closed
    std::deque<yas_served_result> results;
    std::vector<double> latencies;          // ms, since the last stats reset
    long long batches = 0, batched_frames = 0;
    Clock::time_point first_submit{}, last_done{};
    bool have_first = false;
    std::atomic<bool> stop{false};
    std::thread worker;
    int worker_error = YAS_OK;
    // batched GN launch
    cudaStream_t gn_stream = nullptr;
    static constexpr int kDesc = 4;  // descriptor buffers in rotation
    GNBatchItem *h_items[kDesc] = {}, *d_items[kDesc] = {};
    unsigned short *h_map[kDesc] = {}, *d_map[kDesc] = {};
    cudaEvent_t gn_done[kDesc] = {};  // after each buffer's batched GN launch
    std::deque<int> pending_gn;
    int desc_next = 0;
    int capacity = 0;  // co-resident CTAs of the batched launch
    int max_items = 0;
    unsigned short *d_zero_map = nullptr;  // gn_per_session: every CTA serves item 0
    std::deque<ServedSession *> own_wait;  // gn_per_session: first halves launched, in order
    int own_ctas_running = 0;              // shares of the own GN launches not known finished
};

namespace {

// Finished frames become results (caller holds the lock).  Returns true if
// any frame finished.
bool collect_done(yas_server *srv) {
    bool any = false;
    for (ServedSession *ss : srv->sessions) {
        // a tracked frame is done only after its second half was launched
        if (!ss || !ss->in_flight || ss->awaiting_gn) continue;
        const cudaError_t q = cudaEventQuery(ss->ev_done);
        if (q == cudaErrorNotReady) continue;
        const Clock::time_point now = Clock::now();
        yas_served_result r;
        memset(&r, 0, sizeof(r));
        r.session = ss->id;
        r.frame = ss->cur.index;
        r.latency_ms = ms_since(ss->cur.arrival, now);
        if (q == cudaSuccess) {
            session_result(ss->s, &r.Tcm, &r.status);
        } else {
            record_cuda_error(q, "served frame", __FILE__, __LINE__);
            r.status = YAS_ERR_CUDA;
        }
        if (srv->results.size() >= (1u << 20)) srv->results.pop_front();
        srv->results.push_back(r);
        srv->latencies.push_back(r.latency_ms);
        srv->last_done = now;
        ss->slot_used[ss->cur.slot] = false;
        ss->in_flight = false;
        if (ss->gn_running) {  // its GN ran before its second half on the same stream
            ss->gn_running = false;
            srv->own_ctas_running -= ss->own_ctas;
        }
        ss->completed++;
        any = true;
    }
    return any;
}

int launch_first(ServedSession *ss) {
    ss->cur = ss->queue.front();
    ss->queue.pop_front();
    const size_t n = (size_t)ss->w * ss->h;
    YAS_TRY(session_copy_input(ss->s, ss->rgb + ss->cur.slot * n * 3, ss->depth + ss->cur.slot * n, 0));
    YAS_TRY(session_launch_first(ss->s));
    YAS_TRY_CUDA(cudaEventRecord(ss->ev_done, session_stream(ss->s)));
    ss->in_flight = true;
    return YAS_OK;
}

// First half of a tracked frame on the session's stream, as soon as the
// frame is taken: input copy, pyramids, raycast, model pyramid, GN reset.
int launch_pre_frame(ServedSession *ss) {
    ss->cur = ss->queue.front();
    ss->queue.pop_front();
    const size_t n = (size_t)ss->w * ss->h;
    YAS_TRY(session_copy_input(ss->s, ss->rgb + ss->cur.slot * n * 3, ss->depth + ss->cur.slot * n, 0));
    YAS_TRY(session_launch_pre(ss->s));
    YAS_TRY_CUDA(cudaEventRecord(ss->ev_pre, session_stream(ss->s)));
    ss->in_flight = true;
    ss->awaiting_gn = true;
    return YAS_OK;
}

// CTA share of a session's own GN launch: by default one CTA per 16 K pixels
// of level 0, at most kOwnMaxCtas.
constexpr int kOwnPixelsPerCta = 16384;
constexpr int kOwnMaxCtas = 32;

// gn_per_session: the frame's own GN launch right after its first half, then
// its second half, all on the session's stream.  The descriptor of each frame
// parity names the tracker's fixed buffers, so it is built once.
int own_share(yas_server *srv, ServedSession *ss) {
    const long long ppc = srv->cfg.gn_pixels_per_cta > 0 ? srv->cfg.gn_pixels_per_cta : kOwnPixelsPerCta;
    const long long n = ((long long)ss->w * ss->h + ppc - 1) / ppc;
    return (int)std::min<long long>(std::min(srv->capacity, kOwnMaxCtas), std::max(1LL, n));
}

int launch_own_gn(yas_server *srv, ServedSession *ss) {
    yas_tracker *tr = session_tracker(ss->s);
    const int p = tr->cur;
    cudaStream_t st = session_stream(ss->s);
    if (!ss->own_ready[p]) {
        // the copy is ordered on the session stream before the launch that reads it
        GNBatchItem &it = ss->h_own[p];
        gn_batch_item_ctas(tr, 0, own_share(srv, ss), &it);
        YAS_TRY_CUDA(cudaMemcpyAsync(ss->d_own + p, &it, sizeof(it), cudaMemcpyHostToDevice, st));
        ss->own_ctas = it.nctas;
        ss->own_pix = gn_batch_pix(&it, 1);
        ss->own_ready[p] = true;
    }
    YAS_TRY_CUDA(launch_gn_batch(ss->d_own + p, srv->d_zero_map, ss->own_ctas, st, ss->own_pix));
    YAS_TRY_CUDA(cudaEventRecord(ss->ev_gn, st));
    ss->gn_running = true;
    srv->own_ctas_running += ss->own_ctas;
    YAS_TRY(session_launch_post(ss->s));
    YAS_TRY_CUDA(cudaEventRecord(ss->ev_done, st));
    ss->awaiting_gn = false;
    srv->batches++;
    srv->batched_frames++;
    return YAS_OK;
}

// gn_per_session: frees the shares of finished GN launches, then launches the
// waiting frames' GN in order while their shares fit.
int dispatch_own(yas_server *srv, bool &launched) {
    for (ServedSession *ss : srv->sessions) {
        if (!ss || !ss->gn_running || cudaEventQuery(ss->ev_gn) == cudaErrorNotReady) continue;
        ss->gn_running = false;
        srv->own_ctas_running -= ss->own_ctas;
    }
    while (!srv->own_wait.empty()) {
        ServedSession *ss = srv->own_wait.front();
        if (srv->own_ctas_running + own_share(srv, ss) > srv->capacity) break;
        srv->own_wait.pop_front();
        YAS_TRY(launch_own_gn(srv, ss));
        launched = true;
    }
    return YAS_OK;
}

// One batched Gauss-Newton launch for every session whose first half is
// queued, then their second halves (pose update, fusion, frame state).
int dispatch_gn(yas_server *srv, const std::vector<ServedSession *> &batch) {
    const int k = srv->desc_next;
    srv->desc_next = (k + 1) % yas_server::kDesc;
    // buffer k's previous batch has finished (its descriptors were consumed)
    YAS_TRY_CUDA(cudaEventSynchronize(srv->gn_done[k]));
    int cta0 = 0;
    for (size_t i = 0; i < batch.size(); ++i) {
        ServedSession *ss = batch[i];
        GNBatchItem &it = srv->h_items[k][i];
        gn_batch_item(session_tracker(ss->s), cta0, &it);
        for (int c = 0; c < it.nctas; ++c) srv->h_map[k][cta0 + c] = (unsigned short)i;
        cta0 += it.nctas;
        YAS_TRY_CUDA(cudaStreamWaitEvent(srv->gn_stream, ss->ev_pre, 0));
    }
    YAS_TRY_CUDA(cudaMemcpyAsync(srv->d_items[k], srv->h_items[k], batch.size() * sizeof(GNBatchItem),
                                 cudaMemcpyHostToDevice, srv->gn_stream));
    YAS_TRY_CUDA(cudaMemcpyAsync(srv->d_map[k], srv->h_map[k], (size_t)cta0 * sizeof(unsigned short),
                                 cudaMemcpyHostToDevice, srv->gn_stream));
    YAS_TRY_CUDA(launch_gn_batch(srv->d_items[k], srv->d_map[k], cta0, srv->gn_stream,
                                 gn_batch_pix(srv->h_items[k], (int)batch.size())));
    YAS_TRY_CUDA(cudaEventRecord(srv->gn_done[k], srv->gn_stream));
    for (ServedSession *ss : batch) {
        cudaStream_t st = session_stream(ss->s);
        YAS_TRY_CUDA(cudaStreamWaitEvent(st, srv->gn_done[k], 0));
        YAS_TRY(session_launch_post(ss->s));
        YAS_TRY_CUDA(cudaEventRecord(ss->ev_done, st));
        ss->awaiting_gn = false;
    }
    srv->pending_gn.push_back(k);
    srv->batches++;
    srv->batched_frames += (long long)batch.size();
    return YAS_OK;
}

// Batched GN launches not yet finished (caller holds the lock).
int pending_gn(yas_server *srv) {
    while (!srv->pending_gn.empty() && cudaEventQuery(srv->gn_done[srv->pending_gn.front()]) == cudaSuccess)
        srv->pending_gn.pop_front();
    return (int)srv->pending_gn.size();
}

void worker_main(yas_server *srv) {
    cudaSetDevice(srv->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    std::vector<ServedSession *> batch;
    while (!srv->stop.load()) {
        if (collect_done(srv)) srv->cv.notify_all();
        int st = YAS_OK;
        bool launched = false, busy = false;
        // every session with a queued frame and none in flight starts it now
        for (ServedSession *ss : srv->sessions) {
            if (!ss) continue;
            if (!ss->closing && !ss->suspended && !ss->in_flight && !ss->queue.empty() && st == YAS_OK) {
                st = session_needs_init(ss->s) ? launch_first(ss) : launch_pre_frame(ss);
                if (st == YAS_OK && ss->awaiting_gn && srv->cfg.gn_per_session) srv->own_wait.push_back(ss);
                launched = true;
            }
            busy = busy || ss->in_flight;
        }
        if (st == YAS_OK && srv->cfg.gn_per_session) st = dispatch_own(srv, launched);
        // the waiting sessions form the next GN batch once fewer than two
        // batches are on the GN stream (while one runs, the next gathers)
        if (st == YAS_OK && !srv->cfg.gn_per_session && pending_gn(srv) < 2) {
            batch.clear();
            int ctas = 0;
            for (ServedSession *ss : srv->sessions) {
                if (!ss || !ss->awaiting_gn) continue;
                const int c = gn_batch_ctas(session_tracker(ss->s));
                if (ctas + c > srv->capacity || (int)batch.size() >= srv->max_items) continue;
                ctas += c;
                batch.push_back(ss);
            }
            if (!batch.empty()) {
                st = dispatch_gn(srv, batch);
                launched = true;
            }
        }
        if (st != YAS_OK) {
            srv->worker_error = st;
            srv->stop.store(true);
            break;
        }
        if (launched) continue;
        if (busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(10));
            lk.lock();
        } else {
            srv->cv.wait_for(lk, std::chrono::milliseconds(2));
        }
    }
    srv->cv.notify_all();
}

}  // namespace

extern "C" {

YAS_API int yas_server_config_default(yas_server_config *cfg) {
    if (!cfg) return YAS_ERR_BAD_ARG;
    memset(cfg, 0, sizeof(*cfg));
    cfg->max_sessions = 64;
    cfg->hbm_reserve_bytes = (size_t)4 << 30;
    cfg->ring_frames = 4;
    cfg->gn_per_session = 1;
    cfg->gn_pixels_per_cta = 0;
    return YAS_OK;
}

YAS_API int yas_server_create(yas_server **out, const yas_server_config *cfg) {
    if (!out || !cfg || cfg->max_sessions <= 0 || cfg->ring_frames <= 0) return YAS_ERR_BAD_ARG;
    *out = nullptr;
    yas_server *srv = new yas_server();
    srv->cfg = *cfg;
    cudaGetDevice(&srv->device);
    srv->capacity = gn_batch_capacity();
    srv->max_items = std::min(cfg->max_sessions, 1024);
    bool ok = srv->capacity > 0 && cudaStreamCreateWithFlags(&srv->gn_stream, cudaStreamNonBlocking) == cudaSuccess;
    for (int k = 0; ok && k < yas_server::kDesc; ++k)
        ok = cudaMallocHost(&srv->h_items[k], srv->max_items * sizeof(GNBatchItem)) == cudaSuccess &&
             cudaMalloc(&srv->d_items[k], srv->max_items * sizeof(GNBatchItem)) == cudaSuccess &&
             cudaMallocHost(&srv->h_map[k], srv->capacity * sizeof(unsigned short)) == cudaSuccess &&
             cudaMalloc(&srv->d_map[k], srv->capacity * sizeof(unsigned short)) == cudaSuccess &&
             cudaEventCreateWithFlags(&srv->gn_done[k], cudaEventDisableTiming) == cudaSuccess;
    // zeroed before any session stream can read it
    ok = ok && cudaMalloc(&srv->d_zero_map, srv->capacity * sizeof(unsigned short)) == cudaSuccess &&
         cudaMemsetAsync(srv->d_zero_map, 0, srv->capacity * sizeof(unsigned short), srv->gn_stream) == cudaSuccess &&
         cudaStreamSynchronize(srv->gn_stream) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        const int code = srv->capacity <= 0 ? YAS_ERR_STATE : YAS_ERR_OOM;
        yas_server_destroy(srv);
        return code;
    }
    srv->worker = std::thread(worker_main, srv);
    *out = srv;
    return YAS_OK;
}

YAS_API int yas_server_open_session(yas_server *srv, const yas_session_config *cfg, int *out_id) {
    if (!srv || !cfg || !out_id || cfg->width <= 0 || cfg->height <= 0) return YAS_ERR_BAD_ARG;
    static std::mutex open_mu;  // admission decisions one at a time
    std::lock_guard<std::mutex> og(open_mu);
    {
        std::lock_guard<std::mutex> g(srv->mu);
        int live = 0;
        for (ServedSession *ss : srv->sessions) live += ss ? 1 : 0;
        if (live >= srv->cfg.max_sessions) return YAS_ERR_CAPACITY;
    }
    cudaSetDevice(srv->device);
    size_t free_b = 0, total_b = 0;
    YAS_TRY_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (free_b < session_bytes_estimate(*cfg) + srv->cfg.hbm_reserve_bytes) return YAS_ERR_OOM;  // not admitted
    ServedSession *ss = new ServedSession();
    int st = yas_session_create(&ss->s, cfg, nullptr);
    ss->w = cfg->width;
    ss->h = cfg->height;
    ss->ring = srv->cfg.ring_frames;
    ss->slot_used.assign(ss->ring, false);
    const size_t n = (size_t)ss->w * ss->h;
    if (st == YAS_OK &&
        (cudaMallocHost(&ss->rgb, ss->ring * n * 3) != cudaSuccess ||
         cudaMallocHost(&ss->depth, ss->ring * n * 2) != cudaSuccess ||
         cudaEventCreateWithFlags(&ss->ev_pre, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&ss->ev_done, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&ss->ev_gn, cudaEventDisableTiming) != cudaSuccess ||
         cudaMalloc(&ss->d_own, 2 * sizeof(GNBatchItem)) != cudaSuccess ||
         cudaMallocHost(&ss->h_own, 2 * sizeof(GNBatchItem)) != cudaSuccess)) {
        cudaGetLastError();
        st = YAS_ERR_OOM;
    }
    if (st != YAS_OK) {
        if (ss->s) yas_session_destroy(ss->s);
        if (ss->rgb) cudaFreeHost(ss->rgb);
        if (ss->depth) cudaFreeHost(ss->depth);
        if (ss->ev_pre) cudaEventDestroy(ss->ev_pre);
        if (ss->ev_done) cudaEventDestroy(ss->ev_done);
        if (ss->ev_gn) cudaEventDestroy(ss->ev_gn);
        if (ss->d_own) cudaFree(ss->d_own);
        if (ss->h_own) cudaFreeHost(ss->h_own);
        delete ss;
        return st;
    }
    std::lock_guard<std::mutex> g(srv->mu);
    ss->id = (int)srv->sessions.size();
    srv->sessions.push_back(ss);
    *out_id = ss->id;
    return YAS_OK;
}

// Session eviction and resumption (MapStruct::Hibernate / ReActivate,
// VoxelMap.cu:894-954): the map's device arrays go to host memory and back.
YAS_API int yas_server_suspend_session(yas_server *srv, int id) {
    if (!srv) return YAS_ERR_BAD_ARG;
    ServedSession *ss = nullptr;
    {
        std::unique_lock<std::mutex> lk(srv->mu);
        if (id < 0 || id >= (int)srv->sessions.size() || !srv->sessions[id]) return YAS_ERR_BAD_ARG;
        ss = srv->sessions[id];
        if (ss->suspended) return YAS_OK;
        ss->suspended = true;  // the worker starts no new frame of it
        srv->cv.wait(lk, [&] { return !ss->in_flight || srv->stop.load(); });
    }
    cudaSetDevice(srv->device);
    YAS_TRY_CUDA(cudaStreamSynchronize(session_stream(ss->s)));
    yas_map *m = nullptr;
    YAS_TRY(yas_session_map(ss->s, &m));
    return yas_map_hibernate(m);
}

YAS_API int yas_server_resume_session(yas_server *srv, int id) {
    if (!srv) return YAS_ERR_BAD_ARG;
    ServedSession *ss = nullptr;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        if (id < 0 || id >= (int)srv->sessions.size() || !srv->sessions[id]) return YAS_ERR_BAD_ARG;
        ss = srv->sessions[id];
        if (!ss->suspended) return YAS_OK;
    }
    cudaSetDevice(srv->device);
    yas_map *m = nullptr;
    YAS_TRY(yas_session_map(ss->s, &m));
    // admission: the map's arrays must fit the free HBM minus the reserve
    size_t free_b = 0, total_b = 0;
    YAS_TRY_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t vb = m->cfg.voxel_format == YAS_VOXEL_F32 ? 8 : 4;
    const size_t need = (size_t)m->cfg.hash_slots * sizeof(HashSlot) + (size_t)m->cfg.max_blocks * (12 + kBlockVoxels * vb);
    if (free_b < need + srv->cfg.hbm_reserve_bytes) return YAS_ERR_OOM;
    YAS_TRY(yas_map_reactivate(m));
    {
        std::lock_guard<std::mutex> g(srv->mu);
        ss->suspended = false;
    }
    srv->cv.notify_all();
    return YAS_OK;
}

YAS_API int yas_server_close_session(yas_server *srv, int id) {
    if (!srv) return YAS_ERR_BAD_ARG;
    ServedSession *ss = nullptr;
    {
        std::unique_lock<std::mutex> lk(srv->mu);
        if (id < 0 || id >= (int)srv->sessions.size() || !srv->sessions[id]) return YAS_ERR_BAD_ARG;
        ss = srv->sessions[id];
        ss->closing = true;
        for (const QueuedFrame &q : ss->queue) ss->slot_used[q.slot] = false;
        ss->queue.clear();
        srv->cv.wait(lk, [&] { return !ss->in_flight || srv->stop.load(); });
        srv->sessions[id] = nullptr;
    }
    cudaStreamSynchronize(session_stream(ss->s));
    yas_session_destroy(ss->s);
    cudaFreeHost(ss->rgb);
    cudaFreeHost(ss->depth);
    cudaEventDestroy(ss->ev_pre);
    cudaEventDestroy(ss->ev_done);
    cudaEventDestroy(ss->ev_gn);
    cudaFree(ss->d_own);
    cudaFreeHost(ss->h_own);
    delete ss;
    return YAS_OK;
}

YAS_API int yas_server_submit(yas_server *srv, int id, const uint8_t *rgb, const uint16_t *depth) {
    if (!srv || !rgb || !depth) return YAS_ERR_BAD_ARG;
    const Clock::time_point arrival = Clock::now();
    ServedSession *ss = nullptr;
    int slot = -1;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        if (srv->worker_error != YAS_OK) return srv->worker_error;
        if (id < 0 || id >= (int)srv->sessions.size() || !srv->sessions[id] || srv->sessions[id]->closing)
            return YAS_ERR_BAD_ARG;
        ss = srv->sessions[id];
        for (int i = 0; i < ss->ring; ++i)
            if (!ss->slot_used[i]) {
                slot = i;
                break;
            }
        if (slot < 0) return YAS_ERR_CAPACITY;  // the session's input ring is full
        ss->slot_used[slot] = true;
    }
    const size_t n = (size_t)ss->w * ss->h;
    memcpy(ss->rgb + slot * n * 3, rgb, n * 3);
    memcpy(ss->depth + slot * n, depth, n * 2);
    {
        std::lock_guard<std::mutex> g(srv->mu);
        ss->queue.push_back(QueuedFrame{slot, ss->submitted++, arrival});
        if (!srv->have_first) {
            srv->first_submit = arrival;
            srv->have_first = true;
        }
    }
    srv->cv.notify_all();
    return YAS_OK;
}

YAS_API int yas_server_poll(yas_server *srv, yas_served_result *out, int capacity, int *out_count) {
    if (!srv || !out_count || (capacity > 0 && !out)) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    int n = 0;
    while (n < capacity && !srv->results.empty()) {
        out[n++] = srv->results.front();
        srv->results.pop_front();
    }
    *out_count = n;
    return srv->worker_error;
}

YAS_API int yas_server_drain(yas_server *srv, double timeout_s) {
    if (!srv) return YAS_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto idle = [&] {
        if (srv->stop.load()) return true;
        for (ServedSession *ss : srv->sessions)
            if (ss && (ss->in_flight || !ss->queue.empty())) return false;
        return true;
    };
    if (!srv->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), idle)) return YAS_ERR_TIMEOUT;
    return srv->worker_error;
}

YAS_API int yas_server_get_stats(yas_server *srv, yas_server_stats *out) {
    if (!srv || !out) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    memset(out, 0, sizeof(*out));
    std::vector<double> v = srv->latencies;
    out->frames = (long long)v.size();
    out->batches = srv->batches;
    out->mean_batch = srv->batches ? (double)srv->batched_frames / (double)srv->batches : 0.0;
    if (!v.empty()) {
        const auto pct = [&](double p) {
            size_t i = std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5));
            std::nth_element(v.begin(), v.begin() + i, v.end());
            return v[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = *std::max_element(v.begin(), v.end());
        const double span = ms_since(srv->first_submit, srv->last_done);
        out->fps = span > 0.0 ? 1000.0 * (double)v.size() / span : 0.0;
    }
    return YAS_OK;
}

YAS_API int yas_server_reset_stats(yas_server *srv) {
    if (!srv) return YAS_ERR_BAD_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    srv->latencies.clear();
    srv->batches = 0;
    srv->batched_frames = 0;
    srv->have_first = false;
    return YAS_OK;
}

YAS_API int yas_server_destroy(yas_server *srv) {
    if (!srv) return YAS_ERR_BAD_ARG;
    srv->stop.store(true);
    srv->cv.notify_all();
    if (srv->worker.joinable()) srv->worker.join();
    for (size_t i = 0; i < srv->sessions.size(); ++i) {
        ServedSession *ss = srv->sessions[i];
        if (!ss) continue;
        cudaStreamSynchronize(session_stream(ss->s));
        yas_session_destroy(ss->s);
        cudaFreeHost(ss->rgb);
        cudaFreeHost(ss->depth);
        cudaEventDestroy(ss->ev_pre);
        cudaEventDestroy(ss->ev_done);
        cudaEventDestroy(ss->ev_gn);
        cudaFree(ss->d_own);
        cudaFreeHost(ss->h_own);
        delete ss;
    }
    if (srv->gn_stream) cudaStreamSynchronize(srv->gn_stream);
    for (int k = 0; k < yas_server::kDesc; ++k) {
        if (srv->h_items[k]) cudaFreeHost(srv->h_items[k]);
        if (srv->d_items[k]) cudaFree(srv->d_items[k]);
        if (srv->h_map[k]) cudaFreeHost(srv->h_map[k]);
        if (srv->d_map[k]) cudaFree(srv->d_map[k]);
        if (srv->gn_done[k]) cudaEventDestroy(srv->gn_done[k]);
    }
    if (srv->d_zero_map) cudaFree(srv->d_zero_map);
    if (srv->gn_stream) cudaStreamDestroy(srv->gn_stream);
    delete srv;
    return YAS_OK;
}

}  // extern "C"
