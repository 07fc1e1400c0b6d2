// h264r_server.cu — continuous-batching server (include/h264r_server.h).
//
// Host code only.  One scheduler thread per server owns every call into the
// engine; the API calls (open / push / end / poll) only touch the server's
// queues under its mutex, so a parser thread per stream can feed it.
//
// A picture moves through three queues of its stream:
//   host_q  records validated and packed in host memory (push)
//   dev_q   records uploaded into one of the stream's device slots
//           (pinned staging + an H2D copy on the server's upload stream)
//   flight  launched in a batch; done when the event recorded after its
//           launch (and its output copy) completes
// Each pass of the scheduler admits waiting streams whose DPB fits the
// budget, retires finished pictures, uploads queued records, and launches,
// in each lane, one batch with the next dependency group of every stream of
// the lane that has one uploaded: continuous batching.  The streams are
// split into lanes by id; a batch waits for the earlier work of its
// streams, so the batches of one lane follow each other while the lanes'
// batches run side by side (at most two in flight per lane).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/h264r_server.h"

namespace {

constexpr uint64_t kAlign = 256;
constexpr int kLanes = 6;               // default batch chains over disjoint stream sets
                                        // (x 2 in flight: within the engine's launch ring of 16)
constexpr int kMaxLanes = 8;
constexpr int kMaxBatchesInFlight = 2;  // per lane
constexpr int kMaxGroupsInFlight = 2;   // per stream
constexpr size_t kIdleMax = 64;         // engine streams kept for reuse

uint64_t align_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Slot {
    uint8_t *dev = nullptr;   // device records
    uint64_t cap = 0;
    bool busy = false;
};

// pinned host buffer holding one picture's packed records
struct Pinned {
    uint8_t *ptr = nullptr;
    uint64_t cap = 0;
};

struct Item {
    Pinned blob;                // packed records: mbs | slices | weights | motion | coef | pcm
    uint64_t size = 0;
    uint64_t off[6] = {0, 0, 0, 0, 0, 0};
    h264r_picture pic{};        // sizes, flags and scaling lists (pointers set on upload)
    int group = 0;
    uint64_t tag = 0;
    uint8_t *out = nullptr;
    double t_push = 0;
    int slot = -1;
    uint64_t up_seq = 0;  // order of its upload on the server's upload stream
    cudaEvent_t uploaded = nullptr, done = nullptr;
};

struct SStream {
    int id = 0;
    h264r_stream_cfg cfg{};
    uint64_t dpb = 0;
    h264r_stream *s = nullptr;
    bool admitted = false, ended = false, finished = false;
    int status = 0;
    int pending = 0;  // pushed, not yet polled
    bool check = false;  // a batch of the stream completed: its finished pictures are looked for
    std::deque<Item *> host_q, dev_q, flight;
    std::vector<Slot> slots;
    int groups_in_flight() const
    {
        int n = 0, last = -1;
        bool first = true;
        for (const Item *it : flight) {
            if (first || it->group != last) n++;
            last = it->group;
            first = false;
        }
        return n;
    }
};

}  // namespace

struct h264r_server {
    h264r_ctx *ctx = nullptr;
    int device = 0;
    uint64_t budget = 0;
    int max_batch = 64, depth = 4, lanes = kLanes;
    std::mutex mu;
    std::condition_variable wake, done_cv;
    std::map<int, SStream *> streams;
    std::vector<SStream *> active;  // admitted and not finished: what a scheduler pass visits
    // engine streams of finished requests by geometry, reused (reset) for the
    // next request of the same geometry instead of a close and an open
    std::multimap<uint64_t, h264r_stream *> idle;
    std::deque<SStream *> waiting;
    std::deque<h264r_server_done> done_q;
    std::vector<double> lat;
    h264r_server_stats st{};
    // per lane, the batches in flight: the event after each and its streams
    struct Batch {
        cudaEvent_t done = nullptr;
        std::vector<SStream *> members;
    };
    std::deque<Batch> batch_done[kMaxLanes];
    std::vector<cudaEvent_t> ev_pool;
    cudaStream_t up = nullptr;
    uint64_t up_seq = 0;
    // per lane: the CUDA stream every batch of the lane runs on (so that a
    // stream's batches follow each other with no per-member events) and the
    // one its output copies run on
    cudaStream_t lane_cs[kMaxLanes] = {}, lane_copy[kMaxLanes] = {};
    // device slots for uploaded records: stream-ordered allocations on `up`
    // from a pool of the server's own, so that a stream's slots come and go
    // without waiting for the device (nullptr: plain allocations)
    cudaMemPool_t rec_pool = nullptr;
    std::thread th;
    // pinned buffers for packed records: push packs each picture straight
    // into one (on the caller's thread), the scheduler only enqueues its H2D
    // copy; a buffer returns to the pool when its picture is reported
    std::mutex pool_mu;
    std::multimap<uint64_t, uint8_t *> pool;
    bool stop = false;
    int next_id = 0;
    size_t rr = 0;
};

namespace {

cudaEvent_t take_event(h264r_server *srv)
{
    if (!srv->ev_pool.empty()) {
        cudaEvent_t e = srv->ev_pool.back();
        srv->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

void give_event(h264r_server *srv, cudaEvent_t &e)
{
    if (e) srv->ev_pool.push_back(e);
    e = nullptr;
}

Pinned take_pinned(h264r_server *srv, uint64_t need)
{
    {
        std::lock_guard<std::mutex> g(srv->pool_mu);
        auto f = srv->pool.lower_bound(need);
        if (f != srv->pool.end() && f->first <= 2 * need + (1 << 20)) {
            Pinned p{f->second, f->first};
            srv->pool.erase(f);
            return p;
        }
    }
    Pinned p;
    const uint64_t cap = align_up(need + need / 8, 1 << 16);
    if (cudaMallocHost(&p.ptr, cap) != cudaSuccess) return Pinned();
    p.cap = cap;
    return p;
}

// device memory of a record slot, and its release once nothing reads it
uint8_t *slot_alloc(h264r_server *srv, uint64_t bytes)
{
    void *p = nullptr;
    if (srv->rec_pool) {
        if (cudaMallocFromPoolAsync(&p, bytes, srv->rec_pool, srv->up) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return (uint8_t *)p;
    }
    return cudaMalloc(&p, bytes) == cudaSuccess ? (uint8_t *)p : nullptr;
}

void slot_free(h264r_server *srv, uint8_t *p)
{
    if (!p) return;
    if (srv->rec_pool) cudaFreeAsync(p, srv->up);
    else cudaFree(p);
}

void give_pinned(h264r_server *srv, Pinned &p)
{
    if (!p.ptr) return;
    std::lock_guard<std::mutex> g(srv->pool_mu);
    srv->pool.emplace(p.cap, p.ptr);
    p = Pinned();
}

void report(h264r_server *srv, SStream *S, Item *it, int status)
{
    give_pinned(srv, it->blob);
    h264r_server_done d;
    d.stream = S->id;
    d.status = status;
    d.tag = it->tag;
    d.latency_ms = now_ms() - it->t_push;
    srv->done_q.push_back(d);
    if (status == 0) srv->lat.push_back(d.latency_ms);
    srv->st.pictures_done++;
    if (it->slot >= 0) S->slots[it->slot].busy = false;
    give_event(srv, it->uploaded);
    give_event(srv, it->done);
    delete it;
    srv->done_cv.notify_all();
}

// A stream that hit an error: every picture it still holds is reported with
// the error, and it closes like a finished stream.
void fail_stream(h264r_server *srv, SStream *S, int status)
{
    if (S->s) h264r_stream_sync(S->s);
    S->status = status;
    for (auto *q : {&S->flight, &S->dev_q, &S->host_q}) {
        while (!q->empty()) {
            report(srv, S, q->front(), status);
            q->pop_front();
        }
    }
}

uint64_t geometry_key(const h264r_stream_cfg &c)
{
    return ((uint64_t)c.width_mbs << 32) | ((uint64_t)c.height_mbs << 16) | c.dpb_slots;
}

void close_stream(h264r_server *srv, SStream *S)
{
    if (S->s) {
        // Every picture of the stream has been reported: its work is done (no
        // h264r_stream_sync here, whose read of the context's error word
        // queues behind the output copies of all the other streams).  The
        // engine stream is kept for the next request of its geometry.
        if (!S->status && srv->idle.size() < kIdleMax) srv->idle.emplace(geometry_key(S->cfg), S->s);
        else h264r_stream_close(S->s);
        S->s = nullptr;
        srv->st.dpb_bytes_in_use -= S->dpb;
        srv->st.streams_open--;
    }
    for (auto &sl : S->slots) {  // no batch reads them any more (the stream is synchronised)
        slot_free(srv, sl.dev);
        sl = Slot();
    }
    S->finished = true;
    srv->st.streams_done++;
}

bool admit(h264r_server *srv)
{
    bool progress = false;
    while (!srv->waiting.empty()) {
        SStream *S = srv->waiting.front();
        int rc = H264R_ERR_BUDGET;
        auto f = srv->idle.find(geometry_key(S->cfg));
        if (f != srv->idle.end()) {
            S->s = f->second;
            srv->idle.erase(f);
            rc = h264r_stream_reset(S->s);
            if (rc != H264R_OK) {
                h264r_stream_close(S->s);
                S->s = nullptr;
            }
        }
        if (!S->s) {
            rc = h264r_stream_open(srv->ctx, &S->cfg, &S->s);
            while (rc == H264R_ERR_BUDGET && !srv->idle.empty()) {  // idle streams give their DPBs back
                h264r_stream_close(srv->idle.begin()->second);
                srv->idle.erase(srv->idle.begin());
                rc = h264r_stream_open(srv->ctx, &S->cfg, &S->s);
            }
        }
        if (rc == H264R_ERR_BUDGET) break;  // wait for finished streams to free their DPBs
        srv->waiting.pop_front();
        srv->st.streams_waiting--;
        progress = true;
        if (rc != H264R_OK) {
            S->s = nullptr;
            fail_stream(srv, S, rc);
            close_stream(srv, S);
            continue;
        }
        S->admitted = true;
        S->slots.resize(srv->depth);
        srv->active.push_back(S);
        {  // the clear of its buffers (open / reset, on its own CUDA stream) before the lane's batches
            cudaEvent_t e = take_event(srv);
            cudaEventRecord(e, (cudaStream_t)h264r_stream_cuda_stream(S->s));
            cudaStreamWaitEvent(srv->lane_cs[S->id % srv->lanes], e, 0);
            give_event(srv, e);
        }
        srv->st.streams_open++;
        srv->st.dpb_bytes_in_use += S->dpb;
        srv->st.dpb_bytes_peak = std::max(srv->st.dpb_bytes_peak, srv->st.dpb_bytes_in_use);
    }
    return progress;
}

bool retire(h264r_server *srv)
{
    bool progress = false;
    // a picture finishes after its batch: only the streams of completed
    // batches are looked at (one event query per lane otherwise)
    for (auto &q : srv->batch_done) {
        while (!q.empty() && cudaEventQuery(q.front().done) == cudaSuccess) {
            for (SStream *S : q.front().members) S->check = true;
            give_event(srv, q.front().done);
            q.pop_front();
        }
    }
    for (SStream *S : srv->active) {
        if (S->finished) continue;
        if (!S->check && !(S->ended && S->flight.empty())) continue;
        S->check = false;
        while (!S->flight.empty() && !S->status) {
            Item *it = S->flight.front();
            cudaError_t e = cudaEventQuery(it->done);
            if (e == cudaErrorNotReady) {
                S->check = true;  // its output copy is still running
                break;
            }
            S->flight.pop_front();
            const int status = e == cudaSuccess ? H264R_OK : H264R_ERR_CUDA;
            report(srv, S, it, status);
            progress = true;
            if (status != H264R_OK) {
                fail_stream(srv, S, status);
                break;
            }
        }
        if (S->ended && S->host_q.empty() && S->dev_q.empty() && S->flight.empty()) {
            close_stream(srv, S);
            progress = true;
        }
    }
    srv->active.erase(std::remove_if(srv->active.begin(), srv->active.end(), [](const SStream *S) { return S->finished; }),
                      srv->active.end());
    return progress;
}

bool upload(h264r_server *srv)
{
    bool progress = false;
    for (SStream *S : srv->active) {
        if (S->finished || S->status) continue;
        while (!S->host_q.empty()) {
            int k = -1;
            for (int i = 0; i < (int)S->slots.size(); i++)
                if (!S->slots[i].busy) { k = i; break; }
            if (k < 0) break;
            Item *it = S->host_q.front();
            Slot &sl = S->slots[k];
            const uint64_t need = it->size;
            if (sl.cap < need) {
                slot_free(srv, sl.dev);  // a free slot: the batch that read it has completed
                sl = Slot();
                const uint64_t cap = align_up(need + need / 8, 1 << 16);
                if (!(sl.dev = slot_alloc(srv, cap))) {
                    sl = Slot();
                    fail_stream(srv, S, H264R_ERR_NO_MEMORY);
                    progress = true;
                    break;
                }
                sl.cap = cap;
            }
            if (cudaMemcpyAsync(sl.dev, it->blob.ptr, need, cudaMemcpyHostToDevice, srv->up) != cudaSuccess) {
                fail_stream(srv, S, H264R_ERR_CUDA);
                progress = true;
                break;
            }
            it->uploaded = take_event(srv);
            cudaEventRecord(it->uploaded, srv->up);
            it->up_seq = ++srv->up_seq;
            sl.busy = true;
            it->slot = k;
            uint8_t *d = sl.dev;
            it->pic.mbs = (const h264r_mb *)(d + it->off[0]);
            it->pic.slices = (const h264r_slice *)(d + it->off[1]);
            it->pic.weights = (const h264r_weight *)(d + it->off[2]);
            it->pic.motion = d + it->off[3];
            it->pic.coef = d + it->off[4];
            it->pic.pcm = d + it->off[5];
            S->host_q.pop_front();
            S->dev_q.push_back(it);
            progress = true;
        }
    }
    return progress;
}

// The device queues (dev_q, flight), the slots and the engine streams are
// the scheduler thread's alone; the server lock (held on entry, as `lk`) is
// released while the batch is submitted and its output copies are queued,
// so that pushes and polls do not wait for the engine calls.
bool launch_lane(h264r_server *srv, int lane, std::unique_lock<std::mutex> &lk)
{
    if ((int)srv->batch_done[lane].size() >= kMaxBatchesInFlight) return false;
    std::vector<SStream *> order;
    for (SStream *S : srv->active)
        if (S->id % srv->lanes == lane && !S->finished && !S->status && !S->dev_q.empty()) order.push_back(S);
    if (order.empty()) return false;
    // round robin over the streams so that a full batch does not always
    // leave out the same ones
    std::rotate(order.begin(), order.begin() + (srv->rr++ % order.size()), order.end());
    std::vector<h264r_stream *> ss;
    std::vector<h264r_picture> pics;
    std::vector<std::pair<SStream *, Item *>> items;
    for (SStream *S : order) {
        if (S->groups_in_flight() >= kMaxGroupsInFlight) continue;
        const int g = S->dev_q.front()->group;
        size_t take = 0;
        while (take < S->dev_q.size() && S->dev_q[take]->group == g && (int)pics.size() < srv->max_batch) {
            Item *it = S->dev_q[take];
            ss.push_back(S->s);
            pics.push_back(it->pic);
            items.emplace_back(S, it);
            take++;
        }
        if ((int)pics.size() >= srv->max_batch) break;
    }
    if (pics.empty()) return false;
    lk.unlock();
    // the records must be on the device before the batch reads them: the
    // upload stream runs in order, so the last upload of the batch covers all
    const cudaStream_t lcs = srv->lane_cs[lane], lcopy = srv->lane_copy[lane];
    Item *last = items[0].second;
    for (auto &pr : items)
        if (pr.second->up_seq > last->up_seq) last = pr.second;
    cudaStreamWaitEvent(lcs, last->uploaded, 0);
    const int rc = h264r_submit_batch_device_on(srv->ctx, lcs, (int)pics.size(), ss.data(), pics.data());
    cudaEvent_t be = nullptr;
    if (rc == H264R_OK) {
        be = take_event(srv);
        cudaEventRecord(be, lcs);
        cudaStreamWaitEvent(lcopy, be, 0);  // the output copies follow the batch
    }
    // move the launched pictures from dev_q to flight (same order)
    for (auto &pr : items) {
        SStream *S = pr.first;
        S->dev_q.pop_front();
        Item *it = pr.second;
        if (rc != H264R_OK) {
            S->flight.push_back(it);
            continue;
        }
        cudaStream_t cs = lcs;
        if (it->out) {
            // the copy runs on the lane's copy stream, beside the lane's next batches
            const uint64_t W = S->cfg.width_mbs * 16ull, H = S->cfg.height_mbs * 16ull;
            h264r_output_async_on(S->s, it->pic.dst_slot, it->out, it->out + W * H, it->out + W * H + W * H / 4, lcopy);
            cs = lcopy;
        }
        it->done = take_event(srv);
        cudaEventRecord(it->done, cs);
        S->flight.push_back(it);
    }
    lk.lock();
    if (rc != H264R_OK) {
        for (auto &pr : items)
            if (!pr.first->flight.empty()) fail_stream(srv, pr.first, rc);
        return true;
    }
    h264r_server::Batch bt;
    bt.done = be;
    for (auto &pr : items)
        if (bt.members.empty() || bt.members.back() != pr.first) bt.members.push_back(pr.first);
    srv->batch_done[lane].push_back(std::move(bt));
    srv->st.batches++;
    srv->st.batch_pictures += pics.size();
    return true;
}

bool launch(h264r_server *srv, std::unique_lock<std::mutex> &lk)
{
    bool progress = false;
    for (int lane = 0; lane < srv->lanes; lane++) progress = launch_lane(srv, lane, lk) || progress;
    return progress;
}

void scheduler(h264r_server *srv)
{
    cudaSetDevice(srv->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        bool progress = admit(srv);
        progress = retire(srv) || progress;
        progress = upload(srv) || progress;
        progress = launch(srv, lk) || progress;
        if (srv->stop && srv->waiting.empty() && srv->active.empty()) break;
        if (!progress) srv->wake.wait_for(lk, std::chrono::microseconds(50));
    }
}

}  // namespace

extern "C" int h264r_server_create(h264r_ctx *ctx, const h264r_server_cfg *cfg, h264r_server **out)
{
    if (!ctx || !out) return H264R_ERR_INVALID_ARG;
    *out = nullptr;
    h264r_server *srv = new (std::nothrow) h264r_server();
    if (!srv) return H264R_ERR_NO_MEMORY;
    srv->ctx = ctx;
    srv->device = h264r_ctx_device(ctx);
    srv->budget = h264r_ctx_dpb_budget(ctx);
    const int ctx_batch = h264r_ctx_max_batch(ctx);
    srv->max_batch = (cfg && cfg->max_batch_pictures) ? (int)std::min<uint32_t>(cfg->max_batch_pictures, ctx_batch) : ctx_batch;
    srv->depth = (cfg && cfg->queue_depth) ? (int)std::min<uint32_t>(cfg->queue_depth, 32) : 4;
    srv->lanes = (cfg && cfg->lanes) ? (int)std::min<uint32_t>(cfg->lanes, kMaxLanes) : kLanes;
    cudaSetDevice(srv->device);
    if (cudaStreamCreateWithFlags(&srv->up, cudaStreamNonBlocking) != cudaSuccess) {
        delete srv;
        return H264R_ERR_CUDA;
    }
    for (int l = 0; l < srv->lanes; l++) {
        if (cudaStreamCreateWithFlags(&srv->lane_cs[l], cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&srv->lane_copy[l], cudaStreamNonBlocking) != cudaSuccess) {
            for (int k = 0; k <= l; k++) {
                if (srv->lane_cs[k]) cudaStreamDestroy(srv->lane_cs[k]);
                if (srv->lane_copy[k]) cudaStreamDestroy(srv->lane_copy[k]);
            }
            cudaStreamDestroy(srv->up);
            delete srv;
            return H264R_ERR_CUDA;
        }
    }
    cudaMemPoolProps pp = {};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.handleTypes = cudaMemHandleTypeNone;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = srv->device;
    if (cudaMemPoolCreate(&srv->rec_pool, &pp) == cudaSuccess) {
        uint64_t keep = ~0ull;  // freed slots stay in the pool for the next streams
        cudaMemPoolSetAttribute(srv->rec_pool, cudaMemPoolAttrReleaseThreshold, &keep);
    } else {
        srv->rec_pool = nullptr;
        cudaGetLastError();
    }
    srv->th = std::thread(scheduler, srv);
    *out = srv;
    return H264R_OK;
}

extern "C" int h264r_server_destroy(h264r_server *srv)
{
    if (!srv) return H264R_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        for (auto &kv : srv->streams) kv.second->ended = true;
        srv->stop = true;
    }
    srv->wake.notify_all();
    srv->th.join();
    cudaSetDevice(srv->device);
    for (auto &kv : srv->streams) delete kv.second;
    for (auto &kv : srv->idle) h264r_stream_close(kv.second);
    for (auto &q : srv->batch_done)
        for (auto &b : q) cudaEventDestroy(b.done);
    for (auto e : srv->ev_pool) cudaEventDestroy(e);
    for (auto &kv : srv->pool) cudaFreeHost(kv.second);
    cudaStreamSynchronize(srv->up);
    for (int l = 0; l < srv->lanes; l++) {
        cudaStreamSynchronize(srv->lane_copy[l]);
        cudaStreamSynchronize(srv->lane_cs[l]);
        cudaStreamDestroy(srv->lane_copy[l]);
        cudaStreamDestroy(srv->lane_cs[l]);
    }
    if (srv->rec_pool) cudaMemPoolDestroy(srv->rec_pool);
    cudaStreamDestroy(srv->up);
    delete srv;
    return H264R_OK;
}

extern "C" int h264r_server_open(h264r_server *srv, const h264r_stream_cfg *cfg, int *stream_id)
{
    if (!srv || !cfg || !stream_id || !cfg->width_mbs || !cfg->height_mbs || !cfg->dpb_slots || cfg->dpb_slots > 32)
        return H264R_ERR_INVALID_ARG;
    const uint64_t dpb = h264r_stream_dpb_bytes(cfg);
    if (dpb > srv->budget) return H264R_ERR_BUDGET;
    SStream *S = new (std::nothrow) SStream();
    if (!S) return H264R_ERR_NO_MEMORY;
    S->cfg = *cfg;
    S->dpb = dpb;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        S->id = srv->next_id++;
        srv->streams[S->id] = S;
        srv->waiting.push_back(S);
        srv->st.streams_waiting++;
        srv->st.waiting_peak = std::max<uint64_t>(srv->st.waiting_peak, srv->st.streams_waiting);
    }
    srv->wake.notify_all();
    *stream_id = S->id;
    return H264R_OK;
}

extern "C" int h264r_server_push(h264r_server *srv, int stream_id, const h264r_picture *pic, int dependency_group, uint64_t tag,
                                 uint8_t *out_planes)
{
    if (!srv || !pic) return H264R_ERR_INVALID_ARG;
    h264r_stream_cfg cfg;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        auto f = srv->streams.find(stream_id);
        if (f == srv->streams.end() || f->second->ended) return H264R_ERR_INVALID_ARG;
        cfg = f->second->cfg;
    }
    if (pic->width_mbs != cfg.width_mbs || pic->height_mbs != cfg.height_mbs) return H264R_ERR_INVALID_ARG;
    int rc = h264r_validate_picture(pic, cfg.dpb_slots);
    if (rc) return rc;
    // pack the records as the device will see them (outside the lock)
    Item *it = new (std::nothrow) Item();
    if (!it) return H264R_ERR_NO_MEMORY;
    const void *src[6] = {pic->mbs, pic->slices, pic->weights, pic->motion, pic->coef, pic->pcm};
    const uint64_t sz[6] = {sizeof(h264r_mb) * pic->num_mbs, sizeof(h264r_slice) * pic->num_slices,
                            sizeof(h264r_weight) * pic->num_weights, pic->motion_bytes, pic->coef_bytes, 384ull * pic->num_pcm};
    uint64_t tot = 0;
    for (int k = 0; k < 6; k++) {
        it->off[k] = tot;
        tot = align_up(tot + sz[k], kAlign);
    }
    it->blob = take_pinned(srv, tot);
    if (!it->blob.ptr) {
        delete it;
        return H264R_ERR_NO_MEMORY;
    }
    it->size = tot;
    for (int k = 0; k < 6; k++)
        if (sz[k]) memcpy(it->blob.ptr + it->off[k], src[k], sz[k]);
    it->pic = *pic;
    it->group = dependency_group;
    it->tag = tag;
    it->out = out_planes;
    it->t_push = now_ms();
    {
        std::lock_guard<std::mutex> g(srv->mu);
        auto f = srv->streams.find(stream_id);
        if (f == srv->streams.end() || f->second->ended) {
            give_pinned(srv, it->blob);
            delete it;
            return H264R_ERR_INVALID_ARG;
        }
        SStream *S = f->second;
        S->pending++;
        if (S->status) {  // the stream failed earlier: report the picture at once
            const int st = S->status;
            report(srv, S, it, st);
            return st;
        }
        S->host_q.push_back(it);
    }
    srv->wake.notify_all();
    return H264R_OK;
}

extern "C" int h264r_server_end(h264r_server *srv, int stream_id)
{
    if (!srv) return H264R_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        auto f = srv->streams.find(stream_id);
        if (f == srv->streams.end()) return H264R_ERR_INVALID_ARG;
        f->second->ended = true;
    }
    srv->wake.notify_all();
    return H264R_OK;
}

extern "C" int h264r_server_poll(h264r_server *srv, h264r_server_done *done, int max, int wait_ms)
{
    if (!srv || !done || max <= 0) return H264R_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    if (srv->done_q.empty() && wait_ms > 0)
        srv->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [srv] { return !srv->done_q.empty(); });
    int n = 0;
    while (n < max && !srv->done_q.empty()) {
        done[n] = srv->done_q.front();
        srv->done_q.pop_front();
        auto f = srv->streams.find(done[n].stream);
        if (f != srv->streams.end()) f->second->pending--;
        n++;
    }
    return n;
}

extern "C" int h264r_server_pending(h264r_server *srv, int stream_id)
{
    if (!srv) return H264R_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    auto f = srv->streams.find(stream_id);
    if (f == srv->streams.end()) return H264R_ERR_INVALID_ARG;
    return f->second->pending;
}

extern "C" int h264r_server_get_stats(h264r_server *srv, h264r_server_stats *out)
{
    if (!srv || !out) return H264R_ERR_INVALID_ARG;
    std::vector<double> l;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        *out = srv->st;
        l = srv->lat;
    }
    out->p50_ms = out->p99_ms = out->max_ms = 0;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        out->p50_ms = l[l.size() / 2];
        out->p99_ms = l[std::min(l.size() - 1, (size_t)(0.99 * l.size()))];
        out->max_ms = l.back();
    }
    return H264R_OK;
}
