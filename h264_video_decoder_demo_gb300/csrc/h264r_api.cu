// h264r_api.cu — host side of the reconstruction engine behind the C ABI of
// include/h264r.h: contexts, streams with device-resident DPBs, record
// staging (pinned host -> device) and the launch sequence
//   k_inter -> k_intra (only when the batch has intra MBs) -> k_bs -> k_deblock
// on the stream's CUDA stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <chrono>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "h264r_device.cuh"

namespace h264r {
__global__ void k_inter(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st);
__global__ void k_inter2(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st);
__global__ void k_inter8(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st);
__global__ void k_intra(const PicDesc *__restrict__ pics, int npics, uint32_t total_rows, LaunchState st);
__global__ void k_bs(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st);
__global__ void k_deblock(const PicDesc *__restrict__ pics, int npics, uint32_t total_units, LaunchState st);
__global__ void k_deblock_frame(const PicDesc *__restrict__ pics, int npics, uint32_t total_units, LaunchState st);
__global__ void k_deblock_frame4(const PicDesc *__restrict__ pics, int npics, uint32_t total_units, LaunchState st);
__global__ void k_bgr24(const uint8_t *__restrict__ yuv, int W, int H, uint8_t *__restrict__ out, int row_bytes, int flip);
}  // namespace h264r

using h264r::PicDesc;
using h264r::LaunchState;

static_assert(sizeof(h264r_mb) == 32, "h264r_mb layout");
static_assert(sizeof(h264r_part) == 16, "h264r_part layout");
static_assert(sizeof(h264r_weight) == 32, "h264r_weight layout");
static_assert(sizeof(h264r_slice) == 8, "h264r_slice layout");

namespace {

constexpr int kRing = 4;                 // in-flight launches per stream
constexpr int kBatchRing = 16;           // in-flight batched launches per context (all pipelines, server lanes)
constexpr uint64_t kAlign = 256;
constexpr unsigned long long kSpinLimit = 1ull << 25;  // ~ seconds of 64 ns sleeps

inline uint64_t align_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

// What a captured launch sequence depends on: the buffers and streams it
// names and the sizes of its launches.  Compared bytewise (zeroed first).
struct GraphKey {
    const void *host, *dev, *bs, *ires;
    cudaStream_t cs, side;
    uint64_t total, mbs, rows;
    uint32_t n, dbf_units, db_units, flags, inter_w, dbf_w;
};

struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec = nullptr;  // instantiated at the second sighting of key
    uint32_t kernels = 0;
    uint64_t used = 0;               // last use (LRU clock)
};
constexpr int kGraphCache = 16;  // shapes remembered per launch buffer

// Per-launch scratch: PicDesc array, wavefront tickets, progress counters,
// bS tables.  Host mirror in pinned memory, device copy uploaded per launch.
struct LaunchBuf {
    uint8_t *host = nullptr;      // pinned: PicDesc array, tickets, progress
    uint64_t host_cap = 0;
    uint8_t *dev = nullptr;       // its device copy
    uint64_t dev_cap = 0;
    uint8_t *bs = nullptr;        // device, bS tables
    uint64_t bs_cap = 0;
    uint8_t *ires = nullptr;      // device, intra residuals (768 bytes per MB)
    uint64_t ires_cap = 0;
    uint8_t *rec_host = nullptr;  // pinned staging for host-resident records
    uint64_t rec_host_cap = 0;
    uint8_t *rec_dev = nullptr;   // device copy of the records
    uint64_t rec_dev_cap = 0;
    cudaEvent_t done = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;  // k_bs on the owner's side stream
    cudaEvent_t uploaded = nullptr;              // host-record upload on the context's upload stream
    bool wait_upload = false;                    // the records of the current use come through `uploaded`
    bool pending = false;
    GraphEntry graphs[kGraphCache];
    int ngraphs = 0;
    uint64_t graph_clock = 0;
};

}  // namespace

// Host worker threads of a context: validation and packing of the records
// of a host-submitted batch run on them and on the calling thread, so that
// the host prepares the next batch at the pace the GPU consumes them.
class WorkerPool {
public:
    explicit WorkerPool(int n)
    {
        for (int i = 0; i < n; i++) th_.emplace_back([this] { loop(); });
    }
    ~WorkerPool()
    {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    int size() const { return (int)th_.size(); }
    // fn(0) .. fn(n-1), on the workers and the calling thread; returns when all are done
    void run(int n, const std::function<void(int)> &fn)
    {
        if (n <= 1 || th_.empty()) {
            for (int i = 0; i < n; i++) fn(i);
            return;
        }
        std::unique_lock<std::mutex> lk(mu_);
        fn_ = &fn;
        n_ = n;
        next_ = 0;
        pending_ = n;
        cv_.notify_all();
        while (pending_ > 0) {
            if (next_ < n_) {
                const int i = next_++;
                lk.unlock();
                fn(i);
                lk.lock();
                --pending_;
            } else {
                done_.wait(lk);
            }
        }
        fn_ = nullptr;
    }

private:
    void loop()
    {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [this] { return stop_ || (fn_ && next_ < n_); });
            if (stop_) return;
            const int i = next_++;
            const std::function<void(int)> *f = fn_;
            lk.unlock();
            (*f)(i);
            lk.lock();
            if (--pending_ == 0) done_.notify_all();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *fn_ = nullptr;
    int n_ = 0, next_ = 0, pending_ = 0;
    bool stop_ = false;
};

struct h264r_ctx {
    int device = 0;
    std::unique_ptr<WorkerPool> pool;
    // host time of h264r_submit_batch calls (seconds): waiting for a free
    // launch slot, validating and packing on the workers, upload and launch
    double host_s[3] = {0, 0, 0};
    bool records_ready = false;  // H264R_CFG_DEVICE_RECORDS_READY
    uint64_t budget = 0, used = 0;
    uint32_t max_batch = 64;
    int *d_error = nullptr;
    int *h_error = nullptr;  // pinned
    std::atomic<uint64_t> launches{0};
    bool timing = false;
    double total_ms[4] = {0, 0, 0, 0};  // inter, intra, bS, deblocking filter
    int timed_launches = 0;
    std::vector<std::array<cudaEvent_t, 5>> ev_free, ev_pending;
    std::mutex timing_mu;
    cudaStream_t batch_stream = nullptr;
    // host-submitted batches upload their records here, so that a batch's
    // upload overlaps the kernels of the batch before it on the same pipeline
    cudaStream_t upload_stream = nullptr;
    // picture buffers of the streams: stream-ordered allocations from a pool
    // that keeps up to the DPB budget for reuse, so that opening and closing
    // a stream (a served request) does not wait for the device
    cudaMemPool_t dpb_pool = nullptr;
    // launch shapes: the default and the autotuner's choice per geometry mix
    std::mutex tune_mu;
    h264r_tuning tuning{4, 8, 0, 0};
    std::unordered_map<uint64_t, h264r_tuning> tuned;
    std::atomic<uint64_t> graph_replays{0}, graphs_captured{0};
    // failure-path tests (h264r_ctx_set_wait_test): spin limit of the
    // device waits, and whether launches withhold their first rows
    std::atomic<unsigned long long> spin_limit{kSpinLimit};
    std::atomic<int> withhold{0};
    LaunchBuf batch_ring[kBatchRing];
    int batch_next = 0;
    std::mutex mu;
    char err[256] = {0};
};

struct h264r_stream {
    h264r_ctx *ctx = nullptr;
    h264r_stream_cfg cfg{};
    uint64_t slot_bytes = 0;
    uint8_t *dpb = nullptr;
    bool pooled = false;        // dpb from the context's pool, cleared on cs
    bool clear_synced = false;  // h264r_slot_device_ptr waited for that clear
    cudaStream_t cs = nullptr;
    cudaStream_t side = nullptr;  // boundary strengths of launches on cs, beside inter and intra
    // h264r_output_async: copies to the host on their own stream; a launch
    // that writes a slot waits for the slot's pending copy
    cudaStream_t out = nullptr;
    cudaEvent_t out_ready = nullptr;
    std::vector<cudaEvent_t> slot_ev;
    std::unique_ptr<std::atomic<uint8_t>[]> slot_pending;
    LaunchBuf ring[kRing];
    int next = 0;
    uint8_t *bgr = nullptr;  // device staging of h264r_output_bgr24
    uint64_t bgr_cap = 0;
};

static void set_err(h264r_ctx *ctx, const char *fmt, ...)
{
    if (!ctx) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
    va_end(ap);
}

#define CUDA_OR(ctx, expr)                                                                  \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            set_err((ctx), "%s: %s", #expr, cudaGetErrorString(e_));                        \
            return H264R_ERR_CUDA;                                                          \
        }                                                                                   \
    } while (0)

extern "C" uint64_t h264r_stream_dpb_bytes(const h264r_stream_cfg *cfg)
{
    if (!cfg) return 0;
    uint64_t W = (uint64_t)cfg->width_mbs * 16, H = (uint64_t)cfg->height_mbs * 16;
    uint64_t slot = align_up(W * H * 3 / 2 + 4 * W + 64, kAlign);
    return slot * cfg->dpb_slots;
}

static uint64_t slot_bytes_of(const h264r_stream_cfg &c)
{
    uint64_t W = (uint64_t)c.width_mbs * 16, H = (uint64_t)c.height_mbs * 16;
    return align_up(W * H * 3 / 2 + 4 * W + 64, kAlign);
}

static void create_events(LaunchBuf &b)
{
    cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b.join, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b.uploaded, cudaEventDisableTiming);
}

extern "C" int h264r_ctx_create(const h264r_cfg *cfg, h264r_ctx **out)
{
    if (!out) return H264R_ERR_INVALID_ARG;
    *out = nullptr;
    h264r_ctx *ctx = new (std::nothrow) h264r_ctx();
    if (!ctx) return H264R_ERR_NO_MEMORY;
    ctx->device = cfg ? cfg->device : 0;
    if (cfg && cfg->max_batch_pictures) ctx->max_batch = cfg->max_batch_pictures;
    ctx->records_ready = cfg && (cfg->flags & H264R_CFG_DEVICE_RECORDS_READY);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        fprintf(stderr, "h264r_ctx_create: cudaSetDevice(%d): %s\n", ctx->device, cudaGetErrorString(e));
        delete ctx;
        return H264R_ERR_CUDA;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->budget = (cfg && cfg->dpb_budget_bytes) ? cfg->dpb_budget_bytes : (uint64_t)(free_b * 0.9);
    if (cudaMalloc(&ctx->d_error, sizeof(int)) != cudaSuccess || cudaMallocHost(&ctx->h_error, sizeof(int)) != cudaSuccess ||
        cudaMemset(ctx->d_error, 0, sizeof(int)) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->batch_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return H264R_ERR_CUDA;
    }
    for (auto &b : ctx->batch_ring) create_events(b);
    {
        cudaMemPoolProps pp = {};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.handleTypes = cudaMemHandleTypeNone;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = ctx->device;
        if (cudaMemPoolCreate(&ctx->dpb_pool, &pp) == cudaSuccess) {
            uint64_t keep = ctx->budget;
            cudaMemPoolSetAttribute(ctx->dpb_pool, cudaMemPoolAttrReleaseThreshold, &keep);
        } else {
            ctx->dpb_pool = nullptr;  // plain allocations then
            cudaGetLastError();
        }
    }
    *ctx->h_error = 0;
    const unsigned hw = std::thread::hardware_concurrency();
    ctx->pool.reset(new (std::nothrow) WorkerPool(hw > 2 ? (int)std::min(hw - 1u, 15u) : 0));
    if (!ctx->pool) {
        h264r_ctx_destroy(ctx);
        return H264R_ERR_NO_MEMORY;
    }
    *out = ctx;
    return H264R_OK;
}

static void free_buf(LaunchBuf &b)
{
    if (b.host) cudaFreeHost(b.host);
    if (b.dev) cudaFree(b.dev);
    if (b.bs) cudaFree(b.bs);
    if (b.ires) cudaFree(b.ires);
    if (b.rec_host) cudaFreeHost(b.rec_host);
    if (b.rec_dev) cudaFree(b.rec_dev);
    if (b.done) cudaEventDestroy(b.done);
    if (b.fork) cudaEventDestroy(b.fork);
    if (b.join) cudaEventDestroy(b.join);
    if (b.uploaded) cudaEventDestroy(b.uploaded);
    for (int i = 0; i < b.ngraphs; i++)
        if (b.graphs[i].exec) cudaGraphExecDestroy(b.graphs[i].exec);
    b = LaunchBuf();
}

extern "C" int h264r_ctx_destroy(h264r_ctx *ctx)
{
    if (!ctx) return H264R_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->batch_stream);
    if (ctx->upload_stream) cudaStreamSynchronize(ctx->upload_stream);
    for (auto &b : ctx->batch_ring) free_buf(b);
    for (auto *pool : {&ctx->ev_free, &ctx->ev_pending})
        for (auto &q : *pool)
            for (auto e : q) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->batch_stream);
    if (ctx->upload_stream) cudaStreamDestroy(ctx->upload_stream);
    if (ctx->dpb_pool) cudaMemPoolDestroy(ctx->dpb_pool);
    cudaFree(ctx->d_error);
    cudaFreeHost(ctx->h_error);
    delete ctx;
    return H264R_OK;
}

extern "C" const char *h264r_last_error(const h264r_ctx *ctx) { return ctx ? ctx->err : "no context"; }

extern "C" uint64_t h264r_ctx_kernel_launches(const h264r_ctx *ctx) { return ctx ? ctx->launches.load() : 0; }

extern "C" int h264r_ctx_device(const h264r_ctx *ctx) { return ctx ? ctx->device : H264R_ERR_INVALID_ARG; }

extern "C" uint64_t h264r_ctx_dpb_budget(const h264r_ctx *ctx) { return ctx ? ctx->budget : 0; }

extern "C" int h264r_ctx_max_batch(const h264r_ctx *ctx) { return ctx ? (int)ctx->max_batch : H264R_ERR_INVALID_ARG; }

static int drain_timing(h264r_ctx *ctx)
{
    std::lock_guard<std::mutex> lk(ctx->timing_mu);
    for (auto &q : ctx->ev_pending) {
        CUDA_OR(ctx, cudaEventSynchronize(q[4]));
        float ms;
        for (int k = 0; k < 4; k++) {
            cudaEventElapsedTime(&ms, q[k], q[k + 1]);
            ctx->total_ms[k] += ms;
        }
        ctx->timed_launches++;
        ctx->ev_free.push_back(q);
    }
    ctx->ev_pending.clear();
    return H264R_OK;
}

extern "C" int h264r_ctx_set_wait_test(h264r_ctx *ctx, uint64_t spin_limit, int withhold_first_rows)
{
    if (!ctx) return H264R_ERR_INVALID_ARG;
    ctx->spin_limit.store(spin_limit ? (unsigned long long)spin_limit : kSpinLimit);
    ctx->withhold.store(withhold_first_rows ? 1 : 0);
    return H264R_OK;
}

extern "C" int h264r_ctx_set_timing(h264r_ctx *ctx, int enable)
{
    if (!ctx) return H264R_ERR_INVALID_ARG;
    int rc = drain_timing(ctx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->timing_mu);
    ctx->timing = enable != 0;
    ctx->total_ms[0] = ctx->total_ms[1] = ctx->total_ms[2] = ctx->total_ms[3] = 0;
    ctx->timed_launches = 0;
    return H264R_OK;
}

extern "C" int h264r_ctx_last_timing(h264r_ctx *ctx, float t[3], int *launches)
{
    if (!ctx || !t) return H264R_ERR_INVALID_ARG;
    int rc = drain_timing(ctx);
    if (rc) return rc;
    t[0] = (float)ctx->total_ms[0];
    t[1] = (float)ctx->total_ms[1];
    t[2] = (float)(ctx->total_ms[2] + ctx->total_ms[3]);
    if (launches) *launches = ctx->timed_launches;
    return H264R_OK;
}

extern "C" int h264r_ctx_host_stats(h264r_ctx *ctx, double s[4])
{
    if (!ctx || !s) return H264R_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    for (int k = 0; k < 3; k++) s[k] = ctx->host_s[k];
    s[3] = ctx->pool ? ctx->pool->size() + 1 : 1;
    return H264R_OK;
}

extern "C" int h264r_ctx_kernel_timing(h264r_ctx *ctx, float t[4], int *launches)
{
    if (!ctx || !t) return H264R_ERR_INVALID_ARG;
    int rc = drain_timing(ctx);
    if (rc) return rc;
    for (int k = 0; k < 4; k++) t[k] = (float)ctx->total_ms[k];
    if (launches) *launches = ctx->timed_launches;
    return H264R_OK;
}

static std::array<cudaEvent_t, 5> *take_events(h264r_ctx *ctx)
{
    std::lock_guard<std::mutex> lk(ctx->timing_mu);
    if (ctx->ev_free.empty()) {
        std::array<cudaEvent_t, 5> q;
        for (auto &e : q) cudaEventCreate(&e);
        ctx->ev_free.push_back(q);
    }
    ctx->ev_pending.push_back(ctx->ev_free.back());
    ctx->ev_free.pop_back();
    return &ctx->ev_pending.back();
}

extern "C" int h264r_stream_open(h264r_ctx *ctx, const h264r_stream_cfg *cfg, h264r_stream **out)
{
    if (!ctx || !cfg || !out) return H264R_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->width_mbs == 0 || cfg->height_mbs == 0 || cfg->width_mbs > 512 || cfg->height_mbs > 512 || cfg->dpb_slots == 0 ||
        cfg->dpb_slots > 32) {
        set_err(ctx, "h264r_stream_open: bad geometry %ux%u MBs, %u slots", cfg->width_mbs, cfg->height_mbs, cfg->dpb_slots);
        return H264R_ERR_INVALID_ARG;
    }
    uint64_t bytes = h264r_stream_dpb_bytes(cfg);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->used + bytes > ctx->budget) {
        set_err(ctx, "h264r_stream_open: DPB of %llu bytes exceeds the remaining budget (%llu of %llu used)",
                (unsigned long long)bytes, (unsigned long long)ctx->used, (unsigned long long)ctx->budget);
        return H264R_ERR_BUDGET;
    }
    h264r_stream *s = new (std::nothrow) h264r_stream();
    if (!s) return H264R_ERR_NO_MEMORY;
    s->ctx = ctx;
    s->cfg = *cfg;
    s->slot_bytes = slot_bytes_of(*cfg);
    cudaSetDevice(ctx->device);
    cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&s->out, cudaStreamNonBlocking);
    // the reference starts every picture buffer cleared (H264PictureBase.cpp:162-181).
    // From the pool: allocated and cleared in the order of cs, which every
    // launch and copy touching the stream's slots follows (a batch waits for
    // the work queued on each of its streams).
    s->pooled = ctx->dpb_pool && cudaMallocFromPoolAsync((void **)&s->dpb, bytes, ctx->dpb_pool, s->cs) == cudaSuccess &&
                cudaMemsetAsync(s->dpb, 0, bytes, s->cs) == cudaSuccess;
    if (!s->pooled) {
        if (s->dpb) cudaFreeAsync(s->dpb, s->cs);
        s->dpb = nullptr;
        cudaGetLastError();
        if (cudaMalloc(&s->dpb, bytes) != cudaSuccess) {
            set_err(ctx, "h264r_stream_open: cudaMalloc(%llu) failed", (unsigned long long)bytes);
            cudaStreamDestroy(s->cs);
            cudaStreamDestroy(s->side);
            cudaStreamDestroy(s->out);
            delete s;
            return H264R_ERR_NO_MEMORY;
        }
        cudaMemset(s->dpb, 0, bytes);
    }
    cudaEventCreateWithFlags(&s->out_ready, cudaEventDisableTiming);
    s->slot_ev.resize(cfg->dpb_slots);
    for (auto &e : s->slot_ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    s->slot_pending.reset(new std::atomic<uint8_t>[cfg->dpb_slots]);
    for (int i = 0; i < cfg->dpb_slots; i++) s->slot_pending[i] = 0;
    for (auto &b : s->ring) create_events(b);
    if (!s->pooled) cudaDeviceSynchronize();  // the legacy-stream clear before any use
    s->clear_synced = !s->pooled;
    ctx->used += bytes;
    *out = s;
    return H264R_OK;
}

extern "C" int h264r_stream_reset(h264r_stream *s)
{
    if (!s) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    CUDA_OR(ctx, cudaStreamSynchronize(s->out));
    for (int i = 0; i < s->cfg.dpb_slots; i++) s->slot_pending[i] = 0;
    CUDA_OR(ctx, cudaMemsetAsync(s->dpb, 0, h264r_stream_dpb_bytes(&s->cfg), s->cs));
    s->clear_synced = false;
    return H264R_OK;
}

extern "C" int h264r_stream_close(h264r_stream *s)
{
    if (!s) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(s->cs);
    for (auto &b : s->ring) free_buf(b);
    if (s->bgr) cudaFree(s->bgr);
    cudaStreamSynchronize(s->side);
    cudaStreamSynchronize(s->out);
    for (auto e : s->slot_ev) cudaEventDestroy(e);
    cudaEventDestroy(s->out_ready);
    if (s->pooled) cudaFreeAsync(s->dpb, s->cs);  // back to the pool once cs is done
    cudaStreamDestroy(s->cs);
    cudaStreamDestroy(s->side);
    cudaStreamDestroy(s->out);
    if (!s->pooled) cudaFree(s->dpb);
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->used -= h264r_stream_dpb_bytes(&s->cfg);
    }
    delete s;
    return H264R_OK;
}

extern "C" void *h264r_stream_cuda_stream(h264r_stream *s) { return s ? (void *)s->cs : nullptr; }
extern "C" void *h264r_stream_output_cuda_stream(h264r_stream *s) { return s ? (void *)s->out : nullptr; }

extern "C" void *h264r_ctx_cuda_stream(h264r_ctx *ctx) { return ctx ? (void *)ctx->batch_stream : nullptr; }

extern "C" int h264r_slot_device_ptr(h264r_stream *s, int slot, void **dev_y)
{
    if (!s || !dev_y || slot < 0 || slot >= s->cfg.dpb_slots) return H264R_ERR_INVALID_ARG;
    // the caller may use the slot on a stream of its own: the clear queued on
    // cs at open must be done first
    if (!s->clear_synced) {
        cudaSetDevice(s->ctx->device);
        cudaStreamSynchronize(s->cs);
        s->clear_synced = true;
    }
    *dev_y = s->dpb + (uint64_t)slot * s->slot_bytes;
    return H264R_OK;
}

// ---------------------------------------------------------------- validator
// partitions of a motion payload shape: 1, 2, or per 8x8 quadrant 1 / 2 / 2 / 4
// (a table over the four 2-bit sub-shapes)
struct PartsTable {
    uint8_t n[256];
    PartsTable()
    {
        for (int v = 0; v < 256; v++) {
            n[v] = 0;
            for (int q = 0; q < 4; q++) {
                const int sc = (v >> (2 * q)) & 3;
                n[v] = (uint8_t)(n[v] + (sc == 0 ? 1 : (sc == 3 ? 4 : 2)));
            }
        }
    }
};
static const PartsTable kPartsTable;

static inline int parts_count(uint32_t shape)
{
    const int mp = shape & 3;
    return mp == 0 ? 1 : (mp != 3 ? 2 : kPartsTable.n[(shape >> 2) & 255]);
}

// MBs of a picture: a field picture (PAFF) holds half the frame's MB rows
static uint32_t picture_mbs(const h264r_picture *pic)
{
    const uint32_t rows = pic->structure == H264R_STRUCT_FRAME ? pic->height_mbs : pic->height_mbs / 2u;
    return (uint32_t)pic->width_mbs * rows;
}

// Picture-level checks: geometry, parameter tables (everything but the MBs).
static int validate_header(const h264r_picture *pic, int dpb_slots)
{
    if (!pic || !pic->mbs || !pic->slices || !pic->weights) return H264R_ERR_INVALID_ARG;
    if (pic->structure > H264R_STRUCT_BOTTOM) return H264R_ERR_BAD_RECORD;
    const bool fpic = pic->structure != H264R_STRUCT_FRAME;
    if (fpic && (pic->mbaff || (pic->height_mbs & 1))) return H264R_ERR_BAD_RECORD;
    if (pic->width_mbs == 0 || pic->height_mbs == 0 || pic->num_mbs != picture_mbs(pic)) return H264R_ERR_BAD_RECORD;
    if (pic->mbaff && (pic->height_mbs & 1)) return H264R_ERR_BAD_RECORD;
    if (pic->dst_slot >= dpb_slots || pic->num_slices == 0 || pic->num_weights == 0) return H264R_ERR_BAD_RECORD;
    if ((pic->motion_bytes && !pic->motion) || (pic->coef_bytes && !pic->coef) || (pic->num_pcm && !pic->pcm))
        return H264R_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < pic->num_weights; i++)
        for (int c = 0; c < 3; c++)
            if (pic->weights[i].log_wd[c] < 0 || pic->weights[i].log_wd[c] > 7) return H264R_ERR_BAD_RECORD;
    for (uint32_t i = 0; i < pic->num_slices; i++)
        if (pic->slices[i].disable_deblocking_filter_idc > 2 || pic->slices[i].slice_type > 4 ||
            pic->slices[i].filter_offset_a < -12 || pic->slices[i].filter_offset_a > 12 ||
            pic->slices[i].filter_offset_b < -12 || pic->slices[i].filter_offset_b > 12)
            return H264R_ERR_BAD_RECORD;
    return H264R_OK;
}

// MBs [a0, a1) of a picture whose header passed: ranges, payload offsets and
// sizes, references.  The significance words of a coefficient payload are
// counted 64 bits at a time.
static int validate_mbs(const h264r_picture *pic, int dpb_slots, uint32_t a0, uint32_t a1)
{
    const bool fpic = pic->structure != H264R_STRUCT_FRAME;
    const uint64_t coef_bytes = pic->coef_bytes, motion_bytes = pic->motion_bytes;
    const uint32_t nslices = pic->num_slices, nweights = pic->num_weights, npcm = pic->num_pcm;
    const int dst = pic->dst_slot;
    const bool own_bottom = pic->structure == H264R_STRUCT_BOTTOM;
    for (uint32_t a = a0; a < a1; a++) {
        const h264r_mb &m = pic->mbs[a];
        if ((m.type > H264R_MB_NONE) | (m.qpy > 51) | (m.slice >= nslices) | (m.i16_mode > 3) | (m.chroma_mode > 3))
            return H264R_ERR_BAD_RECORD;
        if (m.coef != H264R_NONE) {
            if ((m.coef & 3) || (uint64_t)m.coef + 4 > coef_bytes) return H264R_ERR_BAD_RECORD;
            const uint8_t *c = pic->coef + m.coef;
            uint32_t mask;
            memcpy(&mask, c, 4);
            const int t8 = (m.flags & H264R_MBF_T8x8) != 0;
            if ((mask >> 27) || (t8 && (mask & 0xFFF0u))) return H264R_ERR_BAD_RECORD;
            const uint64_t nw = __builtin_popcount(mask) + (t8 ? 3 * __builtin_popcount(mask & 15u) : 0);
            const uint64_t voff = (4 + 2 * nw + 3) & ~3ull;
            if (m.coef + voff > coef_bytes) return H264R_ERR_BAD_RECORD;
            // levels: one per significance bit; whole 64-bit words while they
            // lie inside the payload buffer, 16-bit words for the rest
            uint64_t nl = 0, w = 0;
            const uint64_t room = coef_bytes - m.coef - 4;  // bytes from the first word to the buffer end
            for (; w + 4 <= nw; w += 4) {
                uint64_t v;
                memcpy(&v, c + 4 + 2 * w, 8);
                nl += __builtin_popcountll(v);
            }
            if (w < nw && 2 * w + 8 <= room) {
                uint64_t v;
                memcpy(&v, c + 4 + 2 * w, 8);
                nl += __builtin_popcountll(v & (~0ull >> (64 - 16 * (nw - w))));
            } else {
                for (; w < nw; w++) {
                    uint16_t sw;
                    memcpy(&sw, c + 4 + 2 * w, 2);
                    nl += __builtin_popcount(sw);
                }
            }
            if (m.coef + voff + 2 * nl > coef_bytes) return H264R_ERR_BAD_RECORD;
            // chroma DC of 4:2:0 has scan positions 0..3 only
            for (int b = 17; b <= 18; b++) {
                if (!(mask & (1u << b))) continue;
                const uint32_t before = mask & ((1u << b) - 1u);
                const uint64_t wi = __builtin_popcount(before) + (t8 ? 3 * __builtin_popcount(before & 15u) : 0);
                uint16_t sg;
                memcpy(&sg, c + 4 + 2 * wi, 2);
                if (sg & 0xFFF0u) return H264R_ERR_BAD_RECORD;
            }
        }
        if (m.type == H264R_MB_INTER) {
            if (m.aux == H264R_NONE || (m.aux & 3) || (uint64_t)m.aux + 4 > motion_bytes) return H264R_ERR_BAD_RECORD;
            uint16_t hdr[2];
            memcpy(hdr, pic->motion + m.aux, 4);
            if (hdr[1] != parts_count(hdr[0]) || (uint64_t)m.aux + 4 + 16ull * hdr[1] > motion_bytes) return H264R_ERR_BAD_RECORD;
            const bool mb_field = (m.flags & H264R_MBF_FIELD) && pic->mbaff;
            // per reference byte r (>= 0): the slot exists; a field picture
            // reads fields only and its own slot only for the other parity (the
            // first field of the frame); a frame picture never its own slot,
            // and fields only from field MBs of MBAFF frames (branch-free)
            const uint8_t *pp = pic->motion + m.aux + 4;
            unsigned bad = 0;
            for (int e = 0; e < hdr[1]; e++, pp += 16) {
                uint16_t wt;
                memcpy(&wt, pp + 12, 2);
                bad |= wt >= nweights;
                for (int l = 0; l < 2; l++) {
                    const int r = (int8_t)pp[8 + l];
                    const int slot = r & 31;
                    const unsigned fref = (r >> 5) & 1, bref = (r >> 6) & 1;
                    const unsigned wrong = (slot >= dpb_slots) |
                                           (fpic ? ((fref ^ 1u) | ((slot == dst) & (bref == (unsigned)own_bottom)))
                                                 : ((slot == dst) | (fref & (unsigned)!mb_field)));
                    bad |= (r >= 0) & wrong;
                }
            }
            if (bad) return H264R_ERR_BAD_RECORD;
        } else if (m.type == H264R_MB_IPCM) {
            if (m.aux >= npcm) return H264R_ERR_BAD_RECORD;
        }
    }
    return H264R_OK;
}

extern "C" int h264r_validate_picture(const h264r_picture *pic, int dpb_slots)
{
    const int r = validate_header(pic, dpb_slots);
    return r ? r : validate_mbs(pic, dpb_slots, 0, pic->num_mbs);
}

// ---------------------------------------------------------------- launching
static int ensure(h264r_ctx *ctx, uint8_t **p, uint64_t *cap, uint64_t need, bool pinned)
{
    if (need <= *cap) return H264R_OK;
    uint64_t n = align_up(need + need / 4, 1 << 16);
    if (*p) {
        if (pinned) cudaFreeHost(*p);
        else cudaFree(*p);
        *p = nullptr;
    }
    cudaError_t e = pinned ? cudaMallocHost(p, n) : cudaMalloc(p, n);
    if (e != cudaSuccess) {
        *cap = 0;
        set_err(ctx, "allocation of %llu bytes failed: %s", (unsigned long long)n, cudaGetErrorString(e));
        return H264R_ERR_NO_MEMORY;
    }
    *cap = n;
    return H264R_OK;
}

static int wait_slot(h264r_ctx *ctx, LaunchBuf &b)
{
    if (b.pending) {
        CUDA_OR(ctx, cudaEventSynchronize(b.done));
        b.pending = false;
    }
    return H264R_OK;
}

static bool all_flat(const h264r_picture *pic)
{
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 16; k++)
            if (pic->scaling4x4[i][k] != 16) return false;
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 64; k++)
            if (pic->scaling8x8[i][k] != 16) return false;
    return true;
}

struct BatchItem {
    h264r_stream *s;
    const h264r_picture *pic;  // pointers are device memory
    const uint8_t *scaling_dev;
    bool has_intra;
};

// Build the PicDesc array + counters in b.host, upload, run the kernels.
// a slot about to be written: wait (on cs) for its pending copy to the host
static void wait_slot_copy(h264r_stream *s, int slot, cudaStream_t cs)
{
    if (slot >= 0 && slot < s->cfg.dpb_slots && s->slot_pending[slot].exchange(0))
        cudaStreamWaitEvent(cs, s->slot_ev[slot], 0);
}

// Geometry mix of a batch: an order-independent hash of the width, height
// and MBAFF flag of its pictures (the key of the autotuner's choices).
static uint64_t mix_key(int n, const h264r_picture *const *pics)
{
    uint64_t k = 0;
    for (int i = 0; i < n; i++) {
        uint64_t z = (uint64_t)pics[i]->width_mbs | (uint64_t)pics[i]->height_mbs << 16 | (uint64_t)(pics[i]->mbaff ? 1 : 0) << 32 |
                     (uint64_t)pics[i]->structure << 33;
        z += 0x9e3779b97f4a7c15ull;  // splitmix64 finaliser
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        k += z ^ (z >> 31);
    }
    return k;
}

static bool valid_tuning(const h264r_tuning &t)
{
    return (t.inter_mbs_per_cta == 2 || t.inter_mbs_per_cta == 4 || t.inter_mbs_per_cta == 8) &&
           (t.deblock_pairs_per_cta == 4 || t.deblock_pairs_per_cta == 8);
}

static h264r_tuning tuning_for(h264r_ctx *ctx, uint64_t key)
{
    std::lock_guard<std::mutex> lk(ctx->tune_mu);
    auto it = ctx->tuned.find(key);
    return it != ctx->tuned.end() ? it->second : ctx->tuning;
}

// The sizes of one launch sequence (see launch()).
struct Seq {
    const PicDesc *dd;
    LaunchState st;
    int n;
    uint64_t total, mbs, rows;
    uint32_t dbf_units, db_units;
    bool any_intra, any_deblock, bs_aside;
    int inter_w, dbf_w;
};

// Enqueue the descriptor upload and the kernels of one launch sequence on cs
// (directly, or into a stream capture); *kernels receives how many kernels.
static int enqueue_sequence(h264r_ctx *ctx, cudaStream_t cs, LaunchBuf &b, const Seq &q, cudaStream_t side,
                            const std::array<cudaEvent_t, 5> *ev, uint32_t *kernels, bool early_bs = false)
{
    uint32_t nk = 0;
    const unsigned bs_grid = (unsigned)((q.mbs + h264r::kBsMbsPerBlock - 1) / h264r::kBsMbsPerBlock);
    // The strengths depend on the records alone, so for frame pictures k_bs
    // runs on the side stream of the batch's first stream while k_inter and
    // k_intra fill the device; the deblocking kernels wait for it.  MBAFF
    // strengths cost more and slow the intra wavefront they would share the
    // SMs with (measured: 6 % fewer 1080i frames/s), so they stay in line.
    // Launched directly (not captured), the side stream also takes the
    // descriptor upload and starts k_bs right away, without waiting for the
    // kernels of the batch before on cs: its strengths are ready when this
    // batch's deblocking starts.  (The descriptors and strength tables of
    // this launch slot are free: wait_slot saw its last use complete.)
    if (q.bs_aside && early_bs) {
        if (b.wait_upload) CUDA_OR(ctx, cudaStreamWaitEvent(side, b.uploaded, 0));
        CUDA_OR(ctx, cudaMemcpyAsync(b.dev, b.host, q.total, cudaMemcpyHostToDevice, side));
        CUDA_OR(ctx, cudaEventRecord(b.fork, side));
        h264r::k_bs<<<bs_grid, 128, 0, side>>>(q.dd, q.n, (uint32_t)q.mbs, q.st);
        nk++;
        CUDA_OR(ctx, cudaEventRecord(b.join, side));
        CUDA_OR(ctx, cudaStreamWaitEvent(cs, b.fork, 0));
    } else {
        CUDA_OR(ctx, cudaMemcpyAsync(b.dev, b.host, q.total, cudaMemcpyHostToDevice, cs));
        if (q.bs_aside) {
            CUDA_OR(ctx, cudaEventRecord(b.fork, cs));
            CUDA_OR(ctx, cudaStreamWaitEvent(side, b.fork, 0));
            h264r::k_bs<<<bs_grid, 128, 0, side>>>(q.dd, q.n, (uint32_t)q.mbs, q.st);
            nk++;
            CUDA_OR(ctx, cudaEventRecord(b.join, side));
        }
    }
    if (ev) cudaEventRecord((*ev)[0], cs);
    const unsigned inter_grid = (unsigned)((q.mbs + q.inter_w - 1) / q.inter_w);
    if (q.inter_w == 2)
        h264r::k_inter2<<<inter_grid, 64, 0, cs>>>(q.dd, q.n, (uint32_t)q.mbs, q.st);
    else if (q.inter_w == 8)
        h264r::k_inter8<<<inter_grid, 256, 0, cs>>>(q.dd, q.n, (uint32_t)q.mbs, q.st);
    else
        h264r::k_inter<<<inter_grid, 128, 0, cs>>>(q.dd, q.n, (uint32_t)q.mbs, q.st);
    nk++;
    if (ev) cudaEventRecord((*ev)[1], cs);
    if (q.any_intra) {
        h264r::k_intra<<<(unsigned)q.rows, 32, 0, cs>>>(q.dd, q.n, (uint32_t)q.rows, q.st);
        nk++;
    }
    if (ev) cudaEventRecord((*ev)[2], cs);
    if (q.any_deblock) {
        if (q.bs_aside) {
            CUDA_OR(ctx, cudaStreamWaitEvent(cs, b.join, 0));
        } else {
            h264r::k_bs<<<bs_grid, 128, 0, cs>>>(q.dd, q.n, (uint32_t)q.mbs, q.st);
            nk++;
        }
    }
    if (ev) cudaEventRecord((*ev)[3], cs);
    if (q.any_deblock) {
        if (q.dbf_units) {
            if (q.dbf_w == 4)
                h264r::k_deblock_frame4<<<q.dbf_units, 128, 0, cs>>>(q.dd, q.n, q.dbf_units, q.st);
            else
                h264r::k_deblock_frame<<<q.dbf_units, 32 * h264r::kDbWarps, 0, cs>>>(q.dd, q.n, q.dbf_units, q.st);
            nk++;
        }
        if (q.db_units) {
            h264r::k_deblock<<<q.db_units, 32 * h264r::kMbWarps, 0, cs>>>(q.dd, q.n, q.db_units, q.st);
            nk++;
        }
    }
    if (ev) cudaEventRecord((*ev)[4], cs);
    *kernels = nk;
    return H264R_OK;
}

// The graph cache entry of this launch shape in b, noting a first sighting
// (returns nullptr then: the sequence is launched directly).
static GraphEntry *graph_entry(LaunchBuf &b, const GraphKey &key)
{
    b.graph_clock++;
    for (int i = 0; i < b.ngraphs; i++)
        if (memcmp(&b.graphs[i].key, &key, sizeof(key)) == 0) {
            b.graphs[i].used = b.graph_clock;
            return &b.graphs[i];
        }
    int v = b.ngraphs;
    if (v == kGraphCache) {
        v = 0;
        for (int i = 1; i < kGraphCache; i++)
            if (b.graphs[i].used < b.graphs[v].used) v = i;
        if (b.graphs[v].exec) cudaGraphExecDestroy(b.graphs[v].exec);
    } else {
        b.ngraphs++;
    }
    b.graphs[v] = GraphEntry();
    b.graphs[v].key = key;
    b.graphs[v].used = b.graph_clock;
    return nullptr;
}

// early_bs: the records are complete, or ordered by b.uploaded
// (b.wait_upload): k_bs need not wait for the work queued on cs
static int launch(h264r_ctx *ctx, cudaStream_t cs, LaunchBuf &b, const std::vector<BatchItem> &items, bool any_intra,
                  bool early_bs)
{
    const int n = (int)items.size();
    std::vector<const h264r_picture *> pl(n);
    for (int i = 0; i < n; i++) pl[i] = items[i].pic;
    const h264r_tuning tune = tuning_for(ctx, mix_key(n, pl.data()));
    uint64_t rows = 0, mbs = 0;
    for (auto &it : items) {
        uint32_t uh = (it.pic->mbaff || it.pic->structure != H264R_STRUCT_FRAME) ? it.pic->height_mbs / 2 : it.pic->height_mbs;
        rows += uh;
        mbs += it.pic->num_mbs;
    }
    const uint64_t desc_bytes = align_up(sizeof(PicDesc) * n, kAlign);
    const uint64_t ticket_off = desc_bytes;
    const uint64_t prog_off = ticket_off + kAlign;
    const uint64_t total = prog_off + align_up(12 * rows + 8, kAlign);
    int rc = ensure(ctx, &b.host, &b.host_cap, total, true);
    if (rc) return rc;
    rc = ensure(ctx, &b.dev, &b.dev_cap, total, false);
    if (rc) return rc;
    rc = ensure(ctx, &b.bs, &b.bs_cap, mbs * h264r::kBsBytes + 16, false);
    if (rc) return rc;
    if (any_intra) {
        rc = ensure(ctx, &b.ires, &b.ires_cap, mbs * 768 + 16, false);
        if (rc) return rc;
    }
    memset(b.host, 0, total);
    for (auto &it : items) wait_slot_copy(it.s, it.pic->dst_slot, cs);
    PicDesc *d = (PicDesc *)b.host;
    uint64_t mb_base = 0, row_base = 0, prog = 0, db_base = 0, dbf_base = 0;
    for (int i = 0; i < n; i++) {
        const h264r_picture *pic = items[i].pic;
        h264r_stream *s = items[i].s;
        PicDesc &p = d[i];
        // a field picture runs as a picture of its field's size whose planes
        // step two frame lines from the field's first line
        const int bot = pic->structure == H264R_STRUCT_BOTTOM;
        p.fpic = pic->structure;
        p.wmb = pic->width_mbs;
        p.hmb = p.fpic ? pic->height_mbs / 2 : pic->height_mbs;
        p.W = p.wmb * 16;
        p.H = p.hmb * 16;
        p.Wc = p.W / 2;
        p.Hc = p.H / 2;
        p.fH = pic->height_mbs * 16;
        p.ys = p.fpic ? 2 * p.W : p.W;
        p.cs = p.ys / 2;
        p.mbaff = pic->mbaff;
        p.deblock = pic->deblock;
        p.num_mbs = pic->num_mbs;
        p.num_slices = pic->num_slices;
        p.num_weights = pic->num_weights;
        p.num_pcm = pic->num_pcm;
        p.motion_bytes = pic->motion_bytes;
        p.coef_bytes = pic->coef_bytes;
        p.mbs = pic->mbs;
        p.slices = pic->slices;
        p.weights = pic->weights;
        p.motion = pic->motion;
        p.coef = pic->coef;
        p.pcm = pic->pcm;
        p.scaling = items[i].scaling_dev;
        p.flat_scaling = all_flat(pic) ? 1 : 0;
        p.dpb = s->dpb;
        p.slot_bytes = s->slot_bytes;
        p.nslots = s->cfg.dpb_slots;
        uint8_t *slot = s->dpb + (uint64_t)pic->dst_slot * s->slot_bytes;
        p.dst = slot + (size_t)bot * p.W;
        p.coff = p.W * p.fH + bot * p.Wc - bot * p.W;
        p.cplane = p.Wc * (p.fH / 2);
        p.bs = b.bs + mb_base * h264r::kBsBytes;
        p.ires = any_intra ? (int16_t *)b.ires + mb_base * 384 : nullptr;
        p.units_w = pic->width_mbs;
        p.units_h = pic->mbaff ? pic->height_mbs / 2 : p.hmb;
        p.progress = (int *)(b.dev + prog_off) + prog;
        p.mb_base = (uint32_t)mb_base;
        p.row_base = (uint32_t)row_base;
        p.db_units = h264r::deblock_units(p.mbaff, p.units_h);
        p.db_base = (uint32_t)db_base;
        db_base += p.db_units;
        p.dbf_units = h264r::deblock_frame_units(p.mbaff, p.units_h, (uint32_t)tune.deblock_pairs_per_cta);
        p.dbf_base = (uint32_t)dbf_base;
        dbf_base += p.dbf_units;
        p.deblock_stop = 0xFFFFFFFFu;
        mb_base += pic->num_mbs;
        row_base += p.units_h;
        prog += 3 * p.units_h;
    }
    const bool withhold = ctx->withhold.load() != 0;
    if (withhold) {
        // the wavefronts' first tickets are never handed out: the first
        // picture's first intra row and first deblocking blocks do not run,
        // so the rows below them wait on progress that is never published
        unsigned int *t = (unsigned int *)(b.host + ticket_off);
        t[0] = 1;
        t[1] = 2;
        t[2] = 2;
    }
    Seq q;
    q.dd = (const PicDesc *)b.dev;
    q.st.error = ctx->d_error;
    q.st.ticket = (unsigned int *)(b.dev + ticket_off);
    q.st.spin_limit = ctx->spin_limit.load();
    q.n = n;
    q.total = total;
    q.mbs = mbs;
    q.rows = rows;
    q.dbf_units = (uint32_t)dbf_base;
    q.db_units = (uint32_t)db_base;
    q.any_intra = any_intra;
    q.any_deblock = false;
    for (auto &it : items) q.any_deblock = q.any_deblock || it.pic->deblock;
    // kernel timing keeps k_bs in line, so that each kernel is timed alone
    q.bs_aside = q.any_deblock && db_base == 0 && !ctx->timing;
    q.inter_w = tune.inter_mbs_per_cta;
    q.dbf_w = tune.deblock_pairs_per_cta;
    cudaStream_t side = items[0].s->side;
    uint32_t nk = 0;
    GraphEntry *g = nullptr;
    // no graph of our own inside a capture the caller is making of cs
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (tune.graphs && !ctx->timing && !withhold && cudaStreamIsCapturing(cs, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) {
        GraphKey key;
        memset(&key, 0, sizeof(key));
        key.host = b.host;
        key.dev = b.dev;
        key.bs = b.bs;
        key.ires = any_intra ? b.ires : nullptr;
        key.cs = cs;
        key.side = side;
        key.total = total;
        key.mbs = mbs;
        key.rows = rows;
        key.n = (uint32_t)n;
        key.dbf_units = q.dbf_units;
        key.db_units = q.db_units;
        key.flags = (q.any_intra ? 1u : 0u) | (q.any_deblock ? 2u : 0u) | (q.bs_aside ? 4u : 0u);
        key.inter_w = (uint32_t)q.inter_w;
        key.dbf_w = (uint32_t)q.dbf_w;
        g = graph_entry(b, key);
    }
    if (g && !g->exec) {
        // second sighting of this shape: capture the sequence once
        CUDA_OR(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_sequence(ctx, cs, b, q, side, nullptr, &nk);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(cs, &graph);
        if (rc == H264R_OK && e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (rc) return rc;
        if (e != cudaSuccess) {
            g->exec = nullptr;
            set_err(ctx, "launch graph capture: %s", cudaGetErrorString(e));
            return H264R_ERR_CUDA;
        }
        g->kernels = nk;
        ctx->graphs_captured++;
    }
    if (g) {
        CUDA_OR(ctx, cudaGraphLaunch(g->exec, cs));
        ctx->launches += g->kernels;
        ctx->graph_replays++;
    } else {
        std::array<cudaEvent_t, 5> ev{};
        if (ctx->timing) ev = *take_events(ctx);
        rc = enqueue_sequence(ctx, cs, b, q, side, ctx->timing ? &ev : nullptr, &nk, early_bs);
        b.wait_upload = false;
        if (rc) return rc;
        ctx->launches += nk;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_err(ctx, "kernel launch: %s", cudaGetErrorString(e));
        return H264R_ERR_CUDA;
    }
    CUDA_OR(ctx, cudaEventRecord(b.done, cs));
    b.pending = true;
    return H264R_OK;
}

static bool has_intra_mbs(const h264r_picture *pic)
{
    for (uint32_t a = 0; a < pic->num_mbs; a++) {
        int t = pic->mbs[a].type;
        if (t == H264R_MB_I4x4 || t == H264R_MB_I8x8 || t == H264R_MB_I16x16) return true;
    }
    return false;
}

extern "C" int h264r_submit_picture(h264r_stream *s, const h264r_picture *pic)
{
    if (!s || !pic) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    int rc = h264r_validate_picture(pic, s->cfg.dpb_slots);
    if (rc) {
        set_err(ctx, "h264r_submit_picture: records rejected by the validator (%d)", rc);
        return rc;
    }
    if (pic->width_mbs != s->cfg.width_mbs || pic->height_mbs != s->cfg.height_mbs) {
        set_err(ctx, "h264r_submit_picture: picture size differs from the stream's");
        return H264R_ERR_INVALID_ARG;
    }
    cudaSetDevice(ctx->device);
    LaunchBuf &b = s->ring[s->next];
    s->next = (s->next + 1) % kRing;
    rc = wait_slot(ctx, b);
    if (rc) return rc;
    // pack the records: mbs | slices | weights | motion | coef | pcm | scaling
    uint64_t off[7], sz[7] = {sizeof(h264r_mb) * pic->num_mbs, sizeof(h264r_slice) * pic->num_slices,
                              sizeof(h264r_weight) * pic->num_weights, pic->motion_bytes, pic->coef_bytes,
                              384ull * pic->num_pcm, 480};
    uint64_t tot = 0;
    for (int i = 0; i < 7; i++) {
        off[i] = tot;
        tot = align_up(tot + sz[i], kAlign);
    }
    rc = ensure(ctx, &b.rec_host, &b.rec_host_cap, tot, true);
    if (rc) return rc;
    rc = ensure(ctx, &b.rec_dev, &b.rec_dev_cap, tot, false);
    if (rc) return rc;
    const void *src[6] = {pic->mbs, pic->slices, pic->weights, pic->motion, pic->coef, pic->pcm};
    for (int i = 0; i < 6; i++)
        if (sz[i]) memcpy(b.rec_host + off[i], src[i], sz[i]);
    memcpy(b.rec_host + off[6], pic->scaling4x4, 96);
    memcpy(b.rec_host + off[6] + 96, pic->scaling8x8, 384);
    CUDA_OR(ctx, cudaMemcpyAsync(b.rec_dev, b.rec_host, tot, cudaMemcpyHostToDevice, s->cs));
    CUDA_OR(ctx, cudaEventRecord(b.uploaded, s->cs));
    b.wait_upload = true;
    h264r_picture dp = *pic;
    dp.mbs = (const h264r_mb *)(b.rec_dev + off[0]);
    dp.slices = (const h264r_slice *)(b.rec_dev + off[1]);
    dp.weights = (const h264r_weight *)(b.rec_dev + off[2]);
    dp.motion = b.rec_dev + off[3];
    dp.coef = b.rec_dev + off[4];
    dp.pcm = b.rec_dev + off[5];
    std::vector<BatchItem> items(1);
    items[0].s = s;
    items[0].pic = &dp;
    items[0].scaling_dev = b.rec_dev + off[6];
    items[0].has_intra = has_intra_mbs(pic);
    return launch(ctx, s->cs, b, items, items[0].has_intra, true);
}

// Device-resident records: the scaling lists are read from the host struct
// and staged with the launch buffer.
static int submit_device(h264r_ctx *ctx, cudaStream_t cs, LaunchBuf &b, int n, h264r_stream *const *streams,
                         const h264r_picture *pics)
{
    // scaling lists of every picture go into the record staging area
    uint64_t tot = align_up(480ull * n, kAlign);
    int rc = ensure(ctx, &b.rec_host, &b.rec_host_cap, tot, true);
    if (rc) return rc;
    rc = ensure(ctx, &b.rec_dev, &b.rec_dev_cap, tot, false);
    if (rc) return rc;
    std::vector<BatchItem> items(n);
    bool any_intra = false;
    for (int i = 0; i < n; i++) {
        memcpy(b.rec_host + 480ull * i, pics[i].scaling4x4, 96);
        memcpy(b.rec_host + 480ull * i + 96, pics[i].scaling8x8, 384);
        items[i].s = streams[i];
        items[i].pic = &pics[i];
        items[i].scaling_dev = b.rec_dev + 480ull * i;
        // device records: the intra kernel is always launched (it exits
        // immediately on rows without intra MBs)
        items[i].has_intra = true;
        any_intra = true;
    }
    CUDA_OR(ctx, cudaMemcpyAsync(b.rec_dev, b.rec_host, tot, cudaMemcpyHostToDevice, cs));
    return launch(ctx, cs, b, items, any_intra, ctx->records_ready);
}

static int check_device_pic(h264r_stream *s, const h264r_picture *pic)
{
    if (!s || !pic || !pic->mbs || !pic->slices || !pic->weights) return H264R_ERR_INVALID_ARG;
    if (pic->num_slices == 0 || pic->num_weights == 0) return H264R_ERR_BAD_RECORD;
    if (pic->structure > H264R_STRUCT_BOTTOM) return H264R_ERR_INVALID_ARG;
    if (pic->width_mbs != s->cfg.width_mbs || pic->height_mbs != s->cfg.height_mbs || pic->num_mbs != picture_mbs(pic) ||
        pic->dst_slot >= s->cfg.dpb_slots || ((pic->mbaff || pic->structure != H264R_STRUCT_FRAME) && (pic->height_mbs & 1)) ||
        (pic->mbaff && pic->structure != H264R_STRUCT_FRAME))
        return H264R_ERR_INVALID_ARG;
    return H264R_OK;
}

extern "C" int h264r_submit_picture_device(h264r_stream *s, const h264r_picture *pic)
{
    int rc = check_device_pic(s, pic);
    if (rc) {
        if (s) set_err(s->ctx, "h264r_submit_picture_device: bad picture (%d)", rc);
        return rc;
    }
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    LaunchBuf &b = s->ring[s->next];
    s->next = (s->next + 1) % kRing;
    rc = wait_slot(ctx, b);
    if (rc) return rc;
    h264r_stream *const arr[1] = {s};
    return submit_device(ctx, s->cs, b, 1, arr, pic);
}

static int check_device_batch(h264r_ctx *ctx, int n, h264r_stream *const *streams, const h264r_picture *pics)
{
    if (!ctx || n <= 0 || !streams || !pics) return H264R_ERR_INVALID_ARG;
    if ((uint32_t)n > ctx->max_batch) {
        set_err(ctx, "h264r_submit_batch_device: %d pictures exceed the batch limit %u", n, ctx->max_batch);
        return H264R_ERR_BUSY;
    }
    for (int i = 0; i < n; i++) {
        if (!streams[i] || streams[i]->ctx != ctx) return H264R_ERR_INVALID_ARG;
        int rc = check_device_pic(streams[i], &pics[i]);
        if (rc) {
            set_err(ctx, "h264r_submit_batch_device: picture %d rejected (%d)", i, rc);
            return rc;
        }
    }
    return H264R_OK;
}

extern "C" int h264r_submit_batch_device_on(h264r_ctx *ctx, void *cuda_stream, int n, h264r_stream *const *streams,
                                            const h264r_picture *pics)
{
    int rc = check_device_batch(ctx, n, streams, pics);
    if (rc) return rc;
    if (!cuda_stream) return H264R_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    LaunchBuf &b = ctx->batch_ring[ctx->batch_next];
    ctx->batch_next = (ctx->batch_next + 1) % kBatchRing;
    rc = wait_slot(ctx, b);
    if (rc) return rc;
    return submit_device(ctx, (cudaStream_t)cuda_stream, b, n, streams, pics);
}

extern "C" int h264r_submit_batch_device(h264r_ctx *ctx, int n, h264r_stream *const *streams, const h264r_picture *pics)
{
    int rc = check_device_batch(ctx, n, streams, pics);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    LaunchBuf &b = ctx->batch_ring[ctx->batch_next];
    ctx->batch_next = (ctx->batch_next + 1) % kBatchRing;
    rc = wait_slot(ctx, b);
    if (rc) return rc;
    // the batch runs on the CUDA stream of its first member, after any work
    // already queued on the other members, which then wait for it
    cudaStream_t cs = streams[0]->cs;
    cudaEvent_t ev;
    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (int i = 1; i < n; i++) {
        if (streams[i]->cs == cs) continue;
        cudaEventRecord(ev, streams[i]->cs);
        cudaStreamWaitEvent(cs, ev, 0);
    }
    rc = submit_device(ctx, cs, b, n, streams, pics);
    if (rc == H264R_OK) {
        cudaEventRecord(ev, cs);
        for (int i = 1; i < n; i++)
            if (streams[i]->cs != cs) cudaStreamWaitEvent(streams[i]->cs, ev, 0);
    }
    cudaEventDestroy(ev);
    return rc;
}

extern "C" int h264r_ctx_set_tuning(h264r_ctx *ctx, const h264r_tuning *t)
{
    if (!ctx || !t) return H264R_ERR_INVALID_ARG;
    h264r_tuning v = *t;
    if (!v.inter_mbs_per_cta) v.inter_mbs_per_cta = 4;
    if (!v.deblock_pairs_per_cta) v.deblock_pairs_per_cta = 8;
    v.graphs = v.graphs ? 1 : 0;
    v.reserved = 0;
    if (!valid_tuning(v)) {
        set_err(ctx, "h264r_ctx_set_tuning: %d MBs or %d row pairs per block is not a launch shape", t->inter_mbs_per_cta,
                t->deblock_pairs_per_cta);
        return H264R_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(ctx->tune_mu);
    ctx->tuning = v;
    return H264R_OK;
}

extern "C" int h264r_ctx_get_tuning(h264r_ctx *ctx, int n, const h264r_picture *pics, h264r_tuning *out)
{
    if (!ctx || !out || n < 0 || (n > 0 && !pics)) return H264R_ERR_INVALID_ARG;
    std::vector<const h264r_picture *> pl(n);
    for (int i = 0; i < n; i++) pl[i] = &pics[i];
    if (n == 0) {
        std::lock_guard<std::mutex> lk(ctx->tune_mu);
        *out = ctx->tuning;
    } else {
        *out = tuning_for(ctx, mix_key(n, pl.data()));
    }
    return H264R_OK;
}

extern "C" int h264r_ctx_set_mix_tuning(h264r_ctx *ctx, int n, const h264r_picture *pics, const h264r_tuning *t)
{
    if (!ctx || n <= 0 || !pics || !t) return H264R_ERR_INVALID_ARG;
    h264r_tuning v = *t;
    if (!v.inter_mbs_per_cta) v.inter_mbs_per_cta = 4;
    if (!v.deblock_pairs_per_cta) v.deblock_pairs_per_cta = 8;
    v.graphs = v.graphs ? 1 : 0;
    v.reserved = 0;
    if (!valid_tuning(v)) {
        set_err(ctx, "h264r_ctx_set_mix_tuning: %d MBs or %d row pairs per block is not a launch shape", t->inter_mbs_per_cta,
                t->deblock_pairs_per_cta);
        return H264R_ERR_INVALID_ARG;
    }
    std::vector<const h264r_picture *> pl(n);
    for (int i = 0; i < n; i++) pl[i] = &pics[i];
    const uint64_t key = mix_key(n, pl.data());
    std::lock_guard<std::mutex> lk(ctx->tune_mu);
    ctx->tuned[key] = v;
    return H264R_OK;
}

extern "C" int h264r_autotune_batch_device(h264r_ctx *ctx, int n, h264r_stream *const *streams, const h264r_picture *pics,
                                           int reps, h264r_tuning *best, float *best_ms)
{
    if (!ctx || n <= 0 || !streams || !pics || !streams[0]) return H264R_ERR_INVALID_ARG;
    if (reps < 1) reps = 1;
    std::vector<const h264r_picture *> pl(n);
    for (int i = 0; i < n; i++) pl[i] = &pics[i];
    const uint64_t key = mix_key(n, pl.data());
    // candidates: every shape without and with graph replay; the context's
    // current tuning of this mix is the incumbent
    std::vector<h264r_tuning> cand;
    for (int graphs = 0; graphs < 2; graphs++)
        for (int iw : {2, 4, 8})
            for (int dw : {4, 8}) cand.push_back(h264r_tuning{iw, dw, graphs, 0});
    const h264r_tuning cur = tuning_for(ctx, key);
    size_t inc = 0;
    for (size_t c = 0; c < cand.size(); c++)
        if (cand[c].inter_mbs_per_cta == cur.inter_mbs_per_cta && cand[c].deblock_pairs_per_cta == cur.deblock_pairs_per_cta &&
            cand[c].graphs == cur.graphs)
            inc = c;
    // rounds over all candidates in turn, so that a slow phase of the device
    // (clocks, other work) does not favour one candidate; each keeps its best
    // round
    constexpr int kRounds = 3;
    std::vector<double> best_of(cand.size(), 1e30);
    for (int round = 0; round < kRounds; round++)
        for (size_t c = 0; c < cand.size(); c++) {
            const h264r_tuning &t = cand[c];
            {
                std::lock_guard<std::mutex> lk(ctx->tune_mu);
                ctx->tuned[key] = t;
            }
            // warm-up: with graphs, every launch buffer of the ring sees
            // the shape twice (first sighting, capture) before timing
            const int warm = t.graphs ? 2 * kBatchRing : 1;
            int rc = H264R_OK;
            for (int r = 0; r < warm && rc == H264R_OK; r++) rc = h264r_submit_batch_device(ctx, n, streams, pics);
            if (rc == H264R_OK) rc = h264r_stream_sync(streams[0]);
            const auto t0 = std::chrono::steady_clock::now();
            for (int r = 0; r < reps && rc == H264R_OK; r++) rc = h264r_submit_batch_device(ctx, n, streams, pics);
            if (rc == H264R_OK) rc = h264r_stream_sync(streams[0]);
            const auto t1 = std::chrono::steady_clock::now();
            if (rc) {
                std::lock_guard<std::mutex> lk(ctx->tune_mu);
                ctx->tuned[key] = cur;
                return rc;
            }
            best_of[c] = std::min(best_of[c], std::chrono::duration<double, std::milli>(t1 - t0).count() / reps);
        }
    // the fastest, unless it beats the incumbent by less than 3 % (within
    // the spread of repeated measurements)
    size_t win = inc;
    for (size_t c = 0; c < cand.size(); c++)
        if (best_of[c] < best_of[win]) win = c;
    if (best_of[win] > 0.97 * best_of[inc]) win = inc;
    const h264r_tuning top = cand[win];
    const double top_ms = best_of[win];
    {
        std::lock_guard<std::mutex> lk(ctx->tune_mu);
        ctx->tuned[key] = top;
    }
    if (best) *best = top;
    if (best_ms) *best_ms = (float)top_ms;
    return H264R_OK;
}

extern "C" uint64_t h264r_ctx_graph_replays(const h264r_ctx *ctx) { return ctx ? ctx->graph_replays.load() : 0; }

extern "C" uint64_t h264r_ctx_graphs_captured(const h264r_ctx *ctx) { return ctx ? ctx->graphs_captured.load() : 0; }

extern "C" int h264r_output(h264r_stream *s, int slot, uint8_t *y, uint8_t *cb, uint8_t *cr)
{
    if (!s || slot < 0 || slot >= s->cfg.dpb_slots || !y || !cb || !cr) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const uint64_t W = s->cfg.width_mbs * 16ull, H = s->cfg.height_mbs * 16ull;
    const uint8_t *base = s->dpb + (uint64_t)slot * s->slot_bytes;
    CUDA_OR(ctx, cudaMemcpyAsync(y, base, W * H, cudaMemcpyDeviceToHost, s->cs));
    CUDA_OR(ctx, cudaMemcpyAsync(cb, base + W * H, W * H / 4, cudaMemcpyDeviceToHost, s->cs));
    CUDA_OR(ctx, cudaMemcpyAsync(cr, base + W * H + W * H / 4, W * H / 4, cudaMemcpyDeviceToHost, s->cs));
    return H264R_OK;
}

extern "C" int h264r_output_async(h264r_stream *s, int slot, uint8_t *y, uint8_t *cb, uint8_t *cr)
{
    if (!s || slot < 0 || slot >= s->cfg.dpb_slots || !y || !cb || !cr) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const uint64_t W = s->cfg.width_mbs * 16ull, H = s->cfg.height_mbs * 16ull;
    const uint8_t *base = s->dpb + (uint64_t)slot * s->slot_bytes;
    // after everything enqueued on the stream so far (the picture's batch)
    CUDA_OR(ctx, cudaEventRecord(s->out_ready, s->cs));
    CUDA_OR(ctx, cudaStreamWaitEvent(s->out, s->out_ready, 0));
    if (cb == y + W * H && cr == cb + W * H / 4) {  // one buffer: one copy (the slot's planes follow each other too)
        CUDA_OR(ctx, cudaMemcpyAsync(y, base, W * H * 3 / 2, cudaMemcpyDeviceToHost, s->out));
    } else {
        CUDA_OR(ctx, cudaMemcpyAsync(y, base, W * H, cudaMemcpyDeviceToHost, s->out));
        CUDA_OR(ctx, cudaMemcpyAsync(cb, base + W * H, W * H / 4, cudaMemcpyDeviceToHost, s->out));
        CUDA_OR(ctx, cudaMemcpyAsync(cr, base + W * H + W * H / 4, W * H / 4, cudaMemcpyDeviceToHost, s->out));
    }
    CUDA_OR(ctx, cudaEventRecord(s->slot_ev[slot], s->out));
    s->slot_pending[slot] = 1;
    return H264R_OK;
}

extern "C" int h264r_output_async_on(h264r_stream *s, int slot, uint8_t *y, uint8_t *cb, uint8_t *cr, void *cuda_stream)
{
    if (!s || slot < 0 || slot >= s->cfg.dpb_slots || !y || !cb || !cr || !cuda_stream) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const cudaStream_t os = (cudaStream_t)cuda_stream;
    const uint64_t W = s->cfg.width_mbs * 16ull, H = s->cfg.height_mbs * 16ull;
    const uint8_t *base = s->dpb + (uint64_t)slot * s->slot_bytes;
    if (cb == y + W * H && cr == cb + W * H / 4) {
        CUDA_OR(ctx, cudaMemcpyAsync(y, base, W * H * 3 / 2, cudaMemcpyDeviceToHost, os));
    } else {
        CUDA_OR(ctx, cudaMemcpyAsync(y, base, W * H, cudaMemcpyDeviceToHost, os));
        CUDA_OR(ctx, cudaMemcpyAsync(cb, base + W * H, W * H / 4, cudaMemcpyDeviceToHost, os));
        CUDA_OR(ctx, cudaMemcpyAsync(cr, base + W * H + W * H / 4, W * H / 4, cudaMemcpyDeviceToHost, os));
    }
    CUDA_OR(ctx, cudaEventRecord(s->slot_ev[slot], os));  // a launch rewriting the slot waits for the copy
    s->slot_pending[slot] = 1;
    return H264R_OK;
}

extern "C" int h264r_output_bgr24_device(h264r_stream *s, int slot, void *dst, uint32_t row_bytes, int flip)
{
    if (!s || slot < 0 || slot >= s->cfg.dpb_slots || !dst || ((uintptr_t)dst & 3)) return H264R_ERR_INVALID_ARG;
    const int W = s->cfg.width_mbs * 16, H = s->cfg.height_mbs * 16;
    if ((row_bytes & 3) || row_bytes < 3u * W) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const uint8_t *base = s->dpb + (uint64_t)slot * s->slot_bytes;
    dim3 grid((W / 4 + 255) / 256, H);
    h264r::k_bgr24<<<grid, 256, 0, s->cs>>>(base, W, H, (uint8_t *)dst, (int)row_bytes, flip ? 1 : 0);
    CUDA_OR(ctx, cudaGetLastError());
    ctx->launches++;
    return H264R_OK;
}

extern "C" int h264r_output_bgr24(h264r_stream *s, int slot, uint8_t *dst, uint32_t row_bytes, int flip)
{
    if (!s || !dst) return H264R_ERR_INVALID_ARG;
    const uint64_t bytes = (uint64_t)s->cfg.height_mbs * 16 * row_bytes;
    int rc = ensure(s->ctx, &s->bgr, &s->bgr_cap, bytes, false);
    if (rc) return rc;
    rc = h264r_output_bgr24_device(s, slot, s->bgr, row_bytes, flip);
    if (rc) return rc;
    CUDA_OR(s->ctx, cudaMemcpyAsync(dst, s->bgr, bytes, cudaMemcpyDeviceToHost, s->cs));
    return H264R_OK;
}

static void put_le(uint8_t *p, uint32_t v, int n)
{
    for (int i = 0; i < n; i++) p[i] = (uint8_t)(v >> (8 * i));
}

extern "C" int h264r_write_bmp(const char *path, const uint8_t *bgr, uint32_t width, uint32_t height, uint32_t row_bytes)
{
    if (!path || !bgr || !width || !height || row_bytes < 3u * width) return H264R_ERR_INVALID_ARG;
    FILE *fp = fopen(path, "wb");
    if (!fp) return H264R_ERR_IO;
    // 'BM', then the file header (size, reserved, offset) and the 40-byte info header
    uint8_t hdr[54] = {0};
    hdr[0] = 'B';
    hdr[1] = 'M';
    put_le(hdr + 2, height * row_bytes + 54, 4);
    put_le(hdr + 10, 54, 4);
    put_le(hdr + 14, 40, 4);
    put_le(hdr + 18, width, 4);
    put_le(hdr + 22, height, 4);
    put_le(hdr + 26, 1, 2);
    put_le(hdr + 28, 24, 2);
    put_le(hdr + 34, height * row_bytes, 4);
    bool ok = fwrite(hdr, 1, 54, fp) == 54;
    for (int64_t i = (int64_t)height - 1; ok && i >= 0; i--) ok = fwrite(bgr + (size_t)i * row_bytes, 1, row_bytes, fp) == row_bytes;
    ok = (fclose(fp) == 0) && ok;
    return ok ? H264R_OK : H264R_ERR_IO;
}

extern "C" int h264r_write_yuv(const char *path, const uint8_t *y, const uint8_t *cb, const uint8_t *cr, uint32_t width, uint32_t height)
{
    if (!path || !y || !cb || !cr || !width || !height) return H264R_ERR_INVALID_ARG;
    FILE *fp = fopen(path, "wb");
    if (!fp) return H264R_ERR_IO;
    const size_t ny = (size_t)width * height, nc = ny / 4;
    bool ok = fwrite(y, 1, ny, fp) == ny && fwrite(cb, 1, nc, fp) == nc && fwrite(cr, 1, nc, fp) == nc;
    ok = (fclose(fp) == 0) && ok;
    return ok ? H264R_OK : H264R_ERR_IO;
}

extern "C" int h264r_load_slot(h264r_stream *s, int slot, const uint8_t *y, const uint8_t *cb, const uint8_t *cr)
{
    if (!s || slot < 0 || slot >= s->cfg.dpb_slots || !y || !cb || !cr) return H264R_ERR_INVALID_ARG;
    h264r_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const uint64_t W = s->cfg.width_mbs * 16ull, H = s->cfg.height_mbs * 16ull;
    uint8_t *base = s->dpb + (uint64_t)slot * s->slot_bytes;
    wait_slot_copy(s, slot, s->cs);
    CUDA_OR(ctx, cudaMemcpyAsync(base, y, W * H, cudaMemcpyHostToDevice, s->cs));
    CUDA_OR(ctx, cudaMemcpyAsync(base + W * H, cb, W * H / 4, cudaMemcpyHostToDevice, s->cs));
    CUDA_OR(ctx, cudaMemcpyAsync(base + W * H + W * H / 4, cr, W * H / 4, cudaMemcpyHostToDevice, s->cs));
    // pageable sources: the copy may still read them after return
    CUDA_OR(ctx, cudaStreamSynchronize(s->cs));
    return H264R_OK;
}

static int check_device_error(h264r_ctx *ctx, cudaStream_t cs)
{
    CUDA_OR(ctx, cudaMemcpyAsync(ctx->h_error, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost, cs));
    CUDA_OR(ctx, cudaStreamSynchronize(cs));
    int e = *ctx->h_error;
    if (e != 0) {
        set_err(ctx, "device reported error %d (%s)", e, e == H264R_ERR_DEVICE_TIMEOUT ? "bounded wait expired" : "bad record");
        cudaMemsetAsync(ctx->d_error, 0, sizeof(int), cs);
        cudaStreamSynchronize(cs);
        return e;
    }
    return H264R_OK;
}

extern "C" int h264r_stream_sync(h264r_stream *s)
{
    if (!s) return H264R_ERR_INVALID_ARG;
    cudaSetDevice(s->ctx->device);
    CUDA_OR(s->ctx, cudaStreamSynchronize(s->cs));
    CUDA_OR(s->ctx, cudaStreamSynchronize(s->out));
    return check_device_error(s->ctx, s->cs);
}

extern "C" int h264r_ctx_sync(h264r_ctx *ctx)
{
    if (!ctx) return H264R_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    CUDA_OR(ctx, cudaDeviceSynchronize());
    return check_device_error(ctx, ctx->batch_stream);
}

// ---------------------------------------------------------------- host batch
extern "C" int h264r_submit_batch(h264r_ctx *ctx, int n, h264r_stream *const *streams, const h264r_picture *pics)
{
    if (!ctx || n <= 0 || !streams || !pics) return H264R_ERR_INVALID_ARG;
    if ((uint32_t)n > ctx->max_batch) {
        set_err(ctx, "h264r_submit_batch: %d pictures exceed the batch limit %u", n, ctx->max_batch);
        return H264R_ERR_BUSY;
    }
    for (int i = 0; i < n; i++)
        if (!streams[i] || streams[i]->ctx != ctx || !pics[i].mbs) return H264R_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    LaunchBuf &b = ctx->batch_ring[ctx->batch_next];
    ctx->batch_next = (ctx->batch_next + 1) % kBatchRing;
    const auto t0 = std::chrono::steady_clock::now();
    int rc = wait_slot(ctx, b);
    if (rc) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    ctx->host_s[0] += std::chrono::duration<double>(t1 - t0).count();
    // layout of the packed records of every picture, then one host -> device copy
    std::vector<std::array<uint64_t, 7>> offs(n);
    uint64_t tot = 0;
    for (int i = 0; i < n; i++) {
        const h264r_picture *pic = &pics[i];
        uint64_t sz[7] = {sizeof(h264r_mb) * pic->num_mbs, sizeof(h264r_slice) * pic->num_slices,
                          sizeof(h264r_weight) * pic->num_weights, pic->motion_bytes, pic->coef_bytes,
                          384ull * pic->num_pcm, 480};
        for (int k = 0; k < 7; k++) {
            offs[i][k] = tot;
            tot = align_up(tot + sz[k], kAlign);
        }
    }
    rc = ensure(ctx, &b.rec_host, &b.rec_host_cap, tot, true);
    if (rc) return rc;
    rc = ensure(ctx, &b.rec_dev, &b.rec_dev_cap, tot, false);
    if (rc) return rc;
    // validate and pack the pictures on the host workers: the picture-level
    // checks here, then every picture in K chunks of MBs and of each record
    // array, so that all workers stay busy whatever the batch size
    std::vector<h264r_picture> dp(pics, pics + n);
    std::vector<BatchItem> items(n);
    for (int i = 0; i < n; i++) {
        const h264r_picture *pic = &pics[i];
        int r = validate_header(pic, streams[i]->cfg.dpb_slots);
        if (r == H264R_OK && (pic->width_mbs != streams[i]->cfg.width_mbs || pic->height_mbs != streams[i]->cfg.height_mbs))
            r = H264R_ERR_INVALID_ARG;
        if (r) {
            set_err(ctx, "h264r_submit_batch: picture %d rejected (%d)", i, r);
            return r;
        }
    }
    const int workers = ctx->pool->size() + 1;
    int K = 1;
    while (K < 8 && n * K < 2 * workers) K *= 2;
    std::vector<int> prc((size_t)n * K, H264R_OK);
    std::vector<uint8_t> pintra((size_t)n * K, 0);
    ctx->pool->run(n * K, [&](int t) {
        const int i = t / K, c = t % K;
        const h264r_picture *pic = &pics[i];
        const uint32_t a0 = (uint32_t)((uint64_t)pic->num_mbs * c / K), a1 = (uint32_t)((uint64_t)pic->num_mbs * (c + 1) / K);
        const int r = validate_mbs(pic, streams[i]->cfg.dpb_slots, a0, a1);
        prc[t] = r;
        if (r) return;
        for (uint32_t a = a0; a < a1; a++) {
            const int ty = pic->mbs[a].type;
            if (ty == H264R_MB_I4x4 || ty == H264R_MB_I8x8 || ty == H264R_MB_I16x16) {
                pintra[t] = 1;
                break;
            }
        }
        const uint8_t *src[6] = {(const uint8_t *)pic->mbs, (const uint8_t *)pic->slices, (const uint8_t *)pic->weights,
                                 pic->motion, pic->coef, pic->pcm};
        const uint64_t sz[6] = {sizeof(h264r_mb) * pic->num_mbs, sizeof(h264r_slice) * pic->num_slices,
                                sizeof(h264r_weight) * pic->num_weights, pic->motion_bytes, pic->coef_bytes, 384ull * pic->num_pcm};
        for (int k = 0; k < 6; k++) {
            const uint64_t b0 = sz[k] * c / K, b1 = sz[k] * (c + 1) / K;
            if (b1 > b0) memcpy(b.rec_host + offs[i][k] + b0, src[k] + b0, b1 - b0);
        }
        if (c == 0) {
            memcpy(b.rec_host + offs[i][6], pic->scaling4x4, 96);
            memcpy(b.rec_host + offs[i][6] + 96, pic->scaling8x8, 384);
            dp[i].mbs = (const h264r_mb *)(b.rec_dev + offs[i][0]);
            dp[i].slices = (const h264r_slice *)(b.rec_dev + offs[i][1]);
            dp[i].weights = (const h264r_weight *)(b.rec_dev + offs[i][2]);
            dp[i].motion = b.rec_dev + offs[i][3];
            dp[i].coef = b.rec_dev + offs[i][4];
            dp[i].pcm = b.rec_dev + offs[i][5];
            items[i].s = streams[i];
            items[i].pic = &dp[i];
            items[i].scaling_dev = b.rec_dev + offs[i][6];
        }
    });
    bool any_intra = false;
    for (int t = 0; t < n * K; t++) {
        if (prc[t]) {
            set_err(ctx, "h264r_submit_batch: picture %d rejected (%d)", t / K, prc[t]);
            return prc[t];
        }
        any_intra = any_intra || pintra[t];
    }
    for (int i = 0; i < n; i++) {
        items[i].has_intra = false;
        for (int c = 0; c < K; c++) items[i].has_intra = items[i].has_intra || pintra[(size_t)i * K + c];
    }
    const auto t2 = std::chrono::steady_clock::now();
    ctx->host_s[1] += std::chrono::duration<double>(t2 - t1).count();
    cudaStream_t cs = streams[0]->cs;
    cudaEvent_t ev;
    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (int i = 1; i < n; i++) {
        if (streams[i]->cs == cs) continue;
        cudaEventRecord(ev, streams[i]->cs);
        cudaStreamWaitEvent(cs, ev, 0);
    }
    rc = H264R_OK;
    // the upload runs on the upload stream: it overlaps the kernels queued on
    // cs before this batch; the batch's kernels wait for it (the staging and
    // device buffers of this ring slot were released by wait_slot)
    if (cudaMemcpyAsync(b.rec_dev, b.rec_host, tot, cudaMemcpyHostToDevice, ctx->upload_stream) != cudaSuccess ||
        cudaEventRecord(b.uploaded, ctx->upload_stream) != cudaSuccess || cudaStreamWaitEvent(cs, b.uploaded, 0) != cudaSuccess) {
        set_err(ctx, "h264r_submit_batch: record upload failed");
        rc = H264R_ERR_CUDA;
    }
    b.wait_upload = true;  // an early k_bs on the side stream waits for it too
    if (rc == H264R_OK) rc = launch(ctx, cs, b, items, any_intra, true);
    if (rc == H264R_OK) {
        cudaEventRecord(ev, cs);
        for (int i = 1; i < n; i++)
            if (streams[i]->cs != cs) cudaStreamWaitEvent(streams[i]->cs, ev, 0);
    }
    ctx->host_s[2] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t2).count();
    cudaEventDestroy(ev);
    return rc;
}

// ---------------------------------------------------------------- accounting
extern "C" int h264r_picture_bytes(const h264r_picture *pic, uint64_t out[4])
{
    if (!pic || !out || !pic->mbs) return H264R_ERR_INVALID_ARG;
    uint64_t k1 = 0, k2 = 0, k3 = 0, rec = 0;
    rec = sizeof(h264r_mb) * (uint64_t)pic->num_mbs + pic->motion_bytes + pic->coef_bytes + 384ull * pic->num_pcm +
          sizeof(h264r_slice) * pic->num_slices + sizeof(h264r_weight) * pic->num_weights;
    auto coef_len = [&](const h264r_mb &m) -> uint64_t {
        if (m.coef == H264R_NONE || (uint64_t)m.coef + 4 > pic->coef_bytes) return 0;
        uint32_t mask;
        memcpy(&mask, pic->coef + m.coef, 4);
        int t8 = (m.flags & H264R_MBF_T8x8) != 0;
        uint64_t nw = __builtin_popcount(mask) + (t8 ? 3 * __builtin_popcount(mask & 15u) : 0);
        uint64_t nl = 0;
        for (uint64_t w = 0; w < nw && m.coef + 4 + 2 * w + 2 <= pic->coef_bytes; w++) {
            uint16_t s;
            memcpy(&s, pic->coef + m.coef + 4 + 2 * w, 2);
            nl += __builtin_popcount(s);
        }
        return ((4 + 2 * nw + 3) & ~3ull) + 2 * nl;
    };
    for (uint32_t a = 0; a < pic->num_mbs; a++) {
        const h264r_mb &m = pic->mbs[a];
        uint64_t own = sizeof(h264r_mb) + coef_len(m);
        if (m.type == H264R_MB_INTER && m.aux != H264R_NONE && (uint64_t)m.aux + 4 <= pic->motion_bytes) {
            uint16_t hdr[2];
            memcpy(hdr, pic->motion + m.aux, 4);
            own += 4 + 16ull * hdr[1];
            int mp = hdr[0] & 3;
            for (int e = 0; e < hdr[1] && (uint64_t)m.aux + 4 + 16ull * (e + 1) <= pic->motion_bytes; e++) {
                h264r_part p;
                memcpy(&p, pic->motion + m.aux + 4 + 16 * e, 16);
                int w = 16, h = 16;
                if (mp == 1) h = 8;
                else if (mp == 2) w = 8;
                else if (mp == 3) {
                    // quadrant of entry e
                    int base = 0, q = 0, sc = 0;
                    for (q = 0; q < 4; q++) {
                        sc = (hdr[0] >> (2 + 2 * q)) & 3;
                        int cnt = (sc == 0) ? 1 : (sc == 3 ? 4 : 2);
                        if (e < base + cnt) break;
                        base += cnt;
                    }
                    w = (sc == 0 || sc == 1) ? 8 : 4;
                    h = (sc == 0 || sc == 2) ? 8 : 4;
                }
                for (int l = 0; l < 2; l++) {
                    if (p.ref[l] < 0) continue;
                    int fx = p.mv[l][0] & 3, fy = p.mv[l][1] & 3, cx = p.mv[l][0] & 7, cy = p.mv[l][1] & 7;
                    own += (uint64_t)(w + (fx ? 5 : 0)) * (h + (fy ? 5 : 0));
                    own += 2ull * (w / 2 + (cx ? 1 : 0)) * (h / 2 + (cy ? 1 : 0));
                }
            }
            k1 += own + 384;
        } else if (m.type == H264R_MB_IPCM) {
            k1 += own + 384 + 384;
        } else if (m.type == H264R_MB_NONE) {
            k1 += own + 384;
        } else {
            k2 += own + 384;
        }
        if (pic->deblock) k3 += 768 + sizeof(h264r_mb);
    }
    out[0] = k1;
    out[1] = k2;
    out[2] = k3;
    out[3] = rec;
    return H264R_OK;
}
