// h264r_decoder.cu — whole-stream decoder (include/h264r_decoder.h): the
// host front end's pictures reconstructed by the engine on one CUDA stream,
// due pictures copied to pinned host planes (h264r_output_async, beside the
// stream's later pictures) and handed to the callback in output order once
// their copy is done, so that parsing goes on while the GPU works.  Host
// code only.
#include "../../include/h264r_decoder.h"

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <vector>

#include "../../include/h264r_parser.h"

struct h264r_decoder {
    h264r_ctx *ctx = nullptr;
    h264r_parser *parser = nullptr;
    h264r_stream *stream = nullptr;
    h264r_frame_callback cb = nullptr;
    void *user = nullptr;
    std::string err;
    uint32_t decoded = 0, output = 0;
    bool stopped = false, flushed = false;
    int width_mbs = 0, height_mbs = 0;
    size_t plane_bytes = 0;
    std::vector<uint8_t *> pinned;  // one coded-size picture each
    std::vector<uint8_t *> free_bufs;
    std::vector<cudaEvent_t> events, free_events;
    std::vector<uint8_t> slice_types;  // per decoding-order index
    // output pictures whose copy is queued, in output order
    struct Pending {
        uint8_t *buf;
        cudaEvent_t ev;
        int32_t poc;
        uint32_t decode_index;
        int slot;
    };
    std::deque<Pending> pend;
    static constexpr size_t kMaxPending = 8;  // copies in flight before the parser waits

    int fail(int code, const char *fmt, ...)
    {
        char m[320];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(m, sizeof(m), fmt, ap);
        va_end(ap);
        err = m;
        return code;
    }

    ~h264r_decoder()
    {
        if (stream) h264r_stream_sync(stream);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        for (uint8_t *p : pinned) cudaFreeHost(p);
        if (stream) h264r_stream_close(stream);
        if (parser) h264r_parser_destroy(parser);
    }

    int open_stream(const h264r_parsed &pp)
    {
        int w = 0, h = 0, slots = 0;
        h264r_parser_geometry(parser, &w, &h, &slots);
        h264r_stream_cfg cfg;
        memset(&cfg, 0, sizeof(cfg));
        cfg.width_mbs = pp.pic.width_mbs;
        cfg.height_mbs = pp.pic.height_mbs;
        cfg.dpb_slots = (uint16_t)slots;
        const int rc = h264r_stream_open(ctx, &cfg, &stream);
        if (rc) return fail(rc, "stream open: %s", h264r_last_error(ctx));
        width_mbs = cfg.width_mbs;
        height_mbs = cfg.height_mbs;
        plane_bytes = (size_t)width_mbs * height_mbs * 384;
        return H264R_OK;
    }

    // a free pinned picture buffer and copy-done event
    int take_buffer(uint8_t **buf, cudaEvent_t *ev)
    {
        if (free_bufs.empty()) {
            void *p = nullptr;
            if (cudaHostAlloc(&p, plane_bytes, cudaHostAllocDefault) != cudaSuccess)
                return fail(H264R_ERR_NO_MEMORY, "pinned output buffer");
            pinned.push_back((uint8_t *)p);
            free_bufs.push_back((uint8_t *)p);
        }
        if (free_events.empty()) {
            cudaEvent_t e;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(H264R_ERR_CUDA, "event");
            events.push_back(e);
            free_events.push_back(e);
        }
        *buf = free_bufs.back();
        free_bufs.pop_back();
        *ev = free_events.back();
        free_events.pop_back();
        return H264R_OK;
    }

    // hand out the queued pictures whose copy is done (all of them, waiting,
    // when wait_all), in output order
    int deliver(bool wait_all)
    {
        const size_t ysz = (size_t)width_mbs * height_mbs * 256, csz = ysz / 4;
        while (!pend.empty()) {
            Pending f = pend.front();
            const cudaError_t e = wait_all ? cudaEventSynchronize(f.ev) : cudaEventQuery(f.ev);
            if (e == cudaErrorNotReady) return H264R_OK;
            if (e != cudaSuccess) return fail(H264R_ERR_CUDA, "output copy: %s", cudaGetErrorString(e));
            pend.pop_front();
            if (cb && !stopped) {
                h264r_frame fr;
                memset(&fr, 0, sizeof(fr));
                fr.y = f.buf;
                fr.cb = f.buf + ysz;
                fr.cr = f.buf + ysz + csz;
                fr.width = width_mbs * 16;
                fr.height = height_mbs * 16;
                fr.poc = f.poc;
                fr.output_count = (int32_t)output;
                fr.decode_index = f.decode_index;
                fr.slice_type = f.decode_index < slice_types.size() ? slice_types[f.decode_index] : 0;
                fr.slot = f.slot;
                fr.stream = stream;
                output++;
                if (cb(&fr, user, 0) != 0) stopped = true;
            } else if (!stopped) {
                output++;
            }
            free_bufs.push_back(f.buf);
            free_events.push_back(f.ev);
        }
        return H264R_OK;
    }

    // reconstruct every picture the parser completed, queue the copies of the
    // due ones and hand out those whose copy is done
    int pump()
    {
        h264r_parsed pp;
        for (;;) {
            int rc = h264r_parser_next(parser, &pp);
            if (rc < 0) return fail(rc, "%s", h264r_parser_last_error(parser));
            if (rc == 0) return deliver(false);
            if (!stream && (rc = open_stream(pp))) return rc;
            if (pp.pic.width_mbs != width_mbs || pp.pic.height_mbs != height_mbs)
                return fail(H264R_ERR_UNSUPPORTED, "picture size change within the stream");
            // a picture handed to the callback keeps its slot until then
            // (h264r_frame.slot, the compat layer's GPU conversions): one that
            // is about to be overwritten is delivered first
            for (size_t k = 0; k < pend.size(); k++) {
                if (pend[k].slot != (int)pp.pic.dst_slot) continue;
                if (cudaEventSynchronize(pend[k].ev) != cudaSuccess) return fail(H264R_ERR_CUDA, "output copy");
                if ((rc = deliver(false))) return rc;
                break;
            }
            if ((rc = h264r_submit_picture(stream, &pp.pic))) return fail(rc, "submit: %s", h264r_last_error(ctx));
            decoded++;
            slice_types.push_back(pp.slice_type);
            if (stopped) continue;
            const size_t ysz = (size_t)width_mbs * height_mbs * 256, csz = ysz / 4;
            cudaStream_t out = (cudaStream_t)h264r_stream_output_cuda_stream(stream);
            for (uint32_t i = 0; i < pp.num_output; i++) {
                Pending f;
                if ((rc = take_buffer(&f.buf, &f.ev))) return rc;
                if ((rc = h264r_output_async(stream, pp.output_slots[i], f.buf, f.buf + ysz, f.buf + ysz + csz)))
                    return fail(rc, "output: %s", h264r_last_error(ctx));
                if (cudaEventRecord(f.ev, out) != cudaSuccess) return fail(H264R_ERR_CUDA, "event record");
                f.poc = pp.output_poc[i];
                f.decode_index = pp.output_index[i];
                f.slot = pp.output_slots[i];
                pend.push_back(f);
            }
            if ((rc = deliver(false))) return rc;
            while (pend.size() > kMaxPending) {
                // bound the copies in flight: wait for the oldest
                if (cudaEventSynchronize(pend.front().ev) != cudaSuccess) return fail(H264R_ERR_CUDA, "output copy");
                if ((rc = deliver(false))) return rc;
            }
        }
    }

    // everything submitted done: device errors, then the remaining pictures
    int drain()
    {
        if (!stream) return H264R_OK;
        const int rc = h264r_stream_sync(stream);
        if (rc) return fail(rc, "%s", h264r_last_error(ctx));
        return deliver(true);
    }
};

extern "C" int h264r_decoder_create(h264r_ctx *ctx, h264r_decoder **out)
{
    if (!ctx || !out) return H264R_ERR_INVALID_ARG;
    h264r_decoder *d = new (std::nothrow) h264r_decoder();
    if (!d) return H264R_ERR_NO_MEMORY;
    d->ctx = ctx;
    const int rc = h264r_parser_create(&d->parser);
    if (rc) {
        delete d;
        return rc;
    }
    *out = d;
    return H264R_OK;
}

extern "C" int h264r_decoder_destroy(h264r_decoder *d)
{
    if (!d) return H264R_ERR_INVALID_ARG;
    delete d;
    return H264R_OK;
}

extern "C" const char *h264r_decoder_last_error(const h264r_decoder *d) { return d ? d->err.c_str() : "null decoder"; }

extern "C" int h264r_decoder_set_callback(h264r_decoder *d, h264r_frame_callback cb, void *user)
{
    if (!d) return H264R_ERR_INVALID_ARG;
    d->cb = cb;
    d->user = user;
    return H264R_OK;
}

extern "C" int h264r_decoder_push(h264r_decoder *d, const uint8_t *data, size_t size)
{
    if (!d || (!data && size)) return H264R_ERR_INVALID_ARG;
    if (d->flushed) return d->fail(H264R_ERR_INVALID_ARG, "push after flush");
    if (d->stopped) return H264R_OK;
    const int rc = h264r_parser_feed(d->parser, data, size);
    if (rc) return d->fail(rc, "%s", h264r_parser_last_error(d->parser));
    return d->pump();
}

extern "C" int h264r_decoder_flush(h264r_decoder *d)
{
    if (!d) return H264R_ERR_INVALID_ARG;
    if (d->flushed) return H264R_OK;
    d->flushed = true;
    int rc = H264R_OK;
    if (!d->stopped) {
        rc = h264r_parser_end(d->parser);
        if (rc) rc = d->fail(rc, "%s", h264r_parser_last_error(d->parser));
        else rc = d->pump();
    }
    const int drc = d->drain();
    if (!rc) rc = drc;
    // the final call comes whether or not the decode stopped early
    const int last = d->cb ? d->cb(nullptr, d->user, H264R_DECODE_FILE_END) : 0;
    return rc ? rc : last;
}

extern "C" int h264r_decoder_open(h264r_decoder *d, const char *path)
{
    if (!d || !path) return H264R_ERR_INVALID_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) {
        if (d->cb) d->cb(nullptr, d->user, H264R_DECODE_OPEN_FILE_FAILED);
        return d->fail(H264R_ERR_IO, "cannot open %s", path);
    }
    std::vector<uint8_t> chunk(1 << 20);
    int rc = H264R_OK;
    for (;;) {
        const size_t n = fread(chunk.data(), 1, chunk.size(), f);
        if (n == 0) break;
        rc = h264r_decoder_push(d, chunk.data(), n);
        if (rc || d->stopped) break;
    }
    fclose(f);
    const int frc = h264r_decoder_flush(d);
    return rc ? rc : frc;
}

extern "C" uint32_t h264r_decoder_decoded(const h264r_decoder *d) { return d ? d->decoded : 0; }
extern "C" uint32_t h264r_decoder_output(const h264r_decoder *d) { return d ? d->output : 0; }
