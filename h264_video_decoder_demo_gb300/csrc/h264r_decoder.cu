// h264r_decoder.cu — whole-stream decoder (include/h264r_decoder.h): the
// host front end's pictures reconstructed by the engine on one CUDA stream,
// due pictures copied to pinned host planes and handed to the callback in
// output order.  Host code only.
#include "../../include/h264r_decoder.h"

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
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
    std::vector<uint8_t> slice_types;  // per decoding-order index

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

    int pinned_buffers(size_t n)
    {
        while (pinned.size() < n) {
            void *p = nullptr;
            if (cudaHostAlloc(&p, plane_bytes, cudaHostAllocDefault) != cudaSuccess)
                return fail(H264R_ERR_NO_MEMORY, "pinned output buffer");
            pinned.push_back((uint8_t *)p);
        }
        return H264R_OK;
    }

    // reconstruct every picture the parser completed, hand out the due ones
    int pump()
    {
        h264r_parsed pp;
        for (;;) {
            int rc = h264r_parser_next(parser, &pp);
            if (rc < 0) return fail(rc, "%s", h264r_parser_last_error(parser));
            if (rc == 0) return H264R_OK;
            if (!stream && (rc = open_stream(pp))) return rc;
            if (pp.pic.width_mbs != width_mbs || pp.pic.height_mbs != height_mbs)
                return fail(H264R_ERR_UNSUPPORTED, "picture size change within the stream");
            if ((rc = h264r_submit_picture(stream, &pp.pic))) return fail(rc, "submit: %s", h264r_last_error(ctx));
            decoded++;
            slice_types.push_back(pp.slice_type);
            if (pp.num_output == 0 || stopped) continue;
            if ((rc = pinned_buffers(pp.num_output))) return rc;
            const size_t ysz = (size_t)width_mbs * height_mbs * 256, csz = ysz / 4;
            for (uint32_t i = 0; i < pp.num_output; i++) {
                uint8_t *b = pinned[i];
                if ((rc = h264r_output(stream, pp.output_slots[i], b, b + ysz, b + ysz + csz)))
                    return fail(rc, "output: %s", h264r_last_error(ctx));
            }
            if ((rc = h264r_stream_sync(stream))) return fail(rc, "%s", h264r_last_error(ctx));
            for (uint32_t i = 0; i < pp.num_output && !stopped; i++) {
                h264r_frame f;
                memset(&f, 0, sizeof(f));
                f.y = pinned[i];
                f.cb = pinned[i] + ysz;
                f.cr = pinned[i] + ysz + csz;
                f.width = width_mbs * 16;
                f.height = height_mbs * 16;
                f.poc = pp.output_poc[i];
                f.output_count = (int32_t)output;
                f.decode_index = pp.output_index[i];
                f.slice_type = pp.output_index[i] < slice_types.size() ? slice_types[pp.output_index[i]] : 0;
                f.slot = pp.output_slots[i];
                f.stream = stream;
                output++;
                if (cb && cb(&f, user, 0) != 0) stopped = true;
            }
        }
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
