/*
 * H264VideoDecoder.h — the reference decoder's public C++ interface
 * (h264_video_decoder_demo/H264VideoDecoder.h:25-42 and the CH264Picture
 * members its callbacks read, main.cpp:14-51) implemented over the GB300
 * engine: a program written against the reference (its main.cpp, its
 * player) compiles unchanged with -I include/compat and links with
 * libh264r.so.  Header only; the work is done by include/h264r_decoder.h.
 *
 * The picture handed to the callback is valid only during the call: its
 * planes are host copies of the engine's DPB slot, and saveToBmpFile /
 * writeYUV produce the reference's BMP and YUV files (the BGR24 conversion
 * runs on the GPU).
 */
#ifndef H264R_COMPAT_H264_VIDEO_DECODER_H
#define H264R_COMPAT_H264_VIDEO_DECODER_H

#include <stdint.h>
#include <stdlib.h>

#include <string>

#include "../h264r.h"
#include "../h264r_decoder.h"

typedef enum _H264_SLIECE_TYPE_ {
    H264_SLIECE_TYPE_P = 0,
    H264_SLIECE_TYPE_B = 1,
    H264_SLIECE_TYPE_I = 2,
    H264_SLIECE_TYPE_SP = 3,
    H264_SLIECE_TYPE_SI = 4,
    H264_SLIECE_TYPE_P2 = 5,
    H264_SLIECE_TYPE_B2 = 6,
    H264_SLIECE_TYPE_I2 = 7,
    H264_SLIECE_TYPE_SP2 = 8,
    H264_SLIECE_TYPE_SI2 = 9,
} H264_SLIECE_TYPE;

#define H264_SLIECE_TYPE_TO_STR(slice_type) h264r_compat_slice_type_str((int)(slice_type))

typedef enum _H264_DECODE_ERROR_CODE_ {
    H264_DECODE_ERROR_CODE_UNKNOWN = H264R_DECODE_UNKNOWN,
    H264_DECODE_ERROR_CODE_FILE_END = H264R_DECODE_FILE_END,
    H264_DECODE_ERROR_CODE_OPEN_FILE_FAILED = H264R_DECODE_OPEN_FILE_FAILED,
    H264_DECODE_ERROR_CODE_NEED_MORE_DATA,
    H264_DECODE_ERROR_CODE_NO_MORE_FRAMES,
} H264_DECODE_ERROR_CODE;

inline const char *h264r_compat_slice_type_str(int t)
{
    static const char *const names[10] = {"P", "B", "I", "SP", "SI", "P2", "B2", "I2", "SP2", "SI2"};
    return (t >= 0 && t < 10) ? names[t] : "UNKNOWN";
}

class CH264SliceHeader {
public:
    int32_t slice_type;
    CH264SliceHeader() : slice_type(0) {}
};

/* The members of the reference's CH264PictureBase that its callers read. */
class CH264PictureBase {
public:
    uint8_t *m_pic_buff_luma, *m_pic_buff_cb, *m_pic_buff_cr;
    int32_t PicWidthInSamplesL, PicHeightInSamplesL, PicWidthInSamplesC, PicHeightInSamplesC;
    int32_t PicOrderCnt;
    int32_t m_PicNumCnt;  /* decoding order, as in the reference */
    CH264SliceHeader m_h264_slice_header;
    h264r_stream *m_stream;
    int32_t m_slot;

    CH264PictureBase()
        : m_pic_buff_luma(0), m_pic_buff_cb(0), m_pic_buff_cr(0), PicWidthInSamplesL(0), PicHeightInSamplesL(0),
          PicWidthInSamplesC(0), PicHeightInSamplesC(0), PicOrderCnt(0), m_PicNumCnt(0), m_stream(0), m_slot(-1)
    {
    }

    /* 24-bit BMP of the picture (CH264PictureBase::saveToBmpFile). */
    int saveToBmpFile(const char *filename)
    {
        const uint32_t w = (uint32_t)PicWidthInSamplesL, h = (uint32_t)PicHeightInSamplesL;
        const uint32_t row = (3 * w + 3) & ~3u;
        uint8_t *bgr = (uint8_t *)malloc((size_t)row * h);
        if (!bgr) return -1;
        int rc = h264r_output_bgr24(m_stream, m_slot, bgr, row, 0);
        if (rc == 0) rc = h264r_stream_sync(m_stream);
        if (rc == 0) rc = h264r_write_bmp(filename, bgr, w, h, row);
        free(bgr);
        return rc == 0 ? 0 : -1;
    }

    /* Planar YUV 4:2:0 file (CH264PictureBase::writeYUV). */
    int writeYUV(const char *filename)
    {
        return h264r_write_yuv(filename, m_pic_buff_luma, m_pic_buff_cb, m_pic_buff_cr, (uint32_t)PicWidthInSamplesL,
                               (uint32_t)PicHeightInSamplesL) == 0 ? 0 : -1;
    }
};

class CH264Picture {
public:
    CH264PictureBase m_picture_frame;
};

typedef int (*output_frame_callback)(CH264Picture *outPicture, void *userData, int errorCode);

class CH264VideoDecoder {
public:
    std::string m_filename;
    output_frame_callback m_output_frame_callback;
    void *m_userData;

    CH264VideoDecoder() : m_output_frame_callback(0), m_userData(0), m_ctx(0) {}
    ~CH264VideoDecoder() { unInit(); }

    /* engine context on GPU 0 (open() creates it when init() was not called) */
    int init()
    {
        if (m_ctx) return 0;
        h264r_cfg cfg;
        cfg.device = 0;
        cfg.dpb_budget_bytes = 0;
        cfg.max_batch_pictures = 0;
        cfg.flags = 0;
        return h264r_ctx_create(&cfg, &m_ctx) == 0 ? 0 : -1;
    }

    int unInit()
    {
        if (m_ctx) h264r_ctx_destroy(m_ctx);
        m_ctx = 0;
        return 0;
    }

    int set_output_frame_callback_functuin(output_frame_callback cb, void *userData)
    {
        m_output_frame_callback = cb;
        m_userData = userData;
        return 0;
    }

    /* Decode the whole file, calling back every picture in output order,
     * then (NULL, userData, H264_DECODE_ERROR_CODE_FILE_END). */
    int open(const char *url)
    {
        if (!url || init() != 0) return -1;
        m_filename = url;
        h264r_decoder *d = 0;
        if (h264r_decoder_create(m_ctx, &d) != 0) return -1;
        h264r_decoder_set_callback(d, &CH264VideoDecoder::on_frame, this);
        const int rc = h264r_decoder_open(d, url);
        h264r_decoder_destroy(d);
        return rc;
    }

private:
    h264r_ctx *m_ctx;

    static int on_frame(const h264r_frame *f, void *user, int error_code)
    {
        CH264VideoDecoder *self = (CH264VideoDecoder *)user;
        if (!self->m_output_frame_callback) return 0;
        if (!f) return self->m_output_frame_callback(0, self->m_userData, error_code);
        CH264Picture pic;
        CH264PictureBase &b = pic.m_picture_frame;
        b.m_pic_buff_luma = (uint8_t *)f->y;
        b.m_pic_buff_cb = (uint8_t *)f->cb;
        b.m_pic_buff_cr = (uint8_t *)f->cr;
        b.PicWidthInSamplesL = f->width;
        b.PicHeightInSamplesL = f->height;
        b.PicWidthInSamplesC = f->width / 2;
        b.PicHeightInSamplesC = f->height / 2;
        b.PicOrderCnt = f->poc;
        b.m_PicNumCnt = (int32_t)f->decode_index;
        b.m_h264_slice_header.slice_type = f->slice_type;
        b.m_stream = f->stream;
        b.m_slot = f->slot;
        return self->m_output_frame_callback(&pic, self->m_userData, error_code);
    }
};

#endif /* H264R_COMPAT_H264_VIDEO_DECODER_H */
