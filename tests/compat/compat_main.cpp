// compat_main.cpp — a program written against the reference decoder's
// public C++ interface (CH264VideoDecoder, CH264Picture; the pattern of its
// main.cpp): decodes a stream and writes one BMP per output picture,
// out_<W>x<H>.<n>.bmp with n counting output pictures.  Built against
// include/compat and libh264r.so by tests/test_gpu_decoder.py.
#include <stdio.h>

#include "H264VideoDecoder.h"

static int on_picture(CH264Picture *pic, void *user, int error_code)
{
    static int count = 0;
    if (!pic) return error_code == H264_DECODE_ERROR_CODE_FILE_END ? 0 : -1;
    char path[1024];
    snprintf(path, sizeof(path), "%s/out_%dx%d.%d.bmp", (const char *)user, pic->m_picture_frame.PicWidthInSamplesL,
             pic->m_picture_frame.PicHeightInSamplesL, count);
    printf("%d %s %d\n", count, H264_SLIECE_TYPE_TO_STR(pic->m_picture_frame.m_h264_slice_header.slice_type),
           pic->m_picture_frame.PicOrderCnt);
    count++;
    return pic->m_picture_frame.saveToBmpFile(path);
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s <in.h264> <out_dir>\n", argv[0]);
        return 2;
    }
    CH264VideoDecoder vd;
    vd.set_output_frame_callback_functuin(on_picture, argv[2]);
    const int ret = vd.open(argv[1]);
    printf("open: %d\n", ret);
    return ret == 0 ? 0 : 1;
}
