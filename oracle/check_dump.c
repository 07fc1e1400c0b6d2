/*
 * check_dump.c — pins the oracle to the reference decoder (test
 * infrastructure).  Replays a dump written by ref_dump (records plus the
 * reference's own pre-/post-deblocking planes) through h264o_reconstruct and
 * reports the first differing sample of every picture.
 *
 * usage: check_dump <file.dmp> [--chain] [--quiet]
 *   default: after each picture the reference's planes are loaded into the
 *            DPB slot, so every picture is checked in isolation;
 *   --chain: the oracle's own output stays in the DPB (end-to-end).
 * Exit status 0 when every checked plane matches byte for byte.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "h264r_oracle.h"
#include "dumpfmt.h"

#define MAX_SLOTS 32

static int read_all(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

static void report(const char *what, int pic, const uint8_t *a, const uint8_t *b, int W, int H, int *shown)
{
    size_t ny = (size_t)W * H, nc = ny / 4;
    size_t diff = 0, first = (size_t)-1;
    for (size_t i = 0; i < ny + 2 * nc; i++)
        if (a[i] != b[i]) { if (first == (size_t)-1) first = i; diff++; }
    if (!diff) return;
    const char *plane = "Y";
    size_t off = first;
    int w = W;
    if (off >= ny) { off -= ny; plane = "Cb"; w = W / 2; if (off >= nc) { off -= nc; plane = "Cr"; } }
    int x = (int)(off % (size_t)w), y = (int)(off / (size_t)w);
    int mbx = (plane[0] == 'Y') ? x / 16 : x / 8, mby = (plane[0] == 'Y') ? y / 16 : y / 8;
    if (*shown < 40)
        printf("pic %d %s: %zu samples differ; first %s(%d,%d) mb(%d,%d) oracle=%d ref=%d\n", pic, what, diff, plane, x, y,
               mbx, mby, a[first], b[first]);
    (*shown)++;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <file.dmp> [--chain] [--quiet]\n", argv[0]);
        return 2;
    }
    int chain = 0, quiet = 0;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--chain")) chain = 1;
        if (!strcmp(argv[i], "--quiet")) quiet = 1;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) { perror("fopen"); return 2; }
    char magic[8];
    uint32_t ver[2];
    if (!read_all(f, magic, 8) || memcmp(magic, H264R_DUMP_MAGIC, 8) || !read_all(f, ver, 8)) {
        fprintf(stderr, "not a dump file\n");
        return 2;
    }
    uint8_t *dpb[MAX_SLOTS] = {0};
    size_t slot_bytes = 0;
    int pics = 0, bad = 0, shown = 0, unsupported = 0;
    for (;;) {
        h264r_dump_pic h;
        if (fread(&h, 1, sizeof(h), f) != sizeof(h)) break;
        if (h.tag != H264R_DUMP_PIC_TAG) { fprintf(stderr, "corrupt dump\n"); return 2; }
        h264r_picture pic;
        memset(&pic, 0, sizeof(pic));
        pic.width_mbs = h.width_mbs;
        pic.height_mbs = h.height_mbs;
        pic.structure = h.structure;
        pic.mbaff = h.mbaff;
        pic.dst_slot = h.dst_slot;
        pic.deblock = h.deblock;
        pic.num_slices = h.num_slices;
        pic.num_weights = h.num_weights;
        pic.num_mbs = h.num_mbs;
        pic.motion_bytes = h.motion_bytes;
        pic.coef_bytes = h.coef_bytes;
        pic.num_pcm = h.num_pcm;
        memcpy(pic.scaling4x4, h.scaling4x4, sizeof(h.scaling4x4));
        memcpy(pic.scaling8x8, h.scaling8x8, sizeof(h.scaling8x8));
        h264r_mb *mbs = malloc(sizeof(h264r_mb) * h.num_mbs + 1);
        h264r_slice *sl = malloc(sizeof(h264r_slice) * h.num_slices + 1);
        h264r_weight *wt = malloc(sizeof(h264r_weight) * h.num_weights + 1);
        uint8_t *mo = malloc(h.motion_bytes + 1), *co = malloc(h.coef_bytes + 1), *pcm = malloc((size_t)h.num_pcm * 384 + 1);
        uint8_t *pre = malloc(h.plane_bytes + 1), *post = malloc(h.plane_bytes + 1);
        int ok = read_all(f, mbs, sizeof(h264r_mb) * h.num_mbs) && read_all(f, sl, sizeof(h264r_slice) * h.num_slices) &&
                 read_all(f, wt, sizeof(h264r_weight) * h.num_weights) && read_all(f, mo, h.motion_bytes) &&
                 read_all(f, co, h.coef_bytes) && read_all(f, pcm, (size_t)h.num_pcm * 384);
        if (ok && (h.flags & H264R_DUMP_HAS_PRE)) ok = read_all(f, pre, h.plane_bytes);
        if (ok && (h.flags & H264R_DUMP_HAS_POST)) ok = read_all(f, post, h.plane_bytes);
        if (!ok) { fprintf(stderr, "truncated dump\n"); return 2; }
        pic.mbs = mbs; pic.slices = sl; pic.weights = wt; pic.motion = mo; pic.coef = co; pic.pcm = pcm;
        if (!slot_bytes) {
            slot_bytes = h264o_slot_bytes(h.width_mbs, h.height_mbs);
            for (int i = 0; i < MAX_SLOTS; i++) dpb[i] = calloc(1, slot_bytes);
        }
        uint8_t *opre = malloc(h.plane_bytes + 1);
        int rc = h264o_reconstruct(&pic, dpb, MAX_SLOTS, opre);
        int W = h.width_mbs * 16, H = h.height_mbs * 16;
        if (rc == H264R_ERR_UNSUPPORTED) {
            unsupported++;
        } else if (rc) {
            printf("pic %d: oracle error %d\n", pics, rc);
            bad++;
        } else {
            int before = shown;
            if (h.flags & H264R_DUMP_HAS_PRE) report("pre-deblock", pics, opre, pre, W, H, &shown);
            if (h.flags & H264R_DUMP_HAS_POST) report("post-deblock", pics, dpb[h.dst_slot], post, W, H, &shown);
            if (shown != before) bad++;
            else if (!quiet) printf("pic %d (poc %d, slot %d, mbaff %d): bit-exact\n", pics, h.poc, h.dst_slot, h.mbaff);
        }
        if (!chain && (h.flags & H264R_DUMP_HAS_POST)) memcpy(dpb[h.dst_slot], post, h.plane_bytes);
        free(opre); free(mbs); free(sl); free(wt); free(mo); free(co); free(pcm); free(pre); free(post);
        pics++;
    }
    printf("%s: %d pictures, %d mismatching, %d unsupported\n", argv[1], pics, bad, unsupported);
    return bad ? 1 : 0;
}
