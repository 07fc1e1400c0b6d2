// h264r_order.cpp — output order of decoded pictures (include/h264r_order.h).
#include "../../include/h264r_order.h"

#include <new>
#include <vector>

#include "../../include/h264r.h"

struct h264r_order {
    int depth = 0;
    struct Held {
        uint64_t tag;
        int32_t poc;
    };
    std::vector<Held> held;  // decoding order among the held pictures
};

namespace {

// index of the held picture with the lowest POC (the first one on ties, as
// the reference's scan keeps the earliest minimum)
int lowest(const h264r_order *q)
{
    int idx = -1;
    for (int i = 0; i < (int)q->held.size(); i++)
        if (idx < 0 || q->held[i].poc < q->held[idx].poc) idx = i;
    return idx;
}

int drain(h264r_order *q, uint64_t *out, int cap, int n)
{
    while (!q->held.empty()) {
        if (n >= cap) return H264R_ERR_INVALID_ARG;
        const int i = lowest(q);
        out[n++] = q->held[i].tag;
        q->held.erase(q->held.begin() + i);
    }
    return n;
}

}  // namespace

extern "C" int h264r_order_create(int max_num_reorder_frames, h264r_order **out)
{
    if (!out || max_num_reorder_frames < 0 || max_num_reorder_frames > 16) return H264R_ERR_INVALID_ARG;
    h264r_order *q = new (std::nothrow) h264r_order();
    if (!q) return H264R_ERR_NO_MEMORY;
    q->depth = max_num_reorder_frames;
    q->held.reserve(17);
    *out = q;
    return H264R_OK;
}

extern "C" int h264r_order_destroy(h264r_order *q)
{
    if (!q) return H264R_ERR_INVALID_ARG;
    delete q;
    return H264R_OK;
}

extern "C" int h264r_order_push(h264r_order *q, uint64_t tag, int32_t poc, int idr, uint64_t *out, int cap)
{
    if (!q || !out || cap < 1) return H264R_ERR_INVALID_ARG;
    int n = 0;
    if (idr) {  // do_callback's flush before the IDR picture itself
        n = drain(q, out, cap, 0);
        if (n < 0) return n;
    }
    if (q->depth == 0) {
        if (n >= cap) return H264R_ERR_INVALID_ARG;
        out[n++] = tag;
        return n;
    }
    if ((int)q->held.size() < q->depth) {
        q->held.push_back({tag, poc});
        return n;
    }
    const int i = lowest(q);
    if (n >= cap) return H264R_ERR_INVALID_ARG;
    if (poc < q->held[i].poc) {
        out[n++] = tag;
    } else {
        out[n++] = q->held[i].tag;
        q->held[i] = {tag, poc};
    }
    return n;
}

extern "C" int h264r_order_flush(h264r_order *q, uint64_t *out, int cap)
{
    if (!q || (!out && !q->held.empty())) return H264R_ERR_INVALID_ARG;
    return drain(q, out, cap, 0);
}

extern "C" int h264r_order_holds(const h264r_order *q, uint64_t tag)
{
    if (!q) return H264R_ERR_INVALID_ARG;
    for (const auto &h : q->held)
        if (h.tag == tag) return 1;
    return 0;
}

extern "C" int h264r_order_infer_depth(int profile_idc, int constraint_set3_flag, int level_idc, int width_mbs, int frame_height_mbs)
{
    // Table A-1: level_idc -> MaxDpbMbs, as the reference lists it
    static const int kMaxDpbMbs[][2] = {{10, 396},    {11, 900},    {12, 2376},   {13, 2376},   {20, 2376},
                                        {21, 4752},   {22, 8100},   {30, 8100},   {31, 18000},  {32, 20480},
                                        {40, 32768},  {41, 32768},  {42, 34816},  {50, 110400}, {51, 184320},
                                        {52, 184320}, {60, 696320}, {61, 696320}, {62, 696320}};
    if (width_mbs <= 0 || frame_height_mbs <= 0) return H264R_ERR_INVALID_ARG;
    const bool intra_profile = profile_idc == 44 || profile_idc == 86 || profile_idc == 100 || profile_idc == 110 ||
                               profile_idc == 122 || profile_idc == 244;
    if (intra_profile && constraint_set3_flag) return 0;
    for (const auto &e : kMaxDpbMbs)
        if (e[0] == level_idc) {
            const int f = e[1] / (width_mbs * frame_height_mbs);
            return f < 16 ? f : 16;
        }
    return 0;  // a level the table does not list: the reference leaves MaxDpbFrames at 0
}
