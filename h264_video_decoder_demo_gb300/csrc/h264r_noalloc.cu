// h264r_noalloc.cu — deblocking of one picture without allocating device
// memory (h264r_deblock_picture_noalloc in include/h264r.h).
//
// Some callers cannot let a library allocate device memory: a player or
// serving process that hands all of the GPU's memory to its own pool up front
// (a cudaMalloc would exceed the budget it accounts for), and real-time
// decode loops that must not stall other streams (cudaMalloc and cudaFree
// synchronise the device).  For them the deblocking pass runs on scratch that
// is part of the library image itself: one file-scope __device__ array, sized
// for pictures of up to kNoAllocMaxMbs macroblocks, which every GPU that loads
// the library holds until the process exits.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include <mutex>

#include "h264r_device.cuh"

namespace h264r {
__global__ void k_bs(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st);
__global__ void k_deblock(const PicDesc *__restrict__ pics, int npics, uint32_t total_units, LaunchState st);
__global__ void k_deblock_frame(const PicDesc *__restrict__ pics, int npics, uint32_t total_units, LaunchState st);
}  // namespace h264r

using h264r::PicDesc;
using h264r::LaunchState;

namespace {

constexpr uint32_t kNoAllocMaxMbs = H264R_NOALLOC_MAX_MBS;   // 1920x1088 is 8160
constexpr uint32_t kNoAllocMaxRows = H264R_NOALLOC_MAX_MB_ROWS;
constexpr unsigned long long kNoAllocSpinLimit = 1ull << 25;

struct NoAllocScratch {
    PicDesc desc;                             // descriptor the kernels read
    int error;                                // device error word of the call
    unsigned int ticket[3];                   // wavefront tickets
    int progress[3 * kNoAllocMaxRows];        // wavefront progress counters
    alignas(256) uint8_t bs[kNoAllocMaxMbs * h264r::kBsBytes];  // boundary strengths (read with 16-byte loads)
};
static_assert(offsetof(NoAllocScratch, bs) % 256 == 0, "the bS table must start on a 256-byte boundary");

// The scratch: ~2.1 MB per device, shared by every call in the process.
static __device__ __align__(256) NoAllocScratch g_scratch;

// Device address of g_scratch, resolved once per device with that device
// current (the host-side name g_scratch is only a stand-in).
std::mutex g_mu;
NoAllocScratch *g_ptr[64] = {nullptr};

// Clear what must start at zero for this call and publish the descriptor;
// the bS table needs no clearing (k_bs writes every byte the filter reads).
__global__ void k_noalloc_init(PicDesc d, NoAllocScratch *s)
{
    if (threadIdx.x == 0) {
        s->desc = d;
        s->error = 0;
        s->ticket[0] = s->ticket[1] = s->ticket[2] = 0;
    }
    for (uint32_t i = threadIdx.x; i < 3 * kNoAllocMaxRows; i += blockDim.x) s->progress[i] = 0;
}

}  // namespace

extern "C" int h264r_deblock_picture_noalloc(const h264r_picture *pic, uint8_t *planes, void *cuda_stream)
{
    if (!pic || !planes || !pic->mbs || !pic->slices || ((uintptr_t)planes & 15)) return H264R_ERR_INVALID_ARG;
    if (pic->structure != H264R_STRUCT_FRAME) return H264R_ERR_UNSUPPORTED;
    if (pic->width_mbs == 0 || pic->height_mbs == 0 || pic->num_slices == 0 ||
        pic->num_mbs != (uint32_t)pic->width_mbs * pic->height_mbs || (pic->mbaff && (pic->height_mbs & 1)))
        return H264R_ERR_INVALID_ARG;
    const uint32_t rows = pic->mbaff ? pic->height_mbs / 2u : pic->height_mbs;
    if (pic->num_mbs > kNoAllocMaxMbs || rows > kNoAllocMaxRows) return H264R_ERR_TOO_LARGE;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return H264R_ERR_CUDA;
    NoAllocScratch *s = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_ptr[dev]) {
            void *ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) return H264R_ERR_CUDA;
            g_ptr[dev] = (NoAllocScratch *)ptr;
        }
        s = g_ptr[dev];
    }

    PicDesc d;
    memset(&d, 0, sizeof(d));
    d.wmb = pic->width_mbs;
    d.hmb = pic->height_mbs;
    d.W = d.wmb * 16;
    d.H = d.hmb * 16;
    d.Wc = d.W / 2;
    d.Hc = d.H / 2;
    d.ys = d.W;
    d.cs = d.Wc;
    d.fH = d.H;
    d.fpic = 0;
    d.mbaff = pic->mbaff;
    d.deblock = 1;
    d.num_mbs = pic->num_mbs;
    d.num_slices = pic->num_slices;
    d.num_weights = pic->num_weights;
    d.num_pcm = pic->num_pcm;
    d.motion_bytes = pic->motion_bytes;
    d.coef_bytes = pic->coef_bytes;
    d.mbs = pic->mbs;
    d.slices = pic->slices;
    d.weights = pic->weights;
    d.motion = pic->motion;
    d.coef = pic->coef;
    d.pcm = pic->pcm;
    d.flat_scaling = 1;
    d.dst = planes;
    d.coff = d.W * d.H;
    d.cplane = d.Wc * d.Hc;
    d.dpb = planes;
    d.nslots = 1;
    d.bs = s->bs;
    d.progress = s->progress;
    d.units_w = pic->width_mbs;
    d.units_h = rows;
    d.db_base = 0;
    d.db_units = h264r::deblock_units(d.mbaff, rows);
    d.dbf_base = 0;
    d.dbf_units = h264r::deblock_frame_units(d.mbaff, rows);
    d.deblock_stop = 0xFFFFFFFFu;

    cudaStream_t cs = (cudaStream_t)cuda_stream;
    LaunchState st;
    st.error = &s->error;
    st.ticket = s->ticket;
    st.spin_limit = kNoAllocSpinLimit;
    // An error left by the caller's earlier work is reported without being
    // cleared (it is not this call's); once none is pending, an error seen
    // right after a launch belongs to that launch.
    if (cudaPeekAtLastError() != cudaSuccess) return H264R_ERR_CUDA;
    k_noalloc_init<<<1, 256, 0, cs>>>(d, s);
    if (cudaGetLastError() != cudaSuccess) return H264R_ERR_CUDA;
    h264r::k_bs<<<(pic->num_mbs + h264r::kBsMbsPerBlock - 1) / h264r::kBsMbsPerBlock, 128, 0, cs>>>(&s->desc, 1, pic->num_mbs, st);
    if (cudaGetLastError() != cudaSuccess) return H264R_ERR_CUDA;
    if (d.dbf_units) {
        h264r::k_deblock_frame<<<d.dbf_units, 32 * h264r::kDbWarps, 0, cs>>>(&s->desc, 1, d.dbf_units, st);
        if (cudaGetLastError() != cudaSuccess) return H264R_ERR_CUDA;
    }
    if (d.db_units) {
        h264r::k_deblock<<<d.db_units, 32 * h264r::kMbWarps, 0, cs>>>(&s->desc, 1, d.db_units, st);
        if (cudaGetLastError() != cudaSuccess) return H264R_ERR_CUDA;
    }
    int herr = 0;
    if (cudaMemcpyAsync(&herr, &s->error, sizeof(int), cudaMemcpyDeviceToHost, cs) != cudaSuccess) return H264R_ERR_CUDA;
    if (cudaStreamSynchronize(cs) != cudaSuccess) return H264R_ERR_CUDA;
    return herr;
}
