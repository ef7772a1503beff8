// GPU block-size autotuner: the reference's autotune_block_sizes (src/autotune.hh:80-96) times its
// dual-quant on sampled blocks at block sizes 8, 16, 32 and 64 and keeps the fastest.  Here the
// dual-quant kernel itself is timed with CUDA events on a leading slab of the field (a contiguous
// prefix along the slowest axis), at each block size, and the fastest is returned.  (The
// reference's loop times the same configured block size four times; every size is timed here.)
#include <cstdint>

#include "api_common.cuh"
#include "vsz_device.cuh"
#include "vsz_kernels.h"

using namespace vsz;
using namespace vsz::api;

namespace {

// The sample: the leading slab of sample_percent of the slowest axis, at least 64 planes (3D) or
// rows (2D) or 64K elements (1D), at most the field.
Geometry sample_geometry(int ndim, const size_t dims[3], double pct, size_t sdims[3]) {
    sdims[0] = dims[0];
    sdims[1] = ndim > 1 ? dims[1] : 1;
    sdims[2] = ndim > 2 ? dims[2] : 1;
    const size_t last = dims[ndim - 1];
    size_t keep       = (size_t)((pct / 100.0) * (double)last + 0.999);
    const size_t lo   = ndim == 1 ? (size_t)65536 : 64;
    if (keep < lo) keep = lo;
    if (keep > last) keep = last;
    sdims[ndim - 1] = keep;
    return make_geometry(ndim, sdims);
}

struct TuneWs {
    Consts* consts;
    uint32_t* mm;
    int* status;
    unsigned long long* hist;
    uint16_t* code;
    uint8_t* seg_count;
    float* scratch;
    size_t bytes;
};

TuneWs layout_tune(const Geometry& g, int dict, uint8_t* base, size_t cap) {
    Bump b{base, cap};
    TuneWs w{};
    w.consts    = b.take<Consts>(1);
    w.mm        = b.take<uint32_t>(4);
    w.status    = b.take<int>(4);
    w.hist      = b.take<unsigned long long>(dict);
    w.code      = b.take<uint16_t>(g.n + 8);
    w.seg_count = b.take<uint8_t>(g.nseg + 16);
    w.scratch   = b.take<float>(g.nseg * kSegX);
    w.bytes     = b.off + 256;
    return w;
}

}  // namespace

extern "C" {

vsz_status vsz_autotune_workspace_bytes(const vsz_params* p, int ndim, const size_t dims[3], double sample_percent,
                                        size_t* ws_bytes) {
    VSZ_TRY(check_params(p, ndim, dims));
    if (!(sample_percent > 0.0) || sample_percent > 100.0) return VSZ_ERR_INVALID;
    size_t sd[3];
    Geometry g = sample_geometry(ndim, dims, sample_percent, sd);
    if (ws_bytes) *ws_bytes = layout_tune(g, p->dict_size, nullptr, 0).bytes;
    return VSZ_OK;
}

vsz_status vsz_autotune_block_size(const vsz_params* p, int ndim, const size_t dims[3], const float* d_in,
                                   double sample_percent, int iterations, void* d_ws, size_t ws_bytes,
                                   int* best_block_size, double timings_ms[4], void* stream) {
    VSZ_TRY(check_params(p, ndim, dims));
    if (!d_in || !d_ws || !best_block_size || iterations < 1 || !(sample_percent > 0.0) || sample_percent > 100.0)
        return VSZ_ERR_INVALID;
    size_t sd[3];
    Geometry g = sample_geometry(ndim, dims, sample_percent, sd);
    TuneWs w   = layout_tune(g, p->dict_size, reinterpret_cast<uint8_t*>(d_ws), ws_bytes);
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    cudaStream_t st = S(stream);
    VSZ_CUDA(cudaMemsetAsync(w.status, 0, sizeof(int), st));
    VSZ_TRY(launch_eb_setup(p->mode, p->eb, d_in, g.n, w.consts, w.mm, st, w.status));
    Consts c{};
    VSZ_CUDA(cudaMemcpyAsync(&c, w.consts, sizeof(Consts), cudaMemcpyDeviceToHost, st));
    VSZ_CUDA(cudaStreamSynchronize(st));
    if (c.status != VSZ_OK) return c.status;  // e.g. zero value range in r2r
    cudaEvent_t e0, e1;
    VSZ_CUDA(cudaEventCreate(&e0));
    VSZ_CUDA(cudaEventCreate(&e1));
    static const int kSizes[4] = {8, 16, 32, 64};
    int best = kSizes[0], rc = VSZ_OK;
    float best_ms = 3.4e38f;
    for (int k = 0; k < 4 && rc == VSZ_OK; k++) {
        DqArgs a = make_dq_args(g, kSizes[k], p->dict_size, d_in, w.consts, w.code, w.scratch, w.seg_count, w.hist);
        float ms = 0.f;
        for (int it = 0; it <= iterations && rc == VSZ_OK; it++) {  // the first run warms up
            if (it == 1 && cudaEventRecord(e0, st) != cudaSuccess) rc = VSZ_ERR_CUDA;
            if (rc == VSZ_OK && cudaMemsetAsync(w.hist, 0, 8 * (size_t)p->dict_size, st) != cudaSuccess) rc = VSZ_ERR_CUDA;
            if (rc == VSZ_OK) rc = launch_dq_compress(a, ndim, kSizes[k], st, num_sms());
        }
        if (rc == VSZ_OK && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                             cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
            rc = VSZ_ERR_CUDA;
        if (rc != VSZ_OK) break;
        ms /= (float)iterations;
        if (timings_ms) timings_ms[k] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best    = kSizes[k];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VSZ_OK) return rc;
    *best_block_size = best;
    return VSZ_OK;
}

}  // extern "C"
