// GPU block-size autotuner: the reference's autotune_block_sizes (src/autotune.hh:80-96) times its
// dual-quant on sampled blocks at block sizes 8, 16, 32 and 64 and keeps the fastest.  Here the
// dual-quant kernel itself is timed with CUDA events on a leading slab of the field (a contiguous
// prefix along the slowest axis), at each block size, and the fastest is returned.  (The
// reference's loop times the same configured block size four times; every size is timed here.)
#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

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

// ------------------------------------------------------------------------------------------
// Field autotuner.  The block size changes everything downstream of the dual-quant stage -- the
// histogram, the tree, the encoder's and decoder's work and the archive's size -- so each candidate
// (8, 16, 32, 64) is timed through the whole-field entry points, vsz_compress and vsz_decompress,
// on the leading slab, and scored by
//     compress ms + decompress ms + archive bytes / link rate
// (the time to compress a field, move its archive over a link of link_gbs GB/s, and decompress it;
// link_gbs = 0 scores speed alone).  The choice is cached per (dimensionality, size class =
// ceil(log2 elements), eb class = floor(2 log10 eb), mode, dictionary, link rate), so fields of one
// class are tuned once per process.
// ------------------------------------------------------------------------------------------
namespace {

using TuneKey = std::tuple<int, int, int, int, int, long long, int>;
std::mutex g_tune_mu;
std::map<TuneKey, vsz_tune_result> g_tune_cache;

TuneKey tune_key(const vsz_params* p, int ndim, const size_t dims[3], double link_gbs) {
    double n = 1;
    for (int i = 0; i < ndim; i++) n *= (double)dims[i];
    const int nclass  = (int)std::ceil(std::log2(n));
    const int ebclass = (int)std::floor(2.0 * std::log10(p->eb));
    return TuneKey(ndim, nclass, ebclass, p->mode, p->dict_size, (long long)std::llround(link_gbs * 1000.0),
                   p->flags | (p->pad_mode << 4) | (p->pad_type << 8));
}

struct FieldTuneWs {
    uint8_t* cws;      // compress workspace
    size_t cws_bytes;
    uint8_t* archive;  // archive (capacity + 64 readable bytes)
    size_t cap;
    uint8_t* dws;      // decompress workspace
    size_t dws_bytes;
    float* out;
    uint64_t* result;  // 8 u64
    int* status;
    size_t bytes;
};

// Worst-case sizes over the four block sizes: the compress workspace and archive capacity from
// vsz_compress_bounds; the decompress workspace from vsz_decompress_bounds of an archive with the
// largest payload (64 bits per code), every element an outlier and the index.
int layout_field_tune(const vsz_params* p, int ndim, const size_t sd[3], uint8_t* base, size_t cap_bytes,
                      FieldTuneWs& w) {
    static const int kSizes[4] = {8, 16, 32, 64};
    size_t cws = 0, acap = 0, dws = 0;
    const Geometry g = make_geometry(ndim, sd);
    for (int bs : kSizes) {
        vsz_params q   = *p;
        q.block_size   = bs;
        q.lossless     = VSZ_LOSSLESS_NONE;
        size_t a = 0, c = 0;
        VSZ_TRY(vsz_compress_bounds(&q, ndim, sd, &a, &c));
        cws  = a > cws ? a : cws;
        acap = c > acap ? c : acap;
        vsz_archive_desc d{};
        d.ndim = ndim;
        for (int i = 0; i < 3; i++) d.dims[i] = i < ndim ? sd[i] : 1;
        d.payload_bytes = 8 * g.n;
        d.n_outlier     = g.n;
        d.n_pad         = 0;
        d.has_trailer   = 1;
        d.eb_final      = 1.0;
        d.dict_size     = p->dict_size;
        d.block_size    = bs;
        d.chunk_syms    = 512;
        d.n_chunks      = (g.n + 511) / 512;
        size_t dw = 0;
        VSZ_TRY(vsz_decompress_bounds(&d, nullptr, &dw));
        dws = dw > dws ? dw : dws;
    }
    Bump b{base, cap_bytes};
    w.cws       = b.take<uint8_t>(cws);
    w.cws_bytes = cws;
    w.archive   = b.take<uint8_t>(acap + 64);
    w.cap       = acap;
    w.dws       = b.take<uint8_t>(dws);
    w.dws_bytes = dws;
    w.out       = b.take<float>(g.n);
    w.result    = b.take<uint64_t>(8);
    w.status    = b.take<int>(4);
    w.bytes     = b.off + 256;
    return VSZ_OK;
}

}  // namespace

vsz_status vsz_autotune_bounds(const vsz_params* p, int ndim, const size_t dims[3], double sample_percent,
                               size_t* ws_bytes) {
    VSZ_TRY(check_params(p, ndim, dims));
    if (!(sample_percent > 0.0) || sample_percent > 100.0) return VSZ_ERR_INVALID;
    size_t sd[3];
    sample_geometry(ndim, dims, sample_percent, sd);
    FieldTuneWs w{};
    VSZ_TRY(layout_field_tune(p, ndim, sd, nullptr, 0, w));
    if (ws_bytes) *ws_bytes = w.bytes;
    return VSZ_OK;
}

vsz_status vsz_autotune(const vsz_params* p, int ndim, const size_t dims[3], const float* d_in, double sample_percent,
                        int iterations, double link_gbs, void* d_ws, size_t ws_bytes, vsz_tune_result* r,
                        void* stream) {
    VSZ_TRY(check_params(p, ndim, dims));
    if (!d_in || !d_ws || !r || iterations < 1 || !(sample_percent > 0.0) || sample_percent > 100.0 ||
        !(link_gbs >= 0.0))
        return VSZ_ERR_INVALID;
    const TuneKey key = tune_key(p, ndim, dims, link_gbs);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            *r        = it->second;
            r->cached = 1;
            return VSZ_OK;
        }
    }
    size_t sd[3];
    const Geometry g = sample_geometry(ndim, dims, sample_percent, sd);
    FieldTuneWs w{};
    VSZ_TRY(layout_field_tune(p, ndim, sd, reinterpret_cast<uint8_t*>(d_ws), ws_bytes, w));
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    cudaStream_t st = S(stream);
    cudaEvent_t e0, e1;
    VSZ_CUDA(cudaEventCreate(&e0));
    VSZ_CUDA(cudaEventCreate(&e1));
    static const int kSizes[4] = {8, 16, 32, 64};
    vsz_tune_result res{};
    int rc = VSZ_OK;
    std::vector<uint8_t> host;
    auto timed = [&](auto&& once, double* ms_out) -> int {
        VSZ_TRY(once());  // warm-up
        VSZ_CUDA(cudaEventRecord(e0, st));
        for (int it = 0; it < iterations; it++) VSZ_TRY(once());
        VSZ_CUDA(cudaEventRecord(e1, st));
        VSZ_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        VSZ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        *ms_out = ms / iterations;
        return VSZ_OK;
    };
    for (int k = 0; k < 4 && rc == VSZ_OK; k++) {
        vsz_params q = *p;
        q.block_size = kSizes[k];
        q.lossless   = VSZ_LOSSLESS_NONE;
        auto comp    = [&]() {
            return vsz_compress(&q, ndim, sd, d_in, w.cws, w.cws_bytes, w.archive, w.cap, w.result, stream);
        };
        if ((rc = timed(comp, &res.compress_ms[k])) != VSZ_OK) break;
        uint64_t rec[8];
        if (cudaMemcpy(rec, w.result, sizeof(rec), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = VSZ_ERR_CUDA;
            break;
        }
        if (rec[5] != VSZ_OK) {
            rc = (int)rec[5];
            break;
        }
        res.archive_bytes[k] = rec[0];
        host.resize(rec[0] + rec[1]);
        vsz_archive_desc d{};
        if (cudaMemcpy(host.data(), w.archive, host.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = VSZ_ERR_CUDA;
            break;
        }
        if ((rc = vsz_archive_parse(host.data(), host.size(), &d)) != VSZ_OK) break;
        auto dec = [&]() {
            return vsz_decompress(&d, nullptr, w.archive, w.dws, w.dws_bytes, w.out, w.status, stream);
        };
        if ((rc = timed(dec, &res.decompress_ms[k])) != VSZ_OK) break;
        int dst = 0;
        if (cudaMemcpy(&dst, w.status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = VSZ_ERR_CUDA;
            break;
        }
        if (dst != VSZ_OK) {
            rc = dst;
            break;
        }
        res.score_ms[k] = res.compress_ms[k] + res.decompress_ms[k] +
                          (link_gbs > 0.0 ? (double)rec[0] / (link_gbs * 1e9) * 1e3 : 0.0);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VSZ_OK) return rc;
    int best = 0;
    for (int k = 1; k < 4; k++)
        if (res.score_ms[k] < res.score_ms[best]) best = k;
    res.block_size     = kSizes[best];
    res.cached         = 0;
    res.sample_elements = g.n;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = res;
    }
    *r = res;
    return VSZ_OK;
}

void vsz_autotune_cache_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
}

}  // extern "C"
