// Host entry points of the C ABI: the reference's Compress / Decompress interface on host buffers
// (src/vecsz_interface.hh:31-375), with device memory cached between calls, and the lossless pass
// (src/lossless.hh) through the system zstd / zlib libraries loaded at run time.
#include <dlfcn.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "deflate_format.h"
#include "vsz_types.h"

namespace vsz {
void count_launch();                     // vsz_profile.cu
void set_thread_tree_builder(int which);  // vsz_api.cu: -1 = the process setting
}

namespace {

#define VSZ_TRY(x)                     \
    do {                               \
        int _rc = (x);                 \
        if (_rc != VSZ_OK) return _rc; \
    } while (0)
#define VSZ_CUDA(x)                                  \
    do {                                             \
        if ((x) != cudaSuccess) return VSZ_ERR_CUDA; \
    } while (0)

// ---- cached device buffers, one set per device -----------------------------------------------
struct DevBuf {
    void* p    = nullptr;
    size_t cap = 0;
    int grow(size_t need) {
        if (need <= cap) return VSZ_OK;
        if (p) cudaFree(p);
        p   = nullptr;
        cap = 0;
        size_t want = need + need / 8 + 4096;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return VSZ_ERR_NOMEM;
        }
        cap = want;
        return VSZ_OK;
    }
};

struct HostCtx {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    DevBuf in, ws, archive, out, result;
    DevBuf dws, dframe;  // the device gzip pass: workspace and zlib stream
};

HostCtx* ctx_for_device() {
    static HostCtx ctxs[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= 64) return nullptr;
    return &ctxs[dev];
}

int ensure_stream(HostCtx* c) {
    if (!c->stream) VSZ_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    return VSZ_OK;
}

// ---- lossless libraries --------------------------------------------------------------------
struct Zstd {
    bool tried = false, ok = false;
    size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
    size_t (*bound)(size_t) = nullptr;
    unsigned (*is_error)(size_t) = nullptr;
    size_t (*decompress)(void*, size_t, const void*, size_t) = nullptr;
    unsigned long long (*content_size)(const void*, size_t) = nullptr;
};
struct Zlib {
    bool tried = false, ok = false;
    int (*compress2)(uint8_t*, unsigned long*, const uint8_t*, unsigned long, int) = nullptr;
    unsigned long (*bound)(unsigned long) = nullptr;
    int (*uncompress)(uint8_t*, unsigned long*, const uint8_t*, unsigned long) = nullptr;
};

std::mutex g_lib_mu;
Zstd g_zstd;
Zlib g_zlib;

Zstd* zstd() {
    std::lock_guard<std::mutex> lk(g_lib_mu);
    if (!g_zstd.tried) {
        g_zstd.tried = true;
        void* h      = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libzstd.so", RTLD_NOW | RTLD_LOCAL);
        if (h) {
            g_zstd.compress     = (decltype(g_zstd.compress))dlsym(h, "ZSTD_compress");
            g_zstd.bound        = (decltype(g_zstd.bound))dlsym(h, "ZSTD_compressBound");
            g_zstd.is_error     = (decltype(g_zstd.is_error))dlsym(h, "ZSTD_isError");
            g_zstd.decompress   = (decltype(g_zstd.decompress))dlsym(h, "ZSTD_decompress");
            g_zstd.content_size = (decltype(g_zstd.content_size))dlsym(h, "ZSTD_getFrameContentSize");
            g_zstd.ok = g_zstd.compress && g_zstd.bound && g_zstd.is_error && g_zstd.decompress && g_zstd.content_size;
        }
    }
    return g_zstd.ok ? &g_zstd : nullptr;
}

Zlib* zlib() {
    std::lock_guard<std::mutex> lk(g_lib_mu);
    if (!g_zlib.tried) {
        g_zlib.tried = true;
        void* h      = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
        if (h) {
            g_zlib.compress2  = (decltype(g_zlib.compress2))dlsym(h, "compress2");
            g_zlib.bound      = (decltype(g_zlib.bound))dlsym(h, "compressBound");
            g_zlib.uncompress = (decltype(g_zlib.uncompress))dlsym(h, "uncompress");
            g_zlib.ok         = g_zlib.compress2 && g_zlib.bound && g_zlib.uncompress;
        }
    }
    return g_zlib.ok ? &g_zlib : nullptr;
}

// ---- deflate index --------------------------------------------------------------------------
// Written after the trailer when the gzip pass ran on the device, so the decompressor can inflate
// the chunks independently on the device: [u32 magic "VSZD"][u32 version][u32 chunk bytes]
// [u32 head bytes][u64 chunks][u64 inflated bytes][u64 values][u32 compressed bytes per chunk],
// padded to 8.  Readers that do not know it ignore it (the reference reads lossless_size bytes).
constexpr uint32_t kDeflateIndexMagic   = 0x445A5356u;
constexpr uint32_t kDeflateIndexVersion = 1;
constexpr uint32_t kDeflateIndexHead    = 40;
constexpr uint32_t kDeflateChunk        = (uint32_t)vsz::kDeflateChunk;

size_t deflate_index_bytes(size_t nchunks) { return (kDeflateIndexHead + 4 * nchunks + 7) & ~(size_t)7; }

struct DeflateIndex {
    size_t nchunks = 0, raw = 0, values = 0;
    std::vector<uint32_t> sizes;
    std::vector<unsigned long long> offsets;  // of each chunk in the stream
    uint32_t adler = 0;
};

// The index of an archive [frame (lossless_size)][trailer][index], checked against the frame.
bool read_deflate_index(const uint8_t* h, size_t len, size_t lossless_size, DeflateIndex* ix) {
    if (lossless_size < 8 || len < lossless_size + 64 || h[0] != 0x78 || h[1] != 0x01) return false;
    const uint8_t* t = h + lossless_size;
    uint32_t tu[3];
    memcpy(tu, t, 12);
    if (tu[0] != 0x545A5356u || tu[1] != 1 || tu[2] != 64) return false;  // this library's trailer
    uint64_t tsz;
    memcpy(&tsz, t + 56, 8);
    if (tsz > len - lossless_size || len - lossless_size - tsz < kDeflateIndexHead) return false;
    const uint8_t* di = t + tsz;
    uint32_t u32[4];
    uint64_t u64[3];
    memcpy(u32, di, 16);
    memcpy(u64, di + 16, 24);
    if (u32[0] != kDeflateIndexMagic || u32[1] != kDeflateIndexVersion || u32[2] != kDeflateChunk ||
        u32[3] != kDeflateIndexHead)
        return false;
    const size_t nch = u64[0], raw = u64[1];
    if (nch != (raw + kDeflateChunk - 1) / kDeflateChunk || nch > (len >> 2)) return false;
    if (deflate_index_bytes(nch) > len - lossless_size - tsz) return false;
    ix->nchunks = nch;
    ix->raw     = raw;
    ix->values  = u64[2];
    ix->sizes.resize(nch);
    ix->offsets.resize(nch);
    if (nch) memcpy(ix->sizes.data(), di + kDeflateIndexHead, 4 * nch);
    unsigned long long off = 2;
    for (size_t c = 0; c < nch; c++) {
        if (ix->sizes[c] == 0 || ix->sizes[c] > kDeflateChunk + 5) return false;
        ix->offsets[c] = off;
        off += ix->sizes[c];
    }
    if (off + 6 != lossless_size) return false;  // final empty block (2 bytes) and Adler-32
    const uint8_t* a = h + lossless_size - 4;
    ix->adler = ((uint32_t)a[0] << 24) | ((uint32_t)a[1] << 16) | ((uint32_t)a[2] << 8) | a[3];
    return true;
}

// zlib header check of isZlibFormat (src/lossless.hh:40-57)
bool zlib_magic(const uint8_t* b, size_t len) {
    if (len < 2) return false;
    unsigned m1 = b[0], m2 = b[1];
    if (m1 == 104 && (m2 == 5 || m2 == 129 || m2 == 222)) return true;
    if (m1 == 120 && (m2 == 1 || m2 == 94 || m2 == 156 || m2 == 218)) return true;
    return false;
}

}  // namespace

// ---- stream-ordered host-buffer operations (vsz_host_op_*) ---------------------------------------

struct vsz_host_op {
    int device = 0;
    cudaStream_t stream = nullptr;
    DevBuf in, ws, archive, out, result;
};

namespace {
// The archive (data_size + trailer_size bytes, known only on the device) and the result record
// into pinned host memory: 16-byte pieces where both ends allow, bytes otherwise.
__global__ void __launch_bounds__(256) k_archive_to_host(const uint8_t* __restrict__ a, const uint64_t* __restrict__ r,
                                                         uint8_t* __restrict__ h_out, size_t cap, uint64_t* h_result) {
    const uint64_t total = r[5] == VSZ_OK ? r[0] + r[1] : 0;
    const bool fits      = total <= cap;
    if (blockIdx.x == 0 && threadIdx.x < 8) {
        uint64_t v = r[threadIdx.x];
        if (threadIdx.x == 5 && r[5] == VSZ_OK && !fits) v = VSZ_ERR_CAPACITY;
        h_result[threadIdx.x] = v;
    }
    if (!fits || total == 0) return;
    const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const bool vec   = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(h_out)) & 15u) == 0;
    size_t done      = 0;
    if (vec) {
        const size_t n16 = (size_t)(total / 16);
        const uint4* s   = reinterpret_cast<const uint4*>(a);
        uint4* d         = reinterpret_cast<uint4*>(h_out);
        for (size_t i = tid; i < n16; i += stride) d[i] = s[i];
        done = n16 * 16;
    }
    for (size_t i = done + tid; i < total; i += stride) h_out[i] = a[i];
}
}  // namespace

extern "C" {

void vsz_free_host(void* p) { free(p); }

int vsz_lossless_detect(const uint8_t* h, size_t len) {
    if (!h || len < 2) return 0;
    // ZSTD_getFrameContentSize != ZSTD_CONTENTSIZE_ERROR (src/lossless.hh:62-64); the magic
    // number 0xFD2FB528 is what that check keys on.
    if (len >= 4 && h[0] == 0x28 && h[1] == 0xB5 && h[2] == 0x2F && h[3] == 0xFD) return 1;
    if (zlib_magic(h, len)) return 2;
    return 0;
}

vsz_status vsz_lossless_compress(int which, const uint8_t* h_in, size_t len, uint8_t** h_out, size_t* out_len) {
    if (!h_in || !h_out || !out_len) return VSZ_ERR_INVALID;
    if (which == VSZ_LOSSLESS_ZSTD) {
        Zstd* z = zstd();
        if (!z) return VSZ_ERR_UNSUPPORTED;
        size_t cap = z->bound(len);
        uint8_t* o = (uint8_t*)malloc(cap ? cap : 1);
        if (!o) return VSZ_ERR_NOMEM;
        size_t r = z->compress(o, cap, h_in, len, 3);
        if (z->is_error(r)) {
            free(o);
            return VSZ_ERR_CORRUPT;
        }
        *h_out   = o;
        *out_len = r;
        return VSZ_OK;
    }
    if (which == VSZ_LOSSLESS_GZIP) {
        Zlib* z = zlib();
        if (!z) return VSZ_ERR_UNSUPPORTED;
        unsigned long cap = z->bound((unsigned long)len);
        uint8_t* o        = (uint8_t*)malloc(cap ? cap : 1);
        if (!o) return VSZ_ERR_NOMEM;
        unsigned long ol = cap;
        if (z->compress2(o, &ol, h_in, (unsigned long)len, 3) != 0) {
            free(o);
            return VSZ_ERR_CORRUPT;
        }
        *h_out   = o;
        *out_len = ol;
        return VSZ_OK;
    }
    return VSZ_ERR_INVALID;
}

vsz_status vsz_lossless_decompress(const uint8_t* h_in, size_t len, size_t target, uint8_t** h_out, size_t* out_len) {
    if (!h_in || !h_out || !out_len) return VSZ_ERR_INVALID;
    int kind   = vsz_lossless_detect(h_in, len);
    uint8_t* o = (uint8_t*)malloc(target + 16);
    if (!o) return VSZ_ERR_NOMEM;
    if (kind == 1) {
        Zstd* z = zstd();
        if (!z) {
            free(o);
            return VSZ_ERR_UNSUPPORTED;
        }
        size_t r = z->decompress(o, target, h_in, len);
        if (z->is_error(r)) {
            free(o);
            return VSZ_ERR_CORRUPT;
        }
        *out_len = r;
    } else if (kind == 2) {
        Zlib* z = zlib();
        if (!z) {
            free(o);
            return VSZ_ERR_UNSUPPORTED;
        }
        unsigned long ol = (unsigned long)target;
        if (z->uncompress(o, &ol, h_in, (unsigned long)len) != 0) {
            free(o);
            return VSZ_ERR_CORRUPT;
        }
        *out_len = ol;
    } else {
        free(o);
        return VSZ_ERR_CORRUPT;
    }
    *h_out = o;
    return VSZ_OK;
}

vsz_status vsz_compress_host_bound(const vsz_params* p, int ndim, const size_t dims[3], size_t* out_capacity) {
    size_t ws = 0, cap = 0;
    VSZ_TRY(vsz_compress_bounds(p, ndim, dims, &ws, &cap));
    // a lossless frame of incompressible bytes is slightly longer than its input (zstd's bound is
    // len + len / 256 + a few KB; zlib's and the device pass's are smaller)
    if (p && p->lossless != VSZ_LOSSLESS_NONE) cap += cap / 128 + 4096;
    if (out_capacity) *out_capacity = cap;
    return VSZ_OK;
}

vsz_status vsz_compress_host_into(const vsz_params* p, int ndim, const size_t dims[3], const float* h_in,
                                  uint8_t* h_out, size_t out_capacity, size_t* out_bytes, size_t* data_size,
                                  size_t* lossless_size, size_t* n_outlier) {
    if (!h_in || !h_out) return VSZ_ERR_INVALID;
    size_t ws = 0, cap = 0;
    VSZ_TRY(vsz_compress_bounds(p, ndim, dims, &ws, &cap));
    HostCtx* c = ctx_for_device();
    if (!c) return VSZ_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(c->mu);
    VSZ_TRY(ensure_stream(c));
    size_t n = dims[0] * (ndim > 1 ? dims[1] : 1) * (ndim > 2 ? dims[2] : 1);
    VSZ_TRY(c->in.grow(n * sizeof(float)));
    VSZ_TRY(c->ws.grow(ws));
    VSZ_TRY(c->archive.grow(cap));
    VSZ_TRY(c->result.grow(64));
    VSZ_CUDA(cudaMemcpyAsync(c->in.p, h_in, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    VSZ_TRY(vsz_compress(p, ndim, dims, (const float*)c->in.p, c->ws.p, c->ws.cap, (uint8_t*)c->archive.p,
                         c->archive.cap, (uint64_t*)c->result.p, c->stream));
    vsz_result r;
    VSZ_CUDA(cudaMemcpyAsync(&r, c->result.p, sizeof(r), cudaMemcpyDeviceToHost, c->stream));
    VSZ_CUDA(cudaStreamSynchronize(c->stream));
    if (r.status != VSZ_OK) return (vsz_status)r.status;
    size_t total = r.data_size + r.trailer_size;
    if (p->lossless == VSZ_LOSSLESS_GZIP_DEVICE) {
        // the gzip pass on the device: only the zlib stream and the trailer come back
        size_t dws = 0, fcap = 0;
        VSZ_TRY(vsz_deflate_bounds(r.data_size, &dws, &fcap));
        VSZ_TRY(c->dws.grow(dws));
        VSZ_TRY(c->dframe.grow(fcap));
        VSZ_TRY(vsz_deflate((const uint8_t*)c->archive.p, r.data_size, c->dws.p, c->dws.cap, (uint8_t*)c->dframe.p,
                            c->dframe.cap, (uint64_t*)c->result.p, c->stream));
        uint64_t dr[8];
        VSZ_CUDA(cudaMemcpyAsync(dr, c->result.p, sizeof(dr), cudaMemcpyDeviceToHost, c->stream));
        VSZ_CUDA(cudaStreamSynchronize(c->stream));
        if (dr[1] != VSZ_OK) return (vsz_status)dr[1];
        const size_t flen = dr[0], nch = dr[2];
        const size_t ib   = deflate_index_bytes(nch);
        if (flen + r.trailer_size + ib > out_capacity) return VSZ_ERR_CAPACITY;
        VSZ_CUDA(cudaMemcpyAsync(h_out, c->dframe.p, flen, cudaMemcpyDeviceToHost, c->stream));
        VSZ_CUDA(cudaMemcpyAsync(h_out + flen, (const uint8_t*)c->archive.p + r.data_size, r.trailer_size,
                                 cudaMemcpyDeviceToHost, c->stream));
        uint8_t* di = h_out + flen + r.trailer_size;
        memset(di, 0, ib);
        const uint32_t head[4] = {kDeflateIndexMagic, kDeflateIndexVersion, kDeflateChunk, kDeflateIndexHead};
        const uint64_t counts[3] = {nch, r.data_size, n};
        memcpy(di, head, 16);
        memcpy(di + 16, counts, 24);
        VSZ_TRY(vsz_deflate_chunk_sizes(c->dws.p, r.data_size, reinterpret_cast<uint32_t*>(di + kDeflateIndexHead),
                                        c->stream));
        VSZ_CUDA(cudaStreamSynchronize(c->stream));
        if (out_bytes) *out_bytes = flen + r.trailer_size + ib;
        if (lossless_size) *lossless_size = flen;
    } else if (p->lossless == VSZ_LOSSLESS_NONE) {
        if (total > out_capacity) return VSZ_ERR_CAPACITY;
        VSZ_CUDA(cudaMemcpyAsync(h_out, c->archive.p, total, cudaMemcpyDeviceToHost, c->stream));
        VSZ_CUDA(cudaStreamSynchronize(c->stream));
        if (out_bytes) *out_bytes = total;
        if (lossless_size) *lossless_size = 0;
    } else {
        std::vector<uint8_t> tmp(total);
        VSZ_CUDA(cudaMemcpyAsync(tmp.data(), c->archive.p, total, cudaMemcpyDeviceToHost, c->stream));
        VSZ_CUDA(cudaStreamSynchronize(c->stream));
        uint8_t* frame = nullptr;
        size_t flen    = 0;
        VSZ_TRY(vsz_lossless_compress(p->lossless, tmp.data(), r.data_size, &frame, &flen));
        if (flen + r.trailer_size > out_capacity) {
            free(frame);
            return VSZ_ERR_CAPACITY;
        }
        memcpy(h_out, frame, flen);
        memcpy(h_out + flen, tmp.data() + r.data_size, r.trailer_size);
        free(frame);
        if (out_bytes) *out_bytes = flen + r.trailer_size;
        if (lossless_size) *lossless_size = flen;
    }
    if (data_size) *data_size = r.data_size;
    if (n_outlier) *n_outlier = r.n_outlier;
    return VSZ_OK;
}

vsz_status vsz_compress_host(const vsz_params* p, int ndim, const size_t dims[3], const float* h_in, uint8_t** h_out,
                             size_t* out_bytes, size_t* data_size, size_t* lossless_size, size_t* n_outlier) {
    if (!h_out) return VSZ_ERR_INVALID;
    size_t cap = 0;
    VSZ_TRY(vsz_compress_host_bound(p, ndim, dims, &cap));
    uint8_t* buf = (uint8_t*)malloc(cap);
    if (!buf) return VSZ_ERR_NOMEM;
    size_t ob = 0;
    int rc    = vsz_compress_host_into(p, ndim, dims, h_in, buf, cap, &ob, data_size, lossless_size, n_outlier);
    if (rc) {
        free(buf);
        return rc;
    }
    uint8_t* shrunk = (uint8_t*)realloc(buf, ob ? ob : 1);
    *h_out          = shrunk ? shrunk : buf;
    if (out_bytes) *out_bytes = ob;
    return VSZ_OK;
}

}  // extern "C"

namespace {

// The archive is on the device (c->archive, `used` bytes and 64 zero bytes after them): decode it
// into h_out.  The caller holds c->mu.
int decode_resident(HostCtx* c, const vsz_archive_desc& d, const vsz_decompress_opts* opts, float* h_out,
                    size_t out_capacity, size_t* n_out) {
    const size_t n = d.dims[0] * d.dims[1] * d.dims[2];
    if (n > out_capacity) return VSZ_ERR_CAPACITY;
    size_t ws = 0;
    VSZ_TRY(vsz_decompress_bounds(&d, opts, &ws));
    VSZ_TRY(c->ws.grow(ws));
    VSZ_TRY(c->out.grow(n * sizeof(float)));
    VSZ_TRY(c->result.grow(64));
    VSZ_TRY(vsz_decompress(&d, opts, (const uint8_t*)c->archive.p, c->ws.p, c->ws.cap, (float*)c->out.p,
                           (int*)c->result.p, c->stream));
    int st = 0;
    VSZ_CUDA(cudaMemcpyAsync(&st, c->result.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    VSZ_CUDA(cudaMemcpyAsync(h_out, c->out.p, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    VSZ_CUDA(cudaStreamSynchronize(c->stream));
    if (st != VSZ_OK) return st;
    if (n_out) *n_out = n;
    return VSZ_OK;
}

// -L archives whose frame came from the device gzip pass: inflate on the device from the deflate
// index.  Returns 1 when the archive has no usable index or the stream does not inflate (the
// caller then takes the host library path), else a status.
int decompress_device_inflate(const uint8_t* h, size_t len, size_t data_size, size_t lossless_size,
                              const vsz_decompress_opts* opts, float* h_out, size_t out_capacity, size_t* n_out) {
    DeflateIndex ix;
    if (!read_deflate_index(h, len, lossless_size, &ix)) return 1;
    if (data_size && ix.raw != data_size) return VSZ_ERR_CORRUPT;
    const uint8_t* trailer = h + lossless_size;
    uint64_t tsz;
    memcpy(&tsz, trailer + 56, 8);
    HostCtx* c = ctx_for_device();
    if (!c) return VSZ_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(c->mu);
    VSZ_TRY(ensure_stream(c));
    size_t iws = 0;
    VSZ_TRY(vsz_inflate_bounds(ix.nchunks, &iws));
    const size_t tab = (12 * ix.nchunks + 255) & ~(size_t)255;
    VSZ_TRY(c->dframe.grow(lossless_size + 64));
    VSZ_TRY(c->dws.grow(tab + iws));
    VSZ_TRY(c->archive.grow(ix.raw + tsz + 64));
    VSZ_TRY(c->result.grow(64));
    uint8_t* dws = (uint8_t*)c->dws.p;
    VSZ_CUDA(cudaMemcpyAsync(c->dframe.p, h, lossless_size, cudaMemcpyHostToDevice, c->stream));
    VSZ_CUDA(cudaMemcpyAsync(dws, ix.offsets.data(), 8 * ix.nchunks, cudaMemcpyHostToDevice, c->stream));
    VSZ_CUDA(cudaMemcpyAsync(dws + 8 * ix.nchunks, ix.sizes.data(), 4 * ix.nchunks, cudaMemcpyHostToDevice,
                             c->stream));
    VSZ_TRY(vsz_inflate((const uint8_t*)c->dframe.p, lossless_size, (const unsigned long long*)dws,
                        (const uint32_t*)(dws + 8 * ix.nchunks), ix.nchunks, ix.adler, (uint8_t*)c->archive.p, ix.raw,
                        dws + tab, iws, (int*)c->result.p, c->stream));
    VSZ_CUDA(cudaMemcpyAsync((uint8_t*)c->archive.p + ix.raw, trailer, tsz, cudaMemcpyHostToDevice, c->stream));
    VSZ_CUDA(cudaMemsetAsync((uint8_t*)c->archive.p + ix.raw + tsz, 0, 64, c->stream));
    // the header and the Huffman head come back for the parse
    int st = 0;
    std::vector<uint8_t> head(std::min<size_t>(ix.raw, 64));
    VSZ_CUDA(cudaMemcpyAsync(&st, c->result.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    VSZ_CUDA(cudaMemcpyAsync(head.data(), c->archive.p, head.size(), cudaMemcpyDeviceToHost, c->stream));
    VSZ_CUDA(cudaStreamSynchronize(c->stream));
    if (st != VSZ_OK) return 1;  // not a stream this inflater takes: the host library decides
    if (head.size() >= 4) {
        int32_t nd;
        memcpy(&nd, head.data(), 4);
        if (nd >= 1 && nd <= 3) {
            uint64_t npad;
            memcpy(&npad, head.data() + 4 * (nd + 1) + 8, 8);
            const size_t need = 4 * (size_t)(nd + 1) + 32 + 4 * (size_t)std::min<uint64_t>(npad, 1ull << 40) + 8;
            if (need > head.size() && need <= ix.raw) {
                head.resize(need);
                VSZ_CUDA(cudaMemcpyAsync(head.data(), c->archive.p, need, cudaMemcpyDeviceToHost, c->stream));
                VSZ_CUDA(cudaStreamSynchronize(c->stream));
            }
        }
    }
    vsz_archive_desc d;
    VSZ_TRY(vsz_archive_parse_split(head.data(), head.size(), trailer, len - lossless_size, &d));
    if (d.data_size != ix.raw) return VSZ_ERR_CORRUPT;
    return decode_resident(c, d, opts, h_out, out_capacity, n_out);
}

}  // namespace

extern "C" {

vsz_status vsz_decompress_host_into(const uint8_t* h_archive, size_t len, size_t data_size, size_t lossless_size,
                                    const vsz_decompress_opts* opts, float* h_out, size_t out_capacity, size_t* n_out) {
    if (!h_archive || !h_out) return VSZ_ERR_INVALID;
    if (lossless_size > 0 && lossless_size <= len) {
        const int rc = decompress_device_inflate(h_archive, len, data_size, lossless_size, opts, h_out, out_capacity,
                                                 n_out);
        if (rc != 1) return rc;
    }
    // 1. undo the lossless pass; the trailer (if any) follows the frame
    std::vector<uint8_t> packed;
    const uint8_t* block = h_archive;
    size_t block_len     = len;
    if (lossless_size > 0) {
        if (lossless_size > len) return VSZ_ERR_CORRUPT;
        uint8_t* raw = nullptr;
        size_t rl    = 0;
        VSZ_TRY(vsz_lossless_decompress(h_archive, lossless_size, data_size, &raw, &rl));
        if (rl != data_size) {
            free(raw);
            return VSZ_ERR_CORRUPT;
        }
        packed.resize(data_size + (len - lossless_size));
        memcpy(packed.data(), raw, data_size);
        memcpy(packed.data() + data_size, h_archive + lossless_size, len - lossless_size);
        free(raw);
        block     = packed.data();
        block_len = packed.size();
    }
    vsz_archive_desc d;
    VSZ_TRY(vsz_archive_parse(block, block_len, &d));
    if (data_size && d.data_size != data_size) return VSZ_ERR_CORRUPT;
    size_t n = d.dims[0] * d.dims[1] * d.dims[2];
    if (n > out_capacity) return VSZ_ERR_CAPACITY;
    HostCtx* c = ctx_for_device();
    if (!c) return VSZ_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(c->mu);
    VSZ_TRY(ensure_stream(c));
    size_t used = d.has_trailer ? (size_t)(d.index_offset + 2 * d.n_chunks) : (size_t)d.data_size;
    VSZ_TRY(c->archive.grow(used + 64));
    VSZ_CUDA(cudaMemcpyAsync(c->archive.p, block, used, cudaMemcpyHostToDevice, c->stream));
    VSZ_CUDA(cudaMemsetAsync((uint8_t*)c->archive.p + used, 0, 64, c->stream));
    return decode_resident(c, d, opts, h_out, out_capacity, n_out);
}

vsz_status vsz_decompress_host(const uint8_t* h_archive, size_t len, size_t data_size, size_t lossless_size,
                               const vsz_decompress_opts* opts, float** h_out, size_t* n) {
    if (!h_out) return VSZ_ERR_INVALID;
    // size the output from the header (after the lossless pass if any)
    size_t cap = 0;
    DeflateIndex ix;
    if (lossless_size == 0) {
        vsz_archive_desc d;
        VSZ_TRY(vsz_archive_parse(h_archive, len, &d));
        cap = d.dims[0] * d.dims[1] * d.dims[2];
    } else if (lossless_size <= len && read_deflate_index(h_archive, len, lossless_size, &ix) && ix.values) {
        cap = ix.values;  // the device gzip pass recorded it
    } else {
        uint8_t* raw = nullptr;
        size_t rl    = 0;
        VSZ_TRY(vsz_lossless_decompress(h_archive, lossless_size, data_size, &raw, &rl));
        vsz_archive_desc d;
        int rc = vsz_archive_parse(raw, rl, &d);
        free(raw);
        VSZ_TRY(rc);
        cap = d.dims[0] * d.dims[1] * d.dims[2];
    }
    float* o = (float*)malloc(cap * sizeof(float) + 16);
    if (!o) return VSZ_ERR_NOMEM;
    int rc = vsz_decompress_host_into(h_archive, len, data_size, lossless_size, opts, o, cap, n);
    if (rc) {
        free(o);
        return rc;
    }
    *h_out = o;
    return VSZ_OK;
}

vsz_status vsz_autotune_block_size_host(const vsz_params* p, int ndim, const size_t dims[3], const float* h_in,
                                        double sample_percent, int iterations, int* best_block_size,
                                        double timings_ms[4]) {
    if (!p || !dims || !h_in || !best_block_size) return VSZ_ERR_INVALID;
    size_t ws = 0;
    VSZ_TRY(vsz_autotune_workspace_bytes(p, ndim, dims, sample_percent, &ws));
    HostCtx* c = ctx_for_device();
    if (!c) return VSZ_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(c->mu);
    VSZ_TRY(ensure_stream(c));
    size_t n = dims[0] * (ndim > 1 ? dims[1] : 1) * (ndim > 2 ? dims[2] : 1);
    VSZ_TRY(c->in.grow(n * sizeof(float)));
    VSZ_TRY(c->ws.grow(ws));
    VSZ_CUDA(cudaMemcpyAsync(c->in.p, h_in, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    return vsz_autotune_block_size(p, ndim, dims, (const float*)c->in.p, sample_percent, iterations, c->ws.p,
                                   c->ws.cap, best_block_size, timings_ms, c->stream);
}

vsz_status vsz_host_op_create(vsz_host_op** op) {
    if (!op) return VSZ_ERR_INVALID;
    vsz_host_op* o = new vsz_host_op();
    if (cudaGetDevice(&o->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete o;
        return VSZ_ERR_CUDA;
    }
    *op = o;
    return VSZ_OK;
}

void vsz_host_op_destroy(vsz_host_op* op) {
    if (!op) return;
    if (op->stream) {
        cudaStreamSynchronize(op->stream);
        cudaStreamDestroy(op->stream);
    }
    for (DevBuf* b : {&op->in, &op->ws, &op->archive, &op->out, &op->result})
        if (b->p) cudaFree(b->p);
    delete op;
}

vsz_status vsz_host_op_compress(vsz_host_op* op, const vsz_params* p, int ndim, const size_t dims[3], const float* h_in,
                                uint8_t* h_out, size_t out_capacity, uint64_t* h_result) {
    if (!op || !p || !h_in || !h_out || !h_result) return VSZ_ERR_INVALID;
    if (p->lossless != VSZ_LOSSLESS_NONE) return VSZ_ERR_UNSUPPORTED;
    size_t ws = 0, cap = 0;
    VSZ_TRY(vsz_compress_bounds(p, ndim, dims, &ws, &cap));
    size_t n = dims[0] * (ndim > 1 ? dims[1] : 1) * (ndim > 2 ? dims[2] : 1);
    VSZ_TRY(op->in.grow(n * sizeof(float)));
    VSZ_TRY(op->ws.grow(ws));
    VSZ_TRY(op->archive.grow(cap));
    VSZ_TRY(op->result.grow(64));
    VSZ_CUDA(cudaMemcpyAsync(op->in.p, h_in, n * sizeof(float), cudaMemcpyHostToDevice, op->stream));
    // The device tree builder: host operations run beside other operations' field-sized transfers
    // over the host link, and the host builder's few-KB exchange with the host then waits behind
    // them (pipelined round trips of a 512^3 field: 76, 81, 117 and 117 GB/s over four runs with
    // the host builder; 97, 120 and 120 with this one, whose ~0.7 ms the transfers hide).
    vsz::set_thread_tree_builder(VSZ_TREE_DEVICE);
    const int rc = vsz_compress(p, ndim, dims, (const float*)op->in.p, op->ws.p, op->ws.cap, (uint8_t*)op->archive.p,
                                op->archive.cap, (uint64_t*)op->result.p, op->stream);
    vsz::set_thread_tree_builder(-1);
    VSZ_TRY(rc);
    // enough CTAs to keep the link busy; the kernel strides over what the device says the size is
    k_archive_to_host<<<256, 256, 0, op->stream>>>((const uint8_t*)op->archive.p, (const uint64_t*)op->result.p,
                                                   h_out, out_capacity, h_result);
    vsz::count_launch();
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

vsz_status vsz_host_op_decompress(vsz_host_op* op, const uint8_t* h_archive, size_t len,
                                  const vsz_decompress_opts* opts, float* h_out, size_t out_capacity, int* h_status) {
    if (!op || !h_archive || !h_out || !h_status) return VSZ_ERR_INVALID;
    vsz_archive_desc d;
    VSZ_TRY(vsz_archive_parse(h_archive, len, &d));
    size_t n = d.dims[0] * d.dims[1] * d.dims[2];
    if (n > out_capacity) return VSZ_ERR_CAPACITY;
    size_t ws = 0;
    VSZ_TRY(vsz_decompress_bounds(&d, opts, &ws));
    size_t used = d.has_trailer ? (size_t)(d.index_offset + 2 * d.n_chunks) : (size_t)d.data_size;
    if (used > len) return VSZ_ERR_CORRUPT;
    VSZ_TRY(op->archive.grow(used + 64));
    VSZ_TRY(op->ws.grow(ws));
    VSZ_TRY(op->out.grow(n * sizeof(float)));
    VSZ_TRY(op->result.grow(64));
    VSZ_CUDA(cudaMemcpyAsync(op->archive.p, h_archive, used, cudaMemcpyHostToDevice, op->stream));
    VSZ_CUDA(cudaMemsetAsync((uint8_t*)op->archive.p + used, 0, 64, op->stream));
    VSZ_TRY(vsz_decompress(&d, opts, (const uint8_t*)op->archive.p, op->ws.p, op->ws.cap, (float*)op->out.p,
                           (int*)op->result.p, op->stream));
    VSZ_CUDA(cudaMemcpyAsync(h_status, op->result.p, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
    VSZ_CUDA(cudaMemcpyAsync(h_out, op->out.p, n * sizeof(float), cudaMemcpyDeviceToHost, op->stream));
    return VSZ_OK;
}

vsz_status vsz_host_op_wait(vsz_host_op* op) {
    if (!op) return VSZ_ERR_INVALID;
    return cudaStreamSynchronize(op->stream) == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

}  // extern "C"
