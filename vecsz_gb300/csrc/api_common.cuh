// Internal helpers shared by the single-field (vsz_api.cu) and batch (vsz_batch.cu) entry points:
// argument checks, workspace bump allocation, archive sizes and the archive finalisation.
#pragma once

#include <cstdint>
#include <cstring>

#include "vsz_device.cuh"
#include "vsz_huffman.h"
#include "vsz_kernels.h"

namespace vsz {

int num_sms();  // of the current device (cached)

namespace api {

constexpr uint32_t kTrailerMagic   = 0x545A5356u;  // "VSZT"
constexpr uint32_t kTrailerVersion = 1;
constexpr uint32_t kTrailerFixed   = 64;

#define VSZ_TRY(x)                        \
    do {                                  \
        int _rc = (x);                    \
        if (_rc != VSZ_OK) return _rc;    \
    } while (0)
#define VSZ_CUDA(x)                                    \
    do {                                               \
        if ((x) != cudaSuccess) return VSZ_ERR_CUDA;   \
    } while (0)

// Bump allocator over a caller workspace; with base == nullptr it only measures.
struct Bump {
    uint8_t* base;
    size_t cap;
    size_t off = 0;
    template <class T>
    T* take(size_t count, size_t align = 256) {
        off  = (off + align - 1) & ~(align - 1);
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
    bool fits() const { return off <= cap; }
};


inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool valid_dims(int ndim, const size_t* dims) {
    if (ndim < 1 || ndim > 3 || !dims) return false;
    size_t n = 1;
    for (int i = 0; i < ndim; i++) {
        if (dims[i] == 0 || dims[i] > 0x7fffffffu) return false;  // the archive stores i32 dims
        n *= dims[i];
        if (n > (1ull << 36)) return false;
    }
    return true;
}

inline bool valid_dict(int dict) { return dict >= 2 && dict <= 65536 && (dict % 2) == 0; }
inline bool valid_bs(int bs) { return bs == 8 || bs == 16 || bs == 32 || bs == 64; }

inline int check_params(const vsz_params* p, int ndim, const size_t* dims) {
    if (!p || !valid_dims(ndim, dims)) return VSZ_ERR_INVALID;
    if (!(p->eb > 0.0) || p->eb != p->eb || p->eb > 1e300) return VSZ_ERR_INVALID;
    if (p->mode != VSZ_MODE_ABS && p->mode != VSZ_MODE_R2R) return VSZ_ERR_INVALID;
    if (!valid_dict(p->dict_size)) return VSZ_ERR_INVALID;
    if (p->block_size <= 0) return VSZ_ERR_INVALID;
    if (!valid_bs(p->block_size)) return VSZ_ERR_UNSUPPORTED;
    if (p->flags & ~VSZ_FLAG_STRICT_EB) return VSZ_ERR_INVALID;
    if (p->pad_mode < VSZ_PAD_NONE || p->pad_mode > VSZ_PAD_EDGE) return VSZ_ERR_INVALID;
    if (p->pad_mode != VSZ_PAD_NONE) {
        if (p->pad_type < VSZ_PADV_MAX || p->pad_type > VSZ_PADV_CONST) return VSZ_ERR_INVALID;
        if (p->flags & VSZ_FLAG_STRICT_EB) return VSZ_ERR_UNSUPPORTED;  // strict mode keeps the zero halo
        // 1D block / edge values are raw: codes reach 2 * radius, which must fit the u16 codes
        if (ndim == 1 && p->pad_mode != VSZ_PAD_GLOBAL && p->dict_size > 32768) return VSZ_ERR_UNSUPPORTED;
    }
    return VSZ_OK;
}

// Histogram / codebook symbols: the dictionary, plus the code 2 * radius that a 1D field padded
// with raw block values can produce (the reference's tree takes 2 * dict symbols,
// src/vecsz_interface.hh:160).
inline int symbol_count(int dict, int ndim, int pad_mode) {
    return (ndim == 1 && (pad_mode == VSZ_PAD_BLOCK || pad_mode == VSZ_PAD_EDGE)) ? dict + 1 : dict;
}

inline size_t hdr_bytes(int ndim) { return 4 * (size_t)(ndim + 1) + 8 + 24; }

inline DqArgs make_dq_args(const Geometry& g, int bs, int dict, const float* x, const Consts* c, uint16_t* code,
                    float* scratch, uint8_t* seg_count, unsigned long long* hist) {
    DqArgs a{};
    a.x = x;
    a.code = code;
    a.scratch = scratch;
    a.seg_count = seg_count;
    a.hist = hist;
    a.consts = c;
    a.d0 = g.d0;
    a.d1 = g.d1;
    a.d2 = g.d2;
    a.nxt = g.nxt;
    a.nyg = (g.d1 + 7) / 8;
    a.nzb = (g.ndim == 3) ? (g.d2 + bs - 1) / bs : 1;
    a.xtail = (g.d0 % 8) ? (g.d0 & ~7u) : g.d0;
    a.R = dict / 2;
    a.dict = dict;
    a.smem_hist = dict <= 16384 ? 1 : 0;
    if (g.ndim == 1) a.nunits = (g.nxt + 3) / 4;  // 4 tiles per unit
    else a.nunits = (unsigned long long)g.nxt * a.nyg * a.nzb;
    return a;
}

// ---- archive finalization --------------------------------------------------------------------

struct FinalizeArgs {
    uint8_t* archive;
    int ndim;
    uint32_t dims[3];
    double eb;  // user eb (header field)
    int mode, dict, bs;
    int strict;
    size_t hdr;
    size_t npad;  // pad values after the header (written by the padding stage)
    const Consts* consts;
    const uint32_t* build_info;             // node count, tree bytes, max len
    const unsigned long long* payload_bits;
    const unsigned long long* n_out;
    const int* status;
    unsigned long long* result;             // vsz_result
    const uint16_t* chunk_bits;
    unsigned long long n_chunks;
    int f64;  // an f64 field: 8-byte outliers, counted as two 32-bit words in the header
};

__device__ __forceinline__ void put_bytes(uint8_t* d, const void* src, int n) {
    const uint8_t* s = reinterpret_cast<const uint8_t*>(src);
    for (int i = 0; i < n; i++) d[i] = s[i];
}

__device__ __forceinline__ size_t trailer_index_pad(size_t data_size) {
    size_t start = data_size + kTrailerFixed;
    return ((start + 7) & ~(size_t)7) - data_size;
}

// Header, result record and trailer (one thread of block 0), then the index copy (blocks
// `blk` of `nblk` stride over it).  Writes nothing to the archive after a failure.
__device__ __forceinline__ void finalize_field(const FinalizeArgs& f, unsigned blk, unsigned nblk) {
    const unsigned long long bits = *f.payload_bits;
    const unsigned long long nout = *f.n_out;
    const uint32_t tree           = f.build_info[1];
    const size_t huff_bytes       = 8 + (size_t)tree + (size_t)((bits + 7) >> 3);
    const unsigned long long owords = f.f64 ? 2 * nout : nout;  // outlier section in 32-bit words
    const size_t data_size        = f.hdr + 4 * f.npad + huff_bytes + 4 * (size_t)owords;
    const size_t pad              = trailer_index_pad(data_size);
    const size_t trailer          = ((pad + 2 * (size_t)f.n_chunks) + 7) & ~(size_t)7;
    uint8_t* t                    = f.archive + data_size;
    const int st                  = f.consts->status != VSZ_OK ? f.consts->status : *f.status;
    if (st != VSZ_OK) {
        // sizes from failed stages are not meaningful: report the status, write no archive bytes
        if (blk == 0 && threadIdx.x == 0) {
            for (int i = 0; i < 8; i++) f.result[i] = 0;
            f.result[5] = (unsigned long long)st;
        }
        return;
    }
    if (blk == 0 && threadIdx.x == 0) {
        int32_t nd = f.ndim;
        put_bytes(f.archive, &nd, 4);
        for (int i = 0; i < f.ndim; i++) {
            int32_t d = (int32_t)f.dims[i];
            put_bytes(f.archive + 4 * (1 + i), &d, 4);
        }
        put_bytes(f.archive + 4 * (f.ndim + 1), &f.eb, 8);
        unsigned long long lens[3] = {(unsigned long long)f.npad, (unsigned long long)huff_bytes, owords};
        put_bytes(f.archive + 4 * (f.ndim + 1) + 8, lens, 24);
        // trailer fixed part
        uint32_t u32[4] = {kTrailerMagic, kTrailerVersion, kTrailerFixed, (uint32_t)kChunkSyms};
        put_bytes(t, u32, 16);
        double ebf = f.consts->eb_final, vr = f.consts->range;
        put_bytes(t + 16, &ebf, 8);
        put_bytes(t + 24, &vr, 8);
        // bit 8: strict error-bound mode; bit 9: an f64 field
        int32_t i32[3] = {f.mode | (f.strict ? 0x100 : 0) | (f.f64 ? 0x200 : 0), f.dict, f.bs};
        put_bytes(t + 32, i32, 12);
        uint32_t padu = (uint32_t)pad;
        put_bytes(t + 44, &padu, 4);
        unsigned long long nch = f.n_chunks, tsz = trailer;
        put_bytes(t + 48, &nch, 8);
        put_bytes(t + 56, &tsz, 8);
        for (size_t i = kTrailerFixed; i < pad; i++) t[i] = 0;
        unsigned long long* r = f.result;
        r[0] = data_size;
        r[1] = trailer;
        r[2] = nout;
        r[3] = huff_bytes;
        r[4] = bits;
        r[5] = (unsigned long long)st;
        r[6] = f.build_info[2];
        r[7] = f.build_info[0];
    }
    uint16_t* idx = reinterpret_cast<uint16_t*>(t + pad);
    for (size_t i = blk * (size_t)blockDim.x + threadIdx.x; i < f.n_chunks; i += (size_t)nblk * blockDim.x)
        idx[i] = f.chunk_bits[i];
    if (blk == 0 && threadIdx.x == 0) {
        size_t used = pad + 2 * (size_t)f.n_chunks;
        for (size_t i = used; i < trailer; i++) t[i] = 0;
    }
}

inline size_t codebook_block_bytes(int dict) { return 9 * (size_t)dict + 16; }
// [BE nc][BE dict] + the largest serialised tree a dictionary can give
inline size_t tree_head_max(int dict) { return 8 + tree_bytes_size((uint32_t)(2 * dict - 1)); }

// dict: histogram symbols (symbol_count); npad: pad values (pad_count)
inline size_t archive_capacity(const Geometry& g, int dict, size_t npad = 0) {
    size_t tree_max = tree_bytes_size((uint32_t)(2 * dict - 1));
    size_t n_chunks = (g.n + kChunkSyms - 1) / kChunkSyms;
    return hdr_bytes(g.ndim) + 4 * npad + 8 + tree_max + 8 * g.n + 4 * g.n + kTrailerFixed + 8 + 2 * n_chunks + 64;
}

}  // namespace api
}  // namespace vsz
