// Internal launcher interface between the C-ABI layer (vsz_api.cu) and the kernel files.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "vsz_types.h"

namespace vsz {

struct Consts;

// A byte offset known only on the device once earlier kernels ran (tree size, payload size):
// base + *add_u32 + ceil(*add_bits / 8).
struct DevOffset {
    size_t base;
    const uint32_t* add_u32;
    const unsigned long long* add_bits;
#ifdef __CUDACC__
    __device__ __forceinline__ size_t eval() const {
        size_t o = base;
        if (add_u32) o += *add_u32;
        if (add_bits) o += (size_t)((*add_bits + 7ull) >> 3);
        return o;
    }
#endif
};

// ---- padding (-p) ----------------------------------------------------------------------------
// Where a dual-quant kernel finds the halo values of each Lorenzo block.  Blocks are numbered on
// the reference's grid, get_nblk = (d + bs + 1) / bs per axis (src/dimensions.hh:32), x fastest.
struct PadView {
    const uint8_t* vals;  // f32 values at any byte address; null: the zero halo (no padding)
    int stride;           // values per block: 0 (every block reads value 0), 1, or ndim (edge)
    uint32_t nb0, nb1;    // grid blocks along x and y
};

// Halo values of one block: x-, y- and z-halo cells (src/utils/padding.hh:286-296, 342-373): a
// single value in global / block mode; edge mode 2D {x: v0, y: v1}, 3D {z: v0, y: v1, x: v2}.
// Corner cells take 2D x (x wins), 3D y (y wins in a plane), and z wherever z is the halo.
struct Halo {
    float x, y, z;
};

#ifdef __CUDACC__
__device__ __forceinline__ float pad_value_at(const uint8_t* p, size_t i) {
    const uint8_t* q = p + 4 * i;
    const uint32_t b = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
    return __uint_as_float(b);
}
__device__ __forceinline__ Halo halo_of(const PadView& p, int ndim, uint32_t bx, uint32_t by, uint32_t bz) {
    if (p.stride == 0) {
        const float v = pad_value_at(p.vals, 0);
        return Halo{v, v, v};
    }
    const size_t blk = (size_t)bx + (size_t)p.nb0 * ((size_t)by + (size_t)p.nb1 * bz);
    if (p.stride == 1) {
        const float v = pad_value_at(p.vals, blk);
        return Halo{v, v, v};
    }
    const size_t o = blk * (size_t)p.stride;
    if (ndim == 2) return Halo{pad_value_at(p.vals, o), pad_value_at(p.vals, o + 1), 0.0f};
    return Halo{pad_value_at(p.vals, o + 2), pad_value_at(p.vals, o + 1), pad_value_at(p.vals, o)};
}
#endif

// ---- many fields in one launch -------------------------------------------------------------
// A block-wide unit of work: one field of a batch and a range [u0, u1) of that field's work units
// (warp tiles, 512-code chunks, elements or look-back tiles, by stage).  Tasks are built on the
// host, where every field's geometry is known.
struct BatchTask {
    unsigned long long u0, u1;
    uint32_t field;
    uint32_t pad;
};

struct MinmaxField {
    const float* x;
    uint32_t* mm;  // {max key, min key}, initialised to {0, 0xffffffff}
};

struct ConstsField {
    int mode;
    double eb;
    const uint32_t* mm;
    const float* x;
    Consts* consts;
    int* status;
};

// ---- dual-quant compress ------------------------------------------------------------------
struct DqArgs {
    const float* x;
    uint16_t* code;
    float* scratch;              // outlier values, [segment][128]
    uint8_t* seg_count;          // outliers per segment
    unsigned long long* hist;    // dict entries, accumulated with atomics (caller zeroes)
    const Consts* consts;
    uint32_t d0, d1, d2;
    uint32_t nxt;                // 128-wide x tiles per row
    uint32_t nyg;                // groups of 8 rows
    uint32_t nzb;                // Lorenzo blocks along z (3D) or 1
    uint32_t xtail;              // first tail column: d0 & ~7 when d0 % 8 != 0, else d0
    int R;                       // radius = dict / 2
    int dict;
    int smem_hist;               // 1: histogram privatised in shared memory
    unsigned long long nunits;   // warp work units
    int strict;                  // strict error-bound mode (outliers carry input values)
    PadView pad;                 // padding (-p): the halo each block predicts from
};

struct GatherArgs {
    const uint8_t* seg_count;
    const float* scratch;
    size_t nseg;
    float* out_f32;              // aligned destination, or
    uint8_t* out_bytes;          // byte-addressed destination at out_bytes + out_off.eval()
    DevOffset out_off;
    unsigned long long* total;   // number of outliers (written by the last tile)
    unsigned long long* tile_status;
    uint32_t* tile_counter;
    int* status;
    uint32_t ntiles;
    // optional split copy: the look-back kernel records each segment's outlier offset within its
    // tile (seg_off, nseg) and each tile's first outlier (tile_base, ntiles), and k_outlier_copy
    // moves the values with the whole grid -- for fields with many outliers
    uint32_t* seg_off;
    unsigned long long* tile_base;
};

// ---- dual-quant decompress ----------------------------------------------------------------
struct DqDecArgs {
    const uint16_t* codes;
    const float* outliers;               // compact outlier values (aligned copy)
    unsigned long long n_outliers;       // entries of `outliers`; a rank past it is VSZ_ERR_CORRUPT
    int* status;
    const unsigned long long* seg_off;   // exclusive zero-code offsets per 256-wide row segment, or
    const unsigned long long* chunk_off; // exclusive zero-code offsets per 512-code chunk (block 8),
                                         // relative to chunk_off[0]
    const Consts* consts;
    float* out;
    uint32_t d0, d1, d2;
    size_t n;
    int R;
    uint32_t nxs;                        // 256-wide segments per row
    uint32_t nyb;                        // Lorenzo blocks along y
    uint32_t nbx8;                       // block 8: Lorenzo blocks along x
    uint32_t ygrp;                       // block 8: y-blocks per warp (narrow rows, dq_b8_narrow), else 1
    uint32_t nyb_g;                      // block 8: groups of ygrp y-blocks along y
    uint32_t nbx;                        // Lorenzo blocks along x (general kernel)
    unsigned long long nunits;
    int strict;                          // strict archive: outliers are input values (re-prequantized)
    uint32_t xtail;                      // 3D: first scalar-prequant column (d0 & ~7 when d0 % 8), else d0
    PadView pad;                         // padded archive: the halo of each block (vals = pad section)
    uint32_t* redo;                      // 3D block 8, separable pass: [0] count, then units whose
                                         // values left the exact range (null: reference order only)
    Consts* consts_rw;                   // the same constants when writable: the separable pass of a
                                         // large field records its dequantization check there (or null)
    unsigned long long* dq_cache;        // 4 words kept across calls: the last check's c_d and result
                                         // (or null)
    const unsigned long long* blk_off;   // 3D block 8, fields of at most kW8MaxN elements: exclusive
                                         // zero-code offsets per (row, x-block of 8), or null
};

// 3D block-8 fields up to this many elements take the wavefront reverse Lorenzo
// (k_dq_decompress_w8), which ranks outliers from per-(row, x-block) zero offsets.
constexpr size_t kW8MaxN = size_t(1) << 24;
// ... and those that would take the separable pass only up to this many.
constexpr size_t kW8MaxSeparableN = size_t(1) << 23;

int launch_dq_decompress(DqDecArgs a, int ndim, int bs, bool force_general, cudaStream_t st, int num_sms);
// Block size 8: unit geometry (nxs, nyb, nunits), whether the 16-byte row path applies, and
// whether the separable pass does (3D, vector rows, not strict, no padding, under 1 outlier in 64).
void dq_b8_geometry(DqDecArgs& a, int ndim);
// Block size 8, the reference-order kernel, rows of at most 16 blocks (2D / 3D): a warp takes
// 32 / nbx8 y-blocks side by side, and the unit count is recomputed for that.
void dq_b8_narrow(DqDecArgs& a, int ndim);
bool dq_b8_vec(const DqDecArgs& a);
bool dq_b8_separable(const DqDecArgs& a, int ndim);
// The wavefront pass applies: 3D, no padding, at most kW8MaxN elements (kW8MaxSeparableN for a
// field the separable pass takes), blk_off given (or no outliers), VSZ_DQ_NO_WAVEFRONT unset.
bool dq_w8_applies(const DqDecArgs& a, int ndim);
// Zero codes per (row, x-block of 8), row-major: nrows * ceil(d0 / 8) counts.
int launch_count_zeros_b8(const uint16_t* codes, uint32_t d0, size_t nrows, uint32_t* blk_zero, cudaStream_t st,
                          int num_sms);
// Many fields of one class (ndim, vec, separable), block size 8, no padding: tasks of (field,
// unit range), one warp each, handed out through the counter `next` (zero on entry; the class's
// own word).  A separable class is followed by launch_dq_redo_batch over its fields.
int launch_dq_decompress_batch(const DqDecArgs* args, const BatchTask* tasks, uint32_t ntasks, int ndim, bool vec,
                               bool sep, uint32_t* next, cudaStream_t st, int num_sms);
int launch_dq_redo_batch(const DqDecArgs* args, const BatchTask* tasks, uint32_t ntasks, cudaStream_t st,
                         int num_sms);
int launch_count_zeros(const uint16_t* codes, uint32_t d0, size_t nrows, uint32_t* seg_zero, cudaStream_t st,
                       int num_sms);

// ---- f64 fields (dq_f64.cu) ---------------------------------------------------------------
struct F64Args {
    const double* x;          // compress: the field
    long long* s;             // compress: prequantized values (n)
    uint16_t* code;           // codes (n): written by compress, read by decompress and the gather
    unsigned long long* hist; // compress: dict bins
    const Consts* consts;
    int* status;
    size_t n;
    uint32_t d0, d1, d2;
    int bs, dict;
    uint8_t* archive;             // compress: the archive (the gather writes its outlier section)
    const uint8_t* outliers;      // decompress: the archive's outlier section (8 bytes each, any alignment)
    unsigned long long n_out;     // decompress: outliers in it
    double* out;                  // decompress: the field
};
int launch_eb_setup_f64(int mode, double eb, const double* d_in, size_t n, Consts* c, unsigned long long* mm,
                        int* status, cudaStream_t st, int num_sms);
int launch_dq_compress_f64(F64Args a, int ndim, cudaStream_t st, int num_sms);
int launch_gather_f64(F64Args a, const unsigned long long* seg_off, DevOffset out_off, cudaStream_t st, int num_sms);
int launch_dq_decompress_f64(F64Args a, int ndim, const unsigned long long* seg_off, cudaStream_t st);

int launch_eb_setup(int mode, double eb, const float* d_in, size_t n, Consts* d_consts, uint32_t* d_mm,
                    cudaStream_t st, int* status_word = nullptr);
int launch_dq_compress(DqArgs a, int ndim, int bs, cudaStream_t st, int num_sms);
int launch_outlier_gather(GatherArgs g, cudaStream_t st, int num_sms = 0);

// Pad values of a field (-p).  Writes the archive's pad section (`arch`, any alignment) and, in
// global mode, the value the compressor's 2D/3D blocks predict from (`halo_g`).  ws: pad_ws_bytes.
struct PadArgs {
    const float* x;
    int ndim, bs, mode, type;
    float cst;
    uint32_t d0, d1, d2;
    uint32_t nb0, nb1, nb2;      // reference grid
    const Consts* consts;
    uint8_t* arch;
    float* halo_g;
    void* ws;
};
size_t pad_ws_bytes();
size_t pad_count(int ndim, const uint32_t d[3], int bs, int mode);
int launch_pad_values(const PadArgs& a, cudaStream_t st, int num_sms);

// Batched launchers (device arrays of per-field arguments and of tasks).  A dual-quant batch
// holds fields of one kernel class: ndim, block size, vec (d0 % 4 == 0 and aligned), tail
// (d0 % 8 != 0); hist_words = shared-memory histogram words (0 when no field uses one); next =
// the launch's task counter (zero on entry), through which free blocks take tasks.
int launch_minmax_batch(const MinmaxField* f, const BatchTask* tasks, uint32_t ntasks, cudaStream_t st, int num_sms);
int launch_consts_batch(const ConstsField* f, uint32_t nfields, cudaStream_t st);
int launch_dq_compress_batch(const DqArgs* args, const BatchTask* tasks, uint32_t ntasks, int ndim, int bs, bool vec,
                             bool tail, uint32_t hist_words, uint32_t* next, cudaStream_t st, int num_sms);
int launch_outlier_gather_batch(const GatherArgs* args, const BatchTask* tasks, uint32_t ntasks, cudaStream_t st,
                                int num_sms);
size_t gather_tmp_bytes(size_t nseg);
int set_spin_limit_dq(long long polls);  // test hook: this unit's look-back spin limit

// Geometry helpers shared by compress and decompress.
struct Geometry {
    int ndim;
    uint32_t d0, d1, d2;
    size_t n;
    uint32_t nxt;   // 128-wide tiles per row
    size_t nrows;   // d1 * d2
    size_t nseg;    // nrows * nxt
};

inline Geometry make_geometry(int ndim, const size_t* dims) {
    Geometry g{};
    g.ndim  = ndim;
    g.d0    = (uint32_t)dims[0];
    g.d1    = ndim > 1 ? (uint32_t)dims[1] : 1u;
    g.d2    = ndim > 2 ? (uint32_t)dims[2] : 1u;
    g.n     = (size_t)g.d0 * g.d1 * g.d2;
    g.nxt   = (g.d0 + 127u) / 128u;
    g.nrows = (size_t)g.d1 * g.d2;
    g.nseg  = g.nrows * g.nxt;
    return g;
}

}  // namespace vsz
