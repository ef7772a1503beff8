/*
 * vecsz_gb300.h -- C ABI of the GB300-native dual-quantization compressor (the SZ / vecSZ path).
 *
 * Every entry point takes plain pointers and sizes.  Device pointers are named d_*, host pointers
 * h_*; `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).  Device-side
 * entry points are stream-ordered and do not synchronise unless their comment says so.
 *
 * Field layout is the reference's: dims[0] is the fastest axis (x), dims[1] y, dims[2] z; a field
 * with ndim < 3 ignores the trailing dims.  dict_size is the reference's `-d` (quantization radius
 * = dict_size / 2), block_size its `-b`, eb its `-e`, mode its `-m`.
 *
 * Each entry point names the reference function (szcompressor/vecSZ, file:line) it replaces.
 * The library ships a ctypes binding (vecsz_gb300/_lib.py) for Python callers; C and C++ callers
 * include this header and link libvecsz_gb300.so.
 */
#ifndef VECSZ_GB300_H
#define VECSZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: the reference calls exit(); every entry point here returns one --------- */
typedef int vsz_status;
#define VSZ_OK 0
#define VSZ_ERR_INVALID 1     /* bad argument (dims, eb, dict_size, block_size, null pointer) */
#define VSZ_ERR_CUDA 2        /* a CUDA runtime call failed */
#define VSZ_ERR_CORRUPT 3     /* archive or bitstream does not parse */
#define VSZ_ERR_CAPACITY 4    /* caller buffer or workspace too small */
#define VSZ_ERR_TIMEOUT 5     /* a bounded device-side wait gave up */
#define VSZ_ERR_UNSUPPORTED 6 /* accepted by the reference, not supported here (documented) */
#define VSZ_ERR_RANGE 7       /* r2r with zero value range: the reference exits (src/types.cc:51-54) */
#define VSZ_ERR_NOMEM 8       /* device or host allocation failed */
#define VSZ_ERR_NO_DEVICE 9   /* no CUDA device */
#define VSZ_ERR_CANCELLED 10  /* request server: withdrawn by vsz_server_cancel before it ran */

#define VSZ_MODE_ABS 0 /* -m abs */
#define VSZ_MODE_R2R 1 /* -m r2r: eb relative to the value range */

#define VSZ_LOSSLESS_NONE 0
#define VSZ_LOSSLESS_ZSTD 1 /* -L zstd: host library, level 3 (src/lossless.hh:179-200) */
#define VSZ_LOSSLESS_GZIP 2 /* -L gzip: host library, level 3 */
/* -L gzip on the GPU (vsz_deflate): a zlib stream that the reference's lossless pass detects and
 * decodes (src/lossless.hh:40-76), with bytes of its own (not zlib's level 3 output). */
#define VSZ_LOSSLESS_GZIP_DEVICE 3

/* Compression settings: the ArgParse fields that reach the path
 * (src/argument_parser/argparse.hh:62-77; reference defaults eb 1e-4, dict 4096, block 8). */
typedef struct vsz_params {
    double eb;      /* -e */
    int mode;       /* -m: VSZ_MODE_ABS | VSZ_MODE_R2R */
    int dict_size;  /* -d: number of quant bins, even, 2..65536 */
    int block_size; /* -b: Lorenzo block edge: 8, 16, 32 or 64 */
    int lossless;   /* -L: VSZ_LOSSLESS_* (applied by the host entry points only) */
    int flags;      /* VSZ_FLAG_*; 0 = the reference's behaviour */
    int pad_mode;   /* -p: VSZ_PAD_*; 0 = the zero halo (no -p) */
    int pad_type;   /* -p: VSZ_PADV_* (the reference's default: constant) */
    float pad_constant; /* -p constant value (the number in the -p string) */
} vsz_params;

/* Padding (-p; src/utils/padding.hh, src/argument_parser/argparse.cc:399-415): the value(s) that
 * replace the zero halo of every Lorenzo block, stored in the packed block's pad section.
 *   global: one value from the whole field; block: one per block; edge: one per block face
 *   (1D: one per block).  Blocks are counted as the reference does, (d + bs + 1) / bs per axis.
 *   1D block / edge values are raw (not prequantized), as in the reference; such fields may give
 *   the code 2 * radius, so their dict_size must be at most 32768.
 *   Cells outside the field count as 0 (the reference reads past the field there).
 * Single-field entry points only (vsz_compress and the host / server paths built on it). */
#define VSZ_PAD_NONE 0
#define VSZ_PAD_GLOBAL 1
#define VSZ_PAD_BLOCK 2
#define VSZ_PAD_EDGE 3
#define VSZ_PADV_MAX 0
#define VSZ_PADV_MIN 1
#define VSZ_PADV_AVG 2   /* float running sum in field order, as the reference (a serial pass) */
#define VSZ_PADV_CONST 3
/* Parses a -p string as the reference's command line does: "global" / "block" / "edge",
 * "max" / "min" / "avg" / "constant" and the first number in it, into p->pad_*; global wins over
 * block and edge, block over edge (argparse.cc:156-170).  The type stays constant when none is
 * named. */
vsz_status vsz_parse_padding(const char* spec, vsz_params* p);
/* Number of pad values a packed block of this geometry holds (0 without padding). */
size_t vsz_pad_count(int ndim, const size_t dims[3], int block_size, int pad_mode);

/* Strict error-bound mode (opt-in; no counterpart in the reference).  Every element satisfies
 * |x - x^| <= eb: an element whose reconstruction would miss eb -- rounding overshoot, |x| / 2eb
 * beyond float precision, the reference's dropped 2D tail columns -- is stored as an outlier
 * carrying its input value.  Such archives are not byte-compatible with the reference's (their
 * outliers are input values, recorded in this library's trailer); single-field entry points only. */
#define VSZ_FLAG_STRICT_EB 1

/* What a compress produced (device-side vsz_compress writes these 8 u64 into d_result). */
typedef struct vsz_result {
    uint64_t data_size;    /* bytes of the packed block (the reference's data_size) */
    uint64_t trailer_size; /* bytes of this library's index trailer after the packed block */
    uint64_t n_outlier;    /* the reference's num_outlier */
    uint64_t huff_bytes;   /* Huffman section: 8 + tree bytes + payload */
    uint64_t payload_bits; /* Huffman bitstream length */
    uint64_t status;       /* VSZ_OK or the first device-side error */
    uint64_t max_code_len; /* longest codeword of the tree */
    uint64_t node_count;   /* Huffman tree nodes (2 * used symbols - 1) */
} vsz_result;

/* Parsed archive: the reference's packed block (src/utils/datapack.hh:17-56) plus, when present,
 * this library's trailer (r2r-final eb, block size, dict size and a decode index). */
typedef struct vsz_archive_desc {
    int ndim;
    uint64_t dims[3];
    double eb;              /* eb field of the packed block: the user's eb */
    uint64_t n_pad, huff_bytes, n_outlier;
    uint64_t header_bytes;  /* 4 (ndim + 1) + 8 + 24 */
    uint64_t huff_offset;   /* byte offset of the Huffman section */
    uint32_t node_count;
    uint64_t tree_bytes;
    uint64_t payload_offset;
    uint64_t payload_bytes;
    uint64_t outlier_offset;
    uint64_t data_size;     /* packed block bytes */
    int has_trailer;
    double eb_final;        /* trailer: absolute eb actually used */
    double value_range;     /* trailer: r2r value range (0 for abs) */
    int mode, dict_size, block_size;
    uint32_t chunk_syms;    /* trailer: codewords per index entry */
    uint64_t n_chunks;
    uint64_t index_offset;  /* trailer: byte offset of u16 bits-per-chunk, 8-byte aligned */
    uint64_t trailer_size;
    int strict;             /* trailer: written in strict error-bound mode (VSZ_FLAG_STRICT_EB) */
    int f64;                /* trailer: an f64 field (vsz_compress_f64); n_outlier counts 8-byte values */
} vsz_archive_desc;

/* Options a decompressor needs that the packed block does not store (the reference takes them
 * from the command line, src/vecsz_interface.hh:270-285).  Ignored where the trailer has them. */
typedef struct vsz_decompress_opts {
    int dict_size;      /* -d used at compression */
    int block_size;     /* -b used at compression */
    int mode;           /* -m used at compression */
    double value_range; /* r2r: value range of the original field (the reference re-reads it) */
} vsz_decompress_opts;

/* Size in bytes of the device-resident constant block written by vsz_eb_setup. */
#define VSZ_CONSTS_BYTES 64

const char* vsz_status_string(vsz_status status);
const char* vsz_version(void);

/* =============================================================================================
 * Stage-level entry points (device buffers).  Each replaces one reference routine; together they
 * are the compress/decompress workflow of src/vecsz_interface.hh.
 * ============================================================================================= */

/* Error-bound family on the device.  r2r: min/max pass over d_in, range = (float)max - (float)min.
 * Replaces GetDatumValueRange (src/types.cc:28-35), ChangeToRelativeMode (:49-60) and
 * InitializeErrorBoundFamily (:84-92).  d_consts: VSZ_CONSTS_BYTES; d_tmp: 16 bytes. */
vsz_status vsz_eb_setup(const vsz_params* p, const float* d_in, size_t n, void* d_consts, void* d_tmp, void* stream);
/* Reads {eb_final, 2 eb, 1/(2 eb), value range} and the constants' status.  Synchronises. */
vsz_status vsz_consts_read(const void* d_consts, double h_out[4], int* h_status, void* stream);

/* Number of 128-wide row segments used to rank outliers: d1 * d2 * ceil(d0 / 128). */
size_t vsz_outlier_segments(int ndim, const size_t dims[3]);

/* Prequant + Lorenzo + quant codes, fused with the code histogram and per-segment outlier
 * ranking.  Replaces c_lorenzo_{1,2,3}d1l (src/dualquant.hh:19-913) and the histogram loop of
 * initHuffman (src/huffman.hh:239-242).  d_code: n u16; d_scratch: segments * 128 floats;
 * d_seg_count: segments bytes; d_hist: dict_size u64, accumulated (zero it first). */
vsz_status vsz_dualquant(int ndim, const size_t dims[3], int block_size, int dict_size, const float* d_in,
                         const void* d_consts, uint16_t* d_code, float* d_scratch, uint8_t* d_seg_count,
                         uint64_t* d_hist, void* stream);

/* Outlier values in row-major order of code == 0 (src/vecsz_interface.hh:166-170) into d_out
 * (aligned floats); *d_count = their number.  d_tmp: vsz_outlier_gather_tmp_bytes. */
size_t vsz_outlier_gather_tmp_bytes(int ndim, const size_t dims[3]);
vsz_status vsz_outlier_gather(int ndim, const size_t dims[3], const uint8_t* d_seg_count, const float* d_scratch,
                              float* d_out, uint64_t* d_count, void* d_tmp, size_t tmp_bytes, void* stream);

/* The same gather for callers that cannot call cudaMalloc (a serving process whose device memory
 * another allocator owns, a latency-critical loop that cannot take an allocation's implicit
 * synchronisation, a plugin host that only hands over input and output buffers): it takes no
 * workspace and allocates nothing.  No counterpart in the reference.  Its scratch is a static
 * device array of about 512 KiB that every GPU loading this library holds until exit; fields with
 * more than 2^28 row segments (vsz_outlier_segments) are rejected with VSZ_ERR_CAPACITY, and dims
 * outside the limits of vsz_outlier_gather (each <= 2^31 - 1, at most 2^36 elements) with
 * VSZ_ERR_INVALID.  Every call looks up the array's device address on the current device (it is
 * not cached, so a reset device is handled); the first call on a device may load the library's
 * device code, so make it before any stream capture.  All calls share the array: calls that
 * overlap on the GPU (different streams, or different host threads) race and must be serialised
 * by the caller. */
vsz_status vsz_outlier_gather_noalloc(int ndim, const size_t dims[3], const uint8_t* d_seg_count,
                                      const float* d_scratch, float* d_out, uint64_t* d_count, void* stream);

/* Heap-tree Huffman codebook from a histogram, bit-identical to initHuffman + build_code +
 * convert_HuffTree_to_bytes_anyStates (src/huffman.hh:116-266, 374-502).
 * d_codebook: vsz_codebook_bytes(dict); d_huff_head: 8 + tree bytes, [BE nodeCount][BE dict][tree]
 * (capacity vsz_huff_head_max(dict)); d_info: 4 u32 {node count, tree bytes, max len, nodes}. */
size_t vsz_codebook_bytes(int dict_size);
size_t vsz_huff_head_max(int dict_size);
size_t vsz_huffman_build_tmp_bytes(int dict_size);
vsz_status vsz_huffman_build(const uint64_t* d_hist, int dict_size, void* d_codebook, uint8_t* d_huff_head,
                             uint32_t* d_info, void* d_tmp, size_t tmp_bytes, void* stream);

/* The same codebook and tree built on the calling host thread from a host histogram (host
 * pointers only): what vsz_compress runs inside its stream-ordered host step.  h_codebook:
 * [cb_word dict x u64][cb_len dict x u8]; h_huff_head: vsz_huff_head_max(dict) bytes.  Returns
 * VSZ_ERR_INVALID when no symbol occurs.  No counterpart in the reference (whose build is host
 * code inside Compress, src/vecsz_interface.hh:121-123). */
vsz_status vsz_huffman_build_host(const uint64_t* h_hist, int dict_size, void* h_codebook, uint8_t* h_huff_head,
                                  uint32_t h_info[4]);

/* Where vsz_compress builds the Huffman tree.  VSZ_TREE_HOST (the default): a kernel on the same
 * stream posts the histogram in pinned host memory, a library host thread builds the tree there,
 * and the kernel brings the codebook and tree back -- stream-ordered, no synchronisation of the
 * calling thread.  Streams under graph capture always use the device builder.  VSZ_TREE_DEVICE: the
 * one-CTA device builder (vsz_huffman_build).  The environment variable VSZ_TREE_BUILD=device
 * selects the device builder at load.  Process-wide; returns the previous setting (a negative
 * argument only queries). */
#define VSZ_TREE_DEVICE 1
#define VSZ_TREE_HOST 2
int vsz_set_tree_builder(int which);

/* Bit packing of codes with a codebook: the payload of HuffmanEncode (src/huffman.hh:268-341),
 * MSB-first codewords, ceil(bits / 8) bytes, written at d_payload (any alignment; the bytes of its
 * first 32-bit word before d_payload are preserved; 4 writable bytes past the end are needed).
 * *d_bits = payload length in bits; d_chunk_bits (optional): bits per 512 codes. */
size_t vsz_huffman_encode_tmp_bytes(size_t n);
vsz_status vsz_huffman_encode(const uint16_t* d_code, size_t n, const void* d_codebook, int dict_size,
                              uint8_t* d_payload, uint64_t* d_bits, uint16_t* d_chunk_bits, void* d_tmp,
                              size_t tmp_bytes, void* stream);

/* Decode n codes from a Huffman section [BE nodeCount][BE dict][tree][payload] (decode_withTree,
 * src/huffman.hh:679-691) without an index, by self-synchronising chunk decoding.  d_huff needs
 * 8 readable bytes past huff_bytes.  Synchronises (the synchronisation rounds are host-driven). */
size_t vsz_huffman_decode_tmp_bytes(size_t huff_bytes, size_t n, int dict_size);
vsz_status vsz_huffman_decode(const uint8_t* d_huff, size_t huff_bytes, size_t n, int dict_size, uint16_t* d_code,
                              void* d_tmp, size_t tmp_bytes, void* stream);

/* Reverse prediction-quantization: outlier placement + x_lorenzo_{1,2,3}d1l
 * (src/vecsz_interface.hh:313-354, src/dualquant.hh:915-1043).  d_outliers: the compact outlier
 * list (aligned), n_outlier entries. */
size_t vsz_dualquant_decompress_tmp_bytes(int ndim, const size_t dims[3]);
vsz_status vsz_dualquant_decompress(int ndim, const size_t dims[3], int block_size, int dict_size,
                                    const uint16_t* d_code, const float* d_outliers, uint64_t n_outlier,
                                    const void* d_consts, float* d_out, void* d_tmp, size_t tmp_bytes, void* stream);

/* =============================================================================================
 * Whole-field entry points (device buffers, stream-ordered, no host synchronisation):
 * the Compress / Decompress workflow of src/vecsz_interface.hh:31-229 and :232-375.
 * ============================================================================================= */

/* Workspace and archive capacity for one field. */
vsz_status vsz_compress_bounds(const vsz_params* p, int ndim, const size_t dims[3], size_t* ws_bytes,
                               size_t* archive_capacity);
/* Packed block (byte-identical to the reference's Compress output without -L) followed by this
 * library's trailer, into d_archive; 8 u64 of vsz_result into d_result (device memory). */
vsz_status vsz_compress(const vsz_params* p, int ndim, const size_t dims[3], const float* d_in, void* d_ws,
                        size_t ws_bytes, uint8_t* d_archive, size_t archive_capacity, uint64_t* d_result,
                        void* stream);

/* ---- many fields at once -------------------------------------------------------------------
 * A batch of fields of any shapes, dimensionalities, error bounds and dictionary sizes is
 * compressed in a handful of launches: each stage is one launch (one per kernel class for the
 * dual-quant stage) over a device-side table of per-field arguments and a list of block-wide
 * tasks, and the Huffman trees are built on the device, one CTA per field.  Every field's archive
 * and result are byte-identical to vsz_compress of that field alone.  No counterpart in the
 * reference, which compresses one field per process.
 *
 * vsz_batch_create lays out the caller's workspace (vsz_batch_workspace_bytes), resolves every
 * pointer and uploads the tables once (synchronous; it allocates the tables).  vsz_batch_compress
 * then only enqueues device work on `stream` -- memsets and launches, no host synchronisation and no
 * allocation -- so it may be captured in a CUDA graph and replayed; each replay recompresses the
 * current contents of the fields' input buffers.  d_results: 8 u64 (vsz_result) per field. */
typedef struct vsz_batch_field {
    const float* d_in;     /* device field */
    int ndim;
    size_t dims[3];
    vsz_params params;     /* lossless is ignored: the batch writes packed blocks */
    uint8_t* d_archive;    /* device output of at least vsz_compress_bounds' archive capacity */
    size_t archive_capacity;
} vsz_batch_field;
typedef struct vsz_batch vsz_batch;
vsz_status vsz_batch_workspace_bytes(const vsz_batch_field* fields, int nfields, size_t* ws_bytes);
vsz_status vsz_batch_create(const vsz_batch_field* fields, int nfields, void* d_ws, size_t ws_bytes,
                            uint64_t* d_results, vsz_batch** batch);
vsz_status vsz_batch_compress(vsz_batch* batch, void* stream);
void vsz_batch_destroy(vsz_batch* batch);
/* Work per block-wide task: dual-quant warp units (default 32) and encoder 512-code chunks
 * (default 64).  Rebuilds and uploads the task lists (synchronous): call before capturing
 * vsz_batch_compress in a graph.  vsz_batch_autotune times vsz_batch_compress over dual-quant sizes
 * {8, 16, 32, 64, 128}, then encoder sizes {16, 32, 64, 128, 256} (`iterations` timed runs each
 * after one warm-up, CUDA events on `stream`, synchronising), keeps the fastest pair and reports it;
 * the fields' archives are overwritten by the runs.  Archives do not depend on the task sizes. */
vsz_status vsz_batch_set_task_sizes(vsz_batch* batch, int dq_units, int enc_chunks);
vsz_status vsz_batch_autotune(vsz_batch* batch, int iterations, int* best_dq_units, int* best_enc_chunks,
                              void* stream);

/* ---- many archives at once: the batched decompress ----------------------------------------
 * Archives written by this library (packed block + trailer with the decode index), of any shapes,
 * dimensionalities, error bounds and dictionary sizes, decompressed in a handful of launches: the
 * Huffman tables one CTA per field in one launch, both index scans once over all fields' chunks,
 * decoding and the reverse Lorenzo over block-wide tasks of many fields per launch.  Every field's
 * output and status are the same as vsz_decompress of that archive alone.  Block size 8 without
 * padding and without strict mode only (VSZ_ERR_UNSUPPORTED otherwise; vsz_decompress takes the
 * rest).  No counterpart in the reference, which decompresses one field per process
 * (Decompress, src/vecsz_interface.hh:232-374).
 *
 * vsz_dbatch_create lays out the caller's workspace (vsz_dbatch_workspace_bytes) and uploads the
 * argument tables and task lists once (synchronous; it allocates them).  vsz_dbatch_decompress then
 * only enqueues device work on `stream` -- memsets and launches, no host synchronisation and no
 * allocation -- so it may be captured in a CUDA graph; each call decompresses the current contents
 * of the archives' device buffers, which must still parse as `desc` says.  d_status: one int per
 * field (device), the field's status after each call. */
typedef struct vsz_dbatch_field {
    const uint8_t* d_archive;  /* device archive bytes (16 readable bytes past its end) */
    vsz_archive_desc desc;     /* vsz_archive_parse of the same bytes */
    float* d_out;              /* device output: dims[0] * dims[1] * dims[2] floats */
} vsz_dbatch_field;
typedef struct vsz_dbatch vsz_dbatch;
vsz_status vsz_dbatch_workspace_bytes(const vsz_dbatch_field* fields, int nfields, size_t* ws_bytes);
vsz_status vsz_dbatch_create(const vsz_dbatch_field* fields, int nfields, void* d_ws, size_t ws_bytes, int* d_status,
                             vsz_dbatch** batch);
vsz_status vsz_dbatch_decompress(vsz_dbatch* batch, void* stream);
void vsz_dbatch_destroy(vsz_dbatch* batch);

/* GPU block-size autotuner (autotune_block_sizes, src/autotune.hh:80-96; the CLI's -a): times the
 * dual-quant kernel on a leading slab of the field (sample_percent of the slowest axis, at least 64
 * planes / rows, 64K elements in 1D) at block sizes 8, 16, 32 and 64, `iterations` runs each after
 * one warm-up, with CUDA events on `stream` (synchronising), and returns the fastest in
 * *best_block_size (timings_ms[4], optional: ms per run).  The block size changes the archive, as
 * with the reference's -a.  d_ws: vsz_autotune_workspace_bytes. */
vsz_status vsz_autotune_workspace_bytes(const vsz_params* p, int ndim, const size_t dims[3], double sample_percent,
                                        size_t* ws_bytes);
vsz_status vsz_autotune_block_size(const vsz_params* p, int ndim, const size_t dims[3], const float* d_in,
                                   double sample_percent, int iterations, void* d_ws, size_t ws_bytes,
                                   int* best_block_size, double timings_ms[4], void* stream);

/* Field autotuner, extending autotune_block_sizes (src/autotune.hh:22-126): the block size changes
 * the histogram, the tree, the encoder's and decoder's work and the archive's size, so each
 * candidate (8, 16, 32, 64) is timed through vsz_compress and vsz_decompress on the leading slab
 * (sample_percent of the slowest axis, at least 64 planes / rows, 64K elements in 1D), `iterations`
 * runs each after one warm-up (CUDA events on `stream`; synchronising), and scored by
 *     compress ms + decompress ms + archive bytes / (link_gbs GB/s)
 * -- the time to compress, move the archive over a link and decompress (link_gbs = 0: speed
 * alone).  The lowest score wins.  Results are cached process-wide per (dimensionality, size class
 * ceil(log2 elements), eb class floor(2 log10 eb), mode, dictionary, link rate, flags and
 * padding): a later field of the same class returns the cached result with cached = 1 and times
 * nothing.  d_ws: vsz_autotune_bounds bytes. */
typedef struct vsz_tune_result {
    int block_size;             /* the choice */
    int cached;                 /* 1: taken from the cache */
    uint64_t sample_elements;   /* elements of the slab timed */
    double compress_ms[4];      /* per candidate 8, 16, 32, 64: ms per run on the slab */
    double decompress_ms[4];
    uint64_t archive_bytes[4];  /* packed block bytes of the slab */
    double score_ms[4];
} vsz_tune_result;
vsz_status vsz_autotune_bounds(const vsz_params* p, int ndim, const size_t dims[3], double sample_percent,
                               size_t* ws_bytes);
vsz_status vsz_autotune(const vsz_params* p, int ndim, const size_t dims[3], const float* d_in, double sample_percent,
                        int iterations, double link_gbs, void* d_ws, size_t ws_bytes, vsz_tune_result* result,
                        void* stream);
void vsz_autotune_cache_clear(void);

/* The same search on a field in host memory (copied to the device first): what the command line's
 * -a runs. */
vsz_status vsz_autotune_block_size_host(const vsz_params* p, int ndim, const size_t dims[3], const float* h_in,
                                        double sample_percent, int iterations, int* best_block_size,
                                        double timings_ms[4]);

/* ---- request server ---------------------------------------------------------------------------
 * Continuous admission of compress / decompress requests under a device-memory budget, their work
 * overlapping on the device.  Requests queue in arrival order; a dispatcher thread admits the head
 * request as soon as one of `slots` streams is free and its workspace and output fit in the budget
 * (one device arena of budget_bytes, allocated at creation; admission never calls cudaMalloc).
 * The workspace returns to the arena when the request completes; the output (compress: the archive,
 * trimmed to its real size; decompress: the field) stays until vsz_server_release.  Results are
 * the same as vsz_compress / vsz_decompress of the request alone.  Decompress requests carry the
 * parsed archive (vsz_archive_parse); archives without this library's index synchronise their
 * slot's stream, which holds the dispatcher meanwhile.  No counterpart in the reference. */
#define VSZ_REQ_COMPRESS 0
#define VSZ_REQ_DECOMPRESS 1
typedef struct vsz_request {
    int kind;                  /* VSZ_REQ_COMPRESS | VSZ_REQ_DECOMPRESS */
    const void* d_in;          /* compress: device field; decompress: device archive (16 readable bytes past it) */
    int ndim;                  /* compress */
    size_t dims[3];            /* compress */
    vsz_params params;         /* compress (lossless ignored) */
    vsz_archive_desc desc;     /* decompress */
    vsz_decompress_opts opts;  /* decompress */
} vsz_request;
typedef struct vsz_completion {
    int status;                /* VSZ_OK or why the request failed */
    void* d_out;               /* device output inside the server's arena, valid until released */
    size_t out_bytes;          /* compress: packed block + trailer; decompress: 4 N */
    double t_submit, t_start, t_done;  /* host steady-clock seconds: queued, admitted, completed */
    uint64_t result[8];        /* compress: vsz_result */
} vsz_completion;
typedef struct vsz_server vsz_server;
vsz_status vsz_server_create(size_t budget_bytes, int slots, vsz_server** server);
/* Non-blocking; VSZ_ERR_CAPACITY when the request could never fit in the budget. */
vsz_status vsz_server_submit(vsz_server* server, const vsz_request* request, uint64_t* ticket);
/* Blocks until the request completed (VSZ_ERR_TIMEOUT after timeout_s).  VSZ_ERR_INVALID for an
 * unknown ticket, or when another thread releases the ticket while this one waits. */
vsz_status vsz_server_wait(vsz_server* server, uint64_t ticket, double timeout_s, vsz_completion* done);
/* Frees a completed request's output and forgets its ticket (VSZ_ERR_INVALID before completion). */
vsz_status vsz_server_release(vsz_server* server, uint64_t ticket);
/* Withdraws a request that is still queued: it completes at once with status VSZ_ERR_CANCELLED and
 * no output (wait returns it; release it as any other).  VSZ_ERR_UNSUPPORTED once the request has
 * been admitted (it runs to completion), VSZ_ERR_INVALID for an unknown ticket. */
vsz_status vsz_server_cancel(vsz_server* server, uint64_t ticket);
vsz_status vsz_server_stats(vsz_server* server, uint64_t* completed, uint64_t* input_bytes_completed,
                            size_t* arena_bytes_in_use, int* queued);
void vsz_server_destroy(vsz_server* server);

/* The same parse from the block's first head_len bytes (the header, the pad values and the Huffman
 * head) and the bytes from the block's end on (the trailer), for a block that lives on the device. */
vsz_status vsz_archive_parse_split(const uint8_t* head, size_t head_len, const uint8_t* tail, size_t tail_len,
                                   vsz_archive_desc* d);
/* Parse a packed block (+ optional trailer) held in host memory. */
vsz_status vsz_archive_parse(const uint8_t* h_archive, size_t len, vsz_archive_desc* desc);
vsz_status vsz_decompress_bounds(const vsz_archive_desc* desc, const vsz_decompress_opts* opts, size_t* ws_bytes);
/* Decompress a device-resident archive (d_archive needs 16 readable bytes past its end).
 * *d_status (device int, optional) receives VSZ_OK or the first device-side error.  Archives
 * without this library's trailer are decoded by self-synchronisation, which synchronises the
 * stream. */
vsz_status vsz_decompress(const vsz_archive_desc* desc, const vsz_decompress_opts* opts, const uint8_t* d_archive,
                          void* d_ws, size_t ws_bytes, float* d_out, int* d_status, void* stream);

/* =============================================================================================
 * Host entry points: the reference's interface, host buffers in and out, device memory managed
 * by the library (cached between calls).  Synchronous.
 * ============================================================================================= */

/* vecsz::interface::Compress<float,int> (src/vecsz_interface.hh:31): returns a malloc'd buffer
 * holding the packed block (or its lossless frame when p->lossless != NONE) followed by the
 * trailer.  *data_size, *lossless_size, *n_outlier as the reference reports them;
 * *out_bytes = total bytes in *h_out.  Free with vsz_free_host. */
vsz_status vsz_compress_host(const vsz_params* p, int ndim, const size_t dims[3], const float* h_in, uint8_t** h_out,
                             size_t* out_bytes, size_t* data_size, size_t* lossless_size, size_t* n_outlier);
/* Same, into a caller buffer (pinned memory gives full-speed copies); *out_bytes as above. */
vsz_status vsz_compress_host_into(const vsz_params* p, int ndim, const size_t dims[3], const float* h_in,
                                  uint8_t* h_out, size_t out_capacity, size_t* out_bytes, size_t* data_size,
                                  size_t* lossless_size, size_t* n_outlier);
/* Capacity vsz_compress_host_into needs for this field. */
vsz_status vsz_compress_host_bound(const vsz_params* p, int ndim, const size_t dims[3], size_t* out_capacity);

/* vecsz::interface::Decompress<float,int> (src/vecsz_interface.hh:232).  h_archive holds the
 * packed block (data_size bytes) or its lossless frame (lossless_size bytes, > 0), optionally
 * followed by this library's trailer; len = all bytes available.  *h_out malloc'd, *n floats. */
vsz_status vsz_decompress_host(const uint8_t* h_archive, size_t len, size_t data_size, size_t lossless_size,
                               const vsz_decompress_opts* opts, float** h_out, size_t* n);
/* Same, into a caller buffer of out_capacity floats. */
vsz_status vsz_decompress_host_into(const uint8_t* h_archive, size_t len, size_t data_size, size_t lossless_size,
                                    const vsz_decompress_opts* opts, float* h_out, size_t out_capacity, size_t* n);
void vsz_free_host(void* p);

/* Stream-ordered host-buffer operations.  A vsz_host_op owns a CUDA stream and device buffers
 * (grown on demand, kept between calls); its compress / decompress enqueue all their work and
 * return without synchronising, so several ops overlap their host<->device copies and kernels
 * (host-to-device and device-to-host copies run concurrently on the link).  Host buffers must be
 * pinned (cudaHostAlloc / cudaHostRegister).  No lossless pass (VSZ_ERR_UNSUPPORTED).
 *   compress:   h_in (n floats) -> h_out (the packed block and this library's trailer;
 *               out_capacity from vsz_compress_host_bound) and h_result (the 8-u64 vsz_result:
 *               data_size + trailer_size bytes of h_out are valid; status VSZ_ERR_CAPACITY when
 *               they did not fit).  The archive's size is known only on the device: a kernel
 *               copies exactly those bytes into h_out.  The Huffman tree is built on the device
 *               (as VSZ_TREE_DEVICE), whatever vsz_set_tree_builder says: these operations share
 *               the host link with other operations' field-sized transfers, which the host
 *               builder's small exchange would wait behind; the archive is the same.
 *   decompress: h_archive (len bytes, complete: the host parses its header) -> h_out (n floats),
 *               *h_status = VSZ_OK or the device-side error.
 *   wait:       blocks until the op's enqueued work is done; returns VSZ_ERR_CUDA if it failed. */
typedef struct vsz_host_op vsz_host_op;
vsz_status vsz_host_op_create(vsz_host_op** op);
void vsz_host_op_destroy(vsz_host_op* op);
vsz_status vsz_host_op_compress(vsz_host_op* op, const vsz_params* p, int ndim, const size_t dims[3], const float* h_in,
                                uint8_t* h_out, size_t out_capacity, uint64_t* h_result);
vsz_status vsz_host_op_decompress(vsz_host_op* op, const uint8_t* h_archive, size_t len,
                                  const vsz_decompress_opts* opts, float* h_out, size_t out_capacity, int* h_status);
vsz_status vsz_host_op_wait(vsz_host_op* op);

/* Lossless pass on host memory (src/lossless.hh:179-221): level 3 zstd or zlib through the
 * system libzstd / libz.  *h_out malloc'd.  VSZ_ERR_UNSUPPORTED when the library is absent. */
vsz_status vsz_lossless_compress(int which, const uint8_t* h_in, size_t len, uint8_t** h_out, size_t* out_len);
vsz_status vsz_lossless_decompress(const uint8_t* h_in, size_t len, size_t target, uint8_t** h_out, size_t* out_len);
/* 1 zstd frame, 2 zlib stream, 0 neither (is_lossless_compressed_data, src/lossless.hh:59-76). */
int vsz_lossless_detect(const uint8_t* h_in, size_t len);

/* The gzip pass on the device (replaces zlib_compress, src/lossless.hh:84-142, for -L gzip):
 * d_in[len] -> a zlib stream (RFC 1950 around RFC 1951 deflate) in d_out.  Chunks of
 * vsz_deflate_chunk_bytes() (16 KiB) are encoded independently (one CTA each: hash-chain match search, dynamic, fixed or stored block,
 * whichever is shortest, then an empty stored block so the next chunk starts on a byte).
 * d_result (device, 8 x u64): [0] stream bytes, [1] status (VSZ_ERR_CAPACITY when out_capacity is
 * too small), [2] chunks, [3] stored, [4] fixed, [5] dynamic chunks.  Stream-ordered, no sync. */
vsz_status vsz_deflate_bounds(size_t len, size_t* ws_bytes, size_t* out_capacity);
vsz_status vsz_deflate(const uint8_t* d_in, size_t len, void* d_ws, size_t ws_bytes, uint8_t* d_out,
                       size_t out_capacity, uint64_t* d_result, void* stream);
size_t vsz_deflate_chunk_bytes(void);
/* Compressed bytes of each chunk of the last vsz_deflate on this workspace (u32 per chunk,
 * host or device dst, stream-ordered): the deflate index the host entry points append after the
 * trailer of a VSZ_LOSSLESS_GZIP_DEVICE archive. */
vsz_status vsz_deflate_chunk_sizes(const void* d_ws, size_t len, uint32_t* dst, void* stream);

/* Inflate on the device for streams written by vsz_deflate (replaces zlib_uncompress,
 * src/lossless.hh:144-177, for them): chunk c (its compressed bytes at d_chunk_offsets[c] in the
 * stream, d_chunk_bytes[c] of them) inflates to d_out[vsz_deflate_chunk_bytes() * c ..], one warp
 * per chunk; the
 * Adler-32 of the output is checked against adler32.  *d_status (device int) = VSZ_ERR_CORRUPT for
 * anything that is not such a stream; reads and writes stay inside the given buffers. */
vsz_status vsz_inflate_bounds(size_t n_chunks, size_t* ws_bytes);
vsz_status vsz_inflate(const uint8_t* d_stream, size_t stream_len, const unsigned long long* d_chunk_offsets,
                       const uint32_t* d_chunk_bytes, size_t n_chunks, uint32_t adler32, uint8_t* d_out,
                       size_t out_len, void* d_ws, size_t ws_bytes, int* d_status, void* stream);

/* Per-stage device timing: when enabled, the whole-field entry points record a CUDA event pair
 * around each stage on the launching stream.  vsz_profile_read synchronises, returns the number of
 * stages and fills ms[i] (milliseconds summed over all calls since the last reset), counts[i]
 * (recorded launches) and names[i] (static strings).  No counterpart in the reference, which
 * prints wall-clock stage times instead (src/vecsz_interface.hh:107-175). */
void vsz_profile_enable(int on);
void vsz_profile_reset(void);
int vsz_profile_read(double* ms, int* counts, const char** names, int max_stages);

/* Kernels this library has launched in this process, all entry points and devices together (a
 * relaxed atomic count taken at each launch).  No counterpart in the reference. */
uint64_t vsz_launch_count(void);

/* ---- f64 fields ----------------------------------------------------------------------------
 * The reference parses -t f64 (src/argument_parser/argparse.cc:454-462) but reads its input as
 * float (src/vecsz.cc:32) and its dual-quant loops are float AVX code (src/dualquant.hh:86-92), so
 * it has no f64 arithmetic to match.  These entry points run the same pipeline in double precision
 * with the error bound guaranteed, as the strict mode does for f32: prequantized values
 * s = rint(x / 2eb) are exact integers, the Lorenzo predictor is integer arithmetic, an element
 * keeps its code only if s * 2eb is within eb of x (and |x / 2eb| < 2^59), and every other element
 * is an outlier stored as its 8-byte input value.  So |x - xhat| <= eb everywhere (checked in
 * double), outliers (NaN and infinities included) come back bit for bit.  abs and r2r modes,
 * dictionaries and block sizes as for f32; no padding (VSZ_ERR_UNSUPPORTED).  The archive is the
 * packed-block layout with 8-byte outliers, counted as two 32-bit words in the header's outlier
 * count, and the trailer marks it (vsz_archive_desc.f64); vsz_decompress refuses it and
 * vsz_decompress_f64 takes only it.  Device entry points are stream-ordered as vsz_compress /
 * vsz_decompress; the host ones allocate device memory per call and synchronise (-L zstd / gzip
 * through the host library, the trailer after the frame). */
vsz_status vsz_compress_f64_bounds(const vsz_params* p, int ndim, const size_t dims[3], size_t* ws_bytes,
                                   size_t* archive_capacity);
vsz_status vsz_compress_f64(const vsz_params* p, int ndim, const size_t dims[3], const double* d_in, void* d_ws,
                            size_t ws_bytes, uint8_t* d_archive, size_t archive_capacity, uint64_t* d_result,
                            void* stream);
vsz_status vsz_decompress_f64_bounds(const vsz_archive_desc* desc, size_t* ws_bytes);
vsz_status vsz_decompress_f64(const vsz_archive_desc* desc, const uint8_t* d_archive, void* d_ws, size_t ws_bytes,
                              double* d_out, int* d_status, void* stream);
vsz_status vsz_compress_host_f64(const vsz_params* p, int ndim, const size_t dims[3], const double* h_in,
                                 uint8_t** h_out, size_t* out_bytes, size_t* data_size, size_t* lossless_size,
                                 size_t* n_outlier);
vsz_status vsz_decompress_host_f64(const uint8_t* h_archive, size_t len, size_t data_size, size_t lossless_size,
                                   double** h_out, size_t* n);

/* ---- test hooks: no counterpart in the reference ---------------------------------------------
 * Every cross-CTA wait of this library (the decoupled look-back of the outlier gather, the
 * encoder's chunk scan and the device-wide scans) polls at most a bounded number of times, then
 * records VSZ_ERR_TIMEOUT in the call's status word and returns instead of hanging.
 * vsz_debug_set_spin_limit sets that bound for every kernel of the library (polls <= 0: the
 * default, 2^22); process-wide, synchronous.  vsz_debug_scan_stalled_predecessor runs the
 * device-wide scan over n (<= 2^24) values with its tile ticket started past tile 0, so one tile
 * waits on a predecessor that never publishes; it allocates, synchronises and stores the scan's
 * status word (VSZ_ERR_TIMEOUT when the wait ran out) in *h_status. */
vsz_status vsz_debug_set_spin_limit(long long polls);
vsz_status vsz_debug_scan_stalled_predecessor(size_t n, int* h_status);

/* The host tree build of vsz_compress is a handoff: a kernel posts the histogram in pinned memory
 * and waits for a host worker thread's answer, at most a bounded time (2 s), then records
 * VSZ_ERR_TIMEOUT in the call's status word and returns.  vsz_debug_tree_hold(1) makes the worker
 * leave new requests unanswered (0: answer them again, the held ones too);
 * vsz_debug_set_tree_wait_ns sets the kernel's bound for later calls (ns <= 0: the default). */
vsz_status vsz_debug_tree_hold(int hold);
vsz_status vsz_debug_set_tree_wait_ns(long long ns);

/* Three environment variables, read by vsz_decompress on every call, make it take another of its
 * kernels for the same result, so that tests can compare the kernels on one archive:
 * VSZ_DECODE_NO_WINDOW (set: the general indexed decoder instead of the window decoder),
 * VSZ_FORCE_GENERAL_DECOMPRESS (set: the per-block-row reverse Lorenzo for block size 8 instead of
 * the block-8 kernels) and VSZ_DQ_NO_WAVEFRONT (set: the block-8 kernels also for 3D fields of at
 * most 2^24 elements, which otherwise take the wavefront kernel).  Unset, the library picks its
 * fastest exact kernel. */

#ifdef __cplusplus
}
#endif

#endif /* VECSZ_GB300_H */
