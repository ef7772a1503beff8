// Internal interface of the Huffman kernels (huffman.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "vsz_kernels.h"
#include "vsz_types.h"

namespace vsz {

constexpr int kDecBits     = 12;   // primary decode table: 4096 entries
constexpr int kDec2Max     = 8;    // widest secondary table: codewords of up to 20 bits in two lookups

// Decode table entries (k_huff_table).  Primary table, indexed by the next kDecBits bits:
//   (sym << 8) | len           len in 1..kDecBits: a whole codeword
//   (off << 12) | (w2 << 8) | 0x80   a longer codeword: index table2[off + next w2 bits]
//   (node << 8)                walk the tree bit by bit from `node` after kDecBits bits
// Secondary table2 entries: (sym << 8) | total length, or (node << 8) to walk from `node` after
// kDecBits + w2 bits (codewords longer than kDecBits + kDec2Max).  A zero entry is not a codeword.
// Capacity: every secondary table hangs off a distinct internal node at depth kDecBits, and one
// with L leaves below it is at most 2^min(kDec2Max, L - 1) entries wide (a subtree of depth D has
// at least D + 1 leaves), so a tree of `leaves` leaves needs at most 256 / 9 entries per leaf.
// k_huff_table leaves the walk entries in place of secondary tables that would not fit.
__host__ __device__ inline size_t table2_capacity(uint32_t max_nodes) {
    const size_t leaves = ((size_t)max_nodes + 1) / 2;
    return ((size_t)(1u << kDec2Max) * leaves + 8) / 9 + 256;
}
constexpr int kChunkSyms   = 512;  // codewords per entry of this library's decode index
constexpr int kSyncBits    = 8192; // chunk size (bits) of the self-synchronising decoder

// Width of the serialized child indices (src/huffman.hh:425-502).
__host__ __device__ inline int tree_index_width(uint32_t nc) { return nc <= 256 ? 1 : (nc <= 65536 ? 2 : 4); }
// [u8 endian][L][R][C u32][t u8]
__host__ __device__ inline size_t tree_bytes_size(uint32_t nc) {
    int w = tree_index_width(nc);
    return 1 + 2 * (size_t)w * nc + 4 * (size_t)nc + nc;
}

struct HuffBuildArgs {
    const unsigned long long* hist;
    int dict;                     // symbols [0, dict) (a 1D padded field adds one: 2 * radius)
    int hdr_dict;                 // dictionary size written into the head; 0: dict
    unsigned long long* cb_word;  // right-aligned codeword per symbol
    uint8_t* cb_len;              // codeword length per symbol (0 = unused)
    uint8_t* out;                 // [BE nc][BE dict][tree bytes], any alignment
    uint32_t* info;               // [0] node count [1] tree bytes [2] max code length [3] nodes created
    void* scratch;                // huff_build_scratch_bytes(dict), used when shared memory is too small
    int ws_in_smem;
    int* status;
};

struct HuffEncodeArgs {
    const uint16_t* codes;
    size_t n;
    const unsigned long long* cb_word;
    const uint8_t* cb_len;
    int dict;
    uint8_t* out;                     // payload start = out + out_off.eval(), any alignment;
    DevOffset out_off;                // bytes before the payload start are kept
    unsigned long long* total_bits;
    uint16_t* chunk_bits;             // nchunks: bits per 512 codes (scan input; the decode index)
    unsigned long long* chunk_off;    // nchunks: first bit of each chunk
    unsigned long long* scan_status;  // scan scratch: scan_tmp_tiles(nchunks) + 1
    uint32_t* scan_counter;
    unsigned long long* edge_idx;     // 2 nchunks: word index of a chunk's partial first / last word
    uint32_t* edge_bits;              // 2 nchunks: its bits (stored byte order)
    int* status;
    size_t nchunks;
    int codes_aligned;
    int cb_in_smem;
    const uint32_t* build_info;       // optional: the tree's info; max length > 64 is refused
};

struct HuffTableArgs {
    const uint8_t* huff;  // [BE nc][BE dict][tree bytes]...
    size_t huff_bytes;
    int dict;
    uint32_t max_nodes;
    uint32_t* table;      // 1 << kDecBits entries
    uint32_t* child;      // 2 * max_nodes
    uint32_t* node_sym;   // max_nodes: 0x80000000 | symbol for leaves
    uint32_t* parent;     // max_nodes (scratch)
    uint32_t* walk;       // max_nodes: both children of an internal node, 16 bits each:
                          // 0x8000 | symbol for a leaf, else the node index (dict <= 16384)
    uint32_t* table2;     // table2_capacity(max_nodes) secondary entries
    uint32_t* info;       // [0] single-symbol tree flag [1] its symbol [2] longest codeword (255: > 64)
    int* status;
};

struct HuffDecodeArgs {
    const uint8_t* payload;  // any alignment; 8 readable bytes past the end are required
    unsigned long long payload_bits;
    const uint32_t* table;
    const uint32_t* table2;
    const uint32_t* child;
    const uint32_t* node_sym;
    const uint32_t* walk;                 // packed children (k_huff_table), when walk_smem
    int walk_smem;                        // 1: dict <= 16384, the walk array is copied to shared memory
    uint32_t nodes;                       // node count of the tree
    const unsigned long long* start_bit;  // per chunk, relative to start_bit[0] (indexed path)
    const uint16_t* chunk_len;            // indexed path: bits of each chunk
    uint32_t* chunk_zero;                 // indexed path: zero codes per chunk (may be null)
    const unsigned long long* out_begin;  // per chunk, or null: chunk * chunk_syms
    const uint32_t* nsym;                 // per chunk, or null: chunk_syms
    size_t nchunks;
    uint32_t chunk_syms;
    uint16_t* codes;
    size_t n;
    uint32_t* seg_zero;                   // zero codes per 256-wide row segment (may be null)
    uint32_t d0, nxs;
    uint32_t max_nodes;                   // node indices past this are a corrupt tree
    const uint32_t* tree_info;            // k_huff_table's info ([2] longest codeword), or null
    int* status;
};

struct HuffSyncArgs {
    const uint8_t* payload;
    unsigned long long payload_bits;
    const uint32_t* table;
    const uint32_t* table2;
    const uint32_t* child;
    const uint32_t* node_sym;
    size_t nchunks;
    uint32_t chunk_bits;
    unsigned long long* start;   // nchunks
    unsigned long long* exit_a;  // nchunks
    uint32_t* count;             // nchunks
    uint32_t max_nodes;
    int* status;
};

int launch_huff_build(HuffBuildArgs a, cudaStream_t st);
// Batches: one CTA per field; in_smem for every field when huff_build_in_smem(dict) (the others
// need HuffBuildArgs::scratch).  Encode: tasks of (field, 512-code chunk range); all fields' chunk
// bits are scanned at once (all_bits / all_off hold total_chunks + 1 entries, the fields' ranges
// in field order; each field's chunk_bits / chunk_off point into them).
bool huff_build_in_smem(int dict);
int launch_huff_build_batch(const HuffBuildArgs* args, uint32_t nfields, bool in_smem, int dict_max, cudaStream_t st,
                            int num_sms);
int launch_huff_encode_batch(const HuffEncodeArgs* args, uint32_t nfields, const BatchTask* tasks, uint32_t ntasks,
                             int cb_dict_max, uint16_t* all_bits, unsigned long long* all_off, size_t total_chunks,
                             unsigned long long* scan_status, uint32_t* scan_counter, int* batch_status,
                             cudaStream_t st, int num_sms);
void huff_encode_prepare(HuffEncodeArgs& a);
void huff_build_prepare();  // one-time kernel attributes of launch_huff_build (call outside capture)
size_t huff_build_scratch_bytes(int dict);
int launch_huff_encode(HuffEncodeArgs a, cudaStream_t st, int num_sms);
int launch_huff_table(HuffTableArgs a, cudaStream_t st);
// Many fields: decode tables one CTA per field; decoding over tasks of (field, 256-chunk range
// of the field's index), every field's tree by the decoder of its kind (the window decoder for
// codewords up to 32 bits, the general one beyond), and const_tasks (one-symbol trees) by a
// constant fill.
int launch_huff_table_batch(const HuffTableArgs* args, uint32_t nfields, cudaStream_t st, int num_sms);
int launch_huff_decode_batch(const HuffDecodeArgs* args, const BatchTask* tasks, uint32_t ntasks,
                             const BatchTask* const_tasks, uint32_t nconst, cudaStream_t st, int num_sms);
int launch_huff_decode(HuffDecodeArgs a, cudaStream_t st);
int launch_huff_const(uint16_t* codes, size_t n, const uint32_t* info, uint32_t* seg_zero, uint32_t d0, uint32_t nxs,
                      const int* status, cudaStream_t st, int num_sms);
int launch_huff_sync_init(HuffSyncArgs a, cudaStream_t st);
int launch_huff_sync_round(HuffSyncArgs a, const unsigned long long* exit_in, unsigned long long* exit_out,
                           int* changed, cudaStream_t st);
int launch_scan_u16(const uint16_t* in, unsigned long long* out, size_t n, unsigned long long* tile_status,
                    uint32_t* tile_counter, unsigned long long* total, int* status, cudaStream_t st);
int launch_scan_u32(const uint32_t* in, unsigned long long* out, size_t n, unsigned long long* tile_status,
                    uint32_t* tile_counter, unsigned long long* total, int* status, cudaStream_t st);
size_t scan_tmp_tiles(size_t n);
// Test hooks (vsz_debug_*): this unit's look-back spin limit; a scan whose first tile never runs.
int set_spin_limit_huffman(long long polls);
int debug_scan_stalled(size_t n, int* status_out);

}  // namespace vsz
