// Tree-Huffman coding of quant codes on sm_103a, bit-compatible with vecSZ's src/huffman.hh.
//
//   k_huff_build    initHuffman heap build + build_code + convert_HuffTree_to_bytes_anyStates
//                   (src/huffman.hh:169-266, 374-502): exact replay of the reference's heap, one
//                   thread, then the serialized tree and the codebook written by the whole CTA.
//   k_huff_encode   HuffmanEncode (src/huffman.hh:268-341): persistent CTAs, 4096 codes per tile,
//                   bit offsets from a block scan plus decoupled look-back, codewords packed into a
//                   shared-memory word buffer and stored MSB-first into the payload.
//   k_huff_table    reconstruct_HuffTree_from_bytes_anyStates (src/huffman.hh:561-635): 12-bit
//                   lookup table plus a child array for longer codes.
//   k_huff_decode   decode (src/huffman.hh:343-372): one thread per chunk of codewords whose first
//                   bit is known (from this library's chunk index, or found by self-synchronising
//                   rounds k_huff_sync_* for archives written by the reference).
#include <cstdint>
#include <cstdlib>

#include "scan.cuh"
#include "vsz_device.cuh"
#include "vsz_huffman.h"
#include "vsz_profile.h"

namespace vsz {

// ------------------------------------------------------------------------------------------
// K2: heap-tree build
// ------------------------------------------------------------------------------------------

constexpr int kKeyShift = 20;  // heap key = freq << 20 | node  (node < 2^20, freq < 2^44)
constexpr uint32_t kNodeMask = (1u << kKeyShift) - 1u;

__device__ __forceinline__ unsigned long long kfreq(unsigned long long k) { return k >> kKeyShift; }

// Working set of the tree build (shared memory when it fits, else the global scratch).
struct BuildWs {
    unsigned long long* heap;  // 2 dict + 8 (room for speculative reads below the heap end)
    uint32_t* used;            // dict: symbol of leaf i
    int32_t* lchild;           // dict: children of internal node k (node nused + k)
    int32_t* rchild;
    uint32_t* size;            // 2 dict: subtree sizes
    uint32_t* pre;             // 2 dict: preorder index (pad_tree_* numbering)
    unsigned long long* code;  // 2 dict: codeword, right-aligned
    uint32_t* depth;           // 2 dict
};

__host__ __device__ inline size_t build_ws_bytes(int dict) {
    size_t d = (size_t)dict;
    return 8 * (2 * d + 8) + 4 * d + 8 * d + 4 * 2 * d * 2 + 8 * 2 * d + 4 * 2 * d + 256;
}

__device__ inline BuildWs carve_build_ws(uint8_t* p, int dict) {
    size_t d = (size_t)dict;
    BuildWs w;
    w.heap   = reinterpret_cast<unsigned long long*>(p);
    p += 8 * (2 * d + 8);
    w.code   = reinterpret_cast<unsigned long long*>(p);
    p += 8 * 2 * d;
    w.used   = reinterpret_cast<uint32_t*>(p);
    p += 4 * d;
    w.lchild = reinterpret_cast<int32_t*>(p);
    p += 4 * d;
    w.rchild = reinterpret_cast<int32_t*>(p);
    p += 4 * d;
    w.size   = reinterpret_cast<uint32_t*>(p);
    p += 4 * 2 * d;
    w.pre    = reinterpret_cast<uint32_t*>(p);
    p += 4 * 2 * d;
    w.depth  = reinterpret_cast<uint32_t*>(p);
    return w;
}

// Heap key layouts: freq in the high bits, node in the low bits.  K32: 32 | 32 (histogram total
// below 2^32, the usual case: the frequency is the high register, one 32-bit compare); otherwise
// 44 | 20.  Only the frequency part is ever compared, as in the reference.
template <bool K32>
struct HeapKey {
    static __device__ __forceinline__ unsigned long long fq(unsigned long long k) {
        return K32 ? (unsigned long long)(uint32_t)(k >> 32) : (k >> kKeyShift);
    }
    static __device__ __forceinline__ unsigned long long make(unsigned long long f, uint32_t node) {
        return K32 ? ((f << 32) | node) : ((f << kKeyShift) | node);
    }
    static __device__ __forceinline__ uint32_t node(unsigned long long k) {
        return K32 ? (uint32_t)k : (uint32_t)(k & kNodeMask);
    }
};

// The reference's heap, operation for operation (src/huffman.hh:169-192, 248-262).  Returns the
// number of nodes created.
template <bool K32>
__device__ __forceinline__ int heap_replay(BuildWs& w, int nused, int* fail) {
    using K  = HeapKey<K32>;
    int qend = 1;
    for (int i = 0; i < nused; i++) {  // leaves: qinsert(new_node(freq, i)) in symbol order
        const unsigned long long key = K::make(w.code[i], (uint32_t)i);
        const unsigned long long fk  = K::fq(key);
        int ii = qend++, j;
        while ((j = ii >> 1)) {
            const unsigned long long pj = w.heap[j];
            if (K::fq(pj) <= fk) break;
            w.heap[ii] = pj;
            ii         = j;
        }
        w.heap[ii] = key;
    }
    int nnodes = nused;
    // merges: new_node(.., qremove(), qremove()) -- the first removal is the RIGHT child
    while (qend > 2) {
        unsigned long long rem[2];
#pragma unroll
        for (int r = 0; r < 2; r++) {
            // qremove: the hole sinks along the smaller child (ties: left) to the bottom, then takes
            // the last element, without sifting it up.  Children of both candidates are loaded one
            // level ahead.
            const unsigned long long top = w.heap[1];
            qend--;
            const unsigned long long last = w.heap[qend];
            int i = 1, l = 2;
            ulonglong2 pr = *reinterpret_cast<const ulonglong2*>(&w.heap[2]);
            while (l < qend) {
                const ulonglong2 ga = *reinterpret_cast<const ulonglong2*>(&w.heap[2 * l]);
                const ulonglong2 gb = *reinterpret_cast<const ulonglong2*>(&w.heap[2 * l + 2]);
                const bool right    = (l + 1 < qend) && (K::fq(pr.y) < K::fq(pr.x));
                w.heap[i] = right ? pr.y : pr.x;
                i         = right ? l + 1 : l;
                l         = 2 * i;
                pr        = right ? gb : ga;
            }
            w.heap[i] = last;
            rem[r]    = top;
        }
        const int k = nnodes - nused;
        nnodes++;
        w.rchild[k] = (int32_t)K::node(rem[0]);
        w.lchild[k] = (int32_t)K::node(rem[1]);
        const unsigned long long key = K::make(K::fq(rem[0]) + K::fq(rem[1]), (uint32_t)(nused + k));
        const unsigned long long fk  = K::fq(key);
        int ii = qend++, j;
        while ((j = ii >> 1)) {
            const unsigned long long pj = w.heap[j];
            if (K::fq(pj) <= fk) break;
            w.heap[ii] = pj;
            ii         = j;
        }
        w.heap[ii] = key;
    }
    (void)fail;
    return nnodes;
}

template <bool IN_SMEM>
__device__ __forceinline__ void build_field(const HuffBuildArgs& a, uint8_t* s_build_dyn) {
    __shared__ uint32_t s_info[4];
    __shared__ int s_fail;
    __shared__ uint32_t s_scan[33];
    __shared__ unsigned long long s_fsum[8];
    if (*a.status != VSZ_OK) return;  // an earlier stage failed (uniform: one CTA)
    const int dict = a.dict;
    BuildWs w      = carve_build_ws(IN_SMEM ? s_build_dyn : reinterpret_cast<uint8_t*>(a.scratch), dict);
    if (threadIdx.x == 0) s_fail = 0;
    for (int i = threadIdx.x; i < 2 * dict + 8; i += blockDim.x) w.heap[i] = 0ull;
    for (int i = threadIdx.x; i < dict; i += blockDim.x) {
        a.cb_word[i] = 0ull;
        a.cb_len[i]  = 0;
    }
    // ---- used symbols in symbol order (src/huffman.hh:248-254), block-wide compaction
    const int per = (dict + blockDim.x - 1) / blockDim.x;
    const int s0  = threadIdx.x * per;
    uint32_t cnt  = 0;
    unsigned long long fsum = 0;
    for (int k = 0; k < per; k++) {
        int sym = s0 + k;
        if (sym < dict) {
            unsigned long long f = a.hist[sym];
            cnt += (f != 0ull);
            fsum += f;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
    if ((threadIdx.x & 31) == 0) s_fsum[threadIdx.x >> 5] = fsum;
    uint32_t tot;
    uint32_t off = block_exclusive_scan<uint32_t>(cnt, s_scan, &tot);
    for (int k = 0; k < per; k++) {
        int sym = s0 + k;
        if (sym < dict) {
            unsigned long long f = a.hist[sym];
            if (f != 0ull) {
                w.used[off]   = (uint32_t)sym;
                w.code[off++] = f;  // leaf frequencies, until the codewords are computed
            }
        }
    }
    __syncthreads();
    const int nused = (int)tot;

    if (threadIdx.x == 0) {
        unsigned long long total = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) total += s_fsum[i];
        int nnodes = nused;
        if (nused == 0) s_fail = VSZ_ERR_INVALID;
        else if (total >= (1ull << (64 - kKeyShift))) s_fail = VSZ_ERR_UNSUPPORTED;
        else if (total < (1ull << 32)) nnodes = heap_replay<true>(w, nused, &s_fail);
        else nnodes = heap_replay<false>(w, nused, &s_fail);
        uint32_t node_count = 0, max_len = 0;
        if (!s_fail) {
            const int nint = nnodes - nused;
            // subtree sizes bottom-up (children are always created before their parent)
            for (int i = 0; i < nused; i++) w.size[i] = 1u;
            for (int k = 0; k < nint; k++) w.size[nused + k] = 1u + w.size[w.lchild[k]] + w.size[w.rchild[k]];
            // root = the last node created (a one-leaf tree: the leaf); preorder numbering of
            // pad_tree_* (src/huffman.hh:374-423) and codewords of build_code (:200-227) top-down
            const int root = nnodes - 1;
            w.pre[root]   = 0u;
            w.code[root]  = 0ull;
            w.depth[root] = 0u;
            for (int k = nint - 1; k >= 0; k--) {
                const int v = nused + k, l = w.lchild[k], r = w.rchild[k];
                const uint32_t pv = w.pre[v], dv = w.depth[v] + 1u;
                const unsigned long long cv = w.code[v] << 1;
                w.pre[l]   = pv + 1u;
                w.pre[r]   = pv + 1u + w.size[l];
                w.code[l]  = cv;
                w.code[r]  = cv | 1ull;
                w.depth[l] = dv;
                w.depth[r] = dv;
                if (dv > max_len) max_len = dv;
            }
            node_count = (uint32_t)nnodes;
        }
        s_info[0] = node_count;
        s_info[1] = (uint32_t)tree_bytes_size(node_count);
        s_info[2] = max_len;
        s_info[3] = (uint32_t)nnodes;
    }
    __syncthreads();
    if (s_fail) {
        if (threadIdx.x == 0) set_status(a.status, s_fail);
        return;
    }
    const uint32_t nc = s_info[0];
    const int nused_c = nused;
    const int wdt     = tree_index_width(nc);
    // [BE nodeCount][BE dict][u8 0][L][R][C u32 LE][t]  (src/huffman.hh:649-653, 438-444)
    uint8_t* o = a.out;
    if (threadIdx.x == 0) {
        o[0] = (uint8_t)(nc >> 24);
        o[1] = (uint8_t)(nc >> 16);
        o[2] = (uint8_t)(nc >> 8);
        o[3] = (uint8_t)nc;
        uint32_t dh = (uint32_t)(a.hdr_dict ? a.hdr_dict : dict);
        o[4] = (uint8_t)(dh >> 24);
        o[5] = (uint8_t)(dh >> 16);
        o[6] = (uint8_t)(dh >> 8);
        o[7] = (uint8_t)dh;
        o[8] = 0;
    }
    uint8_t* pL = o + 9;
    uint8_t* pR = pL + (size_t)wdt * nc;
    uint8_t* pC = pR + (size_t)wdt * nc;
    uint8_t* pT = pC + 4 * (size_t)nc;
    for (uint32_t v = threadIdx.x; v < nc; v += blockDim.x) {
        const uint32_t idx = w.pre[v];
        const bool leaf    = (int)v < nused_c;
        uint32_t l = 0, r = 0, c = 0;
        if (leaf) {
            c = w.used[v];
            a.cb_len[c]  = (uint8_t)(w.depth[v] > 255u ? 255u : w.depth[v]);
            a.cb_word[c] = w.code[v];
        } else {
            l = w.pre[w.lchild[v - nused_c]];
            r = w.pre[w.rchild[v - nused_c]];
        }
        for (int b = 0; b < wdt; b++) {
            pL[(size_t)idx * wdt + b] = (uint8_t)(l >> (8 * b));
            pR[(size_t)idx * wdt + b] = (uint8_t)(r >> (8 * b));
        }
        pC[4 * (size_t)idx + 0] = (uint8_t)c;
        pC[4 * (size_t)idx + 1] = (uint8_t)(c >> 8);
        pC[4 * (size_t)idx + 2] = (uint8_t)(c >> 16);
        pC[4 * (size_t)idx + 3] = (uint8_t)(c >> 24);
        pT[idx]                 = leaf ? 1 : 0;
    }
    if (threadIdx.x < 4) a.info[threadIdx.x] = s_info[threadIdx.x];
}

template <bool IN_SMEM>
__global__ void __launch_bounds__(256) k_huff_build(HuffBuildArgs a) {
    extern __shared__ __align__(16) uint8_t s_build_dyn[];
    build_field<IN_SMEM>(a, s_build_dyn);
}

// Many fields: one CTA per field (grid-stride).
template <bool IN_SMEM>
__global__ void __launch_bounds__(256) k_huff_build_batch(const HuffBuildArgs* __restrict__ args, uint32_t nfields) {
    extern __shared__ __align__(16) uint8_t s_build_dyn[];
    for (uint32_t f = blockIdx.x; f < nfields; f += gridDim.x) {
        build_field<IN_SMEM>(args[f], s_build_dyn);
        __syncthreads();
    }
}

int launch_scan_u32(const uint32_t* in, unsigned long long* out, size_t n, unsigned long long* tile_status,
                    uint32_t* tile_counter, unsigned long long* total, int* status, cudaStream_t st);

// ------------------------------------------------------------------------------------------
// K3: encoder, two passes over the codes with no cross-warp waiting.  The unit is a chunk of 512
// codes -- one warp, 16 codes per lane -- the same chunk the decode index records:
//   k_huff_count  bits per chunk (chunk_bits, also the archive's decode index)
//   k_scan_excl   exclusive scan of chunk_bits -> each chunk's first bit, total bits
//   k_huff_pack   per chunk: warp scan of lane bit counts, codewords packed into the warp's
//                 shared-memory word buffer, interior words stored, the partial first and last
//                 words left to k_huff_encode_edges.  No block-wide barriers; the next chunk's
//                 codes are loaded while the current one is packed.
// ------------------------------------------------------------------------------------------

constexpr int kEncThreads   = 256;
constexpr int kEncPerThread = 16;
constexpr int kEncChunk     = 32 * kEncPerThread;        // 512 codes per warp chunk (= kChunkSyms)
constexpr int kEncWarpWords = kEncChunk * 64 / 32 + 4;   // codes are at most 64 bits
static_assert(kEncChunk == kChunkSyms, "the encoder chunk is the decode index chunk");

// Raw 16 codes of one lane (two 16-byte loads when aligned and whole) and how many are valid.
struct Codes16 {
    uint4 v0, v1;
    uint32_t nvalid;
};

__device__ __forceinline__ Codes16 load_codes16(const HuffEncodeArgs& a, size_t c0) {
    Codes16 r;
    r.nvalid = c0 >= a.n ? 0u : (uint32_t)min((size_t)kEncPerThread, a.n - c0);
    if (r.nvalid == (uint32_t)kEncPerThread && a.codes_aligned) {
        const uint4* p = reinterpret_cast<const uint4*>(a.codes + c0);
        r.v0 = __ldcs(p);
        r.v1 = __ldcs(p + 1);
    } else {
        uint32_t t[kEncPerThread];
#pragma unroll
        for (int k = 0; k < kEncPerThread; k++) t[k] = ((uint32_t)k < r.nvalid) ? a.codes[c0 + k] : 0u;
        r.v0 = make_uint4(t[0] | (t[1] << 16), t[2] | (t[3] << 16), t[4] | (t[5] << 16), t[6] | (t[7] << 16));
        r.v1 = make_uint4(t[8] | (t[9] << 16), t[10] | (t[11] << 16), t[12] | (t[13] << 16), t[14] | (t[15] << 16));
    }
    return r;
}

__device__ __forceinline__ uint32_t code_k(const Codes16& c, int k) {
    const uint32_t w8[8] = {c.v0.x, c.v0.y, c.v0.z, c.v0.w, c.v1.x, c.v1.y, c.v1.z, c.v1.w};
    return (w8[k >> 1] >> (16 * (k & 1))) & 0xffffu;
}

// Refuses a tree the encoder cannot pack (no tree, or codewords longer than 64 bits).
__device__ __forceinline__ bool encode_tree_ok(const HuffEncodeArgs& a) {
    if (a.build_info && (a.build_info[2] > 64u || a.build_info[0] == 0u)) {
        if (threadIdx.x == 0 && blockIdx.x == 0)
            set_status(a.status, a.build_info[0] ? VSZ_ERR_UNSUPPORTED : VSZ_ERR_INVALID);
        return false;
    }
    return true;
}

// Bits of chunks c, c + cstep, ... < c1 of one field (one warp per chunk).
__device__ __forceinline__ void count_chunks(const HuffEncodeArgs& a, size_t c, size_t c1, size_t cstep,
                                             uint8_t* s_len_dyn) {
    const uint8_t* cl = a.cb_len;
    if (a.cb_in_smem) {
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x) s_len_dyn[i] = a.cb_len[i];
        __syncthreads();
        cl = s_len_dyn;
    }
    const unsigned lane = threadIdx.x & 31u;
    for (; c < c1; c += cstep) {
        const Codes16 cc = load_codes16(a, c * kEncChunk + lane * kEncPerThread);
        uint32_t bits    = 0;
        if (cc.nvalid == (uint32_t)kEncPerThread) {  // all but the field's last lanes
#pragma unroll
            for (int k = 0; k < kEncPerThread; k++) bits += cl[code_k(cc, k)];
        } else {
#pragma unroll
            for (int k = 0; k < kEncPerThread; k++)
                if ((uint32_t)k < cc.nvalid) bits += cl[code_k(cc, k)];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bits += __shfl_xor_sync(0xffffffffu, bits, o);
        if (lane == 0) a.chunk_bits[c] = (uint16_t)bits;  // <= 512 x 64
    }
}

__global__ void __launch_bounds__(kEncThreads) k_huff_count(HuffEncodeArgs a) {
    extern __shared__ uint8_t s_len_dyn[];
    if (*a.status != VSZ_OK || !encode_tree_ok(a)) return;
    count_chunks(a, blockIdx.x * (size_t)(kEncThreads / 32) + (threadIdx.x >> 5), a.nchunks,
                 (size_t)gridDim.x * (kEncThreads / 32), s_len_dyn);
}

// Many fields: tasks of (field, chunk range).
__global__ void __launch_bounds__(kEncThreads)
    k_huff_count_batch(const HuffEncodeArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    extern __shared__ uint8_t s_len_dyn[];
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk       = tasks[t];
        const HuffEncodeArgs& a  = args[tk.field];
        if (*a.status != VSZ_OK || !encode_tree_ok(a)) continue;  // same answer for the whole block
        count_chunks(a, tk.u0 + (threadIdx.x >> 5), tk.u1, kEncThreads / 32, s_len_dyn);
        __syncthreads();
    }
}

// Chunks c, c + cstep, ... < c1 of one field (one warp per chunk); the next chunk's codes are
// loaded while the current one is packed.
__device__ __forceinline__ void pack_chunks(const HuffEncodeArgs& a, size_t c, size_t c1, size_t cstep,
                                            uint8_t* s_dyn) {
    uint32_t* s_words = reinterpret_cast<uint32_t*>(s_dyn);                                     // 8 x kEncWarpWords
    unsigned long long* s_cw = reinterpret_cast<unsigned long long*>(s_words + 8 * kEncWarpWords);  // dict (if cached)
    uint8_t* s_len = reinterpret_cast<uint8_t*>(s_cw + (a.cb_in_smem ? a.dict : 0));
    const unsigned long long* cw = a.cb_word;
    const uint8_t* cl            = a.cb_len;
    if (a.cb_in_smem) {
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x) {
            s_cw[i]  = a.cb_word[i];
            s_len[i] = a.cb_len[i];
        }
        cw = s_cw;
        cl = s_len;
        __syncthreads();
    }
    const unsigned lane   = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t* sw          = s_words + warp * kEncWarpWords;
    uint8_t* out          = a.out + a.out_off.eval();
    const uint32_t base0  = (uint32_t)(reinterpret_cast<uintptr_t>(out) & 3u) * 8u;
    uint32_t* gw          = reinterpret_cast<uint32_t*>(reinterpret_cast<uintptr_t>(out) & ~(uintptr_t)3);
    // a batch scans all fields' chunks at once: offsets are relative to the field's first chunk
    const unsigned long long off0 = a.chunk_off[0];
    Codes16 nxt                   = load_codes16(a, c * kEncChunk + lane * kEncPerThread);
    for (; c < c1; c += cstep) {
        const Codes16 cc = nxt;
        if (c + cstep < c1) nxt = load_codes16(a, (c + cstep) * kEncChunk + lane * kEncPerThread);
        uint32_t sym[kEncPerThread], len[kEncPerThread], bits = 0;
#pragma unroll
        for (int k = 0; k < kEncPerThread; k++) {
            sym[k] = code_k(cc, k);
            len[k] = ((uint32_t)k < cc.nvalid) ? (uint32_t)cl[sym[k]] : 0u;
            bits += len[k];
        }
        uint32_t incl = bits;  // warp inclusive scan of lane bit counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned)o) incl += t;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
        const unsigned long long gstart = base0 + (a.chunk_off[c] - off0);  // chunk's first bit on the word grid
        const uint32_t r0               = (uint32_t)(gstart & 31u);
        const unsigned long long F      = gstart >> 5;
        const uint32_t nwords           = tot ? (r0 + tot + 31) >> 5 : 0u;
        for (uint32_t i = lane; i < nwords; i += 32) sw[i] = 0u;
        __syncwarp();
        // pack this lane's codewords; only a lane's first and last word can be shared with its
        // neighbours, so only those use shared-memory atomics
        {
            const uint32_t pos = r0 + incl - bits;
            uint32_t wi        = pos >> 5;
            uint32_t nb        = pos & 31u;  // bits already taken in the current word
            bool first         = true;
            unsigned long long acc = 0;       // MSB-aligned pending bits of word wi
            auto emit = [&](uint32_t word) {
                if (first && (pos & 31u)) atomicOr(&sw[wi], word);
                else sw[wi] = word;
                first = false;
                wi++;
            };
            auto append = [&](unsigned long long v, uint32_t l) {  // l <= 32
                if (l == 0) return;
                acc |= v << (64 - nb - l);
                nb += l;
                if (nb >= 32) {
                    emit((uint32_t)(acc >> 32));
                    acc <<= 32;
                    nb -= 32;
                }
            };
#pragma unroll
            for (int k = 0; k < kEncPerThread; k++) {
                if (len[k] == 0) continue;
                const unsigned long long v = cw[sym[k]];
                if (len[k] > 32) {
                    append(v >> 32, len[k] - 32);
                    append(v & 0xffffffffull, 32);
                } else {
                    append(v, len[k]);
                }
            }
            if (nb > 0) atomicOr(&sw[wi], (uint32_t)(acc >> 32));
        }
        __syncwarp();
        // interior words are plain stores; a partial first or last word (shared with the
        // neighbouring chunk, or with the tree bytes before the payload) goes to the edge records
        const bool first_partial = (r0 != 0);
        const bool last_partial  = ((r0 + tot) & 31u) != 0;
        for (uint32_t i = lane; i < nwords; i += 32) {
            if (i == 0 && first_partial) continue;
            if (i == nwords - 1 && last_partial) continue;
            gw[F + i] = bswap32(sw[i]);
        }
        if (lane == 0) {
            const unsigned long long none = ~0ull;
            a.edge_idx[2 * c]      = (nwords && first_partial) ? F : none;
            a.edge_bits[2 * c]     = nwords ? bswap32(sw[0]) : 0u;
            a.edge_idx[2 * c + 1]  = (nwords && last_partial) ? F + nwords - 1 : none;
            a.edge_bits[2 * c + 1] = nwords ? bswap32(sw[nwords - 1]) : 0u;
        }
        __syncwarp();
    }
}

// Codewords of at most kPackFastLen bits: the codebook is one u32 per symbol in shared memory,
// (codeword << 6) | length, and a lane appends its 16 codewords to a right-aligned 64-bit
// accumulator with no branch at all: the word a codeword completes is stored under a predicate.
// A word is completed -- and stored, with a plain store -- by exactly one lane, the one holding
// its last bit; the bits of it that earlier lanes hold are their unfinished tails, OR-ed in after
// a warp barrier.  The chunk's last word may be completed by nobody, so it alone is zeroed
// first.  Same words as pack_chunks.
constexpr uint32_t kPackFastLen = 26;

__device__ __forceinline__ void pack_chunks_fast(const HuffEncodeArgs& a, size_t c, size_t c1, size_t cstep,
                                                 uint8_t* s_dyn) {
    uint32_t* s_words = reinterpret_cast<uint32_t*>(s_dyn);      // 8 x kEncWarpWords
    uint32_t* s_tab   = s_words + 8 * kEncWarpWords;             // dict entries
    for (int i = threadIdx.x; i < a.dict; i += blockDim.x) {
        const uint32_t l = a.cb_len[i];
        s_tab[i]         = l ? ((uint32_t)a.cb_word[i] << 6) | l : 0u;
    }
    __syncthreads();
    const unsigned lane  = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t* sw         = s_words + warp * kEncWarpWords;
    uint8_t* out         = a.out + a.out_off.eval();
    const uint32_t base0 = (uint32_t)(reinterpret_cast<uintptr_t>(out) & 3u) * 8u;
    uint32_t* gw         = reinterpret_cast<uint32_t*>(reinterpret_cast<uintptr_t>(out) & ~(uintptr_t)3);
    const unsigned long long off0 = a.chunk_off[0];
    Codes16 nxt                   = load_codes16(a, c * kEncChunk + lane * kEncPerThread);
    unsigned long long nxt_off    = c < c1 ? a.chunk_off[c] : 0ull;
    for (; c < c1; c += cstep) {
        const Codes16 cc = nxt;
        const unsigned long long coff = nxt_off;
        if (c + cstep < c1) {
            nxt     = load_codes16(a, (c + cstep) * kEncChunk + lane * kEncPerThread);
            nxt_off = a.chunk_off[c + cstep];
        }
        uint32_t e[kEncPerThread], bits = 0;
        if (cc.nvalid == (uint32_t)kEncPerThread) {  // all but the field's last lanes
#pragma unroll
            for (int k = 0; k < kEncPerThread; k++) e[k] = s_tab[code_k(cc, k)];
        } else {
#pragma unroll
            for (int k = 0; k < kEncPerThread; k++) e[k] = ((uint32_t)k < cc.nvalid) ? s_tab[code_k(cc, k)] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kEncPerThread; k++) bits += e[k] & 63u;
        uint32_t incl = bits;  // warp inclusive scan of lane bit counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned)o) incl += t;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
        const unsigned long long gstart = base0 + (coff - off0);  // chunk's first bit on the word grid
        const uint32_t r0               = (uint32_t)(gstart & 31u);
        const unsigned long long F      = gstart >> 5;
        const uint32_t nwords           = tot ? (r0 + tot + 31) >> 5 : 0u;
        if (lane == 0 && nwords) sw[nwords - 1] = 0u;
        __syncwarp();
        const uint32_t pos = r0 + incl - bits;
        uint32_t wi        = pos >> 5;
        uint32_t nb        = pos & 31u;  // bits pending in hi:lo; the leading ones belong to earlier lanes
        uint32_t hi = 0, lo = 0;         // right-aligned pending bits (above them: spent bits)
#pragma unroll
        for (int k = 0; k < kEncPerThread; k++) {
            const uint32_t l = e[k] & 63u;  // <= 26: 32-bit funnel shifts move the 64-bit pair
            hi = __funnelshift_l(lo, hi, l);
            lo = (lo << l) | (e[k] >> 6);
            nb += l;                         // <= 57
            const bool done  = nb >= 32u;    // word wi is complete: the 32 bits above the nb - 32 newest
            const uint32_t w = __funnelshift_r(lo, hi, nb);  // shift nb & 31, which is nb - 32 when done
            if (done) sw[wi] = w;
            wi += done ? 1u : 0u;
            nb &= 31u;
        }
        __syncwarp();
        if (bits && nb > 0) atomicOr(&sw[wi], lo << (32 - nb));
        __syncwarp();
        const bool first_partial = (r0 != 0);
        const bool last_partial  = ((r0 + tot) & 31u) != 0;
        for (uint32_t i = lane; i < nwords; i += 32) {
            if (i == 0 && first_partial) continue;
            if (i == nwords - 1 && last_partial) continue;
            gw[F + i] = bswap32(sw[i]);
        }
        if (lane == 0) {
            const unsigned long long none = ~0ull;
            a.edge_idx[2 * c]      = (nwords && first_partial) ? F : none;
            a.edge_bits[2 * c]     = nwords ? bswap32(sw[0]) : 0u;
            a.edge_idx[2 * c + 1]  = (nwords && last_partial) ? F + nwords - 1 : none;
            a.edge_bits[2 * c + 1] = nwords ? bswap32(sw[nwords - 1]) : 0u;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kEncThreads, 4) k_huff_pack(HuffEncodeArgs a) {
    extern __shared__ uint8_t s_dyn[];
    if (*a.status != VSZ_OK) return;  // set before this launch: uniform across the grid
    const size_t c0 = blockIdx.x * (size_t)(kEncThreads / 32) + (threadIdx.x >> 5);
    const size_t cs = (size_t)gridDim.x * (kEncThreads / 32);
    // max code length from the tree build (device-resident); uniform
    if (a.cb_in_smem && a.build_info && a.build_info[2] <= kPackFastLen) pack_chunks_fast(a, c0, a.nchunks, cs, s_dyn);
    else pack_chunks(a, c0, a.nchunks, cs, s_dyn);
}

__global__ void __launch_bounds__(kEncThreads, 4)
    k_huff_pack_batch(const HuffEncodeArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    extern __shared__ uint8_t s_dyn[];
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk      = tasks[t];
        const HuffEncodeArgs& a = args[tk.field];
        if (*a.status != VSZ_OK) continue;  // no kernel of this launch writes it
        // the field's longest codeword: uniform over the task
        if (a.cb_in_smem && a.build_info && a.build_info[2] <= kPackFastLen)
            pack_chunks_fast(a, tk.u0 + (threadIdx.x >> 5), tk.u1, kEncThreads / 32, s_dyn);
        else
            pack_chunks(a, tk.u0 + (threadIdx.x >> 5), tk.u1, kEncThreads / 32, s_dyn);
        __syncthreads();
    }
}

// Boundary words of the chunks: chunk t's partial first word is the same word as chunk t - 1's
// partial last word (a chunk of 512 codewords of >= 1 bit spans >= 512 bits, so no word has a
// third sharer); the payload's first word also holds the last bytes of the tree section, kept as is.
__device__ __forceinline__ void edge_fix(const HuffEncodeArgs& a, size_t t) {
    uint8_t* out         = a.out + a.out_off.eval();
    const uint32_t base0 = (uint32_t)(reinterpret_cast<uintptr_t>(out) & 3u) * 8u;
    uint32_t* gw         = reinterpret_cast<uint32_t*>(reinterpret_cast<uintptr_t>(out) & ~(uintptr_t)3);
    const unsigned long long none = ~0ull;
    const unsigned long long fi   = a.edge_idx[2 * t];
    const unsigned long long li   = a.edge_idx[2 * t + 1];
    if (fi != none) {
        uint32_t v = a.edge_bits[2 * t];
        if (t > 0 && a.edge_idx[2 * t - 1] == fi) v |= a.edge_bits[2 * t - 1];
        if (fi == 0 && base0 != 0) v |= gw[0] & ((1u << base0) - 1u);  // tree bytes before the payload
        gw[fi] = v;
    }
    if (t == a.nchunks - 1 && li != none && li != fi) gw[li] = a.edge_bits[2 * t + 1];
}

__global__ void k_huff_encode_edges(HuffEncodeArgs a) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= a.nchunks || *a.status != VSZ_OK) return;
    edge_fix(a, t);
}

__global__ void k_huff_encode_edges_batch(const HuffEncodeArgs* __restrict__ args, const BatchTask* __restrict__ tasks,
                                          uint32_t ntasks) {
    for (uint32_t k = blockIdx.x; k < ntasks; k += gridDim.x) {
        const BatchTask tk      = tasks[k];
        const HuffEncodeArgs& a = args[tk.field];
        if (*a.status != VSZ_OK) continue;
        for (size_t t = tk.u0 + threadIdx.x; t < tk.u1; t += blockDim.x) edge_fix(a, t);
    }
}

// Many fields: each field's payload length from the scan of all fields' chunk bits (chunk_off has
// an entry past the field's last chunk: the next field's first, or the scan total); a failed scan
// fails every field.
__global__ void k_field_bits(const HuffEncodeArgs* __restrict__ args, uint32_t nfields, const int* scan_status) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfields) return;
    const HuffEncodeArgs& a = args[f];
    if (*scan_status != VSZ_OK) set_status(a.status, *scan_status);
    *a.total_bits = a.nchunks ? a.chunk_off[a.nchunks] - a.chunk_off[0] : 0ull;
}

// ------------------------------------------------------------------------------------------
// K4a: decode table from the serialized tree
// ------------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t rd_index(const uint8_t* p, int w) {
    uint32_t v = 0;
    for (int b = 0; b < w; b++) v |= (uint32_t)p[b] << (8 * b);
    return v;
}

// The decode tables of one field, by the whole CTA (1024 threads; returns are block-uniform).
constexpr int kTableSmemNodes = 4096;

__device__ __forceinline__ void huff_table_run(const HuffTableArgs& a) {
    const uint8_t* h = a.huff;
    __shared__ uint32_t s_nc;
    __shared__ int s_bad;
    __shared__ uint32_t s_w2[1 << kDecBits];  // secondary table width per primary prefix
    __shared__ uint32_t s_scan[33];
    __shared__ uint32_t s_maxlen;             // longest codeword (255: some leaf deeper than 64)
    if (threadIdx.x == 0) {
        s_nc  = ((uint32_t)h[0] << 24) | ((uint32_t)h[1] << 16) | ((uint32_t)h[2] << 8) | (uint32_t)h[3];
        s_bad = 0;
        if (s_nc == 0 || s_nc > a.max_nodes || 8 + tree_bytes_size(s_nc) > a.huff_bytes) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) {
        if (threadIdx.x == 0) set_status(a.status, VSZ_ERR_CORRUPT);
        return;
    }
    const uint32_t nc = s_nc;
    const int w       = tree_index_width(nc);
    const uint8_t* pL = h + 9;
    const uint8_t* pR = pL + (size_t)w * nc;
    const uint8_t* pC = pR + (size_t)w * nc;
    const uint8_t* pT = pC + 4 * (size_t)nc;
    // nc entries: parent << 1 | side; 0xffffffff = none.  In shared memory for trees of up to
    // kTableSmemNodes nodes (dictionaries up to 2048 symbols): every node's depth and code come
    // from a walk up to the root, one dependent read per level, twice.
    __shared__ uint32_t s_parent[kTableSmemNodes];
    uint32_t* parent  = nc <= (uint32_t)kTableSmemNodes ? s_parent : a.parent;
    for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) parent[i] = 0xffffffffu;
    for (uint32_t i = threadIdx.x; i < (1u << kDecBits); i += blockDim.x) a.table[i] = 0u;
    __syncthreads();
    // The reference rebuilds the root as an internal node when nodeCount > 256 and from
    // (C[0], t[0]) otherwise (src/huffman.hh:577,602,627).
    const bool root_leaf = (nc <= 256) && pT[0];
    for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) {
        bool leaf = (i == 0) ? root_leaf : (pT[i] != 0);
        uint32_t c = (uint32_t)pC[4 * (size_t)i] | ((uint32_t)pC[4 * (size_t)i + 1] << 8) |
                     ((uint32_t)pC[4 * (size_t)i + 2] << 16) | ((uint32_t)pC[4 * (size_t)i + 3] << 24);
        a.node_sym[i] = leaf ? (0x80000000u | (c & 0xffffu)) : 0u;
        if (leaf && c >= (uint32_t)a.dict) atomicExch(&s_bad, 1);
        if (!leaf) {
            uint32_t l = rd_index(pL + (size_t)i * w, w), r = rd_index(pR + (size_t)i * w, w);
            if (l == 0 || r == 0 || l >= nc || r >= nc) {
                // an internal node needs both children (the reference would dereference null)
                atomicExch(&s_bad, 1);
                l = r = 0;
            } else {
                atomicExch(&parent[l], (i << 1) | 0u);
                atomicExch(&parent[r], (i << 1) | 1u);
            }
            a.child[2 * (size_t)i]     = l;
            a.child[2 * (size_t)i + 1] = r;
        } else {
            if (a.walk) a.walk[i] = 0u;
            a.child[2 * (size_t)i]     = 0;
            a.child[2 * (size_t)i + 1] = 0;
        }
    }
    __syncthreads();
    if (s_bad) {
        if (threadIdx.x == 0) set_status(a.status, VSZ_ERR_CORRUPT);
        return;
    }
    // packed children for the shared-memory walk: 15-bit fields (dict <= 16384, nc < 32768)
    if (a.walk && nc < 32768u && a.dict <= 16384) {
        for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) {
            const bool leaf = (a.node_sym[i] & 0x80000000u) != 0;
            if (leaf) continue;
            const uint32_t l = a.child[2 * (size_t)i], r = a.child[2 * (size_t)i + 1];
            auto enc = [&](uint32_t c) -> uint32_t {
                const uint32_t ns = a.node_sym[c];
                return (ns & 0x80000000u) ? (0x8000u | (ns & 0x7fffu)) : c;
            };
            a.walk[i] = enc(l) | (enc(r) << 16);
        }
    }
    if (root_leaf) {
        if (threadIdx.x == 0) {
            a.info[0] = 1;  // single-symbol tree: constant output, no bits
            a.info[1] = a.node_sym[0] & 0xffffu;
            a.info[2] = 0;
        }
        return;
    }
    // depth and code of every node by walking up to the root (depth bounded by 64)
    auto depth_code = [&](uint32_t i, uint32_t& depth, unsigned long long& code) -> bool {
        uint32_t cur = i;
        depth        = 0;
        code         = 0;
        while (cur != 0) {
            const uint32_t p = parent[cur];
            if (p == 0xffffffffu || depth >= 64) return false;  // unreachable, or longer than 64 bits
            code |= (unsigned long long)(p & 1u) << depth;
            depth++;
            cur = p >> 1;
        }
        return true;
    };
    const bool table16 = (reinterpret_cast<uintptr_t>(a.table) & 15u) == 0;
    // pass 1: primary entries; width of the secondary table below every depth-kDecBits prefix
    for (uint32_t i = threadIdx.x; i < (1u << kDecBits); i += blockDim.x) s_w2[i] = 0u;
    if (threadIdx.x == 0) s_maxlen = 0u;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) {
        uint32_t depth;
        unsigned long long code;
        bool leaf = (a.node_sym[i] & 0x80000000u) != 0;
        if (!depth_code(i, depth, code)) {  // only the walk can reach it
            if (leaf) atomicMax(&s_maxlen, 255u);
            continue;
        }
        if (leaf) atomicMax(&s_maxlen, depth);
        if (leaf && depth >= 1 && depth <= (uint32_t)kDecBits) {
            uint32_t lo = (uint32_t)(code << (kDecBits - depth));
            uint32_t hi = lo + (1u << (kDecBits - depth));
            uint32_t e  = ((a.node_sym[i] & 0xffffu) << 8) | depth;
            // a short codeword fills up to 2^(kDecBits - 1) entries: 16 bytes at a time (lo and hi
            // are multiples of 4 when depth <= kDecBits - 2)
            if (hi - lo >= 4 && table16) {
                const uint4 e4 = make_uint4(e, e, e, e);
                for (uint32_t t = lo; t < hi; t += 4) *reinterpret_cast<uint4*>(a.table + t) = e4;
            } else {
                for (uint32_t t = lo; t < hi; t++) a.table[t] = e;
            }
        } else if (!leaf && depth == (uint32_t)kDecBits) {
            a.table[(uint32_t)code] = (i << 8);  // walk from node i (until a secondary table replaces it)
        } else if (leaf && depth > (uint32_t)kDecBits) {
            const uint32_t r = depth - kDecBits;
            atomicMax(&s_w2[(uint32_t)(code >> r)], r < (uint32_t)kDec2Max ? r : (uint32_t)kDec2Max);
        }
    }
    __syncthreads();
    // offsets of the secondary tables (exclusive scan of 2^w2, kDecBits-bit prefixes in order)
    constexpr int kPer = (1 << kDecBits) / 1024;
    uint32_t sizes[kPer], mine = 0;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const uint32_t w2 = s_w2[threadIdx.x * kPer + k];
        sizes[k]          = w2 ? (1u << w2) : 0u;
        mine += sizes[k];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan<uint32_t>(mine, s_scan, &total);
    const bool fits = total <= table2_capacity(a.max_nodes);  // always, by the capacity's construction
    if (fits) {
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const uint32_t pfx = threadIdx.x * kPer + k, w2 = s_w2[pfx];
            if (w2) a.table[pfx] = (off << 12) | (w2 << 8) | 0x80u;
            off += sizes[k];
        }
        for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) a.table2[i] = 0u;  // not a codeword
    }
    __syncthreads();
    // pass 2: secondary entries -- leaves within w2 bits of their prefix, and walk entries for the
    // internal nodes w2 bits down (codewords longer than kDecBits + kDec2Max)
    if (fits) {
        for (uint32_t i = threadIdx.x; i < nc; i += blockDim.x) {
            uint32_t depth;
            unsigned long long code;
            if (!depth_code(i, depth, code) || depth <= (uint32_t)kDecBits) continue;
            const uint32_t r   = depth - kDecBits;
            const uint32_t pfx = (uint32_t)(code >> r);
            const uint32_t e   = a.table[pfx];
            if (!(e & 0x80u)) continue;
            const uint32_t w2 = (e >> 8) & 0xfu, base = e >> 12;
            if (r > w2) continue;
            const uint32_t rel = (uint32_t)(code & ((1ull << r) - 1ull));
            const bool leaf    = (a.node_sym[i] & 0x80000000u) != 0;
            if (leaf) {
                const uint32_t lo = base + (rel << (w2 - r)), hi = lo + (1u << (w2 - r));
                const uint32_t v  = ((a.node_sym[i] & 0xffffu) << 8) | depth;
                for (uint32_t t = lo; t < hi; t++) a.table2[t] = v;
            } else if (r == w2) {
                a.table2[base + rel] = (i << 8);
            }
        }
    }
    if (threadIdx.x == 0) {
        a.info[0] = 0;
        a.info[1] = 0;
        a.info[2] = s_maxlen;
    }
}

__global__ void __launch_bounds__(1024) k_huff_table(HuffTableArgs a) { huff_table_run(a); }

// Many fields: one CTA per field (grid-stride); a field whose status is already set is skipped.
__global__ void __launch_bounds__(1024) k_huff_table_batch(const HuffTableArgs* __restrict__ args, uint32_t nfields) {
    for (uint32_t f = blockIdx.x; f < nfields; f += gridDim.x) {
        const HuffTableArgs a = args[f];
        if (*a.status == VSZ_OK) huff_table_run(a);
        __syncthreads();  // the next field reuses the shared arrays
    }
}

// ------------------------------------------------------------------------------------------
// K4b: chunk decoder
// ------------------------------------------------------------------------------------------

struct BitReader {
    const uint32_t* gw;       // aligned word base
    unsigned long long pos;   // bit position on the word grid
    unsigned long long buf;   // MSB-aligned bits starting at `pos`
    int nbits;                // valid bits in buf
    unsigned long long limit; // first bit past the payload on the word grid

    __device__ __forceinline__ void init(const uint32_t* g, unsigned long long p, unsigned long long lim) {
        gw    = g;
        pos   = p;
        limit = lim;
        unsigned long long wi = p >> 5;
        uint32_t off          = (uint32_t)(p & 31u);
        unsigned long long hi = bswap32(__ldg(&gw[wi]));
        unsigned long long lo = bswap32(__ldg(&gw[wi + 1]));
        buf   = ((hi << 32) | lo) << off;
        nbits = 64 - (int)off;
    }
    __device__ __forceinline__ void refill() {
        if (nbits <= 32) {
            unsigned long long wi = (pos + nbits) >> 5;  // word aligned: pos + nbits is a multiple of 32
            unsigned long long v  = bswap32(__ldg(&gw[wi]));
            buf |= v << (32 - nbits);
            nbits += 32;
        }
    }
    __device__ __forceinline__ uint32_t peek(int k) const { return (uint32_t)(buf >> (64 - k)); }
    __device__ __forceinline__ void skip(int k) {
        buf <<= k;
        nbits -= k;
        pos += k;
    }
};

// Decode one symbol; returns 0xffffffff on a malformed walk or on running past the payload.
__device__ __forceinline__ uint32_t decode_one(BitReader& br, const uint32_t* table, const uint32_t* table2,
                                               const uint32_t* child, const uint32_t* node_sym, uint32_t max_nodes) {
    br.refill();  // > 32 valid bits: enough for both table levels
    uint32_t e   = table[br.peek(kDecBits)];
    uint32_t len = e & 0x7fu;
    if (len) {
        if (br.pos + len > br.limit) return 0xffffffffu;
        br.skip((int)len);
        return e >> 8;
    }
    uint32_t node = e >> 8, used = kDecBits;
    if (e & 0x80u) {
        const uint32_t w2 = (e >> 8) & 0xfu;
        const uint32_t e2 = __ldg(&table2[(e >> 12) + (br.peek(kDecBits + (int)w2) & ((1u << w2) - 1u))]);
        len               = e2 & 0xffu;
        if (len) {
            if (br.pos + len > br.limit) return 0xffffffffu;
            br.skip((int)len);
            return e2 >> 8;
        }
        node = e2 >> 8;
        used = kDecBits + w2;
    }
    if (node == 0 || node >= max_nodes) return 0xffffffffu;  // prefix not in the tree
    if (br.pos + used > br.limit) return 0xffffffffu;
    br.skip((int)used);
    for (int guard = 0; guard < 4096; guard++) {
        br.refill();
        if (br.pos + 1 > br.limit) return 0xffffffffu;
        uint32_t b = br.peek(1);
        br.skip(1);
        node = __ldg(&child[2 * (size_t)node + b]);
        if (node == 0 || node >= max_nodes) return 0xffffffffu;
        uint32_t s = __ldg(&node_sym[node]);
        if (s & 0x80000000u) return s & 0xffffu;
    }
    return 0xffffffffu;
}

__global__ void __launch_bounds__(256) k_huff_decode(HuffDecodeArgs a) {
    __shared__ uint32_t s_table[1 << kDecBits];
    for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) s_table[i] = a.table[i];
    __syncthreads();
    const size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= a.nchunks) return;
    if (*a.status != VSZ_OK) return;  // e.g. the tree failed to parse: tables are not valid
    const unsigned long long out0 = a.out_begin ? a.out_begin[j] : (unsigned long long)j * a.chunk_syms;
    if (out0 >= a.n) return;
    unsigned long long cnt = a.nsym ? a.nsym[j] : (unsigned long long)a.chunk_syms;
    if (out0 + cnt > a.n) cnt = a.n - out0;
    const uint32_t base0 = (uint32_t)(reinterpret_cast<uintptr_t>(a.payload) & 3u) * 8u;
    const uint32_t* gw   = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(a.payload) & ~(uintptr_t)3);
    BitReader br;
    br.init(gw, base0 + a.start_bit[j], base0 + a.payload_bits);
    // output position -> (row, x) for the per-segment zero counts
    unsigned long long row = out0 / a.d0;
    uint32_t x             = (uint32_t)(out0 - row * a.d0);
    uint32_t zeros         = 0;
    auto flush = [&]() {
        if (zeros && a.seg_zero) atomicAdd(&a.seg_zero[row * a.nxs + (x >> 8)], zeros);
        zeros = 0;
    };
    uint16_t* out = a.codes + out0;
    for (unsigned long long k = 0; k < cnt; k++) {
        uint32_t s = decode_one(br, s_table, a.table2, a.child, a.node_sym, a.max_nodes);
        if (s == 0xffffffffu) {
            set_status(a.status, VSZ_ERR_CORRUPT);
            return;
        }
        out[k] = (uint16_t)s;
        zeros += (s == 0);
        x++;
        if (x == a.d0) {
            x--;
            flush();
            x = 0;
            row++;
        } else if ((x & 255u) == 0) {
            x--;
            flush();
            x++;
        }
    }
    flush();
}

// Indexed decode with coalesced output: a warp decodes 32 consecutive chunks of 512 codewords
// (one per lane) in rounds of 32 symbols staged in shared memory, then writes each lane's 32
// symbols (64 contiguous bytes) as 16-byte stores.  The index gives every chunk's first bit and
// length, so the inner loop has no bounds test: a chunk must consume exactly its indexed length
// (checked at the end), and reads stop 64 bits past it whatever the bits say.  Zero codes are
// counted per chunk (outlier ranks for the reverse Lorenzo kernel).
// ------------------------------------------------------------------------------------------
// K4b': indexed decoder for trees whose codewords are at most kWinMaxLen (32) bits -- the table
// builder records the longest one.  Lane j decodes chunk j (512 codewords from its indexed start
// bit).  The lane holds a 96-bit window of its stream in three registers (w0 w1 w2, bit offset
// `off` into w0) and decodes kWinRound codewords per round; a codeword moves the window by at
// most one word, so the move and the ring read are predicated, not branched.  Words come from a
// per-lane ring of kWinRing 16-byte blocks in shared memory that cp.async keeps filled ahead of
// the window: one round reads at most kWinRound * 32 bits = 8 words, and the blocks holding them
// have landed at the round's start.  Block and word counters are 32-bit and relative to the
// chunk's first 16-byte block.  The warp diverges only on codewords longer than the primary
// table.  Decoded codes are packed in registers and stored 16 bytes per lane per round.
// ------------------------------------------------------------------------------------------
constexpr int kWinMaxLen    = 32;
constexpr int kWinRound     = 8;
constexpr int kWinRing      = 8;    // blocks of 16 bytes per lane
constexpr int kWinWait      = 4;    // copy groups left in flight at a round's start
constexpr int kWinLaneWords = kWinRing * 4 + 4;  // a lane's ring, padded: lanes 8 apart share banks
constexpr int kWinThreads   = 256;  // one primary table per CTA, shared by its warps
constexpr int kWinMinBlocks = 4;
// Blocks wn / 4 .. wn / 4 + kWinRing - 2 are requested and all but the newest kWinWait have landed
// at a round's start: at least 4 (kWinRing - 1 - kWinWait) - 3 words from wn, and a round of
// kWinRound codewords of <= 32 bits moves the window by at most kWinRound words.
static_assert(4 * (kWinRing - 1 - kWinWait) - 3 >= kWinRound, "a round may read words still in flight");
static_assert((kWinRing & (kWinRing - 1)) == 0 && (kWinRound == 8 || kWinRound == 4), "ring and round shapes");
constexpr size_t kWinSmem   = (sizeof(uint32_t) << kDecBits) + (size_t)kWinThreads * kWinLaneWords * 4;
typedef uint32_t WinRing[32][kWinLaneWords];  // one warp's rings, [lane][word]

// Lane j of the calling warp decodes chunk j (the table is in s_table; no block barrier inside).
__device__ __forceinline__ void decode_win_lane(const HuffDecodeArgs& a, size_t j, const uint32_t* s_table,
                                                WinRing* s_ring) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (j - lane >= a.nchunks) return;
    const unsigned long long out0 = (unsigned long long)j * kChunkSyms;
    uint32_t cnt = 0;
    if (j < a.nchunks && out0 < a.n) cnt = (uint32_t)min((unsigned long long)kChunkSyms, a.n - out0);
    const uint32_t base0 = (uint32_t)(reinterpret_cast<uintptr_t>(a.payload) & 15u) * 8u;
    const uint8_t* g16   = reinterpret_cast<const uint8_t*>(reinterpret_cast<uintptr_t>(a.payload) & ~(uintptr_t)15);
    // readable bytes from g16: the payload plus the 8 bytes past its end that callers provide
    const unsigned long long readable = base0 / 8u + (a.payload_bits + 7) / 8 + 8;
    uint32_t* ring = s_ring[warp][lane];
    bool bad = false;
    unsigned long long cb = 0;
    const uint8_t* gb = g16;  // the chunk's first 16-byte block
    uint32_t rem = 0;         // readable bytes from gb (clamped)
    uint32_t off = 0, wn = 0, breq = 0;  // bit offset in w0; next word to enter the window; next block
    if (cnt) {
        // offsets relative to the field's first chunk (a batch scans all fields' indexes at once)
        const unsigned long long sb = a.start_bit[j] - a.start_bit[0];
        cb = a.chunk_len[j];
        if (sb + cb > a.payload_bits) bad = true;
        const unsigned long long pos0 = base0 + sb;
        const unsigned long long b0   = pos0 >> 7;
        gb  = g16 + b0 * 16;
        rem = b0 * 16 >= readable ? 0u : (uint32_t)min(readable - b0 * 16, 0x7fffffffull);
        off = (uint32_t)(pos0 & 31u);
        wn  = (uint32_t)(pos0 >> 5) & 3u;
    }
    const bool live = cnt && !bad;
    auto fetch = [&](uint32_t b) {  // block b into slot b % kWinRing, one commit group
        const uint32_t o  = b * 16u;
        const uint32_t nb = o >= rem ? 0u : min(16u, rem - o);
        cp_async16_zfill(ring + 4u * (b % (uint32_t)kWinRing), gb + (nb ? o : 0u), nb);
        cp_async_commit();
    };
    auto ring_word = [&](uint32_t w) -> uint32_t { return bswap32(ring[w % (uint32_t)(4 * kWinRing)]); };
    // blocks [wn / 4, wn / 4 + kWinRing - 1) stay requested: the slot a fetch overwrites held a
    // block whose words entered the window at least one block earlier
    if (live)
        for (int k = 0; k < kWinRing - 1; k++) fetch(breq++);
    cp_async_wait<kWinWait>();
    uint32_t w0 = 0, w1 = 0, w2 = 0;
    if (live) {
        w0 = ring_word(wn);
        w1 = ring_word(wn + 1);
        w2 = ring_word(wn + 2);
        wn += 3;
    }
    const uint32_t pos_first = wn * 32u + off;  // the first bit (wn counts the 3 window words)
    uint32_t zeros = 0;
    uint16_t* dst = a.codes + out0;
    // full rounds are stored in pairs, a whole 32-byte sector at a time: the lanes of a warp write
    // 32 different chunks, and a sector written in halves far apart can leave L2 half written
    uint32_t pkp[kWinRound / 2] = {};
    bool pend = false;  // pkp holds the full round before this one, not yet stored
    // a pair of rounds starts on a 32-byte boundary of the chunk (1024 bytes); so of the field's
    // codes when those are 32-byte aligned (workspace arrays are 256-byte aligned)
    const bool sector_store = (reinterpret_cast<uintptr_t>(a.codes) & 31u) == 0;
    auto store_round = [&](uint32_t at, const uint32_t* q) {
        if constexpr (kWinRound == 8)
            *reinterpret_cast<uint4*>(dst + at) = make_uint4(q[0], q[1], q[kWinRound / 2 - 2], q[kWinRound / 2 - 1]);
        else
            *reinterpret_cast<uint2*>(dst + at) = make_uint2(q[0], q[1]);
    };
    for (uint32_t r0 = 0; r0 < (uint32_t)kChunkSyms; r0 += kWinRound) {
        const uint32_t m = (live && cnt > r0) ? min((uint32_t)kWinRound, cnt - r0) : 0u;
        if (m) {
            const uint32_t bneed = (wn >> 2) + kWinRing - 1;
            while (breq < bneed) fetch(breq++);
        }
        cp_async_wait<kWinWait>();
        uint32_t pk[kWinRound / 2] = {};
        // one codeword; a full round (m == kWinRound) runs it without per-code guards
        auto step = [&](int k) {
            const uint32_t win = __funnelshift_l(w1, w0, off);  // 32 bits from the current position
            const uint32_t e   = s_table[win >> (32 - kDecBits)];
            uint32_t len       = e & 0x7fu;
            uint32_t sy        = e >> 8;
            if (!len) {
                uint32_t node = e >> 8, usedb = kDecBits;
                if (e & 0x80u) {
                    const uint32_t w2b = (e >> 8) & 0xfu;
                    const uint32_t e2 =
                        __ldg(&a.table2[(e >> 12) + ((win >> (32 - kDecBits - w2b)) & ((1u << w2b) - 1u))]);
                    len   = e2 & 0xffu;
                    sy    = e2 >> 8;
                    node  = e2 >> 8;
                    usedb = kDecBits + w2b;
                }
                if (!len) {
                    // longer than both tables: walk the tree over a 64-bit view of the window
                    unsigned long long v = ((((unsigned long long)w0) << 32) | w1) << off;
                    if (off) v |= (unsigned long long)w2 >> (32 - off);
                    sy = 0xffffffffu;
                    if (node != 0 && node < a.max_nodes) {
                        for (uint32_t d = usedb; d < (uint32_t)kWinMaxLen; d++) {
                            node = __ldg(&a.child[2 * (size_t)node + (uint32_t)((v >> (63 - d)) & 1ull)]);
                            if (node == 0 || node >= a.max_nodes) break;
                            const uint32_t ns = __ldg(&a.node_sym[node]);
                            if (ns & 0x80000000u) {
                                sy  = ns & 0xffffu;
                                len = d + 1;
                                break;
                            }
                        }
                    }
                    if (sy == 0xffffffffu) {
                        bad = true;
                        sy  = 0;
                        len = 0;
                    }
                }
            }
            pk[k >> 1] |= (sy & 0xffffu) << (16 * (k & 1));
            zeros += (sy == 0u);
            off += len;
            // at most one word per codeword (len <= 32); refilled without a branch, because some
            // lane of the warp crosses a word boundary on nearly every step.  Only the lanes that
            // cross read the ring (a predicated load), so fewer lanes share its banks.
            const bool adv = off >= 32u;
            uint32_t nw    = w2;
            if (adv) nw = ring_word(wn);
            off = adv ? off - 32u : off;
            w0  = adv ? w1 : w0;
            w1  = adv ? w2 : w1;
            w2  = adv ? nw : w2;
            wn += adv ? 1u : 0u;
        };
        if (m == (uint32_t)kWinRound) {
#pragma unroll
            for (int k = 0; k < kWinRound; k++) step(k);
            if (pend) {
                if constexpr (kWinRound == 8) {
                    if (sector_store) {  // one 256-bit store: the whole sector in one request
                        asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst + r0 - kWinRound),
                                     "r"(pkp[0]), "r"(pkp[1]), "r"(pkp[2]), "r"(pkp[3]), "r"(pk[0]), "r"(pk[1]),
                                     "r"(pk[2]), "r"(pk[3])
                                     : "memory");
                    } else {
                        store_round(r0 - kWinRound, pkp);
                        store_round(r0, pk);
                    }
                } else {
                    store_round(r0 - kWinRound, pkp);
                    store_round(r0, pk);
                }
            } else {
#pragma unroll
                for (int k = 0; k < kWinRound / 2; k++) pkp[k] = pk[k];
            }
            pend = !pend;
        } else {
            if (pend) store_round(r0 - kWinRound, pkp);
            pend = false;
#pragma unroll
            for (int k = 0; k < kWinRound; k++)
                if ((uint32_t)k < m) step(k);
            for (uint32_t k = 0; k < m; k++) dst[r0 + k] = (uint16_t)(pk[k >> 1] >> (16 * (k & 1)));
        }
    }
    if (pend) store_round((uint32_t)kChunkSyms - kWinRound, pkp);  // not reached: 512 / kWinRound is even
    cp_async_wait<0>();  // no copy into this CTA's shared memory may outlive it
    // bits consumed: the position now minus the first (a chunk spans < 2^32 bits)
    const unsigned long long used = live ? (unsigned long long)(wn * 32u + off - pos_first) : 0ull;
    if (cnt && (bad || used != cb)) set_status(a.status, VSZ_ERR_CORRUPT);  // must fill exactly its length
    if (j < a.nchunks && a.chunk_zero) a.chunk_zero[j] = zeros;
}

__global__ void __launch_bounds__(kWinThreads, kWinMinBlocks) k_huff_decode_win(HuffDecodeArgs a) {
    extern __shared__ __align__(16) uint8_t s_win_dyn[];
    // [primary table: 1 << kDecBits words][rings: warp][lane][kWinLaneWords] (kWinSmem bytes)
    uint32_t* s_table = reinterpret_cast<uint32_t*>(s_win_dyn);
    WinRing* s_ring   = reinterpret_cast<WinRing*>(s_win_dyn + (sizeof(uint32_t) << kDecBits));
    if (!a.tree_info || a.tree_info[2] > (uint32_t)kWinMaxLen) return;  // uniform: k_huff_decode_idx's trees
    for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) s_table[i] = a.table[i];
    __syncthreads();
    if (*a.status != VSZ_OK) return;  // no block barrier below
    decode_win_lane(a, blockIdx.x * (size_t)blockDim.x + threadIdx.x, s_table, s_ring);
}

constexpr int kDecRound = 16;                 // codes per lane staged before the coalesced store
constexpr int kDecParts = kDecRound / 8;      // 16-byte pieces per staged row

// Shared memory of the general indexed decoder (the walk array, when in shared memory, follows).
struct IdxSmem {
    uint32_t table[1 << kDecBits];
    __align__(16) uint16_t stage[8][32][kDecRound + 8];  // +8: keep rows 16-byte aligned
    __align__(16) uint4 ring[8][4][32];                   // per lane: 4 blocks of its stream
};

// Lane j of the calling warp decodes chunk j of a tree with codewords over kWinMaxLen bits.
template <bool WALK_SMEM>
__device__ __forceinline__ void decode_idx_lane(const HuffDecodeArgs& a, size_t j, IdxSmem& sm, const uint32_t* s_walk) {
    auto& s_table = sm.table;
    auto& s_stage = sm.stage;
    auto& s_ring  = sm.ring;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const size_t jw0    = j - lane;  // first chunk of this warp
    if (jw0 >= a.nchunks) return;
    const bool active   = j < a.nchunks;
    const unsigned long long out0 = (unsigned long long)j * kChunkSyms;
    uint32_t cnt = 0;
    if (active && out0 < a.n) cnt = (uint32_t)min((unsigned long long)kChunkSyms, a.n - out0);
    // Bits come through a per-lane ring of four 16-byte blocks in shared memory, filled by
    // cp.async three blocks (~380 bits, ~60 codewords) ahead of use: the 32 lanes of a warp read
    // 32 separate streams, which thrash L1 when fetched word by word.  Positions are bits from the
    // 16-byte aligned base; bytes past the readable end are zero-filled by the copy.
    const uint32_t base0 = (uint32_t)(reinterpret_cast<uintptr_t>(a.payload) & 15u) * 8u;
    const uint8_t* g16   = reinterpret_cast<const uint8_t*>(reinterpret_cast<uintptr_t>(a.payload) & ~(uintptr_t)15);
    // readable bytes from g16: the payload plus the 8 bytes past its end that callers provide
    const unsigned long long readable = base0 / 8u + (a.payload_bits + 7) / 8 + 8;
    uint4* ring = &s_ring[warp][0][lane];  // slot k at ring[32 k]
    auto fetch = [&](unsigned long long b) {  // block b into slot b % 4, one commit group
        const unsigned long long off = b * 16;
        const uint32_t nb = off >= readable ? 0u : (uint32_t)min(16ull, readable - off);
        cp_async16_zfill(ring + 32 * (uint32_t)(b & 3), g16 + (nb ? off : 0), nb);
        cp_async_commit();
    };
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    int nq = 0;
    unsigned long long blk = 0;  // next block to take from the ring
    // blocks blk, blk + 1, blk + 2 are in flight here; slot (blk + 3) % 4 was read one block ago
    auto next_block = [&]() {
        cp_async_wait<2>();
        q = ring[32 * (uint32_t)(blk & 3)];
        fetch(blk + 3);
        blk++;
        nq = 4;
    };
    auto pop = [&]() -> uint32_t {
        if (nq == 0) next_block();
        const uint32_t w = q.x;
        q.x = q.y;
        q.y = q.z;
        q.z = q.w;
        nq--;
        return bswap32(w);
    };
    bool bad = false;
    unsigned long long pos = 0, end = 0;
    unsigned long long buf = 0;
    int nbits = 0;
    if (cnt) {
        const unsigned long long sb = a.start_bit[j] - a.start_bit[0], cb = a.chunk_len[j];
        if (sb + cb > a.payload_bits) bad = true;
        pos = base0 + sb;
        end = pos + cb;
        if (!bad) {
            const unsigned long long wi = pos >> 5;
            const uint32_t off          = (uint32_t)(pos & 31u);
            blk = wi >> 2;
            fetch(blk);
            fetch(blk + 1);
            fetch(blk + 2);
            for (uint32_t k = 0; k < (uint32_t)(wi & 3u); k++) pop();
            const uint32_t w0 = pop();
            const uint32_t w1 = pop();
            buf   = ((((unsigned long long)w0) << 32) | w1) << off;
            nbits = 64 - (int)off;
        }
    }
    uint32_t zeros = 0;
    for (uint32_t r0 = 0; r0 < (uint32_t)kChunkSyms; r0 += kDecRound) {
        const uint32_t m = (cnt > r0 && !bad) ? min((uint32_t)kDecRound, cnt - r0) : 0u;
        for (uint32_t k = 0; k < m; k++) {
            if (nbits <= 32) {
                const unsigned long long nxt = pos + (unsigned long long)nbits;  // word aligned
                if (nxt > end + 64) {
                    bad = true;
                    break;
                }
                buf |= ((unsigned long long)pop()) << (32 - nbits);
                nbits += 32;
            }
            const uint32_t e = s_table[(uint32_t)(buf >> (64 - kDecBits))];
            uint32_t len     = e & 0x7fu;
            uint32_t sy      = e >> 8;
            uint32_t node = 0, used = 0;
            if (!len) {
                // a longer codeword: the secondary table (next w2 bits) resolves it, or gives the
                // node to walk from (nbits > 32 covers both lookups)
                node = e >> 8;
                used = kDecBits;
                if (e & 0x80u) {
                    const uint32_t w2 = (e >> 8) & 0xfu;
                    const uint32_t e2 =
                        __ldg(&a.table2[(e >> 12) + ((uint32_t)(buf >> (64 - kDecBits - w2)) & ((1u << w2) - 1u))]);
                    len  = e2 & 0xffu;
                    sy   = e2 >> 8;
                    node = e2 >> 8;
                    used = kDecBits + w2;
                }
            }
            if (!len) {
                // codeword longer than both tables: walk the tree bit by bit, refilling as it goes
                // (codewords may be up to 64 bits)
                sy = 0xffffffffu;
                if (node == 0 || node >= a.max_nodes) {
                    bad = true;
                    break;
                }
                buf <<= used;
                nbits -= (int)used;
                pos += used;
                for (int guard = 0; guard < 64; guard++) {
                    if (nbits <= 32) {
                        const unsigned long long nxt = pos + (unsigned long long)nbits;
                        if (nxt > end + 64) break;
                        buf |= ((unsigned long long)pop()) << (32 - nbits);
                        nbits += 32;
                    }
                    const uint32_t bit = (uint32_t)(buf >> 63);
                    buf <<= 1;
                    nbits--;
                    pos++;
                    if (WALK_SMEM) {
                        const uint32_t ent = (s_walk[node] >> (16 * bit)) & 0xffffu;
                        if (ent & 0x8000u) {
                            sy = ent & 0x7fffu;
                            break;
                        }
                        node = ent;
                        if (node == 0 || node >= a.nodes) break;
                    } else {
                        node = __ldg(&a.child[2 * (size_t)node + bit]);
                        if (node == 0 || node >= a.max_nodes) break;
                        const uint32_t ns = __ldg(&a.node_sym[node]);
                        if (ns & 0x80000000u) {
                            sy = ns & 0xffffu;
                            break;
                        }
                    }
                }
                if (sy == 0xffffffffu) {
                    bad = true;
                    break;
                }
                len = 0;  // already consumed
            }
            buf <<= len;
            nbits -= (int)len;
            pos += len;
            s_stage[warp][lane][k] = (uint16_t)sy;
            zeros += (sy == 0u);
        }
        __syncwarp();
        // 32 rows x kDecParts pieces of 8 symbols; piece pq * 32 + lane
#pragma unroll
        for (int pq = 0; pq < kDecParts; pq++) {
            const uint32_t piece = pq * 32 + lane, src = piece / kDecParts, part = piece % kDecParts;
            const size_t jj      = jw0 + src;
            const uint32_t cnt_s = __shfl_sync(0xffffffffu, cnt, src);
            const uint32_t ms    = (cnt_s > r0) ? min((uint32_t)kDecRound, cnt_s - r0) : 0u;
            const uint32_t p0    = part * 8;
            if (jj < a.nchunks && p0 < ms) {
                uint16_t* dst = a.codes + jj * kChunkSyms + r0 + p0;
                if (p0 + 8 <= ms) {
                    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(&s_stage[warp][src][p0]);
                } else {
                    for (uint32_t e2 = p0; e2 < ms; e2++) dst[e2 - p0] = s_stage[warp][src][e2];
                }
            }
        }
        __syncwarp();
    }
    cp_async_wait<0>();  // no copy into this CTA's shared memory may outlive it
    if (cnt && !bad && pos != end) bad = true;  // the chunk must fill exactly its indexed length
    if (bad) set_status(a.status, VSZ_ERR_CORRUPT);
    if (active && a.chunk_zero) a.chunk_zero[j] = zeros;
}

template <bool WALK_SMEM>
__global__ void __launch_bounds__(256) k_huff_decode_idx(HuffDecodeArgs a) {
    __shared__ IdxSmem sm;
    extern __shared__ uint32_t s_walk[];  // WALK_SMEM: a.nodes entries
    for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) sm.table[i] = a.table[i];
    if (WALK_SMEM)
        for (uint32_t i = threadIdx.x; i < a.nodes; i += blockDim.x) s_walk[i] = a.walk[i];
    __syncthreads();
    if (*a.status != VSZ_OK) return;
    if (a.tree_info && a.tree_info[2] <= (uint32_t)kWinMaxLen) return;  // k_huff_decode_win's trees
    decode_idx_lane<WALK_SMEM>(a, blockIdx.x * (size_t)blockDim.x + threadIdx.x, sm, s_walk);
}

// ---- many fields: tasks of (field, chunk range [256 k, 256 k + 256) of its index), one CTA
// each; lane t of the CTA decodes chunk u0 + t.  A kernel takes the tasks of the fields whose trees
// are of its kind (read from k_huff_table's results, so uniform over the CTA) and skips the rest.
__global__ void __launch_bounds__(kWinThreads, kWinMinBlocks)
    k_huff_decode_win_batch(const HuffDecodeArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    extern __shared__ __align__(16) uint8_t s_win_dyn[];
    uint32_t* s_table = reinterpret_cast<uint32_t*>(s_win_dyn);
    WinRing* s_ring = reinterpret_cast<WinRing*>(s_win_dyn + (sizeof(uint32_t) << kDecBits));
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk     = tasks[t];
        const HuffDecodeArgs a = args[tk.field];
        if (a.tree_info[2] > (uint32_t)kWinMaxLen) continue;
        for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) s_table[i] = a.table[i];
        __syncthreads();
        if (*a.status == VSZ_OK) decode_win_lane(a, tk.u0 + threadIdx.x, s_table, s_ring);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256)
    k_huff_decode_idx_batch(const HuffDecodeArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    __shared__ IdxSmem sm;
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk     = tasks[t];
        const HuffDecodeArgs a = args[tk.field];
        if (a.tree_info[2] <= (uint32_t)kWinMaxLen) continue;
        for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) sm.table[i] = a.table[i];
        __syncthreads();
        if (*a.status == VSZ_OK) decode_idx_lane<false>(a, tk.u0 + threadIdx.x, sm, nullptr);
        __syncthreads();
    }
}

// One-symbol trees: every code of the chunk is the symbol (src/huffman.hh:348-352); zero counts
// per chunk for the outlier ranks.
__global__ void __launch_bounds__(256)
    k_huff_const_batch(const HuffDecodeArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk     = tasks[t];
        const HuffDecodeArgs a = args[tk.field];
        if (*a.status != VSZ_OK) continue;
        const uint16_t c = (uint16_t)a.tree_info[1];
        const size_t lo = tk.u0 * (size_t)kChunkSyms, hi = min((size_t)a.n, (size_t)(tk.u1 * kChunkSyms));
        for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) a.codes[i] = c;
        for (size_t j = tk.u0 + threadIdx.x; j < tk.u1; j += blockDim.x)
            a.chunk_zero[j] = c == 0 ? (uint32_t)min((size_t)kChunkSyms, (size_t)(a.n - j * kChunkSyms)) : 0u;
    }
}

int launch_huff_table_batch(const HuffTableArgs* args, uint32_t nfields, cudaStream_t st, int num_sms) {
    if (nfields == 0) return VSZ_OK;
    const uint32_t grid = nfields < (uint32_t)num_sms ? nfields : (uint32_t)num_sms;
    k_huff_table_batch<<<grid, 1024, 0, st>>>(args, nfields);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_decode_batch(const HuffDecodeArgs* args, const BatchTask* tasks, uint32_t ntasks,
                             const BatchTask* const_tasks, uint32_t nconst, cudaStream_t st, int num_sms) {
    if (ntasks) {
        const uint32_t cap  = (uint32_t)num_sms * kWinMinBlocks;
        const uint32_t grid = ntasks < cap ? ntasks : cap;
        static std::atomic<unsigned long long> attr{0};
        smem_limit_once(k_huff_decode_win_batch, (int)kWinSmem, attr);
        k_huff_decode_win_batch<<<grid, kWinThreads, kWinSmem, st>>>(args, tasks, ntasks);
        count_launch();
        k_huff_decode_idx_batch<<<grid, 256, 0, st>>>(args, tasks, ntasks);
        count_launch();
    }
    if (nconst) {
        const uint32_t cap = (uint32_t)num_sms * 8;
        k_huff_const_batch<<<nconst < cap ? nconst : cap, 256, 0, st>>>(args, const_tasks, nconst);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

// Constant fill for a one-symbol tree (src/huffman.hh:348-352).
__global__ void k_huff_const(uint16_t* codes, size_t n, const uint32_t* info, uint32_t* seg_zero, uint32_t d0, uint32_t nxs,
                             const int* status) {
    if (*status != VSZ_OK) return;
    const uint16_t c = (uint16_t)info[1];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        codes[i] = c;
        if (c == 0 && seg_zero) {
            size_t row = i / d0;
            uint32_t x = (uint32_t)(i - row * d0);
            atomicAdd(&seg_zero[row * nxs + (x >> 8)], 1u);
        }
    }
}

// ------------------------------------------------------------------------------------------
// K4c: self-synchronising chunk boundaries for streams without an index (reference archives).
// Chunk j owns the codewords that START in [j C, (j+1) C).  Round 0 decodes every chunk from its
// nominal start; each later round re-decodes chunks whose start moved (the exit of chunk j - 1
// from the previous round) until no exit changes.  Tree-Huffman codes resynchronise within a few
// codewords, so this normally converges in two rounds.
// ------------------------------------------------------------------------------------------

__device__ void sync_decode_chunk(const HuffSyncArgs& a, const uint32_t* table, size_t j, unsigned long long start,
                                  unsigned long long* exit_out, uint32_t* cnt_out) {
    const uint32_t base0 = (uint32_t)(reinterpret_cast<uintptr_t>(a.payload) & 3u) * 8u;
    const uint32_t* gw   = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(a.payload) & ~(uintptr_t)3);
    const unsigned long long end = (unsigned long long)(j + 1) * a.chunk_bits;
    BitReader br;
    br.init(gw, base0 + start, base0 + a.payload_bits);
    uint32_t cnt = 0;
    while (br.pos - base0 < end && br.pos - base0 < a.payload_bits) {
        uint32_t s = decode_one(br, table, a.table2, a.child, a.node_sym, a.max_nodes);
        if (s == 0xffffffffu) break;  // padding at the stream end, or a wrong (unsynchronised) start
        cnt++;
    }
    *exit_out = br.pos - base0;
    *cnt_out  = cnt;
}

__global__ void __launch_bounds__(256) k_huff_sync_init(HuffSyncArgs a) {
    __shared__ uint32_t s_table[1 << kDecBits];
    for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) s_table[i] = a.table[i];
    __syncthreads();
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= a.nchunks) return;
    if (*a.status != VSZ_OK) {
        a.start[j] = 0;
        a.exit_a[j] = 0;
        a.count[j] = 0;
        return;
    }
    unsigned long long st = (unsigned long long)j * a.chunk_bits;
    a.start[j] = st;
    sync_decode_chunk(a, s_table, j, st, &a.exit_a[j], &a.count[j]);
}

__global__ void __launch_bounds__(256) k_huff_sync_round(HuffSyncArgs a, const unsigned long long* exit_in,
                                                         unsigned long long* exit_out, int* changed) {
    __shared__ uint32_t s_table[1 << kDecBits];
    for (int i = threadIdx.x; i < (1 << kDecBits); i += blockDim.x) s_table[i] = a.table[i];
    __syncthreads();
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= a.nchunks) return;
    if (*a.status != VSZ_OK) {
        exit_out[j] = exit_in[j];
        return;
    }
    unsigned long long want = (j == 0) ? 0ull : exit_in[j - 1];
    if (want == a.start[j]) {
        exit_out[j] = exit_in[j];
        return;
    }
    a.start[j] = want;
    unsigned long long ex;
    uint32_t c;
    if (want >= (unsigned long long)(j + 1) * a.chunk_bits || want >= a.payload_bits) {
        ex = want;  // the previous chunk's last codeword reaches past this chunk: it owns none
        c  = 0;
    } else {
        sync_decode_chunk(a, s_table, j, want, &ex, &c);
    }
    a.count[j]  = c;
    exit_out[j] = ex;
    if (ex != exit_in[j]) atomicExch(changed, 1);
}

// ------------------------------------------------------------------------------------------
// Generic exclusive scan (decoupled look-back) of u16/u32 values into u64 offsets.
// ------------------------------------------------------------------------------------------

template <typename TIn>
__global__ void __launch_bounds__(256) k_scan_excl(const TIn* __restrict__ in, unsigned long long* __restrict__ out,
                                                   size_t n, unsigned long long* tile_status, uint32_t* tile_counter,
                                                   unsigned long long* total, int* status) {
    constexpr int PER = 16;
    __shared__ unsigned long long s_scan[33];
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const size_t i0     = (size_t)tile * 256 * PER + (size_t)threadIdx.x * PER;
    unsigned long long v[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; k++) {
        v[k] = (i0 + k < n) ? (unsigned long long)in[i0 + k] : 0ull;
        sum += v[k];
    }
    unsigned long long tot;
    unsigned long long ex = block_exclusive_scan<unsigned long long>(sum, s_scan, &tot);
    if (threadIdx.x < 32) {
        const unsigned long long b = lookback_publish_warp(tile_status, tile, tot, status);
        if (threadIdx.x == 0) {
            s_base = b;
            if ((size_t)(tile + 1) * 256 * PER >= n && total) *total = b + tot;
        }
    }
    __syncthreads();
    unsigned long long run = s_base + ex;
#pragma unroll
    for (int k = 0; k < PER; k++) {
        if (i0 + k < n) out[i0 + k] = run;
        run += v[k];
    }
}

// ------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------

void huff_build_prepare() {
    static std::atomic<unsigned long long> attr{0};
    smem_limit_once(k_huff_build<true>, 220 * 1024, attr);
}

int launch_huff_build(HuffBuildArgs a, cudaStream_t st) {
    size_t bytes = build_ws_bytes(a.dict);
    a.ws_in_smem = bytes <= 220 * 1024 ? 1 : 0;
    if (a.ws_in_smem) {
        huff_build_prepare();
        k_huff_build<true><<<1, 256, bytes, st>>>(a);
        count_launch();
    } else {
        k_huff_build<false><<<1, 256, 0, st>>>(a);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

size_t huff_build_scratch_bytes(int dict) { return build_ws_bytes(dict); }

bool huff_build_in_smem(int dict) { return build_ws_bytes(dict) <= 220 * 1024; }

int launch_huff_build_batch(const HuffBuildArgs* args, uint32_t nfields, bool in_smem, int dict_max, cudaStream_t st,
                            int num_sms) {
    if (nfields == 0) return VSZ_OK;
    const uint32_t grid = nfields < (uint32_t)num_sms * 8 ? nfields : (uint32_t)num_sms * 8;
    if (in_smem) {
        static std::atomic<unsigned long long> attr{0};
        smem_limit_once(k_huff_build_batch<true>, 220 * 1024, attr);
        k_huff_build_batch<true><<<grid, 256, build_ws_bytes(dict_max), st>>>(args, nfields);
    } else {
        k_huff_build_batch<false><<<grid, 256, 0, st>>>(args, nfields);
    }
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_encode_batch(const HuffEncodeArgs* args, uint32_t nfields, const BatchTask* tasks, uint32_t ntasks,
                             int cb_dict_max, uint16_t* all_bits, unsigned long long* all_off, size_t total_chunks,
                             unsigned long long* scan_status, uint32_t* scan_counter, int* batch_status,
                             cudaStream_t st, int num_sms) {
    if (ntasks == 0) return VSZ_OK;
    const size_t cb_bytes = (size_t)cb_dict_max * 9;  // fields with cb_in_smem: codebook cached per task
    const size_t smem     = (size_t)8 * kEncWarpWords * 4 + cb_bytes + 16;
    static std::atomic<unsigned long long> attr_pack{0}, attr_count{0};
    smem_limit_once(k_huff_pack_batch, 8 * kEncWarpWords * 4 + 64 * 1024 + 1024, attr_pack);
    smem_limit_once(k_huff_count_batch, 64 * 1024 + 1024, attr_count);
    {
        StageTimer t(kStHuffCount, st);
        const uint32_t grid = ntasks < (uint32_t)num_sms * 8 ? ntasks : (uint32_t)num_sms * 8;
        k_huff_count_batch<<<grid, kEncThreads, (size_t)cb_dict_max, st>>>(args, tasks, ntasks);
        count_launch();
        int rc = launch_scan_u16(all_bits, all_off, total_chunks, scan_status, scan_counter, all_off + total_chunks,
                                 batch_status, st);
        if (rc) return rc;
        k_field_bits<<<(nfields + 127) / 128, 128, 0, st>>>(args, nfields, batch_status);
        count_launch();
    }
    {
        StageTimer t(kStHuffPack, st);
        const uint32_t grid = ntasks < (uint32_t)num_sms * 4 ? ntasks : (uint32_t)num_sms * 4;
        k_huff_pack_batch<<<grid, kEncThreads, smem, st>>>(args, tasks, ntasks);
        count_launch();
        k_huff_encode_edges_batch<<<grid, 256, 0, st>>>(args, tasks, ntasks);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

// Per-field encoder flags a batch table needs (launch_huff_encode sets them for one field).
void huff_encode_prepare(HuffEncodeArgs& a) {
    a.nchunks       = (a.n + kEncChunk - 1) / kEncChunk;
    a.codes_aligned = (reinterpret_cast<uintptr_t>(a.codes) & 15u) == 0;
    a.cb_in_smem    = (size_t)a.dict * 9 <= 64 * 1024 ? 1 : 0;
}

int launch_huff_encode(HuffEncodeArgs a, cudaStream_t st, int num_sms) {
    a.nchunks = (a.n + kEncChunk - 1) / kEncChunk;
    if (a.nchunks == 0) return cudaMemsetAsync(a.total_bits, 0, 8, st) == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
    a.codes_aligned = (reinterpret_cast<uintptr_t>(a.codes) & 15u) == 0;
    size_t cb_bytes = (size_t)a.dict * 9;
    a.cb_in_smem    = cb_bytes <= 64 * 1024 ? 1 : 0;
    size_t smem     = (size_t)8 * kEncWarpWords * 4 + (a.cb_in_smem ? cb_bytes : 0) + 16;
    static std::atomic<unsigned long long> attr_pack{0}, attr_count{0};
    smem_limit_once(k_huff_pack, 8 * kEncWarpWords * 4 + 64 * 1024 + 1024, attr_pack);
    smem_limit_once(k_huff_count, 64 * 1024 + 1024, attr_count);
    const long long blocks = (long long)((a.nchunks + 7) / 8);
    {
        StageTimer t(kStHuffCount, st);
        int grid = (int)min(blocks, (long long)num_sms * 8);
        k_huff_count<<<grid, kEncThreads, a.cb_in_smem ? (size_t)a.dict : 0, st>>>(a);
        count_launch();
        int rc = launch_scan_u16(a.chunk_bits, a.chunk_off, a.nchunks, a.scan_status, a.scan_counter, a.total_bits,
                                 a.status, st);
        if (rc) return rc;
    }
    {
        StageTimer t(kStHuffPack, st);
        int pgrid = (int)min(blocks, (long long)num_sms * 4);
        k_huff_pack<<<pgrid, kEncThreads, smem, st>>>(a);
        count_launch();
        k_huff_encode_edges<<<(unsigned)((a.nchunks + 255) / 256), 256, 0, st>>>(a);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_table(HuffTableArgs a, cudaStream_t st) {
    k_huff_table<<<1, 1024, 0, st>>>(a);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_decode(HuffDecodeArgs a, cudaStream_t st) {
    if (a.nchunks == 0) return VSZ_OK;
    int grid = (int)((a.nchunks + 255) / 256);
    const bool indexed = !a.out_begin && !a.nsym && a.chunk_syms == (uint32_t)kChunkSyms &&
                         (reinterpret_cast<uintptr_t>(a.codes) & 15u) == 0 && a.chunk_len;
    if (indexed) {
        if (a.tree_info) {
            static std::atomic<unsigned long long> attr_win{0};
            smem_limit_once(k_huff_decode_win, (int)kWinSmem, attr_win);
            k_huff_decode_win<<<(unsigned)((a.nchunks + kWinThreads - 1) / kWinThreads), kWinThreads, kWinSmem, st>>>(a);
            count_launch();
        }
        if (a.walk_smem) {
            size_t smem = (size_t)a.nodes * 4;
            static std::atomic<unsigned long long> attr{0};
            smem_limit_once(k_huff_decode_idx<true>, 140 * 1024, attr);
            k_huff_decode_idx<true><<<grid, 256, smem, st>>>(a);
            count_launch();
        } else {
            k_huff_decode_idx<false><<<grid, 256, 0, st>>>(a);
            count_launch();
        }
    } else {
        k_huff_decode<<<grid, 256, 0, st>>>(a);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_const(uint16_t* codes, size_t n, const uint32_t* info, uint32_t* seg_zero, uint32_t d0, uint32_t nxs,
                      const int* status, cudaStream_t st, int num_sms) {
    int grid = (int)min((long long)((n + 255) / 256), (long long)num_sms * 8);
    if (grid < 1) grid = 1;
    k_huff_const<<<grid, 256, 0, st>>>(codes, n, info, seg_zero, d0, nxs, status);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_sync_init(HuffSyncArgs a, cudaStream_t st) {
    if (a.nchunks == 0) return VSZ_OK;
    k_huff_sync_init<<<(unsigned)((a.nchunks + 255) / 256), 256, 0, st>>>(a);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_huff_sync_round(HuffSyncArgs a, const unsigned long long* exit_in, unsigned long long* exit_out, int* changed,
                           cudaStream_t st) {
    k_huff_sync_round<<<(unsigned)((a.nchunks + 255) / 256), 256, 0, st>>>(a, exit_in, exit_out, changed);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

template <typename TIn>
int launch_scan_excl_t(const TIn* in, unsigned long long* out, size_t n, unsigned long long* tile_status,
                       uint32_t* tile_counter, unsigned long long* total, int* status, cudaStream_t st) {
    size_t ntiles = (n + 4095) / 4096;
    if (ntiles == 0) {
        if (total) return cudaMemsetAsync(total, 0, 8, st) == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
        return VSZ_OK;
    }
    if (cudaMemsetAsync(tile_status, 0, 8 * ntiles, st) != cudaSuccess) return VSZ_ERR_CUDA;
    if (cudaMemsetAsync(tile_counter, 0, 4, st) != cudaSuccess) return VSZ_ERR_CUDA;
    k_scan_excl<TIn><<<(unsigned)ntiles, 256, 0, st>>>(in, out, n, tile_status, tile_counter, total, status);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_scan_u16(const uint16_t* in, unsigned long long* out, size_t n, unsigned long long* ts, uint32_t* tc,
                    unsigned long long* total, int* status, cudaStream_t st) {
    return launch_scan_excl_t<uint16_t>(in, out, n, ts, tc, total, status, st);
}
int launch_scan_u32(const uint32_t* in, unsigned long long* out, size_t n, unsigned long long* ts, uint32_t* tc,
                    unsigned long long* total, int* status, cudaStream_t st) {
    return launch_scan_excl_t<uint32_t>(in, out, n, ts, tc, total, status, st);
}

size_t scan_tmp_tiles(size_t n) { return (n + 4095) / 4096; }

int set_spin_limit_huffman(long long polls) { return set_spin_limit_this_unit(polls); }

// Test hook: the device-wide scan of n ones with its tile ticket started at 1 instead of 0, so no
// tile takes ticket 0 and the tile after it waits on a predecessor that never publishes.  That
// wait gives up after the current spin limit and records VSZ_ERR_TIMEOUT, which *status_out
// receives; the scan's later tiles then finish.  Allocates and synchronises (testing only).
int debug_scan_stalled(size_t n, int* status_out) {
    if (n == 0 || n > (1u << 24) || !status_out) return VSZ_ERR_INVALID;
    const size_t ntiles = (n + 4095) / 4096;
    uint32_t* in = nullptr;
    unsigned long long *out = nullptr, *ts = nullptr;
    uint32_t* tc = nullptr;
    int* st      = nullptr;
    int rc       = VSZ_ERR_NOMEM;
    if (cudaMalloc(reinterpret_cast<void**>(&in), 4 * n) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&out), 8 * n) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&ts), 8 * (ntiles + 2)) == cudaSuccess &&  // ticket ntiles publishes too
        cudaMalloc(reinterpret_cast<void**>(&tc), 4) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&st), 4) == cudaSuccess) {
        const uint32_t one = 1;
        rc = VSZ_ERR_CUDA;
        if (cudaMemset(in, 0, 4 * n) == cudaSuccess && cudaMemset(ts, 0, 8 * (ntiles + 2)) == cudaSuccess &&
            cudaMemset(st, 0, 4) == cudaSuccess && cudaMemcpy(tc, &one, 4, cudaMemcpyHostToDevice) == cudaSuccess) {
            k_scan_excl<uint32_t><<<(unsigned)ntiles, 256>>>(in, out, n, ts, tc, nullptr, st);
            count_launch();
            if (cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
                cudaMemcpy(status_out, st, 4, cudaMemcpyDeviceToHost) == cudaSuccess)
                rc = VSZ_OK;
        }
    }
    cudaFree(in);
    cudaFree(out);
    cudaFree(ts);
    cudaFree(tc);
    cudaFree(st);
    return rc;
}

}  // namespace vsz
