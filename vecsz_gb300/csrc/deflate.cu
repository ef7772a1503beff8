// The -L gzip pass on the GPU: a deflate (RFC 1951) encoder writing a zlib stream (RFC 1950), the
// container the reference's lossless pass produces and detects (src/lossless.hh:40-57 isZlibFormat,
// :84-142 zlib_compress at level 3; src/vecsz_interface.hh:206-217, :237-243).  The stream decodes
// with any inflate, the reference's included; its bytes are not zlib's (a different match search).
//
// Layout of the work.  The input is cut into 16 KiB chunks (kDeflateChunk), one CTA each, two CTAs
// per SM.  Matches never reach back before their chunk, so chunks are independent:
//   1. candidates: eight warps each sweep 2 KiB of the chunk, 32 positions a step, and record for
//      every position the previous position with the same 4-byte hash (within the step by
//      __match_any_sync, before it from the warp's hash head table); a position without one
//      takes the last occurrence in the nearest earlier 2 KiB range from that range's final head
//      table.  The records form hash chains, as zlib's prev[] does.
//   2. parse: thread t parses bytes [64 t, 64 t + 64) greedily, following up to kChain chain
//      links per position; matches end at the thread's range end.  Tokens go to shared memory,
//      symbol counts to shared histograms.
//   3. codes: length-limited (15-bit) Huffman codes for literal/length and distance symbols and
//      a 7-bit code-length code; the block is emitted with dynamic codes, the fixed codes or
//      stored, whichever is shortest.
//   4. emit: a block scan of per-thread bit counts places every thread's tokens; bits go to a
//      shared buffer, then to the chunk's staging slot in global memory.  A dynamic or fixed
//      block is followed by an empty stored block (a sync flush), so every chunk ends on a byte.
// k_deflate_finish (one CTA) then scans the chunk sizes, combines the per-chunk Adler-32 sums and
// writes the zlib header and tail; k_deflate_copy moves the chunks into place.
#include <cstdint>

#include <cuda_runtime.h>

#include "deflate_format.h"
#include "vsz_types.h"

namespace vsz {
void count_launch();  // vsz_profile.cu
}

namespace {

constexpr int kChunk      = vsz::kDeflateChunk;  // input bytes per chunk
constexpr int kThreads    = 256;
constexpr int kSeg        = kChunk / kThreads;  // 64 bytes parsed per thread
constexpr int kWarps      = kThreads / 32;
constexpr int kRange      = kChunk / kWarps;    // 2048 positions swept per warp
constexpr int kHashBits   = 11;                 // a head table of kRange entries per warp
constexpr int kHashSize   = 1 << kHashBits;
constexpr int kChain      = 4;
constexpr int kTooFar     = 4096;    // 3-byte matches farther than this are not worth it (zlib's rule)
constexpr uint16_t kNone  = 0xFFFF;
constexpr int kSlot       = kChunk + 64;  // staging bytes per chunk: a stored block is kChunk + 5
constexpr uint32_t kAdlerMod = 65521;

constexpr int kLitSyms  = 286;
constexpr int kDistSyms = 30;
constexpr int kClSyms   = 19;
// transmission order of the code-length code lengths (RFC 1951 3.2.7)
__constant__ uint8_t kClOrder[kClSyms] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// shared-memory layout (bytes)
constexpr int kDataBytes = kChunk + 16;          // chunk bytes, zero padded for word reads
constexpr int kPrevBytes = 2 * kChunk;           // prev[] (phases 1-2), then the output bits
constexpr int kHeadBytes = 2 * kHashSize * kWarps;  // head tables (phase 1), then the tokens
constexpr int kTagBytes  = kHashSize * kWarps;      // per-warp lane tags of the candidate sweep
static_assert(kHeadBytes == 2 * kChunk, "one u16 token slot per position");
static_assert(kChunk <= 32768 && kSeg * kThreads == kChunk, "distances within the zlib window");
static_assert(kPrevBytes >= kChunk + 256, "bit buffer holds any block shorter than a stored one");

struct DeflateSmem {
    uint32_t lit_freq[kLitSyms + 2];
    uint32_t dist_freq[kDistSyms + 2];
    uint32_t cl_freq[kClSyms + 1];
    uint16_t lit_code[kLitSyms + 2];
    uint8_t lit_len[kLitSyms + 2];
    uint16_t dist_code[kDistSyms + 2];
    uint8_t dist_len[kDistSyms + 2];
    uint16_t cl_code[kClSyms + 1];
    uint8_t cl_len[kClSyms + 1];
    // Huffman build: counts with the two-symbol minimum, symbols by ascending count, scratch
    uint32_t lf[kLitSyms + 2], df[kDistSyms + 2], cf[kClSyms + 1];
    uint16_t sorted_lit[kLitSyms + 2], sorted_dist[kDistSyms + 2], sorted_cl[kClSyms + 1];
    uint32_t iw[kLitSyms + 2];
    uint16_t parent[2 * kLitSyms + 4];
    uint8_t depth[2 * kLitSyms + 4];
    uint16_t bl_count[24];
    // code-length RLE of the dynamic header: sym | extra << 5
    uint16_t rle[kLitSyms + kDistSyms + 4];
    uint32_t nrle;
    uint32_t ntok[kThreads];
    uint32_t bits[kThreads];  // per-thread token bits, then their exclusive prefix
    uint32_t extra_bits;
    uint32_t adler_s[kThreads], adler_t[kThreads];
    uint32_t header_bits;     // bits of the block header
    uint32_t eob_pos, flush_pos;  // end-of-block code; byte-aligned LEN/NLEN of the sync flush
    float wpart_ent[kWarps];      // per-warp partial sums of the bounds
    uint32_t wpart_fixed[kWarps];
    uint32_t wsum[kWarps];        // per-warp bit totals of the emit scan
    uint32_t nlit_syms, ndist_syms;  // literal/length and distance symbols of the parse
    uint64_t fixed_bits;
    int skip_dynamic;
    int nlit, ndist, ncl;
    int btype;   // 0 stored, 1 fixed, 2 dynamic
    int dyn_ok;  // the dynamic codes were built
    uint64_t pb_part[kWarps];          // per-warp payload bits of the dynamic codes
    uint32_t cnt[3][16], next[3][16];  // per alphabet (literal/length, distance, code length): codes per length, first code
};

constexpr size_t kSmemBytes = kDataBytes + kPrevBytes + kHeadBytes + kTagBytes;  // dynamic part

__device__ __forceinline__ uint32_t load_word(const uint32_t* w, uint32_t i) {
    return __funnelshift_r(w[i >> 2], w[(i >> 2) + 1], (i & 3) * 8);
}

__device__ __forceinline__ uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHashBits); }

// length 3..258 -> symbol index 0..28 (symbol 257 + index), extra bits and their value
__device__ __forceinline__ void length_symbol(uint32_t len, uint32_t& idx, uint32_t& ebits, uint32_t& evalue) {
    const uint32_t v = len - 3;
    if (v < 8) {
        idx = v, ebits = 0, evalue = 0;
    } else if (v == 255) {
        idx = 28, ebits = 0, evalue = 0;
    } else {
        const uint32_t e = 31 - __clz(v) - 2;
        idx = 4 * e + (v >> e), ebits = e, evalue = v & ((1u << e) - 1);
    }
}

// distance 1..32768 -> symbol 0..29, extra bits and their value
__device__ __forceinline__ void distance_symbol(uint32_t dist, uint32_t& sym, uint32_t& ebits, uint32_t& evalue) {
    const uint32_t v = dist - 1;
    if (v < 4) {
        sym = v, ebits = 0, evalue = 0;
    } else {
        const uint32_t e = 31 - __clz(v) - 1;
        sym = 2 * e + 2 + ((v >> e) & 1), ebits = e, evalue = v & ((1u << e) - 1);
    }
}

// Fixed-code lengths (RFC 1951 3.2.6)
__device__ __forceinline__ uint32_t fixed_lit_len(uint32_t s) { return s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8; }
__device__ __forceinline__ uint32_t fixed_lit_code(uint32_t s) {
    return s < 144 ? 0x30 + s : s < 256 ? 0x190 + (s - 144) : s < 280 ? s - 256 : 0xC0 + (s - 280);
}

__device__ __forceinline__ uint32_t reverse_bits(uint32_t code, uint32_t len) { return __brev(code) >> (32 - len); }

// Rank the symbols in use by (frequency, symbol), all threads of the CTA: sorted[rank] = symbol.
// Returns the number of symbols in use (to every thread, after a barrier).
__device__ __forceinline__ int rank_symbols(const uint32_t* freq, int n, uint16_t* sorted) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t f = freq[i];
        if (!f) continue;
        int r = 0;
        for (int j = 0; j < n; j++) {
            const uint32_t g = freq[j];
            r += g && (g < f || (g == f && j < i));
        }
        sorted[r] = (uint16_t)i;
    }
    int m = 0;
    for (int j = 0; j < n; j++) m += freq[j] != 0;
    __syncthreads();
    return m;
}

// Length-limited Huffman code lengths (one thread).  sorted[0..m) holds the symbols in use by
// ascending (frequency, symbol), m >= 2; len[] is zero on entry and stays zero for the others.  Returns false if the limit
// cannot be met with a complete code (the caller then uses another block type).
__device__ __forceinline__ bool lengths_from_sorted(const uint32_t* freq, const uint16_t* sorted, int m, int n, int limit,
                                    uint8_t* len, DeflateSmem& s) {
    (void)n;  // len[0..n) is zero on entry: only the used symbols are written
    if (m < 2) return false;
    // two-queue Huffman: leaves 0..m-1 by ascending weight, internal nodes m..2m-2 in creation
    // order (their weights come out nondecreasing, so the queue head is the lightest)
    int leaf = 0, node = m, made = m;
    for (int k = 0; k < m - 1; k++) {
        int pick[2];
        uint32_t wsum = 0;
        for (int q = 0; q < 2; q++) {
            const uint32_t lw = leaf < m ? freq[sorted[leaf]] : 0;
            if (leaf < m && (node >= made || lw <= s.iw[node - m])) {
                pick[q] = leaf++;
                wsum += lw;
            } else {
                pick[q] = node;
                wsum += s.iw[node - m];
                node++;
            }
        }
        s.iw[made - m]    = wsum;
        s.parent[pick[0]] = (uint16_t)made;
        s.parent[pick[1]] = (uint16_t)made;
        made++;
    }
    const int root = made - 1;
    s.depth[root]  = 0;
    for (int k = root - 1; k >= m; k--) s.depth[k] = (uint8_t)min(255, s.depth[s.parent[k]] + 1);
    for (int i = 0; i < 24; i++) s.bl_count[i] = 0;
    int overflow = 0;
    for (int i = 0; i < m; i++) {
        int d = s.depth[s.parent[i]] + 1;
        if (d > limit) {
            d = limit;
            overflow++;
        }
        s.bl_count[d]++;
    }
    // zlib's gen_bitlen adjustment: move leaves up until the code is complete again
    while (overflow > 0) {
        int bits = limit - 1;
        while (bits > 0 && s.bl_count[bits] == 0) bits--;
        if (bits == 0) return false;
        s.bl_count[bits]--;
        s.bl_count[bits + 1] += 2;
        s.bl_count[limit]--;
        overflow -= 2;
    }
    uint32_t kraft = 0, leaves = 0;  // a complete code over the m symbols: sum of 2^(limit - l) == 2^limit
    for (int l = 1; l <= limit; l++) {
        kraft += (uint32_t)s.bl_count[l] << (limit - l);
        leaves += s.bl_count[l];
    }
    if (kraft != (1u << limit) || leaves != (uint32_t)m) return false;
    // the least frequent symbols take the longest codes
    int k = 0;
    for (int l = limit; l >= 1; l--)
        for (int c = 0; c < s.bl_count[l]; c++) len[sorted[k++]] = (uint8_t)l;
    return true;
}

// shared-memory bit writer: atomics because neighbouring threads share boundary words
__device__ __forceinline__ void put_bits(uint32_t* out, uint32_t& pos, uint32_t v, uint32_t n) {
    if (n == 0) return;
    const uint32_t word = pos >> 5, sh = pos & 31;
    atomicOr(&out[word], v << sh);
    if (sh + n > 32) atomicOr(&out[word + 1], v >> (32 - sh));
    pos += n;
}

__global__ void __launch_bounds__(kThreads, 2)
    k_deflate_chunks(const uint8_t* __restrict__ in, size_t len, uint8_t* __restrict__ staging,
                     uint32_t* __restrict__ sizes, uint32_t* __restrict__ adler, uint32_t* __restrict__ kinds) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint8_t* data   = smem;
    uint32_t* dataw = reinterpret_cast<uint32_t*>(smem);
    uint16_t* prev  = reinterpret_cast<uint16_t*>(smem + kDataBytes);
    uint32_t* outw  = reinterpret_cast<uint32_t*>(smem + kDataBytes);  // after the parse
    uint16_t* head  = reinterpret_cast<uint16_t*>(smem + kDataBytes + kPrevBytes);
    uint16_t* tok   = head;  // after the candidate sweep
    uint8_t* tags   = smem + kDataBytes + kPrevBytes + kHeadBytes;
    __shared__ DeflateSmem s;  // static, so every access is known to be to shared memory

    const int tid   = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const size_t c0 = (size_t)blockIdx.x * kChunk;
    const int n     = (int)min((size_t)kChunk, len - c0);

    // ---- load the chunk; zero the padding, the head tables and the histograms ----
    const uint8_t* src = in + c0;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        for (int i = tid; i < n / 16; i += kThreads)
            reinterpret_cast<uint4*>(data)[i] = reinterpret_cast<const uint4*>(src)[i];
        for (int i = (n & ~15) + tid; i < n; i += kThreads) data[i] = src[i];
    } else {
        for (int i = tid; i < n; i += kThreads) data[i] = src[i];
    }
    for (int i = n + tid; i < kDataBytes; i += kThreads) data[i] = 0;
    for (int i = tid; i < kHashSize * kWarps / 2; i += kThreads) reinterpret_cast<uint32_t*>(head)[i] = 0xFFFFFFFFu;
    for (int i = tid; i < kLitSyms + 2; i += kThreads) s.lit_freq[i] = 0;
    if (tid < kDistSyms + 2) s.dist_freq[tid] = 0;
    if (tid < kClSyms + 1) s.cl_freq[tid] = 0;
    if (tid == 0) s.extra_bits = 0, s.nlit_syms = 1, s.ndist_syms = 0;
    __syncthreads();

    // ---- Adler-32 parts of this thread's 128 bytes (as a standalone sequence) ----
    {
        const int b0 = tid * kSeg, b1 = min(n, b0 + kSeg);
        uint32_t S = 0, T = 0;
        for (int i = b0; i < b1; i++) {
            S += data[i];  // <= 128 * 255
            T += S;        // <= 128 * 128 * 255 < 2^22
        }
        s.adler_s[tid] = S % kAdlerMod;
        s.adler_t[tid] = T % kAdlerMod;
    }

    // ---- 1. candidates ----
    {
        uint16_t* h     = head + warp * kHashSize;
        uint8_t* tag    = tags + warp * kHashSize;
        const int base  = warp * kRange;
        for (int step = 0; step < kRange / 32; step++) {
            const int i      = base + step * 32 + lane;
            const bool valid = i + 4 <= n;
            const uint32_t hv = valid ? hash4(load_word(dataw, i)) : (uint32_t)(kHashSize + lane);
            // distinct hashes in this step (the common case on varied data) need no grouping:
            // one lane of each shared hash loses the tag write and flags the step
            if (valid) tag[hv] = (uint8_t)lane;
            __syncwarp();
            const bool dup = valid && tag[hv] != lane;
            uint16_t cand  = kNone;
            if (__ballot_sync(0xFFFFFFFFu, dup) == 0) {
                if (valid) cand = h[hv];
                __syncwarp();
                if (valid) h[hv] = (uint16_t)i;
            } else {
                const uint32_t same  = __match_any_sync(0xFFFFFFFFu, hv);
                const uint32_t lower = same & ((1u << lane) - 1);
                if (valid) cand = lower ? (uint16_t)(base + step * 32 + (31 - __clz(lower))) : h[hv];
                __syncwarp();
                if (valid && (same >> lane) == 1u) h[hv] = (uint16_t)i;  // the last lane of each group
            }
            prev[i] = cand;
            __syncwarp();
        }
    }
    __syncthreads();
    // positions with no earlier occurrence in their own range: nearest earlier range's last one
    for (int i = tid; i < n; i += kThreads) {
        const int w = i / kRange;
        if (w == 0 || prev[i] != kNone || i + 4 > n) continue;
        const uint32_t hv = hash4(load_word(dataw, i));
        for (int k = w - 1; k >= 0; k--) {
            const uint16_t c = head[k * kHashSize + hv];
            if (c != kNone) {
                prev[i] = c;
                break;
            }
        }
    }
    __syncthreads();

    // ---- 2. parse ----
    // tokens: literal = byte; match = 0x8000 | (len - 3), then distance - 1
    {
        const int b0 = tid * kSeg, b1 = min(n, b0 + kSeg);
        uint16_t* t  = tok + tid * kSeg;
        int nt = 0, nmatch = 0;
        uint32_t extra = 0;
        int i = b0;
        while (i < b1) {
            const int limit = min(258, b1 - i);
            int best = 0, best_c = 0;
            if (limit >= 3) {
                const uint32_t w0 = load_word(dataw, i);
                int c = prev[i];
                for (int depth = 0; depth < kChain && c != kNone; depth++) {
                    const int next = prev[c];  // the next link, loaded ahead of the compare
                    uint32_t x     = load_word(dataw, c) ^ w0;
                    // a candidate must share the first 3 bytes (hash collisions usually do not)
                    if ((x & 0xFFFFFFu) == 0) {
                        int k = 0;
                        while (true) {
                            if (x) {
                                k += (__ffs(x) - 1) >> 3;
                                break;
                            }
                            k += 4;
                            if (k >= limit) break;
                            x = load_word(dataw, c + k) ^ load_word(dataw, i + k);
                        }
                        k = min(k, limit);
                        if (k > best) {
                            best   = k;
                            best_c = c;
                            if (k == limit) break;
                        }
                    }
                    c = next;
                }
            }
            if (best >= 4 || (best == 3 && i - best_c <= kTooFar)) {
                uint32_t li, le, lv, ds, de, dv;
                length_symbol(best, li, le, lv);
                distance_symbol(i - best_c, ds, de, dv);
                atomicAdd(&s.lit_freq[257 + li], 1u);
                atomicAdd(&s.dist_freq[ds], 1u);
                extra += le + de;
                t[nt++] = (uint16_t)(0x8000 | (best - 3));
                t[nt++] = (uint16_t)(i - best_c - 1);
                nmatch++;
                i += best;
            } else {
                atomicAdd(&s.lit_freq[data[i]], 1u);
                t[nt++] = data[i];
                i++;
            }
        }
        s.ntok[tid] = nt;
        atomicAdd(&s.extra_bits, extra);
        atomicAdd(&s.nlit_syms, (uint32_t)(nt - nmatch));
        atomicAdd(&s.ndist_syms, (uint32_t)nmatch);
    }
    if (tid == 0) s.lit_freq[256] = 1;  // end of block
    __syncthreads();

    // ---- 3. codes and block type ----
    // First, by all threads: the fixed-code bits, and the entropy of the symbol counts, a lower
    // bound on the payload of any code built from them.  A chunk whose dynamic block could not
    // save 1/256 of a stored block's size is stored (or fixed-coded) without building codes.
    {
        const float l2n_lit = __log2f((float)s.nlit_syms), l2n_dist = __log2f((float)max(s.ndist_syms, 1u));
        float ent      = 0.f;
        uint32_t fixed = 0;
        for (int i = tid; i < kLitSyms + kDistSyms; i += kThreads) {
            const bool lit    = i < kLitSyms;
            const uint32_t f  = lit ? s.lit_freq[i] : s.dist_freq[i - kLitSyms];
            if (f) ent += (float)f * ((lit ? l2n_lit : l2n_dist) - __log2f((float)f));
            fixed += f * (lit ? fixed_lit_len(i) : 5u);
        }
        for (int off = 16; off > 0; off >>= 1) {
            ent += __shfl_xor_sync(0xFFFFFFFFu, ent, off);
            fixed += __shfl_xor_sync(0xFFFFFFFFu, fixed, off);
        }
        if (lane == 0) s.wpart_ent[warp] = ent, s.wpart_fixed[warp] = fixed;
        __syncthreads();
        if (tid == 0) {
            float e        = 0.f;
            uint64_t fb    = 3 + (uint64_t)s.extra_bits;
            for (int w = 0; w < kWarps; w++) e += s.wpart_ent[w], fb += s.wpart_fixed[w];
            const uint64_t stored_bits = 8 * (uint64_t)(5 + n);
            const double lower         = (double)e * 0.999 + s.extra_bits + 3 + 14 + 12 + 42;
            s.fixed_bits               = fb;
            s.skip_dynamic             = lower >= (double)(stored_bits - stored_bits / 256);
        }
        // the dynamic codes need two used symbols per alphabet: unused ones get a count of one
        // for the tree only (their codes are never emitted)
        for (int i = tid; i < kLitSyms + kDistSyms; i += kThreads) {
            if (i < kLitSyms) s.lf[i] = s.lit_freq[i];
            else s.df[i - kLitSyms] = s.dist_freq[i - kLitSyms];
        }
        __syncthreads();
        if (tid == 0) {  // usually stops after the first few symbols
            int lu = 0, du = 0;
            for (int i = 0; i < kLitSyms && lu < 2; i++) lu += s.lit_freq[i] != 0;
            for (int i = 0; i < kDistSyms && du < 2; i++) du += s.dist_freq[i] != 0;
            for (int i = 0; lu < 2 && i < kLitSyms; i++)
                if (!s.lf[i]) s.lf[i] = 1, lu++;
            for (int i = 0; du < 2 && i < kDistSyms; i++)
                if (!s.df[i]) s.df[i] = 1, du++;
        }
        __syncthreads();
    }
    const bool try_dynamic = !s.skip_dynamic;
    int m_lit = 0, m_dist = 0;
    for (int k = tid; k < kLitSyms + kDistSyms + kClSyms + 4; k += kThreads) {
        if (k < kLitSyms + 2) s.lit_len[k] = 0;
        else if (k < kLitSyms + kDistSyms + 4) s.dist_len[k - kLitSyms - 2] = 0;
        else if (k - kLitSyms - kDistSyms - 4 < kClSyms + 1) s.cl_len[k - kLitSyms - kDistSyms - 4] = 0;
    }
    __syncthreads();
    if (try_dynamic) {
        m_lit  = rank_symbols(s.lf, kLitSyms, s.sorted_lit);
        m_dist = rank_symbols(s.df, kDistSyms, s.sorted_dist);
    }
    if (tid == 0) {  // the code lengths and the dynamic header: serial, on small alphabets
        bool dyn_ok = try_dynamic && lengths_from_sorted(s.lf, s.sorted_lit, m_lit, kLitSyms, 15, s.lit_len, s) &&
                      lengths_from_sorted(s.df, s.sorted_dist, m_dist, kDistSyms, 15, s.dist_len, s);
        if (dyn_ok) {
            int nlit = kLitSyms, ndist = kDistSyms;
            while (nlit > 257 && s.lit_len[nlit - 1] == 0) nlit--;
            while (ndist > 1 && s.dist_len[ndist - 1] == 0) ndist--;
            // run-length code of the code lengths (RFC 1951 3.2.7); runs may cross from the
            // literal/length lengths into the distance lengths
            uint32_t nr = 0;
            const int total = nlit + ndist;
            auto L = [&](int k) -> int { return k < nlit ? s.lit_len[k] : s.dist_len[k - nlit]; };
            for (int i = 0; i < kClSyms; i++) s.cl_freq[i] = 0;
            int i = 0;
            while (i < total) {
                const int cur = L(i);
                int run = 1;
                while (i + run < total && L(i + run) == cur) run++;
                if (cur == 0) {
                    int r = run;
                    while (r >= 11) {
                        const int q = min(r, 138);
                        s.rle[nr++] = (uint16_t)(18 | ((q - 11) << 5));
                        s.cl_freq[18]++;
                        r -= q;
                    }
                    if (r >= 3) {
                        s.rle[nr++] = (uint16_t)(17 | ((r - 3) << 5));
                        s.cl_freq[17]++;
                        r = 0;
                    }
                    for (; r > 0; r--) {
                        s.rle[nr++] = 0;
                        s.cl_freq[0]++;
                    }
                } else {
                    s.rle[nr++] = (uint16_t)cur;
                    s.cl_freq[cur]++;
                    int r = run - 1;
                    while (r >= 3) {
                        const int q = min(r, 6);
                        s.rle[nr++] = (uint16_t)(16 | ((q - 3) << 5));
                        s.cl_freq[16]++;
                        r -= q;
                    }
                    for (; r > 0; r--) {
                        s.rle[nr++] = (uint16_t)cur;
                        s.cl_freq[cur]++;
                    }
                }
                i += run;
            }
            s.nrle = nr;
            int cused = 0;
            for (int k = 0; k < kClSyms; k++) cused += (s.cf[k] = s.cl_freq[k]) != 0;
            for (int k = 0; cused < 2 && k < kClSyms; k++)
                if (!s.cf[k]) s.cf[k] = 1, cused++;
            // 19 symbols: insertion sort by (count, symbol)
            int m_cl = 0;
            for (int k = 0; k < kClSyms; k++) {
                if (!s.cf[k]) continue;
                int j = m_cl++;
                while (j > 0 && s.cf[s.sorted_cl[j - 1]] > s.cf[k]) {
                    s.sorted_cl[j] = s.sorted_cl[j - 1];
                    j--;
                }
                s.sorted_cl[j] = (uint16_t)k;
            }
            dyn_ok = lengths_from_sorted(s.cf, s.sorted_cl, m_cl, kClSyms, 7, s.cl_len, s);
            if (dyn_ok) {
                int ncl = kClSyms;
                while (ncl > 4 && s.cl_len[kClOrder[ncl - 1]] == 0) ncl--;
                uint64_t hb = 3 + 5 + 5 + 4 + 3 * (uint64_t)ncl;
                for (uint32_t r = 0; r < nr; r++) {
                    const uint32_t sym = s.rle[r] & 31;
                    hb += s.cl_len[sym] + (sym == 16 ? 2 : sym == 17 ? 3 : sym == 18 ? 7 : 0);
                }
                s.nlit        = nlit;
                s.ndist       = ndist;
                s.ncl         = ncl;
                s.header_bits = (uint32_t)hb;
            }
        }
        s.dyn_ok = dyn_ok;
    }
    __syncthreads();
    // payload bits of the dynamic codes (block reduction), then the block type (thread 0)
    if (s.dyn_ok) {
        uint64_t pb = 0;
        for (int k = tid; k < kLitSyms + kDistSyms; k += kThreads)
            pb += k < kLitSyms ? (uint64_t)s.lit_freq[k] * s.lit_len[k]
                               : (uint64_t)s.dist_freq[k - kLitSyms] * s.dist_len[k - kLitSyms];
        for (int off = 16; off > 0; off >>= 1) pb += __shfl_xor_sync(0xffffffffu, pb, off);
        if (lane == 0) s.pb_part[warp] = pb;
    }
    for (int i = tid; i < 3 * 16; i += kThreads) (&s.cnt[0][0])[i] = 0u;
    __syncthreads();
    if (tid == 0) {
        uint64_t dyn_bits = ~0ull;
        if (s.dyn_ok) {
            dyn_bits = (uint64_t)s.header_bits + s.extra_bits;
            for (int w = 0; w < kWarps; w++) dyn_bits += s.pb_part[w];
        }
        // a dynamic or fixed block is followed by an empty stored block: 3 bits, pad, 4 bytes
        const uint64_t flush       = 3 + 7 + 32;
        const uint64_t stored_bits = 8 * (uint64_t)(5 + n);
        int bt        = 0;
        uint64_t best = stored_bits;
        if (s.fixed_bits + flush < best) bt = 1, best = s.fixed_bits + flush;
        if (s.dyn_ok && dyn_bits + flush < best) bt = 2, best = dyn_bits + flush;
        s.btype = bt;
        if (bt == 1) s.header_bits = 3;
    }
    __syncthreads();
    if (s.btype == 1) {  // the fixed codes (RFC 1951 3.2.6)
        for (int k = tid; k < kLitSyms + kDistSyms; k += kThreads) {
            if (k < kLitSyms) {
                s.lit_len[k]  = (uint8_t)fixed_lit_len(k);
                s.lit_code[k] = (uint16_t)reverse_bits(fixed_lit_code(k), fixed_lit_len(k));
            } else {
                s.dist_len[k - kLitSyms]  = 5;
                s.dist_code[k - kLitSyms] = (uint16_t)reverse_bits(k - kLitSyms, 5);
            }
        }
    } else if (s.btype == 2) {  // canonical codes (RFC 1951 3.2.2) of the three alphabets
        const uint8_t* lens[3] = {s.lit_len, s.dist_len, s.cl_len};
        uint16_t* codes[3]     = {s.lit_code, s.dist_code, s.cl_code};
        const int nsym[3]      = {kLitSyms, kDistSyms, kClSyms};
        for (int k = tid; k < kLitSyms + kDistSyms + kClSyms; k += kThreads) {
            const int a = k < kLitSyms ? 0 : (k < kLitSyms + kDistSyms ? 1 : 2);
            const int i = k - (a == 0 ? 0 : a == 1 ? kLitSyms : kLitSyms + kDistSyms);
            if (lens[a][i]) atomicAdd(&s.cnt[a][lens[a][i]], 1u);
        }
        __syncthreads();
        if (tid < 3) {
            uint32_t c = 0;
            s.next[tid][0] = 0;
            for (int l = 1; l < 16; l++) {
                c              = (c + (l > 1 ? s.cnt[tid][l - 1] : 0u)) << 1;
                s.next[tid][l] = c;
            }
        }
        __syncthreads();
        for (int k = tid; k < kLitSyms + kDistSyms + kClSyms; k += kThreads) {
            const int a  = k < kLitSyms ? 0 : (k < kLitSyms + kDistSyms ? 1 : 2);
            const int i  = k - (a == 0 ? 0 : a == 1 ? kLitSyms : kLitSyms + kDistSyms);
            const int l  = lens[a][i];
            uint32_t rnk = 0;  // symbols before i with the same length
            if (l)
                for (int j = 0; j < i; j++) rnk += lens[a][j] == l;
            codes[a][i] = l ? (uint16_t)reverse_bits(s.next[a][l] + rnk, l) : 0;
        }
        (void)nsym;
    }
    __syncthreads();
    const int bt = s.btype;

    uint32_t chunk_bytes;
    if (bt == 0) {
        // stored: [BFINAL 0, BTYPE 00, pad][LEN][NLEN][bytes]
        uint8_t* dst = staging + (size_t)blockIdx.x * kSlot;
        if (tid == 0) {
            dst[0] = 0;
            dst[1] = (uint8_t)(n & 0xFF);
            dst[2] = (uint8_t)(n >> 8);
            dst[3] = (uint8_t)(~n & 0xFF);
            dst[4] = (uint8_t)((~n >> 8) & 0xFF);
        }
        for (int i = tid; i < n; i += kThreads) dst[5 + i] = data[i];
        chunk_bytes = 5 + n;
    } else {
        // ---- 4. bit counts, their prefix, then the bits ----
        uint32_t nb = 0;
        {
            const uint16_t* t = tok + tid * kSeg;
            const int nt      = s.ntok[tid];
            for (int k = 0; k < nt; k++) {
                const uint32_t v = t[k];
                if (v & 0x8000) {
                    uint32_t li, le, lv, ds, de, dv;
                    length_symbol((v & 0xFF) + 3, li, le, lv);
                    distance_symbol(t[++k] + 1u, ds, de, dv);
                    nb += s.lit_len[257 + li] + le + s.dist_len[ds] + de;
                } else {
                    nb += s.lit_len[v];
                }
            }
        }
        // exclusive prefix of the bit counts (block scan), after the block header
        uint32_t incl = nb;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= off) incl += v;
        }
        if (lane == 31) s.wsum[warp] = incl;
        // the parse area (prev[]) becomes the bit buffer: clear it
        __syncthreads();
        const int out_words = (kPrevBytes / 4);
        for (int i = tid; i < out_words; i += kThreads) outw[i] = 0;
        uint32_t woff = s.header_bits;
        for (int w = 0; w < warp; w++) woff += s.wsum[w];
        s.bits[tid] = woff + incl - nb;
        if (tid == kThreads - 1) {
            // end of block, then the empty stored block's 3 header bits, padded to the byte
            s.eob_pos   = woff + incl;
            s.flush_pos = (woff + incl + s.lit_len[256] + 3 + 7) & ~7u;
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t pos = 0;
            put_bits(outw, pos, 0, 1);       // BFINAL = 0
            put_bits(outw, pos, bt, 2);      // BTYPE
            if (bt == 2) {
                put_bits(outw, pos, s.nlit - 257, 5);
                put_bits(outw, pos, s.ndist - 1, 5);
                put_bits(outw, pos, s.ncl - 4, 4);
                for (int k = 0; k < s.ncl; k++) put_bits(outw, pos, s.cl_len[kClOrder[k]], 3);
                for (uint32_t r = 0; r < s.nrle; r++) {
                    const uint32_t sym = s.rle[r] & 31, ev = s.rle[r] >> 5;
                    put_bits(outw, pos, s.cl_code[sym], s.cl_len[sym]);
                    if (sym == 16) put_bits(outw, pos, ev, 2);
                    if (sym == 17) put_bits(outw, pos, ev, 3);
                    if (sym == 18) put_bits(outw, pos, ev, 7);
                }
            }
            // end of block and the sync flush (empty stored block)
            uint32_t p = s.eob_pos;
            put_bits(outw, p, s.lit_code[256], s.lit_len[256]);
            put_bits(outw, p, 0, 3);
            p = s.flush_pos;
            put_bits(outw, p, 0x0000u, 16);
            put_bits(outw, p, 0xFFFFu, 16);
        }
        {
            uint32_t pos      = s.bits[tid];
            const uint16_t* t = tok + tid * kSeg;
            const int nt      = s.ntok[tid];
            for (int k = 0; k < nt; k++) {
                const uint32_t v = t[k];
                if (v & 0x8000) {
                    uint32_t li, le, lv, ds, de, dv;
                    length_symbol((v & 0xFF) + 3, li, le, lv);
                    distance_symbol(t[++k] + 1u, ds, de, dv);
                    put_bits(outw, pos, s.lit_code[257 + li], s.lit_len[257 + li]);
                    put_bits(outw, pos, lv, le);
                    put_bits(outw, pos, s.dist_code[ds], s.dist_len[ds]);
                    put_bits(outw, pos, dv, de);
                } else {
                    put_bits(outw, pos, s.lit_code[v], s.lit_len[v]);
                }
            }
        }
        __syncthreads();
        chunk_bytes = s.flush_pos / 8 + 4;
        uint32_t* dst = reinterpret_cast<uint32_t*>(staging + (size_t)blockIdx.x * kSlot);
        for (uint32_t i = tid; i < (chunk_bytes + 3) / 4; i += kThreads) dst[i] = outw[i];
    }

    // ---- Adler-32 of the chunk: ordered combination of the per-thread parts ----
    if (warp == 0) {
        // lane L combines threads 8L .. 8L+7 in order, then lanes combine in order
        uint64_t S = 0, T = 0, N = 0;
        for (int k = 0; k < 8; k++) {
            const int th = lane * 8 + k;
            const int b0 = th * kSeg, cnt = max(0, min(n, b0 + kSeg) - b0);
            T = (T + s.adler_t[th] + (uint64_t)cnt * S) % kAdlerMod;
            S = (S + s.adler_s[th]) % kAdlerMod;
            N += cnt;
        }
        for (int off = 1; off < 32; off <<= 1) {
            // combine (left = lane - off) with (right = this lane), leftmost lanes keep theirs
            const uint64_t S_l = __shfl_up_sync(0xFFFFFFFFu, S, off);
            const uint64_t T_l = __shfl_up_sync(0xFFFFFFFFu, T, off);
            const uint64_t N_l = __shfl_up_sync(0xFFFFFFFFu, N, off);
            if (lane >= off) {
                T = (T_l + T + (N % kAdlerMod) * S_l) % kAdlerMod;
                S = (S_l + S) % kAdlerMod;
                N = N_l + N;
            }
        }
        if (lane == 31) {
            sizes[blockIdx.x]         = chunk_bytes;
            adler[2 * blockIdx.x]     = (uint32_t)S;
            adler[2 * blockIdx.x + 1] = (uint32_t)T;
            kinds[blockIdx.x]         = (uint32_t)bt;
        }
    }
}

// One CTA: exclusive scan of chunk sizes, Adler-32 of the whole input, zlib header and tail.
// result: [0] stream bytes, [1] status, [2] chunks, [3] stored, [4] fixed, [5] dynamic chunks
__global__ void __launch_bounds__(1024)
    k_deflate_finish(const uint32_t* __restrict__ sizes, const uint32_t* __restrict__ adler,
                     const uint32_t* __restrict__ kinds, size_t nchunks, size_t len,
                     unsigned long long* __restrict__ offsets, uint8_t* __restrict__ out, size_t out_capacity,
                     unsigned long long* __restrict__ result) {
    __shared__ unsigned long long s_sum[1024];
    __shared__ unsigned long long s_S[1024], s_T[1024], s_N[1024];
    __shared__ unsigned long long s_kind[3];
    const int tid = threadIdx.x;
    const size_t per = (nchunks + 1023) / 1024;
    const size_t a = min(nchunks, (size_t)tid * per), b = min(nchunks, a + per);
    unsigned long long sum = 0, S = 0, T = 0, N = 0;
    if (tid < 3) s_kind[tid] = 0;
    __syncthreads();
    unsigned long long kc[3] = {0, 0, 0};
    for (size_t c = a; c < b; c++) {
        sum += sizes[c];
        const uint64_t cn = min((size_t)kChunk, len - c * kChunk);
        T = (T + adler[2 * c + 1] + (cn % kAdlerMod) * S) % kAdlerMod;
        S = (S + adler[2 * c]) % kAdlerMod;
        N += cn;
        kc[min(kinds[c], 2u)]++;
    }
    s_sum[tid] = sum;
    s_S[tid] = S, s_T[tid] = T, s_N[tid] = N;
    for (int k = 0; k < 3; k++)
        if (kc[k]) atomicAdd(&s_kind[k], kc[k]);
    __syncthreads();
    if (tid == 0) {
        unsigned long long acc = 0, AS = 0, AT = 0;
        for (int k = 0; k < 1024; k++) {
            const unsigned long long v = s_sum[k];
            s_sum[k] = acc;
            acc += v;
            AT = (AT + s_T[k] + (s_N[k] % kAdlerMod) * AS) % kAdlerMod;
            AS = (AS + s_S[k]) % kAdlerMod;
        }
        // Adler-32 = B << 16 | A with A = 1 + sum, B = len + sum of prefix sums (mod 65521)
        const uint32_t A = (uint32_t)((1 + AS) % kAdlerMod);
        const uint32_t B = (uint32_t)(((len % kAdlerMod) + AT) % kAdlerMod);
        const uint32_t ad = (B << 16) | A;
        const unsigned long long total = 2 + acc + 2 + 4;
        result[0] = total;
        result[2] = nchunks;
        result[3] = s_kind[0];
        result[4] = s_kind[1];
        result[5] = s_kind[2];
        if (total > out_capacity) {
            result[1] = VSZ_ERR_CAPACITY;
        } else {
            result[1] = VSZ_OK;
            out[0] = 0x78;  // CM 8, CINFO 7 (32 KiB window)
            out[1] = 0x01;  // FLEVEL 0, no dictionary; (0x7801 % 31 == 0)
            uint8_t* tail = out + 2 + acc;
            tail[0] = 0x03;  // final empty block with fixed codes: BFINAL 1, BTYPE 01, end of block
            tail[1] = 0x00;
            tail[2] = (uint8_t)(ad >> 24);
            tail[3] = (uint8_t)(ad >> 16);
            tail[4] = (uint8_t)(ad >> 8);
            tail[5] = (uint8_t)ad;
        }
    }
    __syncthreads();
    const unsigned long long base = s_sum[tid];
    unsigned long long run = 0;
    for (size_t c = a; c < b; c++) {
        offsets[c] = 2 + base + run;
        run += sizes[c];
    }
}

// One CTA per chunk: staging slot -> its place in the stream.  Whole aligned words where the
// destination allows, single bytes at the two ends.
__global__ void __launch_bounds__(256)
    k_deflate_copy(const uint8_t* __restrict__ staging, const uint32_t* __restrict__ sizes,
                   const unsigned long long* __restrict__ offsets, uint8_t* __restrict__ out,
                   const unsigned long long* __restrict__ result) {
    if (result[1] != VSZ_OK) return;
    const size_t c     = blockIdx.x;
    const uint8_t* src = staging + c * kSlot;
    const size_t dst0  = offsets[c];
    const uint32_t n   = sizes[c];
    const size_t head  = min((size_t)n, (size_t)((4 - (dst0 & 3)) & 3));
    if (threadIdx.x < head) out[dst0 + threadIdx.x] = src[threadIdx.x];
    const size_t words = (n - head) / 4;
    uint32_t* dw       = reinterpret_cast<uint32_t*>(out + dst0 + head);
    for (size_t w = threadIdx.x; w < words; w += blockDim.x) {
        const uint8_t* p = src + head + 4 * w;
        dw[w] = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    }
    const size_t done = head + 4 * words;
    if (threadIdx.x < n - done) out[dst0 + done + threadIdx.x] = src[done + threadIdx.x];
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

struct DeflateWs {
    uint8_t* staging;
    uint32_t* sizes;
    uint32_t* adler;
    uint32_t* kinds;
    unsigned long long* offsets;
    size_t bytes;
};

DeflateWs deflate_ws(uint8_t* base, size_t nchunks) {
    DeflateWs w{};
    size_t off = 0;
    auto take  = [&](size_t b) {
        uint8_t* p = base ? base + off : nullptr;
        off += align256(b);
        return p;
    };
    w.staging = take(nchunks * (size_t)kSlot);
    w.sizes   = reinterpret_cast<uint32_t*>(take(4 * nchunks));
    w.adler   = reinterpret_cast<uint32_t*>(take(8 * nchunks));
    w.kinds   = reinterpret_cast<uint32_t*>(take(4 * nchunks));
    w.offsets = reinterpret_cast<unsigned long long*>(take(8 * nchunks));
    w.bytes   = off + 256;
    return w;
}

}  // namespace

extern "C" {

size_t vsz_deflate_chunk_bytes(void) { return (size_t)kChunk; }

vsz_status vsz_deflate_bounds(size_t len, size_t* ws_bytes, size_t* out_capacity) {
    const size_t nchunks = (len + kChunk - 1) / kChunk;
    if (ws_bytes) *ws_bytes = deflate_ws(nullptr, nchunks).bytes;
    if (out_capacity) *out_capacity = 2 + len + 5 * nchunks + 6;
    return VSZ_OK;
}

vsz_status vsz_deflate_chunk_sizes(const void* d_ws, size_t len, uint32_t* dst, void* stream) {
    if (!d_ws || !dst) return VSZ_ERR_INVALID;
    const size_t nchunks = (len + kChunk - 1) / kChunk;
    DeflateWs w = deflate_ws(static_cast<uint8_t*>(const_cast<void*>(d_ws)), nchunks);
    if (!nchunks) return VSZ_OK;
    return cudaMemcpyAsync(dst, w.sizes, 4 * nchunks, cudaMemcpyDefault, static_cast<cudaStream_t>(stream)) ==
                   cudaSuccess
               ? VSZ_OK
               : VSZ_ERR_CUDA;
}

vsz_status vsz_deflate(const uint8_t* d_in, size_t len, void* d_ws, size_t ws_bytes, uint8_t* d_out,
                       size_t out_capacity, uint64_t* d_result, void* stream) {
    if ((!d_in && len) || !d_ws || !d_out || !d_result) return VSZ_ERR_INVALID;
    const size_t nchunks = (len + kChunk - 1) / kChunk;
    if (nchunks > 0x7FFFFFFFu) return VSZ_ERR_INVALID;
    DeflateWs w = deflate_ws(static_cast<uint8_t*>(d_ws), nchunks);
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaFuncSetAttribute(k_deflate_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) !=
        cudaSuccess)
        return VSZ_ERR_CUDA;
    if (cudaMemsetAsync(d_result, 0, 8 * sizeof(uint64_t), st) != cudaSuccess) return VSZ_ERR_CUDA;
    if (nchunks) {
        k_deflate_chunks<<<(unsigned)nchunks, kThreads, kSmemBytes, st>>>(d_in, len, w.staging, w.sizes, w.adler,
                                                                          w.kinds);
        vsz::count_launch();
    }
    k_deflate_finish<<<1, 1024, 0, st>>>(w.sizes, w.adler, w.kinds, nchunks, len, w.offsets, d_out, out_capacity,
                                         reinterpret_cast<unsigned long long*>(d_result));
    vsz::count_launch();
    if (nchunks) {
        k_deflate_copy<<<(unsigned)nchunks, 256, 0, st>>>(w.staging, w.sizes, w.offsets, d_out,
                                                          reinterpret_cast<const unsigned long long*>(d_result));
        vsz::count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

}  // extern "C"
