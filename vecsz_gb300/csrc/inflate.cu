// Inflate on the device for the zlib streams vsz_deflate writes: the decompress side of the -L gzip
// pass (replaces zlib_uncompress, src/lossless.hh:144-177, for those streams).  vsz_deflate's
// chunks are independent (no match reaches before its chunk, every chunk starts on a byte), so
// with the chunk sizes from the archive's deflate index each chunk inflates on its own: one warp
// per chunk, the chunk's output (16 KiB) in shared memory, its compressed bytes read through the
// read-only cache.  All lanes run the same decode (broadcast reads, no divergence), lane 0 builds
// the code tables (a 9-bit primary table and a canonical walk for longer codewords) and writes
// literals, the warp copies matches and stored blocks together.  Every read is bounded by the
// chunk's bytes, every write by its output size; anything else (another encoder's stream, a
// damaged one) sets VSZ_ERR_CORRUPT and the host falls back to the host library.  The Adler-32 of
// the output is checked against the stream's.
#include <cstdint>

#include <cuda_runtime.h>

#include "deflate_format.h"
#include "vsz_types.h"

namespace vsz {
void count_launch();  // vsz_profile.cu
}

namespace {

constexpr int kChunk         = vsz::kDeflateChunk;  // output bytes per chunk, as vsz_deflate writes them
constexpr int kLitBits       = 9;      // primary table of the literal/length code
constexpr int kDistBits      = 6;      // primary table of the distance code
constexpr uint32_t kAdlerMod = 65521;

// code tables of a warp's chunk, in shared memory
struct LaneTables {
    uint16_t lit[1 << kLitBits];    // symbol | len << 9; 0: codeword longer than kLitBits
    uint16_t dist[1 << kDistBits];  // symbol | len << 9
    uint16_t lcount[16], dcount[16];
    uint16_t lsym[288], dsym[32];  // symbols by (length, symbol): the canonical walk's table
    uint8_t lens[288 + 32];
};

__constant__ uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                      31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
__constant__ uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
__constant__ uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
__constant__ uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
__constant__ uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// LSB-first bit reader over the chunk's bytes in global memory (read-only, cached; every lane of
// the warp reads the same word), with a 64-bit window in registers refilled a word at a time.
// Words are aligned; bytes outside the chunk read as zero, and positions past its end are caught
// by the caller's position checks.
struct Bits {
    const uint32_t* w;  // aligned words covering the chunk
    uint32_t skew;      // bytes of the first word before the chunk
    uint32_t cb;        // chunk bytes
    uint32_t pos;       // bits consumed
    uint32_t nw;        // next word to enter the window
    uint32_t cnt;       // valid bits in the window
    uint64_t buf;
    __device__ __forceinline__ uint32_t word(uint32_t i) const {
        const uint32_t lo = 4 * i;  // byte offset of the word from w, the chunk starts at skew
        if (lo >= skew && lo + 4 - skew <= cb) return __ldg(&w[i]);
        const uint8_t* b = reinterpret_cast<const uint8_t*>(w);
        uint32_t v = 0;
        for (uint32_t q = 0; q < 4; q++) {
            const uint32_t at = lo + q;
            if (at >= skew && at - skew < cb) v |= (uint32_t)__ldg(&b[at]) << (8 * q);
        }
        return v;
    }
    __device__ __forceinline__ void seek(uint32_t p) {
        pos = p;
        const uint32_t bit = 8 * skew + p;
        buf = word(bit >> 5) >> (bit & 31);
        cnt = 32 - (bit & 31);
        nw  = (bit >> 5) + 1;
    }
    __device__ __forceinline__ uint32_t peek() {  // at least 32 valid bits
        if (cnt < 32) {
            buf |= (uint64_t)word(nw++) << cnt;
            cnt += 32;
        }
        return (uint32_t)buf;
    }
    __device__ __forceinline__ void drop(uint32_t k) {
        buf >>= k;
        cnt -= k;
        pos += k;
    }
    __device__ __forceinline__ uint32_t get(uint32_t k) {
        if (k == 0) return 0;
        const uint32_t v = peek() & ((1u << k) - 1);
        drop(k);
        return v;
    }
    __device__ __forceinline__ void align_byte() {
        peek();
        drop((8 - (pos & 7)) & 7);
    }
};

__device__ __forceinline__ uint32_t reverse_bits(uint32_t code, uint32_t len) { return __brev(code) >> (32 - len); }

// Decode tables from code lengths (RFC 1951 3.2.2).  Returns false for an over-subscribed set,
// or an incomplete one (allowed only for a single distance code, as zlib allows).
__device__ bool build_table(const uint8_t* len, int n, int pbits, uint16_t* primary, uint16_t* count, uint16_t* sym,
                            bool allow_single) {
    for (int l = 0; l < 16; l++) count[l] = 0;
    for (int i = 0; i < n; i++) count[len[i]]++;
    count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; l++) {
        left = 2 * left - count[l];
        if (left < 0) return false;
    }
    int used = 0;
    for (int l = 1; l < 16; l++) used += count[l];
    if (left > 0 && !(allow_single && used == 1)) return false;
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; l++) offs[l + 1] = offs[l] + count[l];
    for (int i = 0; i < n; i++)
        if (len[i]) sym[offs[len[i]]++] = (uint16_t)i;
    for (int i = 0; i < (1 << pbits); i++) primary[i] = 0;
    uint32_t code = 0, k = 0;
    for (int l = 1; l < 16; l++) {
        for (int c = 0; c < count[l]; c++, k++) {
            if (l <= pbits) {
                const uint32_t r = reverse_bits(code, l);
                for (uint32_t e = r; e < (1u << pbits); e += 1u << l) primary[e] = (uint16_t)(sym[k] | (l << 9));
            }
            code++;
        }
        code <<= 1;
    }
    return true;
}

// One codeword: primary table, else the canonical walk over up to 15 bits.  -1 on a bad code.
__device__ __forceinline__ int decode_sym(Bits& br, const uint16_t* primary, int pbits, const uint16_t* count,
                                          const uint16_t* sym) {
    const uint32_t bits = br.peek();
    const uint16_t e    = primary[bits & ((1u << pbits) - 1)];
    if (e) {
        br.drop(e >> 9);
        return e & 0x1FF;
    }
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; l++) {
        code |= (bits >> (l - 1)) & 1;
        const int c = count[l];
        if (code - first < c) {
            br.drop(l);
            return sym[index + code - first];
        }
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

// dynamic shared memory of a CTA (one warp, one chunk)
struct InflateSmem {
    uint8_t out[kChunk];
    LaneTables t;
    int bad;
};

__global__ void __launch_bounds__(32)
    k_inflate_chunks(const uint8_t* __restrict__ stream, size_t stream_len, const unsigned long long* __restrict__ chunk_off,
                     const uint32_t* __restrict__ chunk_bytes, size_t nchunks, uint8_t* __restrict__ out,
                     size_t out_len, uint32_t* __restrict__ adler, int* __restrict__ status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    InflateSmem& m    = *reinterpret_cast<InflateSmem*>(smem_raw);
    LaneTables& t     = m.t;
    const uint32_t lane = threadIdx.x;
    const size_t c    = blockIdx.x;
    if (c >= nchunks) return;
    const size_t o0     = c * (size_t)kChunk;
    const uint32_t want = (uint32_t)min((size_t)kChunk, out_len - o0);
    const unsigned long long off = chunk_off[c];
    const uint32_t cb            = chunk_bytes[c];
    if (off > stream_len || cb > stream_len - off || cb > (uint32_t)(kChunk + 5)) {  // an index that does not fit
        if (lane == 0) {
            atomicExch(status, VSZ_ERR_CORRUPT);
            adler[2 * c] = adler[2 * c + 1] = 0;
        }
        return;
    }
    const uint8_t* src  = stream + off;
    const uint32_t skew = (uint32_t)(reinterpret_cast<uintptr_t>(src) & 3);
    if (lane == 0) m.bad = 0;
    __syncwarp();
    Bits br{reinterpret_cast<const uint32_t*>(src - skew), skew, cb, 0, 0, 0, 0};
    br.seek(0);
    const uint32_t end_bits = 8 * cb;
    uint32_t have = 0;
    bool bad      = false;
    // blocks until the chunk's bytes are used up; a dynamic or fixed block is followed by an
    // empty stored block, a stored block of data ends on a byte itself
    for (int guard = 0; !bad && br.pos < end_bits; guard++) {
        if (guard > 64) {
            bad = true;
            break;
        }
        const uint32_t final = br.get(1);
        const uint32_t type  = br.get(2);
        if (final || type == 3) {  // chunks never hold the final block
            bad = true;
            break;
        }
        if (type == 0) {
            br.align_byte();
            const uint32_t len = br.get(16), nlen = br.get(16);
            if ((len ^ 0xFFFFu) != nlen || len > want - have || br.pos + 8 * len > end_bits) {
                bad = true;
                break;
            }
            const uint32_t bp = br.pos / 8;  // the block's bytes start here in the chunk
            for (uint32_t k = lane; k < len; k += 32) m.out[have + k] = __ldg(&src[bp + k]);
            __syncwarp();
            have += len;
            br.seek(br.pos + 8 * len);
            continue;
        }
        bool ok = true;
        if (type == 1) {  // fixed codes (RFC 1951 3.2.6)
            if (lane == 0) {
                for (int i = 0; i < 288; i++) t.lens[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
                for (int i = 0; i < 30; i++) t.lens[288 + i] = 5;
                m.bad = !build_table(t.lens, 288, kLitBits, t.lit, t.lcount, t.lsym, false) ||
                        !build_table(t.lens + 288, 30, kDistBits, t.dist, t.dcount, t.dsym, true);
            }
            __syncwarp();
            ok = !m.bad;
        } else {  // dynamic codes (RFC 1951 3.2.7)
            const int nlit = (int)br.get(5) + 257, ndist = (int)br.get(5) + 1, ncl = (int)br.get(4) + 4;
            if (nlit > 286 || ndist > 30) {
                bad = true;
                break;
            }
            uint8_t cl[19];
            for (int i = 0; i < 19; i++) cl[i] = 0;
            for (int i = 0; i < ncl; i++) cl[kClOrder[i]] = (uint8_t)br.get(3);
            // the code-length code goes through the literal tables' space
            if (lane == 0) m.bad = !build_table(cl, 19, 7, t.lit, t.lcount, t.lsym, false);
            __syncwarp();
            if (m.bad) {
                bad = true;
                break;
            }
            // every lane decodes the lengths (the reader positions stay equal); lane 0 stores them
            int k = 0;
            uint8_t prev = 0;
            while (k < nlit + ndist) {
                const int sy = decode_sym(br, t.lit, 7, t.lcount, t.lsym);
                if (sy < 0 || br.pos > end_bits) {
                    bad = true;
                    break;
                }
                int rep;
                uint8_t v;
                if (sy < 16) {
                    rep = 1;
                    v   = (uint8_t)sy;
                } else if (sy == 16) {
                    if (k == 0) {
                        bad = true;
                        break;
                    }
                    v   = prev;
                    rep = 3 + (int)br.get(2);
                } else {
                    v   = 0;
                    rep = sy == 17 ? 3 + (int)br.get(3) : 11 + (int)br.get(7);
                }
                if (k + rep > nlit + ndist) {
                    bad = true;
                    break;
                }
                if (lane == 0)
                    for (int r = 0; r < rep; r++) {
                        const int at = k + r;  // literal/length lengths at [0, nlit), distance ones at 288 +
                        t.lens[at < nlit ? at : 288 + (at - nlit)] = v;
                    }
                k += rep;
                prev = v;
            }
            if (bad) break;
            if (lane == 0) {
                for (int i = nlit; i < 288; i++) t.lens[i] = 0;
                for (int i = ndist; i < 32; i++) t.lens[288 + i] = 0;
                m.bad = t.lens[256] == 0 || !build_table(t.lens, 288, kLitBits, t.lit, t.lcount, t.lsym, false) ||
                        !build_table(t.lens + 288, 30, kDistBits, t.dist, t.dcount, t.dsym, true);
            }
            __syncwarp();
            ok = !m.bad;
        }
        if (!ok) {
            bad = true;
            break;
        }
        // symbols up to the end of the block
        while (true) {
            const int sy = decode_sym(br, t.lit, kLitBits, t.lcount, t.lsym);
            if (sy < 0 || br.pos > end_bits) {
                bad = true;
                break;
            }
            if (sy < 256) {
                if (have >= want) {
                    bad = true;
                    break;
                }
                if (lane == 0) m.out[have] = (uint8_t)sy;
                have++;
                continue;
            }
            if (sy == 256) break;
            if (sy > 285) {
                bad = true;
                break;
            }
            const uint32_t len = kLenBase[sy - 257] + br.get(kLenExtra[sy - 257]);
            const int ds       = decode_sym(br, t.dist, kDistBits, t.dcount, t.dsym);
            if (ds < 0 || ds > 29) {
                bad = true;
                break;
            }
            const uint32_t dist = kDistBase[ds] + br.get(kDistExtra[ds]);
            if (dist > have || len > want - have) {
                bad = true;
                break;
            }
            __syncwarp();  // the literals lane 0 wrote are read below
            for (uint32_t k = lane; k < len; k += 32)
                m.out[have + k] = m.out[have - dist + (k < dist ? k : k % dist)];
            __syncwarp();
            have += len;
        }
        __syncwarp();
    }
    if (br.pos != end_bits) bad = true;
    if (have != want) bad = true;
    __syncwarp();
    // Adler-32 parts of the chunk: lane l sums bytes [kChunk / 32 * l, ...), then an ordered scan
    uint64_t S = 0, T = 0, N = 0;
    if (!bad) {
        const uint32_t b0 = lane * (kChunk / 32), b1 = min(want, b0 + kChunk / 32);
        for (uint32_t i = b0; i < b1; i++) {
            S += m.out[i];
            T += S;
        }
        N = b1 > b0 ? b1 - b0 : 0;
        S %= kAdlerMod;
        T %= kAdlerMod;
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t S_l = __shfl_up_sync(0xFFFFFFFFu, S, o);
            const uint64_t T_l = __shfl_up_sync(0xFFFFFFFFu, T, o);
            const uint64_t N_l = __shfl_up_sync(0xFFFFFFFFu, N, o);
            if (lane >= (uint32_t)o) {
                T = (T_l + T + (N % kAdlerMod) * S_l) % kAdlerMod;
                S = (S_l + S) % kAdlerMod;
                N = N_l + N;
            }
        }
        // the chunk's output to global memory
        uint8_t* dst = out + o0;
        if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
            for (uint32_t k = lane; k < want / 16; k += 32)
                reinterpret_cast<uint4*>(dst)[k] = reinterpret_cast<const uint4*>(m.out)[k];
            for (uint32_t k = (want & ~15u) + lane; k < want; k += 32) dst[k] = m.out[k];
        } else {
            for (uint32_t k = lane; k < want; k += 32) dst[k] = m.out[k];
        }
    }
    if (lane == 31) {
        if (bad) atomicExch(status, VSZ_ERR_CORRUPT);
        adler[2 * c]     = (uint32_t)S;
        adler[2 * c + 1] = (uint32_t)T;
    }
}

// One CTA: the Adler-32 of the whole output from the per-chunk parts, against the stream's.
__global__ void __launch_bounds__(1024)
    k_inflate_check(const uint32_t* __restrict__ adler, size_t nchunks, size_t out_len, uint32_t expect,
                    int* __restrict__ status) {
    __shared__ unsigned long long s_S[1024], s_T[1024], s_N[1024];
    const int tid = threadIdx.x;
    const size_t per = (nchunks + 1023) / 1024;
    const size_t a = min(nchunks, (size_t)tid * per), b = min(nchunks, a + per);
    unsigned long long S = 0, T = 0, N = 0;
    for (size_t c = a; c < b; c++) {
        const uint64_t cn = min((size_t)kChunk, out_len - c * kChunk);
        T = (T + adler[2 * c + 1] + (cn % kAdlerMod) * S) % kAdlerMod;
        S = (S + adler[2 * c]) % kAdlerMod;
        N += cn;
    }
    s_S[tid] = S, s_T[tid] = T, s_N[tid] = N;
    __syncthreads();
    if (tid == 0) {
        unsigned long long AS = 0, AT = 0;
        for (int k = 0; k < 1024; k++) {
            AT = (AT + s_T[k] + (s_N[k] % kAdlerMod) * AS) % kAdlerMod;
            AS = (AS + s_S[k]) % kAdlerMod;
        }
        const uint32_t A = (uint32_t)((1 + AS) % kAdlerMod);
        const uint32_t B = (uint32_t)(((out_len % kAdlerMod) + AT) % kAdlerMod);
        if (((B << 16) | A) != expect) atomicExch(status, VSZ_ERR_CORRUPT);
    }
}

}  // namespace

extern "C" {

vsz_status vsz_inflate_bounds(size_t n_chunks, size_t* ws_bytes) {
    if (ws_bytes) *ws_bytes = 8 * n_chunks + 256;
    return VSZ_OK;
}

vsz_status vsz_inflate(const uint8_t* d_stream, size_t stream_len, const unsigned long long* d_chunk_offsets,
                       const uint32_t* d_chunk_bytes, size_t n_chunks, uint32_t adler32, uint8_t* d_out,
                       size_t out_len, void* d_ws, size_t ws_bytes, int* d_status, void* stream) {
    if (!d_stream || !d_chunk_offsets || !d_chunk_bytes || !d_status || (out_len && !d_out)) return VSZ_ERR_INVALID;
    if (n_chunks != (out_len + kChunk - 1) / kChunk || stream_len < 2) return VSZ_ERR_INVALID;
    if (ws_bytes < 8 * n_chunks + 256 || (!d_ws && n_chunks)) return VSZ_ERR_CAPACITY;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(d_status, 0, sizeof(int), st) != cudaSuccess) return VSZ_ERR_CUDA;
    uint32_t* adler = static_cast<uint32_t*>(d_ws);
    const size_t smem = sizeof(InflateSmem);
    if (cudaFuncSetAttribute(k_inflate_chunks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return VSZ_ERR_CUDA;
    if (n_chunks) {
        k_inflate_chunks<<<(unsigned)n_chunks, 32, smem, st>>>(
            d_stream, stream_len, d_chunk_offsets, d_chunk_bytes, n_chunks, d_out, out_len, adler, d_status);
        vsz::count_launch();
    }
    k_inflate_check<<<1, 1024, 0, st>>>(adler, n_chunks, out_len, adler32, d_status);
    vsz::count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

}  // extern "C"
