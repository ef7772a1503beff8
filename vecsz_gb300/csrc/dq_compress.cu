// Dual-quantization compress on sm_103a: value range (r2r), error-bound constants, fused
// prequant + Lorenzo + quant-code + histogram + outlier ranking, and outlier compaction.
//
// Replaces, from szcompressor/vecSZ:
//   GetDatumValueRange / ChangeToRelativeMode / InitializeErrorBoundFamily  src/types.cc:28-92
//   c_lorenzo_{1,2,3}d1l                                                    src/dualquant.hh:19-913
//   histogram loop of initHuffman                                           src/huffman.hh:239-242
//   outlier gather                                                          src/vecsz_interface.hh:166-170
//
// Element rules (pinned against the reference by the oracle):
//   s   = rint(x *f32 r_f)                       all 1D/2D elements, 3D columns x < d0 & ~7
//   s   = (float) round((double) x * r_d)        3D tail columns x >= d0 & ~7 when d0 % 8 != 0
//   pred: 1D s[x-1]; 2D W + (N - NW); 3D (XYZ - (XY + (XZ + YZ))) + (X + (Y + Z)),
//         3D tail columns left to right XYZ - XY - XZ - YZ + X + Y + Z; zero halo per block,
//         or with padding (-p) the block's pad values (dq_pad.cu)
//   e   = s - pred (always integer valued, so the reference's sqrt(e*e) < R is |e| < R)
//   code = |e| < R ? e + R : 0;  outlier value = s where code == 0
//   2D tail columns (d0 % 8 != 0): code 0, outlier 0.0 -- the reference skips those AVX chunks
//   and never runs its scalar tail (src/dualquant.hh:490-495).
#include <cstdint>
#include <type_traits>

#include "api_common.cuh"
#include "scan.cuh"
#include "vsz_device.cuh"
#include "vsz_kernels.h"

namespace vsz {

// ------------------------------------------------------------------------------------------
// K0: min / max of the field for r2r (GetDatumValueRange, src/types.cc:28-35)
// ------------------------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_minmax(const float* __restrict__ x, size_t n, uint32_t* __restrict__ mm) {
    uint32_t kmax = 0u, kmin = 0xffffffffu;
    size_t tid    = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    const bool aligned = ((reinterpret_cast<uintptr_t>(x) & 15u) == 0);
    size_t n4 = aligned ? n / 4 : 0;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    for (size_t i = tid; i < n4; i += stride) {
        float4 v = __ldcs(&x4[i]);
        float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (e[j] == e[j]) {
                uint32_t k = f2key(e[j]);
                kmax       = max(kmax, k);
                kmin       = min(kmin, k);
            }
        }
    }
    for (size_t i = n4 * 4 + tid; i < n; i += stride) {
        float v = x[i];
        if (v == v) {
            uint32_t k = f2key(v);
            kmax       = max(kmax, k);
            kmin       = min(kmin, k);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
        kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
    }
    __shared__ uint32_t smax[8], smin[8];
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        smax[w] = kmax;
        smin[w] = kmin;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) {
            kmax = max(kmax, smax[i]);
            kmin = min(kmin, smin[i]);
        }
        atomicMax(&mm[0], kmax);
        atomicMin(&mm[1], kmin);
    }
}

// Error-bound constants (one thread).  For r2r: range = (double)((float)max - (float)min), with
// std::max_element's rule that a NaN first element wins; a zero range is VSZ_ERR_RANGE, as the
// reference exits there (src/types.cc:49-56).
__device__ __forceinline__ void consts_of(int mode, double eb, const uint32_t* __restrict__ mm,
                                          const float* __restrict__ x, Consts* __restrict__ c, int* status_word) {
    double ebf   = eb;
    double range = 0.0;
    int status   = VSZ_OK;
    if (mode == VSZ_MODE_R2R) {
        float x0 = x[0];
        float mx, mn;
        if (x0 != x0) {
            mx = x0;
            mn = x0;
        } else {
            mx = key2f(mm[0]);
            mn = key2f(mm[1]);
        }
        float r = __fsub_rn(mx, mn);
        range   = (double)r;
        if (range == 0.0) status = VSZ_ERR_RANGE;
        ebf = __dmul_rn(ebf, range);
    }
    c->eb_final = ebf;
    c->r_d      = 1.0 / __dmul_rn(2.0, ebf);  // src/types.cc:91
    c->c_d      = __dmul_rn(2.0, ebf);        // src/types.cc:90
    c->range    = range;
    c->r_f      = __double2float_rn(c->r_d);
    float ch    = __double2float_rn(c->c_d);
    float cl    = __double2float_rn(__dsub_rn(c->c_d, (double)ch));
    c->c_hi     = ch;
    c->c_lo     = cl;
    auto normal = [](float f) {
        uint32_t e = __float_as_uint(f) & 0x7f800000u;
        return e != 0u && e != 0x7f800000u;
    };
    c->dq_fast  = normal(ch) && (cl == 0.0f || normal(cl));
    c->status   = status;
    c->dq_mul   = 0;  // until k_dq_mul_verify has checked the two-operation dequantization
    c->dq_exc   = 0.f;
    c->dq_exc_y = 0.f;
    if (status != VSZ_OK && status_word) set_status(status_word, status);
}

__global__ void k_consts(int mode, double eb, const uint32_t* __restrict__ mm, const float* __restrict__ x,
                         Consts* __restrict__ c, int* status_word) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    consts_of(mode, eb, mm, x, c, status_word);
}

// ------------------------------------------------------------------------------------------
// K1: fused prequant + Lorenzo + quant codes + histogram + outlier ranking.
//
// Work unit = one warp tile: 128 consecutive x (4 per lane) by 8 rows (y) by one Lorenzo block
// of planes (z, 3D) -- or 4 consecutive 128-element tiles in 1D.  Every lane keeps its 4 x 8
// prequantized values of the current and the previous plane in registers; the x - 1 neighbour
// of its first column comes from the lane to its left (shuffle), the y - 1 row above a warp
// tile that starts inside a Lorenzo block (block_size > 8) is reloaded from global memory, so
// warps never wait on each other.  Tile widths (128) are multiples of every block size, so a
// tile's first column always starts a Lorenzo block.
//
// Outliers: for each row segment (one tile row, 128 elements) the warp ranks its outliers with
// four ballots and writes them to scratch[seg * 128 + rank]; seg_count[seg] holds the count.
// k_outlier_gather then places them in global row-major order, as the reference's serial gather.
// ------------------------------------------------------------------------------------------

struct HistAcc {
    // A private counter for the code R (zero residual), the most frequent code of a smooth field,
    // so a warp of smooth data does not serialise on one shared-memory bin; every other code goes
    // to the block's shared-memory histogram (the field's global one when dict is large).
    uint32_t c1 = 0;
    __device__ __forceinline__ void add(int code, int R, uint32_t* s_hist, int dict, unsigned long long* g_hist) {
        if (code == R) {
            c1++;
        } else if (s_hist) {
            atomicAdd(&s_hist[code], 1u);
        } else {
            atomicAdd(&g_hist[code], 1ull);
        }
    }
    __device__ __forceinline__ void flush(int R, uint32_t* s_hist, int dict, unsigned long long* g_hist) {
        if (!c1) return;
        if (s_hist) atomicAdd(&s_hist[R], c1);
        else atomicAdd(&g_hist[R], (unsigned long long)c1);
    }
};

// One row of 4 elements per lane: store codes, count histogram, rank and write outliers.
template <bool VEC, bool FULL = false>
__device__ __forceinline__ void emit_row(const DqArgs& a, size_t row, uint32_t xb, uint32_t xt, bool row_in,
                                         const int code[4], const float outv[4], HistAcc& h, uint32_t* s_hist) {
    const unsigned lane = lane_id();
    if (FULL) row_in = true;
    bool in[4];
#pragma unroll
    for (int j = 0; j < 4; j++) in[j] = FULL || (row_in && (xb + j < a.d0));
    uint16_t* crow = a.code + row * a.d0;
    if (VEC && in[0]) {
        // d0 % 4 == 0: all four columns are in range together; 8-byte aligned store.
        uint2 v;
        v.x = (uint32_t)code[0] | ((uint32_t)code[1] << 16);
        v.y = (uint32_t)code[2] | ((uint32_t)code[3] << 16);
        *reinterpret_cast<uint2*>(crow + xb) = v;
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (in[j]) crow[xb + j] = (uint16_t)code[j];
    }
    if (s_hist) {
        // predicated, not branched: the zero-residual code counts in a register, the others in the
        // block's shared histogram
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const bool hot = code[j] == a.R;
            h.c1 += (in[j] && hot) ? 1u : 0u;
            if (in[j] && !hot) atomicAdd(&s_hist[code[j]], 1u);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (in[j]) h.add(code[j], a.R, s_hist, a.dict, a.hist);
    }
    // Outlier ranking inside the row segment: element (lane, j) precedes (lane', j') iff
    // 4 lane + j < 4 lane' + j'.  Most rows of a smooth field have none: one vote decides.
    bool o[4];
#pragma unroll
    for (int j = 0; j < 4; j++) o[j] = in[j] && code[j] == 0;
    const size_t seg = row * a.nxt + xt;
    if (!__any_sync(0xffffffffu, o[0] | o[1] | o[2] | o[3])) {
        if (row_in && lane == 0) a.seg_count[seg] = 0;
        return;
    }
    unsigned m[4];
#pragma unroll
    for (int j = 0; j < 4; j++) m[j] = __ballot_sync(0xffffffffu, o[j]);
    if (!row_in) return;
    const unsigned lt = lanemask_lt();
    unsigned before   = __popc(m[0] & lt) + __popc(m[1] & lt) + __popc(m[2] & lt) + __popc(m[3] & lt);
    unsigned total    = __popc(m[0]) + __popc(m[1]) + __popc(m[2]) + __popc(m[3]);
    if (lane == 0) a.seg_count[seg] = (uint8_t)total;
    if (total) {
        float* dst = a.scratch + seg * kSegX;
        unsigned r = before;
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (o[j]) {
                float v = outv[j];
                // a NaN input's prequantized value is that NaN, quieted (the GPU multiply would
                // give its canonical NaN); strict outliers are input values already
                if (v != v && !a.strict) {
                    const float xv = a.x[row * a.d0 + xb + j];
                    if (xv != xv) v = quiet_nan(xv);
                }
                dst[r++] = v;
            }
    }
}

// (int)(e + R) for an integer-valued residual with |e| < R <= 32768: e + R + 1.5 * 2^23 is exact
// (an integer below 2^24), and its bits minus those of 1.5 * 2^23 are e + R -- two full-rate
// instructions instead of a float-to-int conversion.  rmagic = (float)R + 1.5 * 2^23.
__device__ __forceinline__ int code_of(float e, float rmagic) {
    return __float_as_int(__fadd_rn(e, rmagic)) - 0x4B400000;
}

template <int NDIM, bool TAIL>
__device__ __forceinline__ float prequant_at(float v, uint32_t col, uint32_t xtail, float r_f, double r_d) {
    if (NDIM == 3 && TAIL && col >= xtail) return prequant_scalar(v, r_d);
    return prequant_vec(v, r_f);
}

// Raw values of 4 consecutive columns [xb, xb+4) of one row (zeros outside the field).
template <bool VEC, bool FULL = false>
__device__ __forceinline__ float4 load_raw(const DqArgs& a, size_t row, bool row_in, uint32_t xb) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!FULL && !row_in) return v;
    const float* rowp = a.x + row * a.d0;
    if (VEC) {
        if (FULL || xb < a.d0) v = __ldcs(reinterpret_cast<const float4*>(rowp + xb));
    } else {
        if (xb < a.d0) v.x = __ldcs(rowp + xb);
        if (xb + 1 < a.d0) v.y = __ldcs(rowp + xb + 1);
        if (xb + 2 < a.d0) v.z = __ldcs(rowp + xb + 2);
        if (xb + 3 < a.d0) v.w = __ldcs(rowp + xb + 3);
    }
    return v;
}

// Prequantized values of a raw row; zero outside the field.
template <int NDIM, bool TAIL, bool FULL = false>
__device__ __forceinline__ void prequant_row(const DqArgs& a, float4 v, bool row_in, uint32_t xb, float r_f, double r_d,
                                             float S[4]) {
    const float t[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const bool in = FULL || (row_in && (xb + j < a.d0));
        S[j]          = in ? prequant_at<NDIM, TAIL>(t[j], xb + j, a.xtail, r_f, r_d) : 0.0f;
    }
}

// 2D / 3D.  Work unit = one warp tile: 128 consecutive x (4 per lane) by 8 rows (y) by one
// Lorenzo block of planes (z).  Rows are processed one at a time (the next row's values are
// loaded while the current one is coded); a lane keeps in registers only its 4 values of the
// current row and of the row above, in this plane and in the previous one.  The previous plane's
// 8 rows live in shared memory [row][column][lane] (conflict-free), each row overwritten by the
// current plane's once it has been used.  x - 1 neighbours come from the lane to the left.
typedef float PrevRows[8][4][32];

// Strict error-bound mode: an element keeps its quant code only if the decompressor, predicting
// from the same neighbours with its own operation order, reproduces the prequantized value `cur`
// (pd + e == cur) and the dequantized value is within eb of the input.  Otherwise it becomes an
// outlier carrying the input value, from which the decompressor re-derives `cur` by the same
// prequant rule -- so both sides' predictor chains stay identical, element by element.
__device__ __forceinline__ bool strict_keep(bool q, float pd, float e, float cur, float x, const Consts& c) {
    if (!q) return false;
    if (__fadd_rn(pd, e) != cur) return false;
    const float xh = dequant(cur, c.c_d, c.c_hi, c.c_lo, c.dq_fast);
    return fabs((double)x - (double)xh) <= c.eb_final;
}

// The histogram share of a block: the threads' private hot-code counters into shared memory, then
// shared memory into the field's histogram.
__device__ __forceinline__ void hist_flush_block(const DqArgs& a, uint32_t* s_hist, HistAcc& h) {
    h.flush(a.R, s_hist, a.dict, a.hist);
    if (s_hist) {
        __syncthreads();
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x) {
            uint32_t v = s_hist[i];
            if (v) atomicAdd(&a.hist[i], (unsigned long long)v);
        }
    }
}

// Warp units u0, u0 + ustep, ... < u1 of one field.  STRICT: the strict error-bound mode (see
// strict_keep).  PAD: padding (-p), the halo of each block from a.pad instead of zeros.
template <int NDIM, int BS, bool VEC, bool TAIL, bool STRICT = false, bool PAD = false>
__device__ __forceinline__ void dq23_units(const DqArgs& a, const Consts& c, unsigned long long u0,
                                           unsigned long long u1, unsigned long long ustep, uint32_t* s_hist,
                                           PrevRows* s_prev, HistAcc& h) {
    const float r_f     = c.r_f;
    const double r_d    = c.r_d;
    const float Rf      = (float)a.R;
    const float rmagic  = Rf + 12582912.0f;
    const unsigned lane = lane_id();
    const unsigned wib  = threadIdx.x >> 5;
    const bool xbound   = ((lane * 4) % BS) == 0;  // my first column starts a Lorenzo block
    auto left = [&](float v, float halo) {         // x - 1 neighbour of my first column
        const float t = __shfl_up_sync(0xffffffffu, v, 1);
        return xbound ? halo : t;
    };
    // unit indices fit 32 bits (n <= 2^36 elements, 1024 per unit): 32-bit divisions only
    for (uint32_t u = (uint32_t)u0; u < (uint32_t)u1; u += (uint32_t)ustep) {
        const uint32_t xt = u % a.nxt;
        const uint32_t r = u / a.nxt;
        const uint32_t yg = r % a.nyg;
        const uint32_t zb = r / a.nyg;
        const uint32_t xb = xt * kTileX + lane * 4;
        const uint32_t y0 = yg * 8;
        const bool yhalo  = (BS > 8) && (y0 % BS) != 0;  // the row above is inside the block
        const uint32_t z0 = (NDIM == 3) ? zb * BS : 0;
        const int nz      = (NDIM == 3) ? (int)min((uint32_t)BS, a.d2 - z0) : 1;

        // a tile wholly inside the field (the common case) runs without per-element range checks
        const bool full = VEC && (xt + 1) * kTileX <= a.d0 && y0 + 8 <= a.d1;
        auto unit_body = [&](auto full_c) {
            constexpr bool FULL = decltype(full_c)::value;
            // halo values of my block: x-, y- and z-halo cells (zero without padding; lanes past the
            // field read none); hxy: the (x-1, y-1) neighbour of my first column when the row above is
            // the halo row -- the corner cell at a block start (2D: x-halo, 3D: y-halo), else a y-halo
            // cell of the lane to the left, same block
            float hx = 0.f, hy = 0.f, hz = 0.f;
            if (PAD && xb < a.d0) {
                const Halo hv = halo_of(a.pad, NDIM, xb / BS, y0 / BS, zb);
                hx = hv.x;
                hy = hv.y;
                hz = hv.z;
            }
            const float hxy = (xbound && NDIM == 2) ? hx : hy;

            float Ph[4] = {hz, hz, hz, hz}, PhL = hz;  // previous plane's halo row (y0 - 1)
            float4 nxt = load_raw<VEC, FULL>(a, (size_t)z0 * a.d1 + y0, y0 < a.d1, xb);
            for (int zz = 0; zz < nz; zz++) {
                const uint32_t z = z0 + zz;
                const bool zp    = zz > 0;  // a previous plane inside the block
                float Sp[4] = {hy, hy, hy, hy}, SpL = hxy;  // row above, this plane (halo row at i = 0)
                if (yhalo) {
                    prequant_row<NDIM, TAIL, FULL>(a, load_raw<VEC, FULL>(a, (size_t)z * a.d1 + (y0 - 1), true, xb), true, xb, r_f,
                                             r_d, Sp);
                    SpL = left(Sp[3], hx);
                }
                const float ShNext[4] = {Sp[0], Sp[1], Sp[2], Sp[3]};
                const float ShNextL   = SpL;
                float Pp[4] = {Ph[0], Ph[1], Ph[2], Ph[3]}, PpL = PhL;  // row above, previous plane
#pragma unroll 2
                for (int i = 0; i < 8; i++) {
                    const uint32_t y  = y0 + i;
                    const bool row_in = y < a.d1;
                    const float4 raw  = nxt;
                    {  // the next row of this plane, or the first row of the next plane
                        const bool last_row = (i == 7);
                        const uint32_t zn = last_row ? z + 1 : z, yn = last_row ? y0 : y + 1;
                        const bool more = !last_row || zz + 1 < nz;
                        nxt = more ? load_raw<VEC, FULL>(a, (size_t)zn * a.d1 + yn, yn < a.d1, xb) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    float S[4];
                    prequant_row<NDIM, TAIL, FULL>(a, raw, row_in, xb, r_f, r_d, S);
                    const float SL = left(S[3], hx);
                    float Pc[4] = {hz, hz, hz, hz}, PcL = hz;  // this row, previous plane
                    if (NDIM == 3) {
#pragma unroll
                        for (int j = 0; j < 4; j++) Pc[j] = zp ? s_prev[wib][i][j][lane] : hz;
                        PcL = left(Pc[3], zp ? hx : hz);
                    }
                    int code[4];
                    float outv[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const uint32_t col = xb + j;
                        const float cur    = S[j];
                        const float X      = j ? S[j - 1] : SL;
                        const float Y      = Sp[j];
                        const float XY     = j ? Sp[j - 1] : SpL;
                        const bool tail    = TAIL && col >= a.xtail;
                        float pred;
                        if (NDIM == 2) {
                            pred = __fadd_rn(X, __fsub_rn(Y, XY));  // W + (N - NW)
                        } else {
                            const float Z   = Pc[j];
                            const float XZ  = j ? Pc[j - 1] : PcL;
                            const float YZ  = Pp[j];
                            const float XYZ = j ? Pp[j - 1] : PpL;
                            if (!tail) {
                                float dist1 = __fadd_rn(X, __fadd_rn(Y, Z));
                                float dist2 = __fadd_rn(XY, __fadd_rn(XZ, YZ));
                                pred        = __fadd_rn(__fsub_rn(XYZ, dist2), dist1);
                            } else {
                                pred = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fsub_rn(XYZ, XY), XZ), YZ), X), Y),
                                                 Z);
                            }
                        }
                        const float e = __fsub_rn(cur, pred);
                        const bool q  = fabsf(e) < Rf;
                        code[j]       = q ? code_of(e, rmagic) : 0;
                        outv[j]       = cur;
                        if (STRICT) {
                            const float xr = j == 0 ? raw.x : (j == 1 ? raw.y : (j == 2 ? raw.z : raw.w));
                            float pd;  // the decompressor's prediction from the same (in-step) neighbours
                            if (NDIM == 2) {
                                pd = __fsub_rn(__fadd_rn(Y, X), XY);
                            } else {
                                const float Z   = Pc[j];
                                const float XZ  = j ? Pc[j - 1] : PcL;
                                const float YZ  = Pp[j];
                                const float XYZ = j ? Pp[j - 1] : PpL;
                                pd = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fsub_rn(XYZ, XY), XZ), YZ), X), Y), Z);
                            }
                            if (!strict_keep(q, pd, e, cur, xr, c)) code[j] = 0;
                            outv[j] = xr;  // strict outliers carry the input value
                        } else if (NDIM == 2 && tail) {
                            code[j] = 0;
                            outv[j] = 0.0f;
                        }
                    }
                    emit_row<VEC, FULL>(a, (size_t)z * a.d1 + y, xb, xt, row_in, code, outv, h, s_hist);
                    if (NDIM == 3) {
#pragma unroll
                        for (int j = 0; j < 4; j++) s_prev[wib][i][j][lane] = S[j];  // row i of plane z
                    }
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        Sp[j] = S[j];
                        Pp[j] = Pc[j];
                    }
                    SpL = SL;
                    PpL = PcL;
                }
#pragma unroll
                for (int j = 0; j < 4; j++) Ph[j] = ShNext[j];
                PhL = ShNextL;
            }
        };
        if (full) unit_body(std::true_type{});
        else unit_body(std::false_type{});
    }
}

template <int NDIM, int BS, bool VEC, bool TAIL, bool STRICT = false, bool PAD = false>
__global__ void __launch_bounds__(256, 4) k_dq_compress_23d(DqArgs a) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    uint32_t* s_hist = a.smem_hist ? s_dyn : nullptr;
    PrevRows* s_prev = reinterpret_cast<PrevRows*>(s_dyn + (a.smem_hist ? ((a.dict + 3) & ~3) : 0));
    const Consts c   = *a.consts;
    if (c.status != VSZ_OK) return;  // uniform across the grid
    if (s_hist) {
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x) s_hist[i] = 0u;
        __syncthreads();
    }
    const unsigned long long warps_total = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long warp0       = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    HistAcc h;
    dq23_units<NDIM, BS, VEC, TAIL, STRICT, PAD>(a, c, warp0, a.nunits, warps_total, s_hist, s_prev, h);
    hist_flush_block(a, s_hist, h);
}

// Many fields in one launch: block-wide tasks (one field, a range of its warp units), each taken
// by the next free block (`next`: the launch's task counter, zero at launch), so that blocks do
// not idle behind uneven tasks.  hist_words = shared-memory histogram words reserved before the
// planes.
__device__ __forceinline__ uint32_t dq_block_next_task(uint32_t* next, uint32_t* s_task) {
    __syncthreads();  // every thread has read the previous task number
    if (threadIdx.x == 0) *s_task = atomicAdd(next, 1u);
    __syncthreads();
    return *s_task;
}

template <int NDIM, int BS, bool VEC, bool TAIL>
__global__ void __launch_bounds__(256, 3)
    k_dq_compress_23d_batch(const DqArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks,
                            uint32_t hist_words, uint32_t* __restrict__ next) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ uint32_t s_task;
    PrevRows* s_prev = reinterpret_cast<PrevRows*>(s_dyn + hist_words);
    for (uint32_t t = dq_block_next_task(next, &s_task); t < ntasks; t = dq_block_next_task(next, &s_task)) {
        const BatchTask tk = tasks[t];
        const DqArgs& a    = args[tk.field];  // read-only table: loads stay cached
        const Consts c     = *a.consts;
        if (c.status != VSZ_OK) continue;  // uniform: the whole block is on this task
        uint32_t* s_hist = a.smem_hist ? s_dyn : nullptr;
        if (s_hist) {
            for (int i = threadIdx.x; i < a.dict; i += blockDim.x) s_hist[i] = 0u;
            __syncthreads();
        }
        HistAcc h;
        dq23_units<NDIM, BS, VEC, TAIL>(a, c, tk.u0 + (threadIdx.x >> 5), tk.u1, blockDim.x >> 5, s_hist, s_prev, h);
        hist_flush_block(a, s_hist, h);
        __syncthreads();  // the next task reuses shared memory
    }
}

// 1D: 4 consecutive 128-element tiles per warp unit; the x - 1 neighbour comes from the lane to
// the left or, at a tile start, from the previous tile's last lane.  Blocks start on multiples of
// block_size (which divide 128), so tile starts are block starts.
template <int BS, bool VEC, bool STRICT = false, bool PAD = false>
__device__ __forceinline__ void dq1d_units(const DqArgs& a, const Consts& c, unsigned long long u0, unsigned long long u1,
                                           unsigned long long ustep, uint32_t* s_hist, HistAcc& h) {
    const float r_f     = c.r_f;
    const float Rf      = (float)a.R;
    const float rmagic  = Rf + 12582912.0f;
    const unsigned lane = lane_id();
    const bool xbound   = ((lane * 4) % BS) == 0;
    constexpr int U     = 4;
    for (unsigned long long u = u0; u < u1; u += ustep) {
        float S[U][4];
        float4 RW[STRICT ? U : 1];
#pragma unroll
        for (int t = 0; t < U; t++) {
            const uint32_t xt = (uint32_t)(u * U + t);
            const uint32_t xb = xt * kTileX + lane * 4;
            const float4 rw   = load_raw<VEC>(a, 0, xt < a.nxt, xb);
            if (STRICT) RW[STRICT ? t : 0] = rw;
            prequant_row<1, false>(a, rw, xt < a.nxt, xb, r_f, 0.0, S[t]);
        }
#pragma unroll
        for (int t = 0; t < U; t++) {
            const uint32_t xt = (uint32_t)(u * U + t);
            const uint32_t xb = xt * kTileX + lane * 4;
            float L           = __shfl_up_sync(0xffffffffu, S[t][3], 1);
            if (xbound) L = (PAD && xb < a.d0) ? halo_of(a.pad, 1, xb / BS, 0, 0).x : 0.f;
            // PAD: the reference's two postquant forms, which differ once a raw (non-integer) pad
            // value makes the first residual of a block fractional -- AVX for blocks ending before
            // the last element (sqrt(e*e) < R, code rint(e + R), outlier andnot(q, s)), scalar for
            // the others (|e| < R, code (int)(e + R), outlier (1 - q) * s); src/dualquant.hh:112-205.
            const bool full = PAD && (xb / BS) * BS + BS < a.d0;
            int code[4];
            float outv[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float pred = j ? S[t][j - 1] : L;
                const float e    = __fsub_rn(S[t][j], pred);
                if (PAD) {
                    if (full) {
                        const bool q = __fsqrt_rn(__fmul_rn(e, e)) < Rf;
                        code[j]      = q ? __float2int_rn(__fadd_rn(e, Rf)) : 0;
                        outv[j]      = q ? 0.0f : S[t][j];
                    } else {
                        const bool q = fabsf(e) < Rf;
                        code[j]      = q ? __float2int_rz(__fadd_rn(e, Rf)) : 0;
                        outv[j]      = q ? __fmul_rn(0.0f, S[t][j]) : S[t][j];
                    }
                    continue;
                }
                const bool q     = fabsf(e) < Rf;
                // (1D block / edge pads make e fractional here: truncation, as the reference's scalar form)
                code[j]          = q ? (PAD ? (int)__fadd_rn(e, Rf) : code_of(e, rmagic)) : 0;
                outv[j]          = S[t][j];
                if (STRICT) {
                    const float4 rw = RW[STRICT ? t : 0];
                    const float xr  = j == 0 ? rw.x : (j == 1 ? rw.y : (j == 2 ? rw.z : rw.w));
                    if (!strict_keep(q, pred, e, S[t][j], xr, c)) code[j] = 0;
                    outv[j] = xr;
                }
            }
            emit_row<VEC>(a, 0, xb, xt, xt < a.nxt, code, outv, h, s_hist);
        }
    }
}

template <int BS, bool VEC, bool STRICT = false, bool PAD = false>
__global__ void __launch_bounds__(256) k_dq_compress_1d(DqArgs a) {
    extern __shared__ uint32_t s_hist_dyn[];
    uint32_t* s_hist = a.smem_hist ? s_hist_dyn : nullptr;
    const Consts c   = *a.consts;
    if (c.status != VSZ_OK) return;
    if (s_hist) {
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x) s_hist[i] = 0u;
        __syncthreads();
    }
    const unsigned long long warps_total = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long warp0       = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    HistAcc h;
    dq1d_units<BS, VEC, STRICT, PAD>(a, c, warp0, a.nunits, warps_total, s_hist, h);
    hist_flush_block(a, s_hist, h);
}

template <int BS, bool VEC>
__global__ void __launch_bounds__(256)
    k_dq_compress_1d_batch(const DqArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks,
                           uint32_t* __restrict__ next) {
    extern __shared__ uint32_t s_hist_dyn[];
    __shared__ uint32_t s_task;
    for (uint32_t t = dq_block_next_task(next, &s_task); t < ntasks; t = dq_block_next_task(next, &s_task)) {
        const BatchTask tk = tasks[t];
        const DqArgs& a    = args[tk.field];
        const Consts c     = *a.consts;
        if (c.status != VSZ_OK) continue;
        uint32_t* s_hist = a.smem_hist ? s_hist_dyn : nullptr;
        if (s_hist) {
            for (int i = threadIdx.x; i < a.dict; i += blockDim.x) s_hist[i] = 0u;
            __syncthreads();
        }
        HistAcc h;
        dq1d_units<BS, VEC>(a, c, tk.u0 + (threadIdx.x >> 5), tk.u1, blockDim.x >> 5, s_hist, h);
        hist_flush_block(a, s_hist, h);
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------
// Outlier compaction: exclusive scan of seg_count in segment (= row-major) order with a single
// pass decoupled look-back, then each warp copies whole segments from scratch to their final
// place.  The destination is a byte address (the outlier section of a packed block need not be
// 4-byte aligned).
// ------------------------------------------------------------------------------------------

constexpr int kGatherThreads = 256;
constexpr int kGatherPerThread = 16;
constexpr int kGatherTile = kGatherThreads * kGatherPerThread;  // segments per tile

// One tile of 4096 row segments of one field: the next ticket of the field's look-back.  The
// status is read once per block, so the early exit is uniform.
// Copies the n outliers of segment s from scratch to outlier index dst0 of the destination (one
// warp).  A byte destination is written as whole aligned words, each the bytes of two neighbouring
// values (funnel shift); only the partial words at the run's two ends, shared with the
// neighbouring runs, are written byte by byte.
__device__ __forceinline__ void copy_segment(const GatherArgs& g, uint8_t* out_bytes, size_t s, uint32_t n,
                                             unsigned long long dst0) {
    const unsigned lane = lane_id();
    const float* src    = g.scratch + s * kSegX;
    if (g.out_f32) {
        for (uint32_t i = lane; i < n; i += 32) g.out_f32[dst0 + i] = src[i];
        return;
    }
    uint8_t* d          = out_bytes + 4 * dst0;
    const uint32_t a    = (uint32_t)(reinterpret_cast<uintptr_t>(d) & 3u);
    const uint32_t* s32 = reinterpret_cast<const uint32_t*>(src);
    if (a == 0) {
        uint32_t* dw = reinterpret_cast<uint32_t*>(d);
        for (uint32_t i = lane; i < n; i += 32) dw[i] = s32[i];
        return;
    }
    uint32_t* dw = reinterpret_cast<uint32_t*>(d + (4 - a));  // word j: top a bytes of value j, low 4 - a of j + 1
    for (uint32_t j = lane; j + 1 < n; j += 32) dw[j] = __funnelshift_r(s32[j], s32[j + 1], 8 * (4 - a));
    if (lane == 0) {
        const uint32_t b0 = s32[0], bl = s32[n - 1];
        for (uint32_t t = 0; t < 4 - a; t++) d[t] = (uint8_t)(b0 >> (8 * t));                    // value 0, low bytes
        for (uint32_t t = 0; t < a; t++) d[4 * n - a + t] = (uint8_t)(bl >> (8 * (4 - a + t)));  // value n-1, top bytes
    }
}

__device__ __forceinline__ void gather_tile(const GatherArgs& g) {
    __shared__ uint32_t s_off[kGatherTile];
    __shared__ uint8_t s_cnt[kGatherTile];
    __shared__ uint32_t s_warp[kGatherThreads / 32];
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_tile;
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        s_ok = (*g.status == VSZ_OK);
        if (s_ok) s_tile = atomicAdd(g.tile_counter, 1u);
    }
    __syncthreads();
    if (!s_ok) return;
    const uint32_t tile = s_tile;
    const size_t seg0   = (size_t)tile * kGatherTile + (size_t)threadIdx.x * kGatherPerThread;
    uint32_t cnt[kGatherPerThread];
    uint32_t sum = 0;
    if (seg0 + kGatherPerThread <= g.nseg && (reinterpret_cast<uintptr_t>(g.seg_count) & 15u) == 0) {
        const uint4 v = *reinterpret_cast<const uint4*>(g.seg_count + seg0);
        const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < kGatherPerThread; k++) {
            cnt[k] = (w4[k >> 2] >> (8 * (k & 3))) & 0xffu;
            sum += cnt[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < kGatherPerThread; k++) {
            size_t s = seg0 + k;
            cnt[k]   = (s < g.nseg) ? g.seg_count[s] : 0u;
            sum += cnt[k];
        }
    }
    // block exclusive scan of per-thread sums
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += v;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t run = 0;
        for (int i = 0; i < kGatherThreads / 32; i++) run += s_warp[i];
        const unsigned long long b = lookback_publish_warp(g.tile_status, tile, run, g.status);
        if (threadIdx.x == 0) {
            uint32_t r2 = 0;
            for (int i = 0; i < kGatherThreads / 32; i++) {
                uint32_t v = s_warp[i];
                s_warp[i]  = r2;
                r2 += v;
            }
            s_base = b;
            if (tile == g.ntiles - 1) *g.total = b + run;
        }
    }
    __syncthreads();
    uint32_t run = incl - sum + s_warp[w];
#pragma unroll
    for (int k = 0; k < kGatherPerThread; k++) {
        s_off[threadIdx.x * kGatherPerThread + k] = run;
        s_cnt[threadIdx.x * kGatherPerThread + k] = (uint8_t)cnt[k];
        run += cnt[k];
    }
    __syncthreads();
    const unsigned long long base = s_base;
    const size_t tseg0            = (size_t)tile * kGatherTile;
    if (g.seg_off) {  // split copy: record the offsets, k_outlier_copy moves the values
        for (int k = threadIdx.x; k < kGatherTile; k += kGatherThreads)
            if (tseg0 + k < g.nseg) g.seg_off[tseg0 + k] = s_off[k];
        if (threadIdx.x == 0) g.tile_base[tile] = base;
        return;
    }
    uint8_t* out_bytes = g.out_bytes ? g.out_bytes + g.out_off.eval() : nullptr;
    // warp-cooperative copies of the non-empty segments: each warp scans 32 segment counts at a
    // time from shared memory and visits only those with outliers
    for (int k0 = w * 32; k0 < kGatherTile; k0 += kGatherThreads) {
        const int kk = k0 + (int)lane;
        const bool has = (tseg0 + kk < g.nseg) && s_cnt[kk] != 0;
        unsigned nz = __ballot_sync(0xffffffffu, has);
        while (nz) {
            const int k = k0 + __ffs(nz) - 1;
            nz &= nz - 1;
            copy_segment(g, out_bytes, tseg0 + k, s_cnt[k], base + s_off[k]);
        }
    }
}

__global__ void __launch_bounds__(kGatherThreads) k_outlier_gather(GatherArgs g) { gather_tile(g); }

// Split copy: every warp of the grid takes 32 segments at a time and copies the non-empty ones.
__global__ void __launch_bounds__(256) k_outlier_copy(GatherArgs g) {
    if (*g.status != VSZ_OK || *g.total == 0) return;  // a field without outliers returns at once
    const unsigned lane = lane_id();
    uint8_t* out_bytes  = g.out_bytes ? g.out_bytes + g.out_off.eval() : nullptr;
    const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t s0 = ((size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; s0 < g.nseg;
         s0 += nwarps * 32) {
        const size_t s    = s0 + lane;
        const uint32_t cn = (s < g.nseg) ? g.seg_count[s] : 0u;
        unsigned nz       = __ballot_sync(0xffffffffu, cn != 0u);
        while (nz) {
            const int k = __ffs(nz) - 1;
            nz &= nz - 1;
            const size_t sk = s0 + k;
            const uint32_t n = __shfl_sync(0xffffffffu, cn, k);
            copy_segment(g, out_bytes, sk, n, g.tile_base[sk / kGatherTile] + g.seg_off[sk]);
        }
    }
}

// Many fields: one task per tile of each field (tasks[t].field; the field's tickets keep its tiles
// in look-back order, and the holder of every earlier ticket is already running).
__global__ void __launch_bounds__(kGatherThreads)
    k_outlier_gather_batch(const GatherArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const GatherArgs g = args[tasks[t].field];
        gather_tile(g);
        __syncthreads();  // the next task reuses shared memory
    }
}

// Many fields: min/max over element ranges (tasks[t] = field, [u0, u1) elements, u0 a multiple of 4).
__global__ void __launch_bounds__(256)
    k_minmax_batch(const MinmaxField* __restrict__ f, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    __shared__ uint32_t smax[8], smin[8];
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk = tasks[t];
        const float* x     = f[tk.field].x;
        uint32_t kmax = 0u, kmin = 0xffffffffu;
        const bool aligned = ((reinterpret_cast<uintptr_t>(x) & 15u) == 0);
        const unsigned long long q0 = aligned ? tk.u0 / 4 : 0, q1 = aligned ? tk.u1 / 4 : 0;
        const float4* x4 = reinterpret_cast<const float4*>(x);
        for (unsigned long long i = q0 + threadIdx.x; i < q1; i += blockDim.x) {
            const float4 v   = __ldcs(&x4[i]);
            const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (e[j] == e[j]) {
                    kmax = max(kmax, f2key(e[j]));
                    kmin = min(kmin, f2key(e[j]));
                }
        }
        for (unsigned long long i = (aligned ? q1 * 4 : tk.u0) + threadIdx.x; i < tk.u1; i += blockDim.x) {
            const float v = x[i];
            if (v == v) {
                kmax = max(kmax, f2key(v));
                kmin = min(kmin, f2key(v));
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
            kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
        }
        if ((threadIdx.x & 31) == 0) {
            smax[threadIdx.x >> 5] = kmax;
            smin[threadIdx.x >> 5] = kmin;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int i = 1; i < (int)(blockDim.x >> 5); i++) {
                kmax = max(kmax, smax[i]);
                kmin = min(kmin, smin[i]);
            }
            atomicMax(&f[tk.field].mm[0], kmax);
            atomicMin(&f[tk.field].mm[1], kmin);
        }
        __syncthreads();
    }
}

// Many fields: error-bound constants, one thread per field.
__global__ void k_consts_batch(const ConstsField* __restrict__ f, uint32_t nfields) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nfields) return;
    const ConstsField c = f[i];
    consts_of(c.mode, c.eb, c.mm, c.x, c.consts, c.status);
}

// ------------------------------------------------------------------------------------------
// Host-side launchers
// ------------------------------------------------------------------------------------------

int launch_eb_setup(int mode, double eb, const float* d_in, size_t n, Consts* d_consts, uint32_t* d_mm,
                    cudaStream_t st, int* status_word) {
    if (mode == VSZ_MODE_R2R) {
        // {0, 0xffffffff} by memsets: a copy from a host array would, under stream capture, bake
        // that host address into the graph
        if (cudaMemsetAsync(d_mm, 0, 4, st) != cudaSuccess || cudaMemsetAsync(d_mm + 1, 0xff, 4, st) != cudaSuccess)
            return VSZ_ERR_CUDA;
        size_t nb = (n + 1023) / 1024; int blocks = (int)(nb < (size_t)(152 * 8) ? nb : (size_t)(152 * 8));
        if (blocks < 1) blocks = 1;
        k_minmax<<<blocks, 256, 0, st>>>(d_in, n, d_mm);
        count_launch();
    }
    k_consts<<<1, 32, 0, st>>>(mode, eb, d_mm, d_in, d_consts, status_word);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

// The most dynamic shared memory a dual-quant kernel takes: a shared histogram of up to 16384
// bins and the 3D previous planes.  Every kernel is opted in to it once, so that a later launch
// with a larger dictionary than the first still fits.
constexpr int kDqSmemMax = 16384 * 4 + 8 * (int)sizeof(PrevRows);

template <int NDIM, int BS>
static void launch_23d(const DqArgs& a, bool vec, int grid, size_t smem, cudaStream_t st) {
    // tail columns exist only when d0 % 8 != 0 (and then never with 16-byte rows)
    const bool tail = (a.d0 % 8) != 0;
    // dynamic shared memory: [histogram, padded to 16 bytes][3D: previous plane, 8 warps x 4 KB]
    if (a.smem_hist) smem = (size_t)((a.dict + 3) & ~3) * sizeof(uint32_t);
    if (NDIM == 3) smem += 8 * 8 * 4 * 32 * sizeof(float);
    static std::atomic<unsigned long long> attr[4];
    auto go = [&](auto kern, std::atomic<unsigned long long>& at) {
        smem_limit_once(kern, kDqSmemMax, at);
        kern<<<grid, 256, smem, st>>>(a);
    };
    static std::atomic<unsigned long long> attr_strict{0}, attr_pad{0};
    // strict and padded fields: general loads, tail columns decided at run time
    if (a.strict) go(k_dq_compress_23d<NDIM, BS, false, true, true>, attr_strict);
    else if (a.pad.vals) go(k_dq_compress_23d<NDIM, BS, false, true, false, true>, attr_pad);
    else if (vec && !tail) go(k_dq_compress_23d<NDIM, BS, true, false>, attr[0]);
    else if (vec) go(k_dq_compress_23d<NDIM, BS, true, true>, attr[1]);
    else if (!tail) go(k_dq_compress_23d<NDIM, BS, false, false>, attr[2]);
    else go(k_dq_compress_23d<NDIM, BS, false, true>, attr[3]);
    count_launch();
}

template <int BS>
static void launch_1d(const DqArgs& a, bool vec, int grid, size_t smem, cudaStream_t st) {
    static std::atomic<unsigned long long> attr[4];
    auto go = [&](auto kern, std::atomic<unsigned long long>& at) {
        smem_limit_once(kern, kDqSmemMax, at);
        kern<<<grid, 256, smem, st>>>(a);
    };
    if (a.strict) go(k_dq_compress_1d<BS, false, true>, attr[0]);
    else if (a.pad.vals) go(k_dq_compress_1d<BS, false, false, true>, attr[1]);
    else if (vec) go(k_dq_compress_1d<BS, true>, attr[2]);
    else go(k_dq_compress_1d<BS, false>, attr[3]);
    count_launch();
}

template <int NDIM>
static int dispatch_bs(const DqArgs& a, int bs, bool vec, int grid, size_t smem, cudaStream_t st) {
    // Block sizes must divide the 128-wide warp tile so every tile starts a Lorenzo block.
    auto go = [&](auto bs_c) {
        constexpr int B = decltype(bs_c)::value;
        if constexpr (NDIM == 1) launch_1d<B>(a, vec, grid, smem, st);
        else launch_23d<NDIM, B>(a, vec, grid, smem, st);
    };
    switch (bs) {
        case 8: go(std::integral_constant<int, 8>{}); break;
        case 16: go(std::integral_constant<int, 16>{}); break;
        case 32: go(std::integral_constant<int, 32>{}); break;
        case 64: go(std::integral_constant<int, 64>{}); break;
        default: return VSZ_ERR_UNSUPPORTED;
    }
    return VSZ_OK;
}

int launch_dq_compress(DqArgs a, int ndim, int bs, cudaStream_t st, int num_sms) {
    const bool vec = (a.d0 % 4 == 0) && ((reinterpret_cast<uintptr_t>(a.x) & 15u) == 0) &&
                     ((reinterpret_cast<uintptr_t>(a.code) & 7u) == 0);
    if (a.nunits == 0) return VSZ_OK;
    size_t smem = a.smem_hist ? (size_t)a.dict * sizeof(uint32_t) : 0;
    long long want = (long long)((a.nunits + 7) / 8);
    long long cap = (long long)num_sms * 16; int grid = (int)(want < cap ? want : cap);
    if (grid < 1) grid = 1;
    int rc;
    if (ndim == 1) rc = dispatch_bs<1>(a, bs, vec, grid, smem, st);
    else if (ndim == 2) rc = dispatch_bs<2>(a, bs, vec, grid, smem, st);
    else rc = dispatch_bs<3>(a, bs, vec, grid, smem, st);
    if (rc) return rc;
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_outlier_gather(GatherArgs g, cudaStream_t st, int num_sms) {
    g.ntiles = (uint32_t)((g.nseg + kGatherTile - 1) / kGatherTile);
    if (g.ntiles == 0) {
        return cudaMemsetAsync(g.total, 0, sizeof(unsigned long long), st) == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
    }
    if (cudaMemsetAsync(g.tile_status, 0, sizeof(unsigned long long) * g.ntiles, st) != cudaSuccess) return VSZ_ERR_CUDA;
    if (cudaMemsetAsync(g.tile_counter, 0, sizeof(uint32_t), st) != cudaSuccess) return VSZ_ERR_CUDA;
    k_outlier_gather<<<g.ntiles, kGatherThreads, 0, st>>>(g);
    count_launch();
    if (g.seg_off) {
        const long long want = (long long)((g.nseg + 255) / 256), cap = (long long)(num_sms > 0 ? num_sms : 152) * 8;
        k_outlier_copy<<<(unsigned)(want < cap ? want : cap), 256, 0, st>>>(g);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_minmax_batch(const MinmaxField* f, const BatchTask* tasks, uint32_t ntasks, cudaStream_t st, int num_sms) {
    if (ntasks == 0) return VSZ_OK;
    const uint32_t grid = ntasks < (uint32_t)num_sms * 8 ? ntasks : (uint32_t)num_sms * 8;
    k_minmax_batch<<<grid, 256, 0, st>>>(f, tasks, ntasks);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_consts_batch(const ConstsField* f, uint32_t nfields, cudaStream_t st) {
    if (nfields == 0) return VSZ_OK;
    k_consts_batch<<<(nfields + 127) / 128, 128, 0, st>>>(f, nfields);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_dq_compress_batch(const DqArgs* args, const BatchTask* tasks, uint32_t ntasks, int ndim, int bs, bool vec,
                             bool tail, uint32_t hist_words, uint32_t* next, cudaStream_t st, int num_sms) {
    if (ntasks == 0) return VSZ_OK;
    size_t smem = (size_t)hist_words * sizeof(uint32_t);
    if (ndim == 3) smem += sizeof(PrevRows) * 8;
    const uint32_t cap = (uint32_t)num_sms * (ndim == 1 ? 8u : 3u);
    const uint32_t grid = ntasks < cap ? ntasks : cap;
    int rc = VSZ_OK;
    auto go23 = [&](auto kern, std::atomic<unsigned long long>& attr) {
        smem_limit_once(kern, kDqSmemMax, attr);
        kern<<<grid, 256, smem, st>>>(args, tasks, ntasks, hist_words, next);
    };
    auto go1 = [&](auto kern, std::atomic<unsigned long long>& attr) {
        smem_limit_once(kern, kDqSmemMax, attr);
        kern<<<grid, 256, smem, st>>>(args, tasks, ntasks, next);
    };
    auto pick = [&](auto nd_c, auto bs_c) {
        constexpr int ND = decltype(nd_c)::value, B = decltype(bs_c)::value;
        static std::atomic<unsigned long long> attr[4];
        if constexpr (ND == 1) {
            if (vec) go1(k_dq_compress_1d_batch<B, true>, attr[0]);
            else go1(k_dq_compress_1d_batch<B, false>, attr[1]);
        } else {
            if (vec && !tail) go23(k_dq_compress_23d_batch<ND, B, true, false>, attr[0]);
            else if (vec) go23(k_dq_compress_23d_batch<ND, B, true, true>, attr[1]);
            else if (!tail) go23(k_dq_compress_23d_batch<ND, B, false, false>, attr[2]);
            else go23(k_dq_compress_23d_batch<ND, B, false, true>, attr[3]);
        }
    };
    auto by_bs = [&](auto nd_c) {
        switch (bs) {
            case 8: pick(nd_c, std::integral_constant<int, 8>{}); break;
            case 16: pick(nd_c, std::integral_constant<int, 16>{}); break;
            case 32: pick(nd_c, std::integral_constant<int, 32>{}); break;
            case 64: pick(nd_c, std::integral_constant<int, 64>{}); break;
            default: rc = VSZ_ERR_UNSUPPORTED;
        }
    };
    if (ndim == 1) by_bs(std::integral_constant<int, 1>{});
    else if (ndim == 2) by_bs(std::integral_constant<int, 2>{});
    else by_bs(std::integral_constant<int, 3>{});
    if (rc) return rc;
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_outlier_gather_batch(const GatherArgs* args, const BatchTask* tasks, uint32_t ntasks, cudaStream_t st,
                                int num_sms) {
    if (ntasks == 0) return VSZ_OK;
    const uint32_t cap  = (uint32_t)num_sms * 4;
    const uint32_t grid = ntasks < cap ? ntasks : cap;
    k_outlier_gather_batch<<<grid, kGatherThreads, 0, st>>>(args, tasks, ntasks);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int set_spin_limit_dq(long long polls) { return set_spin_limit_this_unit(polls); }

size_t gather_tmp_bytes(size_t nseg) {
    size_t ntiles = (nseg + kGatherTile - 1) / kGatherTile;
    return 16 + 8 * (ntiles + 1);
}

}  // namespace vsz

// ------------------------------------------------------------------------------------------
// Allocation-free outlier gather.
//
// Some callers of this library cannot call cudaMalloc: a serving process whose device memory is
// wholly owned by another allocator or budget, a latency-critical loop that cannot afford the
// implicit synchronisation and unpredictable latency of an allocation, or a plugin host that hands
// a plugin only its input and output buffers.  vsz_outlier_gather_noalloc gives them the gather
// without a caller workspace: its look-back scratch (a status word, a tile ticket and one status
// entry per tile of 4096 row segments) lives in the file-scope array below, which every GPU that
// loads this library holds until the process exits.
// ------------------------------------------------------------------------------------------
namespace vsz {

constexpr size_t kNoAllocGatherMaxTiles   = 65536;                                  // tiles of 4096 segments
constexpr size_t kNoAllocGatherMaxSegments = kNoAllocGatherMaxTiles * kGatherTile;  // 2^28 row segments
constexpr size_t kNoAllocGatherBytes      = 256 + 8 * (kNoAllocGatherMaxTiles + 1);  // ~512 KiB

static __device__ __align__(256) uint8_t g_noalloc_gather_scratch[kNoAllocGatherBytes];

// The array's name is only a host-side stand-in in host code; its device address comes from
// cudaGetSymbolAddress with the device current.  It is looked up on every call (a table lookup in
// the runtime, no allocation), never cached: after cudaDeviceReset, or a primary context torn down
// and recreated, the library's device code is loaded again and the array may move.  The first call
// on a device may load that code, so make it before any stream capture.
static int noalloc_gather_scratch(uint8_t** out) {
    void* p        = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_gather_scratch);
    if (rc != cudaSuccess || !p) return VSZ_ERR_CUDA;
    *out = reinterpret_cast<uint8_t*>(p);
    return VSZ_OK;
}

}  // namespace vsz

extern "C" vsz_status vsz_outlier_gather_noalloc(int ndim, const size_t dims[3], const uint8_t* d_seg_count,
                                                 const float* d_scratch, float* d_out, uint64_t* d_count,
                                                 void* stream) {
    using namespace vsz;
    // the same field limits as vsz_outlier_gather: each dim <= 2^31 - 1, at most 2^36 elements
    if (!api::valid_dims(ndim, dims) || !d_seg_count || !d_scratch || !d_out || !d_count) return VSZ_ERR_INVALID;
    Geometry g = make_geometry(ndim, dims);
    if (g.nseg > kNoAllocGatherMaxSegments) return VSZ_ERR_CAPACITY;  // beyond the static scratch
    uint8_t* base = nullptr;
    int rc        = noalloc_gather_scratch(&base);
    if (rc != VSZ_OK) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    GatherArgs ga{};
    ga.status       = reinterpret_cast<int*>(base);
    ga.tile_counter = reinterpret_cast<uint32_t*>(base + 4);
    ga.tile_status  = reinterpret_cast<unsigned long long*>(base + 256);
    ga.seg_count    = d_seg_count;
    ga.scratch      = d_scratch;
    ga.nseg         = g.nseg;
    ga.out_f32      = d_out;
    ga.total        = reinterpret_cast<unsigned long long*>(d_count);
    // The array keeps the previous call's contents: clear the status word here; the launcher
    // clears the tile ticket and the tile statuses it will use.
    if (cudaMemsetAsync(ga.status, 0, sizeof(int), st) != cudaSuccess) return VSZ_ERR_CUDA;
    return launch_outlier_gather(ga, st);
}

