// Dual-quantization decompress on sm_103a: outlier placement + reverse Lorenzo + dequantization.
//
// Replaces, from szcompressor/vecSZ:
//   outlier scatter           src/vecsz_interface.hh:313-317
//   x_lorenzo_{1,2,3}d1l      src/dualquant.hh:915-1043
//
// Per element, in the reference's FP32 operation order (zero halo per block, or with padding the
// block's pad values from the archive's pad section, src/dualquant.hh:946-1016):
//   s = code == 0 ? outlier : (float)(pred + (float)(code - R))
//   pred: 1D s[x-1]; 2D (N + W) - NW; 3D XYZ - XY - XZ - YZ + X + Y + Z, left to right
//   xhat = (float)((double) s * 2eb)                 (dequant(), vsz_device.cuh)
// The outlier of an element with code 0 is found by its rank among the zero codes in row-major
// order: seg_off[row segment of 256 columns] (an exclusive scan of the zero counts the Huffman
// decoder produced) plus the zeros before it inside the segment.
#include <cstdint>
#include <cstdlib>
#include <type_traits>

#include "vsz_device.cuh"
#include "vsz_kernels.h"

namespace vsz {

constexpr int kDSeg = 256;  // decompress row segment (one warp of 8-wide blocks)

// ------------------------------------------------------------------------------------------
// Fast path, block size 8: one lane reconstructs one whole Lorenzo block (8 x by 8 y, plane by
// plane in z) -- the x, y and z recurrences never leave the thread.  A warp covers 32 consecutive
// blocks (one 256-wide row segment), so code loads (16 B) and value stores (32 B) of a row are
// contiguous across the warp.  Codes are prefetched one row ahead into registers; the previous
// plane of every lane's block lives in shared memory [row][column][lane] (lane-minor, so
// conflict-free).  Rows are processed in a rolled loop (8 columns unrolled): the body stays small
// enough for the instruction cache (two rows per iteration measured fastest).
// ------------------------------------------------------------------------------------------

// Any zero 16-bit half in a word (exact: a borrow out of the low half needs the low half zero).
__device__ __forceinline__ uint32_t zero_halves(uint32_t w) { return (w - 0x00010001u) & ~w & 0x80008000u; }

// Strict archives: an outlier is the input value; the Lorenzo chain continues from its
// prequantized value, by the compressor's rule for that column.
template <int NDIM>
__device__ __forceinline__ float strict_prequant(float v, uint32_t col, const DqDecArgs& a, const Consts& c) {
    if (NDIM == 3 && col >= a.xtail) return prequant_scalar(v, c.r_d);
    return prequant_vec(v, c.r_f);
}

typedef float DqPlane[8][8][32];  // one warp's plane of 8 x 8 blocks, [row][column][lane]
typedef float4 DqPlaneV[8][2][32];  // the same bytes for the separable pass: [row][half][lane] x 4 columns

// Units ui = first, first + stride, ... < end of one field (one warp each; `wib` = this warp's
// plane in s_prev).  REDO: the units the separable kernel listed instead (end = their count,
// read by the caller: final in stream order).
template <int NDIM, bool VEC, bool PAD, bool REDO>
__device__ __forceinline__ void dq_b8_units(const DqDecArgs& a, uint32_t first, uint32_t end, uint32_t stride,
                                            DqPlane* s_prev, unsigned wib) {
    const Consts c = *a.consts;
    if (c.status != VSZ_OK || *a.status != VSZ_OK) return;
    const int R           = a.R;
    // (float)(code - R) exactly: 2^23 + code as float bits, minus 2^23 + R (both exact, R < 2^16)
    const float rbias     = 8388608.0f + (float)R;
    const uint32_t rpair  = (uint32_t)R | ((uint32_t)R << 16);
    const unsigned lane   = lane_id();

    // Narrow rows (a.ygrp > 1, rows of at most 16 blocks): the warp takes ygrp consecutive
    // y-blocks of one z-block, a group of nbx8 lanes per y-block (lanes past ygrp * nbx8 idle), so
    // that its lanes are not spent on columns past the row's end.  A lane still reconstructs one
    // whole block; the lanes of a group share a row, and outliers are ranked per group.
    const uint32_t G   = (REDO || PAD || NDIM == 1) ? 1u : a.ygrp;
    const uint32_t gw  = G > 1 ? a.nbx8 : 32u;  // lanes per group
    const uint32_t grp = G > 1 ? lane / gw : 0u;
    const uint32_t gl0 = grp * gw;              // the group's first lane
    const uint32_t lbx = lane - gl0;            // this lane's block along x in its segment
    const uint32_t gll = min(gl0 + gw - 1u, 31u);  // the group's last lane
    const unsigned gmy = (gw >= 32u) ? 0xffffffffu : (((1u << gw) - 1u) << gl0);  // my group's lanes
    // When a unit spans whole rows (one segment per row), the rows of a block in one plane are
    // consecutive in the field, so the outlier rank at a row's start is the one at the previous
    // row's start plus that row's zeros: the zeros from the chunk start are counted once per plane.
    const bool carry = NDIM >= 2 && a.chunk_off != nullptr && a.nxs == 1u;

    // unit indices fit 32 bits (n <= 2^36 elements, 2048 per unit): 32-bit divisions only.
    for (uint32_t ui = first; ui < end; ui += stride) {
        const uint32_t u  = REDO ? a.redo[1 + ui] : ui;
        uint32_t xs, yb, zb;
        if (G > 1) {  // units: (group of G y-blocks, z-block)
            xs = 0;
            yb = (u % a.nyb_g) * G + grp;
            zb = (NDIM == 3) ? u / a.nyb_g : 0u;
        } else {
            xs = u % a.nxs;
            const uint32_t r = u / a.nxs;
            yb = (NDIM >= 2) ? r % a.nyb : 0u;
            zb = (NDIM == 3) ? r / a.nyb : 0u;
        }
        const bool blk_in = grp < G && (NDIM < 2 || yb < a.nyb);  // my block exists
        const uint32_t x0 = xs * kDSeg + lbx * 8;
        const uint32_t y0 = yb * 8, z0 = zb * 8;
        const int ny = (NDIM >= 2) ? (blk_in ? (int)min(8u, a.d1 - y0) : 0) : 1;
        const int nz = (NDIM == 3) ? (int)min(8u, a.d2 - z0) : 1;
        const bool col_in = blk_in && x0 < a.d0;  // VEC: d0 % 8 == 0, so all 8 columns or none
        // halo of my block (zero without padding): x-, y- and z-halo cells; in 3D the (x-1, y-1)
        // cell of a halo row is the y-halo's, in 2D the x-halo's
        float hx = 0.f, hy = 0.f, hz = 0.f;
        if (PAD && col_in) {
            const Halo hv = halo_of(a.pad, NDIM, x0 / 8, yb, zb);
            hx = hv.x;
            hy = hv.y;
            hz = hv.z;
        }

        // the 8 codes of this lane's columns (VEC: one 16-byte load), a row ahead of their use;
        // cells outside the field read as R (no zero codes, so they never enter the outlier path)
        auto load_row = [&](int zz, int y) -> uint4 {
            const size_t row = (size_t)(z0 + zz) * a.d1 + (y0 + y);
            if (VEC) {
                if (!(col_in && y < ny && zz < nz)) return make_uint4(rpair, rpair, rpair, rpair);
                return __ldcs(reinterpret_cast<const uint4*>(a.codes + row * a.d0 + x0));
            }
            const bool rin       = y < ny && zz < nz;
            const uint16_t* crow = a.codes + row * a.d0;
            uint32_t t[8];
#pragma unroll
            for (int k = 0; k < 8; k++) t[k] = (rin && x0 + k < a.d0) ? (uint32_t)crow[x0 + k] : (uint32_t)R;
            return make_uint4(t[0] | (t[1] << 16), t[2] | (t[3] << 16), t[4] | (t[5] << 16), t[6] | (t[7] << 16));
        };
        uint4 cv_next = load_row(0, 0);

        if (NDIM == 3) {
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int k = 0; k < 8; k++) s_prev[wib][i][k][lane] = hz;
        }

        for (int zz = 0; zz < nz; zz++) {
            float Cm[8];  // row y - 1 of this plane (the halo row above the block)
            float Zm[8], Zn[8];  // 3D: row y - 1 and row y of plane z - 1
#pragma unroll
            for (int k = 0; k < 8; k++) Cm[k] = hy;
            unsigned long long rbase = 0;  // carry: my group's rank at the next row's start, once known
            bool rknown = false;
#pragma unroll 2
            for (int y = 0; y < 8; y++) {
                const bool row_in = y < ny;
                const size_t row  = ((size_t)(z0 + zz) * a.d1 + (y0 + y));
                const bool all_in = row_in && (x0 + 7 < a.d0);
                const uint4 cv    = cv_next;
                cv_next           = (y < 7) ? load_row(zz, y + 1) : load_row(zz + 1, 0);
                const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                auto code_at = [&](int k) -> uint32_t { return (cw[k >> 1] >> (16 * (k & 1))) & 0xffffu; };
                auto in_at   = [&](int k) -> bool { return all_in || (row_in && x0 + (uint32_t)k < a.d0); };
                // ---- outliers of this row segment, ranked in row-major order.  Cells outside the
                // field read code R (never 0), so no range test is needed here or in the row pass:
                // their values only ever feed other cells outside the field.
                uint32_t zm = 0;
                if (zero_halves(cv.x) | zero_halves(cv.y) | zero_halves(cv.z) | zero_halves(cv.w)) {
#pragma unroll
                    for (int k = 0; k < 8; k++) zm |= (code_at(k) == 0u) ? (1u << k) : 0u;
                }
                unsigned long long obase = 0;
                const unsigned zlanes = __ballot_sync(0xffffffffu, zm != 0u);
                if (zlanes) {
                    uint32_t cnt = __popc(zm), incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= (unsigned)o) incl += t;
                    }
                    if (G > 1) {  // ranks within my group's row: less the lanes of earlier groups
                        const uint32_t before = __shfl_sync(0xffffffffu, incl, gl0 ? gl0 - 1 : 0);
                        if (gl0) incl -= before;
                    }
                    unsigned long long seg_base = rbase;
                    if (a.chunk_off) {
                        // zeros before this row segment: the chunk's offset plus the zeros between the
                        // chunk start and the segment start, counted by the warp (at most 511 codes),
                        // once for each group that has an outlier in this row and no carried rank
                        const unsigned long long q = row * a.d0 + (unsigned long long)xs * kDSeg;
                        const unsigned need = carry ? __ballot_sync(0xffffffffu, zm != 0u && !rknown) : zlanes;
                        for (uint32_t g = 0; g < G; g++) {
                            const unsigned gmask = (gw >= 32u) ? 0xffffffffu : (((1u << gw) - 1u) << (g * gw));
                            if (!(need & gmask)) continue;  // the same for the whole warp
                            const unsigned long long qg = __shfl_sync(0xffffffffu, q, g * gw);
                            const unsigned long long c0 = qg & ~511ull;
                            uint32_t zc = 0;
                            const unsigned long long lo = c0 + (unsigned long long)lane * 16;
#pragma unroll
                            for (int t = 0; t < 16; t++)
                                if (lo + t < qg) zc += (a.codes[lo + t] == 0);
#pragma unroll
                            for (int o = 16; o > 0; o >>= 1) zc += __shfl_xor_sync(0xffffffffu, zc, o);
                            if (g == grp) seg_base = a.chunk_off[qg >> 9] - a.chunk_off[0] + zc;  // relative: batches
                        }
                        if (carry) {  // the next row starts this row's zeros later
                            const uint32_t tot = __shfl_sync(0xffffffffu, incl, gll);
                            if (zlanes & gmy) {
                                rbase  = seg_base + tot;
                                rknown = true;
                            }
                        }
                    } else {
                        seg_base = a.seg_off[row * a.nxs + xs];
                    }
                    obase = seg_base + (incl - cnt);
                }
                // ---- reverse Lorenzo along the row; an element with code 0 takes its outlier
                float C[8];
                auto row_pass = [&](auto with_outliers) {
                    float pZ = 0.f, pYZ = 0.f;
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        float pred;
                        if (NDIM == 1) {
                            pred = k ? C[k - 1] : hx;
                        } else if (NDIM == 2) {
                            const float X  = k ? C[k - 1] : hx;
                            const float XY = k ? Cm[k - 1] : hx;
                            pred           = __fsub_rn(__fadd_rn(Cm[k], X), XY);  // (N + W) - NW
                        } else {
                            // previous plane: this row (z-1, y) from shared memory, the row above
                            // (z-1, y-1) kept from the row before; both rolled along x
                            const float Z   = s_prev[wib][y][k][lane];
                            const float YZ  = y ? Zm[k] : (zz ? hy : hz);
                            Zn[k]           = Z;
                            const float XYZ = k ? pYZ : (zz ? (y ? hx : hy) : hz);
                            const float XZ  = k ? pZ : (zz ? hx : hz);
                            pZ              = Z;
                            pYZ             = YZ;
                            const float XY  = k ? Cm[k - 1] : (y ? hx : hy);
                            const float X   = k ? C[k - 1] : hx;
                            pred = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fsub_rn(XYZ, XY), XZ), YZ), X), Cm[k]),
                                             Z);
                        }
                        const uint32_t cd = code_at(k);
                        float s = __fadd_rn(pred, __fsub_rn(__uint_as_float(0x4B000000u | cd), rbias));
                        if (decltype(with_outliers)::value) {
                            if (zm & (1u << k)) {
                                const unsigned long long oi = obase + __popc(zm & ((1u << k) - 1u));
                                s = 0.f;
                                if (oi < a.n_outliers) s = a.outliers[oi];
                                else set_status(a.status, VSZ_ERR_CORRUPT);
                                if (a.strict) s = strict_prequant<NDIM>(s, x0 + (uint32_t)k, a, c);
                            }
                        }
                        C[k] = s;
                    }
                };
                if (zm) row_pass(std::true_type{});
                else row_pass(std::false_type{});
                float* orow = a.out + row * a.d0;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    float xo[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) xo[k] = dequant(C[4 * h + k], c.c_d, c.c_hi, c.c_lo, c.dq_fast);
                    if (a.strict && zm) {  // strict outliers are output as stored
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const int kk = 4 * h + k;
                            if (zm & (1u << kk)) {
                                const unsigned long long oi = obase + __popc(zm & ((1u << kk) - 1u));
                                xo[k] = oi < a.n_outliers ? a.outliers[oi] : 0.f;
                            }
                        }
                    }
                    if (VEC && all_in) {
                        __stcs(reinterpret_cast<float4*>(orow + x0 + 4 * h), make_float4(xo[0], xo[1], xo[2], xo[3]));
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            if (in_at(4 * h + k)) orow[x0 + 4 * h + k] = xo[k];
                    }
                }
                if (NDIM == 3 && y > 0) {  // row y-1 of this plane is no longer needed as "plane z-1"
#pragma unroll
                    for (int k = 0; k < 8; k++) s_prev[wib][y - 1][k][lane] = Cm[k];
                }
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    Cm[k] = C[k];
                    if (NDIM == 3) Zm[k] = Zn[k];
                }
                if (NDIM == 1) break;
            }
            if (NDIM == 3) {
#pragma unroll
                for (int k = 0; k < 8; k++) s_prev[wib][7][k][lane] = Cm[k];
            }
        }
    }
}

template <int NDIM, bool VEC, bool PAD = false, bool REDO = false>
__global__ void __launch_bounds__(128, 6) k_dq_decompress_b8(DqDecArgs a) {
    extern __shared__ __align__(16) uint8_t s_dq_dyn[];
    const unsigned wib = threadIdx.x >> 5;  // warp in block (4 warps)
    const uint32_t end = REDO ? a.redo[0] : (uint32_t)a.nunits;
    dq_b8_units<NDIM, VEC, PAD, REDO>(a, blockIdx.x * (blockDim.x >> 5) + wib, end, gridDim.x * (blockDim.x >> 5),
                                      reinterpret_cast<DqPlane*>(s_dq_dyn), wib);
}

// ------------------------------------------------------------------------------------------
// Separable pass, 3D, block 8, zero halo (no padding), not strict.  With a zero halo the Lorenzo
// inverse is the block's 3D inclusive prefix sum of the residuals q = code - R, so an element takes
// three adds -- A = A(z-1) + q, B = B(y-1) + A, s = s(x-1) + B -- instead of the predictor's seven.
// While every value of the block stays below 2^21 in magnitude, every partial sum of the
// reference's order and of this one is an integer below 2^24, exact in FP32, so both give the same
// bits.  An outlier sets s; B and A are corrected from it (B = s - s(x-1), A = B - B(y-1)).  A warp
// with a block whose values leave that range (or meet a NaN or an infinity) lists its unit in
// a.redo, and the reference-order kernel redoes it afterwards.
// ------------------------------------------------------------------------------------------
// Units u = first, first + stride, ... < end of one field; s_A: A of the previous plane.
// CARRY: rows of one segment carry their outlier rank (checked at run time).
template <bool CARRY>
__device__ __forceinline__ void dq_b8s_units(const DqDecArgs& a, uint32_t first, uint32_t end, uint32_t stride,
                                             DqPlane* s_A, unsigned wib) {
    const Consts c = *a.consts;
    if (c.status != VSZ_OK || *a.status != VSZ_OK) return;
    const int R                = a.R;
    const float rbias          = 8388608.0f + (float)R;
    const uint32_t rpair       = (uint32_t)R | ((uint32_t)R << 16);
    const unsigned lane        = lane_id();
    // rows start on 32-byte boundaries (d0 % 8 == 0) when the output does
    const bool out32           = (reinterpret_cast<uintptr_t>(a.out) & 31u) == 0;
    // one segment per row: a row's outlier rank is the previous row's plus its zeros (as
    // k_dq_decompress_b8)
    const bool carry           = CARRY && a.chunk_off != nullptr && a.nxs == 1u;

    for (uint32_t u = first; u < end; u += stride) {
        const uint32_t xs = u % a.nxs;
        const uint32_t r  = u / a.nxs;
        const uint32_t yb = r % a.nyb;
        const uint32_t zb = r / a.nyb;
        const uint32_t x0 = xs * kDSeg + lane * 8;
        const uint32_t y0 = yb * 8, z0 = zb * 8;
        const int ny      = (int)min(8u, a.d1 - y0);
        const int nz      = (int)min(8u, a.d2 - z0);
        const bool col_in = x0 < a.d0;  // d0 % 8 == 0: all 8 columns or none
        auto load_row = [&](int zz, int y) -> uint4 {
            if (!(col_in && y < ny && zz < nz)) return make_uint4(rpair, rpair, rpair, rpair);
            const size_t row = (size_t)(z0 + zz) * a.d1 + (y0 + y);
            return __ldcs(reinterpret_cast<const uint4*>(a.codes + row * a.d0 + x0));
        };
        uint4 cv_next = load_row(0, 0);
        DqPlaneV* sAv = reinterpret_cast<DqPlaneV*>(s_A);  // a row's 8 A values: two 16-byte accesses
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int h = 0; h < 2; h++) sAv[wib][i][h][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t big = 0;  // largest |value| of the block, as float bits (NaN and infinity above all)

        for (int zz = 0; zz < nz; zz++) {
            float Bm[8];  // B of the row above (zero above the block)
#pragma unroll
            for (int k = 0; k < 8; k++) Bm[k] = 0.f;
            unsigned long long rbase = 0;  // carry: the rank at the next row's start, once known
            bool rknown = false;
#pragma unroll 2
            for (int y = 0; y < 8; y++) {
                const bool row_in = y < ny;
                const size_t row  = ((size_t)(z0 + zz) * a.d1 + (y0 + y));
                const bool all_in = row_in && col_in;
                const uint4 cv    = cv_next;
                cv_next           = (y < 7) ? load_row(zz, y + 1) : load_row(zz + 1, 0);
                {  // the row 4 ahead into L2 (rows of this unit only): the load one row ahead then hits L2
                    const int za = y < 4 ? zz : zz + 1, ya = (y + 4) & 7;
                    if (col_in && za < nz && ya < ny) {
                        const size_t rowa = (size_t)(z0 + za) * a.d1 + (y0 + ya);
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(a.codes + rowa * a.d0 + x0));
                    }
                }
                const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                auto code_at = [&](int k) -> uint32_t { return (cw[k >> 1] >> (16 * (k & 1))) & 0xffffu; };
                // outliers of this row segment, ranked in row-major order (as k_dq_decompress_b8)
                uint32_t zm = 0;
                if (zero_halves(cv.x) | zero_halves(cv.y) | zero_halves(cv.z) | zero_halves(cv.w)) {
#pragma unroll
                    for (int k = 0; k < 8; k++) zm |= (code_at(k) == 0u) ? (1u << k) : 0u;
                }
                unsigned long long obase = 0;
                if (__any_sync(0xffffffffu, zm != 0u)) {
                    uint32_t cnt = __popc(zm), incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= (unsigned)o) incl += t;
                    }
                    unsigned long long seg_base = rbase;
                    if (a.chunk_off) {
                        if (!rknown) {  // the same for the whole warp
                            const unsigned long long q  = row * a.d0 + (unsigned long long)xs * kDSeg;
                            const unsigned long long c0 = q & ~511ull;
                            uint32_t zc = 0;
                            const unsigned long long lo = c0 + (unsigned long long)lane * 16;
#pragma unroll
                            for (int t = 0; t < 16; t++)
                                if (lo + t < q) zc += (a.codes[lo + t] == 0);
#pragma unroll
                            for (int o = 16; o > 0; o >>= 1) zc += __shfl_xor_sync(0xffffffffu, zc, o);
                            seg_base = a.chunk_off[q >> 9] - a.chunk_off[0] + zc;  // relative: batches
                        }
                        if (carry) {
                            rbase  = seg_base + __shfl_sync(0xffffffffu, incl, 31);
                            rknown = true;
                        }
                    } else {
                        seg_base = a.seg_off[row * a.nxs + xs];
                    }
                    obase = seg_base + (incl - cnt);
                }
                float C[8], Ar[8];  // Ar: A of the row in the previous plane, then of this one
                {
                    const float4 a0 = sAv[wib][y][0][lane], a1 = sAv[wib][y][1][lane];
                    Ar[0] = a0.x, Ar[1] = a0.y, Ar[2] = a0.z, Ar[3] = a0.w;
                    Ar[4] = a1.x, Ar[5] = a1.y, Ar[6] = a1.z, Ar[7] = a1.w;
                }
                auto row_pass = [&](auto with_outliers) {
                    float sl = 0.f;  // s of the element to the left (zero left of the block)
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const float q = __fsub_rn(__uint_as_float(0x4B000000u | code_at(k)), rbias);
                        float A       = __fadd_rn(Ar[k], q);
                        float B       = __fadd_rn(Bm[k], A);
                        float sv      = __fadd_rn(sl, B);
                        if (decltype(with_outliers)::value) {
                            if (zm & (1u << k)) {
                                const unsigned long long oi = obase + __popc(zm & ((1u << k) - 1u));
                                sv = 0.f;
                                if (oi < a.n_outliers) sv = a.outliers[oi];
                                else set_status(a.status, VSZ_ERR_CORRUPT);
                                B = __fsub_rn(sv, sl);
                                A = __fsub_rn(B, Bm[k]);
                            }
                        }
                        Ar[k]                = A;
                        Bm[k]                = B;
                        sl                   = sv;
                        C[k]                 = sv;
                        big                  = max(big, __float_as_uint(sv) & 0x7fffffffu);
                    }
                };
                if (zm) row_pass(std::true_type{});
                else row_pass(std::false_type{});
                sAv[wib][y][0][lane] = make_float4(Ar[0], Ar[1], Ar[2], Ar[3]);
                sAv[wib][y][1][lane] = make_float4(Ar[4], Ar[5], Ar[6], Ar[7]);
                if (all_in) {
                    float* orow = a.out + row * a.d0;
                    float xo[8];
#pragma unroll
                    for (int k = 0; k < 8; k++) xo[k] = dequant_small(C[k], c);
                    if (out32) {  // the lane's 8 values are one 32-byte sector: one 256-bit store
                        asm volatile("st.global.cs.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(orow + x0),
                                     "f"(xo[0]), "f"(xo[1]), "f"(xo[2]), "f"(xo[3]), "f"(xo[4]), "f"(xo[5]), "f"(xo[6]),
                                     "f"(xo[7])
                                     : "memory");
                    } else {
#pragma unroll
                        for (int h = 0; h < 2; h++)
                            __stcs(reinterpret_cast<float4*>(orow + x0 + 4 * h),
                                   make_float4(xo[4 * h], xo[4 * h + 1], xo[4 * h + 2], xo[4 * h + 3]));
                    }
                }
            }
        }
        // 0x4A000000 = 2^21: a block with a larger value (or a NaN / infinity) is redone
        if (__any_sync(0xffffffffu, big >= 0x4A000000u) && lane == 0) {
            const uint32_t i = atomicAdd(a.redo, 1u);
            a.redo[1 + i]    = u;
        }
    }
}

// A check result kept in the caller's workspace: c_d's bits, the mode and exception, and a check
// word, so that bytes left there by anything else are not taken for a result.
constexpr unsigned long long kDqCacheMagic = 0x9e3779b97f4a7c15ull;
__device__ __forceinline__ unsigned long long dq_cache_check(unsigned long long key, unsigned long long v0,
                                                             unsigned long long v1) {
    return (key * kDqCacheMagic) ^ (v0 + 0x632be59bd9b4e019ull) ^ (v1 * 0xc2b2ae3d27d4eb4full) ^ 0x5bd1e995ull;
}

// Checks, for every integer 0 < s < 2^21, the two-operation dequantization of dequant_small()
// against the reference's (float)((double)s * c_d), and sets c->dq_mul (negative s follow: both
// forms are odd).  scratch: 3 words, zero on entry (mismatches, one mismatching s, block ticket);
// the last block to finish sets the mode and zeroes scratch[0] again.  cache (4 words, or null):
// the last result for this workspace; a hit for the same c_d skips the check.
__global__ void __launch_bounds__(256) k_dq_mul_verify(Consts* __restrict__ c, uint32_t* __restrict__ scratch,
                                                       unsigned long long* __restrict__ cache) {
    __shared__ uint32_t s_bad;
    const Consts k = *c;
    const unsigned long long key = (unsigned long long)__double_as_longlong(k.c_d);
    if (cache && k.status == VSZ_OK) {
        const unsigned long long ck = cache[0], v0 = cache[1], v1 = cache[2], chk = cache[3];
        if (ck == key && chk == dq_cache_check(ck, v0, v1) && (v0 & 0xffu) <= 2u) {  // uniform over the grid
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                c->dq_mul   = (int)(v0 & 0xffu);
                c->dq_exc   = __uint_as_float((uint32_t)(v0 >> 32));
                c->dq_exc_y = __uint_as_float((uint32_t)v1);
            }
            return;
        }
    }
    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    uint32_t bad = 0, which = 0;
    if (k.status == VSZ_OK) {
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1; i < (1u << 21); i += gridDim.x * blockDim.x) {
            const float s   = (float)i;  // exact
            const float y1  = __fmaf_rn(s, k.c_hi, __fmul_rn(s, k.c_lo));
            const float y2  = __double2float_rn(__dmul_rn((double)i, k.c_d));
            const bool diff = __float_as_uint(y1) != __float_as_uint(y2);
            bad += diff ? 1u : 0u;
            which = diff ? i : which;
        }
    }
    if (bad) {
        atomicAdd(&s_bad, bad);
        atomicExch(&scratch[1], which);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    if (s_bad) atomicAdd(&scratch[0], s_bad);
    __threadfence();
    if (atomicAdd(&scratch[2], 1u) != gridDim.x - 1) return;
    __threadfence();
    const uint32_t nbad = atomicAdd(&scratch[0], 0u), s1 = atomicAdd(&scratch[1], 0u);
    const int mode      = k.status != VSZ_OK ? 0 : nbad == 0 ? 1 : nbad == 1 ? 2 : 0;
    const float exc   = mode == 2 ? (float)s1 : 0.f;
    const float exc_y = mode == 2 ? __double2float_rn(__dmul_rn((double)s1, k.c_d)) : 0.f;
    c->dq_exc   = exc;
    c->dq_exc_y = exc_y;
    c->dq_mul   = mode;
    scratch[0]  = 0u;  // the separable pass counts its redo units here
    if (cache && k.status == VSZ_OK) {
        const unsigned long long v0 = (unsigned long long)mode | ((unsigned long long)__float_as_uint(exc) << 32);
        const unsigned long long v1 = __float_as_uint(exc_y);
        cache[0] = key;
        cache[1] = v0;
        cache[2] = v1;
        cache[3] = dq_cache_check(key, v0, v1);
    }
}

template <bool CARRY>
__global__ void __launch_bounds__(128, 6) k_dq_decompress_b8s(DqDecArgs a) {
    extern __shared__ __align__(16) uint8_t s_dq_dyn[];
    const unsigned wib = threadIdx.x >> 5;
    dq_b8s_units<CARRY>(a, blockIdx.x * (blockDim.x >> 5) + wib, (uint32_t)a.nunits, gridDim.x * (blockDim.x >> 5),
                 reinterpret_cast<DqPlane*>(s_dq_dyn), wib);
}

// ------------------------------------------------------------------------------------------
// Wavefront pass, 3D, block 8, no padding, fields of at most kW8MaxN elements.  The block-8
// kernels give each lane a whole 8 x 8 x 8 block, 512 elements one after another; a field with
// fewer warp units than the GPU holds then takes that chain's latency (0.1-0.3 ms) whatever its
// size.  Here a block has 8 lanes, one per row y, and lane y runs one plane behind lane y - 1: at
// step t it reconstructs row (y, z = t - y) from its own row of plane z - 1 (in registers) and
// lane y - 1's rows of planes z and z - 1 (shuffled one lane up after each step).  15 steps of 8
// elements per lane instead of 512; the predictor is the reference's, in its FP32 order, so the
// values are the same bits.  A warp holds 4 blocks along x.  Outliers are ranked from blk_off
// (zero codes before each row's x-block), so no lane waits on another for a rank.
// ------------------------------------------------------------------------------------------
template <bool VEC>
__global__ void __launch_bounds__(128, 4) k_dq_decompress_w8(DqDecArgs a) {
    const Consts c = *a.consts;
    if (c.status != VSZ_OK || *a.status != VSZ_OK) return;
    const int R           = a.R;
    const float rbias     = 8388608.0f + (float)R;
    const uint32_t rpair  = (uint32_t)R | ((uint32_t)R << 16);
    const unsigned lane   = lane_id();
    const int y           = (int)(lane & 7u);  // row of the block
    const uint32_t nxq    = (a.nbx8 + 3) / 4;  // groups of 4 blocks along x
    const bool ranks      = a.n_outliers != 0;
    const unsigned long long wtot = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    for (unsigned long long u = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         u < a.nunits; u += wtot) {
        const uint32_t xq = (uint32_t)(u % nxq);
        const unsigned long long r = u / nxq;
        const uint32_t yb = (uint32_t)(r % a.nyb), zb = (uint32_t)(r / a.nyb);
        const uint32_t bx = xq * 4 + (lane >> 3);
        const uint32_t x0 = bx * 8, z0 = zb * 8, yr = yb * 8 + (uint32_t)y;
        const int nz        = (int)min(8u, a.d2 - z0);  // the same for the whole warp
        const bool row_in   = bx < a.nbx8 && yr < a.d1;  // this lane's row exists (in every plane)
        const bool all_in   = row_in && x0 + 7 < a.d0;
        auto row_of = [&](int zz) -> size_t { return (size_t)(z0 + zz) * a.d1 + yr; };
        // the 8 codes of the lane's row in plane zz (cells outside the field read R: never an
        // outlier, and their values only feed other cells outside the field)
        auto load_row = [&](int zz) -> uint4 {
            if (!(row_in && zz < nz)) return make_uint4(rpair, rpair, rpair, rpair);
            const uint16_t* crow = a.codes + row_of(zz) * a.d0;
            if (VEC) return __ldcs(reinterpret_cast<const uint4*>(crow + x0));
            uint32_t t[8];
#pragma unroll
            for (int k = 0; k < 8; k++) t[k] = (x0 + k < a.d0) ? (uint32_t)crow[x0 + k] : (uint32_t)R;
            return make_uint4(t[0] | (t[1] << 16), t[2] | (t[3] << 16), t[4] | (t[5] << 16), t[6] | (t[7] << 16));
        };
        auto load_off = [&](int zz) -> unsigned long long {
            return (ranks && row_in && zz < nz) ? a.blk_off[row_of(zz) * a.nbx8 + bx] : 0ull;
        };
        float Zp[8], Y[8], Yp[8];  // own row of plane z - 1; rows y - 1 of planes z and z - 1
#pragma unroll
        for (int k = 0; k < 8; k++) Zp[k] = Y[k] = Yp[k] = 0.f;
        uint4 cv               = load_row(0);
        unsigned long long off = load_off(0);
        for (int t = 0; t < nz + 7; t++) {
            float up[8];  // lane y - 1's newest row (row y - 1 of the plane this lane takes now)
#pragma unroll
            for (int k = 0; k < 8; k++) up[k] = __shfl_up_sync(0xffffffffu, Zp[k], 1);
            const int zz = t - y;
            if (zz >= 0 && zz < nz) {
                const uint4 cw4 = cv;
                const unsigned long long obase = off;
                cv  = load_row(zz + 1);
                off = load_off(zz + 1);
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    Yp[k] = Y[k];
                    Y[k]  = y ? up[k] : 0.f;
                }
                const uint32_t cw[4] = {cw4.x, cw4.y, cw4.z, cw4.w};
                auto code_at = [&](int k) -> uint32_t { return (cw[k >> 1] >> (16 * (k & 1))) & 0xffffu; };
                uint32_t zm = 0;
                if (zero_halves(cw4.x) | zero_halves(cw4.y) | zero_halves(cw4.z) | zero_halves(cw4.w)) {
#pragma unroll
                    for (int k = 0; k < 8; k++) zm |= (code_at(k) == 0u) ? (1u << k) : 0u;
                }
                float C[8];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const float X   = k ? C[k - 1] : 0.f;
                    const float XY  = k ? Y[k - 1] : 0.f;
                    const float XZ  = k ? Zp[k - 1] : 0.f;
                    const float XYZ = k ? Yp[k - 1] : 0.f;
                    const float pred =
                        __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fsub_rn(XYZ, XY), XZ), Yp[k]), X), Y[k]), Zp[k]);
                    float s = __fadd_rn(pred, __fsub_rn(__uint_as_float(0x4B000000u | code_at(k)), rbias));
                    if (zm & (1u << k)) {
                        const unsigned long long oi = obase + __popc(zm & ((1u << k) - 1u));
                        s = 0.f;
                        if (oi < a.n_outliers) s = a.outliers[oi];
                        else set_status(a.status, VSZ_ERR_CORRUPT);
                        if (a.strict) s = strict_prequant<3>(s, x0 + (uint32_t)k, a, c);
                    }
                    C[k] = s;
                }
                float xo[8];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    xo[k] = dequant(C[k], c.c_d, c.c_hi, c.c_lo, c.dq_fast);
                    if (a.strict && (zm & (1u << k))) {  // strict outliers are output as stored
                        const unsigned long long oi = obase + __popc(zm & ((1u << k) - 1u));
                        xo[k] = oi < a.n_outliers ? a.outliers[oi] : 0.f;
                    }
                }
                float* orow = a.out + row_of(zz) * a.d0;
                if (VEC && all_in) {
                    __stcs(reinterpret_cast<float4*>(orow + x0), make_float4(xo[0], xo[1], xo[2], xo[3]));
                    __stcs(reinterpret_cast<float4*>(orow + x0 + 4), make_float4(xo[4], xo[5], xo[6], xo[7]));
                } else if (row_in) {
#pragma unroll
                    for (int k = 0; k < 8; k++)
                        if (x0 + (uint32_t)k < a.d0) orow[x0 + k] = xo[k];
                }
#pragma unroll
                for (int k = 0; k < 8; k++) Zp[k] = C[k];
            }
        }
    }
}

// Zero codes per (row, x-block of 8) in row-major order, for k_dq_decompress_w8's ranks.
__global__ void __launch_bounds__(256) k_count_zeros_b8(const uint16_t* __restrict__ codes, uint32_t d0, uint32_t nbx8,
                                                        size_t m, uint32_t* __restrict__ blk_zero) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row     = i / nbx8;
        const uint32_t x0    = (uint32_t)(i - row * nbx8) * 8u;
        const uint16_t* crow = codes + row * d0;
        uint32_t z = 0;
#pragma unroll
        for (uint32_t k = 0; k < 8; k++) z += (x0 + k < d0 && crow[x0 + k] == 0) ? 1u : 0u;
        blk_zero[i] = z;
    }
}

int launch_count_zeros_b8(const uint16_t* codes, uint32_t d0, size_t nrows, uint32_t* blk_zero, cudaStream_t st,
                          int num_sms) {
    const uint32_t nbx8 = (d0 + 7) / 8;
    const size_t m      = nrows * nbx8;
    if (m == 0) return VSZ_OK;
    long long want = (long long)((m + 255) / 256), cap = (long long)num_sms * 8;
    k_count_zeros_b8<<<(int)(want < cap ? want : cap), 256, 0, st>>>(codes, d0, nbx8, m, blk_zero);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

bool dq_w8_applies(const DqDecArgs& a, int ndim) {
    if (ndim != 3 || a.pad.vals || a.n > kW8MaxN || !(a.blk_off || a.n_outliers == 0)) return false;
    if (getenv("VSZ_DQ_NO_WAVEFRONT") != nullptr) return false;
    // the separable pass catches up with the wavefront between 160^3 and 256^3 (measured: 0.123
    // vs 0.060 ms at 160^3, 0.099 vs 0.127 ms at 256^3, zero scans included)
    return a.n <= kW8MaxSeparableN || !dq_b8_separable(a, ndim);
}

// ------------------------------------------------------------------------------------------
// General block sizes (16, 32, 64; also 8): one thread per block row, skewed pipeline.
// Thread t (row y = t of the block) visits its elements in (z, x) order one step behind thread
// t - 1, so every neighbour it reads was written in an earlier step; planes alternate between
// two shared-memory buffers.  A CTA runs G = 128 / bs blocks side by side.
// 1D: one thread per block, sequential along x.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t zeros_before(const uint16_t* crow, uint32_t from, uint32_t to) {
    uint32_t n = 0;
    for (uint32_t x = from; x < to; x++) n += (crow[x] == 0);
    return n;
}

template <int NDIM, int BS, bool PAD = false>
__global__ void __launch_bounds__(128) k_dq_decompress_gen(DqDecArgs a) {
    constexpr int G = (128 / BS) > 0 ? (128 / BS) : 1;
    extern __shared__ float s_buf[];  // G blocks x 2 planes x BS x BS
    const Consts c = *a.consts;
    if (c.status != VSZ_OK || *a.status != VSZ_OK) return;  // uniform across the grid
    const int R = a.R;
    if (NDIM == 1) {
        size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
        size_t x0 = b * BS;
        if (x0 >= a.d0) return;
        uint32_t seg_x0 = (uint32_t)(x0 & ~(size_t)(kDSeg - 1));
        uint32_t zb = zeros_before(a.codes, seg_x0, (uint32_t)x0);
        const float hx = PAD ? halo_of(a.pad, 1, (uint32_t)(x0 / BS), 0, 0).x : 0.f;
        float prev = 0.f;
        for (int k = 0; k < BS; k++) {
            size_t x = x0 + k;
            if (x >= a.d0) break;
            uint32_t cd = a.codes[x];
            float s, xo;
            if (cd == 0u) {
                if ((x & (kDSeg - 1)) == 0) zb = 0;
                unsigned long long oi = a.seg_off[x / kDSeg] + zb;
                if (oi < a.n_outliers) s = a.outliers[oi];
                else {
                    s = 0.f;
                    set_status(a.status, VSZ_ERR_CORRUPT);
                }
                zb++;
                xo = s;  // strict: the stored input value
                if (a.strict) s = strict_prequant<1>(s, (uint32_t)x, a, c);
                else xo = dequant(s, c.c_d, c.c_hi, c.c_lo, c.dq_fast);
            } else {
                if ((x & (kDSeg - 1)) == 0) zb = 0;
                s  = __fadd_rn(k ? prev : hx, (float)((int)cd - R));
                xo = dequant(s, c.c_d, c.c_hi, c.c_lo, c.dq_fast);
            }
            prev     = s;
            a.out[x] = xo;
        }
        return;
    }
    const int g = threadIdx.x / BS, t = threadIdx.x % BS;
    const unsigned long long blk = (unsigned long long)blockIdx.x * G + g;
    const bool active = blk < a.nunits;
    const uint32_t bx = active ? (uint32_t)(blk % a.nbx) : 0u;
    const unsigned long long rr = active ? blk / a.nbx : 0ull;
    const uint32_t by = (uint32_t)(rr % a.nyb);
    const uint32_t bz = (NDIM == 3) ? (uint32_t)(rr / a.nyb) : 0u;
    const uint32_t x0 = bx * BS, y = by * BS + t, z0 = bz * BS;
    float hx = 0.f, hy = 0.f, hz = 0.f;  // halo of this block (zero without padding)
    if (PAD && active) {
        const Halo hv = halo_of(a.pad, NDIM, bx, by, bz);
        hx = hv.x;
        hy = hv.y;
        hz = hv.z;
    }
    float* S0 = s_buf + (size_t)g * 2 * BS * BS;
    float* S1 = S0 + BS * BS;
    for (int i = t; i < 2 * BS * BS; i += BS) S0[i] = 0.f;
    __syncthreads();
    const int nsteps = (NDIM == 3) ? (BS * BS + BS - 1) : (2 * BS - 1);
    uint32_t zrun = 0;  // zeros seen in the current row segment before the current x
    for (int step = 0; step < nsteps; step++) {
        const int q = step - t;
        const int lim = (NDIM == 3) ? BS * BS : BS;
        if (active && q >= 0 && q < lim) {
            const int zl = (NDIM == 3) ? q / BS : 0, xl = (NDIM == 3) ? q % BS : q;
            const uint32_t z = z0 + zl, x = x0 + xl;
            float* Sc = (zl & 1) ? S1 : S0;  // plane z
            float* Sp = (zl & 1) ? S0 : S1;  // plane z - 1
            const bool in = (x < a.d0) && (y < a.d1) && (NDIM < 3 || z < a.d2);
            float s = 0.f;
            if (in) {
                const size_t row     = (size_t)z * a.d1 + y;
                const uint16_t* crow = a.codes + row * a.d0;
                if (xl == 0) zrun = zeros_before(crow, x0 & ~(uint32_t)(kDSeg - 1), x0);
                else if ((x & (kDSeg - 1)) == 0) zrun = 0;
                uint32_t cd = crow[x];
                float pred;
                // halo cells: 2D (x-1, y-1) is the x-halo's, 3D the y-halo's; z - 1 = halo: hz
                const float X  = xl ? Sc[t * BS + xl - 1] : hx;
                const float Y  = t ? Sc[(t - 1) * BS + xl] : hy;
                const float XY = (t && xl) ? Sc[(t - 1) * BS + xl - 1]
                                           : (NDIM == 2 ? (xl ? hy : hx) : (t ? hx : hy));
                if (NDIM == 2) {
                    pred = __fsub_rn(__fadd_rn(Y, X), XY);
                } else {
                    const bool zp   = zl > 0;
                    const float XYZ = (zp && t && xl) ? Sp[(t - 1) * BS + xl - 1] : (zp ? (t ? hx : hy) : hz);
                    const float XZ  = (zp && xl) ? Sp[t * BS + xl - 1] : (zp ? hx : hz);
                    const float YZ  = (zp && t) ? Sp[(t - 1) * BS + xl] : (zp ? hy : hz);
                    const float Z   = zp ? Sp[t * BS + xl] : hz;
                    pred = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fsub_rn(XYZ, XY), XZ), YZ), X), Y), Z);
                }
                float xo;
                if (cd == 0u) {
                    unsigned long long oi = a.seg_off[row * a.nxs + (x / kDSeg)] + zrun;
                    if (oi < a.n_outliers) s = a.outliers[oi];
                    else set_status(a.status, VSZ_ERR_CORRUPT);
                    zrun++;
                    xo = s;  // strict: the stored input value
                    if (a.strict) s = strict_prequant<NDIM>(s, x, a, c);
                    else xo = dequant(s, c.c_d, c.c_hi, c.c_lo, c.dq_fast);
                } else {
                    s  = __fadd_rn(pred, (float)((int)cd - R));
                    xo = dequant(s, c.c_d, c.c_hi, c.c_lo, c.dq_fast);
                }
                a.out[row * a.d0 + x] = xo;
            }
            Sc[t * BS + xl] = s;
        }
        __syncthreads();
    }
}

// Zero codes per 256-wide row segment, for callers that hold codes but no decoder counts.
__global__ void __launch_bounds__(256) k_count_zeros(const uint16_t* __restrict__ codes, uint32_t d0, size_t nrows,
                                                     uint32_t nxs, uint32_t* __restrict__ seg_zero) {
    const unsigned lane = lane_id();
    const size_t nseg   = nrows * nxs;
    const size_t wtot   = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t sgi = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5); sgi < nseg; sgi += wtot) {
        size_t row = sgi / nxs;
        uint32_t xs = (uint32_t)(sgi - row * nxs);
        const uint16_t* crow = codes + row * d0;
        uint32_t z = 0;
        for (uint32_t x = xs * kDSeg + lane; x < min(d0, (xs + 1) * kDSeg); x += 32) z += (crow[x] == 0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
        if (lane == 0) seg_zero[sgi] = z;
    }
}

int launch_count_zeros(const uint16_t* codes, uint32_t d0, size_t nrows, uint32_t* seg_zero, cudaStream_t st,
                       int num_sms) {
    uint32_t nxs = (d0 + kDSeg - 1) / kDSeg;
    size_t nseg  = nrows * nxs;
    if (nseg == 0) return VSZ_OK;
    long long want = (long long)((nseg + 7) / 8), cap = (long long)num_sms * 16;
    int grid = (int)(want < cap ? want : cap);
    k_count_zeros<<<grid, 256, 0, st>>>(codes, d0, nrows, nxs, seg_zero);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

template <int NDIM, int BS, bool PAD>
static int launch_gen(const DqDecArgs& a, cudaStream_t st) {
    constexpr int G = (128 / BS) > 0 ? (128 / BS) : 1;
    if (NDIM == 1) {
        size_t nblk = (a.d0 + BS - 1) / BS;
        k_dq_decompress_gen<1, BS, PAD><<<(unsigned)((nblk + 127) / 128), 128, 0, st>>>(a);
        count_launch();
    } else {
        size_t smem = (size_t)G * 2 * BS * BS * sizeof(float);
        static std::atomic<unsigned long long> attr{0};
        smem_limit_once(k_dq_decompress_gen<NDIM, BS, PAD>, (int)smem, attr);
        unsigned grid = (unsigned)((a.nunits + G - 1) / G);
        k_dq_decompress_gen<NDIM, BS, PAD><<<grid, G * BS, smem, st>>>(a);
        count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

void dq_b8_geometry(DqDecArgs& a, int ndim) {
    a.nxs   = (a.d0 + kDSeg - 1) / kDSeg;
    a.nyb   = (a.d1 + 7) / 8;
    a.nbx8  = (a.d0 + 7) / 8;
    a.ygrp  = 1;
    a.nyb_g = a.nyb;
    unsigned long long nzb = (ndim == 3) ? (a.d2 + 7) / 8 : 1;
    a.nunits = (unsigned long long)a.nxs * (ndim >= 2 ? a.nyb : 1) * nzb;
}

void dq_b8_narrow(DqDecArgs& a, int ndim) {
    if (ndim < 2 || a.nbx8 == 0 || a.nbx8 > 16) return;
    a.ygrp  = 32 / a.nbx8;
    a.nyb_g = (a.nyb + a.ygrp - 1) / a.ygrp;
    const unsigned long long nzb = (ndim == 3) ? (a.d2 + 7) / 8 : 1;
    a.nunits = (unsigned long long)a.nyb_g * nzb;
}

bool dq_b8_vec(const DqDecArgs& a) {
    return (a.d0 % 8 == 0) && ((reinterpret_cast<uintptr_t>(a.codes) & 15u) == 0) &&
           ((reinterpret_cast<uintptr_t>(a.out) & 15u) == 0);
}

bool dq_b8_separable(const DqDecArgs& a, int ndim) {
    return ndim == 3 && dq_b8_vec(a) && a.redo && !a.strict && !a.pad.vals && a.n_outliers * 64 < a.n;
}

// ---- many fields (block size 8, no padding): tasks of (field, unit range), taken one at a time
// by whichever warp is free (`next`: the class's task counter, zero at launch), so that warps do
// not idle behind uneven tasks.  Per field the result is k_dq_decompress_b8 / _b8s's.
__device__ __forceinline__ uint32_t dq_next_task(uint32_t* next) {
    uint32_t t = 0;
    if (lane_id() == 0) t = atomicAdd(next, 1u);
    return __shfl_sync(0xffffffffu, t, 0);
}

template <int NDIM, bool VEC>
__global__ void __launch_bounds__(128, 6)
    k_dq_decompress_b8_batch(const DqDecArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks,
                             uint32_t* __restrict__ next) {
    extern __shared__ __align__(16) uint8_t s_dq_dyn[];
    const unsigned wib = threadIdx.x >> 5;
    for (uint32_t t = dq_next_task(next); t < ntasks; t = dq_next_task(next)) {
        const BatchTask tk = tasks[t];  // the field's arguments are read in place (a copy spills)
        dq_b8_units<NDIM, VEC, false, false>(args[tk.field], (uint32_t)tk.u0, (uint32_t)tk.u1, 1u,
                                             reinterpret_cast<DqPlane*>(s_dq_dyn), wib);
    }
}

__global__ void __launch_bounds__(128, 6)
    k_dq_decompress_b8s_batch(const DqDecArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks,
                              uint32_t* __restrict__ next) {
    extern __shared__ __align__(16) uint8_t s_dq_dyn[];
    const unsigned wib = threadIdx.x >> 5;
    for (uint32_t t = dq_next_task(next); t < ntasks; t = dq_next_task(next)) {
        const BatchTask tk = tasks[t];
        dq_b8s_units<true>(args[tk.field], (uint32_t)tk.u0, (uint32_t)tk.u1, 1u, reinterpret_cast<DqPlane*>(s_dq_dyn), wib);
    }
}

// The units the separable pass listed, one CTA per field (tasks carry only the field).
__global__ void __launch_bounds__(128, 6)
    k_dq_decompress_redo_batch(const DqDecArgs* __restrict__ args, const BatchTask* __restrict__ tasks, uint32_t ntasks) {
    extern __shared__ __align__(16) uint8_t s_dq_dyn[];
    const unsigned wib = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const DqDecArgs& a = args[tasks[t].field];  // read in place: fewer registers than a copy
        dq_b8_units<3, true, false, true>(a, wib, a.redo[0], 4u, reinterpret_cast<DqPlane*>(s_dq_dyn), wib);
    }
}

int launch_dq_decompress_batch(const DqDecArgs* args, const BatchTask* tasks, uint32_t ntasks, int ndim, bool vec,
                               bool sep, uint32_t* next, cudaStream_t st, int num_sms) {
    if (ntasks == 0) return VSZ_OK;
    const uint32_t cap  = (uint32_t)num_sms * 6;  // resident CTAs of 4 warps
    const uint32_t want = (ntasks + 3) / 4;
    const uint32_t grid = want < cap ? want : cap;
    const size_t smem   = (ndim == 3) ? 4 * sizeof(DqPlane) : 0;
    static std::atomic<unsigned long long> attr[8];
    auto go = [&](auto kern, int slot) {
        if (smem > 48 * 1024) smem_limit_once(kern, (int)smem, attr[slot]);
        kern<<<grid, 128, smem, st>>>(args, tasks, ntasks, next);
        count_launch();
    };
    if (sep) go(k_dq_decompress_b8s_batch, 0);
    else if (ndim == 3) vec ? go(k_dq_decompress_b8_batch<3, true>, 1) : go(k_dq_decompress_b8_batch<3, false>, 2);
    else if (ndim == 2) vec ? go(k_dq_decompress_b8_batch<2, true>, 3) : go(k_dq_decompress_b8_batch<2, false>, 4);
    else vec ? go(k_dq_decompress_b8_batch<1, true>, 5) : go(k_dq_decompress_b8_batch<1, false>, 6);
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_dq_redo_batch(const DqDecArgs* args, const BatchTask* tasks, uint32_t ntasks, cudaStream_t st,
                         int num_sms) {
    if (ntasks == 0) return VSZ_OK;
    const uint32_t cap  = (uint32_t)num_sms * 6;
    const uint32_t grid = ntasks < cap ? ntasks : cap;
    static std::atomic<unsigned long long> attr{0};
    smem_limit_once(k_dq_decompress_redo_batch, (int)(4 * sizeof(DqPlane)), attr);
    k_dq_decompress_redo_batch<<<grid, 128, 4 * sizeof(DqPlane), st>>>(args, tasks, ntasks);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

// Fields from this size on check the two-operation dequantization before the separable pass.
constexpr size_t kDqVerifyMin = (size_t)1 << 22;

int launch_dq_decompress(DqDecArgs a, int ndim, int bs, bool force_general, cudaStream_t st, int num_sms) {
    if (a.n == 0) return VSZ_OK;
    if (bs == 8 && !force_general) {
        dq_b8_geometry(a, ndim);
        const bool vec = dq_b8_vec(a);
        if (dq_w8_applies(a, ndim)) {  // small 3D field: the wavefront pass
            a.nunits = (unsigned long long)((a.nbx8 + 3) / 4) * a.nyb * ((a.d2 + 7) / 8);
            const long long want = (long long)((a.nunits + 3) / 4), cap = (long long)num_sms * 16;
            const int grid = (int)(want < cap ? want : cap);
            if (vec) k_dq_decompress_w8<true><<<grid, 128, 0, st>>>(a);
            else k_dq_decompress_w8<false><<<grid, 128, 0, st>>>(a);
            count_launch();
            return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
        }
        if (!a.pad.vals && !dq_b8_separable(a, ndim)) dq_b8_narrow(a, ndim);  // the reference-order kernel
        long long want = (long long)((a.nunits + 3) / 4);
        long long cap  = (long long)num_sms * 16;
        int grid = (int)(want < cap ? want : cap);
        if (grid < 1) grid = 1;
        static std::atomic<unsigned long long> attr[12];
        const bool pad = a.pad.vals != nullptr;
        auto go = [&](auto kern, int nd) {
            const size_t smem = (nd == 3) ? 4 * 8 * 8 * 32 * 4 : 0;  // previous plane per warp
            if (smem > 48 * 1024)
                smem_limit_once(kern, (int)smem, attr[(nd - 1) * 4 + (vec ? 1 : 0) + (pad ? 2 : 0)]);
            kern<<<grid, 128, smem, st>>>(a);
            count_launch();
        };
        if (pad) {
            if (ndim == 3) vec ? go(k_dq_decompress_b8<3, true, true>, 3) : go(k_dq_decompress_b8<3, false, true>, 3);
            else if (ndim == 2) vec ? go(k_dq_decompress_b8<2, true, true>, 2) : go(k_dq_decompress_b8<2, false, true>, 2);
            else vec ? go(k_dq_decompress_b8<1, true, true>, 1) : go(k_dq_decompress_b8<1, false, true>, 1);
        } else if (dq_b8_separable(a, ndim)) {
            // separable pass, then the reference-order kernel over the units it listed.  A large
            // field first checks the cheaper dequantization (a few microseconds, all SMs).
            const bool verify = a.consts_rw && a.n >= kDqVerifyMin;
            if (cudaMemsetAsync(a.redo, 0, (verify ? 3 : 1) * sizeof(uint32_t), st) != cudaSuccess)
                return VSZ_ERR_CUDA;
            if (verify) {
                k_dq_mul_verify<<<(unsigned)num_sms * 4, 256, 0, st>>>(a.consts_rw, a.redo, a.dq_cache);
                count_launch();
            }
            // fields of one segment per row carry outlier ranks; wider ones keep the lighter kernel
            a.nxs == 1 ? go(k_dq_decompress_b8s<true>, 3) : go(k_dq_decompress_b8s<false>, 3);
            go(k_dq_decompress_b8<3, true, false, true>, 3);
        } else {
            if (ndim == 3) vec ? go(k_dq_decompress_b8<3, true>, 3) : go(k_dq_decompress_b8<3, false>, 3);
            else if (ndim == 2) vec ? go(k_dq_decompress_b8<2, true>, 2) : go(k_dq_decompress_b8<2, false>, 2);
            else vec ? go(k_dq_decompress_b8<1, true>, 1) : go(k_dq_decompress_b8<1, false>, 1);
        }
        return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
    }
    a.nxs = (a.d0 + kDSeg - 1) / kDSeg;
    a.nbx = (a.d0 + bs - 1) / bs;
    a.nyb = (a.d1 + bs - 1) / bs;
    unsigned long long nzb = (ndim == 3) ? (a.d2 + bs - 1) / bs : 1;
    a.nunits = (unsigned long long)a.nbx * a.nyb * nzb;
    auto go = [&](auto bs_c) -> int {
        constexpr int B = decltype(bs_c)::value;
        if (a.pad.vals) {
            if (ndim == 3) return launch_gen<3, B, true>(a, st);
            if (ndim == 2) return launch_gen<2, B, true>(a, st);
            return launch_gen<1, B, true>(a, st);
        }
        if (ndim == 3) return launch_gen<3, B, false>(a, st);
        if (ndim == 2) return launch_gen<2, B, false>(a, st);
        return launch_gen<1, B, false>(a, st);
    };
    switch (bs) {
        case 8: return go(std::integral_constant<int, 8>{});
        case 16: return go(std::integral_constant<int, 16>{});
        case 32: return go(std::integral_constant<int, 32>{});
        case 64: return go(std::integral_constant<int, 64>{});
        default: return VSZ_ERR_UNSUPPORTED;
    }
}

}  // namespace vsz
