// Dual quantization of f64 fields (the reference's -t f64, src/argument_parser/argparse.cc:454-462).
//
// The reference parses -t f64 but always reads its input as float (src/vecsz.cc:32), and its
// dual-quant loops use float AVX intrinsics (src/dualquant.hh:86-92), so it has no f64 arithmetic to
// match.  This is the same algorithm in double precision, with the error bound guaranteed in the
// manner of the strict mode:
//   s    = rint(x / (2 eb))             prequantized value, in double, kept as an exact integer
//                                       (0 for non-finite x or |x / (2 eb)| >= 2^59)
//   pred = the Lorenzo predictor of the block's s values (zero halo per block), in 64-bit integer
//          arithmetic: exact whatever the order
//   code = e + R for e = s - pred when |e| < R, x is finite, |x / (2 eb)| < 2^59 and the
//          decompressor's value s * 2eb lies within eb of x (checked in double); otherwise 0 and
//          the element is an outlier carrying x itself (8 bytes)
// The decompressor rebuilds s exactly (integers) and outputs s * 2eb, or the stored x for an
// outlier, whose s it derives from x by the same rule -- both sides' predictor chains are the same
// integers, so every output is within eb of its input (outliers exactly equal).
#include <cstdint>
#include <type_traits>

#include "vsz_device.cuh"
#include "vsz_kernels.h"

namespace vsz {

constexpr double kF64SMax = 576460752303423488.0;  // 2^59: |s| below it keeps every predictor in int64

__device__ __forceinline__ bool f64_quantizable(double x, double r_d) {
    const double v = x * r_d;
    return isfinite(v) && fabs(v) < kF64SMax;
}

__device__ __forceinline__ long long prequant_f64(double x, double r_d) {
    return f64_quantizable(x, r_d) ? __double2ll_rn(x * r_d) : 0ll;
}

// Order-preserving map of doubles onto u64 (NaNs are skipped by the caller).
__device__ __forceinline__ unsigned long long d2key(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key2d(unsigned long long k) {
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// ---- value range (r2r) and constants --------------------------------------------------------
__global__ void __launch_bounds__(256) k_minmax_f64(const double* __restrict__ x, size_t n,
                                                    unsigned long long* __restrict__ mm) {
    unsigned long long mx = 0ull, mn = ~0ull;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        if (v != v) continue;
        const unsigned long long k = d2key(v);
        mx = k > mx ? k : mx;
        mn = k < mn ? k : mn;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, mx, o), b = __shfl_xor_sync(0xffffffffu, mn, o);
        mx = a > mx ? a : mx;
        mn = b < mn ? b : mn;
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicMax(&mm[0], mx);
        atomicMin(&mm[1], mn);
    }
}

// eb_final = eb (abs) or eb * (max - min) (r2r, in double); r_d = 1 / (2 eb_final), c_d = 2 eb_final.
__global__ void k_consts_f64(int mode, double eb, const unsigned long long* __restrict__ mm, Consts* __restrict__ c,
                             int* status_word) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double ebf = eb, range = 0.0;
    int status = VSZ_OK;
    if (mode == VSZ_MODE_R2R) {
        if (mm[1] == ~0ull) {  // every value is a NaN
            status = VSZ_ERR_RANGE;
        } else {
            range = key2d(mm[0]) - key2d(mm[1]);
            if (!(range > 0.0) || !isfinite(range)) status = VSZ_ERR_RANGE;
        }
        ebf = eb * range;
    }
    c->eb_final = ebf;
    c->c_d      = 2.0 * ebf;
    c->r_d      = 1.0 / c->c_d;
    c->range    = range;
    c->r_f      = 0.f;
    c->c_hi     = 0.f;
    c->c_lo     = 0.f;
    c->dq_fast  = 0;
    c->dq_mul   = 0;
    c->dq_exc   = 0.f;
    c->dq_exc_y = 0.f;
    if (status == VSZ_OK && !(c->r_d > 0.0 && isfinite(c->r_d) && isfinite(c->c_d))) status = VSZ_ERR_INVALID;
    c->status = status;
    if (status != VSZ_OK && status_word) set_status(status_word, status);
}

// ---- compress ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_prequant_f64(const double* __restrict__ x, size_t n, const Consts* __restrict__ c,
                                                      long long* __restrict__ s) {
    if (c->status != VSZ_OK) return;
    const double r_d = c->r_d;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        s[i] = prequant_f64(x[i], r_d);
}

// Codes and histogram: one thread per element, its block's neighbours' prequantized values read
// from s (zero across the block's lower faces).
template <int NDIM>
__global__ void __launch_bounds__(256) k_lorenzo_f64(F64Args a) {
    extern __shared__ uint32_t s_hist_f64[];
    const Consts c = *a.consts;
    if (c.status != VSZ_OK) return;  // uniform
    const bool smem = a.dict <= 16384;
    if (smem) {
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x) s_hist_f64[i] = 0u;
        __syncthreads();
    }
    const long long R = a.dict / 2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / a.d0;
        const uint32_t x = (uint32_t)(i - row * a.d0);
        const uint32_t y = (uint32_t)(row % a.d1);
        const uint32_t z = (uint32_t)(row / a.d1);
        const bool bx = (x % a.bs) != 0, by = NDIM >= 2 && (y % a.bs) != 0, bz = NDIM == 3 && (z % a.bs) != 0;
        const size_t sy = a.d0, sz = (size_t)a.d0 * a.d1;
        auto S = [&](bool ok, size_t j) -> long long { return ok ? a.s[j] : 0ll; };
        long long pred;
        if (NDIM == 1) {
            pred = S(bx, i - 1);
        } else if (NDIM == 2) {
            pred = S(bx, i - 1) + S(by, i - sy) - S(bx && by, i - 1 - sy);
        } else {
            pred = S(bx, i - 1) + S(by, i - sy) + S(bz, i - sz) - S(bx && by, i - 1 - sy) - S(bx && bz, i - 1 - sz) -
                   S(by && bz, i - sy - sz) + S(bx && by && bz, i - 1 - sy - sz);
        }
        const double xv   = a.x[i];
        const long long s = a.s[i];
        const long long e = s - pred;
        uint32_t code     = 0;
        if (e > -R && e < R && f64_quantizable(xv, c.r_d) && fabs(xv - (double)s * c.c_d) <= c.eb_final)
            code = (uint32_t)(e + R);
        a.code[i] = (uint16_t)code;
        if (smem) atomicAdd(&s_hist_f64[code], 1u);
        else atomicAdd(&a.hist[code], 1ull);
    }
    if (smem) {
        __syncthreads();
        for (int i = threadIdx.x; i < a.dict; i += blockDim.x)
            if (s_hist_f64[i]) atomicAdd(&a.hist[i], (unsigned long long)s_hist_f64[i]);
    }
}

// Outliers in row-major order of code 0: one warp per 256-wide row segment (seg_off: exclusive
// scan of the zero codes per segment), 8 bytes each at out + 8 rank (any alignment).
__global__ void __launch_bounds__(256) k_gather_f64(F64Args a, const unsigned long long* __restrict__ seg_off,
                                                    DevOffset out_off) {
    if (*a.status != VSZ_OK || a.consts->status != VSZ_OK) return;
    uint8_t* out        = a.archive + out_off.eval();
    const unsigned lane = threadIdx.x & 31u;
    const size_t nxs    = (a.d0 + 255) / 256;
    const size_t nseg   = (a.n / a.d0) * nxs;
    for (size_t sg = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5; sg < nseg;
         sg += ((size_t)gridDim.x * blockDim.x) >> 5) {
        const size_t row = sg / nxs;
        const uint32_t x0 = (uint32_t)(sg - row * nxs) * 256;
        unsigned long long rank = seg_off[sg];
        for (uint32_t k = 0; k < 256; k += 32) {
            const uint32_t x = x0 + k + lane;
            const bool o     = x < a.d0 && a.code[row * a.d0 + x] == 0;
            const unsigned m = __ballot_sync(0xffffffffu, o);
            if (o) {
                const unsigned long long r = rank + __popc(m & ((1u << lane) - 1u));
                const double v             = a.x[row * a.d0 + x];
                const unsigned long long b = (unsigned long long)__double_as_longlong(v);
                uint8_t* d                 = out + 8 * r;
#pragma unroll
                for (int q = 0; q < 8; q++) d[q] = (uint8_t)(b >> (8 * q));
            }
            rank += __popc(m);
        }
    }
}

// ---- decompress -------------------------------------------------------------------------------
__device__ __forceinline__ double ld_f64_bytes(const uint8_t* p) {
    unsigned long long b = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) b |= (unsigned long long)p[q] << (8 * q);
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ uint32_t zeros_between(const uint16_t* crow, uint32_t from, uint32_t to) {
    uint32_t n = 0;
    for (uint32_t x = from; x < to; x++) n += (crow[x] == 0);
    return n;
}

// One element: its s from the code (or from the stored outlier) and its output.
__device__ __forceinline__ long long xl_element(const F64Args& a, const Consts& c, uint32_t cd, long long pred,
                                                unsigned long long oi, double* out) {
    if (cd == 0u) {
        double v = 0.0;
        if (oi < a.n_out) v = ld_f64_bytes(a.outliers + 8 * oi);
        else set_status(a.status, VSZ_ERR_CORRUPT);
        *out = v;
        return prequant_f64(v, c.r_d);
    }
    const long long s = pred + ((long long)cd - (long long)(a.dict / 2));
    *out              = (double)s * c.c_d;
    return s;
}

// 1D: one thread per block, in order.
__global__ void __launch_bounds__(128) k_xlorenzo_f64_1d(F64Args a, const unsigned long long* __restrict__ seg_off) {
    const Consts c = *a.consts;
    if (c.status != VSZ_OK || *a.status != VSZ_OK) return;
    const size_t b  = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t x0 = b * a.bs;
    if (x0 >= a.d0) return;
    uint32_t zrun = zeros_between(a.code, (uint32_t)(x0 & ~(size_t)255), (uint32_t)x0);
    long long prev = 0;
    for (uint32_t k = 0; k < (uint32_t)a.bs && x0 + k < a.d0; k++) {
        const size_t x = x0 + k;
        if ((x & 255u) == 0) zrun = 0;
        const uint32_t cd = a.code[x];
        double v;
        prev = xl_element(a, c, cd, prev, seg_off[x / 256] + zrun, &v);
        zrun += (cd == 0u);
        a.out[x] = v;
    }
}

// 2D / 3D: thread t of a block is its row t; it visits its elements in (z, x) order one step behind
// thread t - 1, so every neighbour it reads was written in an earlier step (planes z and z - 1
// alternate between two shared-memory buffers of BS x BS values per block).
template <int NDIM, int BS>
__global__ void __launch_bounds__(128) k_xlorenzo_f64(F64Args a, const unsigned long long* __restrict__ seg_off) {
    constexpr int G = 128 / BS;
    extern __shared__ long long s_pl[];  // G blocks x 2 planes x BS x BS
    const Consts c = *a.consts;
    if (c.status != VSZ_OK || *a.status != VSZ_OK) return;  // uniform
    const int g = threadIdx.x / BS, t = threadIdx.x % BS;
    const uint32_t nbx = (a.d0 + BS - 1) / BS, nby = (a.d1 + BS - 1) / BS;
    const unsigned long long nzb = NDIM == 3 ? (a.d2 + BS - 1) / BS : 1;
    const unsigned long long blk = (unsigned long long)blockIdx.x * G + g;
    const bool active            = blk < (unsigned long long)nbx * nby * nzb;
    const uint32_t bx            = active ? (uint32_t)(blk % nbx) : 0u;
    const unsigned long long rr  = active ? blk / nbx : 0ull;
    const uint32_t by = (uint32_t)(rr % nby), bz = NDIM == 3 ? (uint32_t)(rr / nby) : 0u;
    const uint32_t x0 = bx * BS, y = by * BS + t, z0 = bz * BS;
    const size_t nxs  = (a.d0 + 255) / 256;
    long long* P0 = s_pl + (size_t)g * 2 * BS * BS;
    long long* P1 = P0 + BS * BS;
    for (int i = t; i < 2 * BS * BS; i += BS) P0[i] = 0;
    __syncthreads();
    const int nsteps = NDIM == 3 ? BS * BS + BS - 1 : 2 * BS - 1;
    uint32_t zrun = 0;  // zeros before the current x in its row segment
    for (int step = 0; step < nsteps; step++) {
        const int q   = step - t;
        const int lim = NDIM == 3 ? BS * BS : BS;
        if (active && q >= 0 && q < lim) {
            const int zl = NDIM == 3 ? q / BS : 0, xl = NDIM == 3 ? q % BS : q;
            const uint32_t z = z0 + zl, x = x0 + xl;
            long long* Sc = (zl & 1) ? P1 : P0;  // plane z
            long long* Sp = (zl & 1) ? P0 : P1;  // plane z - 1
            const bool in = x < a.d0 && y < a.d1 && (NDIM < 3 || z < a.d2);
            long long s   = 0;
            if (in) {
                const size_t row     = (size_t)z * a.d1 + y;
                const uint16_t* crow = a.code + row * a.d0;
                if (xl == 0) zrun = zeros_between(crow, x0 & ~255u, x0);
                else if ((x & 255u) == 0) zrun = 0;
                const long long X  = xl ? Sc[t * BS + xl - 1] : 0;
                const long long Y  = t ? Sc[(t - 1) * BS + xl] : 0;
                const long long XY = (t && xl) ? Sc[(t - 1) * BS + xl - 1] : 0;
                long long pred     = X + Y - XY;
                if (NDIM == 3 && zl > 0)
                    pred += Sp[t * BS + xl] - (xl ? Sp[t * BS + xl - 1] : 0) - (t ? Sp[(t - 1) * BS + xl] : 0) +
                            ((t && xl) ? Sp[(t - 1) * BS + xl - 1] : 0);
                const uint32_t cd = crow[x];
                double v;
                s = xl_element(a, c, cd, pred, seg_off[row * nxs + x / 256] + zrun, &v);
                zrun += (cd == 0u);
                a.out[row * a.d0 + x] = v;
            }
            Sc[t * BS + xl] = s;
        }
        __syncthreads();
    }
}

// ---- launchers ----------------------------------------------------------------------------------
int launch_eb_setup_f64(int mode, double eb, const double* d_in, size_t n, Consts* c, unsigned long long* mm,
                        int* status, cudaStream_t st, int num_sms) {
    if (mode == VSZ_MODE_R2R) {
        if (cudaMemsetAsync(mm, 0, 8, st) != cudaSuccess || cudaMemsetAsync(mm + 1, 0xff, 8, st) != cudaSuccess)
            return VSZ_ERR_CUDA;
        const size_t nb = (n + 2047) / 2048;
        const int grid  = (int)(nb < (size_t)num_sms * 8 ? (nb ? nb : 1) : (size_t)num_sms * 8);
        k_minmax_f64<<<grid, 256, 0, st>>>(d_in, n, mm);
        count_launch();
    }
    k_consts_f64<<<1, 32, 0, st>>>(mode, eb, mm, c, status);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_dq_compress_f64(F64Args a, int ndim, cudaStream_t st, int num_sms) {
    if (a.n == 0) return VSZ_OK;
    const size_t want = (a.n + 255) / 256;
    const int grid    = (int)(want < (size_t)num_sms * 16 ? want : (size_t)num_sms * 16);
    k_prequant_f64<<<grid, 256, 0, st>>>(a.x, a.n, a.consts, a.s);
    count_launch();
    const size_t smem = a.dict <= 16384 ? 4 * (size_t)a.dict : 0;
    static std::atomic<unsigned long long> attr[3];
    auto go = [&](auto kern, int slot) {
        if (smem > 48 * 1024) smem_limit_once(kern, (int)smem, attr[slot]);
        kern<<<grid, 256, smem, st>>>(a);
        count_launch();
    };
    if (ndim == 1) go(k_lorenzo_f64<1>, 0);
    else if (ndim == 2) go(k_lorenzo_f64<2>, 1);
    else go(k_lorenzo_f64<3>, 2);
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_gather_f64(F64Args a, const unsigned long long* seg_off, DevOffset out_off, cudaStream_t st, int num_sms) {
    if (a.n == 0) return VSZ_OK;
    const size_t nseg = (a.n / a.d0) * ((a.d0 + 255) / 256);
    const size_t want = (nseg + 7) / 8;
    const int grid    = (int)(want < (size_t)num_sms * 8 ? want : (size_t)num_sms * 8);
    k_gather_f64<<<grid, 256, 0, st>>>(a, seg_off, out_off);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

int launch_dq_decompress_f64(F64Args a, int ndim, const unsigned long long* seg_off, cudaStream_t st) {
    if (a.n == 0) return VSZ_OK;
    if (ndim == 1) {
        const size_t nb = (a.d0 + a.bs - 1) / a.bs;
        k_xlorenzo_f64_1d<<<(unsigned)((nb + 127) / 128), 128, 0, st>>>(a, seg_off);
        count_launch();
        return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
    }
    auto go = [&](auto nd_c, auto bs_c) -> int {
        constexpr int ND = decltype(nd_c)::value, B = decltype(bs_c)::value;
        constexpr int G  = 128 / B;
        const unsigned long long nb = (unsigned long long)((a.d0 + B - 1) / B) * ((a.d1 + B - 1) / B) *
                                      (ND == 3 ? (a.d2 + B - 1) / B : 1);
        const size_t smem = (size_t)G * 2 * B * B * sizeof(long long);
        static std::atomic<unsigned long long> attr{0};
        if (smem > 48 * 1024) smem_limit_once(k_xlorenzo_f64<ND, B>, (int)smem, attr);
        k_xlorenzo_f64<ND, B><<<(unsigned)((nb + G - 1) / G), 128, smem, st>>>(a, seg_off);
        count_launch();
        return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
    };
    auto by_bs = [&](auto nd_c) -> int {
        switch (a.bs) {
            case 8: return go(nd_c, std::integral_constant<int, 8>{});
            case 16: return go(nd_c, std::integral_constant<int, 16>{});
            case 32: return go(nd_c, std::integral_constant<int, 32>{});
            case 64: return go(nd_c, std::integral_constant<int, 64>{});
            default: return VSZ_ERR_UNSUPPORTED;
        }
    };
    return ndim == 2 ? by_bs(std::integral_constant<int, 2>{}) : by_bs(std::integral_constant<int, 3>{});
}

}  // namespace vsz
