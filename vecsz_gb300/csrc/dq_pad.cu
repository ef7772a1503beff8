// Padding (-p) on sm_103a: the values that replace the zero halo of every Lorenzo block.
//
// Replaces, from szcompressor/vecSZ:
//   global pad value (find_pad_value over the field)     src/vecsz_interface.hh:70-80
//   per-block / per-edge values                          src/dualquant.hh:36-46, 224-246, 551-573
//   find_pad_value / find_edge_pad_value / block_pad / edge_pad   src/utils/padding.hh:122-301
//
// Rules, each what the single-threaded reference computes:
//   blocks       get_nblk = (d + bs + 1) / bs per axis (phantom blocks past the field included),
//                values stored block by block, x fastest; edge mode stores ndim values per block
//                (1D: one).
//   max / min    m = v[0]; m = v[i] > m ? v[i] : m  (first extreme wins; a leading NaN sticks)
//   avg          float running sum in visiting order, divided by (float)count
//   constant     the given value
//   1D block / edge: the raw value (not prequantized, src/dualquant.hh:40)
//   2D / 3D block / edge: roundf((float)((double)v * r_d)) (padding.hh:218-220, 260-263)
//   global       archive value (float)round((double)p * r_d) (interface:79); the compressor's 2D/3D
//                blocks predict from roundf((float)((double)p * r_d)) instead (block_pad runs on
//                the global value as a constant), 1D from the archive value
//   edge faces   2D [row y=0, column x=0]; 3D [face z=0 (x, y), face x=0 (y, z), face y=0 (x, z)],
//                first-listed axis fastest (padding.hh:161-199)
//   cells outside the field count as 0.0f
//
// Kernels: per-block values, one thread per block (the reductions are short serial chains over a
// block, as in the reference); global max / min, a grid-wide keyed reduction plus, for a zero
// extreme, the first index holding it (the sign of the first zero); global avg, one CTA whose
// warps stage the field through shared memory while one thread runs the serial float sum -- the
// reference's running sum has no reassociation-free parallel form, so this pass is bound by the
// FP32 add latency (about 4 cycles per element).
#include <cstdint>

#include "vsz_device.cuh"
#include "vsz_kernels.h"

namespace vsz {

namespace {

struct PadWs {
    uint32_t key[2];            // ordered keys: [0] max, [1] min (NaNs skipped)
    unsigned long long first;   // first index holding a zero extreme
    float sum;                  // global avg: the running sum
    float pad0;
};

struct PadReduce {
    int type;
    float cst;
    float m;
    float s;
    bool any;
    __device__ __forceinline__ void add(float v) {
        if (type == VSZ_PADV_AVG) {
            // x86 NaN propagation: a NaN sum stays, a NaN term enters quieted
            if (s == s) s = (v == v) ? __fadd_rn(s, v) : quiet_nan(v);
        } else if (!any) {
            m   = v;
            any = true;
        } else if (type == VSZ_PADV_MAX) {
            m = (v > m) ? v : m;
        } else {
            m = (v < m) ? v : m;
        }
    }
    __device__ __forceinline__ float result(unsigned long long count) const {
        if (type == VSZ_PADV_CONST) return cst;
        if (type == VSZ_PADV_AVG) return (s == s) ? __fdiv_rn(s, __ull2float_rn(count)) : s;
        return m;
    }
};

__device__ __forceinline__ float prequant_pad(float v, double r_d) {
    if (v != v) return quiet_nan(v);
    return roundf(__double2float_rn(__dmul_rn((double)v, r_d)));  // v *= r_d (float); round(v)
}

__device__ __forceinline__ float field_at(const PadArgs& a, uint32_t i, uint32_t j, uint32_t k) {
    return (i < a.d0 && j < a.d1 && k < a.d2) ? a.x[(size_t)i + (size_t)a.d0 * ((size_t)j + (size_t)a.d1 * k)] : 0.0f;
}

// One thread per block of the reference grid.
__global__ void __launch_bounds__(128) k_pad_blocks(PadArgs a) {
    const Consts* c = a.consts;
    if (c->status != VSZ_OK) return;
    const unsigned long long nblk = (unsigned long long)a.nb0 * a.nb1 * a.nb2;
    const unsigned long long b    = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const uint32_t b0 = (uint32_t)(b % a.nb0);
    const unsigned long long r = b / a.nb0;
    const uint32_t b1 = (uint32_t)(r % a.nb1), b2 = (uint32_t)(r / a.nb1);
    const uint32_t bs = (uint32_t)a.bs;
    const uint32_t o0 = b0 * bs, o1 = b1 * bs, o2 = b2 * bs;
    const double r_d = c->r_d;
    auto fresh = [&]() { return PadReduce{a.type, a.cst, 0.0f, 0.0f, false}; };
    if (a.ndim == 1) {
        PadReduce p = fresh();
        if (a.type != VSZ_PADV_CONST)
            for (uint32_t i = 0; i < bs; i++) p.add(field_at(a, o0 + i, 0, 0));
        st_f32_bytes(a.arch + 4 * b, p.result(bs));  // raw
        return;
    }
    if (a.mode == VSZ_PAD_BLOCK) {
        PadReduce p = fresh();
        const uint32_t nk = a.ndim == 3 ? bs : 1u;
        if (a.type != VSZ_PADV_CONST)
            for (uint32_t k = 0; k < nk; k++)
                for (uint32_t j = 0; j < bs; j++)
                    for (uint32_t i = 0; i < bs; i++) p.add(field_at(a, o0 + i, o1 + j, o2 + k));
        st_f32_bytes(a.arch + 4 * b, prequant_pad(p.result((unsigned long long)bs * bs * nk), r_d));
        return;
    }
    uint8_t* out = a.arch + 4 * b * (unsigned long long)a.ndim;
    if (a.ndim == 2) {
        PadReduce top = fresh(), lft = fresh();
        if (a.type != VSZ_PADV_CONST)
            for (uint32_t i = 0; i < bs; i++) {
                top.add(field_at(a, o0 + i, o1, 0));
                lft.add(field_at(a, o0, o1 + i, 0));
            }
        st_f32_bytes(out, prequant_pad(top.result(bs), r_d));
        st_f32_bytes(out + 4, prequant_pad(lft.result(bs), r_d));
        return;
    }
    PadReduce fr = fresh(), lf = fresh(), tp = fresh();
    if (a.type != VSZ_PADV_CONST)
        for (uint32_t j = 0; j < bs; j++)
            for (uint32_t i = 0; i < bs; i++) {
                fr.add(field_at(a, o0 + i, o1 + j, o2));  // front face z = 0: x fastest, then y
                lf.add(field_at(a, o0, o1 + i, o2 + j));  // left face x = 0: y fastest, then z
                tp.add(field_at(a, o0 + i, o1, o2 + j));  // top face y = 0: x fastest, then z
            }
    const unsigned long long f = (unsigned long long)bs * bs;
    st_f32_bytes(out, prequant_pad(fr.result(f), r_d));
    st_f32_bytes(out + 4, prequant_pad(lf.result(f), r_d));
    st_f32_bytes(out + 8, prequant_pad(tp.result(f), r_d));
}

// Global max / min, pass 1: ordered keys of the extremes (NaNs skipped).
__global__ void __launch_bounds__(256) k_pad_extreme(const float* __restrict__ x, size_t n, PadWs* ws) {
    uint32_t kmax = 0u, kmin = 0xffffffffu;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const float v = __ldcs(x + i);
        if (v == v) {
            const uint32_t k = f2key(v);
            kmax = max(kmax, k);
            kmin = min(kmin, k);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
        kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&ws->key[0], kmax);
        atomicMin(&ws->key[1], kmin);
    }
}

// Global max / min, pass 2 (zero extreme only): the first index holding +-0, whose sign the
// reference's first-wins scan keeps.  Each thread stops at its first match.
__global__ void __launch_bounds__(256) k_pad_first_zero(const float* __restrict__ x, size_t n, int type, PadWs* ws) {
    const float e = key2f(type == VSZ_PADV_MAX ? ws->key[0] : ws->key[1]);
    if (e != 0.0f) return;  // uniform
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        if (x[i] == 0.0f) {
            atomicMin(&ws->first, (unsigned long long)i);
            break;
        }
    }
}

// Global avg: the serial float sum.  Warps 1.. stage tile t + 1 into shared memory while thread 0
// adds tile t.
constexpr int kAvgTile = 4096;
__global__ void __launch_bounds__(512) k_pad_avg(const float* __restrict__ x, size_t n, PadWs* ws) {
    __shared__ __align__(16) float buf[2][kAvgTile];
    const size_t ntiles = (n + kAvgTile - 1) / kAvgTile;
    auto stage = [&](size_t t, int slot, int tid, int nthr) {
        const size_t base = t * kAvgTile;
        const int len     = (int)min((size_t)kAvgTile, n - base);
        for (int i = tid; i < len; i += nthr) buf[slot][i] = __ldcs(x + base + i);
    };
    stage(0, 0, threadIdx.x, blockDim.x);
    __syncthreads();
    float s = 0.0f, s_prev = 0.0f;
    bool nan_seen = false;
    for (size_t t = 0; t < ntiles; t++) {
        if (threadIdx.x >= 32) {
            if (t + 1 < ntiles) stage(t + 1, (int)((t + 1) & 1), threadIdx.x - 32, blockDim.x - 32);
        } else if (threadIdx.x == 0 && !nan_seen) {  // a NaN sum stays as it is
            const float* b = buf[t & 1];
            const int len  = (int)min((size_t)kAvgTile, n - t * kAvgTile);
            int i          = 0;
            for (; i + 4 <= len; i += 4) {
                const float4 v = *reinterpret_cast<const float4*>(b + i);
                s = __fadd_rn(s, v.x);
                s = __fadd_rn(s, v.y);
                s = __fadd_rn(s, v.z);
                s = __fadd_rn(s, v.w);
            }
            for (; i < len; i++) s = __fadd_rn(s, b[i]);
            // x86 NaN propagation (rare): redo the tile keeping the first NaN's bits
            if (s != s && !nan_seen) {
                nan_seen = true;
                s        = s_prev;
                for (int k = 0; k < len; k++)
                    if (s == s) s = (b[k] == b[k]) ? __fadd_rn(s, b[k]) : quiet_nan(b[k]);
            }
            s_prev = s;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) ws->sum = s;
}

// Global value, its archive form and the compressor's halo value (one thread).
__global__ void k_pad_global_finish(PadArgs a, size_t n, const PadWs* ws) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const Consts* c = a.consts;
    if (c->status != VSZ_OK) return;
    float p;
    if (a.type == VSZ_PADV_CONST) {
        p = a.cst;
    } else if (a.type == VSZ_PADV_AVG) {
        p = (ws->sum == ws->sum) ? __fdiv_rn(ws->sum, __ull2float_rn((unsigned long long)n)) : ws->sum;
    } else {
        const float x0 = a.x[0];
        if (x0 != x0) {
            p = x0;  // a leading NaN is never replaced
        } else {
            p = key2f(a.type == VSZ_PADV_MAX ? ws->key[0] : ws->key[1]);
            if (p == 0.0f) p = a.x[ws->first];
        }
    }
    const float arch = (p != p) ? quiet_nan(p) : __double2float_rn(round(__dmul_rn((double)p, c->r_d)));
    st_f32_bytes(a.arch, arch);
    *a.halo_g = (a.ndim == 1) ? arch : prequant_pad(p, c->r_d);
}

}  // namespace

size_t pad_ws_bytes() { return sizeof(PadWs); }

size_t pad_count(int ndim, const uint32_t d[3], int bs, int mode) {
    if (mode == VSZ_PAD_GLOBAL) return 1;
    if (mode != VSZ_PAD_BLOCK && mode != VSZ_PAD_EDGE) return 0;
    size_t nb = 1;
    for (int i = 0; i < 3; i++) nb *= ((size_t)d[i] + (size_t)bs + 1) / (size_t)bs;
    return (mode == VSZ_PAD_EDGE && ndim > 1) ? nb * (size_t)ndim : nb;
}

int launch_pad_values(const PadArgs& a, cudaStream_t st, int num_sms) {
    if (a.mode == VSZ_PAD_NONE) return VSZ_OK;
    if (a.mode == VSZ_PAD_BLOCK || a.mode == VSZ_PAD_EDGE) {
        const unsigned long long nblk = (unsigned long long)a.nb0 * a.nb1 * a.nb2;
        k_pad_blocks<<<(unsigned)((nblk + 127) / 128), 128, 0, st>>>(a);
        count_launch();
        return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
    }
    const size_t n = (size_t)a.d0 * a.d1 * a.d2;
    PadWs* ws      = static_cast<PadWs*>(a.ws);
    if (a.type == VSZ_PADV_MAX || a.type == VSZ_PADV_MIN) {
        if (cudaMemsetAsync(&ws->key[0], 0x00, 4, st) != cudaSuccess ||
            cudaMemsetAsync(&ws->key[1], 0xff, 4, st) != cudaSuccess ||
            cudaMemsetAsync(&ws->first, 0xff, 8, st) != cudaSuccess)
            return VSZ_ERR_CUDA;
        long long want = (long long)((n + 2047) / 2048), cap = (long long)num_sms * 8;
        int grid = (int)(want < cap ? want : cap);
        if (grid < 1) grid = 1;
        k_pad_extreme<<<grid, 256, 0, st>>>(a.x, n, ws);
        count_launch();
        k_pad_first_zero<<<grid, 256, 0, st>>>(a.x, n, a.type, ws);
        count_launch();
    } else if (a.type == VSZ_PADV_AVG) {
        k_pad_avg<<<1, 512, 0, st>>>(a.x, n, ws);
        count_launch();
    }
    k_pad_global_finish<<<1, 32, 0, st>>>(a, n, ws);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

}  // namespace vsz
