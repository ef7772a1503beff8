// Device-side building blocks shared by every kernel of the dual-quantization path.
//
// Arithmetic rule: every floating-point step that the reference performs as a separately rounded
// IEEE-754 operation is written here with an explicit round-to-nearest intrinsic
// (__fadd_rn/__fsub_rn/__fmul_rn/__fsqrt_rn), and the library is compiled with -fmad=false, so
// no contraction or reassociation can change a single bit of a quant code or a reconstruction.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "vsz_types.h"

namespace vsz {

constexpr int kWarp = 32;
// Width (in x) of the tile one warp owns in the dual-quant kernels: 32 lanes x 4 columns.
constexpr int kTileX = 128;
// Row segment used to rank outliers in row-major order for compaction: one warp tile row.
constexpr int kSegX = kTileX;

// Bounded spin for every cross-CTA wait (decoupled look-back): after this many polls the kernel
// records VSZ_ERR_TIMEOUT in the status word and gives up instead of hanging the GPU.
constexpr long long kSpinLimit = 1ll << 22;

// Counts one kernel launch of this library (read through vsz_launch_count); called after every
// <<<>>> launch.
void count_launch();

// Raises a kernel's dynamic shared-memory limit on the current device once per (kernel, device):
// the attribute is per device, and the host call stays out of later launches.  The bit is set
// only after the attribute is, so a racing thread at worst sets it twice.
template <class K>
inline void smem_limit_once(K kern, int bytes, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_release);
}

// ------------------------------------------------------------------------------------------
// Constants derived from the error bound, resident in device memory so that r2r fields can
// compute them on the device (value range -> eb) without a host round trip.
// ------------------------------------------------------------------------------------------
struct Consts {
    double eb_final;  // absolute error bound (eb, or eb * value range for r2r)
    double r_d;       // 1 / (2 eb)           ebs_L4[EBx2_r], src/types.cc:91
    double c_d;       // 2 eb                 ebs_L4[EBx2],   src/types.cc:90
    double range;     // value range used (r2r), 0 for abs
    float r_f;        // (float) r_d          the AVX prequant multiplier, src/dualquant.hh:264
    float c_hi;       // (float) c_d          split of c_d for the FP32 dequant, see dequant()
    float c_lo;       // (float)(c_d - c_hi)
    int dq_fast;      // 1 when c_hi and c_lo are normal floats, so dequant() may take its FP32 path
    int status;       // VSZ_OK, or why the constants are unusable (zero value range)
    int dq_mul;       // dequant_small(): 0 dequant(); 1 fmaf(s, c_hi, s * c_lo) is exact for every
                      // integer |s| < 2^21; 2 the same except at s = +-dq_exc (k_dq_mul_verify)
    float dq_exc;     // the one s > 0 where the two-operation form differs (dq_mul 2)
    float dq_exc_y;   // (float)((double)dq_exc * c_d)
};

// ------------------------------------------------------------------------------------------
// Prequantization (compress) -- reference rules, one element.
// ------------------------------------------------------------------------------------------

// AVX form: rint(x *f32 r_f)   (src/dualquant.hh:89,290,622,784)
__device__ __forceinline__ float prequant_vec(float x, float r_f) { return rintf(__fmul_rn(x, r_f)); }

// Scalar form: (float) round((double) x * r_d)   (src/dualquant.hh:109,298,631,796)
__device__ __forceinline__ float prequant_scalar(float x, double r_d) {
    return __double2float_rn(round(__dmul_rn((double)x, r_d)));
}

// ------------------------------------------------------------------------------------------
// Dequantization: (float)((double)s * c_d)   (src/dualquant.hh:941,980,1038)
//
// Blackwell Ultra has a small FP64 rate, so the double multiply is emulated in FP32 where that
// is provably exact and falls back to a real double multiply otherwise:
//   c_d = c_hi + delta, c_lo = RN32(delta);  P = s*c_d exactly = p + e1 + s*delta
//   p = RN32(s*c_hi), e1 = s*c_hi - p (exact, fma), t = RN32(s*c_lo + e1)
//   y = RN32(p + t) is RN32(P) unless P lies within a tiny margin of a float midpoint (where
//   single rounding and the reference's double rounding can differ) -- the error of p + t
//   against P is below ulp(y) * 2^-21, the double-rounding tie window is ulp(y) * 2^-30, and the
//   margin tested is ulp(y) * 2^-17.  Powers of two, tiny or huge results and non-finite s take
//   the double path.  tests/test_gpu_exact.py checks every integer s in [-2^24, 2^24] against
//   the double multiply on the device.
// ------------------------------------------------------------------------------------------
// NaN bits as the reference's x86 arithmetic leaves them: an operation on a NaN operand returns that
// NaN, quieted (payload kept), where the GPU's FP32 arithmetic returns its canonical NaN.  Applied
// where a NaN can reach the archive or the output: outlier values, pad values, reconstructions.
__device__ __forceinline__ float quiet_nan(float v) { return __uint_as_float(__float_as_uint(v) | 0x00400000u); }

__device__ __forceinline__ float dequant_fp64(float s, double c_d) {
    if (s != s) return quiet_nan(s);
    return __double2float_rn(__dmul_rn((double)s, c_d));
}

__device__ __forceinline__ float dequant(float s, double c_d, float c_hi, float c_lo, int fast) {
    if (!fast) return dequant_fp64(s, c_d);
    if (s == 0.0f) return __fmul_rn(s, c_hi);  // +-0 * c = +-0
    float p  = __fmul_rn(s, c_hi);
    float e1 = __fmaf_rn(s, c_hi, -p);
    float t  = __fmaf_rn(s, c_lo, e1);
    float y  = __fadd_rn(p, t);
    float r  = __fadd_rn(__fsub_rn(p, y), t);
    uint32_t yb = __float_as_uint(y);
    uint32_t ye = yb & 0x7f800000u;
    // Fast path only for results with exponent field in (50, 253) that are not powers of two
    // (|y| > 2^-77 keeps e1, h and tau normal); everything else goes to FP64.
    bool ok = (ye > (50u << 23)) && (ye < (253u << 23)) && ((yb & 0x007fffffu) != 0u);
    if (ok) {
        float h    = __uint_as_float(ye - (24u << 23));  // half an ulp of y
        float dist = fabsf(__fsub_rn(fabsf(r), h));     // distance of P to the nearest midpoint
        float tau  = __uint_as_float(ye - (41u << 23)); // h * 2^-17
        ok         = dist > tau;
    }
    if (ok) return y;
    return dequant_fp64(s, c_d);
}

// Dequantization of an integer |s| < 2^21 (the separable reverse Lorenzo's values; larger ones are
// redone through dequant()).  When k_dq_mul_verify has compared, for every such s, the
// two-operation form RN32(s * c_hi + RN32(s * c_lo)) with the reference's (float)((double)s * c_d)
// and found them equal (or equal but at one pair +-dq_exc), that form is used; both are odd in s.
__device__ __forceinline__ float dequant_small(float s, const Consts& c) {
    if (c.dq_mul == 0) return dequant(s, c.c_d, c.c_hi, c.c_lo, c.dq_fast);
    float y = __fmaf_rn(s, c.c_hi, __fmul_rn(s, c.c_lo));
    if (c.dq_mul == 2 && fabsf(s) == c.dq_exc) y = copysignf(c.dq_exc_y, s);
    return y;
}

// Order-preserving map of floats onto unsigned integers (NaNs are skipped by the caller).
__device__ __forceinline__ uint32_t f2key(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key2f(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(b);
}

// A float at any byte address (archive sections need not be 4-byte aligned).
__device__ __forceinline__ float ld_f32_bytes(const uint8_t* p) {
    const uint32_t b = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    return __uint_as_float(b);
}
__device__ __forceinline__ void st_f32_bytes(uint8_t* p, float v) {
    const uint32_t b = __float_as_uint(v);
    p[0] = (uint8_t)b;
    p[1] = (uint8_t)(b >> 8);
    p[2] = (uint8_t)(b >> 16);
    p[3] = (uint8_t)(b >> 24);
}

// ------------------------------------------------------------------------------------------
// Status word: first error wins; kernels check it to skip work after a failure.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void set_status(int* status, int code) { atomicCAS(status, VSZ_OK, code); }

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// 16-byte asynchronous global -> shared copy (cp.async.cg); only the first src_bytes (0..16)
// are read, the rest of the 16 bytes is zero-filled.  Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16_zfill(void* smem, const void* gmem, uint32_t src_bytes) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// Wait until at most N of this thread's committed groups are still in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Big-endian byte order of a 32-bit word (the bitstream is MSB-first bytes).
__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

// Volatile / acquire-release helpers for decoupled look-back.
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

}  // namespace vsz
