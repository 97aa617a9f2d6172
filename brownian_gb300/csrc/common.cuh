// Device helpers shared by the MPCD kernels (sm_103a).
//
// GB300 executes FP64 at about 2 operations per clock per SM (DDIV near 0.25),
// against ~126 FP32 and ~64 INT32 operations.  The helpers here therefore keep
// the reference's FP64 semantics exactly but move every range test, truncation
// and conversion to integer operations on the IEEE bit pattern, and reach for
// an FP64 divide only in the rare cases where the reference's rounding could
// make a difference.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bgb {

// ------------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3"
// (SC'11): ten rounds of two 32x32 multiplies, key bumped by the Weyl constants.
__device__ __host__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k.x += 0x9E3779B9u; k.y += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

// Draw domains: counter word w carries (domain << 24) | block.
enum : uint32_t {
  DOM_SHIFT = 1, DOM_AXIS = 2, DOM_COLL = 3, DOM_TUMBLE = 4, DOM_ROTDIFF = 5,
  DOM_INIT_CPOS = 6, DOM_INIT_CVEL = 7, DOM_INIT_FPOS = 8, DOM_INIT_FVEL = 9
};

__device__ __host__ __forceinline__ uint4 draw4(uint2 key, uint32_t dom, uint32_t blk, uint32_t a, uint32_t b,
                                                 uint32_t t) {
  return philox(make_uint4(a, b, t, (dom << 24) | (blk & 0xFFFFFFu)), key);
}

// The double v 2^-k for an odd v < 2^53 (negated if neg), assembled on the
// integer pipe: the leading-bit position b of v gives the exponent, v shifted up
// to bit 52 the mantissa.  Exact (v has at most 53 significant bits).
__device__ __forceinline__ double odd_scaled(unsigned long long v, int k, bool neg) {
  const int b = 63 - __clzll((long long)v);
  const unsigned long long bits =
      ((unsigned long long)(1023 + b - k) << 52) | ((v << (52 - b)) & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)(bits | (neg ? 0x8000000000000000ull : 0ull)));
}

// uniform in (0,1): (w + 1/2) 2^-32 = (2w + 1) 2^-33, exact in double.  The device
// assembles it from bits: a GB300 SM runs one FP64 instruction of a warp per ~64
// cycles, the integer form costs a few cycles; both give the same double.
__device__ __host__ __forceinline__ double u01(uint32_t w) {
#ifdef __CUDA_ARCH__
  return odd_scaled(2ull * w + 1ull, 33, false);
#else
  return ((double)w + 0.5) * 2.3283064365386963e-10;
#endif
}

// 2 u01(w) - 1 = (2w + 1 - 2^32) 2^-32, exact (the reference's 2 ran - 1)
__device__ __forceinline__ double pm1(uint32_t w) {
  const long long n = 2ll * (long long)w + 1ll - 4294967296ll;  // odd, |n| < 2^32
  return odd_scaled((unsigned long long)(n < 0 ? -n : n), 32, n < 0);
}

// ------------------------------------------------------------- exact FP64 helpers
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// int(x) for 0 <= x < 2^31 (the reference's truncating cell coordinate), on the
// integer pipe: mantissa shifted by the unbiased exponent.
// Values at or above 2^30 (and NaN/inf) return 2^30; negative values return 0.
__device__ __forceinline__ int trunc_nonneg(double x) {
  long long b = dbits(x);
  int e = (int)(b >> 52) - 1023;
  if (e < 0) return 0;
  if (e >= 30) return 1 << 30;
  unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  return (int)(m >> (52 - e));
}

// Parameters of one periodic dimension for the exact wrap/image operations.
struct Dim {
  double L, halfL;
  long long lo_bits;    // bits of 2^-30 L: for L > a >= 2^-30 L, mod(a, L) == a
  long long L_bits;     // bits of L
  long long img_bits;   // bits of 0.49 L: |a| < 0.49 L  =>  img(a, L) == a
  long long img1_bits;  // bits of 0.51 L: 0.51 L < |a| < 1.49 L  =>  img(a, L) == a - L sign(a)
  long long img2_bits;  // bits of 1.49 L
};

// The reference's mod(a, L) = a - L*lround((a - L/2)/L) (cpp/parameters.hpp:75).
// The quotient rounds to 0 for a in [2^-30 L, L) (result a), to 1 for a in
// [L, 1.49 L) (result a - L*1) and to -1 for a in (-0.49 L, -0] (result
// a - L*(-1)); those subtractions are the reference's own, so the results are
// bit-identical.  Only a in [0, 2^-30 L), where rounding decides, and values
// further out take the reference's division (mod(0, L) == L comes from there).
__device__ __forceinline__ double ref_mod(double a, const Dim &d) {
  long long b = dbits(a);
  if (b >= d.lo_bits && b < d.L_bits) return a;
  if (b >= d.L_bits && b < d.img2_bits) return __dsub_rn(a, d.L);
  if (b < 0 && (b & 0x7FFFFFFFFFFFFFFFll) < d.img_bits) return __dsub_rn(a, -d.L);
  double q = __ddiv_rn(__dsub_rn(a, d.halfL), d.L);
  return __dsub_rn(a, __dmul_rn(d.L, (double)llround(q)));
}

// The reference's img(a, L) = a - L*lround(a/L) (cpp/parameters.hpp:76).  For
// |a| < 0.49 L the quotient rounds to 0 (result a); for 0.51 L < |a| < 1.49 L it
// rounds to sign(a) (result a - L sign(a), one subtraction as in the reference);
// only the bands around L/2 and beyond take the division.
__device__ __forceinline__ double ref_img(double a, const Dim &d) {
  long long b = dbits(a) & 0x7FFFFFFFFFFFFFFFll;
  if (b < d.img_bits) return a;
  if (b > d.img1_bits && b < d.img2_bits) return __dsub_rn(a, a > 0 ? d.L : -d.L);
  return __dsub_rn(a, __dmul_rn(d.L, (double)llround(__ddiv_rn(a, d.L))));
}

// (x*x + y*y) + z*z with separately rounded products, as point::sum() of a*a.
__device__ __forceinline__ double norm2_ref(double x, double y, double z) {
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// ---------------------------------------------------------------- fixed point
// round(x * 2^k) to the nearest integer (ties to even), computed from the bit
// pattern.  Integer sums of these are exact and independent of summation order,
// which makes every cell and colloid sum deterministic.  Caller bounds |x| so the
// result fits.
__device__ __forceinline__ long long to_fix(double x, int k) {
  long long b = dbits(x);
  int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0;
  unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  int sh = e - 1075 + k;
  unsigned long long r;
  if (sh >= 0) {
    r = m << sh;
  } else if (sh > -64) {
    int s = -sh;
    r = m >> s;
    unsigned long long rem = m & ((1ull << s) - 1ull), half = 1ull << (s - 1);
    if (rem > half || (rem == half && (r & 1ull))) r += 1ull;
  } else {
    r = 0;
  }
  return b < 0 ? -(long long)r : (long long)r;
}

__device__ __forceinline__ double from_fix(long long v, double inv_scale) { return (double)v * inv_scale; }

// ------------------------------------------------------------------ small math
struct d3 { double x, y, z; };
__device__ __forceinline__ d3 mk(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ d3 ld3(const double *x, const double *y, const double *z, int i) { return mk(x[i], y[i], z[i]); }
__device__ __forceinline__ void st3(double *x, double *y, double *z, int i, d3 v) { x[i] = v.x; y[i] = v.y; z[i] = v.z; }
// component-wise operations with separately rounded steps, matching the
// reference's point operators (cpp/parameters.hpp:47-58)
__device__ __forceinline__ d3 add3(d3 a, d3 b) { return mk(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)); }
__device__ __forceinline__ d3 sub3(d3 a, d3 b) { return mk(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)); }
__device__ __forceinline__ d3 mul3s(d3 a, double s) { return mk(__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s)); }
__device__ __forceinline__ d3 div3s(d3 a, double s) { return mk(__ddiv_rn(a.x, s), __ddiv_rn(a.y, s), __ddiv_rn(a.z, s)); }
__device__ __forceinline__ double dot_ref(d3 a, d3 b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
// crossmul of cpp/fluid_colloid_collision.cpp:3-5
__device__ __forceinline__ d3 cross_ref(d3 a, d3 b) {
  return mk(__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
            __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

}  // namespace bgb
