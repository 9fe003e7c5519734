// Split of an FP64 value into its FP32 rounding and a BF16 residual, by
// integer arithmetic on the FP64 bits:
//   hi = RN_fp32(x),  lo = RN_bf16(x - hi)   (x - hi is exact in FP64)
// the same numbers as the FP64 conversions (x - (double)(float)x rounded to
// BF16), without the FP64 pipe.  Plain C++ so that the device kernel and a
// host test compile the same function.  Magnitudes outside [2^-60, 2^128),
// zeros, subnormals, infinities and NaNs are left to the FP64 conversions
// (return value false).
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define FVG_HD __host__ __device__ __forceinline__
#else
#define FVG_HD inline
#endif

namespace fvg {

FVG_HD int split_bitlen(uint32_t v) {  // bits of v > 0
#if defined(__CUDA_ARCH__)
  return 32 - __clz((int)v);
#else
  return 32 - __builtin_clz(v);
#endif
}

// xb: the FP64 bits.  On true: *hb = FP32 bits of hi (an infinity when hi
// overflows, with *lob = 0), *lob = BF16 bits of lo.
FVG_HD bool split_bits(uint64_t xb, uint32_t* hb, uint16_t* lob) {
  const int e = (int)((xb >> 52) & 0x7ff) - 1023;  // unbiased exponent
  if (e < -60 || e > 127) return false;
  const uint32_t s = (uint32_t)(xb >> 63);
  const uint64_t f = xb & 0xfffffffffffffull;  // 52 fraction bits
  const uint32_t top = (uint32_t)(f >> 29);     // the 23 that FP32 keeps
  const uint32_t low = (uint32_t)(f & 0x1fffffffu);
  // truncation, then round to nearest even on the 29 dropped bits (a carry
  // out of the fraction moves to the next binade, or to infinity)
  const bool up = low > (1u << 28) || (low == (1u << 28) && (top & 1u));
  const uint32_t h = ((s << 31) | ((uint32_t)(e + 127) << 23) | top) + (up ? 1u : 0u);
  *hb = h;
  if ((h & 0x7fffffffu) == 0x7f800000u) {  // |x| rounds past the FP32 range
    *lob = 0;
    return true;
  }
  // x - hi = R * 2^(e-52), R < 2^29, with the sign of x (rounded down) or
  // the opposite sign (rounded up)
  const uint32_t R = up ? (1u << 29) - low : low;
  if (R == 0) {
    *lob = 0;  // +0, as x - hi in FP64
    return true;
  }
  const uint32_t rs = up ? (s ^ 1u) : s;
  const int nb = split_bitlen(R);
  int ex = nb - 1 + e - 52;  // R * 2^(e-52) lies in [2^ex, 2^(ex+1))
  uint32_t q;                 // 8 significant bits, rounded to nearest even
  if (nb <= 8) {
    q = R << (8 - nb);
  } else {
    const int sh = nb - 8;
    q = R >> sh;
    const uint32_t rem = R & ((1u << sh) - 1u), half = 1u << (sh - 1);
    if (rem > half || (rem == half && (q & 1u))) q++;
    if (q == 256u) {
      q = 128u;
      ex++;
    }
  }
  *lob = (uint16_t)((rs << 15) | ((uint32_t)(ex + 127) << 7) | (q & 127u));
  return true;
}

}  // namespace fvg
