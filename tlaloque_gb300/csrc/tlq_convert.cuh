// tlq_convert.cuh -- double <-> float conversions on the integer pipe.
//
// On GB300 the F2F conversion instructions issue on the FP64 pipe (measured:
// a double->float or float->double conversion costs one DADD slot, and the
// FP64 pipe runs at 1/64 of the FP32 rate).  The mixed-precision step
// converts every state value it touches, so it converts with integer
// operations instead (measured 5.7x faster).  Both conversions flush FP32
// subnormals to zero (the mixed path is built with -ftz=true anyway) and keep
// infinities and NaNs.
#pragma once

namespace tlq {

// double -> float, round to nearest even.  One funnel shift takes the
// exponent's low 9 bits and the top 23 mantissa bits; subtracting
// 384 << 23 (= 896 mod 2^9) rebiases the exponent 1023 -> 127 for every
// exponent of FP32's normal range (the 9-bit field stays below 256, bit 31
// clear).  The increment rounds to nearest with ties to even: the 29
// dropped bits plus the kept lsb exceed half an ulp exactly when the result
// rounds up.
__device__ __forceinline__ float d2f(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u, ex = hi & 0x7ff00000u;
  unsigned r = __funnelshift_r(lo, hi, 29) - (384u << 23);
  r += ((lo & 0x1fffffffu) + (r & 1u)) > 0x10000000u ? 1u : 0u;  // a carry may raise the exponent
  r = (r & 0x7fffffffu) | sign;
  if (ex < (897u << 20)) r = sign;  // below FP32's normal range: signed zero
  if (ex >= (1151u << 20)) r = (ex == 0x7ff00000u && ((hi & 0xfffffu) | lo)) ? 0x7fc00000u : (sign | 0x7f800000u);
  return __uint_as_float(r);
}

// float -> double, exact for normal numbers: the magnitude's bits shifted
// right by 3 are the double's high word with the exponent still biased by
// 127; adding 896 << 20 rebiases it to 1023.
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u, ex = b & 0x7f800000u;
  unsigned hi = (((b & 0x7fffffffu) >> 3) + (896u << 20)) | sign;
  unsigned lo = b << 29;
  if (ex == 0u) { hi = sign; lo = 0u; }
  if (ex == 0x7f800000u) hi = sign | 0x7ff00000u | ((b & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

}  // namespace tlq
