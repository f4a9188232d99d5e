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

// double -> float, round to nearest even.
__device__ __forceinline__ float d2f(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  const unsigned man = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 of the 52 mantissa bits
  const unsigned rem = lo & 0x1fffffffu;                     // the 29 dropped bits
  unsigned r = sign | ((unsigned)(e - 896) << 23) | man;     // exponent bias 1023 -> 127
  r += (rem > 0x10000000u || (rem == 0x10000000u && (man & 1u))) ? 1u : 0u;  // a carry may raise the exponent
  if (e <= 896) r = sign;                                    // below FP32's normal range: signed zero
  if (e >= 1151) r = (e == 2047 && ((hi & 0xfffffu) | lo)) ? 0x7fc00000u : (sign | 0x7f800000u);
  return __uint_as_float(r);
}

// float -> double, exact for normal numbers.
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u;
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned m = b & 0x7fffffu;
  unsigned hi = sign | ((e + 896u) << 20) | (m >> 3);
  unsigned lo = m << 29;
  if (e == 0u) { hi = sign; lo = 0u; }
  if (e == 255u) hi = sign | 0x7ff00000u | (m >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

}  // namespace tlq
