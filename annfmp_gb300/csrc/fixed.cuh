// fixed.cuh -- exact fixed-point helpers of the exact projection: an FP64 value as a 128-bit
// integer of 2^-sh units, and such an integer rounded once to the nearest FP32 value.
#pragma once

namespace annf {

// D * 2^-sh rounded to the nearest float (ties to even), integer arithmetic only
__device__ __forceinline__ float fixed_to_float(__int128 D, int sh) {
  if (D == 0) return 0.0f;
  const bool neg = D < 0;
  const unsigned __int128 A = neg ? (unsigned __int128)(-D) : (unsigned __int128)D;
  const unsigned long long hi = (unsigned long long)(A >> 64), lo = (unsigned long long)A;
  const int p = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);  // top bit
  unsigned long long mant;
  int e;
  if (p <= 23) {
    mant = lo;
    e = -sh;
  } else {
    const int s = p - 23;
    const unsigned __int128 q = A >> s;
    const unsigned __int128 r = A - (q << s);
    const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
    mant = (unsigned long long)q;
    if (r > half || (r == half && (mant & 1ull))) ++mant;  // may reach 2^24: still exact below
    e = s - sh;
  }
  const float f = ldexpf((float)mant, e);
  return neg ? -f : f;
}

// m * 2^sh rounded to an integer (m FP64); exact whenever m's last bit weighs at least 2^-sh
__device__ __forceinline__ __int128 double_to_fixed(double m, int sh) {
  if (m == 0.0) return 0;
  int e;
  const double f = frexp(fabs(m), &e);                          // |m| = f 2^e, f in [0.5, 1)
  const long long mant = (long long)ldexp(f, 53);                // exact 53-bit integer
  const int s = e - 53 + sh;                                     // |m| 2^sh = mant 2^s
  __int128 v;
  if (s >= 0) {
    v = (__int128)mant << s;
  } else if (s > -64) {
    const long long q = mant >> (-s), r = mant - (q << (-s)), half = 1LL << (-s - 1);
    v = q + ((r > half || (r == half && (q & 1))) ? 1 : 0);
  } else {
    v = 0;
  }
  return m < 0 ? -v : v;
}

}  // namespace annf
