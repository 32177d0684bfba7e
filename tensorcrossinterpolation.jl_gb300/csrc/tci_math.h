// Deterministic double-precision exp and cos used by the registered device
// functions.
//
// Both the CUDA kernels and the CPU oracle compile this header, so a function
// value computed on the GPU is bit-identical to the one computed on the host:
// every step is an IEEE-754 basic operation (+, -, *, /), an explicitly
// requested fused multiply-add (fma, correctly rounded on both sides), rint
// (round-half-even) or an exact power-of-two scaling built from bits.  The
// host side must be compiled with -ffp-contract=off; the device side with
// -fmad=false, so that no compiler contracts a*b+c on its own.
//
// Method (classical, from the mathematics):
//   exp: Cody-Waite reduction x = n*ln2 + r with ln2 split into a 32-bit head
//        (exact products n*LN2_HI for |n| < 2^21) and a tail; exp(r) for
//        |r| <= ln2/2 by the Taylor series to degree 13 evaluated with Horner
//        (truncation error < 5e-18 relative); scaling by 2^n from bits, in two
//        steps where the result is subnormal or near overflow.
//   cos: Cody-Waite reduction x = n*pi/2 + r with pi/2 split into two 33-bit
//        heads and a tail (exact products for |n| < 2^20, i.e. |x| < 1.6e6);
//        sin/cos of |r| <= pi/4 by their Taylor series (degree 17 / 18), the
//        quadrant picked from n mod 4.
// The Taylor coefficients are 1/k! rounded to double.  The split constants
// were computed with 300-bit arithmetic (head = value truncated to 32 or 33
// significant bits, tail = remainder rounded to double).
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define TCI_HD __host__ __device__ __forceinline__
#else
#define TCI_HD static inline
#endif

TCI_HD double tci_bits_to_double(uint64_t b) {
  union { uint64_t u; double d; } c; c.u = b; return c.d;
}
TCI_HD uint64_t tci_double_to_bits(double d) {
  union { uint64_t u; double d; } c; c.d = d; return c.u;
}
// 2^e for -1022 <= e <= 1023, exactly.
TCI_HD double tci_pow2i(int e) {
  return tci_bits_to_double((uint64_t)(e + 1023) << 52);
}
// p * 2^k, exact unless the result is subnormal (then a single IEEE rounding).
TCI_HD double tci_scale2(double p, int k) {
  if (k > 1023) return (p * tci_pow2i(k - 1023)) * tci_pow2i(1023);
  if (k < -1022) return (p * tci_pow2i(k + 1000)) * tci_pow2i(-1000);
  return p * tci_pow2i(k);
}

#define TCI_LN2_HI 0.6931471803691238        /* 0x3fe62e42fee00000 */
#define TCI_LN2_LO 1.9082149292705877e-10    /* 0x3dea39ef35793c76 */
#define TCI_INV_LN2 1.4426950408889634
#define TCI_PIO2_1 1.5707963267341256        /* 0x3ff921fb54400000 */
#define TCI_PIO2_2 6.077100506303966e-11     /* 0x3dd0b4611a600000 */
#define TCI_PIO2_3 2.0222662487959506e-21
#define TCI_TWO_OVER_PI 0.6366197723675814

TCI_HD double tci_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return tci_bits_to_double(0x7ff0000000000000ULL);
  if (x < -745.1332191019412) return 0.0;
  double n = rint(x * TCI_INV_LN2);
  double r = (x - n * TCI_LN2_HI) - n * TCI_LN2_LO;
  double p = 1.6059043836821613e-10;           // 1/13!
  p = fma(p, r, 2.08767569878681e-09);         // 1/12!
  p = fma(p, r, 2.505210838544172e-08);        // 1/11!
  p = fma(p, r, 2.755731922398589e-07);        // 1/10!
  p = fma(p, r, 2.7557319223985893e-06);       // 1/9!
  p = fma(p, r, 2.48015873015873e-05);         // 1/8!
  p = fma(p, r, 0.0001984126984126984);        // 1/7!
  p = fma(p, r, 0.001388888888888889);         // 1/6!
  p = fma(p, r, 0.008333333333333333);         // 1/5!
  p = fma(p, r, 0.041666666666666664);         // 1/4!
  p = fma(p, r, 0.16666666666666666);          // 1/3!
  p = fma(p, r, 0.5);                          // 1/2!
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  return tci_scale2(p, (int)n);
}

// sin(r)/r - 1 style polynomial for |r| <= pi/4: r + r^3 * S(r^2)
TCI_HD double tci_sin_poly(double r) {
  double z = r * r;
  double s = 2.8114572543455206e-15;           // 1/17!
  s = fma(s, z, -7.647163731819816e-13);       // -1/15!
  s = fma(s, z, 1.6059043836821613e-10);       // 1/13!
  s = fma(s, z, -2.505210838544172e-08);       // -1/11!
  s = fma(s, z, 2.7557319223985893e-06);       // 1/9!
  s = fma(s, z, -0.0001984126984126984);       // -1/7!
  s = fma(s, z, 0.008333333333333333);         // 1/5!
  s = fma(s, z, -0.16666666666666666);         // -1/3!
  return fma(r * z, s, r);
}
TCI_HD double tci_cos_poly(double r) {
  double z = r * r;
  double c = 1.5619206968586225e-16;           // 1/18!
  c = fma(c, z, -4.779477332387385e-14);       // -1/16!
  c = fma(c, z, 1.1470745597729725e-11);       // 1/14!
  c = fma(c, z, -2.08767569878681e-09);        // -1/12!
  c = fma(c, z, 2.755731922398589e-07);        // 1/10!
  c = fma(c, z, -2.48015873015873e-05);        // -1/8!
  c = fma(c, z, 0.001388888888888889);         // 1/6!
  c = fma(c, z, -0.041666666666666664);        // -1/4!
  c = fma(c, z, 0.5);                          // 1/2!
  return fma(-z, c, 1.0);
}

TCI_HD double tci_cos(double x) {
  if (x != x) return x;
  if (x - x != 0.0) return (x - x);  // +-Inf -> NaN
  double n = rint(x * TCI_TWO_OVER_PI);
  double r = ((x - n * TCI_PIO2_1) - n * TCI_PIO2_2) - n * TCI_PIO2_3;
  int64_t q = (int64_t)n;
  int quadrant = (int)(q & 3);
  switch (quadrant) {
    case 0: return tci_cos_poly(r);
    case 1: return -tci_sin_poly(r);
    case 2: return -tci_cos_poly(r);
    default: return tci_sin_poly(r);
  }
}
