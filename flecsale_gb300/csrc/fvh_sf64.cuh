// FP64 multiplication, addition and division on the integer and FP32 pipes,
// correctly rounded to nearest-even, so they return the same bits as the
// IEEE-754 binary64 operations (and as the hardware DMUL / DADD / division).
//
// Why: GB300 executes 2 FP64 operations per clock per SM, against 64-128
// integer or FP32 operations.  The bit-exact FP64 kernels are bound by that
// pipe while most issue slots stay idle, so a kernel moves part of its FP64
// arithmetic here and keeps the rest on the FP64 pipe; both run at once.
//
// Method (the textbook software floating point of e.g. Muller et al.,
// "Handbook of Floating-Point Arithmetic", 2nd ed., ch. 7-8): unpack sign,
// exponent and significand; compute the exact result significand, or enough of
// it plus a sticky bit; round to nearest-even from the guard bit and the
// sticky bit; repack, letting a rounding carry propagate into the exponent.
// Operands of magnitude within 2^+-500 take this path (every result is then
// normal and finite), and so do zero operands with a finite partner (a product
// or sum with a zero is frequent: a uniform region has zero differences);
// subnormals, infinities, NaNs and extreme exponents go to the hardware
// instruction, so every input gives the IEEE result.
//
//   mul: the 106-bit product of the 53-bit significands from four 32x32-bit
//        integer multiplies.
//   add: the smaller operand aligned with 8 extra low bits and a jammed sticky
//        bit, integer add or subtract, renormalisation.
//   div: long division in base 2^22 (Knuth, TAOCP vol. 2, 4.3.1): each
//        quotient digit estimated from an FP32 reciprocal of the divisor's top
//        24 bits, then corrected by one step either way from the exact integer
//        remainder; 53 quotient bits plus a guard bit, the final remainder
//        gives the sticky bit.
//
// The tests of the exponent and zero bits work on the two 32-bit halves taken
// through an opaque move, so the compiler cannot turn them into FP64
// comparisons (which would run on the FP64 pipe this code exists to relieve).
//
// Checked bitwise against the hardware operations on random and adversarial
// operands by fvh_debug_sf64 (tests/test_gpu_sf64.py).
#pragma once

#include <cstdint>

namespace fvh {
namespace sf64 {

constexpr unsigned long long kM52 = 0x000fffffffffffffull;
constexpr unsigned long long kH52 = 0x0010000000000000ull;

__device__ __forceinline__ unsigned long long bits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double dbl(unsigned long long u) {
  return __longlong_as_double((long long)u);
}

// The two 32-bit halves of a double and back, through an opaque move.
__device__ __forceinline__ void halves(double x, unsigned &lo, unsigned &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
__device__ __forceinline__ double join(unsigned lo, unsigned hi) {
  double x;
  asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
  return x;
}

// Rare operands go to the hardware instruction in an out-of-line call, so it
// takes an FP64 issue slot only when a lane needs it (an inlined fallback is
// issued, predicated off, on every call).
__device__ __noinline__ double mul_rare(double a, double b) { return __dmul_rn(a, b); }
__device__ __noinline__ double add_rare(double a, double b) { return __dadd_rn(a, b); }
__device__ __noinline__ double div_rare(double a, double b) { return __ddiv_rn(a, b); }

// biased exponent field of the high half
__device__ __forceinline__ unsigned expo(unsigned hi) { return (hi >> 20) & 0x7ffu; }
// exponents in [523, 1523] (magnitudes within 2^+-500): sums, differences,
// products and quotients of two such values are normal and finite
__device__ __forceinline__ bool moderate(unsigned e) { return e - 523u < 1001u; }
__device__ __forceinline__ bool is_zero(unsigned lo, unsigned hi) {
  return ((hi & 0x7fffffffu) | lo) == 0u;
}
__device__ __forceinline__ bool is_finite(unsigned hi) {
  return (hi & 0x7ff00000u) != 0x7ff00000u;
}

// Rounded product of two moderate operands (halves al:ah, bl:bh); sign and
// exponent are left to the caller through `sign`.
__device__ __forceinline__ double mul_core(unsigned al, unsigned ah, unsigned bl, unsigned bh,
                                           unsigned ea, unsigned eb, unsigned sign) {
  // significands (53 bits): (mah:al), (mbh:bl); P = product in 32-bit words
  // w3 w2 w1 w0, P in [2^104, 2^106)
  const unsigned mah = (ah & 0xfffffu) | 0x100000u, mbh = (bh & 0xfffffu) | 0x100000u;
  const unsigned long long p0 = (unsigned long long)al * bl;
  const unsigned long long t =
      (unsigned long long)al * mbh + (unsigned long long)mah * bl + (p0 >> 32);
  const unsigned long long u = (unsigned long long)mah * mbh + (t >> 32);
  const unsigned w0 = (unsigned)p0, w1 = (unsigned)t, w2 = (unsigned)u, w3 = (unsigned)(u >> 32);
  // the significand is P >> (32 + s), s = 20, or 21 when P >= 2^105
  const unsigned top = (w3 >> 9) & 1u;
  const unsigned s = 20u + top;
  const unsigned mlo = __funnelshift_r(w1, w2, s), mhi = __funnelshift_r(w2, w3, s);
  const unsigned guard = (w1 >> (s - 1u)) & 1u;
  const unsigned sticky = ((w1 << (33u - s)) | w0) != 0u;
  const unsigned inc = guard & (sticky | (mlo & 1u));
  // exponent field of the result minus one (the significand's leading one,
  // bit 52, adds it back; a rounding carry to 2^53 moves on to the exponent)
  const unsigned e1 = ea + eb - 1024u + top;
  const unsigned long long r =
      ((unsigned long long)(mhi + (e1 << 20)) << 32 | mlo) + (unsigned long long)inc;
  return dbl(r | ((unsigned long long)sign << 32));
}

// a * b
__device__ __forceinline__ double mul(double a, double b) {
  unsigned al, ah, bl, bh;
  halves(a, al, ah);
  halves(b, bl, bh);
  const unsigned ea = expo(ah), eb = expo(bh);
  const unsigned sign = (ah ^ bh) & 0x80000000u;
  if (!(moderate(ea) & moderate(eb))) {
    // a zero times a finite value is the zero of the product's sign
    if ((is_zero(al, ah) & is_finite(bh)) | (is_zero(bl, bh) & is_finite(ah)))
      return join(0u, sign);
    return mul_rare(a, b);
  }
  return mul_core(al, ah, bl, bh, ea, eb, sign);
}

// a + b
__device__ __forceinline__ double add(double a, double b) {
  unsigned al, ah, bl, bh;
  halves(a, al, ah);
  halves(b, bl, bh);
  // x: the operand of larger magnitude
  const unsigned long long xa = ((unsigned long long)(ah & 0x7fffffffu) << 32) | al;
  const unsigned long long xb = ((unsigned long long)(bh & 0x7fffffffu) << 32) | bl;
  const bool swap = xa < xb;
  const unsigned long long mx = swap ? xb : xa, my = swap ? xa : xb;
  const unsigned sx = (swap ? bh : ah) & 0x80000000u;
  const unsigned ex = (unsigned)(mx >> 52), ey = (unsigned)(my >> 52);
  if (!(moderate(ex) & (ey != 0u))) {
    if ((my == 0) & (ex != 2047u)) {  // x + (+-0), x finite
      if (mx == 0) return join(0u, ah & bh & 0x80000000u);  // -0 only for (-0) + (-0)
      return swap ? b : a;
    }
    return add_rare(a, b);
  }
  // (ex moderate, y normal: the result exponent stays within [466, 1524])
  int d = (int)(ex - ey);
  d = d > 63 ? 63 : d;  // beyond 63 only the sticky bit remains either way
  const unsigned long long A = ((mx & kM52) | kH52) << 8;  // leading one at bit 60
  const unsigned long long B = ((my & kM52) | kH52) << 8;
  const unsigned long long Bs =
      d == 0 ? B : ((B >> d) | (unsigned long long)((B << (64 - d)) != 0));
  const bool sub = ((ah ^ bh) & 0x80000000u) != 0;
  const unsigned long long S = sub ? A - Bs : A + Bs;
  unsigned long long N;
  int e;
  if (S >> 61) {  // carry out of an addition
    N = (S >> 1) | (S & 1);
    e = (int)ex + 1;
  } else if (S >> 60) {
    N = S;
    e = (int)ex;
  } else {  // cancellation
    if (S == 0) return 0.0;  // x - x = +0 when rounding to nearest
    const int lz = __clzll((long long)S);  // >= 4
    N = S << (lz - 3);
    e = (int)ex - (lz - 3);
  }
  unsigned long long m = N >> 8;
  const unsigned guard = (unsigned)(N >> 7) & 1u;
  const unsigned sticky = (N & 0x7f) != 0;
  m += guard & (sticky | ((unsigned)m & 1u));
  return dbl((((unsigned long long)(e - 1) << 52) + m) | ((unsigned long long)sx << 32));
}

__device__ __forceinline__ double sub(double a, double b) {
  unsigned bl, bh;
  halves(b, bl, bh);
  return add(a, join(bl, bh ^ 0x80000000u));
}

// The integer v < 2^24 as a float, without the int-to-float conversion
// instruction: 2^23 + (v mod 2^23) by bit assembly, then 2^23 taken off again
// when v < 2^23.
__device__ __forceinline__ float u24_to_float(unsigned v) {
  const float f = __int_as_float(0x4b000000 | (v & 0x7fffffu));
  return (v >> 23) ? f : f - 8388608.0f;
}

// One quotient digit of K bits: q = floor(r 2^K / d), r <- r 2^K - q d, for
// 0 <= r < d, 2^52 <= d < 2^53.  ginv = 2^K / float(d >> 29) (FP32 reciprocal,
// relative error below 2^-23).  The estimate floor(float(r >> 29) * ginv) is
// within one of q: truncating r and d and the reciprocal's error each move
// r 2^K / d by less than 1/2 for K <= 22; the remainder, exact in 64-bit
// two's complement, then corrects it.
template <int K>
__device__ __forceinline__ unsigned div_digit(unsigned long long &r, unsigned long long d,
                                              float ginv) {
  const float fr = u24_to_float((unsigned)(r >> 29));
  // floor(fr * ginv) for a value below 2^23: round toward zero onto 2^23
  const float qf = __fmaf_rz(fr, ginv, 8388608.0f);
  unsigned q = (unsigned)__float_as_int(qf) & 0x7fffffu;
  long long rr = (long long)((r << K) - (unsigned long long)q * d);
  if (rr < 0) {
    q -= 1;
    rr += (long long)d;
  }
  if (rr >= (long long)d) {
    q += 1;
    rr -= (long long)d;
  }
  r = (unsigned long long)rr;
  return q;
}

// Rounded quotient of two moderate operands.
__device__ __forceinline__ double div_core(unsigned al, unsigned ah, unsigned bl, unsigned bh,
                                           unsigned ea, unsigned eb, unsigned sign) {
  unsigned long long x = ((unsigned long long)((ah & 0xfffffu) | 0x100000u) << 32) | al;
  const unsigned long long d = ((unsigned long long)((bh & 0xfffffu) | 0x100000u) << 32) | bl;
  const bool lt = x < d;
  const unsigned e1 = ea - eb + 1022u - (unsigned)lt;  // exponent field of the quotient - 1
  x <<= lt;  // d <= x < 2d: the quotient's leading bit is one
  unsigned long long r = x - d;
  const unsigned dh = (unsigned)(d >> 29);                           // in [2^23, 2^24)
  const float fd = __int_as_float(0x4b000000 | (dh & 0x7fffffu));  // == dh
  float inv;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(fd));
  // 52 quotient bits below the leading one plus the guard bit: 22 + 22 + 9
  const unsigned q1 = div_digit<22>(r, d, inv * 4194304.0f);
  const unsigned q2 = div_digit<22>(r, d, inv * 4194304.0f);
  const unsigned q3 = div_digit<9>(r, d, inv * 512.0f);
  const unsigned long long Q = (1ull << 53) | ((unsigned long long)q1 << 31) |
                               ((unsigned long long)q2 << 9) | q3;
  unsigned long long m = Q >> 1;
  const unsigned guard = (unsigned)Q & 1u;
  const unsigned sticky = r != 0;
  m += guard & (sticky | ((unsigned)m & 1u));
  return dbl((((unsigned long long)e1 << 52) + m) | ((unsigned long long)sign << 32));
}

// a / b
__device__ __forceinline__ double div(double a, double b) {
  unsigned al, ah, bl, bh;
  halves(a, al, ah);
  halves(b, bl, bh);
  const unsigned ea = expo(ah), eb = expo(bh);
  const unsigned sign = (ah ^ bh) & 0x80000000u;
  if (!(moderate(ea) & moderate(eb))) {
    // zero over a finite nonzero value: the zero of the quotient's sign
    if (is_zero(al, ah) & is_finite(bh) & !is_zero(bl, bh)) return join(0u, sign);
    return div_rare(a, b);
  }
  return div_core(al, ah, bl, bh, ea, eb, sign);
}

// ---------------------------------------------------------------------------
// Branch-free forms for optimistic evaluation: the integer path for every
// operand, with zeros handled by a select; `rare` collects whether any
// operand needs the hardware instruction, in which case the caller discards
// the results and evaluates the whole unit of work again with the FP64
// instructions.  A kernel then has no branch per operation.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double mul_opt(double a, double b, unsigned &rare) {
  unsigned al, ah, bl, bh;
  halves(a, al, ah);
  halves(b, bl, bh);
  // A zero times a finite value is a zero; (a zero) & finite(b) | (b zero) &
  // finite(a) is (either zero) & finite(a) & finite(b).  Fewer instructions
  // than testing each case apart (2D FP64 step 1.474 -> 1.451 ms).
  const unsigned ha = ah & 0x7fffffffu, hb = bh & 0x7fffffffu;
  const unsigned ea = ha >> 20, eb = hb >> 20;
  const unsigned sign = (ah ^ bh) & 0x80000000u;
  const bool zero = ((ha | al) == 0u) | ((hb | bl) == 0u);
  const bool fast = moderate(ea) & moderate(eb);
  rare |= (unsigned)!(fast | (zero & (ea != 0x7ffu) & (eb != 0x7ffu)));
  const double q = mul_core(al, ah, bl, bh, ea, eb, sign);
  return zero ? join(0u, sign) : q;
}

__device__ __forceinline__ double div_opt(double a, double b, unsigned &rare) {
  unsigned al, ah, bl, bh;
  halves(a, al, ah);
  halves(b, bl, bh);
  const unsigned ea = expo(ah), eb = expo(bh);
  const unsigned sign = (ah ^ bh) & 0x80000000u;
  const bool za = is_zero(al, ah);
  const bool fast = moderate(ea) & moderate(eb);
  const bool zero = za & is_finite(bh) & !is_zero(bl, bh);
  rare |= (unsigned)!(fast | zero);
  const double q = div_core(al, ah, bl, bh, ea, eb, sign);
  return za ? join(0u, sign) : q;
}

}  // namespace sf64
}  // namespace fvh
