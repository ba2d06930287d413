// dslash_df64.cu -- the operator on FP64 fields in float-float arithmetic.
//
// GB300 executes FP64 fused multiply-adds at about 1/60 of its FP32 rate
// (measured: 0.60 T DFMA/s against 35 T FFMA/s), so an FP64 Wilson operator
// computed natively is bound by the FP64 pipe, not by HBM. This
// instantiation keeps FP64 storage (fields are read and written as doubles)
// but computes with unevaluated pairs of floats (hi + lo, ~48 significant
// bits) on the FP32 pipes:
//   * sum: Knuth's TwoSum of the high words plus the low words, then
//     renormalised (Fast2Sum);
//   * product: Dekker's exact product of the high words via FMA, plus the two
//     cross terms, renormalised.
// (T. J. Dekker, Numer. Math. 18 (1971) 224; D. E. Knuth, TAOCP vol. 2.)
// Every operation uses the explicitly rounded intrinsics so the compiler can
// neither contract nor reorder them. Conversions between double and the
// float pair are done with integer operations on the bit patterns (the
// hardware conversions run on the FP64 pipe too). Values whose magnitude lies
// outside [2^-74, 2^127) take a slower exact path; doubles below 2^-1022
// (denormals) count as zero. The result differs from FP64 by a few 2^-47
// relative, inside the 1e-13 per-site parity bar.
#include "wilson_kernel.cuh"

namespace qg {

__device__ __forceinline__ float f_from_bits(unsigned b) { return __uint_as_float(b); }

struct FF {
  float h, l;
  FF() = default;
  __device__ __forceinline__ FF(float hi, float lo) : h(hi), l(lo) {}

  // double -> (hi, lo): hi = the leading 24 significand bits (truncated),
  // lo = the next 29 bits rounded to 24, both carrying the sign of d
  __device__ __forceinline__ explicit FF(double d)
  {
    unsigned lo32 = (unsigned)__double2loint(d), hi32 = (unsigned)__double2hiint(d);
    unsigned e = (hi32 >> 20) & 0x7ffu;
    unsigned sign = hi32 & 0x80000000u;
    if (e >= 949u && e <= 1150u) {
      h = f_from_bits(sign | ((e - 896u) << 23) | ((hi32 & 0xfffffu) << 3) | (lo32 >> 29));
      unsigned r = lo32 & 0x1fffffffu;  // value r * 2^(e - 1075)
      // r as a float: two exact 23-bit pieces joined by one rounding FMA
      float f1 = __fsub_rn(f_from_bits(0x4B000000u | (r >> 6)), 8388608.0f);
      float f2 = __fsub_rn(f_from_bits(0x4B000000u | (r & 63u)), 8388608.0f);
      float rf = __fmaf_rn(f1, 64.0f, f2);
      float lo = __fmul_rn(rf, f_from_bits((e - 948u) << 23));
      l = __uint_as_float(__float_as_uint(lo) ^ sign);
    } else if (e == 0u) {
      h = f_from_bits(sign);
      l = 0.0f;
    } else {
      h = __double2float_rn(d);
      l = __double2float_rn(__dsub_rn(d, (double)h));
    }
  }

  // (hi, lo) -> double by integer arithmetic on the significands; lo's bits
  // below the double's last place are truncated (|lo| <= ulp(hi) here)
  __device__ __forceinline__ explicit operator double() const
  {
    unsigned hb = __float_as_uint(h), lb = __float_as_uint(l);
    unsigned eh = (hb >> 23) & 0xffu;
    if ((hb & 0x7fffffffu) == 0u) return (double)l;  // zero hi: lo is the value
    if (eh == 0u || eh == 255u) return __dadd_rn((double)h, (double)l);
    unsigned long long M = (unsigned long long)((hb & 0x7fffffu) | 0x800000u) << 29;
    unsigned el = (lb >> 23) & 0xffu;
    if (el != 0u && el != 255u) {
      unsigned long long ml = (unsigned long long)((lb & 0x7fffffu) | 0x800000u);
      int sh = 29 - ((int)eh - (int)el);
      unsigned long long add = sh >= 0 ? (ml << sh) : (sh > -60 ? (ml >> (-sh)) : 0ull);
      if ((hb ^ lb) & 0x80000000u) M -= add;
      else M += add;
    }
    int e = (int)eh + 896;
    if (M >= (1ull << 53)) {
      M >>= 1;
      e += 1;
    } else if (M < (1ull << 52)) {
      if (M == 0ull) return 0.0;
      int z = __clzll((long long)M) - 11;
      M <<= z;
      e -= z;
    }
    return __longlong_as_double((long long)(((unsigned long long)(hb >> 31) << 63) |
                                            ((unsigned long long)e << 52) | (M & ((1ull << 52) - 1))));
  }
};

__device__ __forceinline__ FF fast2sum(float a, float b)
{
  float s = __fadd_rn(a, b);
  return FF(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ FF operator+(FF a, FF b)
{
  float s = __fadd_rn(a.h, b.h);
  float bb = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return fast2sum(s, e);
}
__device__ __forceinline__ FF operator-(FF a) { return FF(-a.h, -a.l); }
__device__ __forceinline__ FF operator-(FF a, FF b) { return a + (-b); }
__device__ __forceinline__ FF operator*(FF a, FF b)
{
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast2sum(p, e);
}

template <>
struct Scalar<FF> {
  __device__ __forceinline__ static FF get(double, float h, float l) { return FF(h, l); }
};

template <bool DAG>
static bool launch_ff(const DArgs &a)
{
  unsigned grid = (unsigned)((a.V + 127) / 128);
  // all 9 link entries are read: rebuilding row 2 costs more float-float
  // arithmetic than the extra 192 bytes per site cost in bandwidth
  k_wilson<DAG, QCDGPU_F64, QCDGPU_F64, 18, FF><<<grid, 128, 0, stream()>>>(a);
  return QG_LAUNCHED("wilson_df64");
}

bool dslash_df64(const DArgs &a, bool dag, int recon)
{
  (void)recon;
  return dag ? launch_ff<true>(a) : launch_ff<false>(a);
}

}  // namespace qg
