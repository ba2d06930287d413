// dslash_df64.cu -- the Wilson-TM operator on FP64 fields in float-float
// arithmetic.
//
// GB300 executes FP64 fused multiply-adds at about 1/60 of its FP32 rate
// (measured: 0.60 T DFMA/s against 35 T FFMA/s), so the FP64 operator
// computed natively is bound by the FP64 pipe, not by HBM. This kernel keeps
// FP64 storage for the spinors (read and written as doubles) and computes on
// the FP32 pipes with unevaluated float pairs (hi + lo, ~47 significant bits):
//   * products: Dekker's exact product of the high words via FMA plus the two
//     cross terms (T. J. Dekker, Numer. Math. 18 (1971) 224);
//   * sums: Knuth's TwoSum (TAOCP vol. 2) into lazy accumulators (s, e) whose
//     error word collects the rounding errors in FP32; an accumulator is
//     renormalised (Fast2Sum) only when its value is consumed.
// Every operation uses the explicitly rounded intrinsics, so the compiler can
// neither contract nor reorder them. The double -> float-pair splits of the
// spinors (eight per hop and thread) use integer bit operations, because the
// hardware conversions run on the FP64 pipe; the pair -> double joins of the
// result (once per output component) use the FP64 pipe. The links come from a copy of the gauge field stored as
// float pairs, made once per field, with the boundary phase e^{i th/L}
// multiplied into the links of twisted directions (U' h for the forward hop,
// U'^+ h = e^{-i th/L} U^+ h for the backward one, as qcd_wilson.c applies it).
// The result differs from FP64 by a few 2^-46 relative, within the 1e-13
// per-site parity bar. Spinor values must lie in [2^-74, 2^127) in magnitude
// for the fast conversion; other values take an exact slower path, and
// doubles below 2^-1022 (denormals) count as zero.
#include "dslash_args.h"

namespace qg {

using namespace qgd;

struct F2 {  // h + l
  float h, l;
};
struct FA {  // accumulator: value s + e, not normalised
  float s, e;
};
struct CF {
  F2 re, im;
};
struct CA {
  FA re, im;
};

// out of line, so the common path does not carry its FP64 conversions
__device__ __noinline__ F2 split_slow(double d)
{
  F2 r;
  r.h = __double2float_rn(d);
  r.l = __double2float_rn(__dsub_rn(d, (double)r.h));
  return r;
}

// double -> float pair. In range (|d| in [2^-74, 2^127)) with integer bit
// operations: hi takes the leading 24 significand bits and lo the next 23
// (both truncated; the pair keeps 47 bits, relative error below 2^-46).
__device__ __forceinline__ F2 split_d(double d)
{
  const unsigned lo32 = (unsigned)__double2loint(d), hi32 = (unsigned)__double2hiint(d);
  const unsigned e = (hi32 >> 20) & 0x7ffu;
  F2 r;
  if (e - 949u <= 201u) {  // e in [949, 1150]
    // (hi32:lo32) << 3 holds the exponent's low 9 bits and the top 23
    // significand bits in float position; e - 896 = (e mod 512) - 384 here,
    // so one subtraction rebiases the exponent, and the sign goes back in
    const unsigned hb = (__funnelshift_l(lo32, hi32, 3) - (384u << 23)) | (hi32 & 0x80000000u);
    r.h = __uint_as_float(hb);
    // the 23 bits below hi as an exact integer-valued float, scaled by
    // 2^(e - 1069) with hi's sign: hi's sign and exponent field less 46
    const float f1 = __fsub_rn(__uint_as_float(0x4B000000u | ((lo32 >> 6) & 0x7fffffu)), 8388608.0f);
    r.l = __fmul_rn(f1, __uint_as_float((hb & 0xff800000u) - (46u << 23)));
  } else if (e == 0u) {
    r.h = __uint_as_float(hi32 & 0x80000000u);
    r.l = 0.0f;
  } else {
    r = split_slow(d);
  }
  return r;
}

// h + l -> double: two exact widenings and one FP64 add, rounded to nearest.
// The join runs once per output component, in the epilogue, where the FP64
// pipe has room; it replaced an integer bit-assembly of the double (~30
// instructions on the issue-bound side): 0.388 -> 0.372 ms per 24^3x48 apply.
__device__ __forceinline__ double join_d(F2 x) { return __dadd_rn((double)x.h, (double)x.l); }

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &q)
{
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  q = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ F2 neg(F2 a) { return F2{-a.h, -a.l}; }
// a + b, unnormalised
__device__ __forceinline__ F2 add(F2 a, F2 b)
{
  F2 r;
  float q;
  two_sum(a.h, b.h, r.h, q);
  r.l = __fadd_rn(q, __fadd_rn(a.l, b.l));
  return r;
}
__device__ __forceinline__ F2 fin(FA a)
{
  float s = __fadd_rn(a.s, a.e);
  return F2{s, __fsub_rn(a.e, __fsub_rn(s, a.s))};
}
// acc += a * b
__device__ __forceinline__ void mac(FA &acc, F2 a, F2 b)
{
  float p = __fmul_rn(a.h, b.h);
  float t = __fmaf_rn(a.h, b.h, -p);
  float s, q;
  two_sum(acc.s, p, s, q);
  float e = __fadd_rn(acc.e, __fadd_rn(t, q));
  e = __fmaf_rn(a.h, b.l, e);
  acc.e = __fmaf_rn(a.l, b.h, e);
  acc.s = s;
}
// acc += x
__device__ __forceinline__ void acc_add(FA &acc, F2 x)
{
  float s, q;
  two_sum(acc.s, x.h, s, q);
  acc.e = __fadd_rn(acc.e, __fadd_rn(q, x.l));
  acc.s = s;
}

// acc = a * b into an empty accumulator: no error-free sum needed
__device__ __forceinline__ FA mac0(F2 a, F2 b)
{
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  return FA{p, __fmaf_rn(a.l, b.h, e)};
}
// acc += x for an unnormalised x
__device__ __forceinline__ void acc_add_fa(FA &acc, FA x)
{
  float s, q;
  two_sum(acc.s, x.s, s, q);
  acc.e = __fadd_rn(acc.e, __fadd_rn(q, x.e));
  acc.s = s;
}
__device__ __forceinline__ FA fneg(FA a) { return FA{-a.s, -a.e}; }
struct CFA {  // complex accumulator value
  FA re, im;
};
// z -> (i z if ifl) then negated if ng
__device__ __forceinline__ CFA coefa(CFA z, bool ifl, bool ng)
{
  CFA r = ifl ? CFA{fneg(z.im), z.re} : z;
  return ng ? CFA{fneg(r.re), fneg(r.im)} : r;
}
__device__ __forceinline__ void cacc_fa(CA &acc, CFA x)
{
  acc_add_fa(acc.re, x.re);
  acc_add_fa(acc.im, x.im);
}

__device__ __forceinline__ CF cadd(CF a, CF b) { return CF{add(a.re, b.re), add(a.im, b.im)}; }
__device__ __forceinline__ CF cneg(CF a) { return CF{neg(a.re), neg(a.im)}; }
__device__ __forceinline__ CF ci(CF a) { return CF{neg(a.im), a.re}; }  // i a
__device__ __forceinline__ void cacc(CA &acc, CF x)
{
  acc_add(acc.re, x.re);
  acc_add(acc.im, x.im);
}

__device__ __forceinline__ CF load_sp(const double2 *base, int64_t stride, int y, int k)
{
  double2 v = __ldg(base + (int64_t)k * stride + y);
  return CF{split_d(v.x), split_d(v.y)};
}
__device__ __forceinline__ CF load_link(const float4 *base, int64_t stride, int y, int mu, int k)
{
  float4 v = __ldg(base + ((int64_t)mu * 9 + k) * stride + y);
  return CF{F2{v.x, v.y}, F2{v.z, v.w}};
}

// z -> (i z if ifl) then negated if ng; ifl and ng are warp-uniform
__device__ __forceinline__ CF coef(CF z, bool ifl, bool ng)
{
  CF r = ifl ? CF{neg(z.im), z.re} : z;
  return ng ? cneg(r) : r;
}

// Thread layout: a block of 96 * kFFGroups threads covers 32 * kFFGroups
// sites as groups of three warps; warp w of a group owns colour row i = w for its 32 sites and
// the four accumulators (spins 0..3) of that colour. Per hop each warp
// projects the neighbour spinor of its colour, the three warps share the
// half spinors through shared memory, and each warp multiplies its link row.
// The eight hops are unrolled (directions and signs compile-time); with S
// the projector sign,
// (1 + S g_mu) in the chiral basis is
//   h0 = p0 + c0 p_b0, h1 = p1 + c1 p_b1            (upper half)
//   b0 = 2 (mu 0,3) or 3 (mu 1,2), b1 = 5 - b0, c = +-1 (mu even) or +-i (odd)
//   c0 = -S ; c1 = -S (mu 0,1) or +S (mu 2,3)
// and the lower half rebuilt from v = U h:
//   r2 = cA v_jA, r3 = cB v_jB ; jA = 1 for mu 1,2 else 0, jB = 1 - jA
//   cA = -S (mu 0) else +S ; cB = +S (mu 1) else -S ; times i for odd mu
// (qcd_wilson.h:17-387).
//
// Each group of three warps synchronises on its own named barrier (ids 1..4,
// 96 threads), so the four groups of a block never wait for one another.
//
// The spin projections (adds of two spinor components) run in native FP64
// straight after the loads, and only the half spinor is split into float
// pairs: two double -> pair conversions per half-spinor component instead of
// four, for four FP64 adds per hop and warp. The FP64 pipe is far too slow
// for the operator's multiply-adds, but it is otherwise idle here, and the
// conversions it saves are integer work on the issue-bound FP32 side.
// Each thread's four spinor components of the next hop are copied into
// shared memory with cp.async while the current hop computes (two stages,
// 128 bytes per thread), so the loads hold no registers.
// (Measured on GB300, 24^3x48: 0.505 -> 0.440 ms per apply; unrolled hops
// and the 47-bit split: 0.425 ms; staged loads: 0.417 ms. Moving more --
// the epilogue, whole hops, or whole site groups -- onto the FP64 pipe was
// slower.)
// Block geometry, measured on GB300 at 24^3x48 (ms per apply, groups x
// blocks per SM: registers): 4 x 3: 56 (spills) 0.372; 4 x 2: 80 0.379;
// 3 x 4: 56 (spills) 0.376; 3 x 3: 72 0.364; 5 x 2: 64 0.391; 6 x 2: 56
// 0.393; 2 x 5: 64 0.409; 2 x 6: 56 0.434; 1 x 10: 64 0.397; 1 x 12: 56
// 0.395. The group barrier's id is a register, so ptxas reserves all 16
// named barriers per block of more than one group, and ncu reports the
// barriers as a limit of four resident blocks per SM. Immediate ids (a
// warp-uniform switch over the groups) lift that limit but cost every form
// 4-11 % (3 x 3: 0.406 ms; the branches sit in the unrolled hop loop).
constexpr int kFFGroups = 3;       // groups of three warps (32 sites) per block
constexpr int kFFMinBlocks = 3;    // resident blocks per SM the registers are sized for
constexpr int kFFSites = 32 * kFFGroups;

__device__ __forceinline__ void group_bar(int grp) { asm volatile("bar.sync %0, 96;" ::"r"(grp + 1) : "memory"); }

// site of output index e; EO: the site of parity eo_par among full indices
// 2e, 2e + 1 (even t extent)
template <bool EO>
__device__ __forceinline__ int ff_site(const DArgs &a, int e, bool act, int c[4])
{
  c[0] = c[1] = c[2] = c[3] = 0;
  if (!act) return e;
  if (EO) {
    coords(a.geo, 2 * e, c);
    const int b = (a.eo_par ^ c[1] ^ c[2] ^ c[3]) & 1;
    c[0] += b;
    return 2 * e + b;
  }
  coords(a.geo, e, c);
  return e;
}

// neighbour of x across direction mu (backwards if back), periodic
__device__ __forceinline__ int ff_nb(const DArgs &a, int x, const int c[4], int mu, bool back)
{
  const int cm = mu == 0 ? c[0] : mu == 1 ? c[1] : mu == 2 ? c[2] : c[3];
  const int Lm = a.geo.L[mu], st = a.geo.st[mu];
  if (back) return cm == 0 ? x + (Lm - 1) * st : x - st;
  return cm == Lm - 1 ? x - (Lm - 1) * st : x + st;
}

// sign flip by integer operation (keeps the FP64 pipe for arithmetic)
__device__ __forceinline__ double dflip(double v, bool ng)
{
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)ng << 63));
}
// z -> (i z if ifl) then negated if ng
__device__ __forceinline__ double2 dcoef(double2 z, bool ifl, bool ng)
{
  return make_double2(dflip(ifl ? z.y : z.x, ng ^ ifl), dflip(ifl ? z.x : z.y, ng));
}
__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// 16-byte asynchronous copy global -> shared (cached in L1: neighbour
// spinors are read by eight sites), and its group fences
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// staging of the four spinor components a thread projects per hop: two
// hops in flight, [stage][component][thread]
constexpr int kFFThreads = 96 * kFFGroups;
constexpr size_t kFFStageBytes = 2 * 4 * kFFThreads * sizeof(double2);

// the float-float operator for one group's 32 sites; returns the thread's |out|^2.
// AOS: in and out in the host layout (site-major, 12 double2 per site)
template <bool DAG, bool EO, bool AOS>
__device__ __forceinline__ double group_ff(const DArgs &a, int grp, int col, int lane, int e, bool act, int x,
                                           const int c[4], CF (*hs)[2][3][32], double2 *stage)
{
  const double2 *sp = (const double2 *)a.in;
  const float4 *gf = (const float4 *)a.gauge;
  constexpr int SF = DAG ? +1 : -1;
  const int tid = threadIdx.x;
  // the four components hop dd projects, copied into stage st
  auto issue = [&](int dd, int st) {
    if (act) {
      const int mu2 = dd >> 1, y2 = ff_nb(a, x, c, mu2, dd & 1), ys2 = EO ? (y2 >> 1) : y2;
      const int b02 = (mu2 == 0 || mu2 == 3) ? 2 : 3;
      const int comp[4] = {col, 3 + col, 3 * b02 + col, 3 * (5 - b02) + col};
#pragma unroll
      for (int i = 0; i < 4; i++)
        cp_async16(stage + (st * 4 + i) * kFFThreads + tid,
                   AOS ? sp + (int64_t)ys2 * 12 + comp[i] : sp + (int64_t)comp[i] * a.stride + ys2);
    }
    cp_async_commit();
  };
  issue(0, 0);
  CA acc[4];
#pragma unroll
  for (int s = 0; s < 4; s++) acc[s] = CA{{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
  for (int d = 0; d < 8; d++) {
    // hop d + 1's components start to arrive while hop d computes
    if (d < 7) {
      issue(d + 1, (d + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const int mu = d >> 1;
    const bool back = d & 1;
    const int S = back ? -SF : SF;
    const int y = act ? ff_nb(a, x, c, mu, back) : x;
    const int ly = back ? y : x;
    const bool odd = mu & 1;
    const bool neg0 = S > 0, neg1 = mu < 2 ? S > 0 : S < 0;
    double2 d0 = make_double2(0.0, 0.0), d1 = d0;
    if (act) {
      const double2 *b = stage + (d & 1) * 4 * kFFThreads + tid;  // this thread's own copies
      const double2 p0 = b[0], p1 = b[kFFThreads], q0 = b[2 * kFFThreads], q1 = b[3 * kFFThreads];
      d0 = dadd(p0, dcoef(q0, odd, neg0));
      d1 = dadd(p1, dcoef(q1, odd, neg1));
    }
    hs[grp][0][col][lane] = CF{split_d(d0.x), split_d(d0.y)};
    hs[grp][1][col][lane] = CF{split_d(d1.x), split_d(d1.y)};
    group_bar(grp);
    CA u0, u1;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      CF g0 = hs[grp][0][k][lane], g1 = hs[grp][1][k][lane];
      // forward: U[col][k]; backward: conj(U[k][col])
      CF wl = act ? load_link(gf, a.gstride, ly, mu, back ? 3 * k + col : 3 * col + k) : CF{{0.f, 0.f}, {0.f, 0.f}};
      F2 wr = wl.re, wi = back ? neg(wl.im) : wl.im, mwi = neg(wi);
      if (k == 0) {
        u0.re = mac0(wr, g0.re);
        u0.im = mac0(wr, g0.im);
        u1.re = mac0(wr, g1.re);
        u1.im = mac0(wr, g1.im);
      } else {
        mac(u0.re, wr, g0.re);
        mac(u0.im, wr, g0.im);
        mac(u1.re, wr, g1.re);
        mac(u1.im, wr, g1.im);
      }
      mac(u0.re, mwi, g0.im);
      mac(u0.im, wi, g0.re);
      mac(u1.re, mwi, g1.im);
      mac(u1.im, wi, g1.re);
    }
    // the products enter the spinor accumulators unnormalised (the first
    // hop assigns them)
    const CFA v0{u0.re, u0.im}, v1{u1.re, u1.im};
    const bool jA = (mu == 1 || mu == 2);
    const bool negA = mu == 0 ? S > 0 : S < 0, negB = mu == 1 ? S < 0 : S > 0;
    const CFA l2 = coefa(jA ? v1 : v0, odd, negA), l3 = coefa(jA ? v0 : v1, odd, negB);
    if (d == 0) {
      acc[0] = CA{v0.re, v0.im};
      acc[1] = CA{v1.re, v1.im};
      acc[2] = CA{l2.re, l2.im};
      acc[3] = CA{l3.re, l3.im};
    } else {
      cacc_fa(acc[0], v0);
      cacc_fa(acc[1], v1);
      cacc_fa(acc[2], l2);
      cacc_fa(acc[3], l3);
    }
    group_bar(grp);  // hs is rewritten by the next hop
  }
  if (!act) return 0.0;
  double n2 = 0.0;
  if (EO) {
    double2 *out = (double2 *)a.out;
    const F2 mp4{a.mp4_h, a.mp4_l}, tm{a.tm_h, a.tm_l}, ch{a.ch_h, a.ch_l};
    const F2 air{a.ai_r_h, a.ai_r_l}, aii{a.ai_i_h, a.ai_i_l};
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const int k = 3 * s + col;
      F2 hr = fin(acc[s].re), hi = fin(acc[s].im);
      if (a.ainv) {  // (ai_r + i ai_i g5) H in
        const F2 gi = s < 2 ? aii : neg(aii);
        FA re{0.f, 0.f}, im{0.f, 0.f};
        mac(re, air, hr);
        mac(re, neg(gi), hi);
        mac(im, air, hi);
        mac(im, gi, hr);
        hr = fin(re);
        hi = fin(im);
      }
      FA re{0.f, 0.f}, im{0.f, 0.f};
      mac(re, ch, hr);
      mac(im, ch, hi);
      if (a.zmode) {
        const CF zv = load_sp((const double2 *)a.z, a.stride, e, k);
        if (a.zmode == 2) {  // + (m+4) z + i tm g5 z
          const F2 g5tm = s < 2 ? tm : neg(tm);
          mac(re, mp4, zv.re);
          mac(re, neg(g5tm), zv.im);
          mac(im, mp4, zv.im);
          mac(im, g5tm, zv.re);
        } else {
          acc_add(re, zv.re);
          acc_add(im, zv.im);
        }
      }
      const double vr = join_d(fin(re)), vi = join_d(fin(im));
      out[(int64_t)k * a.stride + e] = make_double2(vr, vi);
      n2 += vr * vr + vi * vi;
    }
  } else {
    double2 *out = (double2 *)a.out;
    const F2 mp4{a.mp4_h, a.mp4_l}, tm{a.tm_h, a.tm_l};
#pragma unroll
    for (int s = 0; s < 4; s++) {
      // (m+4) psi + i tm g5 psi - acc/2 for component (spin s, colour col)
      const int k = 3 * s + col;
      CF sv = AOS ? load_sp(sp + (int64_t)x * 12, 1, 0, k) : load_sp(sp, a.stride, x, k);
      F2 g5tm = s < 2 ? tm : neg(tm), mg5tm = neg(g5tm);
      F2 ar = fin(acc[s].re), ai = fin(acc[s].im);
      FA re{__fmul_rn(ar.h, -0.5f), __fmul_rn(ar.l, -0.5f)};
      FA im{__fmul_rn(ai.h, -0.5f), __fmul_rn(ai.l, -0.5f)};
      mac(re, mp4, sv.re);
      mac(re, mg5tm, sv.im);
      mac(im, mp4, sv.im);
      mac(im, g5tm, sv.re);
      F2 dr = fin(re), di = fin(im);
      if (a.op_q) {  // i g5: spins 0,1 times i, spins 2,3 times -i
        F2 t = dr;
        if (s < 2) {
          dr = neg(di);
          di = t;
        } else {
          dr = di;
          di = neg(t);
        }
      }
      double vr = join_d(dr), vi = join_d(di);
      out[AOS ? (int64_t)x * 12 + k : (int64_t)k * a.stride + x] = make_double2(vr, vi);
      n2 += vr * vr + vi * vi;
    }
  }
  return n2;
}

// EO: even/odd kernel on half fields (sites of parity a.eo_par; neighbours
// read at (full index) >> 1) with the epilogue ch * [A^{-1}] H in + {z | A z}
template <bool DAG, bool EO, bool AOS>
__global__ void __launch_bounds__(kFFThreads, kFFMinBlocks) k_wilson_ff(const DArgs a)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int grp = w / 3, col = w - 3 * grp;
  const int e = a.x0 + blockIdx.x * kFFSites + grp * 32 + lane;  // output index
  const bool act = e < a.V;
  __shared__ CF hs[kFFGroups][2][3][32];
  int c[4];
  const int x = ff_site<EO>(a, e, act, c);
  extern __shared__ double2 ff_stage[];
  const double n2 = group_ff<DAG, EO, AOS>(a, grp, col, lane, e, act, x, c, hs, ff_stage);
  if (a.partials) block_partial_cg(n2, a);
}

// ------------------------------------------------------ float-pair links
__global__ void k_gauge_to_ff(float4 *dst, int64_t dstride, const double2 *src, int64_t sstride, int64_t V,
                              DArgs phases)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V * 4) return;
  int64_t x = i >> 2;
  int mu = (int)(i & 3);
  bool tw = (phases.twist_mask >> mu) & 1;
  double pr = phases.phr[mu], pi = phases.phi[mu];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    double2 u = src[((int64_t)mu * 9 + k) * sstride + x];
    double re = u.x, im = u.y;
    if (tw) {
      re = u.x * pr - u.y * pi;
      im = u.x * pi + u.y * pr;
    }
    float rh = __double2float_rn(re), ih = __double2float_rn(im);
    dst[((int64_t)mu * 9 + k) * dstride + x] =
        make_float4(rh, __double2float_rn(re - (double)rh), ih, __double2float_rn(im - (double)ih));
  }
}

bool gauge_to_ff(qcdgpu_gauge d, qcdgpu_gauge s)
{
  if (s->prec != QCDGPU_F64) {
    set_error("float-pair links are made from an FP64 gauge field");
    return false;
  }
  DArgs ph;
  ph.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    ph.phr[mu] = 1.0;
    ph.phi[mu] = 0.0;
    if (s->theta[mu] != 0.0) {
      ph.twist_mask |= 1 << mu;
      ph.phr[mu] = cos(s->theta[mu] / (double)s->L[mu]);
      ph.phi[mu] = sin(s->theta[mu] / (double)s->L[mu]);
    }
  }
  d->recon = 18;
  for (int i = 0; i < 4; i++) d->theta[i] = s->theta[i];
  unsigned gr = (unsigned)((s->V * 4 + 127) / 128);
  k_gauge_to_ff<<<gr, 128, 0, stream()>>>((float4 *)d->data, d->stride, (const double2 *)s->data, s->stride, s->V, ph);
  return QG_LAUNCHED("gauge_to_ff");
}

// the staging buffer is dynamic shared memory (36 KB for three groups; the
// attribute lifts the 48 KB default limit for larger blocks): opted in once
// per instantiation
template <bool D, bool E, bool A = false>
static void launch_ff(const DArgs &a, unsigned grid)
{
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_wilson_ff<D, E, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFFStageBytes);
    attr = true;
  }
  k_wilson_ff<D, E, A><<<grid, kFFThreads, kFFStageBytes, stream()>>>(a);
}

bool dslash_df64(const DArgs &a, bool dag, bool eo)
{
  unsigned grid = (unsigned)((a.V - a.x0 + kFFSites - 1) / kFFSites);
  if (eo) {
    if (dag) launch_ff<true, true>(a, grid);
    else launch_ff<false, true>(a, grid);
  } else if (a.aos) {
    if (dag) launch_ff<true, false, true>(a, grid);
    else launch_ff<false, false, true>(a, grid);
  } else {
    if (dag) launch_ff<true, false>(a, grid);
    else launch_ff<false, false>(a, grid);
  }
  return QG_LAUNCHED("wilson_df64");
}

}  // namespace qg
