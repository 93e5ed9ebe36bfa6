// F64X: double-precision BGK collision computed without the FP64 pipe.
//
// GB300's FP64 units run at about 1/60 of its FP32 rate, and double <-> float
// conversions go through them too, so a collision written in `double` is
// compute-bound far below the HBM roofline.  This path keeps the populations
// in FP64 memory (the reference's Pdf buffers) but:
//
//  * splits each loaded double into an unevaluated float pair (h, l) with
//    integer operations only: h is the double truncated to 24 significant
//    bits, l the next 23 bits (|f - (h + l)| < 2^-47 |f|);
//  * evaluates rho, j = sum c f, u, the equilibrium and the BGK/Guo update in
//    double-float arithmetic built from the error-free transformations
//    TwoSum (Knuth), Fast2Sum (Dekker 1971) and the FMA two-product, as used
//    in double-double libraries (Hida, Li & Bailey, "Library for double-double
//    and quad-double arithmetic", 2001);
//  * rebuilds the 64-bit pattern of the result with integer operations.
//
// The fast path covers positive populations in [2^-80, 1), the only values a
// physical state holds.  A cell whose inputs or results fall outside that
// range is recomputed with the exact IEEE double collision, so any state is
// handled; the fast path's results agree with the exact path to about
// 2^-46 relative per step.
#pragma once

#include <cstdint>
#include <cstring>
#ifndef __CUDA_ARCH__
#include <cfenv>
#include <cmath>
#endif

#include "lbm_physics.cuh"

namespace lbm {
namespace x64 {

// ------------------------------------------------------------ primitives
__host__ __device__ __forceinline__ uint32_t fbits(float f)
{
#ifdef __CUDA_ARCH__
   return __float_as_uint(f);
#else
   uint32_t u;
   std::memcpy(&u, &f, 4);
   return u;
#endif
}

__host__ __device__ __forceinline__ float bitsf(uint32_t u)
{
#ifdef __CUDA_ARCH__
   return __uint_as_float(u);
#else
   float f;
   std::memcpy(&f, &u, 4);
   return f;
#endif
}

__host__ __device__ __forceinline__ float ffma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
   return __fmaf_rn(a, b, c);
#else
   return std::fmaf(a, b, c);
#endif
}

// Plain rounded-to-nearest FP32 ops that the compiler must not contract.
__host__ __device__ __forceinline__ float fadd(float a, float b)
{
#ifdef __CUDA_ARCH__
   return __fadd_rn(a, b);
#else
   volatile float r = a + b;
   return r;
#endif
}

__host__ __device__ __forceinline__ float fsub(float a, float b)
{
#ifdef __CUDA_ARCH__
   return __fsub_rn(a, b);
#else
   volatile float r = a - b;
   return r;
#endif
}

__host__ __device__ __forceinline__ float fmul(float a, float b)
{
#ifdef __CUDA_ARCH__
   return __fmul_rn(a, b);
#else
   volatile float r = a * b;
   return r;
#endif
}

// a + b rounded toward zero.
__host__ __device__ __forceinline__ float fadd_rz(float a, float b)
{
#ifdef __CUDA_ARCH__
   return __fadd_rz(a, b);
#else
   const int old = std::fegetround();
   std::fesetround(FE_TOWARDZERO);
   volatile float va = a, vb = b;
   volatile float r = va + vb;
   std::fesetround(old);
   return r;
#endif
}

__host__ __device__ __forceinline__ float frcp(float a)
{
#ifdef __CUDA_ARCH__
   return __frcp_rn(a);
#else
   volatile float r = 1.0f / a;
   return r;
#endif
}

// Low 32 bits of ((hi:lo) << n), 0 <= n < 32.
__host__ __device__ __forceinline__ uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t n)
{
#ifdef __CUDA_ARCH__
   return __funnelshift_l(lo, hi, n);
#else
   const uint64_t v = ((uint64_t)hi << 32) | lo;
   return (uint32_t)((v << n) >> 32);
#endif
}

// ------------------------------------------------------------ double-float
struct df {
   float h, l;
};

// TwoSum (Knuth): s + e == a + b exactly.
__host__ __device__ __forceinline__ df two_sum(float a, float b)
{
   const float s = fadd(a, b);
   const float bb = fsub(s, a);
   const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
   return {s, e};
}

// Fast2Sum (Dekker): exact when |a| >= |b|.
__host__ __device__ __forceinline__ df fast_two_sum(float a, float b)
{
   const float s = fadd(a, b);
   return {s, fsub(b, fsub(s, a))};
}

__host__ __device__ __forceinline__ df df_add(df a, df b)
{
   const df s = two_sum(a.h, b.h);
   return fast_two_sum(s.h, fadd(s.l, fadd(a.l, b.l)));
}

// a + b when |a.h| >= |b.h| is known.
__host__ __device__ __forceinline__ df df_add_fast(df a, df b)
{
   const df s = fast_two_sum(a.h, b.h);
   return fast_two_sum(s.h, fadd(s.l, fadd(a.l, b.l)));
}

__host__ __device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }

__host__ __device__ __forceinline__ df df_mul(df a, df b)
{
   const float p = fmul(a.h, b.h);
   float e = ffma(a.h, b.h, -p);
   e = ffma(a.h, b.l, e);
   e = ffma(a.l, b.h, e);
   return fast_two_sum(p, e);
}

// Product left unnormalised (p + e with |e| <= ~ulp(p)); saves the final Fast2Sum.
__host__ __device__ __forceinline__ df df_mul_u(df a, df b)
{
   const float p = fmul(a.h, b.h);
   float e = ffma(a.h, b.h, -p);
   e = ffma(a.h, b.l, e);
   e = ffma(a.l, b.h, e);
   return {p, e};
}

__host__ __device__ __forceinline__ df df_sqr_u(df a)
{
   const float p = fmul(a.h, a.h);
   float e = ffma(a.h, a.h, -p);
   e = ffma(2.0f * a.h, a.l, e);
   return {p, e};
}

// Exact split of a host double constant into a float pair.
__host__ __device__ __forceinline__ df df_from_double(double d)
{
   const float h = (float)d;
   return {h, (float)(d - (double)h)};
}

// ------------------------------------------------ double <-> float pair
// Fast-path range of the double bit patterns: positive, 2^-80 <= f < 1.
constexpr uint32_t kHiMin = (uint32_t)(1023 - 80) << 20;   // high word of 2^-80
constexpr uint32_t kHiMax = (uint32_t)1023 << 20;          // high word of 1.0 (excluded)

// Split a double (given as its 64-bit pattern, in range) into (h, l).
//   t  = bits 59..28 of the pattern: the low 8 exponent bits above the top
//        23 mantissa bits; adding 2^30 re-biases exponent 1023 to 127
//        (E - 896) within the 8-bit field, valid for E in [897, 1150].
//   l  = next 23 mantissa bits, built as a float with exponent e(h) - 23 and
//        its implicit 1 subtracted (exact by Sterbenz).
__host__ __device__ __forceinline__ df split(uint64_t bits)
{
   const uint32_t lo = (uint32_t)bits, hi = (uint32_t)(bits >> 32);
   const uint32_t t = funnel_l(lo, hi, 3);
   const uint32_t hb = ((t + 0x40000000u) & 0x7FFFFFFFu) | (hi & 0x80000000u);
   const uint32_t a = hb - (23u << 23);
   const uint32_t xb = (a & 0xFF800000u) | ((lo >> 6) & 0x007FFFFFu);
   const uint32_t mb = a & 0xFF800000u;
   return {bitsf(hb), fsub(bitsf(xb), bitsf(mb))};
}

// Rebuild the double pattern of h + l (positive, result in [2^-80, 1)):
//   S   = h + l rounded toward zero (so the remainder E >= 0 stays inside
//         S's binade), E = the remainder;
//   the pattern of S as a double, plus E counted in units of 2^7 double
//   ulps of S, rounded with the 1.5*2^23 magic constant.
__host__ __device__ __forceinline__ uint64_t join(df v)
{
   const float S = fadd_rz(v.h, v.l);
   const float E = fsub(v.l, fsub(S, v.h));
   const uint32_t sb = fbits(S);
   const float scale = bitsf(0x95800000u - (sb & 0x7F800000u));  // 2^(45 - e(S))
   const float y = ffma(E, scale, 12582912.0f);
   const int32_t ei = (int32_t)(fbits(y) - 0x4B400000u);
   const uint64_t d0 = ((uint64_t)sb << 29) + ((uint64_t)0x38000000u << 32);
   return d0 + (uint64_t)((int64_t)ei * 128);
}

__host__ __device__ __forceinline__ bool in_range(uint64_t bits)
{
   const uint32_t hi = (uint32_t)(bits >> 32);
   return hi >= kHiMin && hi < kHiMax;
}

// Result check before join: positive and inside the fast range.
__host__ __device__ __forceinline__ bool out_ok(df v)
{
   const float s = fadd(v.h, v.l);
   return s >= 8.271806125530277e-25f /* 2^-80 */ && s < 0.99999994f;
}

__host__ __device__ __forceinline__ double as_double(uint64_t b)
{
   double d;
#ifdef __CUDA_ARCH__
   d = __longlong_as_double((long long)b);
#else
   std::memcpy(&d, &b, 8);
#endif
   return d;
}

__host__ __device__ __forceinline__ uint64_t double_bits(double d)
{
#ifdef __CUDA_ARCH__
   return (uint64_t)__double_as_longlong(d);
#else
   uint64_t b;
   std::memcpy(&b, &d, 8);
   return b;
#endif
}

// Per-launch constants of the double-float collision.
struct Consts {
   df om1;        // 1 - omega
   df omega;
   df ow[4];      // omega * w for |c|^2 = 0, 1, 2, 3
   df F[3];       // uniform body force
   float om2;     // 1 - omega/2 (multiplies only the small forcing terms)
};

}  // namespace x64

// The fast-path collision on one cell.  bits[] holds the Q input patterns in
// direction order and receives the Q output patterns.  Returns false (leaving
// bits[] untouched) when the cell must take the exact path.
template <int Q>
__host__ __device__ __forceinline__ bool collide_f64x_fast(uint64_t (&bits)[Q], const x64::Consts& k,
                                                          int compat)
{
   using namespace x64;
   uint32_t hmin = 0xFFFFFFFFu, hmax = 0;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const uint32_t hi = (uint32_t)(bits[s] >> 32);
      hmin = hmin < hi ? hmin : hi;
      hmax = hmax > hi ? hmax : hi;
   }
   if (hmin < kHiMin || hmax >= kHiMax) return false;

   df f[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) f[s] = split(bits[s]);

   // rho: start from the rest population (the largest) so every partial sum
   // dominates the next term and Fast2Sum is exact.
   constexpr int R = lat_rest(Q);
   df rho = f[R];
#pragma unroll
   for (int s = 0; s < Q; s++) {
      if (s == R) continue;
      const df t = fast_two_sum(rho.h, f[s].h);
      rho = {t.h, fadd(rho.l, fadd(t.l, f[s].l))};
   }
   rho = fast_two_sum(rho.h, rho.l);

   // j = sum c f per component (TwoSum: partial sums may cancel).
   df j[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
   for (int d = 0; d < 3; d++) {
      bool first = true;
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const int c = lat_c(Q, s, d);
         if (c == 0) continue;
         const df term = c > 0 ? f[s] : df_neg(f[s]);
         if (first) {
            j[d] = term;
            first = false;
         } else {
            const df t = two_sum(j[d].h, term.h);
            j[d] = {t.h, fadd(j[d].l, fadd(t.l, term.l))};
         }
      }
      j[d] = fast_two_sum(j[d].h, j[d].l);
   }

   // v = (j + F/2) / rho; the force is small, so F/2 enters the low word
   // after an exact Fast2Sum of the high words.
   const df* F = k.F;
   const float r0 = frcp(rho.h);
   float e = ffma(-rho.h, r0, 1.0f);
   e = ffma(-rho.l, r0, e);
   const df inv = {r0, fmul(r0, e)};
   df v[3];
#pragma unroll
   for (int d = 0; d < 3; d++) {
      const df jf = df_add(j[d], {0.5f * F[d].h, 0.5f * F[d].l});
      v[d] = df_mul(jf, inv);
   }
   // 3 v (the factor 3 of cu and uu folded in once).
   df v3[3];
#pragma unroll
   for (int d = 0; d < 3; d++) {
      const float p = fmul(3.0f, v[d].h);
      v3[d] = fast_two_sum(p, ffma(3.0f, v[d].h, -p) + 3.0f * v[d].l);
   }
   // uu = 3 v.v ;  base = 1 - uu/2
   df uu = df_mul_u(v3[0], v[0]);
   uu = df_add(uu, df_mul_u(v3[1], v[1]));
   uu = df_add(uu, df_mul_u(v3[2], v[2]));
   const df base = df_add_fast({1.0f, 0.0f}, {-0.5f * uu.h, -0.5f * uu.l});
   const float fu = 3.0f * (F[0].h * v[0].h + F[1].h * v[1].h + F[2].h * v[2].h);

   // omega * w * rho per weight class, folded into one factor.
   df owr[4];
#pragma unroll
   for (int cls = 0; cls < 4; cls++) owr[cls] = df_mul(k.ow[cls], rho);

   df out[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const int c0 = lat_c(Q, s, 0), c1 = lat_c(Q, s, 1), c2 = lat_c(Q, s, 2);
      const int cls = lat_norm2(Q, s);
      // cu = 3 c.v as a double-float
      df cu = {0.f, 0.f};
      bool first = true;
      if (c0 != 0) { cu = c0 > 0 ? v3[0] : df_neg(v3[0]); first = false; }
      if (c1 != 0) {
         const df t = c1 > 0 ? v3[1] : df_neg(v3[1]);
         cu = first ? t : df_add(cu, t);
         first = false;
      }
      if (c2 != 0) {
         const df t = c2 > 0 ? v3[2] : df_neg(v3[2]);
         cu = first ? t : df_add(cu, t);
         first = false;
      }
      // P = 1 + cu + cu^2/2 - uu/2 = (base + cu^2/2) + cu
      df P = base;
      if (!first) {
         const df c2h = df_sqr_u(cu);
         P = df_add_fast(P, {0.5f * c2h.h, 0.5f * c2h.l});
         P = df_add_fast(P, cu);
      }
      const df eqw = df_mul_u(owr[cls], P);  // omega * eq_s
      // forcing: (1 - omega/2) wf (cf - fu + cu cf), small: single precision
      const float cf = 3.0f * ((float)c0 * F[0].h + (float)c1 * F[1].h + (float)c2 * F[2].h);
      float wf = (float)lat_w(Q, s);
      if (Q == 19 && s == R && compat) wf = (float)(1.0 / 36.0);
      const float frc = k.om2 * wf * (cf - fu + cu.h * cf);
      // (1 - omega) f_s + omega eq_s + forcing
      const df a = df_mul_u(k.om1, f[s]);
      const df t = two_sum(a.h, eqw.h);
      out[s] = {t.h, fadd(t.l, fadd(fadd(a.l, eqw.l), frc))};
   }
   bool ok = true;
#pragma unroll
   for (int s = 0; s < Q; s++) ok = ok && out_ok(out[s]);
   if (!ok) return false;
#pragma unroll
   for (int s = 0; s < Q; s++) bits[s] = join(out[s]);
   return true;
}

// F64X cell update with a uniform force: fast path, else the exact IEEE
// double collision.
template <int Q>
__device__ __forceinline__ void collide_f64x(uint64_t (&bits)[Q], const KParams& p)
{
   x64::Consts k;
   k.om1 = {p.x_om1[0], p.x_om1[1]};
   k.omega = {p.x_omega[0], p.x_omega[1]};
#pragma unroll
   for (int c = 0; c < 4; c++) k.ow[c] = {p.x_ow[c][0], p.x_ow[c][1]};
#pragma unroll
   for (int d = 0; d < 3; d++) k.F[d] = {p.x_F[d][0], p.x_F[d][1]};
   k.om2 = p.om2f;
   if (collide_f64x_fast<Q>(bits, k, p.compat)) return;
   double d[Q], o[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) d[s] = x64::as_double(bits[s]);
   collide_f64<Q>(d, o, p.F[0], p.F[1], p.F[2], 0.0, p);
#pragma unroll
   for (int s = 0; s < Q; s++) bits[s] = x64::double_bits(o[s]);
}

}  // namespace lbm
