// F64X: double-precision BGK collision computed without the FP64 pipe.
//
// GB300's FP64 units run at about 1/60 of its FP32 rate, and double <-> float
// conversions are slow as well, so a collision written in `double` (or in
// float with conversions at load and store) is compute-bound far below the
// HBM roofline.  This path keeps the populations
// in FP64 memory (the reference's Pdf buffers) but:
//
//  * splits each loaded double into an unevaluated float pair (h, l): h is
//    the double truncated to 24 significant bits (integer operations), l the
//    remaining 29 mantissa bits rounded to 24 by an integer-to-float
//    conversion and scaled (|f - (h + l)| <= 2^-48 |f|);
//  * sums rho and j = sum c f exactly from 64-bit fixed-point images of the
//    doubles (integer adds);
//  * evaluates u, the equilibrium and the BGK/Guo update in
//    double-float arithmetic built from the error-free transformations
//    TwoSum (Knuth), Fast2Sum (Dekker 1971) and the FMA two-product, as used
//    in double-double libraries (Hida, Li & Bailey, "Library for double-double
//    and quad-double arithmetic", 2001);
//  * rebuilds the 64-bit pattern of the result (the double nearest to h + l)
//    with integer operations and one float-to-int conversion.
//
// The fast path covers positive populations in [2^-32, 1), the only values a
// physical state holds (with further bounds on the rest population and the
// velocity, checked per cell).  A cell whose inputs or results fall outside
// them is recomputed with the exact IEEE double collision, so any state is
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

// High 32 bits of ((hi:lo) << n), 0 <= n < 32.
__host__ __device__ __forceinline__ uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t n)
{
#ifdef __CUDA_ARCH__
   return __funnelshift_l(lo, hi, n);
#else
   const uint64_t v = ((uint64_t)hi << 32) | lo;
   return (uint32_t)((v << n) >> 32);
#endif
}

// Low 32 bits of ((hi:lo) >> n), 0 <= n < 32.
__host__ __device__ __forceinline__ uint32_t funnel_r(uint32_t lo, uint32_t hi, uint32_t n)
{
#ifdef __CUDA_ARCH__
   return __funnelshift_r(lo, hi, n);
#else
   const uint64_t v = ((uint64_t)hi << 32) | lo;
   return (uint32_t)(v >> n);
#endif
}

__host__ __device__ __forceinline__ float i2f_rn(int32_t i)
{
#ifdef __CUDA_ARCH__
   return __int2float_rn(i);
#else
   volatile float r = (float)i;
   return r;
#endif
}

// An integer-valued float (|x| < 2^31) to int32, exactly.
__host__ __device__ __forceinline__ int32_t f2i_exact(float x)
{
#ifdef __CUDA_ARCH__
   return __float2int_rz(x);
#else
   return (int32_t)x;
#endif
}

__host__ __device__ __forceinline__ float u2f_rn(uint32_t u)
{
#ifdef __CUDA_ARCH__
   return __uint2float_rn(u);
#else
   volatile float r = (float)u;
   return r;
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
// Fast-path range of the double bit patterns: positive, 2^-32 <= f < 1.
constexpr uint32_t kHiMin = (uint32_t)(1023 - 32) << 20;   // high word of 2^-32
constexpr uint32_t kHiMax = (uint32_t)1023 << 20;          // high word of 1.0 (excluded)

// Split a positive double in range (given as its 64-bit pattern) into (h, l).
//   h  = bits 60..29 of the pattern (the low 9 exponent bits above the top
//        23 mantissa bits) plus 2^30, masked to 31 bits: exponent E
//        re-biased to E - 896 in the float's 8-bit field, valid for E in
//        [897, 1150];
//   l  = the low 29 mantissa bits as an integer, rounded to nearest 24 bits
//        by the conversion and scaled by 2^(e(h) - 52) (a power of two, no
//        underflow for e(h) >= -74).  |f - (h + l)| <= 2^-48 |f|.
__host__ __device__ __forceinline__ df split(uint64_t bits)
{
   const uint32_t lo = (uint32_t)bits, hi = (uint32_t)(bits >> 32);
   const uint32_t hb = (funnel_l(lo, hi, 3) + 0x40000000u) & 0x7FFFFFFFu;
   const float scale = bitsf((hb & 0x7F800000u) - (52u << 23));
   return {bitsf(hb), fmul(u2f_rn(lo & 0x1FFFFFFFu), scale)};
}

// Fixed-point image of a positive double f in [2^-32, 1) for the moment
// sums: floor(f * 2^53) as a 64-bit integer, the 53-bit mantissa (with its
// implicit bit) shifted right by k = 1022 - E, in [0, 31] for that range.
// Sums of these images are exact; the truncation loses less than 2^-53 per
// population (its mean, half a unit, is added back to rho).
__host__ __device__ __forceinline__ uint64_t fixed53(uint64_t bits)
{
   const uint32_t lo = (uint32_t)bits, hi = (uint32_t)(bits >> 32);
   const uint32_t mh = (hi & 0x000FFFFFu) | 0x00100000u;
   const uint32_t k = 1022u - (hi >> 20);
   return ((uint64_t)(mh >> k) << 32) | funnel_r(lo, mh, k);
}

// Float pair of v * 2^-53 for a signed 64-bit v with |v| < 2^54.  The top
// part is v >> 23 rounded to 24 bits (an integer, so the remainder is exact
// and below 2^30), the remainder is rounded to 24 bits: the pair is exact for
// |v| < 2^47 and within 2^-48 |v| above, relative to v however small it is
// (a momentum sum of a slow flow keeps every bit).  Not normalised: h may be
// 0 or below l.
__host__ __device__ __forceinline__ df fixed53_to_pair(int64_t v)
{
   const uint32_t lo = (uint32_t)v, hi = (uint32_t)((uint64_t)v >> 32);
   const float hf = i2f_rn((int32_t)funnel_l(lo, hi, 9));   // v >> 23 (arithmetic), rounded
   const int32_t r = (int32_t)(lo - ((uint32_t)f2i_exact(hf) << 23));   // v - hf * 2^23, |r| < 2^30
   return {fmul(hf, 0x1p-30f), fmul(i2f_rn(r), 0x1p-53f)};
}

// Non-negative float to unsigned int, rounded to nearest even.
__host__ __device__ __forceinline__ uint32_t f2u_rn(float x)
{
#ifdef __CUDA_ARCH__
   return __float2uint_rn(x);
#else
   return (uint32_t)std::nearbyint(x);
#endif
}

// Running check of the result patterns of one cell: the largest
// sb - pattern(2^-75) as unsigned (a result below 2^-75 wraps around, a
// negative or NaN one lands above the bound).
struct JoinRange {
   uint32_t worst = 0u;
   __host__ __device__ __forceinline__ void add(uint32_t sb)
   {
      const uint32_t d = sb - 0x1A000000u;
      worst = worst > d ? worst : d;
   }
   // 2^-75 <= S < 1 for every result
   __host__ __device__ __forceinline__ bool ok() const { return worst < 0x3F800000u - 0x1A000000u; }
};

// Double pattern of h + l (positive):
//   S  = h + l rounded toward zero; the remainder h + l - S lies in
//        [0, ulp_float(S)); E = l - (S - h) is that remainder rounded to a
//        float (S - h is exact: S and h are within a factor of two).  The
//        remainder of a rounded-toward-zero sum need not be a float: for a
//        tiny negative l, S is h's predecessor and the remainder
//        ulp_float(S) - |l| can round up to ulp_float(S) itself;
//   N  = E in units of one double ulp of S, rounded to the nearest integer,
//        at most 2^29 (one float ulp of S);
//   the pattern of S as a double plus N (an integer add, which carries into
//        the float part and the exponent when N reaches 2^29): within about
//        33 double ulps of h + l.
// S's pattern goes into `range`; the result is valid when range.ok().
__host__ __device__ __forceinline__ uint64_t join(df v, JoinRange& range)
{
   const float S = fadd_rz(v.h, v.l);
   const float E = fsub(v.l, fsub(S, v.h));
   const uint32_t sb = fbits(S);
   range.add(sb);
   const float scale = bitsf(0x99000000u - (sb & 0x7F800000u));  // 2^(52 - e(S))
   const uint32_t n = f2u_rn(fmul(E, scale));
   return (((uint64_t)sb << 29) + ((uint64_t)0x38000000u << 32)) + n;
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
   df F3[3];      // 3 F
   df Kf[27];     // (1 - omega/2) w_s 3 c_s.F per direction: the forcing term linear in F
   df om2w[4];    // (1 - omega/2) w per weight class
   df om2w36;     // (1 - omega/2) / 36 (rest weight of the Q19 AA Unroll kernels)
   float om2;
};

}  // namespace x64

// Host: the collision constants of a launch (relaxation rate, uniform force,
// the Q19 AA Unroll rest-weight switch) in double, float and float-pair form.
// Forcing form of the F64X fast path: 0 no force; 1 any force (the forcing
// terms are added after the equilibrium with error-free sums); 2 a force small
// enough, sum |F_d| <= 0.004 omega, for the terms to be folded into the
// equilibrium's symmetric and antisymmetric parts.  The fast path's inputs
// give rho >= 1/4, |3 v_d| < 0.3, hence omega w rho (Q+ - |3 c.v|) >=
// 0.11 omega w, while the folded terms stay below 6.2 w sum |F_d|, so the
// Fast2Sum operand order still holds (with a 4.5x margin at the bound).
inline int force_mode(const double force[3], double omega)
{
   double fsum = 0.0;
   for (int d = 0; d < 3; d++) fsum += force[d] < 0.0 ? -force[d] : force[d];
   if (fsum == 0.0) return 0;
   return fsum <= 0.004 * omega ? 2 : 1;
}

inline void set_collision_constants(KParams& p, int Q, double omega, const double force[3], int compat)
{
   p.omega = omega;
   p.om1 = 1.0 - omega;
   p.om2 = 1.0 - 0.5 * omega;
   p.omegaf = (float)p.omega;
   p.om1f = (float)p.om1;
   p.om2f = (float)p.om2;
   for (int d = 0; d < 3; d++) {
      p.F[d] = force[d];
      p.Ff[d] = (float)force[d];
   }
   p.compat = compat;
   auto split = [](double d, float* out) {
      const float hi = (float)d;
      out[0] = hi;
      out[1] = (float)(d - (double)hi);
   };
   split(p.om1, p.x_om1);
   split(p.omega, p.x_omega);
   for (int k = 0; k < 4; k++) {
      double w;
      if (Q == 19) w = k == 0 ? 1.0 / 3.0 : (k == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
      else w = k == 0 ? 8.0 / 27.0 : (k == 1 ? 2.0 / 27.0 : (k == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
      split(omega * w, p.x_ow[k]);
      split(p.om2 * w, p.x_om2w[k]);
   }
   for (int d = 0; d < 3; d++) split(force[d], p.x_F[d]);
   for (int s = 0; s < Q; s++) {
      const double cf = 3.0 * (lat_c(Q, s, 0) * force[0] + lat_c(Q, s, 1) * force[1] + lat_c(Q, s, 2) * force[2]);
      split(p.om2 * lat_w(Q, s) * cf, p.x_Kf[s]);
   }
   for (int d = 0; d < 3; d++) split(3.0 * force[d], p.x_F3[d]);
   split(p.om2 / 36.0, p.x_om2w36);
   p.forced = force_mode(force, omega);
}

// Representative s < opp(s) of the p-th opposite pair (direction order of
// the reference: pairs are (0,1), (2,3), ... with the rest direction last).
__host__ __device__ constexpr int pair_dir(int Q, int p)
{
   int seen = 0;
   for (int s = 0; s < Q; s++) {
      if (s < lat_opp(Q, s)) {
         if (seen == p) return s;
         seen++;
      }
   }
   return -1;
}

// Fast-path validity thresholds (high words of the doubles).
constexpr uint32_t kHiQuarter = (uint32_t)(1023 - 2) << 20;   // 0.25

template <int Q, class Again>
__host__ __device__ __forceinline__ x64::df input_pair(const x64::df (&f)[Q], const Again& again, int s)
{
   if constexpr (Again::kRefetch) return again(s);
   else return f[s];
}

// Input policy of the fast path that splits the inputs once and keeps the
// pairs in registers.
struct KeepInputs {
   static constexpr bool kRefetch = false;
   __host__ __device__ __forceinline__ x64::df operator()(int) const { return {0.f, 0.f}; }
};

// The fast-path collision on one cell.  bits[] holds the Q input patterns in
// direction order; each output pattern is handed to emit(s, pattern).
// Returns false when the cell must take the exact path (nothing is emitted
// when an input check fails; after an output check fails every output has
// been emitted, possibly wrong):
//   * inputs: rest population in [0.25, 1), the others in [2^-32, 0.25), and
//     rho < 2;
//   * |3 v_d| < 0.3: |c.u| stays well below 1 - uu/2, so the pair sums
//     (1 - uu/2 + cu^2/2) +- cu keep their larger operand first;
//   * outputs inside [2^-75, 1).
// Work is organised by opposite pairs (s, opp(s)): cu, the quadratic term and
// the omega*w*rho products are shared, since cu(opp) = -cu(s).
// FORCE is the forcing form of force_mode() (0 none, 1 added after the
// equilibrium, 2 folded into it); Again supplies the inputs' float pairs for
// the (1 - omega) f term (KeepInputs, or a second read from shared memory).
//
// ROLLED (D3Q27): the 13 opposite pairs run in three loops over the pair
// classes (axes, planar and body diagonals) instead of unrolled, with the same
// operations in the same order, so the same bits.  The unrolled D3Q27 path
// runs about 2,700 instructions per cell, more code than the instruction cache
// holds; rolled, the pair code exists once per class instead of once per
// pair.  The direction and its velocity are then run-time
// values: outputs go to emit.put(s, opp(s), c_s, pattern), and Kf points at
// the per-direction forcing constants (float pairs, direction-indexed).
template <int Q, int FORCE, class Emit, class Again, bool ROLLED = false>
__host__ __device__ __forceinline__ bool collide_f64x_fast_emit(const uint64_t (&bits)[Q], const x64::Consts& k,
                                                               int compat, Emit& emit, const Again& again,
                                                               const float (*Kf)[2] = nullptr)
{
   using namespace x64;
   constexpr int R = lat_rest(Q);
   constexpr int NP = (Q - 1) / 2;
   uint32_t hmin = 0xFFFFFFFFu, hmax = 0;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      if (s == R) continue;
      const uint32_t hi = (uint32_t)(bits[s] >> 32);
      hmin = hmin < hi ? hmin : hi;
      hmax = hmax > hi ? hmax : hi;
   }
   const uint32_t hr = (uint32_t)(bits[R] >> 32);
   if (hmin < kHiMin || hmax >= kHiQuarter || hr < kHiQuarter || hr >= kHiMax) return false;

   // Float pairs of the inputs for the update's (1 - omega) f term: split
   // here and kept, or made again from a second read of the inputs.
   df f[Q];
   if constexpr (!Again::kRefetch) {
#pragma unroll
      for (int s = 0; s < Q; s++) f[s] = split(bits[s]);
   }

   // rho and j = sum c_s f_s from the exact sums of the fixed-point images
   // floor(f * 2^53); rho < 2 is checked (rho's top word below 2^22).
   // One pass: each image goes straight into the four sums.
   uint64_t rho_x = (uint64_t)(Q / 2);   // mean truncation loss, half a unit per population
   int64_t jx[3] = {0, 0, 0};
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const uint64_t X = fixed53(bits[s]);
      rho_x += X;
#pragma unroll
      for (int d = 0; d < 3; d++) {
         const int c = lat_c(Q, s, d);
         if (c > 0) jx[d] += (int64_t)X;
         if (c < 0) jx[d] -= (int64_t)X;
      }
   }
   if ((rho_x >> 32) >= (1u << 22)) return false;
   df j[3];
#pragma unroll
   for (int d = 0; d < 3; d++) {
      // Fast2Sum is exact here: t.h is 0 or at least ulp-aligned above |t.l|.
      const df t = fixed53_to_pair(jx[d]);
      j[d] = fast_two_sum(t.h, t.l);
   }
   // rho >= 1/4 (the rest population alone): Fast2Sum normalises the pair.
   const df rho0 = fixed53_to_pair((int64_t)rho_x);
   const df rho = fast_two_sum(rho0.h, rho0.l);

   // v = (j + F/2) / rho, left unnormalised (p + e); 3v normalised
   const float r0 = frcp(rho.h);
   float e = ffma(-rho.h, r0, 1.0f);
   e = ffma(-rho.l, r0, e);
   const df inv = {r0, fmul(r0, e)};
   df v[3], v3[3];
#pragma unroll
   for (int d = 0; d < 3; d++) {
      const df jf = FORCE ? df_add(j[d], {0.5f * k.F[d].h, 0.5f * k.F[d].l}) : j[d];
      v[d] = df_mul_u(jf, inv);
      const float p = fmul(3.0f, v[d].h);
      v3[d] = fast_two_sum(p, ffma(3.0f, v[d].h, -p) + 3.0f * v[d].l);
   }
   if (!(fabsf(v3[0].h) < 0.3f && fabsf(v3[1].h) < 0.3f && fabsf(v3[2].h) < 0.3f)) return false;
   // base = 1 - uu/2 with uu = 3 v.v, as a Fast2Sum chain from 1 (each
   // term 3 v_d^2 / 2 < 0.045 stays below the running value); left
   // unnormalised (its low part is a few ulps of its high part at most).
   df base;
   {
      const df p0 = df_mul_u(v3[0], v[0]), p1 = df_mul_u(v3[1], v[1]), p2 = df_mul_u(v3[2], v[2]);
      const df b0 = fast_two_sum(1.0f, -0.5f * p0.h);
      const df b1 = fast_two_sum(b0.h, -0.5f * p1.h);
      const df b2 = fast_two_sum(b1.h, -0.5f * p2.h);
      const float lows = ffma(-0.5f, p2.l, ffma(-0.5f, p1.l, ffma(-0.5f, p0.l, fadd(b0.l, b1.l))));
      base = {b2.h, fadd(b2.l, lows)};
   }
   // fu = 3 F.v (float pair; zero without a force)
   df fu = {0.f, 0.f};
   if (FORCE) {
      fu = df_mul_u(k.F3[0], v[0]);
      fu = df_add(fu, df_mul_u(k.F3[1], v[1]));
      fu = df_add(fu, df_mul_u(k.F3[2], v[2]));
   }

   df owr[4];
#pragma unroll
   for (int cls = 0; cls < 4; cls++) owr[cls] = df_mul_u(k.ow[cls], rho);

   // Each output goes to emit(s, pattern) as soon as it is made; the return
   // value says whether all of them passed the range check (if not, the
   // caller overwrites every one with the exact result).
   JoinRange range;
   // rest direction: P = base
   {
      df A = df_mul_u(owr[0], base);
      if (FORCE == 2) {
         // -(1 - omega/2) wf fu (wf = 1/36 with the Unroll-kernel weights),
         // folded into the equilibrium term
         const df fr = df_mul_u(compat ? k.om2w36 : k.om2w[0], fu);
         const df t2 = fast_two_sum(A.h, -fr.h);
         A = {t2.h, fadd(t2.l, fsub(A.l, fr.l))};
      }
      const df a = df_mul_u(k.om1, input_pair(f, again, R));
      const df t = two_sum(A.h, a.h);
      df out = {t.h, fadd(t.l, fadd(A.l, a.l))};
      if (FORCE == 1) {
         // -(1 - omega/2) wf fu, wf = 1/36 with the Unroll-kernel weights
         const df fr = df_mul_u(compat ? k.om2w36 : k.om2w[0], fu);
         const df t2 = two_sum(out.h, -fr.h);
         out = {t2.h, fadd(t2.l, fsub(out.l, fr.l))};
      }
      emit(R, join(out, range));
   }
   if constexpr (ROLLED) {
      static_assert(Q == 27, "the pair-class loops follow the D3Q27 direction order");
      // One pair (s, o = opp(s)) with c_s = (cx, cy, cz), cu = 3 c_s.v and the
      // class constants: the unrolled loop's body below, operation for operation.
      auto pair = [&](int s, int o, int cx, int cy, int cz, const df cu, const df owc, const df om2wc) {
         const df c2h = df_sqr_u(cu);
         const df qs = fast_two_sum(base.h, 0.5f * c2h.h);
         const df Qp = {qs.h, fadd(qs.l, fadd(base.l, 0.5f * c2h.l))};
         df A = df_mul_u(owc, Qp);
         df B = df_mul_u(owc, cu);
         const df Ks = {Kf[s][0], Kf[s][1]};
         df sym = {0.f, 0.f};
         if (FORCE) {
            const df gc = df_mul_u(Ks, cu);
            const df wf = df_mul_u(om2wc, fu);
            const df t3 = two_sum(gc.h, -wf.h);
            sym = {t3.h, fadd(t3.l, fsub(gc.l, wf.l))};
         }
         if (FORCE == 2) {
            const df as = fast_two_sum(A.h, sym.h);
            A = {as.h, fadd(as.l, fadd(A.l, sym.l))};
            const df bs = two_sum(B.h, Ks.h);
            B = {bs.h, fadd(bs.l, fadd(B.l, Ks.l))};
         }
         {
            const df tp = fast_two_sum(A.h, B.h);
            const df a = df_mul_u(k.om1, input_pair(f, again, s));
            const df t = two_sum(tp.h, a.h);
            df out = {t.h, fadd(t.l, fadd(tp.l, fadd(fadd(A.l, B.l), a.l)))};
            if (FORCE == 1) {
               const df fr = two_sum(Ks.h, sym.h);
               const df t2 = two_sum(out.h, fr.h);
               out = {t2.h, fadd(t2.l, fadd(out.l, fadd(fr.l, fadd(Ks.l, sym.l))))};
            }
            emit.put(s, o, cx, cy, cz, join(out, range));
         }
         {
            const df tm = fast_two_sum(A.h, -B.h);
            const df a = df_mul_u(k.om1, input_pair(f, again, o));
            const df t = two_sum(tm.h, a.h);
            df out = {t.h, fadd(t.l, fadd(tm.l, fadd(fsub(A.l, B.l), a.l)))};
            if (FORCE == 1) {
               const df fr = two_sum(sym.h, -Ks.h);
               const df t2 = two_sum(out.h, fr.h);
               out = {t2.h, fadd(t2.l, fadd(out.l, fadd(fr.l, fsub(sym.l, Ks.l))))};
            }
            emit.put(o, s, -cx, -cy, -cz, join(out, range));
         }
      };
      // axes: (0,1) (2,3) (4,5), c = e_d, cu = 3 v_d
#pragma unroll 1
      for (int d = 0; d < 3; d++) {
         const df cu = d == 0 ? v3[0] : (d == 1 ? v3[1] : v3[2]);
         pair(2 * d, 2 * d + 1, d == 0, d == 1, d == 2, cu, owr[1], k.om2w[1]);
      }
      // planar diagonals (6,11) (7,10) (8,13) (9,12) (14,17) (15,16):
      // c = e_a + sign e_b, a < b, sign -1 for the odd j
#pragma unroll 1
      for (int j = 0; j < 6; j++) {
         const int a = j < 4 ? 0 : 1, b = j < 2 ? 1 : 2;
         const bool neg = (j & 1) != 0;
         const df va = a == 0 ? v3[0] : v3[1];
         const df vb = b == 1 ? v3[1] : v3[2];
         const df t = neg ? df_neg(vb) : vb;
         const df u2 = two_sum(va.h, t.h);
         const df cu = {u2.h, fadd(u2.l, fadd(va.l, t.l))};
         const int sgn = neg ? -1 : 1;
         const int sd = j < 4 ? 6 + j : 10 + j;
         const int od = j < 2 ? 11 - j : (j < 4 ? 15 - j : 31 - sd);
         pair(sd, od, a == 0 ? 1 : 0, a == 1 ? 1 : (b == 1 ? sgn : 0), b == 2 ? sgn : 0, cu, owr[2], k.om2w[2]);
      }
      // body diagonals (18,25) (19,24) (20,23) (21,22): c = (1, +-1, +-1)
#pragma unroll 1
      for (int j = 0; j < 4; j++) {
         const bool ny = j >= 2, nz = (j & 1) != 0;
         const df ty = ny ? df_neg(v3[1]) : v3[1];
         const df u2 = two_sum(v3[0].h, ty.h);
         df cu = {u2.h, fadd(u2.l, fadd(v3[0].l, ty.l))};
         const df tz = nz ? df_neg(v3[2]) : v3[2];
         const df u3 = two_sum(cu.h, tz.h);
         cu = {u3.h, fadd(u3.l, fadd(cu.l, tz.l))};
         pair(18 + j, 25 - j, 1, ny ? -1 : 1, nz ? -1 : 1, cu, owr[3], k.om2w[3]);
      }
   } else {
#pragma unroll
      for (int q = 0; q < NP; q++) {
         const int s = pair_dir(Q, q), o = lat_opp(Q, s);
         const int c0 = lat_c(Q, s, 0), c1 = lat_c(Q, s, 1), c2 = lat_c(Q, s, 2);
         const int cls = lat_norm2(Q, s);
         // cu = 3 c_s.v (two_sum-based, left unnormalised)
         df cu = {0.f, 0.f};
         bool first = true;
         if (c0 != 0) { cu = c0 > 0 ? v3[0] : df_neg(v3[0]); first = false; }
         if (c1 != 0) {
            const df t = c1 > 0 ? v3[1] : df_neg(v3[1]);
            if (first) { cu = t; first = false; }
            else { const df u2 = two_sum(cu.h, t.h); cu = {u2.h, fadd(u2.l, fadd(cu.l, t.l))}; }
         }
         if (c2 != 0) {
            const df t = c2 > 0 ? v3[2] : df_neg(v3[2]);
            if (first) { cu = t; first = false; }
            else { const df u2 = two_sum(cu.h, t.h); cu = {u2.h, fadd(u2.l, fadd(cu.l, t.l))}; }
         }
         // Qp = base + cu^2 / 2
         const df c2h = df_sqr_u(cu);
         const df qs = fast_two_sum(base.h, 0.5f * c2h.h);
         const df Qp = {qs.h, fadd(qs.l, fadd(base.l, 0.5f * c2h.l))};
         df A = df_mul_u(owr[cls], Qp);   // omega * eq, symmetric part
         df B = df_mul_u(owr[cls], cu);   // omega * eq, antisymmetric part
         // forcing om2 w (+-cf - fu + cu cf) = +-Kf[s] + (Kf[s] cu - om2 w fu), with
         // Kf[s] = om2 w cf a float pair made on the host
         df sym = {0.f, 0.f};
         if (FORCE) {
            const df gc = df_mul_u(k.Kf[s], cu);
            const df wf = df_mul_u(k.om2w[cls], fu);
            const df t3 = two_sum(gc.h, -wf.h);
            sym = {t3.h, fadd(t3.l, fsub(gc.l, wf.l))};
         }
         if (FORCE == 2) {
            // small force: sym joins the symmetric part (far below it) and
            // Kf[s] the antisymmetric part (which may vanish, hence TwoSum)
            const df as = fast_two_sum(A.h, sym.h);
            A = {as.h, fadd(as.l, fadd(A.l, sym.l))};
            const df bs = two_sum(B.h, k.Kf[s].h);
            B = {bs.h, fadd(bs.l, fadd(B.l, k.Kf[s].l))};
         }
         // s: A + B ; opp(s): A - B ; then + (1 - omega) f
         {
            const df tp = fast_two_sum(A.h, B.h);
            const df a = df_mul_u(k.om1, input_pair(f, again, s));
            const df t = two_sum(tp.h, a.h);
            df out = {t.h, fadd(t.l, fadd(tp.l, fadd(fadd(A.l, B.l), a.l)))};
            if (FORCE == 1) {
               const df fr = two_sum(k.Kf[s].h, sym.h);
               const df t2 = two_sum(out.h, fr.h);
               out = {t2.h, fadd(t2.l, fadd(out.l, fadd(fr.l, fadd(k.Kf[s].l, sym.l))))};
            }
            emit(s, join(out, range));
         }
         {
            const df tm = fast_two_sum(A.h, -B.h);
            const df a = df_mul_u(k.om1, input_pair(f, again, o));
            const df t = two_sum(tm.h, a.h);
            df out = {t.h, fadd(t.l, fadd(tm.l, fadd(fsub(A.l, B.l), a.l)))};
            if (FORCE == 1) {
               const df fr = two_sum(sym.h, -k.Kf[s].h);
               const df t2 = two_sum(out.h, fr.h);
               out = {t2.h, fadd(t2.l, fadd(out.l, fadd(fr.l, fsub(sym.l, k.Kf[s].l))))};
            }
            emit(o, join(out, range));
         }
      }
   }
   return range.ok();
}

// Emitter that collects the outputs in registers.
template <int Q>
struct EmitToArray {
   uint64_t res[Q];
   __host__ __device__ __forceinline__ void operator()(int s, uint64_t v) { res[s] = v; }
   __host__ __device__ __forceinline__ void put(int s, int, int, int, int, uint64_t v) { res[s] = v; }
};


// The fast path on bits[] in place: returns false, leaving bits[] untouched,
// when the cell must take the exact path.
template <int Q, int FORCE>
__host__ __device__ __forceinline__ bool collide_f64x_fast(uint64_t (&bits)[Q], const x64::Consts& k,
                                                          int compat)
{
   EmitToArray<Q> out;
   if (!collide_f64x_fast_emit<Q, FORCE>(bits, k, compat, out, KeepInputs{})) return false;
#pragma unroll
   for (int s = 0; s < Q; s++) bits[s] = out.res[s];
   return true;
}

// F64X cell update with a uniform force: fast path, else the exact IEEE
// double collision.
template <int Q>
__device__ __forceinline__ x64::Consts collide_consts(const KParams& p)
{
   x64::Consts k;
   k.om1 = {p.x_om1[0], p.x_om1[1]};
   k.omega = {p.x_omega[0], p.x_omega[1]};
#pragma unroll
   for (int c = 0; c < 4; c++) k.ow[c] = {p.x_ow[c][0], p.x_ow[c][1]};
#pragma unroll
   for (int d = 0; d < 3; d++) k.F[d] = {p.x_F[d][0], p.x_F[d][1]};
#pragma unroll
   for (int d = 0; d < 3; d++) k.F3[d] = {p.x_F3[d][0], p.x_F3[d][1]};
#pragma unroll
   for (int s = 0; s < Q; s++) k.Kf[s] = {p.x_Kf[s][0], p.x_Kf[s][1]};
#pragma unroll
   for (int c = 0; c < 4; c++) k.om2w[c] = {p.x_om2w[c][0], p.x_om2w[c][1]};
   k.om2w36 = {p.x_om2w36[0], p.x_om2w36[1]};
   k.om2 = p.om2f;
   return k;
}

template <int Q>
__device__ __forceinline__ void collide_exact_bits(uint64_t (&bits)[Q], const KParams& p)
{
   double d[Q], o[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) d[s] = x64::as_double(bits[s]);
   collide_f64<Q>(d, o, p.F[0], p.F[1], p.F[2], 0.0, p);
#pragma unroll
   for (int s = 0; s < Q; s++) bits[s] = x64::double_bits(o[s]);
}

// F64X cell update with a uniform force: fast path, else the exact IEEE
// double collision.
template <int Q>
__device__ __forceinline__ void collide_f64x(uint64_t (&bits)[Q], const KParams& p)
{
   const x64::Consts k = collide_consts<Q>(p);
   const bool fast = p.forced == 2 ? collide_f64x_fast<Q, 2>(bits, k, p.compat)
                     : p.forced    ? collide_f64x_fast<Q, 1>(bits, k, p.compat)
                                   : collide_f64x_fast<Q, 0>(bits, k, p.compat);
   if (fast) return;
   collide_exact_bits<Q>(bits, p);
}

// Input pattern s read again from shared memory (direction s at byte 256 s
// from the lane's first), raw or split into a float pair.  The load is
// volatile so that the compiler does not keep the first load's value live in
// registers instead.
struct AgainFromShared {
   static constexpr bool kRefetch = true;
   uint32_t addr;
   __device__ __forceinline__ uint64_t raw(int s) const
   {
      unsigned long long v;
      asm volatile("ld.shared.u64 %0, [%1];\n" : "=l"(v) : "r"(addr + 256u * (uint32_t)s));
      return v;
   }
   __device__ __forceinline__ x64::df operator()(int s) const { return x64::split(raw(s)); }
};

// collide_f64x for inputs that stay in shared memory (direction s at in[32 s]),
// with each output handed to emit(s, pattern) as it is made, so neither the
// input nor the output patterns stay in registers through the fast path: the
// moment sums read the inputs once, the update reads them again.  If
// the fast path fails after emitting, the exact results are emitted again
// over them (the fallback reads its inputs from shared memory): a caller's
// emit must let a later emit of the same s win, as stores from one thread to
// one address do.
// ROLLED: the D3Q27 pair-class loops (collide_f64x_fast_emit), whose outputs
// go to emit.put.
template <int Q, bool ROLLED = false, class Emit>
__device__ __forceinline__ void collide_f64x_shared_emit(const unsigned long long* in, const KParams& p, Emit& emit)
{
   uint64_t bits[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) bits[s] = in[s * 32];
   const x64::Consts k = collide_consts<Q>(p);
   const AgainFromShared again{(uint32_t)__cvta_generic_to_shared(in)};
   using A = AgainFromShared;
   const bool fast =
      p.forced == 2 ? collide_f64x_fast_emit<Q, 2, Emit, A, ROLLED>(bits, k, p.compat, emit, again, p.x_Kf)
      : p.forced    ? collide_f64x_fast_emit<Q, 1, Emit, A, ROLLED>(bits, k, p.compat, emit, again, p.x_Kf)
                    : collide_f64x_fast_emit<Q, 0, Emit, A, ROLLED>(bits, k, p.compat, emit, again, p.x_Kf);
   if (fast) return;
#pragma unroll
   for (int s = 0; s < Q; s++) bits[s] = again.raw(s);
   collide_exact_bits<Q>(bits, p);
#pragma unroll
   for (int s = 0; s < Q; s++) emit(s, bits[s]);
}

}  // namespace lbm
