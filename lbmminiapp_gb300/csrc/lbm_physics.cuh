// Collision arithmetic and population storage for the collide-stream kernels.
//
// The physics is the reference's BGK collision with Guo forcing
// (src/kernels/KernelAA_SOA_Base.cpp:186-247):
//   rho = sum f_s,  v = (sum c_s f_s + F/2) / rho
//   eq_s    = w_s rho (1 + cu + cu^2/2 - uu/2),   cu = 3 c_s.v, uu = 3 v.v
//   fdist_s = w_s (cf - fu + cu cf),              cf = 3 c_s.F, fu = 3 F.v
//   f_s'    = (1-omega) f_s + omega eq_s + (1-omega/2) fdist_s
// optionally followed by partial bounce-back with solid fraction sp:
//   post_s  = (1-sp) f_s' + sp f_opp(s)
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

#include "lbm_lattice.cuh"

namespace lbm {

enum StoreKind { ST_F64 = 0, ST_F32 = 1, ST_BF16 = 2, ST_F16 = 3 };
enum ArithKind { AR_F64 = 1, AR_F64X = 2, AR_F32 = 3 };
enum StepKind { K_AA_EVEN = 0, K_AA_ODD = 1, K_AB_PUSH = 2, K_AB_PULL = 3 };

// Scale applied to shifted FP16 populations so that small deviations stay in
// the normal range of binary16 (as in the FP16S format of Lehmann et al.
// 2022, "Accuracy and performance of the lattice Boltzmann method with 64-bit,
// 32-bit, and customized 16-bit number formats").
constexpr float kF16Scale = 32768.0f;

// Everything a step kernel needs, passed by value.
struct KParams {
   int nx, ny, nz;
   int z0;               // first z plane covered by the launch
   int64_t ncell;
   int64_t plane;        // elements between direction planes
   int64_t cstart, cend; // cell range handled by this launch
   double omega, om1, om2;        // omega, 1-omega, 1-0.5*omega (as the reference folds them)
   float omegaf, om1f, om2f;
   double F[3];                   // uniform body force
   float Ff[3];
   int compat;                    // Q19 AA Unroll rest forcing weight
   const uint32_t* links;         // per-cell link word or null
   const double* force_field;     // planar [3][plane] (FP64 arithmetic) or null
   const float* force_field_f;    // planar [3][plane] (FP32 arithmetic) or null
   const double* porosity;        // [plane] or null
   const float* porosity_f;
   // Float-pair (hi, lo) splits of the launch constants for the F64X path,
   // made on the host so no thread converts doubles.
   float x_om1[2], x_omega[2];
   float x_ow[4][2];              // omega * w per weight class (|c|^2 = 0..3)
   float x_F[3][2];               // uniform force
   float x_Kf[27][2];             // (1 - omega/2) w_s 3 c_s.F per direction
   float x_F3[3][2];              // 3 F
   float x_om2w[4][2];            // (1 - omega/2) w per weight class
   float x_om2w36[2];             // (1 - omega/2) / 36
   int forced;                    // uniform force nonzero
   uint32_t* sched;               // [kFeedWords] tile counters of the persistent kernels, zero between launches
};

// Link word: bit s set when the neighbour at x + c_s is solid or outside a
// non-periodic face (half-way bounce-back); bit 31 set when x itself is solid.
constexpr uint32_t kSolidBit = 0x80000000u;

// ---------------------------------------------------------------- storage
template <int ST> struct Store;
template <> struct Store<ST_F64> { using T = double; static constexpr int bytes = 8; };
template <> struct Store<ST_F32> { using T = float; static constexpr int bytes = 4; };
template <> struct Store<ST_BF16> { using T = __nv_bfloat16; static constexpr int bytes = 2; };
template <> struct Store<ST_F16> { using T = __half; static constexpr int bytes = 2; };

// Shifted storage: the stored value is (f - w) (times kF16Scale for FP16).
__device__ __forceinline__ float load_shifted(const float* p) { return *p; }
__device__ __forceinline__ float load_shifted(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float load_shifted(const __half* p)
{
   return __half2float(*p) * (1.0f / kF16Scale);
}
__device__ __forceinline__ void store_shifted(float* p, float g) { *p = g; }
__device__ __forceinline__ void store_shifted(__nv_bfloat16* p, float g) { *p = __float2bfloat16_rn(g); }
__device__ __forceinline__ void store_shifted(__half* p, float g) { *p = __float2half_rn(g * kF16Scale); }

// ------------------------------------------------- exact FP64 collision
// Operation order and association of KernelAA_SOA_Base.cpp:186-247 with every
// operation an explicitly rounded IEEE double op (no FMA contraction), so the
// result is bit-identical to the reference CPU build.  Terms whose stencil
// component is zero are skipped: the reference adds d*0.0 = +-0.0, which
// leaves every non-zero partial sum unchanged.
template <int Q, int S>
__device__ __forceinline__ double cdot_exact(double a0, double a1, double a2)
{
   constexpr int c0 = lat_c(Q, S, 0), c1 = lat_c(Q, S, 1), c2 = lat_c(Q, S, 2);
   double acc = 0.0;
   bool any = false;
   if (c0 != 0) { acc = c0 > 0 ? a0 : -a0; any = true; }
   if (c1 != 0) { acc = any ? (c1 > 0 ? __dadd_rn(acc, a1) : __dsub_rn(acc, a1)) : (c1 > 0 ? a1 : -a1); any = true; }
   if (c2 != 0) { acc = any ? (c2 > 0 ? __dadd_rn(acc, a2) : __dsub_rn(acc, a2)) : (c2 > 0 ? a2 : -a2); any = true; }
   return acc;
}

template <int Q, int S = 0>
__device__ __forceinline__ void eq_update_exact(double (&d)[Q], double (&o)[Q], double rho, double v0,
                                                double v1, double v2, double F0, double F1, double F2,
                                                double vdotv, double fdotv, const KParams& p)
{
   if constexpr (S < Q) {
      const double cdotv = __dmul_rn(3.0, cdot_exact<Q, S>(v0, v1, v2));
      const double cdotf = __dmul_rn(3.0, cdot_exact<Q, S>(F0, F1, F2));
      constexpr double w = lat_w(Q, S);
      const double eq = __dmul_rn(
         __dmul_rn(w, rho),
         __dsub_rn(__dadd_rn(__dadd_rn(1.0, cdotv), __dmul_rn(__dmul_rn(0.5, cdotv), cdotv)),
                   __dmul_rn(0.5, vdotv)));
      const double wf = (Q == 19 && S == lat_rest(Q) && p.compat) ? 1.0 / 36.0 : w;
      const double fdist = __dmul_rn(wf, __dadd_rn(__dsub_rn(cdotf, fdotv), __dmul_rn(cdotv, cdotf)));
      o[S] = __dadd_rn(__dadd_rn(__dmul_rn(p.om1, d[S]), __dmul_rn(p.omega, eq)), __dmul_rn(p.om2, fdist));
      eq_update_exact<Q, S + 1>(d, o, rho, v0, v1, v2, F0, F1, F2, vdotv, fdotv, p);
   }
}

template <int Q>
__device__ __forceinline__ void collide_f64(double (&d)[Q], double (&o)[Q], double F0, double F1,
                                            double F2, double sp, const KParams& p)
{
   double rho = 0.0, v0 = 0.0, v1 = 0.0, v2 = 0.0;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      rho = __dadd_rn(rho, d[s]);
      const int c0 = lat_c(Q, s, 0), c1 = lat_c(Q, s, 1), c2 = lat_c(Q, s, 2);
      if (c0 > 0) v0 = __dadd_rn(v0, d[s]); else if (c0 < 0) v0 = __dsub_rn(v0, d[s]);
      if (c1 > 0) v1 = __dadd_rn(v1, d[s]); else if (c1 < 0) v1 = __dsub_rn(v1, d[s]);
      if (c2 > 0) v2 = __dadd_rn(v2, d[s]); else if (c2 < 0) v2 = __dsub_rn(v2, d[s]);
   }
   v0 = __dadd_rn(v0, __dmul_rn(0.5, F0));
   v1 = __dadd_rn(v1, __dmul_rn(0.5, F1));
   v2 = __dadd_rn(v2, __dmul_rn(0.5, F2));
   const double invRho = __ddiv_rn(1.0, rho);
   v0 = __dmul_rn(v0, invRho);
   v1 = __dmul_rn(v1, invRho);
   v2 = __dmul_rn(v2, invRho);
   const double vdotv =
      __dmul_rn(3.0, __dadd_rn(__dadd_rn(__dmul_rn(v0, v0), __dmul_rn(v1, v1)), __dmul_rn(v2, v2)));
   const double fdotv =
      __dmul_rn(3.0, __dadd_rn(__dadd_rn(__dmul_rn(F0, v0), __dmul_rn(F1, v1)), __dmul_rn(F2, v2)));
   eq_update_exact<Q>(d, o, rho, v0, v1, v2, F0, F1, F2, vdotv, fdotv, p);
   if (sp != 0.0) {
      const double keep = __dsub_rn(1.0, sp);
#pragma unroll
      for (int s = 0; s < Q; s++) o[s] = __dadd_rn(__dmul_rn(keep, o[s]), __dmul_rn(sp, d[lat_opp(Q, s)]));
   }
}

// ------------------------------------------- FP32 shifted collision
// Stored values are G = S (f - w) with S = 2^15 for FP16 and 1 otherwise.
// With drho = sum (f - w) (sum w = 1) and j = sum c (f - w) (sum c w = 0):
//   eq_s - w_s = w_s (drho + rho (cu + cu^2/2 - uu/2))
//   G_s'       = (1-omega) G_s + omega S (eq_s - w_s) + (1-omega/2) S fdist_s
// which keeps the large constant w out of the single-precision arithmetic;
// S enters only through per-cell factors.  Opposite directions share
// cu(opp) = -cu, so S (eq - w) = A +- B with A = w (S drho + S rho (cu^2 - uu)/2)
// and B = w S rho cu.
template <int ST> struct ShiftScale { static constexpr float S = 1.0f; };
template <> struct ShiftScale<ST_F16> { static constexpr float S = kF16Scale; };

__device__ __forceinline__ float load_raw(const float* p) { return *p; }
__device__ __forceinline__ float load_raw(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float load_raw(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ void store_raw(float* p, float g) { *p = g; }
__device__ __forceinline__ void store_raw(__nv_bfloat16* p, float g) { *p = __float2bfloat16_rn(g); }
__device__ __forceinline__ void store_raw(__half* p, float g) { *p = __float2half_rn(g); }

template <int Q, int S_>
__device__ __forceinline__ float cdot_f(const float (&v)[3])
{
   constexpr int c0 = lat_c(Q, S_, 0), c1 = lat_c(Q, S_, 1), c2 = lat_c(Q, S_, 2);
   float r = 0.0f;
   bool any = false;
   if (c0 != 0) { r = c0 > 0 ? v[0] : -v[0]; any = true; }
   if (c1 != 0) { r = any ? (c1 > 0 ? r + v[1] : r - v[1]) : (c1 > 0 ? v[1] : -v[1]); any = true; }
   if (c2 != 0) { r = any ? (c2 > 0 ? r + v[2] : r - v[2]) : (c2 > 0 ? v[2] : -v[2]); }
   return r;
}

// Representative s < opp(s) of the P-th opposite pair (the reference's
// direction order: pairs (0,1), (2,3), ..., the rest direction last).
template <int Q, int P>
__host__ __device__ constexpr int pair_rep()
{
   int seen = 0;
   for (int t = 0; t < Q; t++)
      if (t < lat_opp(Q, t)) {
         if (seen == P) return t;
         seen++;
      }
   return -1;
}

// Per-cell quantities of the shifted collision: 3u, 3F, fu = 3 F.u, uu = 3 u.u
// and the weight-class factors w S drho, w S rho.
struct ShiftedCell {
   float u3[3], F3[3], fu, uu, wSd[4], wSr[4];
};

template <int Q, int ST, bool FORCE>
__device__ __forceinline__ ShiftedCell shifted_cell(const float (&G)[Q], float F0, float F1, float F2)
{
   constexpr float S = ShiftScale<ST>::S;
   constexpr float iS = 1.0f / S;
   ShiftedCell c;
   float Sd = 0.f, j0 = 0.f, j1 = 0.f, j2 = 0.f;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      Sd += G[s];
      const int c0 = lat_c(Q, s, 0), c1 = lat_c(Q, s, 1), c2 = lat_c(Q, s, 2);
      if (c0 > 0) j0 += G[s]; else if (c0 < 0) j0 -= G[s];
      if (c1 > 0) j1 += G[s]; else if (c1 < 0) j1 -= G[s];
      if (c2 > 0) j2 += G[s]; else if (c2 < 0) j2 -= G[s];
   }
   const float rho = fmaf(Sd, iS, 1.0f);
   const float ir = __frcp_rn(rho);
   // 3u and 3F
   const float ir3 = 3.0f * ir;
   c.u3[0] = fmaf(j0, iS, 0.5f * F0) * ir3;
   c.u3[1] = fmaf(j1, iS, 0.5f * F1) * ir3;
   c.u3[2] = fmaf(j2, iS, 0.5f * F2) * ir3;
   c.uu = (c.u3[0] * c.u3[0] + c.u3[1] * c.u3[1] + c.u3[2] * c.u3[2]) * (1.0f / 3.0f);   // 3 u.u
   c.F3[0] = 3.0f * F0;
   c.F3[1] = 3.0f * F1;
   c.F3[2] = 3.0f * F2;
   c.fu = FORCE ? (c.F3[0] * c.u3[0] + c.F3[1] * c.u3[1] + c.F3[2] * c.u3[2]) * (1.0f / 3.0f) : 0.0f;
   const float Sr = S * rho;
#pragma unroll
   for (int k = 0; k < 4; k++) {
      float w;
      if (Q == 19) w = k == 0 ? (float)(1.0 / 3.0) : (k == 1 ? (float)(1.0 / 18.0) : (float)(1.0 / 36.0));
      else w = k == 0 ? (float)(8.0 / 27.0) : (k == 1 ? (float)(2.0 / 27.0) : (k == 2 ? (float)(1.0 / 54.0) : (float)(1.0 / 216.0)));
      c.wSd[k] = w * Sd;
      c.wSr[k] = w * Sr;
   }
   return c;
}

// Outputs of the P-th pair (s, opp(s)) from the inputs Gs, Gob.
template <int Q, int ST, bool FORCE, int P>
__device__ __forceinline__ void shifted_pair(const ShiftedCell& c, float Gs, float Gob, float om1, float omega,
                                             float Som2, float& os, float& oob)
{
   constexpr int s = pair_rep<Q, P>();
   constexpr int cls = lat_norm2(Q, s);
   const float cu = cdot_f<Q, s>(c.u3);
   const float A = fmaf(c.wSr[cls], 0.5f * fmaf(cu, cu, -c.uu), c.wSd[cls]);
   const float B = c.wSr[cls] * cu;
   float fs = 0.0f, fo = 0.0f;
   if (FORCE) {
      constexpr float w = (float)lat_w(Q, s);
      const float cf = cdot_f<Q, s>(c.F3);
      const float sym = fmaf(cu, cf, -c.fu);
      fs = Som2 * w * (cf + sym);
      fo = Som2 * w * (sym - cf);
   }
   os = fmaf(om1, Gs, fmaf(omega, A + B, fs));
   oob = fmaf(om1, Gob, fmaf(omega, A - B, fo));
}

// Output of the rest direction: A = w (S drho + S rho (-uu/2)), forcing -wf fu.
template <int Q, int ST, bool FORCE>
__device__ __forceinline__ float shifted_rest(const ShiftedCell& c, float GR, const KParams& p, float Som2)
{
   const float A = fmaf(c.wSr[0], -0.5f * c.uu, c.wSd[0]);
   float fr = 0.0f;
   if (FORCE) {
      const float wf = (Q == 19 && p.compat) ? (float)(1.0 / 36.0) : (float)lat_w(Q, lat_rest(Q));
      fr = -Som2 * wf * c.fu;
   }
   return fmaf(p.om1f, GR, fmaf(p.omegaf, A, fr));
}

template <int Q, int ST, bool FORCE, int P = 0>
__device__ __forceinline__ void collide_pairs_f32(const float (&G)[Q], float (&o)[Q], const ShiftedCell& c, float om1,
                                                  float omega, float Som2)
{
   if constexpr (P < (Q - 1) / 2) {
      constexpr int s = pair_rep<Q, P>();
      constexpr int ob = lat_opp(Q, s);
      shifted_pair<Q, ST, FORCE, P>(c, G[s], G[ob], om1, omega, Som2, o[s], o[ob]);
      collide_pairs_f32<Q, ST, FORCE, P + 1>(G, o, c, om1, omega, Som2);
   }
}

template <int Q, int ST, bool FORCE>
__device__ __forceinline__ void collide_f32(const float (&G)[Q], float (&o)[Q], float F0, float F1, float F2,
                                            float sp, const KParams& p)
{
   const ShiftedCell c = shifted_cell<Q, ST, FORCE>(G, F0, F1, F2);
   const float Som2 = ShiftScale<ST>::S * p.om2f;
   collide_pairs_f32<Q, ST, FORCE>(G, o, c, p.om1f, p.omegaf, Som2);
   constexpr int R = lat_rest(Q);
   o[R] = shifted_rest<Q, ST, FORCE>(c, G[R], p, Som2);
   if (sp != 0.0f) {
      const float keep = 1.0f - sp;
#pragma unroll
      for (int s = 0; s < Q; s++) o[s] = keep * o[s] + sp * G[lat_opp(Q, s)];
   }
}

// Two cells (inputs G0, G1) with a uniform force: each direction's pair of
// outputs goes to emit(s, o0, o1) as soon as it is made, so no output array
// stays in registers.  The arithmetic per cell is collide_f32's.
template <int Q, int ST, bool FORCE, int P = 0, class Emit2>
__device__ __forceinline__ void collide2_pairs_f32(const float (&G0)[Q], const float (&G1)[Q], const ShiftedCell& c0,
                                                   const ShiftedCell& c1, float om1, float omega, float Som2,
                                                   Emit2& emit)
{
   if constexpr (P < (Q - 1) / 2) {
      constexpr int s = pair_rep<Q, P>();
      constexpr int ob = lat_opp(Q, s);
      float a0, b0, a1, b1;
      shifted_pair<Q, ST, FORCE, P>(c0, G0[s], G0[ob], om1, omega, Som2, a0, b0);
      shifted_pair<Q, ST, FORCE, P>(c1, G1[s], G1[ob], om1, omega, Som2, a1, b1);
      emit(s, a0, a1);
      emit(ob, b0, b1);
      collide2_pairs_f32<Q, ST, FORCE, P + 1>(G0, G1, c0, c1, om1, omega, Som2, emit);
   }
}

template <int Q, int ST, bool FORCE, class Emit2>
__device__ __forceinline__ void collide2_f32_emit(const float (&G0)[Q], const float (&G1)[Q], const KParams& p,
                                                  Emit2& emit)
{
   const float F0 = FORCE ? p.Ff[0] : 0.0f, F1 = FORCE ? p.Ff[1] : 0.0f, F2 = FORCE ? p.Ff[2] : 0.0f;
   const ShiftedCell c0 = shifted_cell<Q, ST, FORCE>(G0, F0, F1, F2);
   const ShiftedCell c1 = shifted_cell<Q, ST, FORCE>(G1, F0, F1, F2);
   const float Som2 = ShiftScale<ST>::S * p.om2f;
   collide2_pairs_f32<Q, ST, FORCE>(G0, G1, c0, c1, p.om1f, p.omegaf, Som2, emit);
   constexpr int R = lat_rest(Q);
   emit(R, shifted_rest<Q, ST, FORCE>(c0, G0[R], p, Som2), shifted_rest<Q, ST, FORCE>(c1, G1[R], p, Som2));
}

}  // namespace lbm
