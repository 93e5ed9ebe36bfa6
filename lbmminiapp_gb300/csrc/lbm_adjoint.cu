// Discrete adjoint of the collide-stream step (no reference counterpart).
//
// Forward model, one step from the pre-collision state f^t (AB push storage,
// slot s = direction s):
//   rho = sum f, j = sum c f + F/2, u = j / rho           (F = F_uniform + F_field(x))
//   C_s = (1 - omega) f_s + omega eq_s(rho, j) + (1 - omega/2) fd_s(rho, j, F)
//   post_s = (1 - sig) C_s + sig f_opp(s)                  (partial bounce-back, sig(x))
//   f^{t+1}_s(x + c_s) = post_s(x), or f^{t+1}_opp(s)(x) = post_s(x) when x + c_s
//   is blocked (half-way bounce-back)
// with eq_s = w_s (rho + 3 c.j + 9/2 (c.j)^2/rho - 3/2 |j|^2/rho) and
// fd_s = w_s (3 c.F - 3 F.u + 9 (c.u)(c.F)).
//
// Adjoint, lam^t = dL/df^t, from lam^{t+1}:
//   mu_s(x)  = lam^{t+1}_s(x + c_s), or lam^{t+1}_opp(s)(x) when blocked   (streaming transposed)
//   nu_s     = (1 - sig) mu_s
//   A_rho    = sum_s nu_s (omega deq_s/drho + (1 - omega/2) dfd_s/drho)
//   A_j      = sum_s nu_s (omega deq_s/dj   + (1 - omega/2) dfd_s/dj)
//   lam^t_k  = (1 - omega) nu_k + sig mu_opp(k) + A_rho + A_j . c_k + dL_t/df_k
//   dL/dF   += (1 - omega/2) sum_s nu_s dfd_s/dF|_j + A_j / 2 + dL_t/dF
//   dL/dsig += sum_s mu_s (f_opp(s) - C_s)
// where deq_s/drho = w_s (1 - 9/2 (c.u)^2 + 3/2 |u|^2),
//       deq_s/dj   = w_s (3 c + 9 (c.u) c - 3 u),
//       dfd_s/dj   = w_s (9 (c.F) c - 3 F) / rho,
//       dfd_s/drho = w_s (3 F.u - 9 (c.u)(c.F)) / rho,
//       dfd_s/dF   = w_s (3 c - 3 u + 9 (c.u) c).
// Loss terms at step t (weight tw, spatial weights W):
//   velocity:  L_t = tw sum_x W(x) . u(x)        dL/df_k = tw W.(c_k - u)/rho, dL/dF = tw W/(2 rho)
//   energy:    L_t = tw sum_x W_0(x) rho|u|^2/2   dL/df_k = tw W_0 (u.c_k - |u|^2/2), dL/dF = tw W_0 u/2
// adjoint_step_kernel works in FP64.  adjoint_step_f32_kernel is the same
// step with lam and the arithmetic in FP32, written on the deviations
// g_s = f_s - w_s (the shifted storage formats hold exactly these), so that
// f_opp(s) - C_s = g_opp(s) - (C_s - w_s) has no cancellation against w; its
// gradients are still accumulated in FP64.  f^t may be stored in any storage
// format.
#include <cuda_runtime.h>

#include "../../include/lbm_gb300.h"
#include "lbm_adjoint.cuh"
#include "lbm_aux.cuh"

namespace lbm {

template <int Q, int ST>
__global__ void __launch_bounds__(128) adjoint_step_kernel(AdjParams a)
{
   const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   int x, y, z;
   if (!cell_xyz(a.g, c, x, y, z)) return;
   const uint32_t lk = a.links ? a.links[c] : 0u;
   if (lk & kSolidBit) {
#pragma unroll
      for (int s = 0; s < Q; s++) a.lam[(int64_t)s * a.g.plane + c] = 0.0;
      return;
   }
   double f[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) f[s] = load_pop<ST>(a.state, (int64_t)s * a.g.plane + c, lat_w(Q, s));
   double F[3] = {a.F[0], a.F[1], a.F[2]};
   if (a.force_field) {
      F[0] += a.force_field[c];
      F[1] += a.force_field[a.g.plane + c];
      F[2] += a.force_field[2 * a.g.plane + c];
   }
   const double sig = a.porosity ? a.porosity[c] : 0.0;
   double rho = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
   for (int s = 0; s < Q; s++) {
      rho += f[s];
      j[0] += f[s] * lat_c(Q, s, 0);
      j[1] += f[s] * lat_c(Q, s, 1);
      j[2] += f[s] * lat_c(Q, s, 2);
   }
   const double ir = 1.0 / rho;
   double u[3];
#pragma unroll
   for (int d = 0; d < 3; d++) {
      j[d] += 0.5 * F[d];
      u[d] = j[d] * ir;
   }
   const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
   const double Fu = F[0] * u[0] + F[1] * u[1] + F[2] * u[2];
   const double om = a.omega, om1 = 1.0 - om, om2 = 1.0 - 0.5 * om;

   double lam[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) lam[s] = 0.0;
   double gF[3] = {0.0, 0.0, 0.0};
   double gsig = 0.0;

   if (a.collide) {
      // mu: streaming transposed
      double mu[Q];
#pragma unroll
      for (int s = 0; s < Q; s++) {
         if (s == lat_rest(Q)) {
            mu[s] = a.lam_next[(int64_t)s * a.g.plane + c];
         } else if ((lk >> s) & 1u) {
            mu[s] = a.lam_next[(int64_t)lat_opp(Q, s) * a.g.plane + c];
         } else {
            const int64_t n = nbr_cell(a.g, x, y, z, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2));
            mu[s] = a.lam_next[(int64_t)s * a.g.plane + n];
         }
      }
      double Arho = 0.0, Aj[3] = {0.0, 0.0, 0.0}, GF[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const double c0 = lat_c(Q, s, 0), c1 = lat_c(Q, s, 1), c2 = lat_c(Q, s, 2);
         const double w = lat_w(Q, s);
         const double cu = c0 * u[0] + c1 * u[1] + c2 * u[2];
         const double cF = c0 * F[0] + c1 * F[1] + c2 * F[2];
         const double cj = c0 * j[0] + c1 * j[1] + c2 * j[2];
         // C_s for the porosity gradient
         const double eq = w * (rho + 3.0 * cj + 4.5 * cj * cu - 1.5 * uu * rho);
         const double fd = w * (3.0 * cF - 3.0 * Fu + 9.0 * cu * cF);
         const double Cs = om1 * f[s] + om * eq + om2 * fd;
         gsig += mu[s] * (f[lat_opp(Q, s)] - Cs);
         const double nu = (1.0 - sig) * mu[s];
         lam[s] += om1 * nu;
         lam[lat_opp(Q, s)] += sig * mu[s];
         // d/drho and d/dj of omega eq + om2 fd
         const double deq_drho = w * (1.0 - 4.5 * cu * cu + 1.5 * uu);
         const double dfd_drho = w * (3.0 * Fu - 9.0 * cu * cF) * ir;
         Arho += nu * (om * deq_drho + om2 * dfd_drho);
         const double ce = 3.0 + 9.0 * cu;      // coefficient of c in deq/dj (over w)
         const double cfd = 9.0 * cF * ir;      // coefficient of c in dfd/dj (over w)
         const double kc = nu * w * (om * ce + om2 * cfd);
         Aj[0] += kc * c0 - nu * w * (om * 3.0 * u[0] + om2 * 3.0 * F[0] * ir);
         Aj[1] += kc * c1 - nu * w * (om * 3.0 * u[1] + om2 * 3.0 * F[1] * ir);
         Aj[2] += kc * c2 - nu * w * (om * 3.0 * u[2] + om2 * 3.0 * F[2] * ir);
         // explicit dfd/dF at fixed j: w (3 c - 3 u + 9 (c.u) c)
         const double kf = nu * om2 * w;
         GF[0] += kf * (3.0 * c0 - 3.0 * u[0] + 9.0 * cu * c0);
         GF[1] += kf * (3.0 * c1 - 3.0 * u[1] + 9.0 * cu * c1);
         GF[2] += kf * (3.0 * c2 - 3.0 * u[2] + 9.0 * cu * c2);
      }
#pragma unroll
      for (int s = 0; s < Q; s++)
         lam[s] += Arho + Aj[0] * lat_c(Q, s, 0) + Aj[1] * lat_c(Q, s, 1) + Aj[2] * lat_c(Q, s, 2);
#pragma unroll
      for (int d = 0; d < 3; d++) gF[d] = GF[d] + 0.5 * Aj[d];
   }

   // loss at this step
   if (a.loss_kind == LBM_LOSS_VELOCITY && a.loss_weight) {
      const double W[3] = {a.loss_weight[c], a.loss_weight[a.g.plane + c], a.loss_weight[2 * a.g.plane + c]};
      const double tw = a.time_weight;
      const double Wu = W[0] * u[0] + W[1] * u[1] + W[2] * u[2];
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const double Wc = W[0] * lat_c(Q, s, 0) + W[1] * lat_c(Q, s, 1) + W[2] * lat_c(Q, s, 2);
         lam[s] += tw * (Wc - Wu) * ir;
      }
#pragma unroll
      for (int d = 0; d < 3; d++) gF[d] += tw * W[d] * 0.5 * ir;
   } else if (a.loss_kind == LBM_LOSS_ENERGY && a.loss_weight) {
      const double tw = a.time_weight * a.loss_weight[c];
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const double uc = u[0] * lat_c(Q, s, 0) + u[1] * lat_c(Q, s, 1) + u[2] * lat_c(Q, s, 2);
         lam[s] += tw * (uc - 0.5 * uu);
      }
#pragma unroll
      for (int d = 0; d < 3; d++) gF[d] += tw * 0.5 * u[d];
   }

#pragma unroll
   for (int s = 0; s < Q; s++) a.lam[(int64_t)s * a.g.plane + c] = lam[s];
   if (a.grad_force) {
#pragma unroll
      for (int d = 0; d < 3; d++) a.grad_force[(int64_t)d * a.g.plane + c] += gF[d];
   }
   if (a.grad_porosity) a.grad_porosity[c] += gsig;
}

// FP32 deviation g = f - w of a stored population.
template <int ST>
__device__ __forceinline__ float load_dev(const void* buf, int64_t idx, double w)
{
   if constexpr (ST == ST_F64) {
      return (float)(static_cast<const double*>(buf)[idx] - w);
   } else {
      return load_shifted(static_cast<const typename Store<ST>::T*>(buf) + idx);
   }
}

template <int Q, int ST>
__global__ void __launch_bounds__(256) adjoint_step_f32_kernel(AdjParams a)
{
   const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   int x, y, z;
   if (!cell_xyz(a.g, c, x, y, z)) return;
   const uint32_t lk = a.links ? a.links[c] : 0u;
   if (lk & kSolidBit) {
#pragma unroll
      for (int s = 0; s < Q; s++) a.lam_f[(int64_t)s * a.g.plane + c] = 0.0f;
      return;
   }
   float g[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) g[s] = load_dev<ST>(a.state, (int64_t)s * a.g.plane + c, lat_w(Q, s));
   float F[3] = {(float)a.F[0], (float)a.F[1], (float)a.F[2]};
   if (a.force_field) {
      F[0] = (float)(a.F[0] + a.force_field[c]);
      F[1] = (float)(a.F[1] + a.force_field[a.g.plane + c]);
      F[2] = (float)(a.F[2] + a.force_field[2 * a.g.plane + c]);
   }
   const float sig = a.porosity ? (float)a.porosity[c] : 0.0f;
   float drho = 0.0f, j[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
   for (int s = 0; s < Q; s++) {
      drho += g[s];
      j[0] += g[s] * (float)lat_c(Q, s, 0);
      j[1] += g[s] * (float)lat_c(Q, s, 1);
      j[2] += g[s] * (float)lat_c(Q, s, 2);
   }
   const float rho = 1.0f + drho;
   const float ir = 1.0f / rho;
   float u[3];
#pragma unroll
   for (int d = 0; d < 3; d++) {
      j[d] += 0.5f * F[d];
      u[d] = j[d] * ir;
   }
   const float uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
   const float Fu = F[0] * u[0] + F[1] * u[1] + F[2] * u[2];
   const float om = (float)a.omega, om1 = (float)(1.0 - a.omega), om2 = (float)(1.0 - 0.5 * a.omega);

   float lam[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) lam[s] = 0.0f;
   float gF[3] = {0.0f, 0.0f, 0.0f};
   float gsig = 0.0f;

   if (a.collide) {
      float mu[Q];
#pragma unroll
      for (int s = 0; s < Q; s++) {
         if (s == lat_rest(Q)) {
            mu[s] = a.lam_next_f[(int64_t)s * a.g.plane + c];
         } else if ((lk >> s) & 1u) {
            mu[s] = a.lam_next_f[(int64_t)lat_opp(Q, s) * a.g.plane + c];
         } else {
            const int64_t n = nbr_cell(a.g, x, y, z, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2));
            mu[s] = a.lam_next_f[(int64_t)s * a.g.plane + n];
         }
      }
      float Arho = 0.0f, Aj[3] = {0.0f, 0.0f, 0.0f}, GF[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const float c0 = (float)lat_c(Q, s, 0), c1 = (float)lat_c(Q, s, 1), c2 = (float)lat_c(Q, s, 2);
         const float w = (float)lat_w(Q, s);
         const float cu = c0 * u[0] + c1 * u[1] + c2 * u[2];
         const float cF = c0 * F[0] + c1 * F[1] + c2 * F[2];
         const float cj = c0 * j[0] + c1 * j[1] + c2 * j[2];
         // C_s - w_s for the porosity gradient
         const float eqd = w * (drho + 3.0f * cj + 4.5f * cj * cu - 1.5f * uu * rho);
         const float fd = w * (3.0f * cF - 3.0f * Fu + 9.0f * cu * cF);
         const float Cd = om1 * g[s] + om * eqd + om2 * fd;
         gsig += mu[s] * (g[lat_opp(Q, s)] - Cd);
         const float nu = (1.0f - sig) * mu[s];
         lam[s] += om1 * nu;
         lam[lat_opp(Q, s)] += sig * mu[s];
         const float deq_drho = w * (1.0f - 4.5f * cu * cu + 1.5f * uu);
         const float dfd_drho = w * (3.0f * Fu - 9.0f * cu * cF) * ir;
         Arho += nu * (om * deq_drho + om2 * dfd_drho);
         const float kc = nu * w * (om * (3.0f + 9.0f * cu) + om2 * 9.0f * cF * ir);
         Aj[0] += kc * c0 - nu * w * (om * 3.0f * u[0] + om2 * 3.0f * F[0] * ir);
         Aj[1] += kc * c1 - nu * w * (om * 3.0f * u[1] + om2 * 3.0f * F[1] * ir);
         Aj[2] += kc * c2 - nu * w * (om * 3.0f * u[2] + om2 * 3.0f * F[2] * ir);
         const float kf = nu * om2 * w;
         GF[0] += kf * (3.0f * c0 - 3.0f * u[0] + 9.0f * cu * c0);
         GF[1] += kf * (3.0f * c1 - 3.0f * u[1] + 9.0f * cu * c1);
         GF[2] += kf * (3.0f * c2 - 3.0f * u[2] + 9.0f * cu * c2);
      }
#pragma unroll
      for (int s = 0; s < Q; s++)
         lam[s] += Arho + Aj[0] * (float)lat_c(Q, s, 0) + Aj[1] * (float)lat_c(Q, s, 1) +
                   Aj[2] * (float)lat_c(Q, s, 2);
#pragma unroll
      for (int d = 0; d < 3; d++) gF[d] = GF[d] + 0.5f * Aj[d];
   }

   if (a.loss_kind == LBM_LOSS_VELOCITY && a.loss_weight) {
      const float tw = (float)a.time_weight;
      const float W[3] = {(float)a.loss_weight[c], (float)a.loss_weight[a.g.plane + c],
                          (float)a.loss_weight[2 * a.g.plane + c]};
      const float Wu = W[0] * u[0] + W[1] * u[1] + W[2] * u[2];
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const float Wc = W[0] * (float)lat_c(Q, s, 0) + W[1] * (float)lat_c(Q, s, 1) + W[2] * (float)lat_c(Q, s, 2);
         lam[s] += tw * (Wc - Wu) * ir;
      }
#pragma unroll
      for (int d = 0; d < 3; d++) gF[d] += tw * W[d] * 0.5f * ir;
   } else if (a.loss_kind == LBM_LOSS_ENERGY && a.loss_weight) {
      const float tw = (float)(a.time_weight * a.loss_weight[c]);
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const float uc = u[0] * (float)lat_c(Q, s, 0) + u[1] * (float)lat_c(Q, s, 1) + u[2] * (float)lat_c(Q, s, 2);
         lam[s] += tw * (uc - 0.5f * uu);
      }
#pragma unroll
      for (int d = 0; d < 3; d++) gF[d] += tw * 0.5f * u[d];
   }

#pragma unroll
   for (int s = 0; s < Q; s++) a.lam_f[(int64_t)s * a.g.plane + c] = lam[s];
   if (a.grad_force) {
#pragma unroll
      for (int d = 0; d < 3; d++) a.grad_force[(int64_t)d * a.g.plane + c] += (double)gF[d];
   }
   if (a.grad_porosity) a.grad_porosity[c] += (double)gsig;
}

// Loss value of the current state (FP64 partial sums per block).
template <int Q, int ST>
__global__ void __launch_bounds__(kReduceThreads) loss_partial_kernel(AdjParams a, double* partials)
{
   double acc = 0.0;
   for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.g.ncell;
        c += (int64_t)gridDim.x * blockDim.x) {
      const uint32_t lk = a.links ? a.links[c] : 0u;
      if (lk & kSolidBit) continue;
      double rho = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const double f = load_pop<ST>(a.state, (int64_t)s * a.g.plane + c, lat_w(Q, s));
         rho += f;
         j[0] += f * lat_c(Q, s, 0);
         j[1] += f * lat_c(Q, s, 1);
         j[2] += f * lat_c(Q, s, 2);
      }
      double F[3] = {a.F[0], a.F[1], a.F[2]};
      if (a.force_field) {
         F[0] += a.force_field[c];
         F[1] += a.force_field[a.g.plane + c];
         F[2] += a.force_field[2 * a.g.plane + c];
      }
      double u[3];
      for (int d = 0; d < 3; d++) u[d] = (j[d] + 0.5 * F[d]) / rho;
      if (a.loss_kind == LBM_LOSS_VELOCITY) {
         acc += a.loss_weight[c] * u[0] + a.loss_weight[a.g.plane + c] * u[1] +
                a.loss_weight[2 * a.g.plane + c] * u[2];
      } else {
         acc += a.loss_weight[c] * 0.5 * rho * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
      }
   }
   __shared__ double sh[kReduceThreads / 32];
   for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, off);
   if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
   __syncthreads();
   if (threadIdx.x == 0) {
      double v = 0.0;
      for (int w = 0; w < kReduceThreads / 32; w++) v += sh[w];
      partials[blockIdx.x] = v * a.time_weight;
   }
}

__global__ void sum_partials_kernel(const double* partials, int n, double* out)
{
   __shared__ double sh[kReduceThreads];
   double v = 0.0;
   for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
   sh[threadIdx.x] = v;
   __syncthreads();
   for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
      if ((int)threadIdx.x < stride) sh[threadIdx.x] += sh[threadIdx.x + stride];
      __syncthreads();
   }
   if (threadIdx.x == 0) out[0] = sh[0];
}

template <int Q, int ST>
cudaError_t launch_adjoint_t(const AdjParams& a, cudaStream_t st)
{
   adjoint_step_kernel<Q, ST><<<(unsigned)((a.g.ncell + 127) / 128), 128, 0, st>>>(a);
   return cudaGetLastError();
}

template <int Q, int ST>
cudaError_t launch_adjoint_f32_t(const AdjParams& a, cudaStream_t st)
{
   adjoint_step_f32_kernel<Q, ST><<<(unsigned)((a.g.ncell + 255) / 256), 256, 0, st>>>(a);
   return cudaGetLastError();
}

template <int Q, int ST>
cudaError_t launch_loss_t(const AdjParams& a, double* partials, int nblocks, double* out, cudaStream_t st)
{
   loss_partial_kernel<Q, ST><<<nblocks, kReduceThreads, 0, st>>>(a, partials);
   sum_partials_kernel<<<1, kReduceThreads, 0, st>>>(partials, nblocks, out);
   return cudaGetLastError();
}

#define LBM_ADJ_DISPATCH(FN, ...)                                                        \
   switch (Q * 10 + st) {                                                                \
      case 190: return FN<19, ST_F64>(__VA_ARGS__);                                      \
      case 191: return FN<19, ST_F32>(__VA_ARGS__);                                      \
      case 192: return FN<19, ST_BF16>(__VA_ARGS__);                                     \
      case 193: return FN<19, ST_F16>(__VA_ARGS__);                                      \
      case 270: return FN<27, ST_F64>(__VA_ARGS__);                                      \
      case 271: return FN<27, ST_F32>(__VA_ARGS__);                                      \
      case 272: return FN<27, ST_BF16>(__VA_ARGS__);                                     \
      default: return FN<27, ST_F16>(__VA_ARGS__);                                       \
   }

cudaError_t launch_adjoint(int Q, int st, const AdjParams& a, cudaStream_t stream)
{
   LBM_ADJ_DISPATCH(launch_adjoint_t, a, stream)
}

cudaError_t launch_adjoint_f32(int Q, int st, const AdjParams& a, cudaStream_t stream)
{
   LBM_ADJ_DISPATCH(launch_adjoint_f32_t, a, stream)
}

cudaError_t launch_loss(int Q, int st, const AdjParams& a, double* partials, int nblocks, double* out,
                        cudaStream_t stream)
{
   LBM_ADJ_DISPATCH(launch_loss_t, a, partials, nblocks, out, stream)
}

}  // namespace lbm
