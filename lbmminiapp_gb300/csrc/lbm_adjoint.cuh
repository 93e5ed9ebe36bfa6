// Parameters of the adjoint and loss kernels (lbm_adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include "lbm_aux.cuh"

namespace lbm {

struct AdjParams {
   GridDims g;
   double omega;
   double F[3];
   const uint32_t* links;
   const double* force_field;     // planar [3][plane] or null
   const double* porosity;        // [plane] or null
   const void* state;             // f^t, the handle's storage, slot s = direction s
   const double* lam_next;        // [Q][plane]
   double* lam;                   // [Q][plane]
   double* grad_force;            // [3][plane] accumulated, or null
   double* grad_porosity;         // [plane] accumulated, or null
   const double* loss_weight;     // velocity: [3][plane]; energy: [plane]; or null
   double time_weight;
   int loss_kind;
   int collide;                   // 0: loss term only (the last state of a rollout)
   const float* lam_next_f;       // FP32 adjoint: [Q][plane]
   float* lam_f;                  // FP32 adjoint: [Q][plane]
};

cudaError_t launch_adjoint(int Q, int storage, const AdjParams& a, cudaStream_t stream);
cudaError_t launch_adjoint_f32(int Q, int storage, const AdjParams& a, cudaStream_t stream);
cudaError_t launch_loss(int Q, int storage, const AdjParams& a, double* partials, int nblocks, double* out,
                        cudaStream_t stream);

}  // namespace lbm
