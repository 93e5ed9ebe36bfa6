// D3Q27 step kernels with shifted FP32 / BF16 / FP16 storage and FP32 arithmetic.
#include "lbm_dispatch.cuh"

namespace lbm {

cudaError_t launch_step_q27_low(int storage, int kind, const Launch& L, const KParams& p,
                                const void* src, void* dst, bool links, bool fields)
{
   switch (storage) {
      case ST_F32: return launch_step_t<27, ST_F32, AR_F32>(kind, L, p, src, dst, links, fields);
      case ST_BF16: return launch_step_t<27, ST_BF16, AR_F32>(kind, L, p, src, dst, links, fields);
      default: return launch_step_t<27, ST_F16, AR_F32>(kind, L, p, src, dst, links, fields);
   }
}

}  // namespace lbm
