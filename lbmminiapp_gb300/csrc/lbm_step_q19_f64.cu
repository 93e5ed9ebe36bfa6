// D3Q19 step kernels with FP64 population storage (exact FP64 and F64X arithmetic).
#include "lbm_dispatch.cuh"

namespace lbm {

cudaError_t launch_step_q19_f64(int arith, int kind, const Launch& L, const KParams& p,
                                const void* src, void* dst, bool links, bool fields)
{
   if (arith == AR_F64X) return launch_step_t<19, ST_F64, AR_F64X>(kind, L, p, src, dst, links, fields);
   return launch_step_t<19, ST_F64, AR_F64>(kind, L, p, src, dst, links, fields);
}

}  // namespace lbm
