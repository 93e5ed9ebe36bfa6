// Host build of the F64X collision (lbmminiapp_gb300/csrc/lbm_f64x.cuh) for
// tests/test_f64x_host.py: runs collide_f64x_fast on the CPU so its precision
// and its fallback conditions can be checked without a GPU.
#include <cmath>
#include <cstdint>
#include <limits>

#include "lbm_f64x.cuh"

namespace {

int force_mode_of(const double* F, double omega)
{
   const double f[3] = {F[0], F[1], F[2]};
   return lbm::force_mode(f, omega);
}

template <int Q, bool ROLLED = false>
int run(const double* in, double* out, int n, double omega, const double* F, int compat, int force_mode, int* fast)
{
   using namespace lbm;
   x64::Consts k;
   k.om1 = x64::df_from_double(1.0 - omega);
   k.omega = x64::df_from_double(omega);
   for (int c = 0; c < 4; c++) {
      double w;
      if (Q == 19) w = c == 0 ? 1.0 / 3.0 : (c == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
      else w = c == 0 ? 8.0 / 27.0 : (c == 1 ? 2.0 / 27.0 : (c == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
      k.ow[c] = x64::df_from_double(omega * w);
   }
   for (int d = 0; d < 3; d++) k.F[d] = x64::df_from_double(F[d]);
   for (int s = 0; s < Q; s++) {
      const double cf = 3.0 * (lat_c(Q, s, 0) * F[0] + lat_c(Q, s, 1) * F[1] + lat_c(Q, s, 2) * F[2]);
      k.Kf[s] = x64::df_from_double((1.0 - 0.5 * omega) * lat_w(Q, s) * cf);
   }
   for (int d = 0; d < 3; d++) k.F3[d] = x64::df_from_double(3.0 * F[d]);
   for (int c = 0; c < 4; c++) {
      double w;
      if (Q == 19) w = c == 0 ? 1.0 / 3.0 : (c == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
      else w = c == 0 ? 8.0 / 27.0 : (c == 1 ? 2.0 / 27.0 : (c == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
      k.om2w[c] = x64::df_from_double((1.0 - 0.5 * omega) * w);
   }
   k.om2w36 = x64::df_from_double((1.0 - 0.5 * omega) / 36.0);
   k.om2 = (float)(1.0 - 0.5 * omega);
   const int mode = force_mode < 0 ? force_mode_of(F, omega) : force_mode;
   int nfast = 0;
   for (int i = 0; i < n; i++) {
      uint64_t bits[Q];
      for (int s = 0; s < Q; s++) bits[s] = x64::double_bits(in[(size_t)i * Q + s]);
      bool ok;
      if constexpr (ROLLED) {
         // the pair-class loops, with the forcing constants as a direction-indexed table
         float Kf[Q][2];
         for (int s = 0; s < Q; s++) {
            Kf[s][0] = k.Kf[s].h;
            Kf[s][1] = k.Kf[s].l;
         }
         EmitToArray<Q> em;
         const KeepInputs keep{};
         ok = mode == 2   ? collide_f64x_fast_emit<Q, 2, EmitToArray<Q>, KeepInputs, true>(bits, k, compat, em, keep, Kf)
              : mode == 1 ? collide_f64x_fast_emit<Q, 1, EmitToArray<Q>, KeepInputs, true>(bits, k, compat, em, keep, Kf)
                          : collide_f64x_fast_emit<Q, 0, EmitToArray<Q>, KeepInputs, true>(bits, k, compat, em, keep, Kf);
         if (ok)
            for (int s = 0; s < Q; s++) bits[s] = em.res[s];
      } else {
         ok = mode == 2   ? collide_f64x_fast<Q, 2>(bits, k, compat)
              : mode == 1 ? collide_f64x_fast<Q, 1>(bits, k, compat)
                          : collide_f64x_fast<Q, 0>(bits, k, compat);
      }
      fast[i] = ok ? 1 : 0;
      nfast += ok;
      for (int s = 0; s < Q; s++)
         out[(size_t)i * Q + s] = ok ? x64::as_double(bits[s]) : std::numeric_limits<double>::quiet_NaN();
   }
   return nfast;
}

}  // namespace

// force_mode: the fast path's forcing form (0, 1, 2 as lbm::force_mode), or
// -1 for the one the library picks for this force and omega.
extern "C" int f64x_collide_host(int Q, const double* in, double* out, int n, double omega, const double* F,
                                 int compat, int force_mode, int* fast)
{
   return Q == 19 ? run<19>(in, out, n, omega, F, compat, force_mode, fast)
                  : run<27>(in, out, n, omega, F, compat, force_mode, fast);
}

// The D3Q27 fast path with the pair-class loops (the rolled form the D3Q27
// step kernels run); same arguments as f64x_collide_host.
extern "C" int f64x_collide_host_q27_rolled(const double* in, double* out, int n, double omega, const double* F,
                                            int compat, int force_mode, int* fast)
{
   return run<27, true>(in, out, n, omega, F, compat, force_mode, fast);
}
