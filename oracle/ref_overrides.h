/*
 * Force-included (-include) ahead of every reference translation unit that
 * the oracle recipe compiles.  It turns the reference's two compile-time
 * physics constants into run-time variables so one build of the reference
 * kernels serves every test configuration:
 *
 *   _OMEGA_   (src/Parameters.hh:26-28, #ifndef-guarded)  -> lbm_ref_omega
 *   _GRAVITY_ (src/Parameters.hh:36, unguarded #define)    -> lbm_ref_gravity
 *
 * _OMEGA_ is defined before Parameters.hh is read, which its guard honours;
 * _GRAVITY_ is re-defined after Parameters.hh, whose include guard keeps the
 * later #include lines from restoring the constant.  The arithmetic the
 * kernels perform is unchanged: with IEEE semantics (no -ffast-math, no FMA
 * contraction) an expression such as (1.0-_OMEGA_) evaluates to the same
 * double whether it is folded at compile time or computed at run time.
 *
 * Test infrastructure only.
 */
#ifndef LBM_REF_OVERRIDES_H
#define LBM_REF_OVERRIDES_H

extern double lbm_ref_omega;
extern double lbm_ref_gravity;

#define _OMEGA_ lbm_ref_omega
#include "Parameters.hh"
#undef _GRAVITY_
#define _GRAVITY_ lbm_ref_gravity

#endif
