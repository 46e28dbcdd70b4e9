// fv_control.cuh -- the per-step control arithmetic of one problem (dt from
// the fused CFL reduction, the loop bound, the active flag), shared by the
// control kernels (fv_aux.cu) and the persistent multi-step kernel
// (fv_batch32.cu) so that both take bit-identical steps.  IEEE double
// operations are written as intrinsics: the including files differ in their
// contraction and fast-math settings.
#pragma once

#include "fv_device.cuh"

namespace fv {

// dt and the active flag of the step a problem is about to take, from its
// control block's constants, the given time / step counter / error flag and
// the reduced CFL maximum in c.slot[step & 1]:
// dt = CFL / max(inv_hyp, inv_tc, inv_visc) (ComputeDt.h:62) and the loop
// bound t + epsilon < tend (main.cpp:51) or the fixed-step mode.  mode 0
// takes dt_given (mode_override 0) or c.dt_given.  bad: a non-finite dt was
// met (the step is then inactive).
__device__ __forceinline__ void step_decide(const StepCtrl& c, double t, long long step, int err,
                                            int mode_override, double dt_given, double& dt, int& active,
                                            bool& bad) {
  const int p = (int)(step & 1);
  const int mode = mode_override >= 0 ? mode_override : c.mode;
  bad = false;
  if (mode == 0) {
    dt = mode_override == 0 ? dt_given : c.dt_given;
    active = 1;
    return;
  }
  const double inv_hyp = __longlong_as_double((long long)c.slot[p]);
  double m = inv_hyp;
  if (c.inv_tc > m) m = c.inv_tc;
  if (c.inv_visc > m) m = c.inv_visc;
  dt = __ddiv_rn(c.cfl, m);
  // mode 2: fixed step count, no time bound; a previous error stops it
  active = mode == 2 ? !err : (__dadd_rn(t, c.epsilon) < c.tend) && (c.max_steps <= 0 || step < c.max_steps);
  if (active && !(dt > 0.0 && dt <= 1.0e300)) {
    bad = true;
    active = 0;
  }
}

// The control step of one problem: dt, active flag, parity, time and step
// counter, next reduction slot cleared.
__device__ __forceinline__ void step_control(StepCtrl& c, int mode_override, double dt_given) {
  const int p = (int)(c.step & 1);
  double dt;
  int active;
  bool bad;
  step_decide(c, c.t, c.step, c.err, mode_override, dt_given, dt, active, bad);
  if (bad) c.err |= 1;
  c.slot[p ^ 1] = 0ull;
  c.parity = p;
  c.active = active;
  c.dt_cur = active ? dt : 0.0;
  if (active) {
    c.t = __dadd_rn(c.t, dt);
    c.step = c.step + 1;
  }
}

}  // namespace fv
