// fv_riemann64.cuh -- HLL and HLLC (RiemannSolvers.h) in FP64 with the
// reference's rounding and fewer FP64 instructions.
//
// States are in the slot order of the sweep (swap_component, States.h:104-111):
// r, normal velocity un, transverse t1, t2, p.  ZS names a transverse slot
// that is identically zero in a 2-D run without a third velocity (1: t1,
// 2: t2, 0: none); its terms are exact zeros in the reference arithmetic and
// are dropped.  Cheaper-but-identical steps, each returning the same bits:
//   - p/(gamma-1) via the corrected quotient with RN(1/(gamma-1));
//   - the five HLL flux components share one reciprocal of SR-SL, and each
//     state's sound speed and kinetic energy share one reciprocal of rho;
//   - HLLC's max(cL, cR) as sqrt(max(cL^2, cR^2)) (sqrt is monotone and
//     correctly rounded), and u*, p* / the star state share reciprocals;
//   - products with 0.5 by exponent arithmetic (half64, exact);
//   - HLLC's wave-speed min / max and region tests on bit patterns
//     (fmin_bits, gt0_bits, ...: integer pipe, same results; measured
//     +1-2 %).  HLL keeps the FP64 forms: there the bit-pattern min / max
//     measured 1 % slower.
#pragma once

#include "fv_device.cuh"
#include "fv_exact64.cuh"

namespace fv {

// (u^2 + t1^2) + t2^2 with the exact zero slot dropped.
template <int ZS>
__device__ __forceinline__ double ke_sum3(double un, double t1, double t2) {
  if (ZS == 1) return un * un + t2 * t2;
  if (ZS == 2) return un * un + t1 * t1;
  return (un * un + t1 * t1) + t2 * t2;
}

// computeFlux (States.h:114-127) given e = p/(gamma-1).
template <int ZS>
__device__ __forceinline__ void euler_flux64(const Slots<double>& q, double e, double F[5]) {
  const double Ek = half64(q.r) * ke_sum3<ZS>(q.un, q.t1, q.t2);
  const double E = e + Ek;
  F[0] = q.r * q.un;
  F[1] = F[0] * q.un + q.p;
  F[2] = ZS == 1 ? 0.0 : F[0] * q.t1;
  F[3] = ZS == 2 ? 0.0 : F[0] * q.t2;
  F[4] = (q.p + E) * q.un;
}

// primToCons (States.h:20-31) given e = p/(gamma-1) and y = RN(1/rho).
template <int ZS>
__device__ __forceinline__ void prim_to_cons64(const Slots<double>& q, double e, double y, double u[5]) {
  u[0] = q.r;
  u[1] = q.r * q.un;
  u[2] = ZS == 1 ? 0.0 : q.r * q.t1;
  u[3] = ZS == 2 ? 0.0 : q.r * q.t2;
  const double Ek = div_by_rcp(half64(ke_sum3<ZS>(u[1], u[2], u[3])), q.r, y);
  u[4] = Ek + e;
}

// HLL with Davis wave speeds, RiemannSolvers.h:6-36.
// pout, when given, receives the interface pressure of RiemannSolvers.h:24-33
// (used only by the z-boundary flux overrides of Update.h:131-143).
template <int ZS>
__device__ __forceinline__ void hll64(const Slots<double>& L, const Slots<double>& R, const Consts64& K,
                                      double flux[5], double* pout = nullptr) {
  // one correctly rounded reciprocal of each density serves both quotients by
  // it (the sound speed's p*gamma/rho and, in the star region, Ek/rho)
  const double yL = 1.0 / L.r, yR = 1.0 / R.r;
  const double aL = sqrt(div_by_rcp(L.p * K.gamma, L.r, yL));
  const double aR = sqrt(div_by_rcp(R.p * K.gamma, R.r, yR));
  const double SL = fmin(L.un - aL, R.un - aR);
  const double SR = fmax(L.un + aL, R.un + aR);
  const double eL = div_by_rcp(L.p, K.gm1, K.inv_gm1);
  const double eR = div_by_rcp(R.p, K.gm1, K.inv_gm1);
  double FL[5], FR[5];
  euler_flux64<ZS>(L, eL, FL);
  euler_flux64<ZS>(R, eR, FR);
  if (SL >= 0.0) {
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = FL[v];
    if (pout) *pout = L.p;
  } else if (SR <= 0.0) {
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = FR[v];
    if (pout) *pout = R.p;
  } else {
    if (pout) *pout = half64(L.p + R.p);
    double uL[5], uR[5];
    prim_to_cons64<ZS>(L, eL, yL, uL);
    prim_to_cons64<ZS>(R, eR, yR, uR);
    const double slsr = SL * SR;
    const double den = SR - SL;
    const double y = 1.0 / den;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if ((ZS == 1 && v == 2) || (ZS == 2 && v == 3)) {
        flux[v] = 0.0;
        continue;
      }
      flux[v] = div_by_rcp((FL[v] * SR - FR[v] * SL) + (uR[v] - uL[v]) * slsr, den, y);
    }
  }
}

// HLLC, RiemannSolvers.h:39-112; the kinetic energy uses un and t1 only, as
// the reference does.
// pout as for hll64 (RiemannSolvers.h:81-104: pL, p*, p*, pR by region).
// KE3 (corrected physics): the kinetic energy of all three velocities.
template <int ZS, bool KE3 = false>
__device__ __forceinline__ void hllc64(const Slots<double>& L, const Slots<double>& R, const Consts64& K,
                                       double flux[5], double* pout = nullptr) {
  const double rL = L.r, uL = L.un, pL = L.p;
  const double rR = R.r, uR = R.un, pR = R.p;
  const double kL = KE3 ? ke_sum3<ZS>(uL, L.t1, L.t2) : (ZS == 1 ? uL * uL : uL * uL + L.t1 * L.t1);
  const double kR = KE3 ? ke_sum3<ZS>(uR, R.t1, R.t2) : (ZS == 1 ? uR * uR : uR * uR + R.t1 * R.t1);
  const double EL = half64(rL) * kL + pL * K.inv_gm1;
  const double ER = half64(rR) * kR + pR * K.inv_gm1;
  const double c2L = pL * K.gamma / rL;
  const double c2R = pR * K.gamma / rR;
  const double cmax = sqrt(fmax_bits(c2L, c2R));
  const double SL = fmin_bits(uL, uR) - cmax;
  const double SR = fmax_bits(uL, uR) + cmax;
  const double rcL = rL * (uL - SL);
  const double rcR = rR * (SR - uR);
  const double D = rcR + rcL;
  const double yD = 1.0 / D;
  const double uS = div_by_rcp(rcR * uR + rcL * uL + (pL - pR), D, yD);
  const double pS = div_by_rcp(rcR * pL + rcL * pR + rcL * rcR * (uL - uR), D, yD);
  double sr, su, st1, st2, sp, E;
  if (gt0_bits(SL)) {
    sr = rL; su = uL; st1 = L.t1; st2 = L.t2; sp = pL; E = EL;
  } else if (gt0_bits(uS) || gt0_bits(SR)) {
    // star regions, tested in the reference's order: uS > 0 -> left star,
    // otherwise SR > 0 -> right star
    const bool left = gt0_bits(uS);
    const double rK = left ? rL : rR, uK = left ? uL : uR, pK = left ? pL : pR, EK = left ? EL : ER;
    const double SK = left ? SL : SR;
    const double den = SK - uS;
    const double y = 1.0 / den;
    sr = div_by_rcp(rK * (SK - uK), den, y);
    E = div_by_rcp((SK - uK) * EK - pK * uK + pS * uS, den, y);
    su = uS;
    sp = pS;
    st1 = left ? L.t1 : R.t1;
    st2 = left ? L.t2 : R.t2;
  } else {
    sr = rR; su = uR; st1 = R.t1; st2 = R.t2; sp = pR; E = ER;
  }
  if (pout) *pout = sp;
  flux[0] = sr * su;
  flux[1] = flux[0] * su + sp;
  flux[2] = ZS == 1 ? 0.0 : flux[0] * st1;
  flux[3] = ZS == 2 ? 0.0 : flux[0] * st2;
  flux[4] = (E + sp) * su;
}

}  // namespace fv
