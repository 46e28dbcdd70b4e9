// fv_pack32.cuh -- two FP32 Riemann solves in one: the packed FP32x2
// arithmetic of the sm_100 family (FADD2 / FMUL2 / FFMA2, one instruction for
// two lanes of a float2) applied to two independent faces.
//
// The column-marching mixed stage solves, per lane and row, one a face and
// one b face; their states are independent, so each arithmetic step of HLL /
// HLLC (RiemannSolvers.h) is issued once for both.  Square roots,
// reciprocals, min / max and the region selection stay per component (the
// region selection becomes selects instead of branches).  The formulas are
// those of hll32 / hllc32 (fv_tile32.cuh); contraction into FFMA2 is written
// out where the scalar code lets the compiler contract.
#pragma once

#include "fv_tile32.cuh"

namespace fv {

struct F2 {
  float2 v;
};

__device__ __forceinline__ F2 f2(float a, float b) { return F2{make_float2(a, b)}; }
__device__ __forceinline__ F2 f2s(float a) { return F2{make_float2(a, a)}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2{__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2{__fmul2_rn(a.v, b.v)}; }
// a - b as a + (-1) b: the product is exact, one rounding
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2{__ffma2_rn(b.v, make_float2(-1.0f, -1.0f), a.v)}; }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return F2{__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 min2(F2 a, F2 b) { return f2(fminf(a.v.x, b.v.x), fminf(a.v.y, b.v.y)); }
__device__ __forceinline__ F2 max2(F2 a, F2 b) { return f2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y)); }
__device__ __forceinline__ F2 rcp2(F2 a) { return f2(1.0f / a.v.x, 1.0f / a.v.y); }
__device__ __forceinline__ F2 sqrt2(F2 a) { return f2(sqrtf(a.v.x), sqrtf(a.v.y)); }

// Per-component selection: m.x / m.y choose a over b.
struct M2 {
  bool x, y;
};
__device__ __forceinline__ M2 gt0(F2 a) { return M2{a.v.x > 0.0f, a.v.y > 0.0f}; }
__device__ __forceinline__ M2 ge0(F2 a) { return M2{a.v.x >= 0.0f, a.v.y >= 0.0f}; }
__device__ __forceinline__ M2 le0(F2 a) { return M2{a.v.x <= 0.0f, a.v.y <= 0.0f}; }
__device__ __forceinline__ M2 operator||(M2 a, M2 b) { return M2{a.x || b.x, a.y || b.y}; }
__device__ __forceinline__ F2 sel(M2 m, F2 a, F2 b) { return f2(m.x ? a.v.x : b.v.x, m.y ? a.v.y : b.v.y); }

// Slots of two faces packed component by component.
__device__ __forceinline__ Slots<F2> pack_slots(const Slots<float>& a, const Slots<float>& b) {
  Slots<F2> s;
  s.r = f2(a.r, b.r);
  s.un = f2(a.un, b.un);
  s.t1 = f2(a.t1, b.t1);
  s.t2 = f2(a.t2, b.t2);
  s.p = f2(a.p, b.p);
  return s;
}

// hll32 for two faces at once (fluxes in slot order: flux[v].v.x, .v.y).
__device__ __forceinline__ void hll_pair(const Slots<F2>& qL, const Slots<F2>& qR, float gamma, float inv_gm1,
                                         F2 flux[5]) {
  const F2 half = f2s(0.5f), g = f2s(gamma), ig = f2s(inv_gm1);
  auto state = [&](const Slots<F2>& q, F2& c, F2& E, F2 F[5]) {
    c = sqrt2(g * q.p * rcp2(q.r));
    E = fma2(q.p, ig, half * q.r * fma2(q.t2, q.t2, fma2(q.t1, q.t1, q.un * q.un)));
    F[0] = q.r * q.un;
    F[1] = fma2(F[0], q.un, q.p);
    F[2] = F[0] * q.t1;
    F[3] = F[0] * q.t2;
    F[4] = (q.p + E) * q.un;
  };
  F2 cL, cR, EL, ER, FL[5], FR[5];
  state(qL, cL, EL, FL);
  state(qR, cR, ER, FR);
  const F2 SL = min2(qL.un - cL, qR.un - cR);
  const F2 SR = max2(qL.un + cL, qR.un + cR);
  const F2 uL[5] = {qL.r, FL[0], qL.r * qL.t1, qL.r * qL.t2, EL};
  const F2 uR[5] = {qR.r, FR[0], qR.r * qR.t1, qR.r * qR.t2, ER};
  const F2 inv = rcp2(SR - SL);
  const F2 slsr = SL * SR;
  const M2 left = ge0(SL), right = le0(SR);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const F2 mid = fma2(slsr, uR[v] - uL[v], SR * FL[v] - SL * FR[v]) * inv;
    flux[v] = sel(left, FL[v], sel(right, FR[v], mid));
  }
}

// hllc32 (reference form: kinetic energy of the normal and first transverse
// velocity) for two faces at once.
__device__ __forceinline__ void hllc_pair(const Slots<F2>& L, const Slots<F2>& R, float gamma, float inv_gm1,
                                          F2 flux[5]) {
  const F2 half = f2s(0.5f), ig = f2s(inv_gm1);
  const F2 kL = fma2(L.t1, L.t1, L.un * L.un);
  const F2 kR = fma2(R.t1, R.t1, R.un * R.un);
  const F2 EL = fma2(L.p, ig, half * L.r * kL);
  const F2 ER = fma2(R.p, ig, half * R.r * kR);
  const F2 cmax = sqrt2(f2s(gamma) * max2(L.p * rcp2(L.r), R.p * rcp2(R.r)));
  const F2 SL = min2(L.un, R.un) - cmax;
  const F2 SR = max2(L.un, R.un) + cmax;
  const F2 rcL = L.r * (L.un - SL);
  const F2 rcR = R.r * (SR - R.un);
  const F2 iD = rcp2(rcR + rcL);
  const F2 uS = fma2(rcR, R.un, fma2(rcL, L.un, L.p - R.p)) * iD;
  const F2 pS = fma2(rcL * rcR, L.un - R.un, fma2(rcR, L.p, rcL * R.p)) * iD;
  // star state of the side the contact leaves behind (left when uS > 0)
  const M2 left = gt0(uS);
  const F2 rK = sel(left, L.r, R.r), uK = sel(left, L.un, R.un), pK = sel(left, L.p, R.p);
  const F2 EK = sel(left, EL, ER), SK = sel(left, SL, SR);
  const F2 inv = rcp2(SK - uS);
  const F2 sKu = SK - uK;
  const F2 srS = rK * sKu * inv;
  const F2 ES = (fma2(sKu, EK, pS * uS) - pK * uK) * inv;
  const F2 t1S = sel(left, L.t1, R.t1), t2S = sel(left, L.t2, R.t2);
  // regions: SL > 0 -> L; else uS > 0 or SR > 0 -> star; else R
  const M2 isL = gt0(SL), isS = left || gt0(SR);
  const F2 sr = sel(isL, L.r, sel(isS, srS, R.r));
  const F2 su = sel(isL, L.un, sel(isS, uS, R.un));
  const F2 st1 = sel(isL, L.t1, sel(isS, t1S, R.t1));
  const F2 st2 = sel(isL, L.t2, sel(isS, t2S, R.t2));
  const F2 sp = sel(isL, L.p, sel(isS, pS, R.p));
  const F2 E = sel(isL, EL, sel(isS, ES, ER));
  flux[0] = sr * su;
  flux[1] = fma2(flux[0], su, sp);
  flux[2] = flux[0] * st1;
  flux[3] = flux[0] * st2;
  flux[4] = (E + sp) * su;
}

}  // namespace fv
