// fv_tile32.cuh -- one stage of one tile in the FP32-mixed form.
//
// Same algorithm and order as fv_tile64.cuh (the reference's euler_step),
// with the precision split:
//   - U^n, the state carried from step to step, is an FP32 (hi, lo) pair per
//     value (float2, 8 bytes): about 48 significant bits, so accumulating
//     many small increments loses nothing measurable;
//   - U*, the RK2 intermediate, is plain FP32 (4 bytes): density and momenta
//     as conserved values, the energy slot holding the internal energy
//     E* - |m*|^2 / (2 rho*) rather than E* (see below);
//   - primitives, slopes, face states, the Riemann solvers, gravity, thermal
//     conduction and viscosity run in FP32 (fast-math division and sqrt);
//   - the RK2 combination 0.5*(U^n + U* + dU) and every update of U^n are
//     done on the (hi, lo) pairs with error-free two-sums (Knuth's TwoSum,
//     Dekker's Fast2Sum);
//   - the pressure recovery p = (gamma-1)(E - |m|^2 / (2 rho)) (States.h:42-43)
//     runs in double-float arithmetic: the kinetic energy is formed from the
//     (hi, lo) pairs of density and momenta as an unevaluated pair (exact
//     squares by FMA, a corrected quotient) and subtracted from E's pair, so
//     at high Mach, where E and the kinetic energy nearly cancel, p keeps
//     about 2^-24 relative accuracy (an FP32 kinetic energy would lose
//     2^-24 of E, i.e. 2^-24 gamma (gamma-1) M^2 / 2 of p).  U* keeps its
//     internal energy for the same reason: E* is rebuilt from it and the
//     stored density and momenta in the same double-float arithmetic;
//   - the CFL maximum is taken over FP32 cell values and turned into dt in
//     FP64 by the control kernel; conservation sums run in FP64.
// Per cell-update the state traffic is 8 (read U^n) + 4 (write U*) + 4 (read
// U*) + 8 (read U^n) + 8 (write U^n+1) = 32 bytes per stored field.
#pragma once

#include "fv_tile64.cuh"

// Cells whose loads one thread issues before converting any of them (phase 1),
// for (hi, lo) pair input.  Measured on shear 4096^2 / RT 512x1536 / Sedov
// 256^2: 3 cells +1.8 / +1.1 / +0.7 % over 2; 4 spill.
#ifndef FV_MIXED_LOAD_BATCH
#define FV_MIXED_LOAD_BATCH 3
#endif
// Minimum resident CTAs per SM requested from the register allocator
// (0: no bound beyond the 256 threads of a tile).
#ifndef FV_MIXED_MIN_CTAS
#define FV_MIXED_MIN_CTAS 4
#endif

namespace fv {

// Storage of one mixed-precision problem: U^n as (hi, lo) pairs, U* FP32.
struct MixedFields {
  float2* un[5];
  float* us[5];
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return make_float2(s, e);
}

// Dekker's Fast2Sum (|a| >= |b|): s + e == a + b exactly.
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return make_float2(s, e);
}

// (hi, lo) + x -> normalised (hi, lo).
__device__ __forceinline__ float2 pair_add(float2 a, float x) {
  const float2 s = two_sum(a.x, x);
  return fast_two_sum(s.x, s.y + a.y);
}

// (hi, lo) + (hi, lo) -> normalised (hi, lo).
__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {
  const float2 s = two_sum(a.x, b.x);
  return fast_two_sum(s.x, s.y + (a.y + b.y));
}

// ---- double-float kinetic energy and pressure recovery -------------------
// The products below use the _rn intrinsics, which the compiler never
// contracts into FMAs: an error-free transformation needs each rounding
// exactly where it is written (the files are built with FMA contraction).

// Exact square of h as an unevaluated pair (p, e): p = RN(h*h), e = h*h - p.
__device__ __forceinline__ float2 two_sq(float h) {
  const float p = __fmul_rn(h, h);
  return make_float2(p, __fmaf_rn(h, h, -p));
}

// |m|^2 / (2 rho) as an unevaluated pair, from pairs of the density and the
// three momenta (storage order; mc ignored unless WACT).  Relative error
// about 2^-44: sums of the exact squares by TwoSum, the cross terms 2 h l
// and the product errors folded into the low part, then one quotient
// corrected by its remainder (computed with FMAs).
template <bool WACT>
__device__ __forceinline__ float2 kinetic_pair(float2 r, float2 ma, float2 mb, float2 mc) {
  const float2 a = two_sq(ma.x), b = two_sq(mb.x);
  float2 s = two_sum(a.x, b.x);
  float lo = s.y + (a.y + b.y);
  lo = __fmaf_rn(2.0f * ma.x, ma.y, lo);
  lo = __fmaf_rn(2.0f * mb.x, mb.y, lo);
  if (WACT) {
    const float2 c = two_sq(mc.x);
    const float2 t = two_sum(s.x, c.x);
    s.x = t.x;
    lo = lo + t.y + c.y;
    lo = __fmaf_rn(2.0f * mc.x, mc.y, lo);
  }
  const float rinv = 1.0f / r.x;  // approximate: the remainder corrects q1
  const float q1 = __fmul_rn(s.x, rinv);
  const float rem = __fadd_rn(__fmaf_rn(-q1, r.x, s.x), __fmaf_rn(-q1, r.y, lo));
  const float q2 = __fmul_rn(rem, rinv);
  return make_float2(0.5f * q1, 0.5f * q2);
}

// E - Ek for an energy pair and a kinetic-energy pair: E.x - k.x is exact
// where they cancel (Sterbenz), so the result keeps 2^-24 of itself.
__device__ __forceinline__ float internal_energy(float2 E, float2 k) {
  return __fadd_rn(__fsub_rn(E.x, k.x), __fsub_rn(E.y, k.y));
}

// consToPrim (States.h:34-45) of a cell held as (hi, lo) pairs (U^n), storage
// order: velocities in FP32 from the rounded values, p from the double-float
// internal energy.
template <int PLANE, bool WACT>
__device__ __forceinline__ void cons_to_prim_pairs(const float2 w[5], float gm1, float q[5]) {
  const float r = w[0].x + w[0].y;
  const float rinv = 1.0f / r;
  q[0] = r;
  q[1] = (w[1].x + w[1].y) * rinv;
  q[2] = (w[2].x + w[2].y) * rinv;
  q[3] = WACT ? (w[3].x + w[3].y) * rinv : 0.0f;
  const float2 k = kinetic_pair<WACT>(w[0], w[1], w[2], WACT ? w[3] : make_float2(0.0f, 0.0f));
  q[4] = internal_energy(w[4], k) * gm1;
}

// consToPrim of a U* cell: conserved density and momenta, internal energy in
// the energy slot.
template <bool WACT>
__device__ __forceinline__ void cons_to_prim_star(const float u[5], float gm1, float q[5]) {
  const float r = u[0];
  const float rinv = 1.0f / r;
  q[0] = r;
  q[1] = u[1] * rinv;
  q[2] = u[2] * rinv;
  q[3] = WACT ? u[3] * rinv : 0.0f;
  q[4] = u[4] * gm1;
}

// The kinetic energy of a U* cell (FP32 values, exact as pairs).
template <bool WACT>
__device__ __forceinline__ float2 kinetic_star(const float u[5]) {
  return kinetic_pair<WACT>(make_float2(u[0], 0.0f), make_float2(u[1], 0.0f), make_float2(u[2], 0.0f),
                            make_float2(WACT ? u[3] : 0.0f, 0.0f));
}

// The CFL term (ComputeDt.h:28-54) of primitives in storage order.
template <int PLANE>
__device__ __forceinline__ float inv_dt_hyp_prim32(const float q[5], const Grid& G) {
  const float cs = sqrtf(q[4] * G.gamma_f / q[0]);
  const float vx = q[1], vy = PLANE == PLANE_XY ? q[2] : q[3], vz = PLANE == PLANE_XY ? q[3] : q[2];
  return (cs + fabsf(vx)) * G.inv_dx_f + (cs + fabsf(vy)) * G.inv_dy_f + (cs + fabsf(vz)) * G.inv_dz_f;
}

// The CFL term of a cell held as (hi, lo) pairs.
template <int PLANE, bool WACT>
__device__ __forceinline__ float inv_dt_hyp32(const float2 w[5], const Grid& G) {
  float q[5];
  cons_to_prim_pairs<PLANE, WACT>(w, G.gm1_f, q);
  return inv_dt_hyp_prim32<PLANE>(q, G);
}

// minmod (Update.h:73-80) in FP32: 0 when the signs differ, else the argument
// of smaller magnitude (ties to the second).
__device__ __forceinline__ float minmod32(float a, float b) {
  const float m = fabsf(a) < fabsf(b) ? a : b;
  return a * b < 0.0f ? 0.0f : m;
}

// Per-state quantities of the FP32 solvers: sound speed, total energy and
// the Euler flux (States.h:114-127) in the sweep's slot order.
struct State32 {
  float r, un, t1, t2, p, c, E, F[5];
};

__device__ __forceinline__ State32 state32(const Slots<float>& q, float gamma, float inv_gm1) {
  State32 s;
  s.r = q.r; s.un = q.un; s.t1 = q.t1; s.t2 = q.t2; s.p = q.p;
  const float rinv = 1.0f / q.r;
  s.c = sqrtf(gamma * q.p * rinv);
  s.E = q.p * inv_gm1 + 0.5f * q.r * (q.un * q.un + q.t1 * q.t1 + q.t2 * q.t2);
  s.F[0] = q.r * q.un;
  s.F[1] = s.F[0] * q.un + q.p;
  s.F[2] = s.F[0] * q.t1;
  s.F[3] = s.F[0] * q.t2;
  s.F[4] = (q.p + s.E) * q.un;
  return s;
}

// HLL with Davis wave speeds (RiemannSolvers.h:6-36) in FP32.  The conserved
// states of the star formula are (r, F0 = r un, r t1, r t2, E).
// pout (optional): the interface pressure of RiemannSolvers.h:24-33.
__device__ __forceinline__ void hll32(const Slots<float>& qL, const Slots<float>& qR, float gamma, float inv_gm1,
                                      float flux[5], float* pout = nullptr) {
  const State32 L = state32(qL, gamma, inv_gm1), R = state32(qR, gamma, inv_gm1);
  const float SL = fminf(L.un - L.c, R.un - R.c);
  const float SR = fmaxf(L.un + L.c, R.un + R.c);
  if (pout) *pout = SL >= 0.0f ? L.p : (SR <= 0.0f ? R.p : 0.5f * (L.p + R.p));
  if (SL >= 0.0f) {
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = L.F[v];
  } else if (SR <= 0.0f) {
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = R.F[v];
  } else {
    const float uL[5] = {L.r, L.F[0], L.r * L.t1, L.r * L.t2, L.E};
    const float uR[5] = {R.r, R.F[0], R.r * R.t1, R.r * R.t2, R.E};
    const float inv = 1.0f / (SR - SL);
    const float slsr = SL * SR;
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = (SR * L.F[v] - SL * R.F[v] + slsr * (uR[v] - uL[v])) * inv;
  }
}

// HLLC (RiemannSolvers.h:39-112) in FP32; the energy uses the normal and
// first transverse velocity only, as the reference does.
// pout (optional): the interface pressure of RiemannSolvers.h:81-104.
// KE3: the kinetic energy of all three velocities (corrected physics).
template <bool KE3 = false>
__device__ __forceinline__ void hllc32(const Slots<float>& L, const Slots<float>& R, float gamma, float inv_gm1,
                                       float flux[5], float* pout = nullptr) {
  const float kL = KE3 ? L.un * L.un + L.t1 * L.t1 + L.t2 * L.t2 : L.un * L.un + L.t1 * L.t1;
  const float kR = KE3 ? R.un * R.un + R.t1 * R.t1 + R.t2 * R.t2 : R.un * R.un + R.t1 * R.t1;
  const float EL = 0.5f * L.r * kL + L.p * inv_gm1;
  const float ER = 0.5f * R.r * kR + R.p * inv_gm1;
  const float cmax = sqrtf(gamma * fmaxf(L.p / L.r, R.p / R.r));
  const float SL = fminf(L.un, R.un) - cmax;
  const float SR = fmaxf(L.un, R.un) + cmax;
  const float rcL = L.r * (L.un - SL);
  const float rcR = R.r * (SR - R.un);
  const float iD = 1.0f / (rcR + rcL);
  const float uS = (rcR * R.un + rcL * L.un + (L.p - R.p)) * iD;
  const float pS = (rcR * L.p + rcL * R.p + rcL * rcR * (L.un - R.un)) * iD;
  float sr, su, st1, st2, sp, E;
  if (SL > 0.0f) {
    sr = L.r; su = L.un; st1 = L.t1; st2 = L.t2; sp = L.p; E = EL;
  } else if (uS > 0.0f || SR > 0.0f) {
    const bool left = uS > 0.0f;
    const float rK = left ? L.r : R.r, uK = left ? L.un : R.un, pK = left ? L.p : R.p, EK = left ? EL : ER;
    const float SK = left ? SL : SR;
    const float inv = 1.0f / (SK - uS);
    sr = rK * (SK - uK) * inv;
    E = ((SK - uK) * EK - pK * uK + pS * uS) * inv;
    su = uS; sp = pS;
    st1 = left ? L.t1 : R.t1;
    st2 = left ? L.t2 : R.t2;
  } else {
    sr = R.r; su = R.un; st1 = R.t1; st2 = R.t2; sp = R.p; E = ER;
  }
  if (pout) *pout = sp;
  flux[0] = sr * su;
  flux[1] = flux[0] * su + sp;
  flux[2] = flux[0] * st1;
  flux[3] = flux[0] * st2;
  flux[4] = (E + sp) * su;
}

// One FP32 face: minmod slopes, PLM states, Riemann flux (storage order).
template <int PLANE, int DIR>
__device__ __forceinline__ void face_flux32(const float c[4][5], int rs, bool plm, bool wb_z, float g_dz,
                                            float gamma, float inv_gm1, float out[5]) {
  float qL[5], qR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    if (plm) {
      const float d01 = c[1][v] - c[0][v], d12 = c[2][v] - c[1][v], d23 = c[3][v] - c[2][v];
      qL[v] = c[1][v] + minmod32(d01, d12) * 0.5f;
      qR[v] = c[2][v] - minmod32(d12, d23) * 0.5f;
    } else {
      qL[v] = c[1][v];
      qR[v] = c[2][v];
    }
  }
  if (DIR == 1 && wb_z) {  // PCM_WB hydrostatic pressure in z (Update.h:27)
    qL[4] = qL[4] + qL[0] * g_dz * 0.5f;
    qR[4] = qR[4] - qR[0] * g_dz * 0.5f;
  }
  const Slots<float> L = to_slots<PLANE, DIR>(qL), R = to_slots<PLANE, DIR>(qR);
  float f[5];
  if (rs == 0)
    hll32(L, R, gamma, inv_gm1, f);
  else
    hllc32(L, R, gamma, inv_gm1, f);
  from_slots<PLANE, DIR>(f, out);
}

// Phase 1: halo rows [h0, h1) of the block whose first cell is (x0, y0)
// (halo row hy is cell row y0 + hy - 2), columns x0-2 .. x0+TX+1: the stage
// input (pairs or U*) -> FP32 primitives (and temperature).  Batches of KB
// cells per thread: every load of a batch is issued before any of them is
// used, to keep many requests in flight.
// PAIRS: compiled for (hi, lo) pair input (FV_MIXED_LOAD_BATCH cells per
// batch) or for U* input (4-byte values, half the registers:
// FV_MIXED_LOAD_BATCH_STAR cells per batch; 4 against 2: +2.2 % on shear
// 4096^2, 3 the same as 4).
#ifndef FV_MIXED_LOAD_BATCH_STAR
#define FV_MIXED_LOAD_BATCH_STAR 4
#endif
template <int PLANE, bool WACT, class TL, bool PAIRS, class PV>
__device__ __forceinline__ void load_prims32_kind(const Grid& G, const MixedFields& M, float2* const src[5],
                                                  const PV& V, int x0, int y0, int h0, int h1, int tid) {
  constexpr int HX = TL::HX, KB = PAIRS ? FV_MIXED_LOAD_BATCH : FV_MIXED_LOAD_BATCH_STAR;
  constexpr bool in_pairs = PAIRS;
  const float gm1 = G.gm1_f;
  const int ncell = (h1 - h0) * HX;
  for (int base = 0; base < ncell; base += KB * kTileThreads) {
    float2 w[KB][5];
    bool ok[KB], fa[KB], fb[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) {
      const int idx = base + tid + k * kTileThreads;
      ok[k] = idx < ncell;
      const int r = idx / HX, hx = idx - r * HX;
      const int sa = bc_source(x0 + hx - 2, G.na, G.bc_a, fa[k]);
      const int sb = bc_source(y0 + h0 + r - 2, G.nb, G.bc_b, fb[k]);
      const long long o = (long long)sb * G.pitch + sa;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        w[k][v] = make_float2(0.0f, 0.0f);
        if (!ok[k] || (v == 3 && !WACT)) continue;
        w[k][v] = in_pairs ? src[v][o] : make_float2(M.us[v][o], 0.0f);
      }
    }
#pragma unroll
    for (int k = 0; k < KB; ++k) {
      if (!ok[k]) continue;
      const int idx = base + tid + k * kTileThreads;
      const int r = idx / HX, hx = idx - r * HX;
      const int hy = h0 + r;
      float q[5];
      if (in_pairs) {
        cons_to_prim_pairs<PLANE, WACT>(w[k], gm1, q);
      } else {
        float u[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) u[v] = w[k][v].x;
        cons_to_prim_star<WACT>(u, gm1, q);
      }
      if (fa[k]) q[1] = -q[1];
      if (fb[k]) q[2] = -q[2];
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) V.q(v, hy, hx) = q[v];
      if (G.tc) V.temp(hy, hx) = q[4] / q[0];
    }
  }
}

template <int PLANE, bool WACT, class TL, class PV>
__device__ __forceinline__ void load_prims32(const Grid& G, const MixedFields& M, float2* const src[5],
                                             bool in_pairs, const PV& V, int x0, int y0, int h0, int h1, int tid) {
  if (in_pairs)
    load_prims32_kind<PLANE, WACT, TL, true>(G, M, src, V, x0, y0, h0, h1, tid);
  else
    load_prims32_kind<PLANE, WACT, TL, false>(G, M, src, V, x0, y0, h0, h1, tid);
}

// Phase 2: a faces of cell rows 0..nr-1 and b faces of face rows fb0..nr.
template <int PLANE, bool WACT, class TL, class PV>
__device__ __forceinline__ void faces32(const Grid& G, const PV& V, int rs, int nr, int fb0, int tid) {
  constexpr int TX = TL::TX;
  const bool plm = G.recon == R_PLM;
  const bool wb_z = PLANE == PLANE_XZ && G.recon == R_PCM_WB;
  const float g_dz = G.g_dz_f, gamma = G.gamma_f;
  const int nfa = (TX + 1) * nr;
  const int nfa_pad = (nfa + 31) & ~31;  // keeps each warp on one face kind
  const int n = nfa_pad + TX * (nr + 1 - fb0);
  for (int it = tid; it < n; it += kTileThreads) {
    float c[4][5], f[5];
    if (it < nfa_pad) {
      if (it >= nfa) continue;
      const int fy = it / (TX + 1), fx = it - fy * (TX + 1);
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int v = 0; v < 5; ++v) c[k][v] = (WACT || v != 3) ? V.q(v, fy + 2, fx + k) : 0.0f;
      face_flux32<PLANE, 0>(c, rs, plm, wb_z, g_dz, gamma, G.inv_gm1_f, f);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) V.fa(v, fy, fx) = f[v];
    } else {
      const int j = it - nfa_pad;
      const int jy = j / TX, fx = j - jy * TX;
      const int fy = fb0 + jy;
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int v = 0; v < 5; ++v) c[k][v] = (WACT || v != 3) ? V.q(v, fy + k, fx + 2) : 0.0f;
      face_flux32<PLANE, 1>(c, rs, plm, wb_z, g_dz, gamma, G.inv_gm1_f, f);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) V.fb(v, fy, fx) = f[v];
    }
  }
}

// Phase 3-5: increments, accumulation on pairs, CFL term for the cells of
// rows 0..nr-1 of the block.  Inputs per kind:
//   STAGE_RK_1 : read U^n (pairs) -> write U* (FP32)
//   STAGE_RK_2 : read U* (FP32) and U^n (pairs) -> write U^n+1 (pairs, over U^n)
//   STAGE_EULER: read U^n (pairs in `src`) -> write U^n+1 (pairs in `dst`)
// VF: the viscous fluxes of the face-only branches come from the shared face
// arrays visc_faces filled (the split form), else every cell evaluates its
// stencil (the fused form).
// RK2: compiled for RK2 stage 2 (kind == STAGE_RK_2) or for the other two
// kinds; update32 picks the copy, so the stage-2 copy can hold U^n from the
// start of a cell's update without the other kinds paying its registers.
template <int PLANE, bool WACT, class TL, bool VF, bool RK2, class PV>
__device__ __forceinline__ void update32_kind(const Grid& G, const PV& V, const MixedFields& M, float2* const src[5],
                                              float2* const dst[5], int kind, float dt, int x0, int y0, int nr,
                                              int tid, float& red, bool& bad) {
  constexpr int TX = TL::TX;
  const bool in_pairs = !RK2;
  const float inv_db = PLANE == PLANE_XY ? G.inv_dy_f : G.inv_dz_f;
  const float dtdx = dt * G.inv_dx_f;
  const float dtdb = dt * inv_db;
  const int ncell = TX * nr;
#pragma unroll 1
  for (int cidx = tid; cidx < ncell; cidx += kTileThreads) {
    const int cx = cidx % TX, cy = cidx / TX;
    const int x = x0 + cx, y = y0 + cy;
    if (x >= G.na || y >= G.nb) continue;
    const long long o = (long long)y * G.pitch + x;
    // RK2 stage 2: U^n of the cell, loaded before the increments are formed
    // so its latency overlaps them (3 % on shear 4096^2, RT 512x1536 and
    // Sedov 256^2 against loading it where it is added)
    float2 un[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) un[v] = (RK2 && (WACT || v != 3)) ? M.un[v][o] : make_float2(0.0f, 0.0f);
    float du[5];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      du[v] = (V.fa(v, cy, cx) - V.fa(v, cy, cx + 1)) * dtdx + (V.fb(v, cy, cx) - V.fb(v, cy + 1, cx)) * dtdb;
    if (PLANE == PLANE_XZ && G.gravity) {
      du[2] += dt * V.q(0, cy + 2, cx + 2) * G.g_f;
      du[4] += dt * 0.5f * (V.fb(0, cy, cx) + V.fb(0, cy + 1, cx)) * G.g_f;
    }
    // stage input at this cell, as a pair (U*: E* rebuilt from its internal
    // energy and the kinetic energy of its stored density and momenta)
    float2 base[5];
    if (in_pairs) {
#pragma unroll
      for (int v = 0; v < 5; ++v)
        base[v] = (v == 3 && !WACT) ? make_float2(0.0f, 0.0f) : src[v][o];
    } else {
      float u[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) u[v] = (v == 3 && !WACT) ? 0.0f : M.us[v][o];
#pragma unroll
      for (int v = 0; v < 4; ++v) base[v] = make_float2(u[v], 0.0f);
      base[4] = pair_add(kinetic_star<WACT>(u), u[4]);
    }
    // density floor on the hydro update (Update.h:160), before TC / viscosity
    {
      const float2 rho = pair_add(base[0], du[0]);
      if (rho.x + rho.y < 1.0e-6f) {
        base[0] = make_float2(1.0e-6f, 0.0f);
        du[0] = 0.0f;
      }
    }
    if (G.tc) {
      const float kf = G.kappa_f;
      const int hy = cy + 2, hx = cx + 2;
      const float TC = V.temp(hy, hx);
      const float FL = kf * (TC - V.temp(hy, hx - 1)) * G.inv_dx_f;
      const float FR = kf * (V.temp(hy, hx + 1) - TC) * G.inv_dx_f;
      const float FU = kf * (TC - V.temp(hy - 1, hx)) * inv_db;
      const float FD = kf * (V.temp(hy + 1, hx) - TC) * inv_db;
      du[4] += dtdx * (FR - FL) + dtdb * (FD - FU);
    }
    if (WACT && G.visc) {
      // fused: every cell evaluates its stencil; split: the face-only
      // branches once per face (17 KB more shared memory per CTA, so fewer
      // resident CTAs: the autotuner chooses per group)
      float vf[3][5];
      if (VF) {
        visc_cell_shared<PLANE>(V, cy, cx, G.inv_dx_f, G.inv_dz_f, G.mu_f, vf);
      } else {
        PlaneVel<PLANE, PV> P{V, cy + 2, cx + 2};
        viscous_plane<PLANE, float>(P, G.inv_dx_f, G.inv_dy_f, G.inv_dz_f, G.mu_f, vf);
      }
#pragma unroll
      for (int var = 1; var < 5; ++var) {
        const int sv = var == 4 ? 4 : phys_slot<PLANE>(var);
        du[sv] += (vf[0][var] + vf[1][var] + vf[2][var]) * dt;
      }
    }
    if (!RK2 && kind == STAGE_RK_1) {
      float us[5];
#pragma unroll
      for (int v = 0; v < 4; ++v) us[v] = (v == 3 && !WACT) ? 0.0f : base[v].x + (base[v].y + du[v]);
      // U* keeps its internal energy: E* (a pair) minus the kinetic energy of
      // the stored density and momenta
      us[4] = internal_energy(pair_add(base[4], du[4]), kinetic_star<WACT>(us));
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) M.us[v][o] = us[v];
      continue;
    }
    // RK2 stage 2: U^n+1 = 0.5 * (U^n + U* + dU); Euler: U^n+1 = U^n + dU
    float2 fin[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if (v == 3 && !WACT) {
        fin[v] = make_float2(0.0f, 0.0f);
        continue;
      }
      float2 r;
      if (RK2) {
        r = pair_add(pair_add(un[v], base[v]), du[v]);
        r = make_float2(0.5f * r.x, 0.5f * r.y);
      } else {
        r = pair_add(base[v], du[v]);
      }
      dst[v][o] = r;
      fin[v] = r;
    }
    const float inv = inv_dt_hyp32<PLANE, WACT>(fin, G);
    bad |= !(inv <= 3.0e38f);  // NaN / inf: reported through the error flag
    red = fmaxf(red, inv);
  }
}

template <int PLANE, bool WACT, class TL, bool VF, class PV>
__device__ __forceinline__ void update32(const Grid& G, const PV& V, const MixedFields& M, float2* const src[5],
                                         float2* const dst[5], int kind, float dt, int x0, int y0, int nr, int tid,
                                         float& red, bool& bad) {
  if (kind == STAGE_RK_2)
    update32_kind<PLANE, WACT, TL, VF, true>(G, V, M, src, dst, kind, dt, x0, y0, nr, tid, red, bad);
  else
    update32_kind<PLANE, WACT, TL, VF, false>(G, V, M, src, dst, kind, dt, x0, y0, nr, tid, red, bad);
}

// Moves halo rows TY..TY+3 of the previous block to rows 0..3 (the rows the
// next block shares with it).  Each cell is moved by the thread that the
// next load_prims32 (rows 4..) assigns to the cell's old row, so program
// order alone keeps the move ahead of that thread's overwrite.
template <bool WACT, class TL, class SM>
__device__ __forceinline__ void carry_rows32(const Grid& G, const SM& S, int tid) {
  constexpr int HX = TL::HX, TY = TL::TY;
  int idx = tid;  // load index (rows from 4) of this thread's cells
  while (idx < (TY - 4) * HX) idx += kTileThreads;
  for (; idx < TY * HX; idx += kTileThreads) {
    const int hy = 4 + idx / HX, hx = idx % HX;
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3) S.q(v, hy - TY, hx) = S.q(v, hy, hx);
    if (G.tc) S.temp(hy - TY, hx) = S.temp(hy, hx);
  }
}

// One mixed-precision stage of the strip segment of cell rows [ya, yb) of
// the TX-wide strip whose first column is x0, marched in blocks of TY rows
// (each block converts only its new rows: the 4 rows it shares with the
// previous block are moved down, carry_rows32, and the b faces on the
// boundary are reused), the arithmetic of every face and cell that of the
// tile form.  Every thread of the CTA calls it; the CFL maximum and the
// non-finite flag are folded into red / bad; smem holds
// TileSmem<float, NV, TL>::bytes(G.tc) bytes, or bytes_vface() for the split
// viscous form (VF, update32).
template <int PLANE, bool WACT, class TL, bool VF>
__device__ __forceinline__ void stage_segment32(const Grid& G, const MixedFields& M, float2* const src[5],
                                                float2* const dst[5], int rs, int kind, float dt, int x0, int ya,
                                                int yb, float* smem, float& red, bool& bad) {
  constexpr int NV = WACT ? 5 : 4;
  constexpr int TX = TL::TX, TY = TL::TY;
  using SM = TileSmem<float, NV, TL>;
  const SM S{smem};
  const int tid = threadIdx.x;
  const bool in_pairs = kind != STAGE_RK_2;
  const PrimView<SM, RowsDirect> V{S, RowsDirect{}};
  for (int y0 = ya; y0 < yb; y0 += TY) {
    const int nr = yb - y0 < TY ? yb - y0 : TY;
    const bool first = y0 == ya;
    if (!first) {  // rows and b faces shared with the previous (full) block
      for (int i = tid; i < NV * TX; i += kTileThreads) {
        const int v = i / TX, fx = i - v * TX;
        const int sv = NV == 5 ? v : (v == 3 ? 4 : v);
        S.fb(sv, 0, fx) = S.fb(sv, TY, fx);
      }
      if (VF && WACT && G.visc && PLANE == PLANE_XY)  // and their viscous fluxes
        for (int i = tid; i < 4 * TX; i += kTileThreads) {
          const int k = i / TX, fx = i - k * TX;
          S.vb(k, 0, fx) = S.vb(k, TY, fx);
        }
      carry_rows32<WACT, TL>(G, S, tid);
    }
    load_prims32<PLANE, WACT, TL>(G, M, src, in_pairs, V, x0, y0, first ? 0 : 4, nr + 4, tid);
    __syncthreads();
    faces32<PLANE, WACT, TL>(G, V, rs, nr, first ? 0 : 1, tid);
    if (VF && WACT && G.visc)
      visc_faces<PLANE, TL>(V, G.inv_dx_f, G.inv_dy_f, G.inv_dz_f, G.mu_f, nr, first ? 0 : 1, tid);
    __syncthreads();
    update32<PLANE, WACT, TL, VF>(G, V, M, src, dst, kind, dt, x0, y0, nr, tid, red, bad);
    __syncthreads();
  }
}

// An inactive mixed Euler step hands its state on (ping-pong pairs).
template <bool WACT, int TX>
__device__ __forceinline__ void pass_on32(const Grid& G, float2* const src[5], float2* const dst[5], int x0, int y0,
                                          int y1, int tid) {
  const int n = TX * (y1 - y0);
  for (int c = tid; c < n; c += kTileThreads) {
    const int x = x0 + c % TX, y = y0 + c / TX;
    if (x < G.na && y < G.nb) {
      const long long o = (long long)y * G.pitch + x;
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) dst[v][o] = src[v][o];
    }
  }
}

}  // namespace fv
