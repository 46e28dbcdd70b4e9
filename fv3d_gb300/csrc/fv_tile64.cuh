// fv_tile64.cuh -- the FP64 stage body shared by the single-problem kernel
// (fv_stage2d.cu) and the persistent batch kernel (fv_batch64.cu).
//
// stage_segment64 performs a whole reference euler_step (Update.h:164-178)
// on a strip segment: TX columns and a run of rows, marched in blocks of
// TX x TY cells with 256 threads.  Per block:
//   1. the new halo rows of the block (all TY + 4 for the first block of a
//      segment, TY afterwards: the 4 rows shared with the previous block stay
//      in a ring of TY + 4 shared rows) -- loaded with the ghost cells
//      synthesised by index remapping (the X-then-Y ghost fill of
//      BoundaryConditions.h:146-192, corners included) or, for interior
//      blocks of the single-problem kernel, staged by TMA tensor copies --
//      and converted to primitives (consToPrim, States.h:34-45);
//   2. every face of the block: minmod slopes and PLM face states
//      (Update.h:14-33,55-88) and one Riemann solve (RiemannSolvers.h) -- the
//      reference solves every face twice, from each side, with equal inputs;
//      the b faces on the boundary with the previous block are reused; with
//      viscosity, the face-only viscous branches once per face;
//   3. the conservative update in the reference's X, Y, Z order with
//      (F*dt)/d increments, gravity on the z sweep and the density floor
//      (Update.h:145-160), then thermal conduction (ThermalConduction.h:38-96)
//      and viscosity (Viscosity.h:127-253) from the same primitive tile;
//   4. for RK2 stage 2 the SSP average 0.5*(U^n + U**) (Update.h:198-204);
//   5. for the last stage of a step, consToPrim of the result and the
//      hyperbolic CFL term of ComputeDt.h:28-54, folded into one maximum per
//      CTA (the TC/viscous terms are constants folded in by the control
//      kernel).
//
// Rounding: every file including this one is compiled without FMA
// contraction, every operation follows the reference's order, and the
// cheaper exact forms of fv_exact64.cuh / fv_riemann64.cuh replace divisions
// and comparisons, so the result is bit-identical to the reference's FP64 CPU
// arithmetic.
//
// The degenerate third axis (one cell whose ghost layers equal it) adds
// exactly zero to every flux difference in the reference arithmetic, so its
// sweep is skipped; its cell size still enters dt.
#pragma once

#include "fv_kernels.h"
#include "fv_plane2d.cuh"
#include "fv_riemann64.cuh"

namespace fv {

constexpr int kTileThreads = 256;

// Geometry of a TX x TY tile handled by kTileThreads threads.
template <int TX_, int TY_>
struct Tile {
  static constexpr int TX = TX_, TY = TY_;
  static constexpr int HX = TX + 4, HY = TY + 4;         // tile + 2-cell halo
  static constexpr int NFA = (TX + 1) * TY;              // a-faces
  static constexpr int NFA_PAD = (NFA + 31) / 32 * 32;   // keeps each warp on one face kind
  static constexpr int NFB = TX * (TY + 1);              // b-faces
  static constexpr int CELLS = TX * TY;
};

// Shared-memory layout for NV stored variables of element type T:
//   Q [NV][HY][HX]   primitives of tile + halo
//   FA[NV][TY][TX+1] a-face fluxes (storage order)
//   FB[NV][TY+1][TX] b-face fluxes (storage order)
//   TT[HY][HX]       temperature p/rho (thermal conduction only)
template <class T, int NV, class TL>
struct TileSmem {
  T* base;
  static constexpr int kQ = 0;
  static constexpr int kFA = NV * TL::HY * TL::HX;
  static constexpr int kFB = kFA + NV * TL::TY * (TL::TX + 1);
  static constexpr int kT = kFB + NV * (TL::TY + 1) * TL::TX;
  static constexpr int kEnd = kT;
  static constexpr size_t bytes(bool tc) { return sizeof(T) * (size_t)(kEnd + (tc ? TL::HY * TL::HX : 0)); }
  // storage variable (0 r, 1 a, 2 b, 3 c, 4 E/p) -> shared-memory slot
  __device__ static constexpr int sv(int v) { return NV == 5 ? v : (v == 4 ? 3 : v); }
  __device__ T& q(int v, int hy, int hx) const { return base[kQ + (sv(v) * TL::HY + hy) * TL::HX + hx]; }
  __device__ T& fa(int v, int fy, int fx) const { return base[kFA + (sv(v) * TL::TY + fy) * (TL::TX + 1) + fx]; }
  __device__ T& fb(int v, int fy, int fx) const { return base[kFB + (sv(v) * (TL::TY + 1) + fy) * TL::TX + fx]; }
  __device__ T& temp(int hy, int hx) const { return base[kT + hy * TL::HX + hx]; }
  // Shared-face viscous fluxes (4 per face: three momentum components and
  // energy), after the temperature tile.
  static constexpr int kVA = kT + TL::HY * TL::HX;
  static constexpr int kVB = kVA + 4 * TL::TY * (TL::TX + 1);
  static constexpr int kVEnd = kVB + 4 * (TL::TY + 1) * TL::TX;
  static constexpr size_t bytes_vface() { return sizeof(T) * (size_t)kVEnd; }
  __device__ T& va(int k, int fy, int fx) const { return base[kVA + (k * TL::TY + fy) * (TL::TX + 1) + fx]; }
  __device__ T& vb(int k, int fy, int fx) const { return base[kVB + (k * (TL::TY + 1) + fy) * TL::TX + fx]; }
};

// The IZ branch of Viscosity.h:214-239 in an x-y run (z is the one-cell
// axis): qi is the centre, the z derivatives vanish, and its y terms do not
// depend on the side.  Accumulates into vz[1..4].
template <class T, class PA>
__device__ __forceinline__ void viscous_iz_xy(const PA& P, T odx, T odz, T mu, T vz[5]) {
  const T two_thirds = T(2.0 / 3.0);
  const T c4x = half_of(half_of(odx)), c4z = half_of(half_of(odz));
  const int U = 1, V = 2, W = 3;
  const T cu = P(1, 1, U), cv = P(1, 1, V), cw = P(1, 1, W);
  const T dvdy = c4z * (P(2, 1, W) - P(0, 1, V) + P(2, 1, W) - P(0, 1, V));
  const T dwdy = c4z * (P(2, 1, V) - P(0, 1, W) + P(2, 1, V) - P(0, 1, W));
#pragma unroll
  for (int s = 1; s < 3; ++s) {
    const T sign = s == 1 ? T(-1) : T(1);
    const T dudx = c4x * (P(1, 2, U) - P(s, 0, U) + P(1, 2, U) - P(s - 1, 0, U));
    const T dwdx = c4x * (P(1, 2, V) - P(s, 0, W) + P(1, 2, V) - P(s - 1, 0, W));
    const T tau_zz = -(two_thirds * (dudx + dvdy));
    const T tau_xz = dwdx;
    const T tau_yz = dwdy;
    vz[1] += sign * mu * tau_xz;
    vz[2] += sign * mu * tau_yz;
    vz[3] += sign * mu * tau_zz;
    vz[4] += sign * mu * (tau_xz * cu + tau_yz * cv + tau_zz * cw);
  }
}

// The IZ branch in an x-z run, with the reference's index / field mix-ups
// (Viscosity.h:214-239).  Some of its terms read the cell's own row, so its
// flux belongs to the cell, not to the face.  Accumulates into vz[1..4].
template <class T, class PA>
__device__ __forceinline__ void viscous_iz_xz(const PA& P, T odx, T odz, T mu, T vz[5]) {
  const T four_thirds = T(4.0 / 3.0);
  const T two_thirds = T(2.0 / 3.0);
  const T c4x = half_of(half_of(odx)), c4z = half_of(half_of(odz));
  const int U = 1, V = 2, W = 3;
#pragma unroll
  for (int s = 1; s < 3; ++s) {
    const T sign = s == 1 ? T(-1) : T(1);
    const T qiu = half_of(P(s, 1, U) + P(s - 1, 1, U));
    const T qiv = half_of(P(s, 1, V) + P(s - 1, 1, V));
    const T qiw = half_of(P(s, 1, W) + P(s - 1, 1, W));
    const T dudz = odz * (P(s, 1, U) - P(s - 1, 1, U));
    const T dvdz = odz * (P(s, 1, V) - P(s - 1, 1, V));
    const T dwdz = odz * (P(s, 1, W) - P(s - 1, 1, W));
    const T dudx = c4x * (P(s, 2, U) - P(1, 0, U) + P(s - 1, 2, U) - P(1, 0, U));
    const T dwdx = c4x * (P(s, 2, V) - P(1, 0, W) + P(s - 1, 2, V) - P(1, 0, W));
    const T dvdy = c4z * (P(s, 1, W) - P(s, 1, V) + P(s - 1, 1, W) - P(s - 1, 1, V));
    const T dwdy = c4z * (P(s, 1, V) - P(s, 1, W) + P(s - 1, 1, V) - P(s - 1, 1, W));
    const T tau_zz = four_thirds * dwdz - two_thirds * (dudx + dvdy);
    const T tau_xz = dudz + dwdx;
    const T tau_yz = dvdz + dwdy;
    vz[1] += sign * mu * tau_xz;
    vz[2] += sign * mu * tau_yz;
    vz[3] += sign * mu * tau_zz;
    vz[4] += sign * mu * (tau_xz * qiu + tau_yz * qiv + tau_zz * qiw);
  }
}

// Viscous fluxes of Viscosity.h:149-243 for a 2-D plane, with the reference's
// arithmetic (including its z-branch index and field mix-ups) on every term
// that is not an exact zero.  The stencil's offsets along the
// one-cell axis read the centre layer, so in the literal formula every
// derivative along that axis is c*((a - a) + b) - b) = 0 and the IY branch of
// an x-z run cancels to (-mu*t) + mu*t = 0; dropping those terms returns the
// same values (at most the sign of an exact zero differs).  P(r, c, var) reads
// velocity var (1 u, 2 v, 3 w) of the cell at offset (r-1, c-1) along (b, a).
// vf receives the per-direction fluxes of components u, v, w, E (index 1..4).
// odx, ody, odz are the reference's one_over_d = RN(1/d) (Viscosity.h:44-46),
// computed once on the host.
template <int PLANE, class T, class PA>
__device__ __forceinline__ void viscous_plane(const PA& P, T odx, T ody, T odz, T mu, T vf[3][5]) {
  const T four_thirds = T(4.0 / 3.0);
  const T two_thirds = T(2.0 / 3.0);
  const T c4x = half_of(half_of(odx)), c4y = half_of(half_of(ody)), c4z = half_of(half_of(odz));
  const int U = 1, V = 2, W = 3;
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int v = 0; v < 5; ++v) vf[d][v] = T(0);
  if (PLANE == PLANE_XY) {
#pragma unroll
    for (int s = 1; s < 3; ++s) {  // IX (Viscosity.h:163-186), z-derivatives vanish
      const T sign = s == 1 ? T(-1) : T(1);
      const T qiu = half_of(P(1, s, U) + P(1, s - 1, U));
      const T qiv = half_of(P(1, s, V) + P(1, s - 1, V));
      const T qiw = half_of(P(1, s, W) + P(1, s - 1, W));
      const T dudx = odx * (P(1, s, U) - P(1, s - 1, U));
      const T dvdx = odx * (P(1, s, V) - P(1, s - 1, V));
      const T dwdx = odx * (P(1, s, W) - P(1, s - 1, W));
      const T dudy = c4y * (P(2, s, U) - P(0, s, U) + P(2, s - 1, U) - P(0, s - 1, U));
      const T dvdy = c4y * (P(2, s, V) - P(0, s, V) + P(2, s - 1, V) - P(0, s - 1, V));
      const T tau_xx = four_thirds * dudx - two_thirds * dvdy;
      const T tau_xy = dvdx + dudy;
      const T tau_xz = dwdx;
      vf[0][1] += sign * mu * tau_xx;
      vf[0][2] += sign * mu * tau_xy;
      vf[0][3] += sign * mu * tau_xz;
      vf[0][4] += sign * mu * (tau_xx * qiu + tau_xy * qiv + tau_xz * qiw);
    }
#pragma unroll
    for (int s = 1; s < 3; ++s) {  // IY (Viscosity.h:188-213), z-derivatives vanish
      const T sign = s == 1 ? T(-1) : T(1);
      const T qiu = half_of(P(s, 1, U) + P(s - 1, 1, U));
      const T qiv = half_of(P(s, 1, V) + P(s - 1, 1, V));
      const T qiw = half_of(P(s, 1, W) + P(s - 1, 1, W));
      const T dudy = ody * (P(s, 1, U) - P(s - 1, 1, U));
      const T dvdy = ody * (P(s, 1, V) - P(s - 1, 1, V));
      const T dwdy = ody * (P(s, 1, W) - P(s - 1, 1, W));
      const T dudx = c4x * (P(s, 2, U) - P(s, 0, U) + P(s - 1, 2, U) - P(s - 1, 0, U));
      const T dvdx = c4x * (P(s, 2, V) - P(s, 0, V) + P(s - 1, 2, V) - P(s - 1, 0, V));
      const T tau_yy = four_thirds * dvdy - two_thirds * dudx;
      const T tau_xy = dvdx + dudy;
      const T tau_yz = dwdy;
      vf[1][1] += sign * mu * tau_xy;
      vf[1][2] += sign * mu * tau_yy;
      vf[1][3] += sign * mu * tau_yz;
      vf[1][4] += sign * mu * (tau_xy * qiu + tau_yy * qiv + tau_yz * qiw);
    }
    viscous_iz_xy(P, odx, odz, mu, vf[2]);
  } else {
#pragma unroll
    for (int s = 1; s < 3; ++s) {  // IX, y-derivatives vanish
      const T sign = s == 1 ? T(-1) : T(1);
      const T qiu = half_of(P(1, s, U) + P(1, s - 1, U));
      const T qiv = half_of(P(1, s, V) + P(1, s - 1, V));
      const T qiw = half_of(P(1, s, W) + P(1, s - 1, W));
      const T dudx = odx * (P(1, s, U) - P(1, s - 1, U));
      const T dvdx = odx * (P(1, s, V) - P(1, s - 1, V));
      const T dwdx = odx * (P(1, s, W) - P(1, s - 1, W));
      const T dudz = c4z * (P(2, s, U) - P(0, s, U) + P(2, s - 1, U) - P(0, s - 1, U));
      const T dwdz = c4z * (P(2, s, W) - P(0, s, W) + P(2, s - 1, W) - P(0, s - 1, W));
      const T tau_xx = four_thirds * dudx - two_thirds * dwdz;
      const T tau_xy = dvdx;
      const T tau_xz = dwdx + dudz;
      vf[0][1] += sign * mu * tau_xx;
      vf[0][2] += sign * mu * tau_xy;
      vf[0][3] += sign * mu * tau_xz;
      vf[0][4] += sign * mu * (tau_xx * qiu + tau_xy * qiv + tau_xz * qiw);
    }
    // IY on the one-cell axis: every term is side-independent and cancels.
    viscous_iz_xz(P, odx, odz, mu, vf[2]);
  }
}

// Plane accessor for viscous_plane over a TileSmem primitive tile.
template <int PLANE, class SM>
struct PlaneVel {
  SM s;
  int hy, hx;
  __device__ __forceinline__ auto operator()(int r, int c, int var) const {
    return s.q(phys_slot<PLANE>(var), hy + r - 1, hx + c - 1);
  }
};

// The viscous flux of one face for the branches whose terms depend on the
// face alone: IX (DIR 0) in both planes and IY (DIR 1) in the x-y plane.  The
// reference evaluates it from each of the two cells, as
// (sign * mu) * t with sign -1 on the cell's lower face and +1 on its upper
// face, from identical operands; (-mu) * t = -(mu * t) exactly, so one
// evaluation serves both cells: g = {mu*t1, mu*t2, mu*t3, mu*(t . qi)} in the
// branch's component order (vf[d][1..4]).  P is centred on the cell above
// the face (the s = 1 side of Viscosity.h's loop).
template <int PLANE, int DIR, class T, class PA>
__device__ __forceinline__ void viscous_face(const PA& P, T odx, T ody, T odz, T mu, T g[4]) {
  const T four_thirds = T(4.0 / 3.0);
  const T two_thirds = T(2.0 / 3.0);
  const int U = 1, V = 2, W = 3;
  if (DIR == 0) {
    const T qiu = half_of(P(1, 1, U) + P(1, 0, U));
    const T qiv = half_of(P(1, 1, V) + P(1, 0, V));
    const T qiw = half_of(P(1, 1, W) + P(1, 0, W));
    const T dudx = odx * (P(1, 1, U) - P(1, 0, U));
    const T dvdx = odx * (P(1, 1, V) - P(1, 0, V));
    const T dwdx = odx * (P(1, 1, W) - P(1, 0, W));
    T tau_xx, tau_xy, tau_xz;
    if (PLANE == PLANE_XY) {
      const T c4y = half_of(half_of(ody));
      const T dudy = c4y * (P(2, 1, U) - P(0, 1, U) + P(2, 0, U) - P(0, 0, U));
      const T dvdy = c4y * (P(2, 1, V) - P(0, 1, V) + P(2, 0, V) - P(0, 0, V));
      tau_xx = four_thirds * dudx - two_thirds * dvdy;
      tau_xy = dvdx + dudy;
      tau_xz = dwdx;
    } else {
      const T c4z = half_of(half_of(odz));
      const T dudz = c4z * (P(2, 1, U) - P(0, 1, U) + P(2, 0, U) - P(0, 0, U));
      const T dwdz = c4z * (P(2, 1, W) - P(0, 1, W) + P(2, 0, W) - P(0, 0, W));
      tau_xx = four_thirds * dudx - two_thirds * dwdz;
      tau_xy = dvdx;
      tau_xz = dwdx + dudz;
    }
    g[0] = mu * tau_xx;
    g[1] = mu * tau_xy;
    g[2] = mu * tau_xz;
    g[3] = mu * (tau_xx * qiu + tau_xy * qiv + tau_xz * qiw);
  } else {
    const T c4x = half_of(half_of(odx));
    const T qiu = half_of(P(1, 1, U) + P(0, 1, U));
    const T qiv = half_of(P(1, 1, V) + P(0, 1, V));
    const T qiw = half_of(P(1, 1, W) + P(0, 1, W));
    const T dudy = ody * (P(1, 1, U) - P(0, 1, U));
    const T dvdy = ody * (P(1, 1, V) - P(0, 1, V));
    const T dwdy = ody * (P(1, 1, W) - P(0, 1, W));
    const T dudx = c4x * (P(1, 2, U) - P(1, 0, U) + P(0, 2, U) - P(0, 0, U));
    const T dvdx = c4x * (P(1, 2, V) - P(1, 0, V) + P(0, 2, V) - P(0, 0, V));
    const T tau_yy = four_thirds * dvdy - two_thirds * dudx;
    const T tau_xy = dvdx + dudy;
    const T tau_yz = dwdy;
    g[0] = mu * tau_xy;
    g[1] = mu * tau_yy;
    g[2] = mu * tau_yz;
    g[3] = mu * (tau_xy * qiu + tau_yy * qiv + tau_yz * qiw);
  }
}

// 0.0 + x without the FP64 pipe: x itself, except that -0 becomes +0.
__device__ __forceinline__ double plus_zero(double x) {
  const long long b = __double_as_longlong(x);
  return b == (long long)0x8000000000000000ull ? 0.0 : x;
}
__device__ __forceinline__ float plus_zero(float x) { return 0.0f + x; }

// viscous_plane with the face-only branches taken from shared face fluxes:
// gl[d] / gr[d] are viscous_face of the cell's lower / upper face along
// branch d (d = 1 used in the x-y plane only).  vf[d][k+1] =
// (0 + (-gl[d][k])) + gr[d][k], the reference's two accumulations; the
// branches that read the cell itself are evaluated here.  Same bits as
// viscous_plane in FP64.
template <int PLANE, class T, class PA>
__device__ __forceinline__ void viscous_plane_shared(const PA& P, const T gl[2][4], const T gr[2][4], T odx, T odz,
                                                     T mu, T vf[3][5]) {
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int v = 0; v < 5; ++v) vf[d][v] = T(0);
#pragma unroll
  for (int k = 0; k < 4; ++k) vf[0][k + 1] = plus_zero(-gl[0][k]) + gr[0][k];
  if (PLANE == PLANE_XY) {
#pragma unroll
    for (int k = 0; k < 4; ++k) vf[1][k + 1] = plus_zero(-gl[1][k]) + gr[1][k];
    viscous_iz_xy(P, odx, odz, mu, vf[2]);
  } else {
    viscous_iz_xz(P, odx, odz, mu, vf[2]);
  }
}

// Viscous fluxes of the face-only branches for the faces of a block: a
// faces of cell rows 0..nr-1 along IX; b faces of face rows fb0..nr along IY
// in the x-y plane (the x-z plane's IZ branch belongs to the cells).
template <int PLANE, class TL, class T, class PV>
__device__ __forceinline__ void visc_faces(const PV& V, T odx, T ody, T odz, T mu, int nr, int fb0, int tid) {
  constexpr int TX = TL::TX;
  const int nfa = (TX + 1) * nr;
  const int nfa_pad = (nfa + 31) & ~31;
  const int n = nfa_pad + (PLANE == PLANE_XY ? TX * (nr + 1 - fb0) : 0);
  for (int it = tid; it < n; it += kTileThreads) {
    T g[4];
    if (it < nfa_pad) {
      if (it >= nfa) continue;
      const int fy = it / (TX + 1), fx = it - fy * (TX + 1);
      const PlaneVel<PLANE, PV> P{V, fy + 2, fx + 2};  // the cell right of a face
      viscous_face<PLANE, 0>(P, odx, ody, odz, mu, g);
#pragma unroll
      for (int k = 0; k < 4; ++k) V.va(k, fy, fx) = g[k];
    } else {
      const int j = it - nfa_pad;
      const int jy = j / TX, fx = j - jy * TX;
      const int fy = fb0 + jy;
      const PlaneVel<PLANE, PV> P{V, fy + 2, fx + 2};  // the cell above b face fy
      viscous_face<PLANE, 1>(P, odx, ody, odz, mu, g);
#pragma unroll
      for (int k = 0; k < 4; ++k) V.vb(k, fy, fx) = g[k];
    }
  }
}

// The shared-face viscous fluxes of cell (cy, cx) of a block.
template <int PLANE, class T, class PV>
__device__ __forceinline__ void visc_cell_shared(const PV& V, int cy, int cx, T odx, T odz, T mu, T vf[3][5]) {
  const PlaneVel<PLANE, PV> P{V, cy + 2, cx + 2};
  T gl[2][4], gr[2][4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    gl[0][k] = V.va(k, cy, cx);
    gr[0][k] = V.va(k, cy, cx + 1);
    gl[1][k] = PLANE == PLANE_XY ? V.vb(k, cy, cx) : T(0);
    gr[1][k] = PLANE == PLANE_XY ? V.vb(k, cy + 1, cx) : T(0);
  }
  viscous_plane_shared<PLANE>(P, gl, gr, odx, odz, mu, vf);
}

// Slots of a sweep (swap_component, States.h:104-111) from storage order
// (r, a, b, c, p): DIR 0 = reference IX (u, v, w); DIR 1 = IY (v, u, w) in
// the x-y plane or IZ (w, v, u) in the x-z plane.
template <int PLANE, int DIR, class T>
__device__ __forceinline__ Slots<T> to_slots(const T q[5]) {
  Slots<T> s;
  s.r = q[0];
  s.p = q[4];
  if (DIR == 0) {
    s.un = q[1];
    s.t1 = PLANE == PLANE_XY ? q[2] : q[3];
    s.t2 = PLANE == PLANE_XY ? q[3] : q[2];
  } else {
    s.un = q[2];
    s.t1 = PLANE == PLANE_XY ? q[1] : q[3];
    s.t2 = PLANE == PLANE_XY ? q[3] : q[1];
  }
  return s;
}

// Flux in slot order -> storage order (the inverse swap).
template <int PLANE, int DIR, class T>
__device__ __forceinline__ void from_slots(const T f[5], T out[5]) {
  out[0] = f[0];
  out[4] = f[4];
  if (DIR == 0) {
    out[1] = f[1];
    out[2] = PLANE == PLANE_XY ? f[2] : f[3];
    out[3] = PLANE == PLANE_XY ? f[3] : f[2];
  } else {
    out[2] = f[1];
    out[1] = PLANE == PLANE_XY ? f[2] : f[3];
    out[3] = PLANE == PLANE_XY ? f[3] : f[2];
  }
}

// One FP64 face: slopes, face states and the Riemann flux, in storage order.
// c[k][v] holds variable v of the four cells around the face (left-left,
// left, right, right-right).
template <int PLANE, bool WACT, int DIR>
__device__ __forceinline__ void face_flux64(const double c[4][5], int rs, bool plm, bool wb_z, const Grid& G,
                                            const Consts64& K, double out[5]) {
  constexpr int ZS = WACT ? 0 : (PLANE == PLANE_XY ? 2 : 1);
  double qL[5], qR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    if (v == 3 && !WACT) {
      qL[v] = 0.0;
      qR[v] = 0.0;
      continue;
    }
    if (plm) {
      const double d01 = c[1][v] - c[0][v], d12 = c[2][v] - c[1][v], d23 = c[3][v] - c[2][v];
      qL[v] = recon_plus(c[1][v], minmod_exact(d01, d12));
      qR[v] = recon_minus(c[2][v], minmod_exact(d12, d23));
    } else {
      qL[v] = c[1][v];
      qR[v] = c[2][v];
    }
  }
  if (DIR == 1 && wb_z) {  // PCM_WB hydrostatic pressure in z (Update.h:27)
    qL[4] = qL[4] + half64(1.0 * qL[0] * G.g * G.dz);
    qR[4] = qR[4] + half64(-1.0 * qR[0] * G.g * G.dz);
  }
  const Slots<double> L = to_slots<PLANE, DIR>(qL), R = to_slots<PLANE, DIR>(qR);
  double f[5];
  if (rs == 0)
    hll64<ZS>(L, R, K, f);
  else
    hllc64<ZS>(L, R, K, f);
  from_slots<PLANE, DIR>(f, out);
}

// Row mapping of the primitive rows held in shared memory: halo row hy of the
// current block (cell row y0 + hy - 2) sits in shared row rows(hy).
struct RowsDirect {  // a tile: every halo row has its own shared row
  __device__ __forceinline__ int operator()(int hy) const { return hy; }
};
template <int RING>
struct RowsRing {  // a strip: a ring of RING rows whose origin advances block by block
  int base;        // 0 <= base < RING; hy <= RING - 1
  __device__ __forceinline__ int operator()(int hy) const {
    const int s = base + hy;
    return s >= RING ? s - RING : s;
  }
};

// The shared tile seen through a row mapping (primitives and temperature);
// face fluxes are stored by block-local face rows.
template <class SM, class RM>
struct PrimView {
  SM s;
  RM rows;
  __device__ __forceinline__ auto& q(int v, int hy, int hx) const { return s.q(v, rows(hy), hx); }
  __device__ __forceinline__ auto& temp(int hy, int hx) const { return s.temp(rows(hy), hx); }
  __device__ __forceinline__ auto& fa(int v, int fy, int fx) const { return s.fa(v, fy, fx); }
  __device__ __forceinline__ auto& fb(int v, int fy, int fx) const { return s.fb(v, fy, fx); }
  __device__ __forceinline__ auto& va(int k, int fy, int fx) const { return s.va(k, fy, fx); }
  __device__ __forceinline__ auto& vb(int k, int fy, int fx) const { return s.vb(k, fy, fx); }
};

// Phase 1: halo rows [h0, h1) of the block whose first cell is (x0, y0),
// columns x0-2 .. x0+TX+1: conserved state -> primitives (and temperature),
// ghost cells synthesised by index remapping (X-then-Y fill of
// BoundaryConditions.h:146-192, corners included).
//
// prims: uin already holds the primitives of the state (the copy the last
// RK2 stage wrote, bit-identical to consToPrim of the state), so only the
// temperature's reciprocal is computed.
template <int PLANE, bool WACT, class TL, class PV>
__device__ __forceinline__ void load_prims64(const Grid& G, const Fields& uin, const PV& V, int x0, int y0, int h0,
                                             int h1, int tid, bool prims = false) {
  constexpr int HX = TL::HX;
  const int n = (h1 - h0) * HX;
  for (int idx = tid; idx < n; idx += kTileThreads) {
    const int r = idx / HX, hx = idx - r * HX;
    const int hy = h0 + r;
    bool fa, fb;
    const int sa = bc_source(x0 + hx - 2, G.na, G.bc_a, fa);
    const int sb = bc_source(y0 + hy - 2, G.nb, G.bc_b, fb);
    const long long o = (long long)sb * G.pitch + sa;
    double u[5], q[5], y = 0.0;
    u[0] = uin.f[0][o];
    u[1] = uin.f[1][o];
    u[2] = uin.f[2][o];
    u[3] = WACT ? uin.f[3][o] : 0.0;
    u[4] = uin.f[4][o];
    if (prims) {
#pragma unroll
      for (int v = 0; v < 5; ++v) q[v] = u[v];
      if (G.tc) y = 1.0 / q[0];
    } else {
      cons_to_prim64<PLANE, WACT>(u, G.gm1, q, y);
    }
    if (fa) q[1] = -q[1];
    if (fb) q[2] = -q[2];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3) V.q(v, hy, hx) = q[v];
    if (G.tc) V.temp(hy, hx) = div_by_rcp(q[4], q[0], y);
  }
}

// Phase 1 for an interior block whose halo rows [h0, h1) were staged by
// tensor copies: the conserved values sit in the primitive slots of their
// own cells and are converted in place (the arithmetic of load_prims64; no
// ghost cells, so no reflections).
template <int PLANE, bool WACT, class TL, class PV>
__device__ __forceinline__ void convert_rows64(const Grid& G, const PV& V, int h0, int h1, int tid,
                                               bool prims = false) {
  constexpr int HX = TL::HX;
  if (prims && !G.tc) return;  // staged primitives need no conversion
  const int n = (h1 - h0) * HX;
  for (int idx = tid; idx < n; idx += kTileThreads) {
    const int r = idx / HX, hx = idx - r * HX;
    const int hy = h0 + r;
    if (prims) {  // only the temperature
      const double r = V.q(0, hy, hx), p = V.q(4, hy, hx);
      V.temp(hy, hx) = div_by_rcp(p, r, 1.0 / r);
      continue;
    }
    double u[5], q[5], y;
    u[0] = V.q(0, hy, hx);
    u[1] = V.q(1, hy, hx);
    u[2] = V.q(2, hy, hx);
    u[3] = WACT ? V.q(3, hy, hx) : 0.0;
    u[4] = V.q(4, hy, hx);
    cons_to_prim64<PLANE, WACT>(u, G.gm1, q, y);
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3) V.q(v, hy, hx) = q[v];
    if (G.tc) V.temp(hy, hx) = div_by_rcp(q[4], q[0], y);
  }
}

// Stages halo rows [h0, h1) (a multiple of kTmaRows, never wrapping the
// ring inside a chunk) of the block whose first cell is (x0, y0) into the
// primitive slots by tensor copies, and waits for them.  Every thread calls
// it; thread 0 issues.  The caller has synchronised the CTA since the slots
// were last read.  Returns false when the wait ran out (ctrl->err is set).
template <bool WACT, class TL, class PV>
__device__ __forceinline__ bool stage_rows_tma(const TmaState* tin, const PV& V, unsigned long long* mbar,
                                               unsigned& phase, int x0, int y0, int h0, int h1, StepCtrl* ctrl) {
  constexpr int HX = TL::HX;
  // a tensor copy's shared-memory destination must be 128-byte aligned: every
  // chunk starts a whole number of chunks into the 128-byte aligned ring
  static_assert((kTmaRows * HX * sizeof(double)) % 128 == 0, "TMA chunk of the ring not a multiple of 128 bytes");
  static_assert(4 % kTmaRows == 0 && TL::TY % kTmaRows == 0, "TMA chunks must tile the ring's new rows");
  if (threadIdx.x == 0) {
    fence_proxy_async();
    const unsigned nf = WACT ? 5u : 4u;
    mbar_arrive_expect_tx(mbar, nf * (unsigned)(h1 - h0) * HX * (unsigned)sizeof(double));
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if (!WACT && v == 3) continue;
      for (int hy = h0; hy < h1; hy += kTmaRows) tma_load_2d(&V.q(v, hy, 0), &tin->m[v], x0 - 2, y0 - 2 + hy, mbar);
    }
  }
  const bool ok = mbar_wait(mbar, phase);
  phase ^= 1u;
  if (!ok) atomicOr(&ctrl->err, 2);
  return ok;
}

// Phase 2: a faces of cell rows 0..nr-1 and b faces of face rows fb0..nr of
// the block (b face row fy lies between cell rows fy-1 and fy), each solved
// once; with VSH, their viscous fluxes too.
template <int PLANE, bool WACT, class TL, bool VSH, class PV>
__device__ __forceinline__ void faces64(const Grid& G, const Consts64& K, const PV& V, int rs, int nr, int fb0,
                                        int tid) {
  constexpr int TX = TL::TX;
  const bool plm = G.recon == R_PLM;
  const bool wb_z = PLANE == PLANE_XZ && G.recon == R_PCM_WB;
  const int nfa = (TX + 1) * nr;
  const int nfa_pad = (nfa + 31) & ~31;  // keeps each warp on one face kind
  const int n = nfa_pad + TX * (nr + 1 - fb0);
  for (int it = tid; it < n; it += kTileThreads) {
    double c[4][5], f[5];
    if (it < nfa_pad) {
      if (it >= nfa) continue;
      const int fy = it / (TX + 1), fx = it - fy * (TX + 1);
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int v = 0; v < 5; ++v) c[k][v] = (WACT || v != 3) ? V.q(v, fy + 2, fx + k) : 0.0;
      face_flux64<PLANE, WACT, 0>(c, rs, plm, wb_z, G, K, f);
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
        for (int v = 0; v < 5; ++v) c[k][v] = (WACT || v != 3) ? V.q(v, fy + k, fx + 2) : 0.0;
      face_flux64<PLANE, WACT, 1>(c, rs, plm, wb_z, G, K, f);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) V.fb(v, fy, fx) = f[v];
    }
  }
  if (VSH && WACT && G.visc) visc_faces<PLANE, TL>(V, G.inv_dx, G.inv_dy, G.inv_dz, G.mu, nr, fb0, tid);
}

// Phase 3-5: the cells of rows 0..nr-1 of the block -- conservative update,
// sources, RK2 combination, CFL term (max folded into red).
//
// qout (optional, last stage of a step): the primitives of the result are
// also written there, in the state's own layout, for the next step's load.
template <int PLANE, bool WACT, class TL, bool P2, bool VSH, class PV>
__device__ __forceinline__ void update64(const Grid& G, const PV& V, const Fields& uin, const Fields& u0,
                                         const Fields& uout, StepCtrl* ctrl, int kind, double dt, int x0, int y0,
                                         int nr, int tid, const Fields* hout, unsigned long long& red,
                                         const Fields* qout = nullptr) {
  constexpr int TX = TL::TX;
  const double db = PLANE == PLANE_XY ? G.dy : G.dz;
  const double inv_db = PLANE == PLANE_XY ? G.inv_dy : G.inv_dz;
  const int ncell = TX * nr;
#pragma unroll 1
  for (int cidx = tid; cidx < ncell; cidx += kTileThreads) {
    const int cx = cidx % TX, cy = cidx / TX;
    const int x = x0 + cx, y = y0 + cy;
    if (x >= G.na || y >= G.nb) continue;
    const long long o = (long long)y * G.pitch + x;
    double un[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) un[v] = (WACT || v != 3) ? uin.f[v][o] : 0.0;

    // IX sweep: un += (F(i-1/2) - F(i+1/2)) * dt / dx
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3)
        un[v] = un[v] + div_cell<P2>((V.fa(v, cy, cx) - V.fa(v, cy, cx + 1)) * dt, G.dx, G.inv_dx);
    // IY sweep (x-y plane) or IZ sweep (x-z plane), gravity on IZ
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3)
        un[v] = un[v] + div_cell<P2>((V.fb(v, cy, cx) - V.fb(v, cy + 1, cx)) * dt, db, inv_db);
    if (PLANE == PLANE_XZ && G.gravity) {
      un[2] = un[2] + dt * V.q(0, cy + 2, cx + 2) * G.g;
      un[4] = un[4] + half64(dt) * (V.fb(0, cy, cx) + V.fb(0, cy + 1, cx)) * G.g;
    }
    un[0] = fmax_bits(1.0e-6, un[0]);

    if (G.tc) {  // ThermalConduction.h:47-95, constant kappa, 2-D
      const double kf = half64(G.kappa + G.kappa);
      const int hy = cy + 2, hx = cx + 2;
      const double TC = V.temp(hy, hx);
      const double FL = div_cell<P2>(kf * (TC - V.temp(hy, hx - 1)), G.dx, G.inv_dx);
      const double FR = div_cell<P2>(kf * (V.temp(hy, hx + 1) - TC), G.dx, G.inv_dx);
      const double FU = div_cell<P2>(kf * (TC - V.temp(hy - 1, hx)), db, inv_db);
      const double FD = div_cell<P2>(kf * (V.temp(hy + 1, hx) - TC), db, inv_db);
      const double dtdx = div_cell<P2>(dt, G.dx, G.inv_dx);
      const double dtdb = div_cell<P2>(dt, db, inv_db);
      un[4] = un[4] + (dtdx * (FR - FL) + dtdb * (FD - FU));
    }
    if (WACT && G.visc) {  // Viscosity.h:245-251
      PlaneVel<PLANE, PV> P{V, cy + 2, cx + 2};
      double vf[3][5];
      if (VSH) {
        visc_cell_shared<PLANE>(V, cy, cx, G.inv_dx, G.inv_dz, G.mu, vf);
      } else {
        viscous_plane<PLANE, double>(P, G.inv_dx, G.inv_dy, G.inv_dz, G.mu, vf);
      }
#pragma unroll
      for (int var = 1; var < 5; ++var) {
        const int sv = var == 4 ? 4 : phys_slot<PLANE>(var);
        un[sv] = un[sv] + (vf[0][var] + vf[1][var] + vf[2][var]) * dt;
      }
    }
    if (kind == STAGE_RK_2) {
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) un[v] = half64(u0.f[v][o] + un[v]);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3) uout.f[v][o] = un[v];
    if (kind != STAGE_RK_1) {
      double q[5];
      const double inv = inv_dt_hyp64<PLANE, WACT, P2>(un, G, q);
      const unsigned long long b = (unsigned long long)__double_as_longlong(inv);
      red = b > red ? b : red;
      if (above_bits(inv, 1.0e300)) atomicOr(&ctrl->err, 1);
      if (hout) {
        const long long h = (long long)y * G.na + x;
#pragma unroll
        for (int v = 0; v < 5; ++v)
          if (hout->f[v]) hout->f[v][h] = q[v];
      }
      if (qout) {
#pragma unroll
        for (int v = 0; v < 5; ++v)
          if (WACT || v != 3) qout->f[v][o] = q[v];
      }
    }
  }
}

// An inactive Euler step still hands its state on (ping-pong buffers); RK2
// stages leave everything in place.  Copies cell rows [y0, y1) of columns
// [x0, x0 + TX).
template <bool WACT, int TX>
__device__ __forceinline__ void pass_on64(const Grid& G, const Fields& uin, const Fields& uout, int x0, int y0,
                                          int y1, int tid) {
  const int n = TX * (y1 - y0);
  for (int c = tid; c < n; c += kTileThreads) {
    const int x = x0 + c % TX, y = y0 + c / TX;
    if (x < G.na && y < G.nb) {
      const long long o = (long long)y * G.pitch + x;
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) uout.f[v][o] = uin.f[v][o];
    }
  }
}

// One strip segment: cell rows [ya, yb) of the TX-wide strip whose first
// column is x0, marched in blocks of TY rows through a ring of TY + 4
// primitive rows, so each block converts only its new rows and reuses the
// b-face fluxes on the boundary with the previous block; with viscosity the
// face-only viscous branches are computed once per face (viscous_face).  The
// arithmetic of every face and cell is that of the reference's euler_step,
// however the rows are split into segments.  Every thread of the CTA calls
// it (ctrl active); the CFL maximum is folded into red; smem holds
// bytes_vface() with viscosity, else bytes(G.tc).
//
// tin / mbar (optional, single-problem kernel): TMA descriptors of uin and
// the CTA's mbarrier; full blocks whose halo lies inside the grid are then
// staged by tensor copies (stage_rows_tma) and converted in place.
// qin (optional): the primitive copy of uin; the halo is then read (or
// staged, tin then describing qin) from it and only the temperature is
// computed.  qout (optional): receives the primitives of uout (update64).
template <int PLANE, bool WACT, class TL, bool P2>
__device__ __forceinline__ void stage_segment64(const Grid& G, const Fields& uin, const Fields& u0,
                                                const Fields& uout, StepCtrl* ctrl, int rs, int kind, double dt,
                                                int x0, int ya, int yb, double* smem, const Fields* hout,
                                                unsigned long long& red, const TmaState* tin = nullptr,
                                                unsigned long long* mbar = nullptr, unsigned* phase = nullptr,
                                                const Fields* qin = nullptr, const Fields* qout = nullptr) {
  constexpr int NV = WACT ? 5 : 4;
  constexpr int TX = TL::TX, TY = TL::TY, HY = TL::HY;
  using SM = TileSmem<double, NV, TL>;
  const SM S{smem};
  const int tid = threadIdx.x;
  const Consts64 K{G.gamma, G.gm1, G.inv_gm1};
  const bool vsh = WACT && G.visc;
  int base = 0;
  for (int y0 = ya; y0 < yb; y0 += TY) {
    const int nr = yb - y0 < TY ? yb - y0 : TY;
    const bool first = y0 == ya;
    const PrimView<SM, RowsRing<HY>> V{S, RowsRing<HY>{base}};
    if (!first) {  // b faces on the boundary with the previous (full) block
      for (int i = tid; i < NV * TX; i += kTileThreads) {
        const int v = i / TX, fx = i - v * TX;
        const int sv = NV == 5 ? v : (v == 3 ? 4 : v);
        S.fb(sv, 0, fx) = S.fb(sv, TY, fx);
      }
      if (vsh && PLANE == PLANE_XY)
        for (int i = tid; i < 4 * TX; i += kTileThreads) {
          const int k = i / TX, fx = i - k * TX;
          S.vb(k, 0, fx) = S.vb(k, TY, fx);
        }
    }
    const int h0 = first ? 0 : 4;
    const bool staged = tin && nr == TY && x0 >= 2 && x0 + TX + 2 <= G.na && y0 + h0 >= 2 && y0 + TY + 2 <= G.nb;
    if (staged) {
      stage_rows_tma<WACT, TL>(tin, V, mbar, *phase, x0, y0, h0, TY + 4, ctrl);
      convert_rows64<PLANE, WACT, TL>(G, V, h0, TY + 4, tid, qin != nullptr);
    } else {
      load_prims64<PLANE, WACT, TL>(G, qin ? *qin : uin, V, x0, y0, h0, nr + 4, tid, qin != nullptr);
    }
    __syncthreads();
    faces64<PLANE, WACT, TL, WACT>(G, K, V, rs, nr, first ? 0 : 1, tid);
    __syncthreads();
    update64<PLANE, WACT, TL, P2, WACT>(G, V, uin, u0, uout, ctrl, kind, dt, x0, y0, nr, tid, hout, red, qout);
    __syncthreads();
    base += TY;
    if (base >= HY) base -= HY;
  }
}

// One stage of a run of cell rows of problem G, marching down TX-wide strips.
// The rows are numbered strip by strip (unit u = strip * nb + row) and the
// CTA owns units [u0_, u1_), processed as strip segments (stage_segment64).
// Host code splits the units evenly over the CTAs that fit on the GPU at
// once, which balances the FP64 work per SM whatever the grid shape.
// qin / qout: the primitive copy of the state read in place of uin's
// conversion (when ctrl->q_valid) / written by the last stage of a step.
template <int PLANE, bool WACT, class TL, bool P2>
__device__ __forceinline__ void stage_strip64(const Grid& G, const Fields& uin, const Fields& u0, const Fields& uout,
                                              StepCtrl* ctrl, int rs, int kind, long long u0_, long long u1_,
                                              double* smem, unsigned long long* s_red, const Fields* hout,
                                              const TmaState* tin = nullptr, unsigned long long* mbar = nullptr,
                                              const Fields* qin = nullptr, const Fields* qout = nullptr) {
  constexpr int TX = TL::TX;
  const int tid = threadIdx.x;
  const int active = ctrl->active;
  const double dt = ctrl->dt_cur;
  const int parity = ctrl->parity;
  unsigned long long red = 0ull;
  unsigned phase = 0u;
  for (long long u = u0_; u < u1_;) {
    const int strip = (int)(u / G.nb);
    const int ya = (int)(u - (long long)strip * G.nb);
    const int yb = (int)(ya + (u1_ - u) < (long long)G.nb ? ya + (u1_ - u) : (long long)G.nb);
    const int x0 = strip * TX;
    u += yb - ya;
    if (!active) {
      if (kind == STAGE_EULER) pass_on64<WACT, TX>(G, uin, uout, x0, ya, yb, tid);
      continue;
    }
    stage_segment64<PLANE, WACT, TL, P2>(G, uin, u0, uout, ctrl, rs, kind, dt, x0, ya, yb, smem, hout, red, tin,
                                         mbar, &phase, qin, qout);
  }
  if (active && kind != STAGE_RK_1) block_max_atomic(red, &ctrl->slot[parity ^ 1], s_red);
  // the copy is complete once this launch is (the next reader is a later kernel)
  if (active && qout && tid == 0) ctrl->q_valid = 1;
}

// Viscous fluxes of Viscosity.h:40-143 with the reference's arithmetic,
// including its z-branch index and field mix-ups (CORR: the z branch as the
// mirror of the x / y branches instead).  P(dk, dj, di, var) reads velocity
// var (1 u, 2 v, 3 w) at offset (dk-1, dj-1, di-1) along (z, y, x), i.e.
// stencil[dk][dj][di][var].
template <bool CORR, class T, class PA>
__device__ __forceinline__ void viscous3d(const PA& P, T odx, T ody, T odz, T mu, T vf[3][5]) {
  const T four_thirds = T(4.0 / 3.0);
  const T two_thirds = T(2.0 / 3.0);
  const T c4x = half_of(half_of(odx)), c4y = half_of(half_of(ody)), c4z = half_of(half_of(odz));
  const int U = 1, V = 2, W = 3;
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int v = 0; v < 5; ++v) vf[d][v] = T(0);
#pragma unroll
  for (int s = 1; s < 3; ++s) {  // IX
    const T sm = (s == 1 ? T(-1) : T(1)) * mu;
    const T qiu = half_of(P(1, 1, s, U) + P(1, 1, s - 1, U));
    const T qiv = half_of(P(1, 1, s, V) + P(1, 1, s - 1, V));
    const T qiw = half_of(P(1, 1, s, W) + P(1, 1, s - 1, W));
    const T dudx = odx * (P(1, 1, s, U) - P(1, 1, s - 1, U));
    const T dvdx = odx * (P(1, 1, s, V) - P(1, 1, s - 1, V));
    const T dwdx = odx * (P(1, 1, s, W) - P(1, 1, s - 1, W));
    const T dudy = c4y * (P(1, 2, s, U) - P(1, 0, s, U) + P(1, 2, s - 1, U) - P(1, 0, s - 1, U));
    const T dvdy = c4y * (P(1, 2, s, V) - P(1, 0, s, V) + P(1, 2, s - 1, V) - P(1, 0, s - 1, V));
    const T dudz = c4z * (P(2, 1, s, U) - P(0, 1, s, U) + P(2, 1, s - 1, U) - P(0, 1, s - 1, U));
    const T dwdz = c4z * (P(2, 1, s, W) - P(0, 1, s, W) + P(2, 1, s - 1, W) - P(0, 1, s - 1, W));
    const T tau_xx = four_thirds * dudx - two_thirds * (dvdy + dwdz);
    const T tau_xy = dvdx + dudy;
    const T tau_xz = dwdx + dudz;
    vf[0][1] += sm * tau_xx;
    vf[0][2] += sm * tau_xy;
    vf[0][3] += sm * tau_xz;
    vf[0][4] += sm * (tau_xx * qiu + tau_xy * qiv + tau_xz * qiw);
  }
#pragma unroll
  for (int s = 1; s < 3; ++s) {  // IY
    const T sm = (s == 1 ? T(-1) : T(1)) * mu;
    const T qiu = half_of(P(1, s, 1, U) + P(1, s - 1, 1, U));
    const T qiv = half_of(P(1, s, 1, V) + P(1, s - 1, 1, V));
    const T qiw = half_of(P(1, s, 1, W) + P(1, s - 1, 1, W));
    const T dudy = ody * (P(1, s, 1, U) - P(1, s - 1, 1, U));
    const T dvdy = ody * (P(1, s, 1, V) - P(1, s - 1, 1, V));
    const T dwdy = ody * (P(1, s, 1, W) - P(1, s - 1, 1, W));
    const T dudx = c4x * (P(1, s, 2, U) - P(1, s, 0, U) + P(1, s - 1, 2, U) - P(1, s - 1, 0, U));
    const T dvdx = c4x * (P(1, s, 2, V) - P(1, s, 0, V) + P(1, s - 1, 2, V) - P(1, s - 1, 0, V));
    const T dwdz = c4z * (P(2, s, 1, W) - P(0, s, 1, W) + P(2, s - 1, 1, W) - P(0, s - 1, 1, W));
    const T dvdz = c4z * (P(2, s, 1, V) - P(0, s, 1, V) + P(2, s - 1, 1, V) - P(0, s - 1, 1, V));
    const T tau_yy = four_thirds * dvdy - two_thirds * (dudx + dwdz);
    const T tau_xy = dvdx + dudy;
    const T tau_yz = dvdz + dwdy;
    vf[1][1] += sm * tau_xy;
    vf[1][2] += sm * tau_yy;
    vf[1][3] += sm * tau_yz;
    vf[1][4] += sm * (tau_xy * qiu + tau_yy * qiv + tau_yz * qiw);
  }
#pragma unroll
  for (int s = 1; s < 3; ++s) {  // IZ, with the reference's mix-ups
    const T sm = (s == 1 ? T(-1) : T(1)) * mu;
    const T qiu = half_of(P(s, 1, 1, U) + P(s - 1, 1, 1, U));
    const T qiv = half_of(P(s, 1, 1, V) + P(s - 1, 1, 1, V));
    const T qiw = half_of(P(s, 1, 1, W) + P(s - 1, 1, 1, W));
    const T dudz = odz * (P(s, 1, 1, U) - P(s - 1, 1, 1, U));
    const T dvdz = odz * (P(s, 1, 1, V) - P(s - 1, 1, 1, V));
    const T dwdz = odz * (P(s, 1, 1, W) - P(s - 1, 1, 1, W));
    T dudx, dwdx, dvdy, dwdy;
    if (CORR) {
      dudx = c4x * (P(s, 1, 2, U) - P(s, 1, 0, U) + P(s - 1, 1, 2, U) - P(s - 1, 1, 0, U));
      dwdx = c4x * (P(s, 1, 2, W) - P(s, 1, 0, W) + P(s - 1, 1, 2, W) - P(s - 1, 1, 0, W));
      dvdy = c4y * (P(s, 2, 1, V) - P(s, 0, 1, V) + P(s - 1, 2, 1, V) - P(s - 1, 0, 1, V));
      dwdy = c4y * (P(s, 2, 1, W) - P(s, 0, 1, W) + P(s - 1, 2, 1, W) - P(s - 1, 0, 1, W));
    } else {
      dudx = c4x * (P(s, 1, 2, U) - P(1, s, 0, U) + P(s - 1, 1, 2, U) - P(1, s - 1, 0, U));
      dwdx = c4x * (P(s, 1, 2, V) - P(1, s, 0, W) + P(s - 1, 1, 2, V) - P(1, s - 1, 0, W));
      dvdy = c4z * (P(s, 2, 1, W) - P(s, 0, 1, V) + P(s - 1, 2, 1, W) - P(s - 1, 0, 1, V));
      dwdy = c4z * (P(s, 2, 1, V) - P(s, 0, 1, W) + P(s - 1, 2, 1, V) - P(s - 1, 0, 1, W));
    }
    const T tau_zz = four_thirds * dwdz - two_thirds * (dudx + dvdy);
    const T tau_xz = dudz + dwdx;
    const T tau_yz = dvdz + dwdy;
    vf[2][1] += sm * tau_xz;
    vf[2][2] += sm * tau_yz;
    vf[2][3] += sm * tau_zz;
    vf[2][4] += sm * (tau_xz * qiu + tau_yz * qiv + tau_zz * qiw);
  }
}


}  // namespace fv
