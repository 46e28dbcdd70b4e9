// fv_stage2d.cu -- the FP64 fused stage kernel of 2-D runs.
//
// One launch performs a whole reference euler_step (Update.h:164-178) for a
// 32x16 tile of cells per CTA (256 threads):
//   1. load the tile plus a 2-cell halo of the stage's input conserved state,
//      synthesising ghost cells by index remapping (the X-then-Y ghost fill of
//      BoundaryConditions.h:146-192, corners included), and convert to
//      primitives (consToPrim, States.h:34-45) in shared memory;
//   2. for every face of the tile: minmod slopes and PLM face states
//      (Update.h:14-33,55-88) and one Riemann solve (RiemannSolvers.h) -- the
//      reference solves every face twice, from each side, with equal inputs;
//   3. the conservative update in the reference's X, Y, Z order with
//      (F*dt)/d increments, gravity on the z sweep and the density floor
//      (Update.h:145-160), then thermal conduction (ThermalConduction.h:38-96)
//      and viscosity (Viscosity.h:127-253) from the same primitive tile;
//   4. for RK2 stage 2 the SSP average 0.5*(U^n + U**) (Update.h:198-204);
//   5. for the last stage of a step, consToPrim of the result and the
//      hyperbolic CFL term of ComputeDt.h:28-54, reduced to one atomic max
//      per CTA (the TC/viscous terms are constants folded in by the control
//      kernel).
//
// Rounding: this file is compiled without FMA contraction, every operation
// follows the reference's order, and the cheaper exact forms of
// fv_exact64.cuh / fv_riemann64.cuh replace divisions and comparisons, so the
// result is bit-identical to the reference's FP64 CPU arithmetic.
//
// The degenerate third axis (one cell whose ghost layers equal it) adds
// exactly zero to every flux difference in the reference arithmetic, so its
// sweep is skipped; its cell size still enters dt.
#include "fv_kernels.h"
#include "fv_plane2d.cuh"
#include "fv_riemann64.cuh"

namespace fv {

namespace {

constexpr int TX = kTileX, TY = kTileY;          // cells per tile
constexpr int BX = 32, BY = 8, NT = BX * BY;     // threads per CTA
constexpr int RPT = TY / BY;                     // rows per thread in the cell phase
constexpr int HX = TX + 4, HY = TY + 4;          // tile + 2-cell halo
constexpr int NFA = (TX + 1) * TY;               // a-faces
constexpr int NFA_PAD = (NFA + 31) / 32 * 32;    // keeps every warp on one face kind
constexpr int NFB = TX * (TY + 1);               // b-faces
static_assert(TY % BY == 0, "tile rows must split evenly over thread rows");

// Shared-memory layout (doubles) for NV stored variables:
//   Q [NV][HY][HX]   primitives of tile + halo
//   FA[NV][TY][TX+1] a-face fluxes (storage order)
//   FB[NV][TY+1][TX] b-face fluxes (storage order)
//   T [HY][HX]       temperature p/rho (thermal conduction only)
template <int NV>
struct Smem {
  double* base;
  static constexpr int kQ = 0;
  static constexpr int kFA = NV * HY * HX;
  static constexpr int kFB = kFA + NV * TY * (TX + 1);
  static constexpr int kT = kFB + NV * (TY + 1) * TX;
  static constexpr int kEnd = kT;  // without T
  // storage variable (0 r, 1 a, 2 b, 3 c, 4 E/p) -> smem slot
  __device__ static constexpr int sv(int v) { return NV == 5 ? v : (v == 4 ? 3 : v); }
  __device__ double& q(int v, int hy, int hx) const { return base[kQ + (sv(v) * HY + hy) * HX + hx]; }
  __device__ double& fa(int v, int fy, int fx) const { return base[kFA + (sv(v) * TY + fy) * (TX + 1) + fx]; }
  __device__ double& fb(int v, int fy, int fx) const { return base[kFB + (sv(v) * (TY + 1) + fy) * TX + fx]; }
  __device__ double& T(int hy, int hx) const { return base[kT + hy * HX + hx]; }
};

// 3x3x3 stencil of the reference's viscosity over a 2-D plane: offsets along
// the degenerate axis return the centre layer (its ghosts are copies of it).
template <int PLANE, int NV>
struct PlaneStencil {
  Smem<NV> s;
  int hy, hx;
  __device__ __forceinline__ double operator()(int dk, int dj, int di, int var) const {
    const int ob = PLANE == PLANE_XY ? dj - 1 : dk - 1;
    return s.q(phys_slot<PLANE>(var), hy + ob, hx + di - 1);
  }
};

// Viscous flux of Viscosity.h:149-243 for the three directions through a
// 3x3x3 stencil accessor st(dk, dj, di, var) with var 1/2/3 = u/v/w, as the
// reference writes it (including its z-branch index and field mix-ups).
template <class ST>
__device__ __forceinline__ void viscous_fluxes(const ST& st, double dx, double dy, double dz, double mu,
                                               double vf[3][5]) {
  const double four_thirds = 4.0 / 3.0;
  const double two_thirds = 2.0 / 3.0;
  const double one_over_dx = 1.0 / dx;
  const double one_over_dy = 1.0 / dy;
  const double one_over_dz = 1.0 / dz;
  const int IU = 1, IV = 2, IW = 3;
#pragma unroll
  for (int dir = 0; dir < 3; ++dir) {
    double flux[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int side = 1; side < 3; ++side) {
      const double sign = (side == 1 ? -1.0 : 1.0);
      if (dir == 0) {
        const double qiu = (st(1, 1, side, IU) + st(1, 1, side - 1, IU)) * 0.5;
        const double qiv = (st(1, 1, side, IV) + st(1, 1, side - 1, IV)) * 0.5;
        const double qiw = (st(1, 1, side, IW) + st(1, 1, side - 1, IW)) * 0.5;
        const double dudx = one_over_dx * (st(1, 1, side, IU) - st(1, 1, side - 1, IU));
        const double dvdx = one_over_dx * (st(1, 1, side, IV) - st(1, 1, side - 1, IV));
        const double dwdx = one_over_dx * (st(1, 1, side, IW) - st(1, 1, side - 1, IW));
        const double dudy = 0.25 * one_over_dy * (st(1, 2, side, IU) - st(1, 0, side, IU)
                                                + st(1, 2, side - 1, IU) - st(1, 0, side - 1, IU));
        const double dvdy = 0.25 * one_over_dy * (st(1, 2, side, IV) - st(1, 0, side, IV)
                                                + st(1, 2, side - 1, IV) - st(1, 0, side - 1, IV));
        const double dudz = 0.25 * one_over_dz * (st(2, 1, side, IU) - st(0, 1, side, IU)
                                                + st(2, 1, side - 1, IU) - st(0, 1, side - 1, IU));
        const double dwdz = 0.25 * one_over_dz * (st(2, 1, side, IW) - st(0, 1, side, IW)
                                                + st(2, 1, side - 1, IW) - st(0, 1, side - 1, IW));
        const double tau_xx = four_thirds * dudx - two_thirds * (dvdy + dwdz);
        const double tau_xy = dvdx + dudy;
        const double tau_xz = dwdx + dudz;
        flux[1] += sign * mu * tau_xx;
        flux[2] += sign * mu * tau_xy;
        flux[3] += sign * mu * tau_xz;
        flux[4] += sign * mu * (tau_xx * qiu + tau_xy * qiv + tau_xz * qiw);
      } else if (dir == 1) {
        const double qiu = (st(1, side, 1, IU) + st(1, side - 1, 1, IU)) * 0.5;
        const double qiv = (st(1, side, 1, IV) + st(1, side - 1, 1, IV)) * 0.5;
        const double qiw = (st(1, side, 1, IW) + st(1, side - 1, 1, IW)) * 0.5;
        const double dudy = one_over_dy * (st(1, side, 1, IU) - st(1, side - 1, 1, IU));
        const double dvdy = one_over_dy * (st(1, side, 1, IV) - st(1, side - 1, 1, IV));
        const double dwdy = one_over_dy * (st(1, side, 1, IW) - st(1, side - 1, 1, IW));
        const double dudx = 0.25 * one_over_dx * (st(1, side, 2, IU) - st(1, side, 0, IU)
                                                + st(1, side - 1, 2, IU) - st(1, side - 1, 0, IU));
        const double dvdx = 0.25 * one_over_dx * (st(1, side, 2, IV) - st(1, side, 0, IV)
                                                + st(1, side - 1, 2, IV) - st(1, side - 1, 0, IV));
        const double dwdz = 0.25 * one_over_dz * (st(2, side, 1, IW) - st(0, side, 1, IW)
                                                + st(2, side - 1, 1, IW) - st(0, side - 1, 1, IW));
        const double dvdz = 0.25 * one_over_dz * (st(2, side, 1, IV) - st(0, side, 1, IV)
                                                + st(2, side - 1, 1, IV) - st(0, side - 1, 1, IV));
        const double tau_yy = four_thirds * dvdy - two_thirds * (dudx + dwdz);
        const double tau_xy = dvdx + dudy;
        const double tau_yz = dvdz + dwdy;
        flux[1] += sign * mu * tau_xy;
        flux[2] += sign * mu * tau_yy;
        flux[3] += sign * mu * tau_yz;
        flux[4] += sign * mu * (tau_xy * qiu + tau_yy * qiv + tau_yz * qiw);
      } else {
        const double qiu = (st(side, 1, 1, IU) + st(side - 1, 1, 1, IU)) * 0.5;
        const double qiv = (st(side, 1, 1, IV) + st(side - 1, 1, 1, IV)) * 0.5;
        const double qiw = (st(side, 1, 1, IW) + st(side - 1, 1, 1, IW)) * 0.5;
        const double dudz = one_over_dz * (st(side, 1, 1, IU) - st(side - 1, 1, 1, IU));
        const double dvdz = one_over_dz * (st(side, 1, 1, IV) - st(side - 1, 1, 1, IV));
        const double dwdz = one_over_dz * (st(side, 1, 1, IW) - st(side - 1, 1, 1, IW));
        const double dudx = 0.25 * one_over_dx * (st(side, 1, 2, IU) - st(1, side, 0, IU)
                                                + st(side - 1, 1, 2, IU) - st(1, side - 1, 0, IU));
        const double dwdx = 0.25 * one_over_dx * (st(side, 1, 2, IV) - st(1, side, 0, IW)
                                                + st(side - 1, 1, 2, IV) - st(1, side - 1, 0, IW));
        const double dvdy = 0.25 * one_over_dz * (st(side, 2, 1, IW) - st(side, 0, 1, IV)
                                                + st(side - 1, 2, 1, IW) - st(side - 1, 0, 1, IV));
        const double dwdy = 0.25 * one_over_dz * (st(side, 2, 1, IV) - st(side, 0, 1, IW)
                                                + st(side - 1, 2, 1, IV) - st(side - 1, 0, 1, IW));
        const double tau_zz = four_thirds * dwdz - two_thirds * (dudx + dvdy);
        const double tau_xz = dudz + dwdx;
        const double tau_yz = dvdz + dwdy;
        flux[1] += sign * mu * tau_xz;
        flux[2] += sign * mu * tau_yz;
        flux[3] += sign * mu * tau_zz;
        flux[4] += sign * mu * (tau_xz * qiu + tau_yz * qiv + tau_zz * qiw);
      }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) vf[dir][v] = flux[v];
  }
}

// One face: slopes, face states and the Riemann flux, stored in storage
// order.  DIR 0 = a sweep (reference IX), 1 = b sweep (IY in the x-y plane,
// IZ in the x-z plane).  c[k][v] holds variable v of the four cells around
// the face (left-left, left, right, right-right).
template <int PLANE, int RS, bool WACT, int DIR>
__device__ __forceinline__ void face_flux(const double c[4][5], bool plm, bool wb_z, const Grid2D& G,
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
    qL[4] = qL[4] + 1.0 * qL[0] * G.g * G.dz * 0.5;
    qR[4] = qR[4] + -1.0 * qR[0] * G.g * G.dz * 0.5;
  }
  Slots<double> L, R;
  L.r = qL[0]; L.p = qL[4];
  R.r = qR[0]; R.p = qR[4];
  if (DIR == 0) {  // IX slots (u, v, w)
    L.un = qL[1]; R.un = qR[1];
    if (PLANE == PLANE_XY) { L.t1 = qL[2]; L.t2 = qL[3]; R.t1 = qR[2]; R.t2 = qR[3]; }
    else                   { L.t1 = qL[3]; L.t2 = qL[2]; R.t1 = qR[3]; R.t2 = qR[2]; }
  } else {  // IY slots (v, u, w) / IZ slots (w, v, u)
    L.un = qL[2]; R.un = qR[2];
    if (PLANE == PLANE_XY) { L.t1 = qL[1]; L.t2 = qL[3]; R.t1 = qR[1]; R.t2 = qR[3]; }
    else                   { L.t1 = qL[3]; L.t2 = qL[1]; R.t1 = qR[3]; R.t2 = qR[1]; }
  }
  double f[5];
  riemann64<RS, ZS>(L, R, K, f);
  out[0] = f[0];
  out[4] = f[4];
  if (DIR == 0) {
    out[1] = f[1];
    if (PLANE == PLANE_XY) { out[2] = f[2]; out[3] = f[3]; }
    else                   { out[2] = f[3]; out[3] = f[2]; }
  } else {
    out[2] = f[1];
    if (PLANE == PLANE_XY) { out[1] = f[2]; out[3] = f[3]; }
    else                   { out[1] = f[3]; out[3] = f[2]; }
  }
}

template <int PLANE, int RS, int KIND, bool WACT>
__global__ void __launch_bounds__(NT, WACT ? 2 : 3)
stage2d_fp64(const Grid2D G, const Fields uin, const Fields u0, const Fields uout, StepCtrl* __restrict__ ctrl) {
  constexpr int NV = WACT ? 5 : 4;
  extern __shared__ double smem_raw[];
  __shared__ unsigned long long s_red[NT / 32];
  const Smem<NV> S{smem_raw};

  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + ty * BX;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int active = ctrl->active;
  const double dt = ctrl->dt_cur;
  const int parity = ctrl->parity;

  if (!active) {
    // An inactive Euler step still hands its state on (ping-pong buffers);
    // RK2 stages leave everything in place.
    if (KIND == STAGE_EULER) {
#pragma unroll
      for (int rr = 0; rr < RPT; ++rr) {
        const int x = x0 + tx, y = y0 + ty + BY * rr;
        if (x < G.na && y < G.nb) {
          const long long o = (long long)y * G.pitch + x;
#pragma unroll
          for (int v = 0; v < 5; ++v)
            if (WACT || v != 3) uout.f[v][o] = uin.f[v][o];
        }
      }
    }
    return;
  }

  const Consts64 K{G.gamma, G.gm1, G.inv_gm1};

  // ---- 1. tile + halo -> primitives (and temperature) in shared memory ----
  for (int idx = tid; idx < HX * HY; idx += NT) {
    const int hy = idx / HX, hx = idx - hy * HX;
    bool fa, fb;
    const int sa = bc_source(x0 + hx - 2, G.na, G.bc_a, fa);
    const int sb = bc_source(y0 + hy - 2, G.nb, G.bc_b, fb);
    const long long o = (long long)sb * G.pitch + sa;
    double u[5], q[5], y;
    u[0] = uin.f[0][o];
    u[1] = uin.f[1][o];
    u[2] = uin.f[2][o];
    u[3] = WACT ? uin.f[3][o] : 0.0;
    u[4] = uin.f[4][o];
    cons_to_prim64<PLANE, WACT>(u, G.gm1, q, y);
    if (fa) q[1] = -q[1];
    if (fb) q[2] = -q[2];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3) S.q(v, hy, hx) = q[v];
    if (G.tc) S.T(hy, hx) = div_by_rcp(q[4], q[0], y);
  }
  __syncthreads();

  // ---- 2. every face of the tile: a faces first, then b faces ----
  const bool plm = G.recon == R_PLM;
  const bool wb_z = PLANE == PLANE_XZ && G.recon == R_PCM_WB;
  for (int it = tid; it < NFA_PAD + NFB; it += NT) {
    double c[4][5], f[5];
    if (it < NFA_PAD) {
      if (it >= NFA) continue;
      const int fy = it / (TX + 1), fx = it - fy * (TX + 1);
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int v = 0; v < 5; ++v) c[k][v] = (WACT || v != 3) ? S.q(v, fy + 2, fx + k) : 0.0;
      face_flux<PLANE, RS, WACT, 0>(c, plm, wb_z, G, K, f);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) S.fa(v, fy, fx) = f[v];
    } else {
      const int j = it - NFA_PAD;
      const int fy = j / TX, fx = j - fy * TX;
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int v = 0; v < 5; ++v) c[k][v] = (WACT || v != 3) ? S.q(v, fy + k, fx + 2) : 0.0;
      face_flux<PLANE, RS, WACT, 1>(c, plm, wb_z, G, K, f);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) S.fb(v, fy, fx) = f[v];
    }
  }
  __syncthreads();

  // ---- 3-5. conservative update, sources, RK2 combination, CFL term ----
  const double db = PLANE == PLANE_XY ? G.dy : G.dz;
  const double inv_db = PLANE == PLANE_XY ? G.inv_dy : G.inv_dz;
  const bool pow2_b = PLANE == PLANE_XY ? G.pow2_y : G.pow2_z;
  unsigned long long red = 0ull;
#pragma unroll 1
  for (int rr = 0; rr < RPT; ++rr) {
    const int cy = ty + BY * rr;
    const int x = x0 + tx, y = y0 + cy;
    if (x >= G.na || y >= G.nb) continue;
    const long long o = (long long)y * G.pitch + x;
    double un[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) un[v] = (WACT || v != 3) ? uin.f[v][o] : 0.0;

    // IX sweep: un += (F(i-1/2) - F(i+1/2)) * dt / dx
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3)
        un[v] = un[v] + div_cell((S.fa(v, cy, tx) - S.fa(v, cy, tx + 1)) * dt, G.dx, G.inv_dx, G.pow2_x);
    // IY sweep (x-y plane) or IZ sweep (x-z plane), gravity on IZ
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3)
        un[v] = un[v] + div_cell((S.fb(v, cy, tx) - S.fb(v, cy + 1, tx)) * dt, db, inv_db, pow2_b);
    if (PLANE == PLANE_XZ && G.gravity) {
      un[2] = un[2] + dt * S.q(0, cy + 2, tx + 2) * G.g;
      un[4] = un[4] + dt * 0.5 * (S.fb(0, cy, tx) + S.fb(0, cy + 1, tx)) * G.g;
    }
    un[0] = fmax(1.0e-6, un[0]);

    if (G.tc) {  // ThermalConduction.h:47-95, constant kappa, 2-D
      const double kf = 0.5 * (G.kappa + G.kappa);
      const int hy = cy + 2, hx = tx + 2;
      const double TC = S.T(hy, hx);
      const double FL = div_cell(kf * (TC - S.T(hy, hx - 1)), G.dx, G.inv_dx, G.pow2_x);
      const double FR = div_cell(kf * (S.T(hy, hx + 1) - TC), G.dx, G.inv_dx, G.pow2_x);
      const double FU = div_cell(kf * (TC - S.T(hy - 1, hx)), db, inv_db, pow2_b);
      const double FD = div_cell(kf * (S.T(hy + 1, hx) - TC), db, inv_db, pow2_b);
      const double dtdx = div_cell(dt, G.dx, G.inv_dx, G.pow2_x);
      const double dtdb = div_cell(dt, db, inv_db, pow2_b);
      un[4] = un[4] + (dtdx * (FR - FL) + dtdb * (FD - FU));
    }
    if (WACT && G.visc) {  // Viscosity.h:245-251
      PlaneStencil<PLANE, NV> st{S, cy + 2, tx + 2};
      double vf[3][5];
      viscous_fluxes(st, G.dx, G.dy, G.dz, G.mu, vf);
#pragma unroll
      for (int var = 1; var < 5; ++var) {
        const int sv = var == 4 ? 4 : phys_slot<PLANE>(var);
        un[sv] = un[sv] + (vf[0][var] + vf[1][var] + vf[2][var]) * dt;
      }
    }
    if (KIND == STAGE_RK_2) {
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (WACT || v != 3) un[v] = 0.5 * (u0.f[v][o] + un[v]);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (WACT || v != 3) uout.f[v][o] = un[v];
    if (KIND != STAGE_RK_1) {
      const double inv = inv_dt_hyp64<PLANE, WACT>(un, G);
      const unsigned long long b = (unsigned long long)__double_as_longlong(inv);
      red = b > red ? b : red;
      if (!(inv <= 1.0e300)) atomicOr(&ctrl->err, 1);
    }
  }
  if (KIND != STAGE_RK_1) block_max_atomic(red, &ctrl->slot[parity ^ 1], s_red);
}

template <int NV>
size_t smem_bytes(bool tc) {
  return sizeof(double) * (size_t)(Smem<NV>::kEnd + (tc ? HY * HX : 0));
}

template <int PLANE, int RS, int KIND, bool WACT>
cudaError_t launch_one(const Grid2D& G, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl, cudaStream_t st) {
  constexpr int NV = WACT ? 5 : 4;
  auto kern = stage2d_fp64<PLANE, RS, KIND, WACT>;
  static bool attr_set = false;  // per instantiation, set once per process
  const size_t bytes = smem_bytes<NV>(G.tc != 0);
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_bytes<NV>(true));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 block(BX, BY), grid((G.na + TX - 1) / TX, (G.nb + TY - 1) / TY);
  kern<<<grid, block, bytes, st>>>(G, uin, u0, uout, ctrl);
  return cudaGetLastError();
}

template <int PLANE, int RS, bool WACT>
cudaError_t launch_kind(const Grid2D& G, int kind, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                        cudaStream_t st) {
  switch (kind) {
    case STAGE_EULER: return launch_one<PLANE, RS, STAGE_EULER, WACT>(G, uin, u0, uout, ctrl, st);
    case STAGE_RK_1: return launch_one<PLANE, RS, STAGE_RK_1, WACT>(G, uin, u0, uout, ctrl, st);
    default: return launch_one<PLANE, RS, STAGE_RK_2, WACT>(G, uin, u0, uout, ctrl, st);
  }
}

template <int PLANE, int RS>
cudaError_t launch_w(const Grid2D& G, int kind, bool wact, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                     cudaStream_t st) {
  return wact ? launch_kind<PLANE, RS, true>(G, kind, uin, u0, uout, ctrl, st)
              : launch_kind<PLANE, RS, false>(G, kind, uin, u0, uout, ctrl, st);
}

}  // namespace

cudaError_t launch_stage2d(const Grid2D& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                           Fields uout, StepCtrl* ctrl, cudaStream_t st) {
  if (G.plane == PLANE_XY)
    return riemann_solver == 0 ? launch_w<PLANE_XY, 0>(G, kind, wact, uin, u0, uout, ctrl, st)
                               : launch_w<PLANE_XY, 1>(G, kind, wact, uin, u0, uout, ctrl, st);
  return riemann_solver == 0 ? launch_w<PLANE_XZ, 0>(G, kind, wact, uin, u0, uout, ctrl, st)
                             : launch_w<PLANE_XZ, 1>(G, kind, wact, uin, u0, uout, ctrl, st);
}

}  // namespace fv
