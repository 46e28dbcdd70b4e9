// fv_stage2d.cu -- FP64 fused stage kernel for 2-D runs, plus the dt
// reduction, control, conversion and conservation-sum kernels.
//
// One launch performs a whole reference euler_step (Update.h:164-178) for a
// 32x8 tile of cells per CTA:
//   1. load the tile plus a 2-cell halo of the stage's input conserved state,
//      synthesising ghost cells by index remapping (the X-then-Y ghost fill of
//      BoundaryConditions.h:146-192, corners included) and converting to
//      primitives (consToPrim, States.h:34-45) into shared memory;
//   2. minmod slopes and PLM face states (Update.h:14-33,55-88), one Riemann
//      solve per face (RiemannSolvers.h) -- the reference solves every face
//      twice, once from each side, with identical inputs;
//   3. the conservative update in the reference's X, Y, Z order with
//      (F*dt)/d increments, gravity on the z sweep, the density floor
//      (Update.h:145-160), thermal conduction (ThermalConduction.h:38-96) and
//      viscosity (Viscosity.h:127-253), all reading the same primitive tile;
//   4. for RK2 stage 2 the SSP average 0.5*(U^n + U**) (Update.h:198-204);
//   5. for the last stage of a step, consToPrim of the result and the
//      hyperbolic CFL term of ComputeDt.h:28-54, reduced to one atomic max
//      per CTA (the TC/viscous terms are constants, folded in on the host).
//
// The degenerate third axis (one cell, ghost layers equal to it) contributes
// exactly zero to every flux difference in the reference arithmetic, so its
// sweep is skipped; its cell size still enters dt.
#include <cstdio>

#include "fv_kernels.h"

namespace fv {

namespace {

constexpr int TX = kTileX, TY = kTileY, NT = TX * TY;
constexpr int HX = TX + 4, HY = TY + 4;

typedef double Tile[HY][HX];

// Storage-order velocity slots: 1 = a (x), 2 = b, 3 = c.  Physical x/y/z
// velocity of the reference -> storage slot.
template <int PLANE>
__device__ __forceinline__ constexpr int phys_slot(int var) {
  return var == 1 ? 1 : (PLANE == PLANE_XY ? (var == 2 ? 2 : 3) : (var == 2 ? 3 : 2));
}

// consToPrim (States.h:34-45) of a state held in storage order; returns
// (rho, u_a, u_b, u_c, p).  The kinetic energy sums the physical x, y, z
// velocities in that order.
template <int PLANE>
__device__ __forceinline__ void cons_to_prim_storage(const double u[5], double gamma, double q[5]) {
  const double r = u[0];
  const double va = u[1] / r, vb = u[2] / r, vc = u[3] / r;
  const double vx = va, vy = PLANE == PLANE_XY ? vb : vc, vz = PLANE == PLANE_XY ? vc : vb;
  const double Ek = 0.5 * r * (vx * vx + vy * vy + vz * vz);
  q[0] = r;
  q[1] = va;
  q[2] = vb;
  q[3] = vc;
  q[4] = (u[4] - Ek) * (gamma - 1.0);
}

// Face-state reconstruction (Update.h:14-33) for one variable; `sign` is +1
// for the left state of a face (right edge of its cell), -1 for the right.
__device__ __forceinline__ double recon_plm(double q, double slope, double sign) {
  return q + slope * sign * 0.5;
}

// Viscous flux of Viscosity.h:149-243 for the three directions, read through
// a 3x3x3 stencil accessor st(dk, dj, di, var) with var 1/2/3 = u/v/w, as the
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

// 3x3x3 stencil of the reference's viscosity over a 2-D plane: offsets along
// the degenerate axis return the centre layer (its ghosts are copies of it).
template <int PLANE>
struct PlaneStencil {
  const Tile* q;
  int hy, hx;
  __device__ __forceinline__ double operator()(int dk, int dj, int di, int var) const {
    const int ob = PLANE == PLANE_XY ? dj - 1 : dk - 1;
    return q[phys_slot<PLANE>(var)][hy + ob][hx + di - 1];
  }
};

// Block-wide max of a non-negative double (as bits, so NaN wins) and one
// atomic per CTA.
__device__ __forceinline__ void block_max_atomic(unsigned long long v, unsigned long long* slot,
                                                 unsigned long long* s_red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  if ((tid & 31) == 0) s_red[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    unsigned long long m = s_red[0];
    for (int w = 1; w < nw; ++w) m = s_red[w] > m ? s_red[w] : m;
    atomicMax(slot, m);
  }
}

// Hyperbolic inverse time step of one cell (ComputeDt.h:49-52) from its
// conserved state in storage order.
template <int PLANE>
__device__ __forceinline__ double inv_dt_hyp_cell(const double u[5], const Grid2D& G) {
  double q[5];
  cons_to_prim_storage<PLANE>(u, G.gamma, q);
  const double cs = sound_speed(q[0], q[4], G.gamma);
  const double vx = q[1], vy = PLANE == PLANE_XY ? q[2] : q[3], vz = PLANE == PLANE_XY ? q[3] : q[2];
  return (cs + fabs(vx)) / G.dx + (cs + fabs(vy)) / G.dy + (cs + fabs(vz)) / G.dz;
}

template <int PLANE, int RS, int KIND, bool WACT>
__global__ void __launch_bounds__(NT, 2)
stage2d_fp64(const Grid2D G, const Fields uin, const Fields u0, const Fields uout, StepCtrl* __restrict__ ctrl) {
  __shared__ Tile s_q[5];                  // primitives (rho, u_a, u_b, u_c, p)
  __shared__ double s_fa[5][TY][TX + 1];   // a-face fluxes, storage order
  __shared__ double s_fb[5][TY + 1][TX];   // b-face fluxes, storage order
  __shared__ unsigned long long s_red[NT / 32];

  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + ty * TX;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int active = ctrl->active;
  const double dt = ctrl->dt_cur;
  const int parity = ctrl->parity;

  if (!active) {
    // An inactive Euler step still has to hand its state on (ping-pong
    // buffers); RK2 stages leave everything in place.
    if (KIND == STAGE_EULER) {
      const int x = x0 + tx, y = y0 + ty;
      if (x < G.na && y < G.nb) {
        const long long o = (long long)y * G.pitch + x;
#pragma unroll
        for (int v = 0; v < 5; ++v)
          if (WACT || v != 3) uout.f[v][o] = uin.f[v][o];
      }
    }
    return;
  }

  // ---- 1. tile + halo -> primitives in shared memory ----
  for (int idx = tid; idx < HX * HY; idx += NT) {
    const int hy = idx / HX, hx = idx - hy * HX;
    bool fa, fb;
    const int sa = bc_source(x0 + hx - 2, G.na, G.bc_a, fa);
    const int sb = bc_source(y0 + hy - 2, G.nb, G.bc_b, fb);
    const long long o = (long long)sb * G.pitch + sa;
    double u[5], q[5];
    u[0] = uin.f[0][o];
    u[1] = uin.f[1][o];
    u[2] = uin.f[2][o];
    u[3] = WACT ? uin.f[3][o] : 0.0;
    u[4] = uin.f[4][o];
    cons_to_prim_storage<PLANE>(u, G.gamma, q);
    if (fa) q[1] = -q[1];
    if (fb) q[2] = -q[2];
#pragma unroll
    for (int v = 0; v < 5; ++v) s_q[v][hy][hx] = q[v];
  }
  __syncthreads();

  const double gamma = G.gamma;
  const bool plm = G.recon == R_PLM;

  // ---- 2. a-direction faces (reference IX sweep) ----
  for (int f = tid; f < (TX + 1) * TY; f += NT) {
    const int fy = f / (TX + 1), fx = f - fy * (TX + 1);
    const int hy = fy + 2, hl = fx + 1, hr = fx + 2;
    double qL[5], qR[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if (v == 3 && !WACT) { qL[v] = 0.0; qR[v] = 0.0; continue; }
      const double a = s_q[v][hy][hl - 1], b = s_q[v][hy][hl], c = s_q[v][hy][hr], d = s_q[v][hy][hr + 1];
      if (plm) {
        qL[v] = recon_plm(b, minmod(b - a, c - b), 1.0);
        qR[v] = recon_plm(c, minmod(c - b, d - c), -1.0);
      } else {
        qL[v] = b;
        qR[v] = c;
      }
    }
    // IX slots: normal = x, t1 = y, t2 = z velocity.
    Slots<double> L, R;
    L.r = qL[0]; L.un = qL[1]; L.p = qL[4];
    R.r = qR[0]; R.un = qR[1]; R.p = qR[4];
    if (PLANE == PLANE_XY) { L.t1 = qL[2]; L.t2 = qL[3]; R.t1 = qR[2]; R.t2 = qR[3]; }
    else                   { L.t1 = qL[3]; L.t2 = qL[2]; R.t1 = qR[3]; R.t2 = qR[2]; }
    double fl[5];
    riemann<double, RS>(L, R, gamma, fl);
    s_fa[0][fy][fx] = fl[0];
    s_fa[1][fy][fx] = fl[1];
    s_fa[4][fy][fx] = fl[4];
    if (PLANE == PLANE_XY) { s_fa[2][fy][fx] = fl[2]; s_fa[3][fy][fx] = fl[3]; }
    else                   { s_fa[2][fy][fx] = fl[3]; s_fa[3][fy][fx] = fl[2]; }
  }

  // ---- 3. b-direction faces (reference IY sweep, or IZ in the x-z plane) ----
  const bool wb_z = PLANE == PLANE_XZ && G.recon == R_PCM_WB;
  for (int f = tid; f < TX * (TY + 1); f += NT) {
    const int fy = f / TX, fx = f - fy * TX;
    const int hx = fx + 2, hl = fy + 1, hr = fy + 2;
    double qL[5], qR[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if (v == 3 && !WACT) { qL[v] = 0.0; qR[v] = 0.0; continue; }
      const double a = s_q[v][hl - 1][hx], b = s_q[v][hl][hx], c = s_q[v][hr][hx], d = s_q[v][hr + 1][hx];
      if (plm) {
        qL[v] = recon_plm(b, minmod(b - a, c - b), 1.0);
        qR[v] = recon_plm(c, minmod(c - b, d - c), -1.0);
      } else {
        qL[v] = b;
        qR[v] = c;
      }
    }
    if (wb_z) {  // PCM_WB hydrostatic pressure in z (Update.h:27)
      qL[4] = qL[4] + 1.0 * qL[0] * G.g * G.dz * 0.5;
      qR[4] = qR[4] + -1.0 * qR[0] * G.g * G.dz * 0.5;
    }
    // IY slots: (v, u, w); IZ slots: (w, v, u).
    Slots<double> L, R;
    L.r = qL[0]; L.un = qL[2]; L.p = qL[4];
    R.r = qR[0]; R.un = qR[2]; R.p = qR[4];
    if (PLANE == PLANE_XY) { L.t1 = qL[1]; L.t2 = qL[3]; R.t1 = qR[1]; R.t2 = qR[3]; }
    else                   { L.t1 = qL[3]; L.t2 = qL[1]; R.t1 = qR[3]; R.t2 = qR[1]; }
    double fl[5];
    riemann<double, RS>(L, R, gamma, fl);
    s_fb[0][fy][fx] = fl[0];
    s_fb[2][fy][fx] = fl[1];
    s_fb[4][fy][fx] = fl[4];
    if (PLANE == PLANE_XY) { s_fb[1][fy][fx] = fl[2]; s_fb[3][fy][fx] = fl[3]; }
    else                   { s_fb[1][fy][fx] = fl[3]; s_fb[3][fy][fx] = fl[2]; }
  }
  __syncthreads();

  // ---- 4. conservative update of the CTA's cells ----
  const int x = x0 + tx, y = y0 + ty;
  const bool inside = x < G.na && y < G.nb;
  unsigned long long red = 0ull;
  if (inside) {
    const long long o = (long long)y * G.pitch + x;
    double un[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) un[v] = (WACT || v != 3) ? uin.f[v][o] : 0.0;

    // IX sweep
#pragma unroll
    for (int v = 0; v < 5; ++v) un[v] += (s_fa[v][ty][tx] - s_fa[v][ty][tx + 1]) * dt / G.dx;
    // IY sweep (x-y plane) or IZ sweep (x-z plane), with gravity on IZ
    const double db = PLANE == PLANE_XY ? G.dy : G.dz;
#pragma unroll
    for (int v = 0; v < 5; ++v) un[v] += (s_fb[v][ty][tx] - s_fb[v][ty + 1][tx]) * dt / db;
    if (PLANE == PLANE_XZ && G.gravity) {
      un[2] += dt * s_q[0][ty + 2][tx + 2] * G.g;
      un[4] += dt * 0.5 * (s_fb[0][ty][tx] + s_fb[0][ty + 1][tx]) * G.g;
    }
    un[0] = fmax(1.0e-6, un[0]);

    if (G.tc) {  // ThermalConduction.h:47-95, constant kappa, 2-D
      const double kf = 0.5 * (G.kappa + G.kappa);
      const int cy = ty + 2, cx = tx + 2;
      const double TC = s_q[4][cy][cx] / s_q[0][cy][cx];
      const double TL = s_q[4][cy][cx - 1] / s_q[0][cy][cx - 1];
      const double TR = s_q[4][cy][cx + 1] / s_q[0][cy][cx + 1];
      const double TU = s_q[4][cy - 1][cx] / s_q[0][cy - 1][cx];
      const double TD = s_q[4][cy + 1][cx] / s_q[0][cy + 1][cx];
      const double FL = kf * (TC - TL) / G.dx;
      const double FR = kf * (TR - TC) / G.dx;
      const double FU = kf * (TC - TU) / db;
      const double FD = kf * (TD - TC) / db;
      un[4] += dt / G.dx * (FR - FL) + dt / db * (FD - FU);
    }
    if (G.visc) {  // Viscosity.h:245-251
      PlaneStencil<PLANE> st{s_q, ty + 2, tx + 2};
      double vf[3][5];
      viscous_fluxes(st, G.dx, G.dy, G.dz, G.mu, vf);
#pragma unroll
      for (int var = 1; var < 5; ++var) {
        const int sv = var == 4 ? 4 : phys_slot<PLANE>(var);
        un[sv] += (vf[0][var] + vf[1][var] + vf[2][var]) * dt;
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
      const double inv = inv_dt_hyp_cell<PLANE>(un, G);
      red = (unsigned long long)__double_as_longlong(inv);
      if (!(inv <= 1.0e300)) atomicOr(&ctrl->err, 1);
    }
  }
  if (KIND != STAGE_RK_1) block_max_atomic(red, &ctrl->slot[parity ^ 1], s_red);
}

template <int PLANE, bool WACT>
__global__ void __launch_bounds__(256) reduce2d_fp64(const Grid2D G, const Fields u, StepCtrl* ctrl, int slot) {
  __shared__ unsigned long long s_red[8];
  unsigned long long red = 0ull;
  const long long n = (long long)G.na * G.nb;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    double w[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) w[v] = (WACT || v != 3) ? u.f[v][o] : 0.0;
    const double inv = inv_dt_hyp_cell<PLANE>(w, G);
    const unsigned long long b = (unsigned long long)__double_as_longlong(inv);
    red = b > red ? b : red;
    if (!(inv <= 1.0e300)) atomicOr(&ctrl->err, 1);
  }
  block_max_atomic(red, &ctrl->slot[slot], s_red);
}

__global__ void control_kernel(StepCtrl* ctrl, int n, int mode_override, double dt_given) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  StepCtrl& c = ctrl[i];
  const int p = (int)(c.step & 1);
  const int mode = mode_override >= 0 ? mode_override : c.mode;
  double dt;
  int active;
  if (mode == 0) {
    dt = mode_override == 0 ? dt_given : c.dt_given;
    active = 1;
  } else {
    // ComputeDt.h:62: CFL / max(inv_hyp, inv_tc, inv_visc); main.cpp:51 loop bound.
    const double inv_hyp = __longlong_as_double((long long)c.slot[p]);
    double m = inv_hyp;
    if (c.inv_tc > m) m = c.inv_tc;
    if (c.inv_visc > m) m = c.inv_visc;
    dt = c.cfl / m;
    // mode 2: fixed step count, no time bound; a previous error stops it
    active = mode == 2 ? !c.err
                       : (c.t + c.epsilon < c.tend) && (c.max_steps <= 0 || c.step < c.max_steps);
    if (active && !(dt > 0.0 && dt <= 1.0e300)) {
      c.err |= 1;
      active = 0;
    }
  }
  c.slot[p ^ 1] = 0ull;
  c.parity = p;
  c.active = active;
  c.dt_cur = active ? dt : 0.0;
  if (active) {
    c.t = c.t + dt;
    c.step = c.step + 1;
  }
}

// primToCons in place (States.h:20-31), rounding as the reference (no
// contraction).  Storage order in and out.
template <int PLANE>
__global__ void prim_to_cons2d(const Grid2D G, const Fields u) {
  const long long n = (long long)G.na * G.nb;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    const double r = u.f[0][o];
    const double ma = __dmul_rn(r, u.f[1][o]), mb = __dmul_rn(r, u.f[2][o]), mc = __dmul_rn(r, u.f[3][o]);
    const double mx = ma, my = PLANE == PLANE_XY ? mb : mc, mz = PLANE == PLANE_XY ? mc : mb;
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(mx, mx), __dmul_rn(my, my)), __dmul_rn(mz, mz));
    const double Ek = __ddiv_rn(__dmul_rn(0.5, s), r);
    const double E = __dadd_rn(Ek, __ddiv_rn(u.f[4][o], G.gamma - 1.0));
    u.f[1][o] = ma;
    u.f[2][o] = mb;
    u.f[3][o] = mc;
    u.f[4][o] = E;
  }
}

// consToPrim (States.h:34-45), rounding as the reference; src and dst may
// alias.
template <int PLANE>
__global__ void cons_to_prim2d(const Grid2D G, const Fields src, const Fields dst) {
  const long long n = (long long)G.na * G.nb;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    const double r = src.f[0][o];
    const double va = __ddiv_rn(src.f[1][o], r), vb = __ddiv_rn(src.f[2][o], r), vc = __ddiv_rn(src.f[3][o], r);
    const double vx = va, vy = PLANE == PLANE_XY ? vb : vc, vz = PLANE == PLANE_XY ? vc : vb;
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
    const double Ek = __dmul_rn(__dmul_rn(0.5, r), s);
    const double p = __dmul_rn(__dsub_rn(src.f[4][o], Ek), G.gamma - 1.0);
    dst.f[0][o] = r;
    dst.f[1][o] = va;
    dst.f[2][o] = vb;
    dst.f[3][o] = vc;
    dst.f[4][o] = p;
  }
}

// Neumaier-compensated accumulation.
__device__ __forceinline__ void kadd(double& s, double& c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x)) c += (s - t) + x;
  else c += (x - t) + s;
  s = t;
}

__global__ void __launch_bounds__(256) totals2d(const Grid2D G, const Fields u, double* partial) {
  __shared__ double s_sum[5][256], s_cmp[5][256];
  double s[5] = {0, 0, 0, 0, 0}, cc[5] = {0, 0, 0, 0, 0};
  const long long n = (long long)G.na * G.nb;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
#pragma unroll
    for (int v = 0; v < 5; ++v) kadd(s[v], cc[v], u.f[v][o]);
  }
  const int t = threadIdx.x;
#pragma unroll
  for (int v = 0; v < 5; ++v) { s_sum[v][t] = s[v]; s_cmp[v][t] = cc[v]; }
  __syncthreads();
  if (t < 5) {
    double S = 0.0, Cm = 0.0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      kadd(S, Cm, s_sum[t][i]);
      Cm += s_cmp[t][i];
    }
    partial[((long long)blockIdx.x * 5 + t) * 2 + 0] = S;
    partial[((long long)blockIdx.x * 5 + t) * 2 + 1] = Cm;
  }
}

template <int PLANE, int RS, bool WACT>
cudaError_t launch_stage_kind(const Grid2D& G, int kind, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                              cudaStream_t st) {
  dim3 block(TX, TY), grid((G.na + TX - 1) / TX, (G.nb + TY - 1) / TY);
  switch (kind) {
    case STAGE_EULER: stage2d_fp64<PLANE, RS, STAGE_EULER, WACT><<<grid, block, 0, st>>>(G, uin, u0, uout, ctrl); break;
    case STAGE_RK_1: stage2d_fp64<PLANE, RS, STAGE_RK_1, WACT><<<grid, block, 0, st>>>(G, uin, u0, uout, ctrl); break;
    default: stage2d_fp64<PLANE, RS, STAGE_RK_2, WACT><<<grid, block, 0, st>>>(G, uin, u0, uout, ctrl); break;
  }
  return cudaGetLastError();
}

template <int PLANE, int RS>
cudaError_t launch_stage_w(const Grid2D& G, int kind, bool wact, Fields uin, Fields u0, Fields uout,
                           StepCtrl* ctrl, cudaStream_t st) {
  return wact ? launch_stage_kind<PLANE, RS, true>(G, kind, uin, u0, uout, ctrl, st)
              : launch_stage_kind<PLANE, RS, false>(G, kind, uin, u0, uout, ctrl, st);
}

int grid_for(long long n, int block) {
  long long b = (n + block - 1) / block;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

}  // namespace

cudaError_t launch_stage2d(const Grid2D& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                           Fields uout, StepCtrl* ctrl, cudaStream_t st) {
  if (G.plane == PLANE_XY)
    return riemann_solver == 0 ? launch_stage_w<PLANE_XY, 0>(G, kind, wact, uin, u0, uout, ctrl, st)
                               : launch_stage_w<PLANE_XY, 1>(G, kind, wact, uin, u0, uout, ctrl, st);
  return riemann_solver == 0 ? launch_stage_w<PLANE_XZ, 0>(G, kind, wact, uin, u0, uout, ctrl, st)
                             : launch_stage_w<PLANE_XZ, 1>(G, kind, wact, uin, u0, uout, ctrl, st);
}

cudaError_t launch_reduce2d(const Grid2D& G, bool wact, Fields u, StepCtrl* ctrl, int slot, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.nb, 256);
  if (G.plane == PLANE_XY) {
    if (wact) reduce2d_fp64<PLANE_XY, true><<<grid, 256, 0, st>>>(G, u, ctrl, slot);
    else reduce2d_fp64<PLANE_XY, false><<<grid, 256, 0, st>>>(G, u, ctrl, slot);
  } else {
    if (wact) reduce2d_fp64<PLANE_XZ, true><<<grid, 256, 0, st>>>(G, u, ctrl, slot);
    else reduce2d_fp64<PLANE_XZ, false><<<grid, 256, 0, st>>>(G, u, ctrl, slot);
  }
  return cudaGetLastError();
}

cudaError_t launch_control(StepCtrl* ctrl, int n, int mode_override, double dt_given, cudaStream_t st) {
  control_kernel<<<(n + 127) / 128, 128, 0, st>>>(ctrl, n, mode_override, dt_given);
  return cudaGetLastError();
}

cudaError_t launch_prim_to_cons2d(const Grid2D& G, Fields u, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.nb, 256);
  if (G.plane == PLANE_XY) prim_to_cons2d<PLANE_XY><<<grid, 256, 0, st>>>(G, u);
  else prim_to_cons2d<PLANE_XZ><<<grid, 256, 0, st>>>(G, u);
  return cudaGetLastError();
}

cudaError_t launch_cons_to_prim2d(const Grid2D& G, Fields src, Fields dst, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.nb, 256);
  if (G.plane == PLANE_XY) cons_to_prim2d<PLANE_XY><<<grid, 256, 0, st>>>(G, src, dst);
  else cons_to_prim2d<PLANE_XZ><<<grid, 256, 0, st>>>(G, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_totals2d(const Grid2D& G, Fields u, double* partial, int max_blocks, int* nblocks,
                            cudaStream_t st) {
  int grid = grid_for((long long)G.na * G.nb, 256);
  if (grid > max_blocks) grid = max_blocks;
  *nblocks = grid;
  totals2d<<<grid, 256, 0, st>>>(G, u, partial);
  return cudaGetLastError();
}

}  // namespace fv
