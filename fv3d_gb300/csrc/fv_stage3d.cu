// fv_stage3d.cu -- the FP64 fused stage kernel of a 3-D problem.
//
// One CTA owns a 16 x 16 block of (x, y) columns and marches up a chunk of
// z layers.  A ring of four z layers of primitives (each with a 2-cell
// in-plane halo) sits in shared memory; layer k+2 is loaded while the x and y
// faces of layer k are solved, then every thread solves the z face above its
// own column and updates its cell.  The z flux below the cell is the one the
// same thread solved one layer earlier (kept in registers), so every face of
// the grid is solved exactly once.  Per layer:
//   1. load layer k+2 (ghost layers synthesised from the boundary
//      conditions, C91 ghosts computed by BoundaryConditions.h:87-134) and
//      convert to primitives (consToPrim, States.h:34-45); solve the x and y
//      faces of layer k (minmod slopes, PLM/PCM/PCM_WB states, HLL/HLLC);
//   2. per column: the z face k+1/2, then the update of Update.h:90-162 in
//      the reference's X, Y, Z order with gravity, the well-balanced / C91
//      z-boundary flux overrides and the density floor, thermal conduction
//      (ThermalConduction.h:38-96, with the fixed-temperature / fixed-gradient
//      z boundaries and z-dependent B02 conductivity), viscosity
//      (Viscosity.h:22-155, literal formula), the RK2 average and the CFL
//      term of ComputeDt.h:28-54 for the last stage of a step.
// Ghost cells follow the reference's fill order (x, then y over the full x
// range, then z over the full x-y range), which for index-mapped boundaries
// is the composition of the three per-axis maps.
//
// Compiled without FMA contraction, operation order as in the reference, the
// exact replacements of fv_exact64.cuh: bit-identical to the reference's FP64
// CPU arithmetic.
#include "fv_tile64.cuh"

namespace fv {

namespace {

constexpr int kTX = 16, kTY = 16;                // columns per CTA
constexpr int kMinLayersPerCta = 8;              // the prologue loads 4 layers and one extra z face
constexpr int kThreads = kTX * kTY;              // one thread per column
constexpr int kHX = kTX + 4, kHY = kTY + 4;      // layer with halo
constexpr int kLayer = kHX * kHY;
// Resident CTAs per SM the register allocation of the 3-D FP64 kernels
// targets.
#ifndef FV_3D64_MIN_CTAS
#define FV_3D64_MIN_CTAS 2
#endif
constexpr int kRing = 4;                         // z layers held
constexpr int kNFA = (kTX + 1) * kTY;            // x faces per layer
constexpr int kNFA_PAD = (kNFA + 31) / 32 * 32;  // keeps each warp on one face kind
constexpr int kNFB = kTX * (kTY + 1);            // y faces per layer
static_assert(kThreads == 256, "one thread per column");

// Shared memory: Q[ring][v][hy][hx] primitives, FA[v][fy][fx] x-face and
// FB[v][fy][fx] y-face fluxes of the current layer, TT[ring][hy][hx]
// temperature p/rho (conduction only).
struct Smem3 {
  double* base;
  static constexpr int kFA = kRing * 5 * kLayer;
  static constexpr int kFB = kFA + 5 * kTY * (kTX + 1);
  static constexpr int kT = kFB + 5 * (kTY + 1) * kTX;
  static constexpr size_t bytes(bool tc) { return sizeof(double) * (size_t)(kT + (tc ? kRing * kLayer : 0)); }
  __device__ double& q(int s, int v, int hy, int hx) const { return base[((s * 5 + v) * kHY + hy) * kHX + hx]; }
  __device__ double& fa(int v, int fy, int fx) const { return base[kFA + (v * kTY + fy) * (kTX + 1) + fx]; }
  __device__ double& fb(int v, int fy, int fx) const { return base[kFB + (v * (kTY + 1) + fy) * kTX + fx]; }
  __device__ double& temp(int s, int hy, int hx) const { return base[kT + (s * kHY + hy) * kHX + hx]; }
};

// Ring slot of z layer kg (kg >= -2).
__device__ __forceinline__ int slot_of(int kg) { return (kg + 4) & 3; }

// consToPrim of one stored cell (x, y, z storage order), RN(1/rho) in y.
// With qsrc (the primitive copy of u, the same bits) the primitives are read
// and y is computed only when need_y.
__device__ __forceinline__ void load_prim(const Fields& u, const Fields* qsrc, long long o, double gm1, double q[5],
                                          double& y, bool need_y = false) {
  if (qsrc) {
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v] = qsrc->f[v][o];
    y = need_y ? 1.0 / q[0] : 0.0;
    return;
  }
  double w[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) w[v] = u.f[v][o];
  cons_to_prim64<PLANE_XY, true>(w, gm1, q, y);
}

// fillC91 (BoundaryConditions.h:87-134) for ghost layer kg of column (sa, sb)
// (already mapped through the x / y boundaries, with their velocity flips).
// Note the reference scales the hydrostatic term by params.gravity, the
// boolean, not by g.
__device__ __forceinline__ void c91_ghost(const Grid& G, const Fields& u, const Fields* qsrc, long long col, bool fa,
                                          bool fb, int kg, double res[5]) {
  const int kref = kg < 0 ? 0 : G.nc - 1;
  const int ksym = kg < 0 ? -kg - 1 : 2 * G.nc - kg - 1;
  double qref[5], qsym[5], y;
  load_prim(u, qsrc, (long long)kref * G.nb * G.pitch + col, G.gm1, qref, y);
  load_prim(u, qsrc, (long long)ksym * G.nb * G.pitch + col, G.gm1, qsym, y);
  if (fa) {
    qref[1] = -qref[1];
    qsym[1] = -qsym[1];
  }
  if (fb) {
    qref[2] = -qref[2];
    qsym[2] = -qsym[2];
  }
  const double grav = G.gravity_flag ? 1.0 : 0.0;
  const double posz = G.zmin + ((double)kg + 0.5) * G.dz;
  if (kg < 0) {
    const double dz = posz - 0.5 * G.dz;
    const double T = 1.0 + posz * G.theta1;
    double p = qref[4] + dz * qref[0] * grav;
    double r = p / T;
    p = fmax(p, 1.0e-6);
    r = fmax(r, 1.0e-6);
    const double dratio = qsym[0] / r;
    res[0] = r;
    res[1] = qsym[1];
    res[2] = qsym[2];
    res[3] = -qsym[3] * dratio;
    res[4] = p;
  } else {
    const double Tref = qref[4] / qref[0];
    const double dz = posz - (1.0 - 0.5 * G.dz);
    const double T = Tref + dz * G.theta1;
    const double P = qref[4] + dz * qref[0] * grav;
    const double rho = P / T;
    res[4] = fmax(P, 1.0e-6);
    res[0] = fmax(rho, 1.0e-6);
    const double dratio = qsym[0] / rho;
    res[1] = qsym[1] * dratio;
    res[2] = qsym[2] * dratio;
    res[3] = -qsym[3] * dratio;
  }
}

// Loads z layer kg of the tile at (x0, y0) into ring slot slot_of(kg)
// (from the primitive copy qsrc of u when given).
__device__ __forceinline__ void load_layer(const Grid& G, const Fields& u, const Fields* qsrc, int x0, int y0, int kg,
                                           const Smem3& S, int tid) {
  const int s = slot_of(kg);
  const bool c91 = G.bc_c == DBC_C91 && (kg < 0 || kg >= G.nc);
  bool fz = false;
  const int sz = c91 ? 0 : bc_source(kg, G.nc, G.bc_c, fz);
  const long long zoff = (long long)sz * G.nb * G.pitch;
  for (int idx = tid; idx < kLayer; idx += kThreads) {
    const int hy = idx / kHX, hx = idx - hy * kHX;
    bool fa, fb;
    const int sa = bc_source(x0 + hx - 2, G.na, G.bc_a, fa);
    const int sb = bc_source(y0 + hy - 2, G.nb, G.bc_b, fb);
    const long long col = (long long)sb * G.pitch + sa;
    double q[5];
    double T = 0.0;
    if (!c91) {
      double y;
      load_prim(u, qsrc, zoff + col, G.gm1, q, y, G.tc != 0);
      if (fa) q[1] = -q[1];
      if (fb) q[2] = -q[2];
      if (fz) q[3] = -q[3];
      if (G.tc) T = div_by_rcp(q[4], q[0], y);
    } else {
      c91_ghost(G, u, qsrc, col, fa, fb, kg, q);
      if (G.tc) T = q[4] / q[0];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) S.q(s, v, hy, hx) = q[v];
    if (G.tc) S.temp(s, hy, hx) = T;
  }
}

// Slots of a sweep from (r, u, v, w, p): IX (u, v, w), IY (v, u, w),
// IZ (w, v, u) -- swap_component, States.h:104-111.
template <int DIR>
__device__ __forceinline__ Slots<double> slots3(const double q[5]) {
  Slots<double> s;
  s.r = q[0];
  s.p = q[4];
  s.un = DIR == 0 ? q[1] : (DIR == 1 ? q[2] : q[3]);
  s.t1 = DIR == 1 ? q[1] : q[2];
  s.t2 = DIR == 2 ? q[1] : q[3];
  return s;
}

template <int DIR>
__device__ __forceinline__ void unslot3(const double f[5], double out[5]) {
  out[0] = f[0];
  out[4] = f[4];
  if (DIR == 0) {
    out[1] = f[1]; out[2] = f[2]; out[3] = f[3];
  } else if (DIR == 1) {
    out[2] = f[1]; out[1] = f[2]; out[3] = f[3];
  } else {
    out[3] = f[1]; out[2] = f[2]; out[1] = f[3];
  }
}

// One face along DIR from the four cells around it (c[0..3]: left-left,
// left, right, right-right), in storage order; pout as in hll64 / hllc64.
// The z slopes take minmod(forward, backward) (Update.h:84), x and y
// minmod(backward, forward); the two orders differ only in the sign of a
// zero slope.
// CORR: corrected physics (HLLC with the kinetic energy of all three
// velocities).
template <int DIR, bool CORR>
__device__ __forceinline__ void face3(const double c[4][5], int rs, int recon, const Grid& G, const Consts64& K,
                                      double out[5], double* pout) {
  double qL[5], qR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    if (recon == R_PLM) {
      const double d01 = c[1][v] - c[0][v], d12 = c[2][v] - c[1][v], d23 = c[3][v] - c[2][v];
      const double sL = DIR == 2 ? minmod_exact(d12, d01) : minmod_exact(d01, d12);
      const double sR = DIR == 2 ? minmod_exact(d23, d12) : minmod_exact(d12, d23);
      qL[v] = recon_plus(c[1][v], sL);
      qR[v] = recon_minus(c[2][v], sR);
    } else {
      qL[v] = c[1][v];
      qR[v] = c[2][v];
    }
  }
  if (DIR == 2 && recon == R_PCM_WB) {  // Update.h:27
    qL[4] = qL[4] + half64(1.0 * qL[0] * G.g * G.dz);
    qR[4] = qR[4] + half64(-1.0 * qR[0] * G.g * G.dz);
  }
  const Slots<double> L = slots3<DIR>(qL), R = slots3<DIR>(qR);
  double f[5];
  if (rs == 0)
    hll64<0>(L, R, K, f, pout);
  else
    hllc64<0, CORR>(L, R, K, f, pout);
  unslot3<DIR>(f, out);
}

// Stencil accessor of viscous3d over the ring (column (hy, hx) of layer k).
struct RingVel {
  Smem3 S;
  int k, hy, hx;
  __device__ __forceinline__ double operator()(int dk, int dj, int di, int var) const {
    return S.q(slot_of(k + dk - 1), var, hy + dj - 1, hx + di - 1);
  }
};

// The viscous flux of one x face (DIR 0) or y face (DIR 1) of a layer for
// Viscosity.h's IX / IY branch, whose terms depend on the face alone:
// g = {mu*t1, mu*t2, mu*t3, mu*(t . qi)}.  The two cells of the face add it
// as (-mu)*t and (+mu)*t, i.e. -(mu*t) and mu*t exactly, so one evaluation
// serves both.  P is centred on the cell above the face (the s = 1 side of
// the reference's loop).
template <int DIR, class PA>
__device__ __forceinline__ void viscous_face3d(const PA& P, double odx, double ody, double odz, double mu,
                                               double g[4]) {
  const double four_thirds = 4.0 / 3.0;
  const double two_thirds = 2.0 / 3.0;
  const double c4x = half64(half64(odx)), c4y = half64(half64(ody)), c4z = half64(half64(odz));
  const int U = 1, V = 2, W = 3;
  if (DIR == 0) {
    const double qiu = half64(P(1, 1, 1, U) + P(1, 1, 0, U));
    const double qiv = half64(P(1, 1, 1, V) + P(1, 1, 0, V));
    const double qiw = half64(P(1, 1, 1, W) + P(1, 1, 0, W));
    const double dudx = odx * (P(1, 1, 1, U) - P(1, 1, 0, U));
    const double dvdx = odx * (P(1, 1, 1, V) - P(1, 1, 0, V));
    const double dwdx = odx * (P(1, 1, 1, W) - P(1, 1, 0, W));
    const double dudy = c4y * (P(1, 2, 1, U) - P(1, 0, 1, U) + P(1, 2, 0, U) - P(1, 0, 0, U));
    const double dvdy = c4y * (P(1, 2, 1, V) - P(1, 0, 1, V) + P(1, 2, 0, V) - P(1, 0, 0, V));
    const double dudz = c4z * (P(2, 1, 1, U) - P(0, 1, 1, U) + P(2, 1, 0, U) - P(0, 1, 0, U));
    const double dwdz = c4z * (P(2, 1, 1, W) - P(0, 1, 1, W) + P(2, 1, 0, W) - P(0, 1, 0, W));
    const double tau_xx = four_thirds * dudx - two_thirds * (dvdy + dwdz);
    const double tau_xy = dvdx + dudy;
    const double tau_xz = dwdx + dudz;
    g[0] = mu * tau_xx;
    g[1] = mu * tau_xy;
    g[2] = mu * tau_xz;
    g[3] = mu * (tau_xx * qiu + tau_xy * qiv + tau_xz * qiw);
  } else {
    const double qiu = half64(P(1, 1, 1, U) + P(1, 0, 1, U));
    const double qiv = half64(P(1, 1, 1, V) + P(1, 0, 1, V));
    const double qiw = half64(P(1, 1, 1, W) + P(1, 0, 1, W));
    const double dudy = ody * (P(1, 1, 1, U) - P(1, 0, 1, U));
    const double dvdy = ody * (P(1, 1, 1, V) - P(1, 0, 1, V));
    const double dwdy = ody * (P(1, 1, 1, W) - P(1, 0, 1, W));
    const double dudx = c4x * (P(1, 1, 2, U) - P(1, 1, 0, U) + P(1, 0, 2, U) - P(1, 0, 0, U));
    const double dvdx = c4x * (P(1, 1, 2, V) - P(1, 1, 0, V) + P(1, 0, 2, V) - P(1, 0, 0, V));
    const double dwdz = c4z * (P(2, 1, 1, W) - P(0, 1, 1, W) + P(2, 0, 1, W) - P(0, 0, 1, W));
    const double dvdz = c4z * (P(2, 1, 1, V) - P(0, 1, 1, V) + P(2, 0, 1, V) - P(0, 0, 1, V));
    const double tau_yy = four_thirds * dvdy - two_thirds * (dudx + dwdz);
    const double tau_xy = dvdx + dudy;
    const double tau_yz = dvdz + dwdy;
    g[0] = mu * tau_xy;
    g[1] = mu * tau_yy;
    g[2] = mu * tau_yz;
    g[3] = mu * (tau_xy * qiu + tau_yy * qiv + tau_yz * qiw);
  }
}

// The IZ branch of Viscosity.h for one cell, with the reference's index /
// field mix-ups (some terms read the cell's own row, so this flux belongs to
// the cell): accumulates into vz[1..4] like viscous3d<false>.
template <class PA>
__device__ __forceinline__ void viscous_iz3d(const PA& P, double odx, double odz, double mu, double vz[5]) {
  const double four_thirds = 4.0 / 3.0;
  const double two_thirds = 2.0 / 3.0;
  const double c4x = half64(half64(odx)), c4z = half64(half64(odz));
  const int U = 1, V = 2, W = 3;
#pragma unroll
  for (int s = 1; s < 3; ++s) {
    const double sm = (s == 1 ? -1.0 : 1.0) * mu;
    const double qiu = half64(P(s, 1, 1, U) + P(s - 1, 1, 1, U));
    const double qiv = half64(P(s, 1, 1, V) + P(s - 1, 1, 1, V));
    const double qiw = half64(P(s, 1, 1, W) + P(s - 1, 1, 1, W));
    const double dudz = odz * (P(s, 1, 1, U) - P(s - 1, 1, 1, U));
    const double dvdz = odz * (P(s, 1, 1, V) - P(s - 1, 1, 1, V));
    const double dwdz = odz * (P(s, 1, 1, W) - P(s - 1, 1, 1, W));
    const double dudx = c4x * (P(s, 1, 2, U) - P(1, s, 0, U) + P(s - 1, 1, 2, U) - P(1, s - 1, 0, U));
    const double dwdx = c4x * (P(s, 1, 2, V) - P(1, s, 0, W) + P(s - 1, 1, 2, V) - P(1, s - 1, 0, W));
    const double dvdy = c4z * (P(s, 2, 1, W) - P(s, 0, 1, V) + P(s - 1, 2, 1, W) - P(s - 1, 0, 1, V));
    const double dwdy = c4z * (P(s, 2, 1, V) - P(s, 0, 1, W) + P(s - 1, 2, 1, V) - P(s - 1, 0, 1, W));
    const double tau_zz = four_thirds * dwdz - two_thirds * (dudx + dvdy);
    const double tau_xz = dudz + dwdx;
    const double tau_yz = dvdz + dwdy;
    vz[1] += sm * tau_xz;
    vz[2] += sm * tau_yz;
    vz[3] += sm * tau_zz;
    vz[4] += sm * (tau_xz * qiu + tau_yz * qiv + tau_zz * qiw);
  }
}

// One stage for the columns (bx, by) and z layers [k0, k1); rs 0 HLL /
// 1 HLLC, kind a StageKind (constants in the one-problem kernel, per work
// item in the batch kernel); P2: every cell size is a power of two (callers
// branch on it once, uniformly).  Every thread of the CTA must call it; the
// CFL maximum is folded into red (the caller reduces it once per CTA or work
// item).
template <bool P2, bool CORR>
__device__ __forceinline__ void stage3d_segment(const Grid& G, const Fields& uin, const Fields& u0,
                                                const Fields& uout, StepCtrl* __restrict__ ctrl, int rs, int kind,
                                                int bx, int by, int k0, int k1, const Fields& hout, double* smem_raw,
                                                unsigned long long& red, const Fields* qin = nullptr,
                                                const Fields* qout = nullptr) {
  const Smem3 S{smem_raw};
  const int tid = threadIdx.x;
  const int x0 = bx * kTX, y0 = by * kTY;
  const int cx = tid % kTX, cy = tid / kTX;
  const int x = x0 + cx, y = y0 + cy;
  const bool own = x < G.na && y < G.nb;
  const long long col = (long long)y * G.pitch + x;
  const long long zstride = (long long)G.nb * G.pitch;

  if (!ctrl->active) {
    if (kind == STAGE_EULER && own) {
      for (int k = k0; k < k1; ++k) {
        const long long o = k * zstride + col;
#pragma unroll
        for (int v = 0; v < 5; ++v) uout.f[v][o] = uin.f[v][o];
      }
    }
    return;
  }
  const double dt = ctrl->dt_cur;
  const Consts64 K{G.gamma, G.gm1, G.inv_gm1};
  const int recon = G.recon;
  const bool need_pout = G.wb_flux_z || G.bc_c == DBC_C91;
  const bool vsh = !CORR && G.visc;  // shared-face viscous fluxes (FA / FB reused)

  // prologue: layers k0-2 .. k0+1, then the z face k0-1/2 of the own column
  for (int kg = k0 - 2; kg <= k0 + 1; ++kg) load_layer(G, uin, qin, x0, y0, kg, S, tid);
  __syncthreads();
  double fzL[5], poutL = 0.0;
  if (own) {
    double c[4][5];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int v = 0; v < 5; ++v) c[m][v] = S.q(slot_of(k0 - 2 + m), v, cy + 2, cx + 2);
    face3<2, CORR>(c, rs, recon, G, K, fzL, need_pout ? &poutL : nullptr);
  }
  __syncthreads();

#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    // ---- 1. layer k+2 in, x and y faces of layer k ----
    load_layer(G, uin, qin, x0, y0, k + 2, S, tid);
    const int sk = slot_of(k);
    for (int it = tid; it < kNFA_PAD + kNFB; it += kThreads) {
      double c[4][5], f[5];
      if (it < kNFA_PAD) {
        if (it >= kNFA) continue;
        const int fy = it / (kTX + 1), fx = it - fy * (kTX + 1);
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int v = 0; v < 5; ++v) c[m][v] = S.q(sk, v, fy + 2, fx + m);
        face3<0, CORR>(c, rs, recon, G, K, f, nullptr);
#pragma unroll
        for (int v = 0; v < 5; ++v) S.fa(v, fy, fx) = f[v];
      } else {
        const int j = it - kNFA_PAD;
        const int fy = j / kTX, fx = j - fy * kTX;
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int v = 0; v < 5; ++v) c[m][v] = S.q(sk, v, fy + m, fx + 2);
        face3<1, CORR>(c, rs, recon, G, K, f, nullptr);
#pragma unroll
        for (int v = 0; v < 5; ++v) S.fb(v, fy, fx) = f[v];
      }
    }
    __syncthreads();

    // ---- 2. z face k+1/2 and the update of the own cell ----
    double un[5], fzR[5], poutR = 0.0;
    const long long o = k * zstride + col;
    if (own) {
      {
        double c[4][5];
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int v = 0; v < 5; ++v) c[m][v] = S.q(slot_of(k - 1 + m), v, cy + 2, cx + 2);
        face3<2, CORR>(c, rs, recon, G, K, fzR, need_pout ? &poutR : nullptr);
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) un[v] = uin.f[v][o];
      // IX, IY: un += (F(-1/2) - F(+1/2)) * dt / d
#pragma unroll
      for (int v = 0; v < 5; ++v)
        un[v] = un[v] + div_cell<P2>((S.fa(v, cy, cx) - S.fa(v, cy, cx + 1)) * dt, G.dx, G.inv_dx);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        un[v] = un[v] + div_cell<P2>((S.fb(v, cy, cx) - S.fb(v, cy + 1, cx)) * dt, G.dy, G.inv_dy);
      // IZ with the z-boundary overrides of Update.h:131-143
      double fL[5], fR[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        fL[v] = fzL[v];
        fR[v] = fzR[v];
      }
      const double rho_c = S.q(sk, 0, cy + 2, cx + 2);
      if (G.wb_flux_z && (k == 0 || k == G.nc - 1)) {
        if (k == 0) {
          fL[0] = 0.0; fL[1] = 0.0; fL[2] = 0.0; fL[4] = 0.0;
          fL[3] = poutR - rho_c * G.g * G.dz;
        } else {
          fR[0] = 0.0; fR[1] = 0.0; fR[2] = 0.0; fR[4] = 0.0;
          fR[3] = poutL + rho_c * G.g * G.dz;
        }
      } else if (G.bc_c == DBC_C91 && (k == 0 || k == G.nc - 1)) {
        if (k == 0) {
          fL[0] = 0.0; fL[1] = 0.0; fL[2] = 0.0; fL[4] = 0.0;
          fL[3] = poutL;
        } else {
          fR[0] = 0.0; fR[1] = 0.0; fR[2] = 0.0; fR[4] = 0.0;
          fR[3] = poutR;
        }
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) un[v] = un[v] + div_cell<P2>((fL[v] - fR[v]) * dt, G.dz, G.inv_dz);
      if (G.gravity) {
        un[3] = un[3] + dt * rho_c * G.g;
        un[4] = un[4] + half64(dt) * (fL[0] + fR[0]) * G.g;
      }
      un[0] = fmax_bits(1.0e-6, un[0]);

      if (G.tc) {  // ThermalConduction.h:38-96
        double kC, kF, kB;
        if (G.kappa_z) {
          kC = G.kappa_z[3 * k];
          kF = G.kappa_z[3 * k + 1];
          kB = G.kappa_z[3 * k + 2];
        } else {
          kC = kF = kB = half64(G.kappa + G.kappa);
        }
        const int hy = cy + 2, hx = cx + 2;
        const double TC = S.temp(sk, hy, hx);
        const double FL = div_cell<P2>(kC * (TC - S.temp(sk, hy, hx - 1)), G.dx, G.inv_dx);
        const double FR = div_cell<P2>(kC * (S.temp(sk, hy, hx + 1) - TC), G.dx, G.inv_dx);
        const double FU = div_cell<P2>(kC * (TC - S.temp(sk, hy - 1, hx)), G.dy, G.inv_dy);
        const double FD = div_cell<P2>(kC * (S.temp(sk, hy + 1, hx) - TC), G.dy, G.inv_dy);
        double FF = div_cell<P2>(kF * (TC - S.temp(slot_of(k - 1), hy, hx)), G.dz, G.inv_dz);
        double FB = div_cell<P2>(kB * (S.temp(slot_of(k + 1), hy, hx) - TC), G.dz, G.inv_dz);
        if (k == 0 && G.bctc_zmin != 0) {
          if (G.bctc_zmin == 1) FF = div_cell<P2>(kF * 2.0 * (TC - G.bctc_zmin_value), G.dz, G.inv_dz);
          else FF = kF * G.bctc_zmin_value;
        }
        if (k == G.nc - 1 && G.bctc_zmax != 0) {
          if (G.bctc_zmax == 1) FB = div_cell<P2>(kB * 2.0 * (G.bctc_zmax_value - TC), G.dz, G.inv_dz);
          else FB = kB * G.bctc_zmax_value;
        }
        const double dtdx = div_cell<P2>(dt, G.dx, G.inv_dx);
        const double dtdy = div_cell<P2>(dt, G.dy, G.inv_dy);
        const double dtdz = div_cell<P2>(dt, G.dz, G.inv_dz);
        un[4] = un[4] + (dtdx * (FR - FL) + dtdy * (FD - FU) + dtdz * (FB - FF));
      }
      if (G.visc && !vsh) {  // Viscosity.h:145-151
        const RingVel P{S, k, cy + 2, cx + 2};
        double vf[3][5];
        viscous3d<CORR, double>(P, G.inv_dx, G.inv_dy, G.inv_dz, G.mu, vf);
        if (CORR) {  // the flux differences divided by the cell sizes
#pragma unroll
          for (int v = 1; v < 5; ++v)
            un[v] = un[v] + dt * (div_cell<P2>(vf[0][v], G.dx, G.inv_dx) + div_cell<P2>(vf[1][v], G.dy, G.inv_dy) +
                                  div_cell<P2>(vf[2][v], G.dz, G.inv_dz));
        } else {
#pragma unroll
          for (int v = 1; v < 5; ++v) un[v] = un[v] + dt * (vf[0][v] + vf[1][v] + vf[2][v]);
        }
      }
    }
    if (vsh) {  // viscosity with the face-only branches solved once per face
      __syncthreads();  // every cell is done with the hydro fluxes in FA / FB
      for (int it = tid; it < kNFA_PAD + kNFB; it += kThreads) {
        double g[4];
        if (it < kNFA_PAD) {
          if (it >= kNFA) continue;
          const int fy = it / (kTX + 1), fx = it - fy * (kTX + 1);
          viscous_face3d<0>(RingVel{S, k, fy + 2, fx + 2}, G.inv_dx, G.inv_dy, G.inv_dz, G.mu, g);
#pragma unroll
          for (int v = 0; v < 4; ++v) S.fa(v, fy, fx) = g[v];
        } else {
          const int j = it - kNFA_PAD;
          const int fy = j / kTX, fx = j - fy * kTX;
          viscous_face3d<1>(RingVel{S, k, fy + 2, fx + 2}, G.inv_dx, G.inv_dy, G.inv_dz, G.mu, g);
#pragma unroll
          for (int v = 0; v < 4; ++v) S.fb(v, fy, fx) = g[v];
        }
      }
      __syncthreads();
      if (own) {  // vf[d][v+1] = (0 + (-g_lower)) + g_upper, then IZ per cell (Viscosity.h:145-151)
        double vf[3][5];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int v = 0; v < 5; ++v) vf[d][v] = 0.0;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          vf[0][v + 1] = plus_zero(-S.fa(v, cy, cx)) + S.fa(v, cy, cx + 1);
          vf[1][v + 1] = plus_zero(-S.fb(v, cy, cx)) + S.fb(v, cy + 1, cx);
        }
        viscous_iz3d(RingVel{S, k, cy + 2, cx + 2}, G.inv_dx, G.inv_dz, G.mu, vf[2]);
#pragma unroll
        for (int v = 1; v < 5; ++v) un[v] = un[v] + dt * (vf[0][v] + vf[1][v] + vf[2][v]);
      }
    }
    if (own) {
      if (kind == STAGE_RK_2) {
#pragma unroll
        for (int v = 0; v < 5; ++v) un[v] = half64(u0.f[v][o] + un[v]);
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) uout.f[v][o] = un[v];
      if (kind != STAGE_RK_1) {
        double q[5];
        const double inv = inv_dt_hyp64<PLANE_XY, true, P2>(un, G, q);
        const unsigned long long b = (unsigned long long)__double_as_longlong(inv);
        red = b > red ? b : red;
        if (above_bits(inv, 1.0e300)) atomicOr(&ctrl->err, 1);
        if (hout.f[0]) {  // primitives to the caller's unpadded arrays
          const long long h = ((long long)k * G.nb + y) * G.na + x;
#pragma unroll
          for (int v = 0; v < 5; ++v)
            if (hout.f[v]) hout.f[v][h] = q[v];
        }
        if (qout) {
#pragma unroll
          for (int v = 0; v < 5; ++v) qout->f[v][o] = q[v];
        }
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) fzL[v] = fzR[v];
      poutL = poutR;
    }
    __syncthreads();
  }
}

// One stage for the columns (bx, by) and z chunk bz of tz layers, reduced
// (the batch kernel's work item).
template <bool P2, bool CORR>
__device__ __forceinline__ void stage3d_body(const Grid& G, const Fields& uin, const Fields& u0, const Fields& uout,
                                             StepCtrl* __restrict__ ctrl, int rs, int kind, int bx, int by, int bz,
                                             int tz, const Fields& hout, double* smem_raw,
                                             unsigned long long* s_red) {
  const int active = ctrl->active, parity = ctrl->parity;
  const int k0 = bz * tz;
  const int k1 = min(k0 + tz, G.nc);
  unsigned long long red = 0ull;
  stage3d_segment<P2, CORR>(G, uin, u0, uout, ctrl, rs, kind, bx, by, k0, k1, hout, smem_raw, red);
  if (active && kind != STAGE_RK_1) block_max_atomic(red, &ctrl->slot[parity ^ 1], s_red);
}

// Units [ub, ue) of the (column block, z layer) numbering, column block by
// column block; returns the CTA's CFL maximum.
template <bool P2, bool CORR, int RS, int KIND>
__device__ __forceinline__ unsigned long long march3d(const Grid& G, const Fields& uin, const Fields& u0,
                                                      const Fields& uout, StepCtrl* __restrict__ ctrl, long long ub,
                                                      long long ue, const Fields& hout, double* smem_raw,
                                                      const Fields* qin, const Fields* qout) {
  const int tiles_x = (G.na + kTX - 1) / kTX;
  unsigned long long red = 0ull;
  for (long long u = ub; u < ue;) {
    const int cb = (int)(u / G.nc);
    const int k0 = (int)(u - (long long)cb * G.nc);
    const int k1 = (int)(k0 + (ue - u) < (long long)G.nc ? k0 + (ue - u) : (long long)G.nc);
    u += k1 - k0;
    stage3d_segment<P2, CORR>(G, uin, u0, uout, ctrl, RS, KIND, cb % tiles_x, cb / tiles_x, k0, k1, hout, smem_raw,
                              red, qin, qout);
  }
  return red;
}

// The one-problem kernel: the (column block, z layer) units, numbered column
// block by column block, are split evenly over the CTAs that fit on the GPU
// at once; a CTA marches each column block of its range over its layers.
template <int RS, int KIND, bool CORR>
__global__ void __launch_bounds__(kThreads, FV_3D64_MIN_CTAS)
stage3d_fp64(const Grid G, const Fields uin, const Fields u0, const Fields uout, StepCtrl* __restrict__ ctrl,
             long long units, const Fields hout, const Fields qin, const Fields qout) {
  extern __shared__ double smem_raw[];
  __shared__ unsigned long long s_red[kThreads / 32];
  pdl_wait();
  const long long ub = units * blockIdx.x / gridDim.x, ue = units * (blockIdx.x + 1) / gridDim.x;
  const int active = ctrl->active, parity = ctrl->parity;
  // the primitive copy of uin, when the last stage that wrote uin left one
  const Fields* qi = qin.f[0] && ctrl->q_valid ? &qin : nullptr;
  const Fields* qo = qout.f[0] ? &qout : nullptr;
  const unsigned long long red =
      G.pow2_all ? march3d<true, CORR, RS, KIND>(G, uin, u0, uout, ctrl, ub, ue, hout, smem_raw, qi, qo)
                 : march3d<false, CORR, RS, KIND>(G, uin, u0, uout, ctrl, ub, ue, hout, smem_raw, qi, qo);
  if (active && KIND != STAGE_RK_1) block_max_atomic(red, &ctrl->slot[parity ^ 1], s_red);
  // the copy is complete once this launch is (the next reader is a later kernel)
  if (active && qo && threadIdx.x == 0) ctrl->q_valid = 1;
  pdl_trigger();
}

int sm_count3d() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 1;
  }
  return n;
}

template <int RS, int KIND, bool CORR>
cudaError_t launch_one(const Grid& G, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl, const Fields* hout,
                       const PrimCopy& pc, cudaStream_t st) {
  auto kern = stage3d_fp64<RS, KIND, CORR>;
  static bool attr_set = false;  // per instantiation, once per process
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Smem3::bytes(true));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  static int resident[2] = {0, 0};  // CTAs per SM without / with conduction
  const int tc = G.tc != 0;
  if (!resident[tc]) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident[tc], kern, kThreads, Smem3::bytes(tc));
    if (e != cudaSuccess) return e;
    if (resident[tc] < 1) resident[tc] = 1;
  }
  const long long cols = (long long)((G.na + kTX - 1) / kTX) * ((G.nb + kTY - 1) / kTY);
  const long long units = cols * G.nc;
  long long ctas = units / kMinLayersPerCta;
  const long long slots = (long long)resident[tc] * sm_count3d();
  if (ctas > slots) ctas = slots;
  if (ctas < 1) ctas = 1;
  const Fields none{};
  const cudaError_t e = launch_pdl(kern, dim3((unsigned)ctas), dim3(kThreads), Smem3::bytes(tc), st, G, uin, u0, uout,
                                   ctrl, units, hout ? *hout : none, pc.qin ? *pc.qin : none,
                                   pc.qout ? *pc.qout : none);
  return e != cudaSuccess ? e : cudaGetLastError();
}

template <int RS, bool CORR>
cudaError_t launch_kind(const Grid& G, int kind, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                        const Fields* hout, const PrimCopy& pc, cudaStream_t st) {
  switch (kind) {
    case STAGE_EULER: return launch_one<RS, STAGE_EULER, CORR>(G, uin, u0, uout, ctrl, hout, pc, st);
    case STAGE_RK_1: return launch_one<RS, STAGE_RK_1, CORR>(G, uin, u0, uout, ctrl, nullptr, pc, st);
    default: return launch_one<RS, STAGE_RK_2, CORR>(G, uin, u0, uout, ctrl, hout, pc, st);
  }
}

template <int RS>
cudaError_t launch_phys(const Grid& G, int kind, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                        const Fields* hout, const PrimCopy& pc, cudaStream_t st) {
  return G.corrected ? launch_kind<RS, true>(G, kind, uin, u0, uout, ctrl, hout, pc, st)
                     : launch_kind<RS, false>(G, kind, uin, u0, uout, ctrl, hout, pc, st);
}

static_assert(sizeof(BatchInst) % 8 == 0, "descriptor copied as 8-byte words");

// Persistent FP64 kernel over a group of 3-D problems (see
// launch_batch_stage3d64): CTAs take work items from the queue counter, find
// their problem by binary search over the first item numbers, and run the
// same body as the one-problem kernel (CORR: the corrected physics).
template <int KIND, int RS, bool CORR>
__global__ void __launch_bounds__(kThreads, FV_3D64_MIN_CTAS)
batch_stage3d64(const BatchInst* __restrict__ insts, int ninst, int ntiles, unsigned* queue, int flip) {
  const int kind = KIND;
  extern __shared__ double smem_raw[];
  __shared__ unsigned long long s_red[kThreads / 32];
  __shared__ BatchInst s_inst;
  __shared__ int s_tile;
  const Fields none{};
  pdl_wait();
  for (;;) {
    __syncthreads();  // the previous item is finished with s_tile, s_inst and smem
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) {
      pdl_trigger();  // no work left for this CTA
      break;
    }
    {
      int lo = 0, hi = ninst - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (insts[mid].tile0 <= t) lo = mid;
        else hi = mid - 1;
      }
      const unsigned long long* src = reinterpret_cast<const unsigned long long*>(insts + lo);
      unsigned long long* dst = reinterpret_cast<unsigned long long*>(&s_inst);
      for (int w = threadIdx.x; w < (int)(sizeof(BatchInst) / 8); w += blockDim.x) dst[w] = src[w];
    }
    __syncthreads();
    const BatchInst& I = s_inst;
    const int lt = t - I.tile0;
    const int per_layer = I.tiles_x * I.tiles_y;
    const int bz = lt / per_layer, rem = lt - bz * per_layer;
    const int by = rem / I.tiles_x, bx = rem - by * I.tiles_x;
    Fields uin, u0, uout;
    if (kind == STAGE_RK_1) {
      uin = I.A; u0 = I.A; uout = I.B;
    } else if (kind == STAGE_RK_2) {
      uin = I.B; u0 = I.A; uout = I.A;
    } else {
      uin = flip ? I.B : I.A; u0 = uin; uout = flip ? I.A : I.B;
    }
    // the group shares the solver (RS); the cell-size form is a uniform branch
    if (I.G.pow2_all)
      stage3d_body<true, CORR>(I.G, uin, u0, uout, I.ctrl, RS, kind, bx, by, bz, I.tz, none, smem_raw, s_red);
    else
      stage3d_body<false, CORR>(I.G, uin, u0, uout, I.ctrl, RS, kind, bx, by, bz, I.tz, none, smem_raw, s_red);
  }
}

typedef void (*Batch3dKernel)(const BatchInst*, int, int, unsigned*, int);

template <int RS, bool CORR>
Batch3dKernel batch3d_kernel_rs(int kind) {
  return kind == STAGE_EULER ? batch_stage3d64<STAGE_EULER, RS, CORR>
                             : (kind == STAGE_RK_1 ? batch_stage3d64<STAGE_RK_1, RS, CORR>
                                                   : batch_stage3d64<STAGE_RK_2, RS, CORR>);
}

// rs: the Riemann solver (bit 0) and the corrected physics (bit 1).
Batch3dKernel batch3d_kernel(int kind, int rs) {
  switch (rs & 3) {
    case 0: return batch3d_kernel_rs<0, false>(kind);
    case 1: return batch3d_kernel_rs<1, false>(kind);
    case 2: return batch3d_kernel_rs<0, true>(kind);
    default: return batch3d_kernel_rs<1, true>(kind);
  }
}

bool batch3d_prepare() {
  static bool done = false;
  if (done) return true;
  for (int rs = 0; rs < 4; ++rs)
    for (int k = 0; k < 3; ++k)
      if (cudaFuncSetAttribute(batch3d_kernel(k, rs), cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)Smem3::bytes(true)) != cudaSuccess)
        return false;
  done = true;
  return true;
}

}  // namespace

int batch3d_columns() { return kTX; }

int batch_stage3d_occupancy64(int rs, bool tc) {
  if (!batch3d_prepare()) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch3d_kernel(STAGE_RK_2, rs), kThreads, Smem3::bytes(tc)) !=
      cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_batch_stage3d64(const BatchInst* insts, int ninst, int ntiles, unsigned* queue, int kind, int flip,
                                   int rs, int grid, bool tc, cudaStream_t st) {
  if (!batch3d_prepare()) return cudaErrorInvalidConfiguration;
  const cudaError_t e =
      launch_pdl(batch3d_kernel(kind, rs), dim3(grid), dim3(kThreads), Smem3::bytes(tc), st, insts, ninst, ntiles, queue, flip);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_stage3d(const Grid& G, int riemann_solver, int kind, Fields uin, Fields u0, Fields uout,
                           StepCtrl* ctrl, cudaStream_t st, const Fields* hout, const PrimCopy* prims) {
  static const PrimCopy no_prims{};
  const PrimCopy& pc = prims ? *prims : no_prims;
  return riemann_solver == 0 ? launch_phys<0>(G, kind, uin, u0, uout, ctrl, hout, pc, st)
                             : launch_phys<1>(G, kind, uin, u0, uout, ctrl, hout, pc, st);
}

}  // namespace fv
