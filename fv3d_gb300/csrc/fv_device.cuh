// fv_device.cuh -- device-side building blocks of the GB300 hydro step.
//
// Everything here is templated on the arithmetic type T (double for the plain
// FP64 path, float for the mixed path) and follows the reference's
// floating-point operation order unless a comment says otherwise.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fv {

// Boundary kinds as seen by the kernels (BC_C91 on x/y behaves as periodic in
// the reference's default branch, BoundaryConditions.h:165,186; the host maps
// it before launch).  DBC_C91 only occurs along z of the 3-D kernel.
enum DevBC : int { DBC_ABSORBING = 0, DBC_REFLECTING = 1, DBC_PERIODIC = 2, DBC_C91 = 3 };
enum Recon : int { R_PCM = 0, R_PCM_WB = 1, R_PLM = 2 };
enum StageKind : int { STAGE_EULER = 0, STAGE_RK_1 = 1, STAGE_RK_2 = 2 };
// The two active axes of a 2-D run: a = x always; b = y (XY plane, Nz == 1)
// or z (XZ plane, Ny == 1).  The third axis c is degenerate (one cell).
enum Plane : int { PLANE_XY = 0, PLANE_XZ = 1 };

// Device-resident control block of one problem (one per instance in batches).
struct StepCtrl {
  double t;            // time at the start of the step in flight
  double dt_cur;       // dt of the step in flight (0 when inactive)
  double tend;         // loop bound of fvgpu_advance
  double dt_given;     // host-supplied dt (mode 0)
  double cfl, inv_tc, inv_visc, epsilon;
  long long step;      // steps taken
  long long max_steps; // <= 0: unlimited
  unsigned long long slot[2];  // max inv_dt_hyp (bits of a non-negative double)
  int active;          // 1 if the step in flight advances the state
  int parity;          // slot read by this step's control = step & 1
  int mode;            // 0: dt = dt_given; 1: CFL dt, loop bound t + eps < tend
  int err;             // sticky: bit0 non-finite/negative state seen
};

// Geometry and physics of one problem as the kernels need it.  A 2-D run
// (ndim 2) has axes a, b and a one-cell axis c; a 3-D run (ndim 3) has
// a = x, b = y, c = z, stored like the x-y plane (rho, m_x, m_y, m_z, E).
// Field arrays hold `rows` = nb * nc rows of `pitch` elements, row index
// k * nb + j.
struct Grid {
  int na, nb;          // interior cells along a and b
  int nc;              // interior cells along c (1 in 2-D)
  int rows;            // nb * nc
  int ndim;            // 2 or 3
  int pitch;           // row pitch in elements
  int plane;           // Plane (PLANE_XY for 3-D)
  long long fstride;   // elements per field array (>= pitch * rows)
  int bc_a, bc_b;      // DevBC along a / b
  int bc_c;            // DevBC along c (3-D kernel)
  int recon;           // Recon
  int gravity, tc, visc;
  double da, db, dc;   // cell size along a, b and the degenerate axis
  double dx, dy, dz;   // the same in reference (x,y,z) naming
  double gamma, g, kappa, mu;
  // Exact-arithmetic helpers (host-computed with IEEE double):
  double inv_dx, inv_dy, inv_dz;   // RN(1/d)
  int pow2_x, pow2_y, pow2_z;      // d is a power of two (1/d exact)
  int pow2_all;                    // all three are
  double gm1, inv_gm1;             // gamma - 1, RN(1/(gamma - 1))
  // FP32 copies for the mixed form (a double->float conversion runs on the
  // slow FP64 pipe, so kernels never convert per cell).
  float gamma_f, gm1_f, inv_gm1_f, g_f, kappa_f, mu_f, g_dz_f;
  float dx_f, dy_f, dz_f, inv_dx_f, inv_dy_f, inv_dz_f;
  // z-boundary physics of the 3-D kernel (Update.h:131-143,
  // BoundaryConditions.h:87-134, ThermalConduction.h:78-92):
  int corrected;                   // fv_physics corrected (3-D kernel only)
  int wb_flux_z;                   // well_balanced_flux_at_z_bc
  int gravity_flag;                // params.gravity as the C91 ghost uses it (0/1)
  int bctc_zmin, bctc_zmax;        // fv_bctc_mode
  double bctc_zmin_value, bctc_zmax_value;
  double zmin, theta1;             // C91 ghost temperature profile
  // Face conductivities per interior z layer when kappa varies with z
  // (B02): kappa_z[3k + {0,1,2}] = in-plane faces, face k-1/2, face k+1/2.
  // Null for constant kappa.
  const double* kappa_z;
};

// Maps a cell index g (may be a ghost, -2 <= g < n+2) along an axis with n
// interior cells to the interior cell whose primitive state the reference's
// ghost fill copies there (BoundaryConditions.h:13-81).  `flip` is set when
// the normal velocity is negated (reflecting).  Indices beyond two ghost
// layers (only reached by the unused corners of partial tiles) are clamped.
__device__ __forceinline__ int bc_source(int g, int n, int bc, bool& flip) {
  flip = false;
  if (g >= 0 && g < n) return g;
  int s;
  if (bc == DBC_PERIODIC) {
    s = g < 0 ? g + n : g - n;
  } else if (bc == DBC_REFLECTING) {
    flip = true;
    s = g < 0 ? -g - 1 : 2 * n - g - 1;
  } else {
    s = g < 0 ? 0 : n - 1;
  }
  return s < 0 ? 0 : (s >= n ? n - 1 : s);
}

// Primitive state in the slot order of one sweep direction (swap_component,
// States.h:104-111): r, normal velocity, first / second transverse velocity, p.
template <class T>
struct Slots {
  T r, un, t1, t2, p;
};

// sqrt(p*gamma/rho), States.h:48-50
template <class T>
__device__ __forceinline__ T sound_speed(T r, T p, T gamma) {
  return sqrt(p * gamma / r);
}

// computeFlux, States.h:114-127 (slot order in, slot order out).
template <class T>
__device__ __forceinline__ void euler_flux(const Slots<T>& q, T gamma, T f[5]) {
  const T Ek = T(0.5) * q.r * (q.un * q.un + q.t1 * q.t1 + q.t2 * q.t2);
  const T E = (q.p / (gamma - T(1)) + Ek);
  f[0] = q.r * q.un;
  f[1] = q.r * q.un * q.un + q.p;
  f[2] = q.r * q.un * q.t1;
  f[3] = q.r * q.un * q.t2;
  f[4] = (q.p + E) * q.un;
}

// primToCons, States.h:20-31 (slot order).
template <class T>
__device__ __forceinline__ void prim_to_cons_slots(const Slots<T>& q, T gamma, T u[5]) {
  u[0] = q.r;
  u[1] = q.r * q.un;
  u[2] = q.r * q.t1;
  u[3] = q.r * q.t2;
  const T Ek = T(0.5) * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / q.r;
  u[4] = (Ek + q.p / (gamma - T(1)));
}

// HLL with Davis wave-speed estimates, RiemannSolvers.h:6-36.
template <class T>
__device__ __forceinline__ void riemann_hll(const Slots<T>& L, const Slots<T>& R, T gamma, T flux[5]) {
  const T aL = sound_speed(L.r, L.p, gamma);
  const T aR = sound_speed(R.r, R.p, gamma);
  const T SL = fmin(L.un - aL, R.un - aR);
  const T SR = fmax(L.un + aL, R.un + aR);
  T FL[5], FR[5];
  euler_flux(L, gamma, FL);
  euler_flux(R, gamma, FR);
  if (SL >= T(0)) {
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = FL[v];
  } else if (SR <= T(0)) {
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = FR[v];
  } else {
    T uL[5], uR[5];
    prim_to_cons_slots(L, gamma, uL);
    prim_to_cons_slots(R, gamma, uR);
    const T slsr = SL * SR;
    const T den = SR - SL;
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = ((FL[v] * SR - FR[v] * SL) + (uR[v] - uL[v]) * slsr) / den;
  }
}

// HLLC, RiemannSolvers.h:39-112.  The kinetic energy uses only the normal
// and first transverse slots, as the reference does (RiemannSolvers.h:52,54).
template <class T>
__device__ __forceinline__ void riemann_hllc(const Slots<T>& L, const Slots<T>& R, T gamma, T flux[5]) {
  const T rL = L.r, uL = L.un, vL = L.t1, pL = L.p;
  const T rR = R.r, uR = R.un, vR = R.t1, pR = R.p;
  const T entho = T(1) / (gamma - T(1));
  const T EL = T(0.5) * rL * (uL * uL + vL * vL) + pL * entho;
  const T ER = T(0.5) * rR * (uR * uR + vR * vR) + pR * entho;
  const T cL = sound_speed(rL, pL, gamma);
  const T cR = sound_speed(rR, pR, gamma);
  const T cmax = fmax(cL, cR);
  const T SL = fmin(uL, uR) - cmax;
  const T SR = fmax(uL, uR) + cmax;
  const T rcL = rL * (uL - SL);
  const T rcR = rR * (SR - uR);
  const T uS = (rcR * uR + rcL * uL + (pL - pR)) / (rcR + rcL);
  const T pS = (rcR * pL + rcL * pR + rcL * rcR * (uL - uR)) / (rcR + rcL);
  T sr, su, st1, st2, sp, E;
  if (SL > T(0)) {
    sr = rL; su = uL; st1 = L.t1; st2 = L.t2; sp = pL; E = EL;
  } else if (uS > T(0)) {
    sr = rL * (SL - uL) / (SL - uS);
    E = ((SL - uL) * EL - pL * uL + pS * uS) / (SL - uS);
    su = uS; st1 = L.t1; st2 = L.t2; sp = pS;
  } else if (SR > T(0)) {
    sr = rR * (SR - uR) / (SR - uS);
    E = ((SR - uR) * ER - pR * uR + pS * uS) / (SR - uS);
    su = uS; st1 = R.t1; st2 = R.t2; sp = pS;
  } else {
    sr = rR; su = uR; st1 = R.t1; st2 = R.t2; sp = pR; E = ER;
  }
  flux[0] = sr * su;
  flux[1] = sr * su * su + sp;
  flux[2] = flux[0] * st1;
  flux[3] = flux[0] * st2;
  flux[4] = (E + sp) * su;
}

template <class T, int RS>
__device__ __forceinline__ void riemann(const Slots<T>& L, const Slots<T>& R, T gamma, T flux[5]) {
  if (RS == 0)
    riemann_hll(L, R, gamma, flux);
  else
    riemann_hllc(L, R, gamma, flux);
}

// minmod of Update.h:73-80: 0 if dL*dR < 0, else the argument of smaller
// magnitude, ties going to the second.
template <class T>
__device__ __forceinline__ T minmod(T dL, T dR) {
  if (dL * dR < T(0)) return T(0);
  return fabs(dL) < fabs(dR) ? dL : dR;
}

// Atomic max of a non-negative double stored as its bit pattern (IEEE order
// of non-negative doubles equals unsigned integer order; NaN sorts above +inf).
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* slot, double v) {
  atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

}  // namespace fv
