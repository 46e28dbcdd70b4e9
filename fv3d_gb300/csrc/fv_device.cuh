// fv_device.cuh -- device-side types shared by every kernel of the GB300
// hydro step: the control block, the grid description, the ghost-cell index
// map, the slot order of a sweep and the CFL atomic.
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
  int err;             // sticky: bit0 non-finite/negative state seen, bit1 a bounded wait (TMA staging) gave up
  int q_valid;         // the primitive copy of the state (2-D RK2 handles) matches it
};

// Programmatic dependent launch (PTX griddepcontrol) for the kernels of the
// step loop: each waits for the previous kernel of the stream to complete
// (its memory visible) before touching memory, and lets the next kernel be
// launched once all its CTAs are done with their work, so that launch
// overlaps this kernel's exit.  The trigger comes at the end, not the start:
// an early trigger let the next grid's CTAs settle on the SMs that happened
// to be free, two to an SM, and halved the speed of grids smaller than the
// GPU.  Outside such a launch both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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
  float zmin_f, theta1_f, bctc_zmin_value_f, bctc_zmax_value_f;  // FP32 copies
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

// Atomic max of a non-negative double stored as its bit pattern (IEEE order
// of non-negative doubles equals unsigned integer order; NaN sorts above +inf).
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* slot, double v) {
  atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

}  // namespace fv
