// fv_plane2d.cuh -- per-cell FP64 helpers shared by the 2-D kernels.
//
// A 2-D run stores its state in "storage order" (rho, m_a, m_b, m_c, E):
// m_a is the x-momentum, m_b the momentum along the second active axis (y in
// the x-y plane, z in the x-z plane) and m_c the momentum along the
// degenerate axis.  These helpers restate the reference's per-cell formulas in
// that order, rounding exactly as the reference does.
#pragma once

#include "fv_device.cuh"
#include "fv_exact64.cuh"

namespace fv {

// Storage slot (1 = a, 2 = b, 3 = c) of the reference's physical velocity
// component var (1 = x, 2 = y, 3 = z).
template <int PLANE>
__device__ __forceinline__ constexpr int phys_slot(int var) {
  return var == 1 ? 1 : (PLANE == PLANE_XY ? (var == 2 ? 2 : 3) : (var == 2 ? 3 : 2));
}

// consToPrim (States.h:34-45) of a state held in storage order; returns
// (rho, u_a, u_b, u_c, p) and, through y, RN(1/rho).  The kinetic energy sums
// the physical x, y, z velocities in the reference's order; with WACT false
// the degenerate velocity is exactly zero and its (exact) zero terms are
// dropped.  The three divisions by rho share one correctly rounded
// reciprocal (Markstein correction, fv_exact64.cuh).
template <int PLANE, bool WACT>
__device__ __forceinline__ void cons_to_prim64(const double u[5], double gm1, double q[5], double& y) {
  const double r = u[0];
  y = 1.0 / r;
  const double va = div_by_rcp(u[1], r, y);
  const double vb = div_by_rcp(u[2], r, y);
  const double vc = WACT ? div_by_rcp(u[3], r, y) : 0.0;
  double ke;
  if (WACT) {
    const double vx = va, vy = PLANE == PLANE_XY ? vb : vc, vz = PLANE == PLANE_XY ? vc : vb;
    ke = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
  } else {
    ke = __dadd_rn(__dmul_rn(va, va), __dmul_rn(vb, vb));
  }
  const double Ek = __dmul_rn(half64(r), ke);
  q[0] = r;
  q[1] = va;
  q[2] = vb;
  q[3] = vc;
  q[4] = __dmul_rn(__dsub_rn(u[4], Ek), gm1);
}

// Hyperbolic inverse time step of one cell, ComputeDt.h:49-52:
// (cs + |u|)/dx + (cs + |v|)/dy + (cs + |w|)/dz with cs = sqrt(p*gamma/rho).
// qout, when given, receives the primitives consToPrim computes on the way.
template <int PLANE, bool WACT, bool P2 = false>
__device__ __forceinline__ double inv_dt_hyp64(const double u[5], const Grid& G, double* qout = nullptr) {
  double q[5], y;
  cons_to_prim64<PLANE, WACT>(u, G.gm1, q, y);
  if (qout) {
#pragma unroll
    for (int v = 0; v < 5; ++v) qout[v] = q[v];
  }
  const double cs = sqrt(div_by_rcp(__dmul_rn(q[4], G.gamma), q[0], y));
  const double vx = q[1], vy = PLANE == PLANE_XY ? q[2] : q[3], vz = PLANE == PLANE_XY ? q[3] : q[2];
  const double tx = div_cell<P2>(__dadd_rn(cs, fabs(vx)), G.dx, G.inv_dx);
  const double ty = div_cell<P2>(__dadd_rn(cs, fabs(vy)), G.dy, G.inv_dy);
  const double tz = div_cell<P2>(__dadd_rn(cs, fabs(vz)), G.dz, G.inv_dz);
  return __dadd_rn(__dadd_rn(tx, ty), tz);
}

// Block-wide max of non-negative doubles held as bit patterns (IEEE order of
// non-negative doubles equals unsigned order; NaN sorts above +inf) and one
// atomic max per CTA.  Every thread of the block must call it.
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

}  // namespace fv
