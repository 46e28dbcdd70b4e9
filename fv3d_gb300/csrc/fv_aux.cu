// fv_aux.cu -- the small kernels around the stage kernel: the standalone CFL
// reduction, the per-step control kernel, primitive <-> conserved
// conversions and the conservation sums.  Built without FMA contraction, like
// the stage kernel, so every value rounds as in the reference.
#include "fv_control.cuh"
#include "fv_kernels.h"
#include "fv_plane2d.cuh"

namespace fv {

namespace {

int grid_for(long long n, int block) {
  long long b = (n + block - 1) / block;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

// ComputeDt.h:28-54 over the interior: max inv_dt_hyp into ctrl->slot[slot].
template <int PLANE, bool WACT>
__global__ void __launch_bounds__(256) reduce2d_fp64(const Grid G, const Fields u, StepCtrl* ctrl, int slot) {
  __shared__ unsigned long long s_red[8];
  unsigned long long red = 0ull;
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    double w[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) w[v] = (WACT || v != 3) ? u.f[v][o] : 0.0;
    const double inv = inv_dt_hyp64<PLANE, WACT>(w, G);
    const unsigned long long b = (unsigned long long)__double_as_longlong(inv);
    red = b > red ? b : red;
    if (!(inv <= 1.0e300)) atomicOr(&ctrl->err, 1);
  }
  block_max_atomic(red, &ctrl->slot[slot], s_red);
}

__global__ void control_kernel(StepCtrl* ctrl, int n, int mode_override, double dt_given) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) step_control(ctrl[i], mode_override, dt_given);
  pdl_trigger();
}

__global__ void batch_control_kernel(StepCtrl* ctrl, int n, unsigned* queue, int nq, int mode_override,
                                     double dt_given) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) step_control(ctrl[i], mode_override, dt_given);
  if (i < nq) queue[i] = 0u;
  pdl_trigger();
}

// primToCons in place (States.h:20-31).  Storage order in and out.
template <int PLANE>
__global__ void prim_to_cons2d(const Grid G, const Fields u) {
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    const double r = u.f[0][o];
    const double ma = __dmul_rn(r, u.f[1][o]), mb = __dmul_rn(r, u.f[2][o]), mc = __dmul_rn(r, u.f[3][o]);
    const double mx = ma, my = PLANE == PLANE_XY ? mb : mc, mz = PLANE == PLANE_XY ? mc : mb;
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(mx, mx), __dmul_rn(my, my)), __dmul_rn(mz, mz));
    const double Ek = __ddiv_rn(__dmul_rn(0.5, s), r);
    const double E = __dadd_rn(Ek, __ddiv_rn(u.f[4][o], G.gm1));
    u.f[1][o] = ma;
    u.f[2][o] = mb;
    u.f[3][o] = mc;
    u.f[4][o] = E;
  }
}

// primToCons from unpadded primitive arrays the GPU can address (a caller's
// host arrays), optionally with the CFL maximum of the result.  Same
// arithmetic as prim_to_cons2d.
// qout (optional): the primitive copy of dst (consToPrim of the result, the
// bits the stage kernels' own conversion gives), with *q_valid set after it.
template <int PLANE, bool WACT, bool REDUCE>
__global__ void __launch_bounds__(256) prim_to_cons_from(const Grid G, const Fields src, const Fields dst,
                                                         StepCtrl* ctrl, int slot, const Fields qout, int* q_valid) {
  __shared__ unsigned long long s_red[8];
  unsigned long long red = 0ull;
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    const double r = src.f[0][c];
    const double va = src.f[1] ? src.f[1][c] : 0.0, vb = src.f[2] ? src.f[2][c] : 0.0;
    const double vc = (WACT && src.f[3]) ? src.f[3][c] : 0.0;
    const double ma = __dmul_rn(r, va), mb = __dmul_rn(r, vb), mc = __dmul_rn(r, vc);
    const double mx = ma, my = PLANE == PLANE_XY ? mb : mc, mz = PLANE == PLANE_XY ? mc : mb;
    const double sq = __dadd_rn(__dadd_rn(__dmul_rn(mx, mx), __dmul_rn(my, my)), __dmul_rn(mz, mz));
    const double Ek = __ddiv_rn(__dmul_rn(0.5, sq), r);
    const double E = __dadd_rn(Ek, __ddiv_rn(src.f[4][c], G.gm1));
    dst.f[0][o] = r;
    dst.f[1][o] = ma;
    dst.f[2][o] = mb;
    if (WACT) dst.f[3][o] = mc;
    dst.f[4][o] = E;
    if (REDUCE || qout.f[0]) {
      const double u[5] = {r, ma, mb, mc, E};
      double q[5];
      if (REDUCE) {
        const double inv = inv_dt_hyp64<PLANE, WACT>(u, G, q);
        const unsigned long long b = (unsigned long long)__double_as_longlong(inv);
        red = b > red ? b : red;
        if (!(inv <= 1.0e300)) atomicOr(&ctrl->err, 1);
      } else {
        double y;
        cons_to_prim64<PLANE, WACT>(u, G.gm1, q, y);
      }
      if (qout.f[0]) {
#pragma unroll
        for (int v = 0; v < 5; ++v)
          if (WACT || v != 3) qout.f[v][o] = q[v];
      }
    }
  }
  if (REDUCE) block_max_atomic(red, &ctrl->slot[slot], s_red);
  // the copy is complete once this launch is (the next reader is a later kernel)
  if (q_valid && threadIdx.x == 0) *q_valid = 1;
}

// consToPrim (States.h:34-45); src and dst may alias.
template <int PLANE>
__global__ void cons_to_prim2d(const Grid G, const Fields src, const Fields dst) {
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    const double r = src.f[0][o];
    const double va = __ddiv_rn(src.f[1][o], r), vb = __ddiv_rn(src.f[2][o], r), vc = __ddiv_rn(src.f[3][o], r);
    const double vx = va, vy = PLANE == PLANE_XY ? vb : vc, vz = PLANE == PLANE_XY ? vc : vb;
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
    const double Ek = __dmul_rn(__dmul_rn(0.5, r), s);
    const double p = __dmul_rn(__dsub_rn(src.f[4][o], Ek), G.gm1);
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

__global__ void __launch_bounds__(256) totals2d(const Grid G, const Fields u, double* partial) {
  __shared__ double s_sum[5][256], s_cmp[5][256];
  double s[5] = {0, 0, 0, 0, 0}, cc[5] = {0, 0, 0, 0, 0};
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
#pragma unroll
    for (int v = 0; v < 5; ++v) kadd(s[v], cc[v], u.f[v][o]);
  }
  const int t = threadIdx.x;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    s_sum[v][t] = s[v];
    s_cmp[v][t] = cc[v];
  }
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

}  // namespace

cudaError_t launch_reduce2d(const Grid& G, bool wact, Fields u, StepCtrl* ctrl, int slot, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.rows, 256);
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
  const cudaError_t e = launch_pdl(control_kernel, dim3((n + 127) / 128), dim3(128), 0, st, ctrl, n, mode_override,
                                   dt_given);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_batch_control(StepCtrl* ctrl, int n, unsigned* queue, int nq, int mode_override, double dt_given,
                                 cudaStream_t st) {
  const int m = n > nq ? n : nq;
  const cudaError_t e = launch_pdl(batch_control_kernel, dim3((m + 127) / 128), dim3(128), 0, st, ctrl, n, queue, nq,
                                   mode_override, dt_given);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_prim_to_cons2d(const Grid& G, Fields u, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.rows, 256);
  if (G.plane == PLANE_XY) prim_to_cons2d<PLANE_XY><<<grid, 256, 0, st>>>(G, u);
  else prim_to_cons2d<PLANE_XZ><<<grid, 256, 0, st>>>(G, u);
  return cudaGetLastError();
}

template <int PLANE, bool WACT>
cudaError_t launch_p2c_from(const Grid& G, Fields src, Fields dst, StepCtrl* ctrl, int slot, const Fields& qout,
                            int* q_valid, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.rows, 256);
  if (ctrl)
    prim_to_cons_from<PLANE, WACT, true><<<grid, 256, 0, st>>>(G, src, dst, ctrl, slot, qout, q_valid);
  else
    prim_to_cons_from<PLANE, WACT, false><<<grid, 256, 0, st>>>(G, src, dst, ctrl, slot, qout, q_valid);
  return cudaGetLastError();
}

cudaError_t launch_prim_to_cons_from(const Grid& G, bool wact, Fields src, Fields dst, StepCtrl* ctrl, int slot,
                                     cudaStream_t st, const Fields* qout, int* q_valid) {
  const Fields q = qout ? *qout : Fields{};
  int* qv = qout ? q_valid : nullptr;
  if (G.plane == PLANE_XY)
    return wact ? launch_p2c_from<PLANE_XY, true>(G, src, dst, ctrl, slot, q, qv, st)
                : launch_p2c_from<PLANE_XY, false>(G, src, dst, ctrl, slot, q, qv, st);
  return wact ? launch_p2c_from<PLANE_XZ, true>(G, src, dst, ctrl, slot, q, qv, st)
              : launch_p2c_from<PLANE_XZ, false>(G, src, dst, ctrl, slot, q, qv, st);
}

cudaError_t launch_cons_to_prim2d(const Grid& G, Fields src, Fields dst, cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.rows, 256);
  if (G.plane == PLANE_XY) cons_to_prim2d<PLANE_XY><<<grid, 256, 0, st>>>(G, src, dst);
  else cons_to_prim2d<PLANE_XZ><<<grid, 256, 0, st>>>(G, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_totals2d(const Grid& G, Fields u, double* partial, int max_blocks, int* nblocks,
                            cudaStream_t st) {
  int grid = grid_for((long long)G.na * G.rows, 256);
  if (grid > max_blocks) grid = max_blocks;
  *nblocks = grid;
  totals2d<<<grid, 256, 0, st>>>(G, u, partial);
  return cudaGetLastError();
}

}  // namespace fv
