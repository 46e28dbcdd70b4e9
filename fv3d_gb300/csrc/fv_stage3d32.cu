// fv_stage3d32.cu -- the FP32-mixed stage of 3-D problems in batches.
//
// The same z-marching organisation as the FP64 3-D kernel (fv_stage3d.cu): a
// CTA owns a 16 x 16 block of columns and a chunk of z layers; a ring of four
// layers of primitives sits in shared memory (FP32 here: 51.6 KB with
// conduction, 4 CTAs per SM); the x and y faces of layer k are solved while
// layer k+2 is loaded; each thread solves the z face above its column and
// updates its cell.  The arithmetic is that of the 2-D mixed form
// (fv_tile32.cuh): U^n carried as an FP32 (hi, lo) pair, U* as FP32,
// primitives / slopes / Riemann solvers / conduction / viscosity in FP32,
// increments accumulated on the pairs with error-free sums, the CFL maximum
// turned into dt in FP64 by the control kernel.  Every reference feature of
// the 3-D FP64 kernel is kept: C91 ghosts, the well-balanced / C91 z-flux
// overrides, gravity, fixed-temperature / fixed-gradient conduction
// boundaries, viscosity with the reference's z-branch quirks, and the
// corrected physics as a template option (B02 conductivity runs on the FP64
// handle only).  Built with fast-math.
#include "fv_tile32.cuh"

namespace fv {

namespace {

// 1: RK2 stage 2 asks L1 for each cell's U^n before its z face and
// increments are formed (no registers held; the load comes where U^n is
// added): +2 % on random 160^3 and 192^3.
#ifndef FV_3D32_UN_PREFETCH
#define FV_3D32_UN_PREFETCH 1
#endif

constexpr int kTX = 16, kTY = 16;
constexpr int kThreads = kTX * kTY;
constexpr int kHX = kTX + 4, kHY = kTY + 4;
constexpr int kLayer = kHX * kHY;
constexpr int kRing = 4;
constexpr int kNFA = (kTX + 1) * kTY;
constexpr int kNFA_PAD = (kNFA + 31) / 32 * 32;
constexpr int kNFB = kTX * (kTY + 1);
static_assert(kThreads == kTileThreads, "one thread per column");

// Shared memory (floats): Q[ring][v][hy][hx], FA, FB of the current layer,
// TT[ring][hy][hx] (conduction only).  Every row is kRowPitch = 20 floats
// apart (FA and FB rows padded to it): a warp owns the columns of rows r and
// r + 4 (column_of), 80 floats = 16 banks apart, so its per-column accesses
// fall on disjoint banks.
constexpr int kRowPitch = kHX;
static_assert(kRowPitch >= kTX + 1 && (4 * kRowPitch) % 32 == 16, "rows r and r+4 on disjoint banks");
struct Smem3f {
  float* base;
  static constexpr int kFA = kRing * 5 * kLayer;
  static constexpr int kFB = kFA + 5 * kTY * kRowPitch;
  static constexpr int kT = kFB + 5 * (kTY + 1) * kRowPitch;
  static constexpr size_t bytes(bool tc) { return sizeof(float) * (size_t)(kT + (tc ? kRing * kLayer : 0)); }
  __device__ float& q(int s, int v, int hy, int hx) const { return base[((s * 5 + v) * kHY + hy) * kHX + hx]; }
  __device__ float& fa(int v, int fy, int fx) const { return base[kFA + (v * kTY + fy) * kRowPitch + fx]; }
  __device__ float& fb(int v, int fy, int fx) const { return base[kFB + (v * (kTY + 1) + fy) * kRowPitch + fx]; }
  __device__ float& temp(int s, int hy, int hx) const { return base[kT + (s * kHY + hy) * kHX + hx]; }
};

// The column (cx, cy) of the 16 x 16 block a thread owns: the two half-warps
// of warp w take rows r and r + 4 (r = (w & 3) + 8 * (w >> 2)).
__device__ __forceinline__ void column_of(int tid, int& cx, int& cy) {
  const int lane = tid & 31, w = tid >> 5;
  cx = lane & 15;
  cy = (w & 3) + ((w >> 2) << 3) + ((lane >> 4) << 2);
}

__device__ __forceinline__ int slot_of(int kg) { return (kg + 4) & 3; }

// The stage input of one stored cell: pairs (U^n) or U* values (internal
// energy in the energy slot).
struct MixedIn {
  const float2* const* pairs;  // src (STAGE_RK_1 / STAGE_EULER)
  const float* const* us;      // U* (STAGE_RK_2)
  bool in_pairs;
};

__device__ __forceinline__ void load_prim32(const MixedIn& in, unsigned o, float gm1, float q[5]) {
  if (in.in_pairs) {
    float2 w[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) w[v] = in.pairs[v][o];
    cons_to_prim_pairs<PLANE_XY, true>(w, gm1, q);
  } else {
    float u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = in.us[v][o];
    cons_to_prim_star<true>(u, gm1, q);
  }
}

// fillC91 (BoundaryConditions.h:87-134) in FP32, as the FP64 kernel's.
__device__ __forceinline__ void c91_ghost32(const Grid& G, const MixedIn& in, unsigned col, bool fa, bool fb, int kg,
                                            float res[5]) {
  const int kref = kg < 0 ? 0 : G.nc - 1;
  const int ksym = kg < 0 ? -kg - 1 : 2 * G.nc - kg - 1;
  float qref[5], qsym[5];
  const unsigned zs = (unsigned)G.nb * (unsigned)G.pitch;
  load_prim32(in, (unsigned)kref * zs + col, G.gm1_f, qref);
  load_prim32(in, (unsigned)ksym * zs + col, G.gm1_f, qsym);
  if (fa) {
    qref[1] = -qref[1];
    qsym[1] = -qsym[1];
  }
  if (fb) {
    qref[2] = -qref[2];
    qsym[2] = -qsym[2];
  }
  const float grav = G.gravity_flag ? 1.0f : 0.0f;
  const float posz = G.zmin_f + ((float)kg + 0.5f) * G.dz_f;
  if (kg < 0) {
    const float dz = posz - 0.5f * G.dz_f;
    const float T = 1.0f + posz * G.theta1_f;
    float p = qref[4] + dz * qref[0] * grav;
    float r = p / T;
    p = fmaxf(p, 1.0e-6f);
    r = fmaxf(r, 1.0e-6f);
    const float dratio = qsym[0] / r;
    res[0] = r;
    res[1] = qsym[1];
    res[2] = qsym[2];
    res[3] = -qsym[3] * dratio;
    res[4] = p;
  } else {
    const float Tref = qref[4] / qref[0];
    const float dz = posz - (1.0f - 0.5f * G.dz_f);
    const float T = Tref + dz * G.theta1_f;
    const float P = qref[4] + dz * qref[0] * grav;
    const float rho = P / T;
    res[4] = fmaxf(P, 1.0e-6f);
    res[0] = fmaxf(rho, 1.0e-6f);
    const float dratio = qsym[0] / rho;
    res[1] = qsym[1] * dratio;
    res[2] = qsym[2] * dratio;
    res[3] = -qsym[3] * dratio;
  }
}

__device__ __forceinline__ void load_layer32(const Grid& G, const MixedIn& in, int x0, int y0, int kg,
                                             const Smem3f& S, int tid) {
  const int s = slot_of(kg);
  const bool c91 = G.bc_c == DBC_C91 && (kg < 0 || kg >= G.nc);
  bool fz = false;
  const int sz = c91 ? 0 : bc_source(kg, G.nc, G.bc_c, fz);
  const unsigned zoff = (unsigned)sz * (unsigned)G.nb * (unsigned)G.pitch;
  for (int idx = tid; idx < kLayer; idx += kThreads) {
    const int hy = idx / kHX, hx = idx - hy * kHX;
    bool fa, fb;
    const int sa = bc_source(x0 + hx - 2, G.na, G.bc_a, fa);
    const int sb = bc_source(y0 + hy - 2, G.nb, G.bc_b, fb);
    const unsigned col = (unsigned)sb * (unsigned)G.pitch + (unsigned)sa;
    float q[5];
    if (!c91) {
      load_prim32(in, zoff + col, G.gm1_f, q);
      if (fa) q[1] = -q[1];
      if (fb) q[2] = -q[2];
      if (fz) q[3] = -q[3];
    } else {
      c91_ghost32(G, in, col, fa, fb, kg, q);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) S.q(s, v, hy, hx) = q[v];
    if (G.tc) S.temp(s, hy, hx) = q[4] / q[0];
  }
}

template <int DIR>
__device__ __forceinline__ Slots<float> slots3f(const float q[5]) {
  Slots<float> s;
  s.r = q[0];
  s.p = q[4];
  s.un = DIR == 0 ? q[1] : (DIR == 1 ? q[2] : q[3]);
  s.t1 = DIR == 1 ? q[1] : q[2];
  s.t2 = DIR == 2 ? q[1] : q[3];
  return s;
}

template <int DIR>
__device__ __forceinline__ void unslot3f(const float f[5], float out[5]) {
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

template <int DIR, bool CORR>
__device__ __forceinline__ void face3f(const float c[4][5], int rs, int recon, const Grid& G, float out[5],
                                       float* pout) {
  float qL[5], qR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    if (recon == R_PLM) {
      const float d01 = c[1][v] - c[0][v], d12 = c[2][v] - c[1][v], d23 = c[3][v] - c[2][v];
      qL[v] = c[1][v] + minmod32(d01, d12) * 0.5f;
      qR[v] = c[2][v] - minmod32(d12, d23) * 0.5f;
    } else {
      qL[v] = c[1][v];
      qR[v] = c[2][v];
    }
  }
  if (DIR == 2 && recon == R_PCM_WB) {  // Update.h:27
    qL[4] = qL[4] + qL[0] * G.g_dz_f * 0.5f;
    qR[4] = qR[4] - qR[0] * G.g_dz_f * 0.5f;
  }
  const Slots<float> L = slots3f<DIR>(qL), R = slots3f<DIR>(qR);
  float f[5];
  if (rs == 0)
    hll32(L, R, G.gamma_f, G.inv_gm1_f, f, pout);
  else
    hllc32<CORR>(L, R, G.gamma_f, G.inv_gm1_f, f, pout);
  unslot3f<DIR>(f, out);
}

struct RingVelF {
  Smem3f S;
  int k, hy, hx;
  __device__ __forceinline__ float operator()(int dk, int dj, int di, int var) const {
    return S.q(slot_of(k + dk - 1), var, hy + dj - 1, hx + di - 1);
  }
};

// One mixed stage of the columns (bx, by), z chunk bz of tz layers (CORR:
// the corrected physics, as the FP64 kernel's).  Inputs
// per kind as the 2-D mixed tile: RK_1 reads U^n pairs and writes U*; RK_2
// reads U* and U^n and writes U^n+1 over U^n; Euler reads pairs `src` and
// writes pairs `dst`.
template <int RS, bool CORR>
__device__ __forceinline__ void stage3d_body32(const Grid& G, const MixedFields& M, float2* const src[5],
                                               float2* const dst[5], StepCtrl* ctrl, int kind, int bx, int by, int bz,
                                               int tz, float* smem, unsigned long long* s_red) {
  const Smem3f S{smem};
  const int tid = threadIdx.x;
  const int x0 = bx * kTX, y0 = by * kTY;
  const int k0 = bz * tz;
  const int k1 = min(k0 + tz, G.nc);
  int cx, cy;
  column_of(tid, cx, cy);
  const int x = x0 + cx, y = y0 + cy;
  const bool own = x < G.na && y < G.nb;
  // 32-bit offsets (the host keeps every field below 2^32 elements for the
  // mixed kernels).  Measured: 3-6% faster than 64-bit offsets here, while the
  // 2-D tile kernels keep 64-bit offsets, which spare them a register spill.
  const unsigned col = (unsigned)y * (unsigned)G.pitch + (unsigned)x;
  const unsigned zstride = (unsigned)G.nb * (unsigned)G.pitch;

  if (!ctrl->active) {
    if (kind == STAGE_EULER && own) {
      for (int k = k0; k < k1; ++k) {
        const unsigned o = (unsigned)k * zstride + col;
#pragma unroll
        for (int v = 0; v < 5; ++v) dst[v][o] = src[v][o];
      }
    }
    return;
  }
  const float dt = (float)ctrl->dt_cur;  // once per work item
  const int parity = ctrl->parity;
  const int recon = G.recon;
  const bool need_pout = G.wb_flux_z || G.bc_c == DBC_C91;
  const MixedIn in{src, M.us, kind != STAGE_RK_2};
  const float dtdx = dt * G.inv_dx_f, dtdy = dt * G.inv_dy_f, dtdz = dt * G.inv_dz_f;

  for (int kg = k0 - 2; kg <= k0 + 1; ++kg) load_layer32(G, in, x0, y0, kg, S, tid);
  __syncthreads();
  float fzL[5], poutL = 0.0f;
  if (own) {
    float c[4][5];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int v = 0; v < 5; ++v) c[m][v] = S.q(slot_of(k0 - 2 + m), v, cy + 2, cx + 2);
    face3f<2, CORR>(c, RS, recon, G, fzL, need_pout ? &poutL : nullptr);
  }
  __syncthreads();

  float red = 0.0f;
  bool bad = false;
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    load_layer32(G, in, x0, y0, k + 2, S, tid);
    const int sk = slot_of(k);
    for (int it = tid; it < kNFA_PAD + kNFB; it += kThreads) {
      float c[4][5], f[5];
      if (it < kNFA_PAD) {
        if (it >= kNFA) continue;
        const int fy = it / (kTX + 1), fx = it - fy * (kTX + 1);
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int v = 0; v < 5; ++v) c[m][v] = S.q(sk, v, fy + 2, fx + m);
        face3f<0, CORR>(c, RS, recon, G, f, nullptr);
#pragma unroll
        for (int v = 0; v < 5; ++v) S.fa(v, fy, fx) = f[v];
      } else {
        const int j = it - kNFA_PAD;
        const int fy = j / kTX, fx = j - fy * kTX;
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int v = 0; v < 5; ++v) c[m][v] = S.q(sk, v, fy + m, fx + 2);
        face3f<1, CORR>(c, RS, recon, G, f, nullptr);
#pragma unroll
        for (int v = 0; v < 5; ++v) S.fb(v, fy, fx) = f[v];
      }
    }
    __syncthreads();

    if (own) {
#if FV_3D32_UN_PREFETCH
      if (kind == STAGE_RK_2) {  // U^n of the cell into L1 while the z face and increments are formed
        const unsigned o = (unsigned)k * zstride + col;
#pragma unroll
        for (int v = 0; v < 5; ++v) asm volatile("prefetch.global.L1 [%0];" ::"l"(M.un[v] + o));
      }
#endif
      float fzR[5], poutR = 0.0f;
      {
        float c[4][5];
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int v = 0; v < 5; ++v) c[m][v] = S.q(slot_of(k - 1 + m), v, cy + 2, cx + 2);
        face3f<2, CORR>(c, RS, recon, G, fzR, need_pout ? &poutR : nullptr);
      }
      const unsigned o = (unsigned)k * zstride + col;
      float fL[5], fR[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        fL[v] = fzL[v];
        fR[v] = fzR[v];
      }
      const float rho_c = S.q(sk, 0, cy + 2, cx + 2);
      if (G.wb_flux_z && (k == 0 || k == G.nc - 1)) {  // Update.h:131-137
        if (k == 0) {
          fL[0] = 0.0f; fL[1] = 0.0f; fL[2] = 0.0f; fL[4] = 0.0f;
          fL[3] = poutR - rho_c * G.g_dz_f;
        } else {
          fR[0] = 0.0f; fR[1] = 0.0f; fR[2] = 0.0f; fR[4] = 0.0f;
          fR[3] = poutL + rho_c * G.g_dz_f;
        }
      } else if (G.bc_c == DBC_C91 && (k == 0 || k == G.nc - 1)) {  // Update.h:138-143
        if (k == 0) {
          fL[0] = 0.0f; fL[1] = 0.0f; fL[2] = 0.0f; fL[4] = 0.0f;
          fL[3] = poutL;
        } else {
          fR[0] = 0.0f; fR[1] = 0.0f; fR[2] = 0.0f; fR[4] = 0.0f;
          fR[3] = poutR;
        }
      }
      float du[5];
#pragma unroll
      for (int v = 0; v < 5; ++v)
        du[v] = (S.fa(v, cy, cx) - S.fa(v, cy, cx + 1)) * dtdx + (S.fb(v, cy, cx) - S.fb(v, cy + 1, cx)) * dtdy +
                (fL[v] - fR[v]) * dtdz;
      if (G.gravity) {
        du[3] += dt * rho_c * G.g_f;
        du[4] += dt * 0.5f * (fL[0] + fR[0]) * G.g_f;
      }
      float2 base[5];  // the stage input at this cell as pairs (U*: E* rebuilt, fv_tile32.cuh)
      if (in.in_pairs) {
#pragma unroll
        for (int v = 0; v < 5; ++v) base[v] = src[v][o];
      } else {
        float u[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) u[v] = M.us[v][o];
#pragma unroll
        for (int v = 0; v < 4; ++v) base[v] = make_float2(u[v], 0.0f);
        base[4] = pair_add(kinetic_star<true>(u), u[4]);
      }
      {  // density floor on the hydro update (Update.h:160)
        const float2 rho = pair_add(base[0], du[0]);
        if (rho.x + rho.y < 1.0e-6f) {
          base[0] = make_float2(1.0e-6f, 0.0f);
          du[0] = 0.0f;
        }
      }
      if (G.tc) {  // ThermalConduction.h:38-96
        const float kC = G.kappa_f, kF = G.kappa_f, kB = G.kappa_f;  // batches take constant kappa
        const int hy = cy + 2, hx = cx + 2;
        const float TC = S.temp(sk, hy, hx);
        const float FL = kC * (TC - S.temp(sk, hy, hx - 1)) * G.inv_dx_f;
        const float FR = kC * (S.temp(sk, hy, hx + 1) - TC) * G.inv_dx_f;
        const float FU = kC * (TC - S.temp(sk, hy - 1, hx)) * G.inv_dy_f;
        const float FD = kC * (S.temp(sk, hy + 1, hx) - TC) * G.inv_dy_f;
        float FF = kF * (TC - S.temp(slot_of(k - 1), hy, hx)) * G.inv_dz_f;
        float FB = kB * (S.temp(slot_of(k + 1), hy, hx) - TC) * G.inv_dz_f;
        if (k == 0 && G.bctc_zmin != 0)
          FF = G.bctc_zmin == 1 ? kF * 2.0f * (TC - G.bctc_zmin_value_f) * G.inv_dz_f : kF * G.bctc_zmin_value_f;
        if (k == G.nc - 1 && G.bctc_zmax != 0)
          FB = G.bctc_zmax == 1 ? kB * 2.0f * (G.bctc_zmax_value_f - TC) * G.inv_dz_f : kB * G.bctc_zmax_value_f;
        du[4] += dtdx * (FR - FL) + dtdy * (FD - FU) + dtdz * (FB - FF);
      }
      if (G.visc) {  // Viscosity.h:145-151
        const RingVelF P{S, k, cy + 2, cx + 2};
        float vf[3][5];
        viscous3d<CORR, float>(P, G.inv_dx_f, G.inv_dy_f, G.inv_dz_f, G.mu_f, vf);
        if (CORR) {  // the flux differences divided by the cell sizes
#pragma unroll
          for (int v = 1; v < 5; ++v)
            du[v] += (vf[0][v] * G.inv_dx_f + vf[1][v] * G.inv_dy_f + vf[2][v] * G.inv_dz_f) * dt;
        } else {
#pragma unroll
          for (int v = 1; v < 5; ++v) du[v] += (vf[0][v] + vf[1][v] + vf[2][v]) * dt;
        }
      }
      if (kind == STAGE_RK_1) {
        float us[5];
#pragma unroll
        for (int v = 0; v < 4; ++v) us[v] = base[v].x + (base[v].y + du[v]);
        us[4] = internal_energy(pair_add(base[4], du[4]), kinetic_star<true>(us));
#pragma unroll
        for (int v = 0; v < 5; ++v) M.us[v][o] = us[v];
      } else {
        float2 fin[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          float2 r;
          if (kind == STAGE_RK_2) {
            r = pair_add(pair_add(M.un[v][o], base[v]), du[v]);
            r = make_float2(0.5f * r.x, 0.5f * r.y);
          } else {
            r = pair_add(base[v], du[v]);
          }
          dst[v][o] = r;
          fin[v] = r;
        }
        const float inv = inv_dt_hyp32<PLANE_XY, true>(fin, G);
        bad |= !(inv <= 3.0e38f);
        red = fmaxf(red, inv);
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) fzL[v] = fzR[v];
      poutL = poutR;
    }
    __syncthreads();
  }
  if (kind != STAGE_RK_1) {
    if (bad) atomicOr(&ctrl->err, 1);
    block_max_atomic((unsigned long long)__double_as_longlong((double)red), &ctrl->slot[parity ^ 1], s_red);
  }
}

static_assert(sizeof(BatchInst) % 8 == 0, "descriptor copied as 8-byte words");

template <int RS, bool CORR>
__global__ void __launch_bounds__(kThreads, 4)
batch_stage3d32(const BatchInst* __restrict__ insts, int ninst, int ntiles, unsigned* queue, int kind, int flip) {
  extern __shared__ float smem_f[];
  __shared__ unsigned long long s_red[kThreads / 32];
  __shared__ BatchInst s_inst;
  __shared__ int s_tile;
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
      const unsigned long long* s = reinterpret_cast<const unsigned long long*>(insts + lo);
      unsigned long long* d = reinterpret_cast<unsigned long long*>(&s_inst);
      for (int w = threadIdx.x; w < (int)(sizeof(BatchInst) / 8); w += blockDim.x) d[w] = s[w];
    }
    __syncthreads();
    const BatchInst& I = s_inst;
    const int lt = t - I.tile0;
    const int per_layer = I.tiles_x * I.tiles_y;
    const int bz = lt / per_layer, rem = lt - bz * per_layer;
    const int by = rem / I.tiles_x, bx = rem - by * I.tiles_x;
    MixedFields M;
    float2* src[5];
    float2* dst[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      M.un[v] = reinterpret_cast<float2*>(I.A.f[v]);
      M.us[v] = reinterpret_cast<float*>(I.B.f[v]);
      float2* a = reinterpret_cast<float2*>(I.A.f[v]);
      float2* b = reinterpret_cast<float2*>(I.B.f[v]);
      src[v] = (kind == STAGE_EULER && flip) ? b : a;
      dst[v] = (kind == STAGE_EULER && !flip) ? b : a;
    }
    stage3d_body32<RS, CORR>(I.G, M, src, dst, I.ctrl, kind, bx, by, bz, I.tz, smem_f, s_red);
  }
}

typedef void (*Batch3dKernel32)(const BatchInst*, int, int, unsigned*, int, int);

// rs: the Riemann solver (bit 0) and the corrected physics (bit 1).
Batch3dKernel32 kernel32(int rs) {
  switch (rs & 3) {
    case 0: return batch_stage3d32<0, false>;
    case 1: return batch_stage3d32<1, false>;
    case 2: return batch_stage3d32<0, true>;
    default: return batch_stage3d32<1, true>;
  }
}

bool prepare32() {
  static bool done = false;
  if (done) return true;
  for (int rs = 0; rs < 4; ++rs)
    if (cudaFuncSetAttribute(kernel32(rs), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Smem3f::bytes(true)) !=
        cudaSuccess)
      return false;
  done = true;
  return true;
}

}  // namespace

int batch_stage3d_occupancy32(int rs, bool tc) {
  if (!prepare32()) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel32(rs), kThreads, Smem3f::bytes(tc)) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_batch_stage3d32(const BatchInst* insts, int ninst, int ntiles, unsigned* queue, int kind, int flip,
                                   int rs, int grid, bool tc, cudaStream_t st) {
  if (!prepare32()) return cudaErrorInvalidConfiguration;
  const cudaError_t e =
      launch_pdl(kernel32(rs), dim3(grid), dim3(kThreads), Smem3f::bytes(tc), st, insts, ninst, ntiles, queue, kind, flip);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace fv
