// fv_batch32.cu -- FP32-mixed persistent stage kernel for batches, plus the
// mixed form's CFL reduction and its (hi, lo) pair conversions.  Built with
// fast-math (FP32 division / sqrt approximations, FMA contraction); the
// error-free pair arithmetic of fv_tile32.cuh is written with adds and _rn
// intrinsics, which contraction leaves alone.
#include "fv_control.cuh"
#include "fv_grid.cuh"
#include "fv_tile32.cuh"

namespace fv {

namespace {

// Work-item shapes (cells along a x rows along b) the autotuner starts
// from, each with the kernel that marches it: strip segments marched in
// blocks of 16 or 8 rows (cells per thread in the update: 32x16 -> 2,
// 64x16 -> 4, 32x8 -> 1, 64x8 -> 2), with the viscous fluxes fused per cell
// or split into a per-face pass (VF).  The rows of an item are a run-time
// value (BatchInst::tz), so shapes of one kernel differ only in their
// starting rows.
struct MixedKernel {
  int tx, block_rows, vface;
};
// Block rows of the two block heights (cells per thread in the update: 2 and
// 1 for 32-wide blocks).
#ifndef FV_MIXED_BR_A
#define FV_MIXED_BR_A 16
#endif
#ifndef FV_MIXED_BR_B
#define FV_MIXED_BR_B 8
#endif
constexpr int kBrA = FV_MIXED_BR_A, kBrB = FV_MIXED_BR_B;
constexpr MixedKernel kKernels32[] = {{32, kBrA, 0}, {64, kBrA, 0}, {32, kBrB, 0},
                                      {64, kBrB, 0}, {32, kBrA, 1}, {64, kBrA, 1}};
constexpr TileShape kShapes32[] = {{32, 2 * kBrA}, {64, kBrA},     {32, kBrA}, {64, 2 * kBrA},
                                   {32, 2 * kBrB}, {64, kBrB},     {32, 2 * kBrA}, {64, kBrA}};
constexpr int kKernelOf32[] = {0, 1, 0, 1, 2, 3, 4, 5};
constexpr int kNumShapes32 = sizeof(kShapes32) / sizeof(kShapes32[0]);

// Copies the descriptor of the problem holding work item t to s_inst and
// returns its index (binary search over the first items).
__device__ __forceinline__ int fetch_inst32(const BatchInst* __restrict__ insts, int ninst, int t,
                                            BatchInst* s_inst) {
  int lo = 0, hi = ninst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (insts[mid].tile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(insts + lo);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(s_inst);
  for (int w = threadIdx.x; w < (int)(sizeof(BatchInst) / 8); w += blockDim.x) dst[w] = src[w];
  return lo;
}

#if FV_MIXED_MIN_CTAS > 0
#define FV_MIXED_BOUNDS __launch_bounds__(kTileThreads, FV_MIXED_MIN_CTAS)
#else
#define FV_MIXED_BOUNDS __launch_bounds__(kTileThreads)
#endif

// One work item t (a strip segment of problem I) of one stage.  active / dt:
// the problem's step in flight; slot_next / err: its CFL maximum slot for the
// next step and its error flag (stages that end a step).  Every thread of
// the CTA calls it; s_inst holds I.
template <int PLANE, bool WACT, class TL, bool VF>
__device__ __forceinline__ void stage_item32(const BatchInst& I, int t, int kind, int flip, bool active, double dt_step,
                                             unsigned long long* slot_next, int* err, float* smem,
                                             unsigned long long* s_red) {
  const int lt = t - I.tile0;
  const int bx = lt % I.tiles_x, by = lt / I.tiles_x;
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
  const int x0 = bx * TL::TX, ya = by * I.tz;  // tz: rows per work item
  const int yb = ya + I.tz < I.G.nb ? ya + I.tz : I.G.nb;
  if (!active) {
    if (kind == STAGE_EULER) pass_on32<WACT, TL::TX>(I.G, src, dst, x0, ya, yb, threadIdx.x);
    return;
  }
  const float dt = (float)dt_step;  // the one FP64 -> FP32 conversion per item
  float red = 0.0f;
  bool bad = false;
  stage_segment32<PLANE, WACT, TL, VF>(I.G, M, src, dst, I.rs, kind, dt, x0, ya, yb, smem, red, bad);
  if (kind != STAGE_RK_1) {
    if (bad) atomicOr(err, 1);
    block_max_atomic((unsigned long long)__double_as_longlong((double)red), slot_next, s_red);
  }
}

template <int PLANE, bool WACT, class TL, bool VF>
__global__ void FV_MIXED_BOUNDS
batch_stage32(const BatchInst* __restrict__ insts, int ninst, int ntiles, unsigned* queue, int kind, int flip) {
  extern __shared__ float smem_f[];
  __shared__ unsigned long long s_red[kTileThreads / 32];
  __shared__ BatchInst s_inst;
  __shared__ int s_tile;
  pdl_wait();
  for (;;) {
    __syncthreads();  // the previous tile is finished with s_tile, s_inst and smem
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) {
      pdl_trigger();  // no work left for this CTA
      break;
    }
    fetch_inst32(insts, ninst, t, &s_inst);
    __syncthreads();
    StepCtrl* ctrl = s_inst.ctrl;
    stage_item32<PLANE, WACT, TL, VF>(s_inst, t, kind, flip, ctrl->active != 0, ctrl->dt_cur,
                                  &ctrl->slot[ctrl->parity ^ 1], &ctrl->err, smem_f, s_red);
  }
}

// Problems a multi-step launch can carry (per-problem step state sits in
// shared memory).
constexpr int kMultiMaxProblems = 256;

// Several RK2 steps of a group in one cooperative launch (every CTA
// resident): per step, each CTA decides every problem's dt and active flag
// itself (step_decide on the reduced CFL maximum, the same arithmetic as the
// control kernel, so every CTA reaches the same values), then stage 1 over
// the work items t = blockIdx.x, blockIdx.x + gridDim.x, ..., a grid
// barrier, stage 2 (CFL maxima by atomics), a grid barrier.  Each work item
// runs the per-stage kernel's body, so the result is bit-identical to the
// per-stage launches.  The time and step counter of each problem are kept in
// shared memory during the launch and written back to the control blocks at
// its end by CTA 0; the CFL slot of the next step is zeroed by CTA 0.  A
// barrier wait that runs out sets bit 1 of every problem's error flag and
// the kernel returns.
template <int PLANE, bool WACT, class TL>
__global__ void FV_MIXED_BOUNDS batch_multi32(const BatchInst* __restrict__ insts, int ninst, int ntiles, int nsteps,
                                              int mode_override, GridBarrier gb) {
  extern __shared__ float smem_f[];
  __shared__ unsigned long long s_red[kTileThreads / 32];
  __shared__ BatchInst s_inst;
  __shared__ double s_t[kMultiMaxProblems], s_dt[kMultiMaxProblems];
  __shared__ long long s_step[kMultiMaxProblems];
  __shared__ int s_act[kMultiMaxProblems], s_par[kMultiMaxProblems], s_err[kMultiMaxProblems];
  __shared__ int s_any;
  auto timed_out = [&]() {
    if (threadIdx.x == 0)
      for (int m = 0; m < ninst; ++m) atomicOr(&insts[m].ctrl->err, 2);
  };
  for (int m = threadIdx.x; m < ninst; m += blockDim.x) {
    const StepCtrl* c = insts[m].ctrl;
    s_t[m] = c->t;
    s_step[m] = c->step;
    s_err[m] = 0;
  }
  __syncthreads();
  unsigned bar = 0;
  // every CTA has read the initial times before CTA 0 may write any control block
  if (!grid_sync(gb, bar++)) {
    timed_out();
    return;
  }
  int k = 0;
  bool decided = false;
  for (; k < nsteps; ++k) {
    if (threadIdx.x == 0) s_any = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < ninst; m += blockDim.x) {
      StepCtrl* c = insts[m].ctrl;
      double dt;
      int active;
      bool bad;
      step_decide(*c, s_t[m], s_step[m], c->err | s_err[m], mode_override, 0.0, dt, active, bad);
      const int p = (int)(s_step[m] & 1);
      if (bad) s_err[m] = 1;
      s_dt[m] = active ? dt : 0.0;
      s_act[m] = active;
      s_par[m] = p;
      if (blockIdx.x == 0) c->slot[p ^ 1] = 0ull;  // read by no CTA in this step
      if (active) {
        s_t[m] = __dadd_rn(s_t[m], dt);
        s_step[m] += 1;
        s_any = 1;
      }
    }
    __syncthreads();
    decided = true;
    if (!s_any) break;  // every CTA decides alike: no problem steps any more
    // kind stays a run-time value, as in the per-stage kernel: a copy of the
    // stage body specialised per kind may contract its multiply-adds
    // differently and break the bit-for-bit equality with the per-stage form
#pragma unroll 1
    for (int kind = STAGE_RK_1; kind <= STAGE_RK_2; ++kind) {
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        __syncthreads();  // the previous item is finished with s_inst and smem
        const int m = fetch_inst32(insts, ninst, t, &s_inst);
        __syncthreads();
        StepCtrl* ctrl = s_inst.ctrl;
        stage_item32<PLANE, WACT, TL, false>(s_inst, t, kind, 0, s_act[m] != 0, s_dt[m], &ctrl->slot[s_par[m] ^ 1],
                                      &ctrl->err, smem_f, s_red);
      }
      if (!grid_sync(gb, bar++)) {
        timed_out();
        return;
      }
    }
  }
  if (blockIdx.x == 0) {  // the control blocks as the per-stage launches leave them
    for (int m = threadIdx.x; m < ninst; m += blockDim.x) {
      StepCtrl* c = insts[m].ctrl;
      if (decided) {
        c->parity = s_par[m];
        c->active = s_act[m];
        c->dt_cur = s_dt[m];
      }
      c->t = s_t[m];
      c->step = s_step[m];
      if (s_err[m]) atomicOr(&c->err, 1);
    }
  }
}

template <int K>
using BlockOf32 = Tile<kKernels32[K].tx, kKernels32[K].block_rows>;

template <int PLANE, bool WACT, int K>
auto kernel_for() {
  return batch_stage32<PLANE, WACT, BlockOf32<K>, kKernels32[K].vface != 0>;
}

template <int K>
size_t smem_for(bool wact, bool tc) {
  if (kKernels32[K].vface && wact) return TileSmem<float, 5, BlockOf32<K>>::bytes_vface();
  return wact ? TileSmem<float, 5, BlockOf32<K>>::bytes(tc) : TileSmem<float, 4, BlockOf32<K>>::bytes(tc);
}

typedef void (*BatchKernel)(const BatchInst*, int, int, unsigned*, int, int);

typedef void (*MultiKernel)(const BatchInst*, int, int, int, int, GridBarrier);

template <int PLANE, bool WACT>
MultiKernel pick_multi(int shape) {  // fused viscous form only (shapes of kernels 0-3)
  switch (kKernelOf32[shape]) {
    case 0: return batch_multi32<PLANE, WACT, BlockOf32<0>>;
    case 1: return batch_multi32<PLANE, WACT, BlockOf32<1>>;
    case 2: return batch_multi32<PLANE, WACT, BlockOf32<2>>;
    default: return batch_multi32<PLANE, WACT, BlockOf32<3>>;
  }
}

MultiKernel pick_multi_any(int plane, bool wact, int shape) {
  if (plane == PLANE_XY) return wact ? pick_multi<PLANE_XY, true>(shape) : pick_multi<PLANE_XY, false>(shape);
  return wact ? pick_multi<PLANE_XZ, true>(shape) : pick_multi<PLANE_XZ, false>(shape);
}

template <int PLANE, bool WACT>
BatchKernel pick(int shape) {
  switch (kKernelOf32[shape]) {
    case 0: return kernel_for<PLANE, WACT, 0>();
    case 1: return kernel_for<PLANE, WACT, 1>();
    case 2: return kernel_for<PLANE, WACT, 2>();
    case 3: return kernel_for<PLANE, WACT, 3>();
    case 4: return kernel_for<PLANE, WACT, 4>();
    default: return kernel_for<PLANE, WACT, 5>();
  }
}

BatchKernel pick_any(int plane, bool wact, int shape) {
  if (plane == PLANE_XY) return wact ? pick<PLANE_XY, true>(shape) : pick<PLANE_XY, false>(shape);
  return wact ? pick<PLANE_XZ, true>(shape) : pick<PLANE_XZ, false>(shape);
}

size_t smem_any(int shape, bool wact, bool tc) {
  switch (kKernelOf32[shape]) {
    case 0: return smem_for<0>(wact, tc);
    case 1: return smem_for<1>(wact, tc);
    case 2: return smem_for<2>(wact, tc);
    case 3: return smem_for<3>(wact, tc);
    case 4: return smem_for<4>(wact, tc);
    default: return smem_for<5>(wact, tc);
  }
}

cudaError_t prepare(int plane, bool wact, int shape) {
  static bool done[2][2][kNumShapes32] = {};
  bool& flag = done[plane == PLANE_XY ? 0 : 1][wact ? 1 : 0][shape];
  if (flag) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(pick_any(plane, wact, shape), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_any(shape, wact, true));
  if (e == cudaSuccess) flag = true;
  return e;
}

cudaError_t prepare_multi(int plane, bool wact, int shape) {
  static bool done[2][2][kNumShapes32] = {};
  bool& flag = done[plane == PLANE_XY ? 0 : 1][wact ? 1 : 0][shape];
  if (flag) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(pick_multi_any(plane, wact, shape),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_any(shape, wact, true));
  if (e == cudaSuccess) flag = true;
  return e;
}

int grid_for(long long n, int block) {
  long long b = (n + block - 1) / block;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

// CFL maximum of a state held as (hi, lo) pairs.
template <int PLANE, bool WACT>
__global__ void __launch_bounds__(256) reduce2d_mixed(const Grid G, const Fields pairs, StepCtrl* ctrl, int slot) {
  __shared__ unsigned long long s_red[8];
  float red = 0.0f;
  bool bad = false;
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
    float2 w[5];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      w[v] = (v == 3 && !WACT) ? make_float2(0.0f, 0.0f) : reinterpret_cast<const float2*>(pairs.f[v])[o];
    const float inv = inv_dt_hyp32<PLANE, WACT>(w, G);
    bad |= !(inv <= 3.0e38f);
    red = fmaxf(red, inv);
  }
  if (bad) atomicOr(&ctrl->err, 1);
  block_max_atomic((unsigned long long)__double_as_longlong((double)red), &ctrl->slot[slot], s_red);
}

// FP64 values -> (hi, lo) float pairs: hi = RN32(d), lo = RN32(d - hi).
__global__ void pairs_from_double(const Grid G, const Fields src, const Fields dst) {
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double d = src.f[v][o];
      const float hi = __double2float_rn(d);
      const float lo = __double2float_rn(d - (double)hi);
      reinterpret_cast<float2*>(dst.f[v])[o] = make_float2(hi, lo);
    }
  }
}

// (hi, lo) pairs -> FP64 values hi + lo (exact).
__global__ void double_from_pairs(const Grid G, const Fields src, const Fields dst) {
  const long long n = (long long)G.na * G.rows;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / G.na), x = (int)(c - (long long)y * G.na);
    const long long o = (long long)y * G.pitch + x;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const float2 w = reinterpret_cast<const float2*>(src.f[v])[o];
      dst.f[v][o] = (double)w.x + (double)w.y;
    }
  }
}

}  // namespace

int batch_tile_shapes32(const TileShape** shapes) {
  *shapes = kShapes32;
  return kNumShapes32;
}

int batch_shape_kernel32(int shape, int* block_rows, int* vface) {
  if (shape < 0 || shape >= kNumShapes32) return -1;
  const MixedKernel& k = kKernels32[kKernelOf32[shape]];
  if (block_rows) *block_rows = k.block_rows;
  if (vface) *vface = k.vface;
  return kKernelOf32[shape];
}

int batch_stage_occupancy32(int plane, bool wact, int shape, bool tc) {
  if (shape < 0 || shape >= kNumShapes32 || prepare(plane, wact, shape) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pick_any(plane, wact, shape), kTileThreads,
                                                    smem_any(shape, wact, tc)) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_batch_stage32(int plane, bool wact, int shape, const BatchInst* insts, int ninst, int ntiles,
                                 unsigned* queue, int kind, int flip, int grid, bool tc, cudaStream_t st) {
  if (shape < 0 || shape >= kNumShapes32) return cudaErrorInvalidValue;
  cudaError_t e = prepare(plane, wact, shape);
  if (e != cudaSuccess) return e;
  e = launch_pdl(pick_any(plane, wact, shape), dim3(grid), dim3(kTileThreads), smem_any(shape, wact, tc), st, insts,
                 ninst, ntiles, queue, kind, flip);
  return e != cudaSuccess ? e : cudaGetLastError();
}

int batch_multi_problems32() { return kMultiMaxProblems; }

int batch_multi_occupancy32(int plane, bool wact, int shape, bool tc) {
  if (shape < 0 || shape >= kNumShapes32 || prepare_multi(plane, wact, shape) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pick_multi_any(plane, wact, shape), kTileThreads,
                                                    smem_any(shape, wact, tc)) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_batch_multi32(int plane, bool wact, int shape, const BatchInst* insts, int ninst, int ntiles,
                                 int nsteps, int mode_override, GridBarrier gb, int grid, bool tc,
                                 cudaStream_t st) {
  if (shape < 0 || shape >= kNumShapes32 || ninst > kMultiMaxProblems) return cudaErrorInvalidValue;
  cudaError_t e = prepare_multi(plane, wact, shape);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kTileThreads);
  cfg.dynamicSmemBytes = smem_any(shape, wact, tc);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident: the grid barriers need it
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, pick_multi_any(plane, wact, shape), insts, ninst, ntiles, nsteps, mode_override, gb);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_reduce2d_mixed(const Grid& G, bool wact, Fields pairs, StepCtrl* ctrl, int slot,
                                  cudaStream_t st) {
  const int grid = grid_for((long long)G.na * G.rows, 256);
  if (G.plane == PLANE_XY) {
    if (wact) reduce2d_mixed<PLANE_XY, true><<<grid, 256, 0, st>>>(G, pairs, ctrl, slot);
    else reduce2d_mixed<PLANE_XY, false><<<grid, 256, 0, st>>>(G, pairs, ctrl, slot);
  } else {
    if (wact) reduce2d_mixed<PLANE_XZ, true><<<grid, 256, 0, st>>>(G, pairs, ctrl, slot);
    else reduce2d_mixed<PLANE_XZ, false><<<grid, 256, 0, st>>>(G, pairs, ctrl, slot);
  }
  return cudaGetLastError();
}

cudaError_t launch_pairs_from_double(const Grid& G, Fields src, Fields dst_pairs, cudaStream_t st) {
  pairs_from_double<<<grid_for((long long)G.na * G.rows, 256), 256, 0, st>>>(G, src, dst_pairs);
  return cudaGetLastError();
}

cudaError_t launch_double_from_pairs(const Grid& G, Fields src_pairs, Fields dst, cudaStream_t st) {
  double_from_pairs<<<grid_for((long long)G.na * G.rows, 256), 256, 0, st>>>(G, src_pairs, dst);
  return cudaGetLastError();
}

}  // namespace fv
