// fv_batch64.cu -- persistent FP64 stage kernel for batches of problems.
//
// One launch per RK stage covers every problem of a group (same plane, same
// third-momentum layout): `grid` resident CTAs repeatedly take the next work
// item from a global work-queue counter, find the problem owning it (binary
// search over the problems' first item numbers), copy its descriptor to
// shared memory and run it.  A work item is a piece of one problem: a strip
// segment of tx columns and BatchInst::tz rows, marched in blocks of 512 cells
// (stage_segment64), so consecutive blocks share boundary rows and faces.
// Each problem keeps its own control block, so its own dt and its own CFL
// reduction slot.  Compiled without FMA contraction: a problem advanced in a
// batch is bit-identical to the same problem advanced alone, and to the
// reference.
#include "fv_tile64.cuh"

namespace fv {

namespace {

// Work-item shapes (cells along a x rows along b) the autotuner starts from;
// the rows of an item are a run-time value (BatchInst::tz), so the shapes
// that share a strip width share a kernel (kKernelOf64: the shape whose
// instantiation serves it).
constexpr TileShape kShapes64[] = {{32, 64}, {32, 32}, {32, 16}, {64, 32}};
constexpr int kKernelOf64[] = {0, 0, 0, 3};
constexpr int kNumShapes64 = sizeof(kShapes64) / sizeof(kShapes64[0]);
constexpr int block_rows(int tx) { return 2 * kTileThreads / tx; }  // 512-cell blocks

static_assert(sizeof(BatchInst) % 8 == 0, "descriptor copied as 8-byte words");

// Finds the problem owning item t and copies its descriptor to shared memory.
__device__ __forceinline__ void fetch_inst(const BatchInst* __restrict__ insts, int ninst, int t, BatchInst* s_inst) {
  int lo = 0, hi = ninst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (insts[mid].tile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(insts + lo);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(s_inst);
  for (int w = threadIdx.x; w < (int)(sizeof(BatchInst) / 8); w += blockDim.x) dst[w] = src[w];
}

template <int PLANE, bool WACT, class TL>
__global__ void __launch_bounds__(kTileThreads, WACT ? FV_FP64_MIN_CTAS_W : FV_FP64_MIN_CTAS)
batch_stage64(const BatchInst* __restrict__ insts, int ninst, int ntiles, unsigned* queue, int kind, int flip) {
  extern __shared__ double smem_raw[];
  __shared__ unsigned long long s_red[kTileThreads / 32];
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
    fetch_inst(insts, ninst, t, &s_inst);
    __syncthreads();
    const BatchInst& I = s_inst;
    const int lt = t - I.tile0;
    const int bx = lt % I.tiles_x, by = lt / I.tiles_x;
    Fields uin, u0, uout;
    if (kind == STAGE_RK_1) {
      uin = I.A; u0 = I.A; uout = I.B;
    } else if (kind == STAGE_RK_2) {
      uin = I.B; u0 = I.A; uout = I.A;
    } else {
      uin = flip ? I.B : I.A; u0 = uin; uout = flip ? I.A : I.B;
    }
    StepCtrl* ctrl = I.ctrl;
    // the primitive copy: read by stage 1 while valid, written by stage 2
    const Fields* qi = kind == STAGE_RK_1 && I.Q.f[0] && ctrl->q_valid ? &I.Q : nullptr;
    const Fields* qo = kind == STAGE_RK_2 && I.Q.f[0] ? &I.Q : nullptr;
    const int x0 = bx * TL::TX, ya = by * I.tz;  // tz: rows per work item
    const int yb = ya + I.tz < I.G.nb ? ya + I.tz : I.G.nb;
    if (!ctrl->active) {
      if (kind == STAGE_EULER) pass_on64<WACT, TL::TX>(I.G, uin, uout, x0, ya, yb, threadIdx.x);
      continue;
    }
    unsigned long long red = 0ull;
    if (I.G.pow2_all)
      stage_segment64<PLANE, WACT, TL, true>(I.G, uin, u0, uout, ctrl, I.rs, kind, ctrl->dt_cur, x0, ya, yb, smem_raw,
                                             nullptr, red, nullptr, nullptr, nullptr, qi, qo);
    else
      stage_segment64<PLANE, WACT, TL, false>(I.G, uin, u0, uout, ctrl, I.rs, kind, ctrl->dt_cur, x0, ya, yb,
                                              smem_raw, nullptr, red, nullptr, nullptr, nullptr, qi, qo);
    if (kind != STAGE_RK_1) block_max_atomic(red, &ctrl->slot[ctrl->parity ^ 1], s_red);
    // the copy is complete once this launch is (the next reader is a later kernel)
    if (qo && threadIdx.x == 0) ctrl->q_valid = 1;
  }
}

template <int S>
using BlockOf = Tile<kShapes64[S].tx, block_rows(kShapes64[S].tx)>;

template <int PLANE, bool WACT, int S>
auto kernel_for() {
  return batch_stage64<PLANE, WACT, BlockOf<S>>;
}

// wact groups (viscosity on, or a non-zero third velocity) get the largest
// layout, the one with shared-face viscous fluxes.
template <int S>
size_t smem_for(bool wact, bool tc) {
  return wact ? TileSmem<double, 5, BlockOf<S>>::bytes_vface() : TileSmem<double, 4, BlockOf<S>>::bytes(tc);
}

typedef void (*BatchKernel)(const BatchInst*, int, int, unsigned*, int, int);

template <int PLANE, bool WACT>
BatchKernel pick(int shape) {
  return kKernelOf64[shape] == 0 ? kernel_for<PLANE, WACT, 0>() : kernel_for<PLANE, WACT, 3>();
}

BatchKernel pick_any(int plane, bool wact, int shape) {
  if (plane == PLANE_XY) return wact ? pick<PLANE_XY, true>(shape) : pick<PLANE_XY, false>(shape);
  return wact ? pick<PLANE_XZ, true>(shape) : pick<PLANE_XZ, false>(shape);
}

size_t smem_any(int shape, bool wact, bool tc) {
  switch (shape) {
    case 0: return smem_for<0>(wact, tc);
    case 1: return smem_for<1>(wact, tc);
    case 2: return smem_for<2>(wact, tc);
    default: return smem_for<3>(wact, tc);
  }
}

// Allows the largest layout (with conduction) once per kernel and process.
cudaError_t prepare(int plane, bool wact, int shape) {
  static bool done[2][2][kNumShapes64] = {};
  bool& flag = done[plane == PLANE_XY ? 0 : 1][wact ? 1 : 0][shape];
  if (flag) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(pick_any(plane, wact, shape), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_any(shape, wact, true));
  if (e == cudaSuccess) flag = true;
  return e;
}

}  // namespace

int batch_tile_shapes64(const TileShape** shapes) {
  *shapes = kShapes64;
  return kNumShapes64;
}

int batch_stage_occupancy64(int plane, bool wact, int shape, bool tc) {
  if (shape < 0 || shape >= kNumShapes64 || prepare(plane, wact, shape) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pick_any(plane, wact, shape), kTileThreads,
                                                    smem_any(shape, wact, tc)) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_batch_stage64(int plane, bool wact, int shape, const BatchInst* insts, int ninst, int ntiles,
                                 unsigned* queue, int kind, int flip, int grid, bool tc, cudaStream_t st) {
  if (shape < 0 || shape >= kNumShapes64) return cudaErrorInvalidValue;
  cudaError_t e = prepare(plane, wact, shape);
  if (e != cudaSuccess) return e;
  e = launch_pdl(pick_any(plane, wact, shape), dim3(grid), dim3(kTileThreads), smem_any(shape, wact, tc), st, insts,
                 ninst, ntiles, queue, kind, flip);
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace fv
