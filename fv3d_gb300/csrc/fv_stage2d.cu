// fv_stage2d.cu -- the FP64 fused stage kernel of one 2-D problem: 32-wide
// strips of cells marched in blocks of 32x16 cells (stage_strip64 in
// fv_tile64.cuh, compiled without FMA contraction, so it rounds exactly like
// the reference).  The strip rows are split evenly over as many CTAs as the
// GPU holds at once, so every SM gets the same FP64 work.
#include "fv_tile64.cuh"
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

namespace fv {

namespace {

using SingleTile = Tile<kTileX, kTileY>;
#ifndef FV_STRIP_MIN_ROWS
#define FV_STRIP_MIN_ROWS 4
#endif
constexpr int kMinRowsPerCta = FV_STRIP_MIN_ROWS;  // fewer CTAs than that many rows each on small grids

// Dynamic shared memory is over-allocated by this much and aligned up, so
// that tensor copies land on 128-byte boundaries.
constexpr size_t kSmemAlign = 128;

template <int PLANE, int RS, int KIND, bool WACT>
__global__ void __launch_bounds__(kTileThreads, WACT ? FV_FP64_MIN_CTAS_W : FV_FP64_MIN_CTAS)
stage2d_fp64(const Grid G, const Fields uin, const Fields u0, const Fields uout, StepCtrl* __restrict__ ctrl,
             const Fields hout, long long units, const __grid_constant__ TmaState tin, int use_tma, const Fields qin,
             const Fields qout, const __grid_constant__ TmaState tq, int use_tq) {
  extern __shared__ __align__(128) unsigned char smem_bytes[];
  __shared__ unsigned long long s_red[kTileThreads / 32];
  __shared__ __align__(8) unsigned long long s_mbar;
  const unsigned sa = smem_u32(smem_bytes);
  double* smem = reinterpret_cast<double*>(smem_bytes + (((sa + kSmemAlign - 1) & ~(unsigned)(kSmemAlign - 1)) - sa));
  pdl_wait();
  if (use_tma || use_tq) {
    if (threadIdx.x == 0) {
      mbar_init(&s_mbar, 1);
      fence_mbar_init();
    }
    __syncthreads();
  }
  // the primitive copy of uin, when the last stage that wrote uin left one
  const bool prims = qin.f[0] != nullptr && ctrl->q_valid != 0;
  const Fields* qi = prims ? &qin : nullptr;
  const Fields* qo = qout.f[0] ? &qout : nullptr;
  const TmaState* tp = prims ? (use_tq ? &tq : nullptr) : (use_tma ? &tin : nullptr);
  const Fields* ho = hout.f[0] ? &hout : nullptr;
  const long long ub = units * blockIdx.x / gridDim.x, ue = units * (blockIdx.x + 1) / gridDim.x;
  if (G.pow2_all)
    stage_strip64<PLANE, WACT, SingleTile, true>(G, uin, u0, uout, ctrl, RS, KIND, ub, ue, smem, s_red, ho, tp,
                                                 &s_mbar, qi, qo);
  else
    stage_strip64<PLANE, WACT, SingleTile, false>(G, uin, u0, uout, ctrl, RS, KIND, ub, ue, smem, s_red, ho, tp,
                                                  &s_mbar, qi, qo);
  pdl_trigger();
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 1;
  }
  return n;
}

template <int PLANE, int RS, int KIND, bool WACT>
cudaError_t launch_one(const Grid& G, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl, const Fields* hout,
                       const TmaState* tin, const PrimCopy& pc, cudaStream_t st) {
  using SM = TileSmem<double, WACT ? 5 : 4, SingleTile>;
  auto kern = stage2d_fp64<PLANE, RS, KIND, WACT>;
  static bool attr_set = false;  // per instantiation, once per process
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)((WACT ? SM::bytes_vface() : SM::bytes(true)) + kSmemAlign));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  static int resident[3] = {0, 0, 0};  // CTAs per SM: plain / conduction / shared-face viscosity
  const int cfg = WACT && G.visc ? 2 : (G.tc != 0);
  const size_t smem = (cfg == 2 ? SM::bytes_vface() : SM::bytes(cfg == 1)) + kSmemAlign;
  if (!resident[cfg]) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident[cfg], kern, kTileThreads, smem);
    if (e != cudaSuccess) return e;
    if (resident[cfg] < 1) resident[cfg] = 1;
  }
  const long long units = (long long)((G.na + kTileX - 1) / kTileX) * G.nb;
  long long ctas = units / kMinRowsPerCta;
  const long long slots = (long long)resident[cfg] * sm_count();
  if (ctas > slots) ctas = slots;
  if (ctas < 1) ctas = 1;
  const Fields none{};
  static const TmaState no_tma{};
  const cudaError_t e = launch_pdl(kern, dim3((unsigned)ctas), dim3(kTileThreads), smem, st, G, uin, u0, uout, ctrl,
                                   hout ? *hout : none, units, tin ? *tin : no_tma, tin ? 1 : 0,
                                   pc.qin ? *pc.qin : none, pc.qout ? *pc.qout : none, pc.tq ? *pc.tq : no_tma,
                                   pc.tq ? 1 : 0);
  return e != cudaSuccess ? e : cudaGetLastError();
}

template <int PLANE, int RS, bool WACT>
cudaError_t launch_kind(const Grid& G, int kind, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                        const Fields* hout, const TmaState* tin, const PrimCopy& pc, cudaStream_t st) {
  switch (kind) {
    case STAGE_EULER: return launch_one<PLANE, RS, STAGE_EULER, WACT>(G, uin, u0, uout, ctrl, hout, tin, pc, st);
    case STAGE_RK_1: return launch_one<PLANE, RS, STAGE_RK_1, WACT>(G, uin, u0, uout, ctrl, nullptr, tin, pc, st);
    default: return launch_one<PLANE, RS, STAGE_RK_2, WACT>(G, uin, u0, uout, ctrl, hout, tin, pc, st);
  }
}

template <int PLANE, int RS>
cudaError_t launch_w(const Grid& G, int kind, bool wact, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                     const Fields* hout, const TmaState* tin, const PrimCopy& pc, cudaStream_t st) {
  return wact ? launch_kind<PLANE, RS, true>(G, kind, uin, u0, uout, ctrl, hout, tin, pc, st)
              : launch_kind<PLANE, RS, false>(G, kind, uin, u0, uout, ctrl, hout, tin, pc, st);
}

}  // namespace

cudaError_t launch_stage2d(const Grid& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                           Fields uout, StepCtrl* ctrl, cudaStream_t st, const Fields* hout, const TmaState* tin,
                           const PrimCopy* prims) {
  static const PrimCopy no_prims{};
  const PrimCopy& pc = prims ? *prims : no_prims;
  if (G.plane == PLANE_XY)
    return riemann_solver == 0 ? launch_w<PLANE_XY, 0>(G, kind, wact, uin, u0, uout, ctrl, hout, tin, pc, st)
                               : launch_w<PLANE_XY, 1>(G, kind, wact, uin, u0, uout, ctrl, hout, tin, pc, st);
  return riemann_solver == 0 ? launch_w<PLANE_XZ, 0>(G, kind, wact, uin, u0, uout, ctrl, hout, tin, pc, st)
                             : launch_w<PLANE_XZ, 1>(G, kind, wact, uin, u0, uout, ctrl, hout, tin, pc, st);
}

bool encode_tma_state(const Grid& G, const Fields& u, TmaState* tin) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (!encode || G.ndim != 2) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)G.na, (cuuint64_t)G.rows};
  const cuuint64_t strides[1] = {(cuuint64_t)G.pitch * sizeof(double)};  // bytes, a multiple of 128
  const cuuint32_t box[2] = {(cuuint32_t)(kTileX + 4), (cuuint32_t)kTmaRows};
  const cuuint32_t estr[2] = {1, 1};
  for (int v = 0; v < 5; ++v) {
    if (!u.f[v] || (reinterpret_cast<uintptr_t>(u.f[v]) & 15u)) return false;
    if (encode(&tin->m[v], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, u.f[v], dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

}  // namespace fv
