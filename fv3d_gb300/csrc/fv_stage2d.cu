// fv_stage2d.cu -- the FP64 fused stage kernel of one 2-D problem: one CTA
// per 32x16 tile, body in fv_tile64.cuh (compiled without FMA contraction, so
// it rounds exactly like the reference).
#include "fv_tile64.cuh"

namespace fv {

namespace {

using SingleTile = Tile<kTileX, kTileY>;

template <int PLANE, int RS, int KIND, bool WACT>
__global__ void __launch_bounds__(kTileThreads, WACT ? FV_FP64_MIN_CTAS_W : FV_FP64_MIN_CTAS)
stage2d_fp64(const Grid G, const Fields uin, const Fields u0, const Fields uout, StepCtrl* __restrict__ ctrl,
             const Fields hout) {
  extern __shared__ double smem_raw[];
  __shared__ unsigned long long s_red[kTileThreads / 32];
  const Fields* ho = hout.f[0] ? &hout : nullptr;
  if (G.pow2_all)
    stage_tile64<PLANE, WACT, SingleTile, true>(G, uin, u0, uout, ctrl, RS, KIND, blockIdx.x, blockIdx.y, smem_raw,
                                                s_red, ho);
  else
    stage_tile64<PLANE, WACT, SingleTile, false>(G, uin, u0, uout, ctrl, RS, KIND, blockIdx.x, blockIdx.y, smem_raw,
                                                 s_red, ho);
}

template <int PLANE, int RS, int KIND, bool WACT>
cudaError_t launch_one(const Grid& G, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl, const Fields* hout,
                       cudaStream_t st) {
  using SM = TileSmem<double, WACT ? 5 : 4, SingleTile>;
  auto kern = stage2d_fp64<PLANE, RS, KIND, WACT>;
  static bool attr_set = false;  // per instantiation, once per process
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM::bytes(true));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid((G.na + kTileX - 1) / kTileX, (G.nb + kTileY - 1) / kTileY);
  const Fields none{};
  kern<<<grid, kTileThreads, SM::bytes(G.tc != 0), st>>>(G, uin, u0, uout, ctrl, hout ? *hout : none);
  return cudaGetLastError();
}

template <int PLANE, int RS, bool WACT>
cudaError_t launch_kind(const Grid& G, int kind, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                        const Fields* hout, cudaStream_t st) {
  switch (kind) {
    case STAGE_EULER: return launch_one<PLANE, RS, STAGE_EULER, WACT>(G, uin, u0, uout, ctrl, hout, st);
    case STAGE_RK_1: return launch_one<PLANE, RS, STAGE_RK_1, WACT>(G, uin, u0, uout, ctrl, nullptr, st);
    default: return launch_one<PLANE, RS, STAGE_RK_2, WACT>(G, uin, u0, uout, ctrl, hout, st);
  }
}

template <int PLANE, int RS>
cudaError_t launch_w(const Grid& G, int kind, bool wact, Fields uin, Fields u0, Fields uout, StepCtrl* ctrl,
                     const Fields* hout, cudaStream_t st) {
  return wact ? launch_kind<PLANE, RS, true>(G, kind, uin, u0, uout, ctrl, hout, st)
              : launch_kind<PLANE, RS, false>(G, kind, uin, u0, uout, ctrl, hout, st);
}

}  // namespace

cudaError_t launch_stage2d(const Grid& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                           Fields uout, StepCtrl* ctrl, cudaStream_t st, const Fields* hout) {
  if (G.plane == PLANE_XY)
    return riemann_solver == 0 ? launch_w<PLANE_XY, 0>(G, kind, wact, uin, u0, uout, ctrl, hout, st)
                               : launch_w<PLANE_XY, 1>(G, kind, wact, uin, u0, uout, ctrl, hout, st);
  return riemann_solver == 0 ? launch_w<PLANE_XZ, 0>(G, kind, wact, uin, u0, uout, ctrl, hout, st)
                             : launch_w<PLANE_XZ, 1>(G, kind, wact, uin, u0, uout, ctrl, hout, st);
}

}  // namespace fv
