// fv_stage2d.cu -- the FP64 fused stage kernel of one 2-D problem: 32-wide
// strips of cells marched in blocks of 32x16 cells (stage_strip64 in
// fv_tile64.cuh, compiled without FMA contraction, so it rounds exactly like
// the reference).  The strip rows are split evenly over as many CTAs as the
// GPU holds at once, so every SM gets the same FP64 work.
#include "fv_tile64.cuh"

namespace fv {

namespace {

using SingleTile = Tile<kTileX, kTileY>;
constexpr int kMinRowsPerCta = 4;

template <int PLANE, int RS, int KIND, bool WACT>
__global__ void __launch_bounds__(kTileThreads, WACT ? FV_FP64_MIN_CTAS_W : FV_FP64_MIN_CTAS)
stage2d_fp64(const Grid G, const Fields uin, const Fields u0, const Fields uout, StepCtrl* __restrict__ ctrl,
             const Fields hout, long long units) {
  extern __shared__ double smem_raw[];
  __shared__ unsigned long long s_red[kTileThreads / 32];
  const Fields* ho = hout.f[0] ? &hout : nullptr;
  const long long ub = units * blockIdx.x / gridDim.x, ue = units * (blockIdx.x + 1) / gridDim.x;
  if (G.pow2_all)
    stage_strip64<PLANE, WACT, SingleTile, true>(G, uin, u0, uout, ctrl, RS, KIND, ub, ue, smem_raw, s_red, ho);
  else
    stage_strip64<PLANE, WACT, SingleTile, false>(G, uin, u0, uout, ctrl, RS, KIND, ub, ue, smem_raw, s_red, ho);
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
                       cudaStream_t st) {
  using SM = TileSmem<double, WACT ? 5 : 4, SingleTile>;
  auto kern = stage2d_fp64<PLANE, RS, KIND, WACT>;
  static bool attr_set = false;  // per instantiation, once per process
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(WACT ? SM::bytes_vface() : SM::bytes(true)));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  static int resident[3] = {0, 0, 0};  // CTAs per SM: plain / conduction / shared-face viscosity
  const int cfg = WACT && G.visc ? 2 : (G.tc != 0);
  const size_t smem = cfg == 2 ? SM::bytes_vface() : SM::bytes(cfg == 1);
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
  kern<<<(unsigned)ctas, kTileThreads, smem, st>>>(G, uin, u0, uout, ctrl, hout ? *hout : none, units);
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
