// fv_init.cu -- the reference's problem generators (Init.h:18-209, the
// InitFunctor of Init.h:228-279) on the GPU.
//
// One thread per interior cell writes the primitive state (rho, u, v, w, p)
// of the generator named by fv_params.problem, with the reference's cell
// positions (getPos, SimInfo.h:162-167) and its operation order, every
// product and sum rounded separately (no fused multiply-add), so that the
// piecewise-constant generators (sod_x/y/z, blast, diffusion) give the
// reference's bits and the others differ only by the last-place rounding of
// cos / pow.  H84 and C91 draw their perturbations from a counter-based
// stream instead of Kokkos' XorShift64 pool, whose draws depend on which
// thread visits which cell: cell c = (k * Ny + j) * Nx + i takes
// splitmix64(key + golden * (c + 1)) >> 11 scaled to [0, 1), with key =
// splitmix64(seed + golden * (stream + 1)) and stream 31 (H84) / 32 (C91).
//
// The output arrays are addressed as [row][pitch] with row = k * Ny + j,
// which covers both the callers' unpadded [Nz][Ny][Nx] arrays (pitch = Nx)
// and the padded storage of a handle or batch (2-D planes have Ny or Nz = 1,
// so the row index is the storage row there too).
#include <cmath>
#include <cstring>

#include "fv3d_gb300.h"
#include "fv_kernels.h"

namespace fv {

namespace {

constexpr unsigned long long kGolden = 0x9E3779B97F4A7C15ull;

__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double stream_uniform(unsigned long long key, unsigned long long c) {
  return __dmul_rn((double)(mix64(key + kGolden * (c + 1ull)) >> 11), 1.0 / 9007199254740992.0);
}

__global__ void __launch_bounds__(256) generate_kernel(const InitSpec S, const Fields out, int pitch, int* flags) {
  const long long n = (long long)S.nx * S.rows;
  unsigned bits = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int row = (int)(c / S.nx), i = (int)(c - (long long)row * S.nx);
    const int k = row / S.ny, j = row - k * S.ny;
    // getPos: min + (index + 0.5) * d
    const double x = __dadd_rn(S.xmin, __dmul_rn(__dadd_rn((double)i, 0.5), S.dx));
    const double y = __dadd_rn(S.ymin, __dmul_rn(__dadd_rn((double)j, 0.5), S.dy));
    const double z = __dadd_rn(S.zmin, __dmul_rn(__dadd_rn((double)k, 0.5), S.dz));
    double q[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    switch (S.kind) {
      case INIT_SOD_X:
      case INIT_SOD_Y:
      case INIT_SOD_Z: {  // Init.h:18-64
        const double d = S.kind == INIT_SOD_X ? x : (S.kind == INIT_SOD_Y ? y : z);
        q[0] = d <= 0.5 ? 1.0 : 0.125;
        q[4] = d <= 0.5 ? 1.0 : 0.1;
        break;
      }
      case INIT_BLAST: {  // Init.h:69-98: r from (mid - pos)
        const double xr = __dadd_rn(S.xmid, -x), yr = __dadd_rn(S.ymid, -y), zr = __dadd_rn(S.zmid, -z);
        const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(xr, xr), __dmul_rn(yr, yr)), __dmul_rn(zr, zr)));
        q[0] = r < 0.2 ? 1.0 : 1.2;
        q[4] = r < 0.2 ? 10.0 : 0.1;
        break;
      }
      case INIT_DIFFUSION: {  // Init.h:153-177: r from (pos - mid)
        const double x0 = __dadd_rn(x, -S.xmid), y0 = __dadd_rn(y, -S.ymid), z0 = __dadd_rn(z, -S.zmid);
        const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x0, x0), __dmul_rn(y0, y0)), __dmul_rn(z0, z0)));
        q[0] = r < 0.2 ? 1.0 : 0.1;
        q[1] = q[2] = q[3] = 1.0;
        q[4] = 1.0;
        break;
      }
      case INIT_RT: {  // Init.h:182-206: P0 + (0.1 g) z, w in the band |z| < 1/3
        q[0] = z < S.zmid ? 1.0 : 2.0;
        q[4] = __dadd_rn(2.5, __dmul_rn(S.c0, z));
        if (z > -1.0 / 3.0 && z < 1.0 / 3.0) {
          const double a = __dadd_rn(1.0, cos(__dmul_rn(S.c1, x)));
          const double b = __dadd_rn(1.0, cos(__dmul_rn(S.c1, y)));
          const double e = __dadd_rn(1.0, cos(__dmul_rn(S.c2, z)));
          q[3] = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(0.01, a), b), e), 4.0);
        }
        break;
      }
      case INIT_H84: {  // Init.h:103-122
        q[0] = pow(z, S.m1);
        q[4] = pow(z, __dadd_rn(S.m1, 1.0));
        q[3] = __dmul_rn(S.pert, __dadd_rn(stream_uniform(S.key, (unsigned long long)c), -0.5));
        break;
      }
      default: {  // INIT_C91, Init.h:127-148
        const double T = __dadd_rn(1.0, __dmul_rn(S.c0, z));
        q[0] = pow(T, S.m1);
        const double prs = pow(T, __dadd_rn(S.m1, 1.0));
        const double pert = __dmul_rn(S.pert, __dadd_rn(stream_uniform(S.key, (unsigned long long)c), -0.5));
        q[4] = __dmul_rn(prs, __dadd_rn(1.0, pert));
        break;
      }
    }
    const long long o = (long long)row * pitch + i;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      out.f[v][o] = q[v];
      if (q[v] != 0.0) bits |= 1u << v;
    }
  }
  bits = __reduce_or_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && bits) atomicOr(flags, (int)bits);
}

}  // namespace

int make_init_spec(const fv_params& p, InitSpec* S) {
  static const struct {
    const char* name;
    int kind;
  } kNames[] = {{"sod_x", INIT_SOD_X},   {"sod_y", INIT_SOD_Y},          {"sod_z", INIT_SOD_Z},
                {"blast", INIT_BLAST},   {"rayleigh-taylor", INIT_RT},   {"diffusion", INIT_DIFFUSION},
                {"H84", INIT_H84},       {"C91", INIT_C91}};
  std::memset(S, 0, sizeof(*S));
  S->kind = -1;
  for (const auto& e : kNames)
    if (std::strncmp(p.problem, e.name, sizeof(p.problem)) == 0) S->kind = e.kind;
  if (S->kind < 0) return FV_ERR_PARAM;
  S->nx = p.Nx;
  S->ny = p.Ny;
  S->rows = p.Ny * p.Nz;
  S->xmin = p.xmin;
  S->ymin = p.ymin;
  S->zmin = p.zmin;
  S->dx = p.dx;
  S->dy = p.dy;
  S->dz = p.dz;
  S->xmid = 0.5 * (p.xmin + p.xmax);
  S->ymid = 0.5 * (p.ymin + p.ymax);
  S->zmid = 0.5 * (p.zmin + p.zmax);
  S->m1 = p.m1;
  S->c1 = 4.0 * M_PI;  // the cos arguments of Init.h:205: (4 pi) x, (4 pi) y, (3 pi) z
  S->c2 = 3.0 * M_PI;
  if (S->kind == INIT_RT) S->c0 = 0.1 * p.g;
  if (S->kind == INIT_C91) S->c0 = p.theta1;
  const bool h84 = S->kind == INIT_H84;
  S->pert = h84 ? p.h84_pert : p.c91_pert;
  S->key = mix64((unsigned long long)(long long)p.seed + kGolden * (h84 ? 32ull : 33ull));
  return FV_OK;
}

cudaError_t launch_generate(const InitSpec& S, const Fields& out, int pitch, int* flags, cudaStream_t st) {
  const long long n = (long long)S.nx * S.rows;
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 255) / 256;
  const int grid = (int)(blocks < 152LL * 16 ? blocks : 152LL * 16);
  generate_kernel<<<grid, 256, 0, st>>>(S, out, pitch, flags);
  return cudaGetLastError();
}

}  // namespace fv
