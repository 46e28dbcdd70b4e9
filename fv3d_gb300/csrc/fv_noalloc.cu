// fv_noalloc.cu -- fvgpu_step_noalloc: one time step of a 2-D or 3-D
// problem on device arrays the caller owns, without allocating any memory.
//
// Why it exists: some host codes cannot call cudaMalloc from their time loop.
// An application whose device memory belongs to another allocator (a memory
// pool or arena that has already reserved the GPU's memory) must not grow its
// footprint behind that allocator's back, and a latency-critical loop cannot
// afford the implicit device synchronisation of cudaMalloc/cudaFree.  The
// regular handle (fvgpu_create) allocates its buffers once; this entry point
// needs no handle and allocates nothing: the stage kernels' scratch -- the
// intermediate RK2 state U* and the control block holding dt and the CFL
// reduction -- lives in one fixed array in device memory, declared below.
//
// Limits and sharing:
//   - kScratchBytes (32 MiB) bounds the problem: 5 fields x pitch x rows
//     x 8 bytes plus 256 bytes of control block must fit, e.g. 786,432 cells
//     (512 x 1536) at pitch 512.  Larger problems are rejected with
//     FV_ERR_PARAM and a message; they need the regular handle.
//   - The array exists once per device and stays allocated until the process
//     exits.  With lazy module loading (CUDA_MODULE_LOADING=LAZY, the default
//     since CUDA 12.2) it is reserved on a device when this file's kernels are
//     first used there; with CUDA_MODULE_LOADING=EAGER every process that
//     loads the library reserves the 32 MiB on each device where it creates a
//     context, whether it calls this entry point or not.
//   - Every call uses the same array and leaves the last call's contents in
//     it; calls whose work overlaps on the GPU (other streams, other host
//     threads) race on it.  The control block is rewritten at the start of
//     every call except its error flag; U* is fully written by the first
//     stage before it is read.
//   - Errors: the error flag (non-finite state, a bounded wait that gave up)
//     is sticky across calls and is read -- then cleared -- only by a call
//     that passes next_dt, which waits for the stream.  A call without
//     next_dt returns once its work is enqueued and reports launch errors
//     only.
//   - The first call on a device looks the array's device address up
//     (cudaGetSymbolAddress, once per device, with that device current); make
//     that first call before any stream capture.  A call with next_dt
//     synchronises its stream and is refused while that stream is capturing.
#include <cmath>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "fv3d_gb300.h"
#include "fv_kernels.h"

namespace fv {
int configure_grid(const fv_params& p, Grid* G, double* inv_tc, double* inv_visc, int* deg_bc,
                   std::string* err);
}

namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;  // 32 MiB per device
constexpr size_t kCtrlBytes = 256;                   // control block, padded
constexpr int kMaxDevices = 64;

// The scratch itself.  In host code this name is only a stand-in for the
// device array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_step_scratch[kScratchBytes];

std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};
bool g_fresh[kMaxDevices] = {};  // the next call on the device is its first

// Writes a fresh control block (all counters, slots and flags zero), except
// the sticky error flag, which is kept unless `first` (the device's first
// call: nothing has written the block yet).
__global__ void init_ctrl_kernel(fv::StepCtrl* ctrl, double cfl, double inv_tc, double inv_visc, double eps,
                                 int first) {
  fv::StepCtrl c;
  memset(&c, 0, sizeof(c));
  c.err = first ? 0 : ctrl->err;
  c.cfl = cfl;
  c.inv_tc = inv_tc;
  c.inv_visc = inv_visc;
  c.epsilon = eps;
  *ctrl = c;
}

int Message(char* buf, size_t len, int code, const char* fmt, ...) __attribute__((format(printf, 4, 5)));
int Message(char* buf, size_t len, int code, const char* fmt, ...) {
  if (buf && len) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, len, fmt, ap);
    va_end(ap);
  }
  return code;
}

// Device address of the scratch array on the current device (set up on the
// first call per device).  *dev_out: the device; *first: no call has yet
// initialised its control block (MarkInitialised clears it).
cudaError_t ScratchAddress(void** out, bool* first, int* dev_out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_step_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = ptr;
    g_fresh[dev] = true;
  }
  *out = g_scratch_addr[dev];
  *first = g_fresh[dev];
  *dev_out = dev;
  return cudaSuccess;
}

void MarkInitialised(int dev) {
  std::lock_guard<std::mutex> lock(g_mutex);
  g_fresh[dev] = false;
}

}  // namespace

extern "C" int fvgpu_step_noalloc(const fv_params* params, double* const fields[5], long pitch, double dt,
                                  double* next_dt, void* stream, char* errbuf, size_t errlen) {
  using fv::Fields;
  using fv::Grid;
  using fv::StepCtrl;
  if (errbuf && errlen) errbuf[0] = '\0';
  if (!params || !fields) return Message(errbuf, errlen, FV_ERR_PARAM, "null params or fields");
  if (!(dt > 0.0) || !std::isfinite(dt))
    return Message(errbuf, errlen, FV_ERR_PARAM, "dt must be positive and finite (got %g): this call has no CFL dt",
                   dt);
  Grid G;
  double inv_tc = 0.0, inv_visc = 0.0;
  int deg_bc = 0;
  std::string err;
  int rc = fv::configure_grid(*params, &G, &inv_tc, &inv_visc, &deg_bc, &err);
  if (rc != FV_OK) return Message(errbuf, errlen, rc, "%s", err.c_str());
  if (pitch < G.na) return Message(errbuf, errlen, FV_ERR_PARAM, "pitch %ld < Nx %d", pitch, G.na);
  // bound pitch before any product with rows can overflow
  const long max_pitch = (long)((kScratchBytes - kCtrlBytes) / (5 * sizeof(double)) / (size_t)G.rows);
  if (pitch > INT_MAX || pitch > max_pitch)
    return Message(errbuf, errlen, FV_ERR_PARAM,
                   "pitch %ld x %d rows does not fit the fixed %zu-byte step scratch (at most pitch %ld); use "
                   "fvgpu_create for larger problems",
                   pitch, G.rows, kScratchBytes, max_pitch);
  const int plane = G.plane;
  // reference order (rho, rho u, rho v, rho w, E) -> storage order (rho, m_a, m_b, m_c, E)
  const int slot_of[5] = {0, 1, plane == fv::PLANE_XY ? 2 : 3, plane == fv::PLANE_XY ? 3 : 2, 4};
  Fields A;
  for (int k = 0; k < 5; ++k) A.f[slot_of[k]] = fields[k];
  if (!A.f[0] || !A.f[1] || !A.f[2] || !A.f[4])
    return Message(errbuf, errlen, FV_ERR_PARAM, "density, energy and in-plane momenta are required");
  const bool wact = A.f[3] != nullptr;
  if (!wact && (params->viscosity_active || G.ndim == 3))
    return Message(errbuf, errlen, FV_ERR_PARAM,
                   G.ndim == 3 ? "a 3-D step needs all five fields"
                               : "viscosity drives the third momentum: pass its array");
  if (G.ndim == 2 && wact && deg_bc == FV_BC_REFLECTING)
    return Message(errbuf, errlen, FV_ERR_UNSUPPORTED,
                   "a third momentum with a reflecting degenerate axis is not built");
  if (G.ndim == 3) {
    // device arrays cannot be checked for a zero velocity along such an axis
    const int n_ax[3] = {params->Nx, params->Ny, params->Nz};
    const int bc_ax[3] = {params->boundary_x, params->boundary_y, params->boundary_z};
    for (int a = 0; a < 3; ++a)
      if (n_ax[a] == 1 && bc_ax[a] == FV_BC_REFLECTING)
        return Message(errbuf, errlen, FV_ERR_UNSUPPORTED, "a reflecting one-cell axis needs fvgpu_create");
    if (params->thermal_conductivity_active && params->thermal_conductivity_mode == FV_TCM_B02)
      return Message(errbuf, errlen, FV_ERR_UNSUPPORTED, "B02 conductivity needs fvgpu_create (a device table)");
  }

  G.pitch = (int)pitch;
  G.fstride = (long long)pitch * G.rows;
  const size_t need = kCtrlBytes + (size_t)5 * (size_t)G.fstride * sizeof(double);
  if (need > kScratchBytes)
    return Message(errbuf, errlen, FV_ERR_PARAM,
                   "problem needs %zu bytes of step scratch, more than the fixed %zu (5 fields x pitch %ld x %d "
                   "rows x 8 B + %zu); use fvgpu_create for larger problems",
                   need, kScratchBytes, pitch, G.rows, kCtrlBytes);

  cudaStream_t st = (cudaStream_t)stream;
  if (next_dt) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(st, &cs);
    if (ce != cudaSuccess)
      return Message(errbuf, errlen, FV_ERR_CUDA, "stream query failed: %s", cudaGetErrorString(ce));
    if (cs != cudaStreamCaptureStatusNone)
      return Message(errbuf, errlen, FV_ERR_PARAM, "next_dt must be NULL while the stream is being captured");
  }

  void* base = nullptr;
  bool first = false;
  int dev = 0;
  cudaError_t e = ScratchAddress(&base, &first, &dev);
  if (e != cudaSuccess)
    return Message(errbuf, errlen, FV_ERR_CUDA, "scratch address lookup failed: %s", cudaGetErrorString(e));
  StepCtrl* ctrl = (StepCtrl*)base;
  double* ustar = (double*)((unsigned char*)base + kCtrlBytes);
  Fields B;
  for (int v = 0; v < 5; ++v) B.f[v] = ustar + (size_t)v * (size_t)G.fstride;

  // control block: fresh every call but for the sticky error flag
  init_ctrl_kernel<<<1, 1, 0, st>>>(ctrl, params->CFL, inv_tc, inv_visc, params->epsilon, first ? 1 : 0);
  e = cudaGetLastError();
  if (e == cudaSuccess && first) MarkInitialised(dev);
  if (e == cudaSuccess) e = fv::launch_control(ctrl, 1, 0, dt, st);
  const int rs = params->riemann_solver == FV_HLL ? 0 : 1;
  if (params->time_stepping == FV_TS_RK2) {
    if (e == cudaSuccess) e = fv::launch_stage(G, rs, fv::STAGE_RK_1, wact, A, A, B, ctrl, st);
    if (e == cudaSuccess) e = fv::launch_stage(G, rs, fv::STAGE_RK_2, wact, B, A, A, ctrl, st);
  } else {
    if (e == cudaSuccess) e = fv::launch_stage(G, rs, fv::STAGE_EULER, wact, A, A, B, ctrl, st);
    for (int v = 0; v < 5 && e == cudaSuccess; ++v) {
      if (v == 3 && !wact) continue;
      e = cudaMemcpy2DAsync(A.f[v], (size_t)pitch * sizeof(double), B.f[v], (size_t)pitch * sizeof(double),
                            (size_t)G.na * sizeof(double), G.rows, cudaMemcpyDeviceToDevice, st);
    }
  }
  if (e != cudaSuccess) return Message(errbuf, errlen, FV_ERR_CUDA, "launch failed: %s", cudaGetErrorString(e));
  if (next_dt) {
    // the last stage reduced max inv_dt_hyp of the new state into slot[1]
    unsigned long long bits = 0;
    int errflag = 0;
    e = cudaMemcpyAsync(&bits, &ctrl->slot[1], sizeof(bits), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&errflag, &ctrl->err, sizeof(errflag), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(&ctrl->err, 0, sizeof(int), st);  // reported: clear
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return Message(errbuf, errlen, FV_ERR_CUDA, "readback failed: %s", cudaGetErrorString(e));
    double inv_hyp;
    std::memcpy(&inv_hyp, &bits, sizeof(inv_hyp));
    double m = inv_hyp;
    if (inv_tc > m) m = inv_tc;
    if (inv_visc > m) m = inv_visc;
    *next_dt = params->CFL / m;
    if (errflag & 2)
      return Message(errbuf, errlen, FV_ERR_TIMEOUT, "a bounded device wait gave up since the last check");
    if (errflag || !(*next_dt > 0.0 && *next_dt <= 1.0e300))
      return Message(errbuf, errlen, FV_ERR_NONFINITE,
                     "non-finite state since the last check, or non-finite dt after the step (dt = %g)", *next_dt);
  }
  return FV_OK;
}
