// fv_api.cpp -- extern "C" entry points for one problem (fvgpu_*).
//
// Host-side runtime of the drop-in: owns the device state of one problem,
// orders all work on one CUDA stream, and drives the fused stage kernels.
// The reference's time loop (main.cpp:51-74) runs on the device: a control
// kernel turns the max reduced by the previous step into dt, decides whether
// the step is active (t + epsilon < tend), and the stage kernels follow;
// fvgpu_advance replays a captured CUDA graph of several such steps and only
// reads the control block back between replays.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "fv3d_gb300.h"
#include "fv_kernels.h"

using fv::Fields;
using fv::Grid;
using fv::StepCtrl;

namespace {

constexpr int kGraphSteps = 8;     // steps per captured graph replay
constexpr int kMaxTotalsBlocks = 1024;

enum KernelClass { KC_STAGE = 0, KC_DT = 1, KC_CONV = 2 };

}  // namespace

struct fv_sim {
  fv_params p{};
  Grid G{};
  bool wact = false;          // third momentum component carried
  int deg_bc = FV_BC_PERIODIC;  // boundary of the one-cell axis (2-D kernels)
  int refl_deg = 0;             // bit a: axis a has one cell and reflects
  double* d_kappa_z = nullptr;  // B02 face conductivities per z layer
  double* buf = nullptr;      // 3 (4 with Q) states x 5 fields x fstride doubles
  Fields A{}, B{}, S{};       // A: state, B: U* / ping-pong, S: scratch
  Fields Q{};                 // RK2: primitives of A, written by stage 2, read by stage 1
  bool q_dirty = false;       // work that may set ctrl->q_valid was enqueued since it was last cleared
  fv::TmaState tma[3];        // TMA descriptors of A, B and Q (2-D plane kernels)
  bool tma_ok = false;
  int cur = 0;                // Euler ping-pong: state in A (0) or B (1)
  StepCtrl* d_ctrl = nullptr;
  StepCtrl* h_ctrl = nullptr; // pinned mirror (read after synchronisation only)
  double* d_partial = nullptr;
  double* h_partial = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  long long step = 0;         // mirror of ctrl->step
  bool slot_valid = false;    // ctrl->slot[step & 1] reduces the current state
  bool state_set = false;
  double inv_tc = 0.0, inv_visc = 0.0;
  std::string err;
  long launches = 0;
  bool profile = false;
  long prof_count[3] = {0, 0, 0};
  double prof_ms[3] = {0, 0, 0};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraphExec_t graph = nullptr;
  const void* graph_key = nullptr;
  cudaStream_t graph_stream = nullptr;
  fv_batch* mixed = nullptr;  // FP32-mixed form: the problem is a batch of one
};

namespace fv {
const char* batch_error(const fv_batch* b);
int batch_compute_dt(fv_batch* b, int i, double* dt, double inv[3]);
int batch_step_dt(fv_batch* b, double dt);
int batch_advance(fv_batch* b, double tend, long max_steps, double* t, long* nsteps);
int batch_totals(fv_batch* b, int i, double out[5]);
}  // namespace fv

namespace {

int Fail(fv_sim* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  return code;
}

#define CUDA_TRY(s, call)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return Fail((s), FV_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
  } while (0)

// computeKappa (ThermalConduction.h:8-21) of the B02 profile at height z.
// Host arithmetic is compiled without contraction, so this rounds as the
// reference's CPU build does.
double KappaB02(const fv_params& p, double z) {
  const double tr = (std::tanh((z - p.b02_zmid) / p.b02_thickness) + 1.0) * 0.5;
  return p.kappa * (p.b02_kappa1 * (1.0 - tr) + p.b02_kappa2 * tr);
}

bool B02(const fv_params& p) { return p.thermal_conductivity_active && p.thermal_conductivity_mode == FV_TCM_B02; }

// The constant TC / viscous terms of ComputeDt.h:36-47, maximised over the
// domain.  The reference passes cell indices as coordinates to computeKappa
// (ComputeDt.h:39), so with B02 the term depends on the padded index k only.
void DtConstants(const fv_params& p, double* inv_tc, double* inv_visc) {
  *inv_tc = p.epsilon;
  if (p.thermal_conductivity_active) {
    auto term = [&](double kap) {
      return std::fmax(std::fmax(2.0 * kap / (p.dx * p.dx), 2.0 * kap / (p.dy * p.dy)), 2.0 * kap / (p.dz * p.dz));
    };
    if (B02(p)) {
      double m = -HUGE_VAL;
      for (int k = p.Ng; k < p.Ng + p.Nz; ++k) m = std::fmax(m, term(KappaB02(p, (double)k)));
      *inv_tc = m;
    } else {
      *inv_tc = term(p.kappa);
    }
  }
  *inv_visc = p.epsilon;
  if (p.viscosity_active)
    *inv_visc = std::fmax(std::fmax(2.0 * p.mu / (p.dx * p.dx), 2.0 * p.mu / (p.dy * p.dy)),
                          2.0 * p.mu / (p.dz * p.dz));
}

// Face conductivities per interior z layer for B02 (ThermalConduction.h:45-50
// with getPos, SimInfo.h:163-167): in-plane faces, face below, face above.
std::vector<double> KappaTable(const fv_params& p) {
  std::vector<double> t(3 * (size_t)p.Nz);
  for (int k = 0; k < p.Nz; ++k) {
    const double z = p.zmin + ((double)k + 0.5) * p.dz;
    const double kc = KappaB02(p, z);
    t[3 * k] = 0.5 * (kc + kc);
    t[3 * k + 1] = 0.5 * (kc + KappaB02(p, z - p.dz));
    t[3 * k + 2] = 0.5 * (kc + KappaB02(p, z + p.dz));
  }
  return t;
}

int DevBC(int bc) { return bc == FV_BC_ABSORBING ? fv::DBC_ABSORBING : bc == FV_BC_REFLECTING ? fv::DBC_REFLECTING : fv::DBC_PERIODIC; }

// True when d > 0 is an exact power of two, so 1/d is exact too.
bool PowerOfTwo(double d) {
  int e;
  return d > 0.0 && std::isfinite(d) && std::frexp(d, &e) == 0.5 && e > -1021 && e < 1022;
}

// Reciprocals and flags the kernels use to replace divisions by the cell
// sizes and by gamma - 1 with operations that round identically.
void SetExactConstants(Grid& G) {
  G.inv_dx = 1.0 / G.dx;
  G.inv_dy = 1.0 / G.dy;
  G.inv_dz = 1.0 / G.dz;
  G.pow2_x = PowerOfTwo(G.dx);
  G.pow2_y = PowerOfTwo(G.dy);
  G.pow2_z = PowerOfTwo(G.dz);
  G.pow2_all = G.pow2_x && G.pow2_y && G.pow2_z;
  G.gm1 = G.gamma - 1.0;
  G.inv_gm1 = 1.0 / G.gm1;
  G.gamma_f = (float)G.gamma;
  G.gm1_f = (float)G.gm1;
  G.inv_gm1_f = (float)G.inv_gm1;
  G.g_f = (float)G.g;
  G.kappa_f = (float)G.kappa;
  G.mu_f = (float)G.mu;
  G.g_dz_f = (float)(G.g * G.dz);
  G.dx_f = (float)G.dx;
  G.dy_f = (float)G.dy;
  G.dz_f = (float)G.dz;
  G.inv_dx_f = (float)G.inv_dx;
  G.inv_dy_f = (float)G.inv_dy;
  G.inv_dz_f = (float)G.inv_dz;
}

// Checks that the parameter set is one this build runs and fills the grid.
// 2-D runs without z-boundary physics use the plane kernels; everything else
// (true 3-D grids, gravity in the x-y plane, the well-balanced / C91 z
// boundaries, B02 conductivity, fixed-temperature / gradient conduction
// boundaries) uses the 3-D kernel.
int Configure(fv_sim* s) {
  const fv_params& p = s->p;
  if (p.Nx < 1 || p.Ny < 1 || p.Nz < 1) return Fail(s, FV_ERR_PARAM, "Nx, Ny, Nz must be >= 1");
  if (p.Ng < 2) return Fail(s, FV_ERR_PARAM, "Nghosts must be >= 2 (slopes read two cells out)");
  if (!(p.dx > 0 && p.dy > 0 && p.dz > 0)) return Fail(s, FV_ERR_PARAM, "cell sizes must be positive");
  if (!(p.gamma0 > 1.0)) return Fail(s, FV_ERR_PARAM, "gamma0 must be > 1");
  if (p.precision != FV_PREC_FP64) return Fail(s, FV_ERR_UNSUPPORTED, "unknown precision");
  if (p.thermal_conductivity_active && p.thermal_conductivity_mode != FV_TCM_CONSTANT && !B02(p))
    return Fail(s, FV_ERR_UNSUPPORTED, "unknown thermal conductivity mode");
  const bool tc_z = p.thermal_conductivity_active && (B02(p) || p.bctc_zmin != FV_BCTC_NONE ||
                                                      p.bctc_zmax != FV_BCTC_NONE);
  // corrected physics runs on the 3-D kernel only (its viscous and HLLC forms)
  const bool z_physics = p.well_balanced_flux_at_z_bc || p.boundary_z == FV_BC_C91 || tc_z ||
                         p.physics == FV_PHYS_CORRECTED;
  Grid& G = s->G;
  G = Grid{};
  int plane = -1;
  if (!z_physics && !p.gravity && p.Nz == 1 && p.Ny >= 2 && p.Nx >= 2) {
    plane = fv::PLANE_XY;
    s->deg_bc = p.boundary_z;
  } else if (!z_physics && p.Ny == 1 && p.Nz >= 2 && p.Nx >= 2) {
    plane = fv::PLANE_XZ;
    s->deg_bc = p.boundary_y;
  }
  // One-cell reflecting axes: the reference's outer ghost layer there is a
  // stale copy of the previous stage, harmless only while the velocity along
  // the axis is zero and no viscous stencil reads it.
  const int n_ax[3] = {p.Nx, p.Ny, p.Nz};
  const int bc_ax[3] = {p.boundary_x, p.boundary_y, p.boundary_z};
  s->refl_deg = 0;
  for (int a = 0; a < 3; ++a)
    if (n_ax[a] == 1 && bc_ax[a] == FV_BC_REFLECTING) s->refl_deg |= 1 << a;
  if (p.viscosity_active && s->refl_deg)
    return Fail(s, FV_ERR_UNSUPPORTED, "viscosity with a reflecting one-cell axis is not built");
  G.rows = 0;
  if (plane >= 0) {
    G.ndim = 2;
    G.plane = plane;
    G.na = p.Nx;
    G.nb = plane == fv::PLANE_XY ? p.Ny : p.Nz;
    G.nc = 1;
    G.bc_a = DevBC(p.boundary_x);
    G.bc_b = DevBC(plane == fv::PLANE_XY ? p.boundary_y : p.boundary_z);
    G.bc_c = DevBC(s->deg_bc);
    G.da = p.dx;
    G.db = plane == fv::PLANE_XY ? p.dy : p.dz;
    G.dc = plane == fv::PLANE_XY ? p.dz : p.dy;
  } else {
    if (p.boundary_z == FV_BC_C91 && p.Nz < 2)
      return Fail(s, FV_ERR_UNSUPPORTED, "the C91 z boundary needs Nz >= 2 (its mirror cell)");
    G.ndim = 3;
    G.plane = fv::PLANE_XY;  // storage order rho, m_x, m_y, m_z, E
    G.na = p.Nx;
    G.nb = p.Ny;
    G.nc = p.Nz;
    G.bc_a = DevBC(p.boundary_x);
    G.bc_b = DevBC(p.boundary_y);
    G.bc_c = p.boundary_z == FV_BC_C91 ? fv::DBC_C91 : DevBC(p.boundary_z);
    G.da = p.dx;
    G.db = p.dy;
    G.dc = p.dz;
  }
  G.rows = G.nb * G.nc;
  G.pitch = (G.na + 15) / 16 * 16;  // 128-byte rows
  G.fstride = ((long long)G.pitch * G.rows + 31) / 32 * 32;
  G.recon = p.reconstruction;
  G.gravity = p.gravity ? 1 : 0;
  G.tc = p.thermal_conductivity_active ? 1 : 0;
  G.visc = p.viscosity_active ? 1 : 0;
  G.dx = p.dx;
  G.dy = p.dy;
  G.dz = p.dz;
  G.gamma = p.gamma0;
  G.g = p.g;
  G.kappa = p.kappa;
  G.mu = p.mu;
  G.wb_flux_z = p.well_balanced_flux_at_z_bc ? 1 : 0;
  G.corrected = p.physics == FV_PHYS_CORRECTED ? 1 : 0;
  G.gravity_flag = p.gravity ? 1 : 0;
  G.bctc_zmin = p.thermal_conductivity_active ? p.bctc_zmin : FV_BCTC_NONE;
  G.bctc_zmax = p.thermal_conductivity_active ? p.bctc_zmax : FV_BCTC_NONE;
  G.bctc_zmin_value = p.bctc_zmin_value;
  G.bctc_zmax_value = p.bctc_zmax_value;
  G.zmin = p.zmin;
  G.theta1 = p.theta1;
  G.zmin_f = (float)p.zmin;
  G.theta1_f = (float)p.theta1;
  G.bctc_zmin_value_f = (float)p.bctc_zmin_value;
  G.bctc_zmax_value_f = (float)p.bctc_zmax_value;
  G.kappa_z = nullptr;  // B02 table: set by fvgpu_create
  SetExactConstants(G);
  DtConstants(p, &s->inv_tc, &s->inv_visc);
  return FV_OK;
}

// The FP32-mixed handle forwards to its batch of one; a failure's message is
// copied to the handle.
int Mixed(fv_sim* s, int rc) {
  if (rc != FV_OK) s->err = fv::batch_error(s->mixed);
  return rc;
}

Fields StateAt(double* base, long long fstride) {
  Fields f;
  for (int v = 0; v < 5; ++v) f.f[v] = base + v * fstride;
  return f;
}

// Storage slot of each reference field (rho, u|mx, v|my, w|mz, p|E).
void StorageOrder(int plane, int slot_of[5]) {
  slot_of[0] = 0;
  slot_of[1] = 1;
  slot_of[2] = plane == fv::PLANE_XY ? 2 : 3;
  slot_of[3] = plane == fv::PLANE_XY ? 3 : 2;
  slot_of[4] = 4;
}

const Fields& Current(const fv_sim* s) { return s->cur == 0 ? s->A : s->B; }

struct Timed {
  fv_sim* s;
  int cls;
  Timed(fv_sim* s_, int cls_) : s(s_), cls(cls_) {
    if (s->profile) cudaEventRecord(s->ev0, s->stream);
  }
  void done() {
    s->launches += 1;
    if (s->profile) {
      cudaEventRecord(s->ev1, s->stream);
      cudaEventSynchronize(s->ev1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, s->ev0, s->ev1);
      s->prof_ms[cls] += ms;
      s->prof_count[cls] += 1;
    }
  }
};

enum StepMode { STEP_LOOP = -1, STEP_GIVEN_DT = 0, STEP_FIXED = 2 };

// Launches the kernels of one time step (control + stages) on the stream.
// STEP_GIVEN_DT uses the host-supplied dt; STEP_LOOP derives dt from the CFL
// reduction and stops at the loop bound; STEP_FIXED derives dt with no bound.
// The TMA descriptors of state u, when the stage kernel can use them.
const fv::TmaState* TmaOf(const fv_sim* s, const Fields& u) {
  if (!s->tma_ok) return nullptr;
  if (u.f[0] == s->A.f[0]) return &s->tma[0];
  if (u.f[0] == s->B.f[0]) return &s->tma[1];
  return nullptr;
}

// Marks the primitive copy Q stale (stream-ordered): called whenever the
// host replaces the state.
int DropPrims(fv_sim* s) {
  if (s->Q.f[0] && s->q_dirty) CUDA_TRY(s, cudaMemsetAsync(&s->d_ctrl->q_valid, 0, sizeof(int), s->stream));
  s->q_dirty = false;
  return FV_OK;
}

int EnqueueStep(fv_sim* s, int mode, double dt, bool counting = true, const Fields* hout = nullptr) {
  {
    Timed t(s, KC_DT);
    cudaError_t e = fv::launch_control(s->d_ctrl, 1, mode, dt, s->stream);
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "control launch: %s", cudaGetErrorString(e));
    if (counting) t.done();
  }
  const int rs = s->p.riemann_solver == FV_HLL ? 0 : 1;
  if (s->p.time_stepping == FV_TS_RK2) {
    fv::PrimCopy read_q, write_q;
    if (s->Q.f[0]) {
      read_q.qin = &s->Q;
      read_q.tq = s->tma_ok ? &s->tma[2] : nullptr;
      write_q.qout = &s->Q;
      s->q_dirty = true;
    }
    {
      Timed t(s, KC_STAGE);
      cudaError_t e = fv::launch_stage(s->G, rs, fv::STAGE_RK_1, s->wact, s->A, s->A, s->B, s->d_ctrl, s->stream,
                                       nullptr, TmaOf(s, s->A), &read_q);
      if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "stage 1 launch: %s", cudaGetErrorString(e));
      if (counting) t.done();
    }
    {
      Timed t(s, KC_STAGE);
      cudaError_t e =
          fv::launch_stage(s->G, rs, fv::STAGE_RK_2, s->wact, s->B, s->A, s->A, s->d_ctrl, s->stream, hout,
                           TmaOf(s, s->B), &write_q);
      if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "stage 2 launch: %s", cudaGetErrorString(e));
      if (counting) t.done();
    }
  } else {
    Timed t(s, KC_STAGE);
    const Fields& in = Current(s);
    const Fields& out = s->cur == 0 ? s->B : s->A;
    cudaError_t e =
        fv::launch_stage(s->G, rs, fv::STAGE_EULER, s->wact, in, in, out, s->d_ctrl, s->stream, hout, TmaOf(s, in));
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "euler stage launch: %s", cudaGetErrorString(e));
    if (counting) t.done();
    s->cur ^= 1;
  }
  return FV_OK;
}

int KernelsPerStep(const fv_sim* s) { return s->p.time_stepping == FV_TS_RK2 ? 3 : 2; }

// Writes fields of the control block from the host (stream-ordered).
int SetCtrl(fv_sim* s, const StepCtrl& c) {
  CUDA_TRY(s, cudaMemcpyAsync(s->d_ctrl, &c, sizeof(StepCtrl), cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return FV_OK;
}

// The status of a non-zero sticky error flag of the control block.
int CtrlError(fv_sim* s, const char* what) {
  if (s->h_ctrl->err & 2) return Fail(s, FV_ERR_TIMEOUT, "%s: a staged tile load did not complete in time", what);
  return Fail(s, FV_ERR_NONFINITE, "%s: non-finite state or dt", what);
}

int ReadCtrl(fv_sim* s) {
  CUDA_TRY(s, cudaMemcpyAsync(s->h_ctrl, s->d_ctrl, sizeof(StepCtrl), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return FV_OK;
}

// Makes ctrl->slot[step & 1] hold max inv_dt_hyp of the current state.
int EnsureSlot(fv_sim* s) {
  if (s->slot_valid) return FV_OK;
  const int slot = (int)(s->step & 1);
  CUDA_TRY(s, cudaMemsetAsync(&s->d_ctrl->slot[slot], 0, sizeof(unsigned long long), s->stream));
  Timed t(s, KC_DT);
  cudaError_t e = fv::launch_reduce2d(s->G, s->wact, Current(s), s->d_ctrl, slot, s->stream);
  if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "dt reduction launch: %s", cudaGetErrorString(e));
  t.done();
  s->slot_valid = true;
  return FV_OK;
}

void ResetGraph(fv_sim* s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  s->graph_key = nullptr;
}

int CopyIn(fv_sim* s, const Fields& dst, const double* const src[5], bool zero_missing) {
  const size_t rowb = (size_t)s->G.na * sizeof(double);
  for (int v = 0; v < 5; ++v) {
    if (src[v]) {
      CUDA_TRY(s, cudaMemcpy2DAsync(dst.f[v], (size_t)s->G.pitch * sizeof(double), src[v], rowb, rowb, s->G.rows,
                                    cudaMemcpyHostToDevice, s->stream));
    } else if (zero_missing) {
      CUDA_TRY(s, cudaMemsetAsync(dst.f[v], 0, (size_t)s->G.fstride * sizeof(double), s->stream));
    }
  }
  return FV_OK;
}

int CopyOut(fv_sim* s, const Fields& src, double* const dst[5]) {
  const size_t rowb = (size_t)s->G.na * sizeof(double);
  for (int v = 0; v < 5; ++v) {
    if (!dst[v]) continue;
    CUDA_TRY(s, cudaMemcpy2DAsync(dst[v], rowb, src.f[v], (size_t)s->G.pitch * sizeof(double), rowb, s->G.rows,
                                  cudaMemcpyDeviceToHost, s->stream));
  }
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return FV_OK;
}

bool AnyNonzero(const double* a, long long n) {
  if (!a) return false;
  for (long long i = 0; i < n; ++i)
    if (a[i] != 0.0) return true;
  return false;
}

// A pointer the GPU can dereference for p (device, managed or pinned host
// memory, or ordinary host memory where the device reads pageable memory),
// or null.  *host tells whether the CPU may read it.
const double* DeviceView(const double* p, bool* host) {
  *host = false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    a.type = cudaMemoryTypeUnregistered;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return (const double*)a.devicePointer;
  *host = true;
  if (a.type == cudaMemoryTypeHost) return (const double*)a.devicePointer;
  int dev = 0, pageable = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess)
    return nullptr;
  return pageable ? p : nullptr;
}

int SetState(fv_sim* s, const double* const ref_fields[5], bool prim) {
  if (!s) return FV_ERR_PARAM;
  int slot_of[5];
  StorageOrder(s->G.plane, slot_of);
  const double* src[5];
  for (int v = 0; v < 5; ++v) src[slot_of[v]] = ref_fields[v];
  if (!src[0] || !src[4]) return Fail(s, FV_ERR_PARAM, "density and pressure/energy arrays are required");
  const long long ncell = (long long)s->G.na * s->G.rows;
  if (s->G.ndim == 3) {
    s->wact = true;
    for (int a = 0; a < 3; ++a)
      if ((s->refl_deg >> a & 1) && AnyNonzero(src[1 + a], ncell))
        return Fail(s, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting one-cell axis is not built");
  } else {
    s->wact = s->p.viscosity_active || AnyNonzero(src[3], ncell);
    if (s->wact && s->deg_bc == FV_BC_REFLECTING)
      return Fail(s, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting degenerate axis is not built");
  }
  ResetGraph(s);
  s->cur = 0;
  int rc = DropPrims(s);
  if (rc) return rc;
  rc = CopyIn(s, s->A, src, true);
  if (rc) return rc;
  if (prim) {
    Timed t(s, KC_CONV);
    cudaError_t e = fv::launch_prim_to_cons2d(s->G, s->A, s->stream);
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "primToCons launch: %s", cudaGetErrorString(e));
    t.done();
  }
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  s->slot_valid = false;
  s->state_set = true;
  return FV_OK;
}

}  // namespace

namespace fv {

// The parameter checks and grid set-up of fvgpu_create, without allocating:
// fills G and the constant CFL terms, or returns a status with a message.
int configure_grid(const fv_params& p, Grid* G, double* inv_tc, double* inv_visc, int* deg_bc,
                   std::string* err) {
  fv_sim s;
  s.p = p;
  const int rc = Configure(&s);
  if (err) *err = s.err;
  if (rc != FV_OK) return rc;
  *G = s.G;
  *inv_tc = s.inv_tc;
  *inv_visc = s.inv_visc;
  *deg_bc = s.deg_bc;
  return FV_OK;
}

}  // namespace fv

extern "C" {

int fvgpu_create(const fv_params* params, fv_sim** out) {
  if (!params || !out) return FV_ERR_PARAM;
  *out = nullptr;
  fv_sim* s = new fv_sim();
  s->p = *params;
  if (params->precision == FV_PREC_FP32_MIXED) {
    // the FP32-mixed form runs through the batch machinery (2-D or 3-D)
    *out = s;
    const int rc = fvgpu_batch_create(params, 1, &s->mixed);
    if (rc != FV_OK) {
      s->err = fv::batch_error(s->mixed);
      fvgpu_batch_destroy(s->mixed);
      s->mixed = nullptr;
    }
    return rc;
  }
  int rc = Configure(s);
  if (rc != FV_OK) {
    // keep the handle so the caller can read the message, but mark it unusable
    *out = s;
    s->state_set = false;
    s->buf = nullptr;
    return rc;
  }
  const bool with_q = s->p.time_stepping == FV_TS_RK2;
  const size_t bytes = (size_t)(with_q ? 4 : 3) * 5 * s->G.fstride * sizeof(double);
  if (cudaMalloc(&s->buf, bytes) != cudaSuccess) {
    *out = s;
    return Fail(s, FV_ERR_NOMEM, "cudaMalloc of %zu bytes failed", bytes);
  }
  // Every initialisation below is ordered on the handle's own (non-blocking)
  // stream and waited for before returning: a legacy-stream cudaMemset or
  // pageable cudaMemcpy is not ordered with non-blocking streams and could
  // land after the first state upload while other work keeps the GPU busy.
  if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    *out = s;
    return Fail(s, FV_ERR_CUDA, "stream creation failed");
  }
  s->stream = s->own_stream;
  if (cudaMemsetAsync(s->buf, 0, bytes, s->own_stream) != cudaSuccess) {
    *out = s;
    return Fail(s, FV_ERR_CUDA, "state initialisation failed");
  }
  if (B02(s->p)) {
    const std::vector<double> table = KappaTable(s->p);
    if (cudaMalloc(&s->d_kappa_z, table.size() * sizeof(double)) != cudaSuccess ||
        cudaMemcpyAsync(s->d_kappa_z, table.data(), table.size() * sizeof(double), cudaMemcpyHostToDevice,
                        s->own_stream) != cudaSuccess ||
        cudaStreamSynchronize(s->own_stream) != cudaSuccess) {
      *out = s;
      return Fail(s, FV_ERR_NOMEM, "conductivity table allocation failed");
    }
    s->G.kappa_z = s->d_kappa_z;
  }
  s->A = StateAt(s->buf, s->G.fstride);
  s->B = StateAt(s->buf + 5 * s->G.fstride, s->G.fstride);
  s->S = StateAt(s->buf + 10 * s->G.fstride, s->G.fstride);
  if (with_q) s->Q = StateAt(s->buf + 15 * s->G.fstride, s->G.fstride);
  s->tma_ok = s->G.ndim == 2 && fv::encode_tma_state(s->G, s->A, &s->tma[0]) &&
              fv::encode_tma_state(s->G, s->B, &s->tma[1]) &&
              (!with_q || fv::encode_tma_state(s->G, s->Q, &s->tma[2]));
  if (cudaMalloc(&s->d_ctrl, sizeof(StepCtrl)) != cudaSuccess ||
      cudaMallocHost(&s->h_ctrl, sizeof(StepCtrl)) != cudaSuccess ||
      cudaMalloc(&s->d_partial, kMaxTotalsBlocks * 10 * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&s->h_partial, kMaxTotalsBlocks * 10 * sizeof(double)) != cudaSuccess) {
    *out = s;
    return Fail(s, FV_ERR_NOMEM, "control block allocation failed");
  }
  if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
    *out = s;
    return Fail(s, FV_ERR_CUDA, "event creation failed");
  }
  StepCtrl c{};
  c.cfl = s->p.CFL;
  c.inv_tc = s->inv_tc;
  c.inv_visc = s->inv_visc;
  c.epsilon = s->p.epsilon;
  c.mode = 1;
  rc = SetCtrl(s, c);
  *out = s;
  return rc;
}

int fvgpu_destroy(fv_sim* s) {
  if (!s) return FV_OK;
  if (s->mixed) fvgpu_batch_destroy(s->mixed);
  if (s->stream) cudaStreamSynchronize(s->stream);
  ResetGraph(s);
  if (s->buf) cudaFree(s->buf);
  if (s->d_kappa_z) cudaFree(s->d_kappa_z);
  if (s->d_ctrl) cudaFree(s->d_ctrl);
  if (s->h_ctrl) cudaFreeHost(s->h_ctrl);
  if (s->d_partial) cudaFree(s->d_partial);
  if (s->h_partial) cudaFreeHost(s->h_partial);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return FV_OK;
}

const char* fvgpu_last_error(const fv_sim* s) { return s ? s->err.c_str() : "null handle"; }

int fvgpu_set_prim(fv_sim* s, const double* rho, const double* u, const double* v, const double* w,
                   const double* p) {
  if (s && s->mixed) return Mixed(s, fvgpu_batch_set_prim(s->mixed, 0, rho, u, v, w, p));
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  const double* f[5] = {rho, u, v, w, p};
  return SetState(s, f, true);
}

int fvgpu_init_problem(fv_sim* s) {
  if (s && s->mixed) return Mixed(s, fvgpu_batch_init_problem(s->mixed, 0));
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  fv::InitSpec spec;
  if (fv::make_init_spec(s->p, &spec) != FV_OK)
    return Fail(s, FV_ERR_PARAM, "unknown problem '%.63s' (Init.h: sod_x, sod_y, sod_z, blast, rayleigh-taylor, "
                "diffusion, H84, C91)", s->p.problem);
  int slot_of[5];
  StorageOrder(s->G.plane, slot_of);
  Fields out;
  for (int v = 0; v < 5; ++v) out.f[v] = s->A.f[slot_of[v]];
  ResetGraph(s);
  s->cur = 0;
  s->state_set = false;
  int rc = DropPrims(s);
  if (rc) return rc;
  int* d_flags = reinterpret_cast<int*>(s->d_partial);
  int* h_flags = reinterpret_cast<int*>(s->h_partial);
  CUDA_TRY(s, cudaMemsetAsync(d_flags, 0, sizeof(int), s->stream));
  cudaError_t e = fv::launch_generate(spec, out, s->G.pitch, d_flags, s->stream);
  if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "generator launch: %s", cudaGetErrorString(e));
  CUDA_TRY(s, cudaMemcpyAsync(h_flags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  const int flags = *h_flags;
  // the checks set_prim makes on the velocities, from the generator's flags
  if (s->G.ndim == 3) {
    s->wact = true;
    for (int a = 0; a < 3; ++a)
      if ((s->refl_deg >> a & 1) && (flags >> (1 + a) & 1))
        return Fail(s, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting one-cell axis is not built");
  } else {
    const int out_of_plane = s->G.plane == fv::PLANE_XY ? 3 : 2;  // w, or v of an x-z run
    s->wact = s->p.viscosity_active || (flags >> out_of_plane & 1);
    if (s->wact && s->deg_bc == FV_BC_REFLECTING)
      return Fail(s, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting degenerate axis is not built");
  }
  {
    Timed t(s, KC_CONV);
    e = fv::launch_prim_to_cons2d(s->G, s->A, s->stream);
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "primToCons launch: %s", cudaGetErrorString(e));
    t.done();
  }
  s->launches += 1;  // the generator
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  s->slot_valid = false;
  s->state_set = true;
  return FV_OK;
}

int fvgpu_generate(const fv_params* p, double* rho, double* u, double* v, double* w, double* pr) {
  if (!p || p->Nx < 1 || p->Ny < 1 || p->Nz < 1) return FV_ERR_PARAM;
  fv::InitSpec spec;
  if (fv::make_init_spec(*p, &spec) != FV_OK) return FV_ERR_PARAM;
  const size_t n = (size_t)p->Nx * p->Ny * p->Nz;
  double* dst[5] = {rho, u, v, w, pr};
  double* d = nullptr;
  cudaStream_t st = nullptr;
  int rc = FV_OK;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return FV_ERR_CUDA;
  if (cudaMallocAsync(&d, 5 * n * sizeof(double) + 256, st) != cudaSuccess) {
    cudaStreamDestroy(st);
    return FV_ERR_NOMEM;
  }
  Fields out;
  for (int k = 0; k < 5; ++k) out.f[k] = d + (size_t)k * n;
  int* flags = reinterpret_cast<int*>(d + 5 * n);
  // the caller's arrays: any memory (device, pinned or pageable host)
  if (cudaMemsetAsync(flags, 0, sizeof(int), st) != cudaSuccess ||
      fv::launch_generate(spec, out, p->Nx, flags, st) != cudaSuccess)
    rc = FV_ERR_CUDA;
  for (int k = 0; k < 5 && rc == FV_OK; ++k)
    if (dst[k] && cudaMemcpyAsync(dst[k], out.f[k], n * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess)
      rc = FV_ERR_CUDA;
  if (cudaFreeAsync(d, st) != cudaSuccess) rc = FV_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) rc = FV_ERR_CUDA;
  cudaStreamDestroy(st);
  return rc;
}

int fvgpu_set_cons(fv_sim* s, const double* rho, const double* mx, const double* my, const double* mz,
                   const double* E) {
  if (s && s->mixed)
    return Fail(s, FV_ERR_UNSUPPORTED, "the FP32-mixed handle takes primitive states (fvgpu_set_prim)");
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  const double* f[5] = {rho, mx, my, mz, E};
  return SetState(s, f, false);
}

int fvgpu_get_prim(fv_sim* s, double* rho, double* u, double* v, double* w, double* p) {
  if (s && s->mixed) return Mixed(s, fvgpu_batch_get_prim(s->mixed, 0, rho, u, v, w, p));
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  int slot_of[5];
  StorageOrder(s->G.plane, slot_of);
  double* ref[5] = {rho, u, v, w, p};
  double* dst[5];
  for (int k = 0; k < 5; ++k) dst[slot_of[k]] = ref[k];
  {
    Timed t(s, KC_CONV);
    cudaError_t e = fv::launch_cons_to_prim2d(s->G, Current(s), s->S, s->stream);
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "consToPrim launch: %s", cudaGetErrorString(e));
    t.done();
  }
  if (!s->wact) {
    CUDA_TRY(s, cudaMemsetAsync(s->S.f[3], 0, (size_t)s->G.fstride * sizeof(double), s->stream));
  }
  return CopyOut(s, s->S, dst);
}

int fvgpu_get_cons(fv_sim* s, double* rho, double* mx, double* my, double* mz, double* E) {
  if (s && s->mixed)
    return Fail(s, FV_ERR_UNSUPPORTED, "the FP32-mixed handle returns primitive states (fvgpu_get_prim)");
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  int slot_of[5];
  StorageOrder(s->G.plane, slot_of);
  double* ref[5] = {rho, mx, my, mz, E};
  double* dst[5];
  for (int k = 0; k < 5; ++k) dst[slot_of[k]] = ref[k];
  if (!s->wact) {
    // the third momentum is identically zero and not stored by the stages
    if (dst[3]) std::memset(dst[3], 0, sizeof(double) * (size_t)s->G.na * s->G.rows);
    dst[3] = nullptr;
  }
  return CopyOut(s, Current(s), dst);
}

int fvgpu_step_host(fv_sim* s, const double* const prim_in[5], double dt, double* const prim_out[5],
                    double* dt_used) {
  if (s && s->mixed) {  // staged copies through the batch calls
    if (!prim_in) return Fail(s, FV_ERR_PARAM, "null argument");
    int rc = Mixed(s, fvgpu_batch_set_prim(s->mixed, 0, prim_in[0], prim_in[1], prim_in[2], prim_in[3], prim_in[4]));
    if (rc) return rc;
    double d = dt;
    if (!(dt > 0.0)) {
      rc = Mixed(s, fv::batch_compute_dt(s->mixed, 0, &d, nullptr));
      if (rc) return rc;
    }
    rc = Mixed(s, fv::batch_step_dt(s->mixed, d));
    if (rc) return rc;
    if (dt_used) *dt_used = d;
    if (!prim_out) return Mixed(s, fvgpu_batch_synchronize(s->mixed));
    return Mixed(s, fvgpu_batch_get_prim(s->mixed, 0, prim_out[0], prim_out[1], prim_out[2], prim_out[3],
                                         prim_out[4]));
  }
  if (!s || !s->buf || !prim_in) return s ? Fail(s, FV_ERR_PARAM, "null argument or unconfigured handle")
                                          : FV_ERR_PARAM;
  int slot_of[5];
  StorageOrder(s->G.plane, slot_of);
  Fields src{}, hout{};
  bool host_in[5] = {false, false, false, false, false};
  for (int k = 0; k < 5; ++k) {
    const int v = slot_of[k];
    if (prim_in[k]) {
      src.f[v] = (double*)DeviceView(prim_in[k], &host_in[v]);
      if (!src.f[v]) return Fail(s, FV_ERR_PARAM, "input array %d is not addressable by the GPU", k);
    }
    if (prim_out && prim_out[k]) {
      bool h;
      hout.f[v] = (double*)DeviceView(prim_out[k], &h);
      if (!hout.f[v]) return Fail(s, FV_ERR_PARAM, "output array %d is not addressable by the GPU", k);
    }
  }
  if (!src.f[0] || !src.f[4]) return Fail(s, FV_ERR_PARAM, "density and pressure arrays are required");
  const long long ncell = (long long)s->G.na * s->G.rows;
  // the same checks as set_prim; arrays only the GPU can read are not scanned
  if (s->G.ndim == 3) {
    s->wact = true;
    for (int a = 0; a < 3; ++a)
      if ((s->refl_deg >> a & 1) && src.f[1 + a] &&
          (!host_in[1 + a] || AnyNonzero(prim_in[1 + a], ncell)))
        return Fail(s, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting one-cell axis is not built");
  } else {
    const double* c = prim_in[slot_of[3]];
    s->wact = s->p.viscosity_active || (c && (!host_in[3] || AnyNonzero(c, ncell)));
    if (s->wact && s->deg_bc == FV_BC_REFLECTING)
      return Fail(s, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting degenerate axis is not built");
  }
  s->cur = 0;
  const bool cfl = !(dt > 0.0);
  const int slot = (int)(s->step & 1);
  if (cfl) CUDA_TRY(s, cudaMemsetAsync(&s->d_ctrl->slot[slot], 0, sizeof(unsigned long long), s->stream));
  {
    // the conversion also writes the primitive copy of the new state (the
    // consToPrim its CFL maximum computes) and marks it valid
    Timed t(s, KC_CONV);
    const bool keep_q = s->Q.f[0] != nullptr;
    cudaError_t e = fv::launch_prim_to_cons_from(s->G, s->wact, src, s->A, cfl ? s->d_ctrl : nullptr, slot,
                                                 s->stream, keep_q ? &s->Q : nullptr,
                                                 keep_q ? &s->d_ctrl->q_valid : nullptr);
    if (keep_q) s->q_dirty = true;
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "primToCons launch: %s", cudaGetErrorString(e));
    t.done();
  }
  s->state_set = true;
  int rc = EnqueueStep(s, cfl ? STEP_FIXED : STEP_GIVEN_DT, dt, true, prim_out ? &hout : nullptr);
  if (rc) return rc;
  s->step += 1;
  s->slot_valid = true;
  rc = ReadCtrl(s);
  if (rc) return rc;
  if (dt_used) *dt_used = s->h_ctrl->dt_cur;
  if (s->h_ctrl->err) return CtrlError(s, "step_host");
  return FV_OK;
}

int fvgpu_compute_dt(fv_sim* s, double* dt, double inv[3]) {
  if (s && s->mixed) return Mixed(s, fv::batch_compute_dt(s->mixed, 0, dt, inv));
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  int rc = EnsureSlot(s);
  if (rc) return rc;
  rc = ReadCtrl(s);
  if (rc) return rc;
  const double inv_hyp = [&] {
    double d;
    unsigned long long b = s->h_ctrl->slot[s->step & 1];
    std::memcpy(&d, &b, sizeof(d));
    return d;
  }();
  double m = inv_hyp;
  if (s->inv_tc > m) m = s->inv_tc;
  if (s->inv_visc > m) m = s->inv_visc;
  const double d = s->p.CFL / m;
  if (inv) {
    inv[0] = inv_hyp;
    inv[1] = s->inv_tc;
    inv[2] = s->inv_visc;
  }
  if (dt) *dt = d;
  if (s->h_ctrl->err) return CtrlError(s, "compute_dt");
  if (!std::isfinite(d)) return Fail(s, FV_ERR_NONFINITE, "non-finite state or dt (dt = %g)", d);
  return FV_OK;
}

int fvgpu_step(fv_sim* s, double dt) {
  if (s && s->mixed) return Mixed(s, fv::batch_step_dt(s->mixed, dt));
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  // stream-ordered and asynchronous: the control kernel takes dt as an argument
  int rc = EnqueueStep(s, STEP_GIVEN_DT, dt);
  if (rc) return rc;
  s->step += 1;
  s->slot_valid = true;
  return FV_OK;
}

int fvgpu_enqueue_steps(fv_sim* s, long nsteps) {
  if (s && s->mixed) return Mixed(s, fvgpu_batch_run(s->mixed, nsteps));
  if (!s || !s->buf) return s ? Fail(s, FV_ERR_STATE, "handle not configured") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  if (nsteps < 0) return Fail(s, FV_ERR_PARAM, "nsteps must be >= 0");
  int rc = EnsureSlot(s);
  if (rc) return rc;
  for (long k = 0; k < nsteps; ++k) {
    rc = EnqueueStep(s, STEP_FIXED, 0.0);
    if (rc) return rc;
  }
  s->step += nsteps;
  s->slot_valid = true;
  return FV_OK;
}

int fvgpu_advance(fv_sim* s, double tend, long max_steps, double* t, long* nsteps) {
  if (s && s->mixed && t) return Mixed(s, fv::batch_advance(s->mixed, tend, max_steps, t, nsteps));
  if (!s || !s->buf || !t) return s ? Fail(s, FV_ERR_PARAM, "null argument") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  int rc = EnsureSlot(s);
  if (rc) return rc;
  rc = ReadCtrl(s);
  if (rc) return rc;
  StepCtrl c = *s->h_ctrl;
  const long long step0 = c.step;
  c.mode = 1;
  c.t = *t;
  c.tend = tend;
  c.max_steps = max_steps > 0 ? step0 + max_steps : 0;
  c.cfl = s->p.CFL;
  c.inv_tc = s->inv_tc;
  c.inv_visc = s->inv_visc;
  c.epsilon = s->p.epsilon;
  rc = SetCtrl(s, c);
  if (rc) return rc;

  // Short fixed-step runs are launched directly; longer ones replay a graph.
  const bool use_graph = !s->profile && !(max_steps > 0 && max_steps < kGraphSteps);
  for (;;) {
    if (use_graph) {
      const void* key = (const void*)Current(s).f[0];
      if (!s->graph || s->graph_key != key || s->graph_stream != s->stream) {
        ResetGraph(s);
        const int cur0 = s->cur;
        cudaGraph_t g;
        CUDA_TRY(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kGraphSteps; ++k) {
          rc = EnqueueStep(s, STEP_LOOP, 0.0, false);
          if (rc) {
            cudaStreamEndCapture(s->stream, &g);
            return rc;
          }
        }
        CUDA_TRY(s, cudaStreamEndCapture(s->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        s->cur = cur0;  // capture only recorded the launches
        s->graph_key = key;
        s->graph_stream = s->stream;
      }
      s->q_dirty = true;
      CUDA_TRY(s, cudaGraphLaunch(s->graph, s->stream));
      s->launches += (long)kGraphSteps * KernelsPerStep(s);
      if (s->p.time_stepping != FV_TS_RK2 && (kGraphSteps & 1)) s->cur ^= 1;
    } else {
      const bool short_run = max_steps > 0 && max_steps < kGraphSteps;
      const int n = short_run ? (int)max_steps : kGraphSteps;
      for (int k = 0; k < n; ++k) {
        rc = EnqueueStep(s, STEP_LOOP, 0.0);
        if (rc) return rc;
      }
      if (short_run) {
        rc = ReadCtrl(s);
        if (rc) return rc;
        break;
      }
    }
    rc = ReadCtrl(s);
    if (rc) return rc;
    if (s->h_ctrl->err) break;
    if (!s->h_ctrl->active) break;
  }
  // Euler ping-pong: inactive steps copy the state through, so the buffer
  // holding it alternates exactly with the launched step count.
  s->step = s->h_ctrl->step;
  s->slot_valid = true;
  *t = s->h_ctrl->t;
  if (nsteps) *nsteps = (long)(s->h_ctrl->step - step0);
  if (s->h_ctrl->err) return CtrlError(s, "advance");
  return FV_OK;
}

int fvgpu_conserved_totals(fv_sim* s, double out[5]) {
  if (s && s->mixed && out) return Mixed(s, fv::batch_totals(s->mixed, 0, out));
  if (!s || !s->buf || !out) return s ? Fail(s, FV_ERR_PARAM, "null argument") : FV_ERR_PARAM;
  if (!s->state_set) return Fail(s, FV_ERR_STATE, "no state set");
  int nb = 0;
  {
    Timed t(s, KC_CONV);
    cudaError_t e = fv::launch_totals2d(s->G, Current(s), s->d_partial, kMaxTotalsBlocks, &nb, s->stream);
    if (e != cudaSuccess) return Fail(s, FV_ERR_CUDA, "totals launch: %s", cudaGetErrorString(e));
    t.done();
  }
  CUDA_TRY(s, cudaMemcpyAsync(s->h_partial, s->d_partial, (size_t)nb * 10 * sizeof(double), cudaMemcpyDeviceToHost,
                              s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  int slot_of[5];
  StorageOrder(s->G.plane, slot_of);
  for (int k = 0; k < 5; ++k) {
    const int v = slot_of[k];
    double S = 0.0, C = 0.0;
    for (int b = 0; b < nb; ++b) {
      const double x = s->h_partial[(b * 5 + v) * 2];
      const double tt = S + x;
      if (std::fabs(S) >= std::fabs(x)) C += (S - tt) + x;
      else C += (x - tt) + S;
      S = tt;
      C += s->h_partial[(b * 5 + v) * 2 + 1];
    }
    out[k] = (v == 3 && !s->wact) ? 0.0 : S + C;
  }
  return FV_OK;
}

int fvgpu_set_stream(fv_sim* s, void* stream) {
  if (s && s->mixed) return Mixed(s, fvgpu_batch_set_stream(s->mixed, stream));
  if (!s) return FV_ERR_PARAM;
  if (s->stream) cudaStreamSynchronize(s->stream);
  s->stream = stream ? (cudaStream_t)stream : s->own_stream;
  ResetGraph(s);
  return FV_OK;
}

int fvgpu_synchronize(fv_sim* s) {
  if (s && s->mixed) return Mixed(s, fvgpu_batch_synchronize(s->mixed));
  if (!s) return FV_ERR_PARAM;
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return FV_OK;
}

int fvgpu_launch_count(const fv_sim* s, long* count) {
  if (s && s->mixed) return fvgpu_batch_launch_count(s->mixed, count);
  if (!s || !count) return FV_ERR_PARAM;
  *count = s->launches;
  return FV_OK;
}

int fvgpu_profile_enable(fv_sim* s, int enable) {
  if (s && s->mixed && enable)
    return Fail(s, FV_ERR_UNSUPPORTED, "per-kernel timing is not built for the FP32-mixed handle");
  if (!s) return FV_ERR_PARAM;
  if (s->stream) cudaStreamSynchronize(s->stream);
  s->profile = enable != 0;
  for (int k = 0; k < 3; ++k) {
    s->prof_count[k] = 0;
    s->prof_ms[k] = 0.0;
  }
  return FV_OK;
}

int fvgpu_kernel_times(fv_sim* s, long counts[3], double ms[3]) {
  if (!s) return FV_ERR_PARAM;
  for (int k = 0; k < 3; ++k) {
    if (counts) counts[k] = s->prof_count[k];
    if (ms) ms[k] = s->prof_ms[k];
  }
  return FV_OK;
}

}  // extern "C"
