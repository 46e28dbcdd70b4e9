// Reference harness -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own FP64 hot-path headers, unmodified, from the
// reference tree (SimInfo.h, States.h, Update.h, RiemannSolvers.h,
// BoundaryConditions.h, ThermalConduction.h, Viscosity.h, ComputeDt.h and
// the generators of Init.h) against the Kokkos/INIReader shims in oracle/shim/, and exposes them through
// a small C ABI (fvref_*) that mirrors the product's fvgpu_* calls so tests can
// run both on identical inputs.  Built by oracle/build.py into oracle/_ref/.
//
// Departures from main.cpp, each forced by the reference itself:
//   - IOManager.h is not included (HDF5/HighFive are absent); the caller
//     injects the primitive state Q, or runs the reference's own generators
//     (Init.h, fvref_generate) with the random pool of oracle/shim, whose
//     draws are not Kokkos' (the H84 / C91 perturbations differ).
//   - RK2: UpdateFunctor::update (Update.h:180-206) allocates U0/Ustar with 3
//     extents for a rank-4 View (Update.h:184-185) and cannot run, so
//     fvref_step performs the same sequence (Update.h:187-204) with correctly
//     sized buffers, calling the public euler_step twice.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <iostream>

#include "SimInfo.h"
#include "ComputeDt.h"
#include "Update.h"
#include "Init.h"

#include "fv3d_gb300.h"

using namespace fv3d;

namespace {

struct RefSim {
  Params params;
  Array U, Unew, Q;
  UpdateFunctor* update = nullptr;
  ComputeDtFunctor* cdt = nullptr;
};

void ParamsToC(const Params& p, fv_params* o) {
  std::memset(o, 0, sizeof(*o));
  o->Nx = p.Nx; o->Ny = p.Ny; o->Nz = p.Nz; o->Ng = p.Ng;
  o->xmin = p.xmin; o->xmax = p.xmax; o->ymin = p.ymin; o->ymax = p.ymax;
  o->zmin = p.zmin; o->zmax = p.zmax;
  o->dx = p.dx; o->dy = p.dy; o->dz = p.dz;
  o->save_freq = p.save_freq; o->tend = p.tend;
  o->boundary_x = p.boundary_x; o->boundary_y = p.boundary_y; o->boundary_z = p.boundary_z;
  o->reconstruction = p.reconstruction; o->riemann_solver = p.riemann_solver;
  o->time_stepping = p.time_stepping; o->CFL = p.CFL;
  o->epsilon = p.epsilon; o->gamma0 = p.gamma0;
  o->gravity = p.gravity; o->g = p.g;
  o->well_balanced_flux_at_z_bc = p.well_balanced_flux_at_z_bc;
  o->well_balanced = p.well_balanced;
  o->thermal_conductivity_active = p.thermal_conductivity_active;
  o->thermal_conductivity_mode = p.thermal_conductivity_mode;
  o->kappa = p.kappa;
  o->bctc_zmin = p.bctc_zmin; o->bctc_zmax = p.bctc_zmax;
  o->bctc_zmin_value = p.bctc_zmin_value; o->bctc_zmax_value = p.bctc_zmax_value;
  o->viscosity_active = p.viscosity_active; o->viscosity_mode = p.viscosity_mode; o->mu = p.mu;
  o->m1 = p.m1; o->theta1 = p.theta1; o->m2 = p.m2; o->theta2 = p.theta2;
  o->h84_pert = p.h84_pert; o->c91_pert = p.c91_pert;
  o->seed = p.seed; o->log_frequency = p.log_frequency;
  std::strncpy(o->problem, p.problem.c_str(), sizeof(o->problem) - 1);
  std::strncpy(o->filename_out, p.filename_out.c_str(), sizeof(o->filename_out) - 1);
}

template <class F>
void ForInterior(const Params& p, F f) {
  for (int k = 0; k < p.Nz; ++k)
    for (int j = 0; j < p.Ny; ++j)
      for (int i = 0; i < p.Nx; ++i)
        f(i + p.ibeg, j + p.jbeg, k + p.kbeg, ((size_t)k * p.Ny + j) * p.Nx + i);
}

void RK2Step(RefSim* s, double dt) {
  const Params& p = s->params;
  Array U0("U0", p.Ntz, p.Nty, p.Ntx, Nfields);
  Array Ustar("Ustar", p.Ntz, p.Nty, p.Ntx, Nfields);
  Array Q = s->Q, Unew = s->Unew;
  Kokkos::deep_copy(U0, Unew);
  Kokkos::deep_copy(Ustar, Unew);
  s->update->euler_step(Q, Ustar, dt);
  Kokkos::deep_copy(Unew, Ustar);
  consToPrim(Ustar, Q, p);
  s->update->euler_step(Q, Unew, dt);
  Kokkos::parallel_for("RK2 Correct", p.range_dom, KOKKOS_LAMBDA(const int i, const int j, const int k) {
    for (int ivar = 0; ivar < Nfields; ++ivar)
      Unew(k, j, i, ivar) = 0.5 * (U0(k, j, i, ivar) + Unew(k, j, i, ivar));
  });
}

}  // namespace

extern "C" {

int fvref_read_ini(const char* path, fv_params* out) {
  if (!path || !out) return FV_ERR_PARAM;
  Params p = readInifile(path);
  ParamsToC(p, out);
  return FV_OK;
}

// readInifile never assigns the B02 profile (SimInfo.h:150-154 declare the
// fields without initialisers and no key sets them), so a B02 run needs them
// set on the Params before the functors copy it, as a C++ caller of the
// reference would; fvref_create_b02 does that.
void* fvref_create_b02(const char* ini_path, double zmid, double kappa1, double kappa2, double thickness) {
  RefSim* s = new RefSim();
  s->params = readInifile(ini_path);
  s->params.b02_zmid = zmid;
  s->params.b02_kappa1 = kappa1;
  s->params.b02_kappa2 = kappa2;
  s->params.b02_thickness = thickness;
  const Params& p = s->params;
  s->U = Array("U", p.Ntz, p.Nty, p.Ntx, Nfields);
  s->Unew = Array("Unew", p.Ntz, p.Nty, p.Ntx, Nfields);
  s->Q = Array("Q", p.Ntz, p.Nty, p.Ntx, Nfields);
  s->update = new UpdateFunctor(s->params);
  s->cdt = new ComputeDtFunctor(s->params);
  return s;
}

void* fvref_create(const char* ini_path) {
  RefSim* s = new RefSim();
  s->params = readInifile(ini_path);
  const Params& p = s->params;
  s->U = Array("U", p.Ntz, p.Nty, p.Ntx, Nfields);
  s->Unew = Array("Unew", p.Ntz, p.Nty, p.Ntx, Nfields);
  s->Q = Array("Q", p.Ntz, p.Nty, p.Ntx, Nfields);
  s->update = new UpdateFunctor(s->params);
  s->cdt = new ComputeDtFunctor(s->params);
  return s;
}

void fvref_destroy(void* h) {
  RefSim* s = (RefSim*)h;
  if (!s) return;
  delete s->update;
  delete s->cdt;
  delete s;
}

// Q interior <- fields; ghosts by BoundaryManager; U <- primToCons(Q) over the
// whole array, the order of main.cpp:43-44 / Init.h:275-277.
int fvref_set_prim(void* h, const double* r, const double* u, const double* v, const double* w,
                   const double* pr) {
  RefSim* s = (RefSim*)h;
  const double* f[5] = {r, u, v, w, pr};
  Array Q = s->Q;
  ForInterior(s->params, [&](int i, int j, int k, size_t n) {
    for (int var = 0; var < 5; ++var) Q(k, j, i, var) = f[var] ? f[var][n] : 0.0;
  });
  s->update->bc_manager.fillBoundaries(Q);
  primToCons(s->Q, s->U, s->params);
  return FV_OK;
}

int fvref_get_prim(void* h, double* r, double* u, double* v, double* w, double* pr) {
  RefSim* s = (RefSim*)h;
  consToPrim(s->U, s->Q, s->params);
  double* f[5] = {r, u, v, w, pr};
  Array Q = s->Q;
  ForInterior(s->params, [&](int i, int j, int k, size_t n) {
    for (int var = 0; var < 5; ++var)
      if (f[var]) f[var][n] = Q(k, j, i, var);
  });
  return FV_OK;
}

int fvref_get_cons(void* h, double* r, double* mx, double* my, double* mz, double* E) {
  RefSim* s = (RefSim*)h;
  double* f[5] = {r, mx, my, mz, E};
  Array U = s->U;
  ForInterior(s->params, [&](int i, int j, int k, size_t n) {
    for (int var = 0; var < 5; ++var)
      if (f[var]) f[var][n] = U(k, j, i, var);
  });
  return FV_OK;
}

// main.cpp:55-57: Q = consToPrim(U), then computeDt(Q).
double fvref_compute_dt(void* h) {
  RefSim* s = (RefSim*)h;
  consToPrim(s->U, s->Q, s->params);
  return s->cdt->computeDt(s->Q, s->params.save_freq, 0.0, false);
}

// init.init(Q); primToCons(Q, U) (main.cpp:42-44, Init.h:247-279): the
// reference's generator named by params.problem fills Q, the interior
// primitives are returned as generated.
int fvref_generate(void* h, double* r, double* u, double* v, double* w, double* pr) {
  RefSim* s = (RefSim*)h;
  InitFunctor init(s->params);
  init.init(s->Q);
  primToCons(s->Q, s->U, s->params);
  double* f[5] = {r, u, v, w, pr};
  Array Q = s->Q;
  ForInterior(s->params, [&](int i, int j, int k, size_t n) {
    for (int var = 0; var < 5; ++var)
      if (f[var]) f[var][n] = Q(k, j, i, var);
  });
  return FV_OK;
}

// One pass of the main.cpp:51-74 loop body with a given dt (no I/O).
int fvref_step(void* h, double dt) {
  RefSim* s = (RefSim*)h;
  Kokkos::deep_copy(s->Unew, s->U);
  consToPrim(s->U, s->Q, s->params);
  if (s->params.time_stepping == TS_RK2)
    RK2Step(s, dt);
  else
    s->update->euler_step(s->Q, s->Unew, dt);
  Kokkos::deep_copy(s->U, s->Unew);
  return FV_OK;
}

// The main.cpp:51-74 loop: dt from Q = consToPrim(U) each step, t += dt.
int fvref_advance(void* h, double tend, long max_steps, double* t, long* nsteps) {
  RefSim* s = (RefSim*)h;
  long n = 0;
  double tt = *t;
  while (tt + s->params.epsilon < tend && (max_steps <= 0 || n < max_steps)) {
    const double dt = fvref_compute_dt(h);
    fvref_step(h, dt);
    tt += dt;
    ++n;
  }
  *t = tt;
  if (nsteps) *nsteps = n;
  return FV_OK;
}

// The two Riemann solvers of RiemannSolvers.h on n state pairs (AoS, 5 per state).
int fvref_riemann(int solver, double gamma0, long n, const double* qL, const double* qR, double* flux,
                  double* pout) {
  Params p{};
  p.gamma0 = gamma0;
  for (long c = 0; c < n; ++c) {
    State a, b, f;
    for (int v = 0; v < 5; ++v) { a[v] = qL[5 * c + v]; b[v] = qR[5 * c + v]; }
    double po = 0.0;
    if (solver == HLL)
      hll(a, b, f, po, p);
    else
      hllc(a, b, f, po, p);
    for (int v = 0; v < 5; ++v) flux[5 * c + v] = f[v];
    pout[c] = po;
  }
  return FV_OK;
}

}  // extern "C"
