/*
 * fv3d_oracle.h -- CPU restatement of the reference fv3d hydro step.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the reference results the GPU path is
 * compared with; the product never links, imports or calls it.
 *
 * The API mirrors the product's fvgpu_* calls (same field layout: interior
 * cells, C order [Nz][Ny][Nx]) so a test runs both on identical inputs.
 */
#ifndef FV3D_ORACLE_H
#define FV3D_ORACLE_H

#include "fv3d_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fvora_sim fvora_sim;

fvora_sim* fvora_create(const fv_params* p);
void fvora_destroy(fvora_sim* s);
int fvora_set_prim(fvora_sim* s, const double* r, const double* u, const double* v, const double* w,
                   const double* p);
int fvora_set_cons(fvora_sim* s, const double* r, const double* mx, const double* my, const double* mz,
                   const double* E);
/* The generators of Init.h (InitFunctor::init then primToCons). */
int fvora_generate(fvora_sim* s, double* r, double* u, double* v, double* w, double* p);
int fvora_get_prim(fvora_sim* s, double* r, double* u, double* v, double* w, double* p);
int fvora_get_cons(fvora_sim* s, double* r, double* mx, double* my, double* mz, double* E);
double fvora_compute_dt(fvora_sim* s, double inv[3]);
int fvora_step(fvora_sim* s, double dt);
int fvora_advance(fvora_sim* s, double tend, long max_steps, double* t, long* nsteps);
int fvora_riemann(int solver, double gamma0, long n, const double* qL, const double* qR, double* flux,
                  double* pout);
int fvora_set_threads(int nthreads);
/* readInifile (SimInfo.h:169-306) on .ini text: fv3d_ini.c. */
int fvora_parse_ini(const char* text, fv_params* out);

#ifdef __cplusplus
}
#endif
#endif
