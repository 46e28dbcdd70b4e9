/*
 * fv3d_oracle.c -- CPU restatement of the reference fv3d FP64 hydro step.
 *
 * TEST INFRASTRUCTURE ONLY: the results the GPU path is compared with
 * (tests/, smoke()) and the timed CPU baseline of bench.py ("port").  The product never links
 * or calls this file.
 *
 * It restates, in plain C with OpenMP, the reference's own algorithm with
 * the same data layout (AoS View(Ntz,Nty,Ntx,5) with Ng ghost layers), the
 * same kernel sequence (c2p, ghost fill X->Y->Z, minmod slopes into arrays,
 * two Riemann solves per cell and direction, thermal conduction, viscosity,
 * RK2 correction) and the same floating-point operation order, so that with
 * -ffp-contract=off its results are bit-identical to the reference's headers
 * compiled against the Kokkos shim (checked by tests/test_oracle_golden.py
 * against fixtures generated from that build).  Each function cites the
 * reference lines it follows.
 */
#include "fv3d_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846 /* <cmath>'s value, which the reference uses */
#endif

enum { IR = 0, IU = 1, IV = 2, IW = 3, IP = 4, IE = 4 };
enum { IX = 0, IY = 1, IZ = 2 };

struct fvora_sim {
  fv_params p;
  int Ntx, Nty, Ntz, ibeg, iend, jbeg, jend, kbeg, kend;
  size_t ncell;
  double *U, *Unew, *Q, *sx, *sy, *sz, *U0, *Ustar;
};

#define AT(s, arr, i, j, k) ((arr) + ((((size_t)(k) * (size_t)(s)->Nty + (size_t)(j)) * (size_t)(s)->Ntx + (size_t)(i)) * 5u))

/* A 3-D index range [b0,e0) x [b1,e1) x [b2,e2) over (i,j,k), as the
 * reference's MDRangePolicy<Rank<3>> ranges (SimInfo.h:297-303). */
typedef struct { int b[3], e[3]; } range3;

static range3 range_tot(const fvora_sim* s) { range3 r = {{0, 0, 0}, {s->Ntx, s->Nty, s->Ntz}}; return r; }
static range3 range_dom(const fvora_sim* s) {
  range3 r = {{s->ibeg, s->jbeg, s->kbeg}, {s->iend, s->jend, s->kend}}; return r;
}

/* ---------------- States.h ---------------- */

/* States.h:20-31 */
static void prim_to_cons(const double* q, double* out, double gamma0) {
  double res[5];
  res[IR] = q[IR];
  res[IU] = q[IR] * q[IU];
  res[IV] = q[IR] * q[IV];
  res[IW] = q[IR] * q[IW];
  double Ek = 0.5 * (res[IU] * res[IU] + res[IV] * res[IV] + res[IW] * res[IW]) / q[IR];
  res[IE] = (Ek + q[IP] / (gamma0 - 1.0));
  memcpy(out, res, sizeof(res));
}

/* States.h:34-45 */
static void cons_to_prim(const double* u, double* out, double gamma0) {
  double res[5];
  res[IR] = u[IR];
  res[IU] = u[IU] / u[IR];
  res[IV] = u[IV] / u[IR];
  res[IW] = u[IW] / u[IR];
  double Ek = 0.5 * res[IR] * (res[IU] * res[IU] + res[IV] * res[IV] + res[IW] * res[IW]);
  res[IP] = (u[IE] - Ek) * (gamma0 - 1.0);
  memcpy(out, res, sizeof(res));
}

/* States.h:48-50 */
static double sound_speed(const double* q, double gamma0) { return sqrt(q[IP] * gamma0 / q[IR]); }

/* States.h:104-111 */
static void swap_component(const double* q, int dir, double* out) {
  double r[5] = {q[0], q[1], q[2], q[3], q[4]};
  if (dir == IY) { r[IU] = q[IV]; r[IV] = q[IU]; }
  else if (dir == IZ) { r[IU] = q[IW]; r[IW] = q[IU]; }
  memcpy(out, r, sizeof(r));
}

/* States.h:114-127 */
static void compute_flux(const double* q, double* f, double gamma0) {
  const double Ek = 0.5 * q[IR] * (q[IU] * q[IU] + q[IV] * q[IV] + q[IW] * q[IW]);
  const double E = (q[IP] / (gamma0 - 1.0) + Ek);
  f[0] = q[IR] * q[IU];
  f[1] = q[IR] * q[IU] * q[IU] + q[IP];
  f[2] = q[IR] * q[IU] * q[IV];
  f[3] = q[IR] * q[IU] * q[IW];
  f[4] = (q[IP] + E) * q[IU];
}

/* ---------------- RiemannSolvers.h ---------------- */

/* RiemannSolvers.h:6-36 (HLL, Davis wave speeds) */
static void hll(const double* qL, const double* qR, double* flux, double* pout, double gamma0) {
  const double aL = sound_speed(qL, gamma0);
  const double aR = sound_speed(qR, gamma0);
  const double sminL = qL[IU] - aL;
  const double smaxL = qL[IU] + aL;
  const double sminR = qR[IU] - aR;
  const double smaxR = qR[IU] + aR;
  const double SL = fmin(sminL, sminR);
  const double SR = fmax(smaxL, smaxR);
  double FL[5], FR[5];
  compute_flux(qL, FL, gamma0);
  compute_flux(qR, FR, gamma0);
  if (SL >= 0.0) {
    memcpy(flux, FL, sizeof(FL));
    *pout = qL[IP];
  } else if (SR <= 0.0) {
    memcpy(flux, FR, sizeof(FR));
    *pout = qR[IP];
  } else {
    double uL[5], uR[5];
    prim_to_cons(qL, uL, gamma0);
    prim_to_cons(qR, uR, gamma0);
    *pout = 0.5 * (qL[IP] + qR[IP]);
    const double slsr = SL * SR;
    const double den = SR - SL;
    for (int v = 0; v < 5; ++v) flux[v] = ((FL[v] * SR - FR[v] * SL) + (uR[v] - uL[v]) * slsr) / den;
  }
}

/* RiemannSolvers.h:39-112 (HLLC) */
/* ke3 (corrected physics only): the kinetic energy of all three velocities
 * instead of the reference's IU, IV slots. */
static void hllc(const double* qL, const double* qR, double* flux, double* pout, double gamma0, int ke3) {
  const double rL = qL[IR], uL = qL[IU], vL = qL[IV], pL = qL[IP];
  const double rR = qR[IR], uR = qR[IU], vR = qR[IV], pR = qR[IP];
  const double entho = 1.0 / (gamma0 - 1.0);
  const double ekL = ke3 ? 0.5 * rL * (uL * uL + vL * vL + qL[IW] * qL[IW]) : 0.5 * rL * (uL * uL + vL * vL);
  const double EL = ekL + pL * entho;
  const double ekR = ke3 ? 0.5 * rR * (uR * uR + vR * vR + qR[IW] * qR[IW]) : 0.5 * rR * (uR * uR + vR * vR);
  const double ER = ekR + pR * entho;
  const double cfastL = sound_speed(qL, gamma0);
  const double cfastR = sound_speed(qR, gamma0);
  const double SL = fmin(uL, uR) - fmax(cfastL, cfastR);
  const double SR = fmax(uL, uR) + fmax(cfastL, cfastR);
  const double rcL = rL * (uL - SL);
  const double rcR = rR * (SR - uR);
  const double uS = (rcR * uR + rcL * uL + (pL - pR)) / (rcR + rcL);
  const double pS = (rcR * pL + rcL * pR + rcL * rcR * (uL - uR)) / (rcR + rcL);
  const double rSL = rL * (SL - uL) / (SL - uS);
  const double ESL = ((SL - uL) * EL - pL * uL + pS * uS) / (SL - uS);
  const double rSR = rR * (SR - uR) / (SR - uS);
  const double ESR = ((SR - uR) * ER - pR * uR + pS * uS) / (SR - uS);
  double st[5], E;
  if (SL > 0.0) {
    memcpy(st, qL, sizeof(st));
    E = EL;
    *pout = pL;
  } else if (uS > 0.0) {
    st[IR] = rSL; st[IU] = uS; st[IV] = qL[IV]; st[IW] = qL[IW]; st[IP] = pS;
    E = ESL;
    *pout = pS;
  } else if (SR > 0.0) {
    st[IR] = rSR; st[IU] = uS; st[IV] = qR[IV]; st[IW] = qR[IW]; st[IP] = pS;
    E = ESR;
    *pout = pS;
  } else {
    memcpy(st, qR, sizeof(st));
    E = ER;
    *pout = pR;
  }
  flux[IR] = st[IR] * st[IU];
  flux[IU] = st[IR] * st[IU] * st[IU] + st[IP];
  flux[IV] = flux[IR] * st[IV];
  flux[IW] = flux[IR] * st[IW];
  flux[IE] = (E + st[IP]) * st[IU];
}

static void riemann(const fvora_sim* s, const double* qL, const double* qR, double* flux, double* pout) {
  if (s->p.riemann_solver == FV_HLL)
    hll(qL, qR, flux, pout, s->p.gamma0);
  else
    hllc(qL, qR, flux, pout, s->p.gamma0, s->p.physics == FV_PHYS_CORRECTED);
}

/* ---------------- SimInfo.h array kernels ---------------- */

/* SimInfo.h:313-321 over range_tot */
static void array_cons_to_prim(const fvora_sim* s, const double* U, double* Q) {
  range3 r = range_tot(s);
  const double g0 = s->p.gamma0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = r.b[2]; k < r.e[2]; ++k)
    for (int j = r.b[1]; j < r.e[1]; ++j)
      for (int i = r.b[0]; i < r.e[0]; ++i) cons_to_prim(AT(s, U, i, j, k), AT(s, Q, i, j, k), g0);
}

/* SimInfo.h:323-331 over range_tot */
static void array_prim_to_cons(const fvora_sim* s, const double* Q, double* U) {
  range3 r = range_tot(s);
  const double g0 = s->p.gamma0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = r.b[2]; k < r.e[2]; ++k)
    for (int j = r.b[1]; j < r.e[1]; ++j)
      for (int i = r.b[0]; i < r.e[0]; ++i) prim_to_cons(AT(s, Q, i, j, k), AT(s, U, i, j, k), g0);
}

/* ---------------- BoundaryConditions.h ---------------- */

/* BoundaryConditions.h:22-53 */
static void fill_reflecting(const fvora_sim* s, const double* Q, int i, int j, int k, int iref, int jref,
                            int kref, int dir, double* out) {
  int isym, jsym, ksym;
  if (dir == IX) {
    int ipiv = (i < iref ? s->ibeg : s->iend);
    isym = 2 * ipiv - i - 1; jsym = j; ksym = k;
  } else if (dir == IY) {
    int jpiv = (j < jref ? s->jbeg : s->jend);
    isym = i; jsym = 2 * jpiv - j - 1; ksym = k;
  } else {
    int kpiv = (k < kref ? s->kbeg : s->kend);
    isym = i; jsym = j; ksym = 2 * kpiv - k - 1;
  }
  memcpy(out, AT(s, Q, isym, jsym, ksym), 5 * sizeof(double));
  if (dir == IX) out[IU] *= -1.0;
  else if (dir == IY) out[IV] *= -1.0;
  else out[IW] *= -1.0;
}

/* BoundaryConditions.h:60-81 */
static void fill_periodic(const fvora_sim* s, const double* Q, int i, int j, int k, int dir, double* out) {
  if (dir == IX) { if (i < s->ibeg) i += s->p.Nx; else i -= s->p.Nx; }
  else if (dir == IY) { if (j < s->jbeg) j += s->p.Ny; else j -= s->p.Ny; }
  else { if (k < s->kbeg) k += s->p.Nz; else k -= s->p.Nz; }
  memcpy(out, AT(s, Q, i, j, k), 5 * sizeof(double));
}

/* SimInfo.h:162-167 */
static void get_pos(const fvora_sim* s, int i, int j, int k, double pos[3]) {
  pos[0] = s->p.xmin + (i - s->ibeg + 0.5) * s->p.dx;
  pos[1] = s->p.ymin + (j - s->jbeg + 0.5) * s->p.dy;
  pos[2] = s->p.zmin + (k - s->kbeg + 0.5) * s->p.dz;
}

/* BoundaryConditions.h:87-134 (uses the boolean `gravity` as a number, as written) */
static void fill_c91(const fvora_sim* s, const double* Q, int i, int j, int k, int kref, double* res) {
  int kpiv = (k < kref ? s->kbeg : s->kend);
  int ksym = 2 * kpiv - k - 1;
  double pos[3];
  get_pos(s, i, j, k, pos);
  const double* qref = AT(s, Q, i, j, kref);
  const double* qsym = AT(s, Q, i, j, ksym);
  const double grav = s->p.gravity ? 1.0 : 0.0;
  memset(res, 0, 5 * sizeof(double));
  if (k < s->kbeg) {
    double dz = pos[IZ] - 0.5 * s->p.dz;
    double T = 1.0 + pos[IZ] * s->p.theta1;
    res[IP] = qref[IP] + dz * qref[IR] * grav;
    res[IR] = res[IP] / T;
    res[IP] = fmax(res[IP], 1.0e-6);
    res[IR] = fmax(res[IR], 1.0e-6);
    const double dratio = qsym[IR] / res[IR];
    res[IU] = qsym[IU];
    res[IV] = qsym[IV];
    res[IW] = -qsym[IW] * dratio;
  } else if (k >= s->kend) {
    const double Tref = qref[IP] / qref[IR];
    const double dz = pos[IZ] - (1.0 - 0.5 * s->p.dz);
    const double T = Tref + dz * s->p.theta1;
    const double P = qref[IP] + dz * qref[IR] * grav;
    const double rho = P / T;
    res[IP] = fmax(P, 1.0e-6);
    res[IR] = fmax(rho, 1.0e-6);
    const double dratio = qsym[IR] / rho;
    res[IU] = qsym[IU] * dratio;
    res[IV] = qsym[IV] * dratio;
    res[IW] = -qsym[IW] * dratio;
  }
}

/* BoundaryManager::fillBoundaries, BoundaryConditions.h:146-215: X over
 * (ghost i, interior j,k), then Y over (all i, ghost j, interior k), then Z
 * over (all i,j, ghost k); corners are therefore the X fill composed with the
 * Y fill (and Z). */
static void fill_boundaries(const fvora_sim* s, double* Q) {
  const int Ng = s->p.Ng;
  const int bcx = s->p.boundary_x, bcy = s->p.boundary_y, bcz = s->p.boundary_z;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = s->kbeg; k < s->kend; ++k)
    for (int j = s->jbeg; j < s->jend; ++j)
      for (int i = 0; i < Ng; ++i) {
        const int is[2] = {i, s->iend + i};
        const int iref[2] = {s->ibeg, s->iend - 1};
        for (int side = 0; side < 2; ++side) {
          double q[5];
          if (bcx == FV_BC_ABSORBING) memcpy(q, AT(s, Q, iref[side], j, k), sizeof(q));
          else if (bcx == FV_BC_REFLECTING) fill_reflecting(s, Q, is[side], j, k, iref[side], j, k, IX, q);
          else fill_periodic(s, Q, is[side], j, k, IX, q);
          memcpy(AT(s, Q, is[side], j, k), q, sizeof(q));
        }
      }
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = s->kbeg; k < s->kend; ++k)
    for (int j = 0; j < Ng; ++j)
      for (int i = 0; i < s->Ntx; ++i) {
        const int js[2] = {j, s->jend + j};
        const int jref[2] = {s->jbeg, s->jend - 1};
        for (int side = 0; side < 2; ++side) {
          double q[5];
          if (bcy == FV_BC_ABSORBING) memcpy(q, AT(s, Q, i, jref[side], k), sizeof(q));
          else if (bcy == FV_BC_REFLECTING) fill_reflecting(s, Q, i, js[side], k, i, jref[side], k, IY, q);
          else fill_periodic(s, Q, i, js[side], k, IY, q);
          memcpy(AT(s, Q, i, js[side], k), q, sizeof(q));
        }
      }
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < Ng; ++k)
    for (int j = 0; j < s->Nty; ++j)
      for (int i = 0; i < s->Ntx; ++i) {
        const int ks[2] = {k, s->kend + k};
        const int kref[2] = {s->kbeg, s->kend - 1};
        for (int side = 0; side < 2; ++side) {
          double q[5];
          if (bcz == FV_BC_ABSORBING) memcpy(q, AT(s, Q, i, j, kref[side]), sizeof(q));
          else if (bcz == FV_BC_REFLECTING) fill_reflecting(s, Q, i, j, ks[side], i, j, kref[side], IZ, q);
          else if (bcz == FV_BC_C91) fill_c91(s, Q, i, j, ks[side], kref[side], q);
          else fill_periodic(s, Q, i, j, ks[side], IZ, q);
          memcpy(AT(s, Q, i, j, ks[side]), q, sizeof(q));
        }
      }
}

/* ---------------- Update.h ---------------- */

static double minmod(double dL, double dR) { /* Update.h:73-80 */
  if (dL * dR < 0.0) return 0.0;
  else if (fabs(dL) < fabs(dR)) return dL;
  else return dR;
}

/* Update.h:55-88 over range_slopes (domain grown by one cell) */
static void compute_slopes(fvora_sim* s, const double* Q) {
  const int b0 = s->ibeg - 1, b1 = s->jbeg - 1, b2 = s->kbeg - 1;
  const int e0 = s->iend + 1, e1 = s->jend + 1, e2 = s->kend + 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = b2; k < e2; ++k)
    for (int j = b1; j < e1; ++j)
      for (int i = b0; i < e0; ++i) {
        const double* q = AT(s, Q, i, j, k);
        const double* qim = AT(s, Q, i - 1, j, k);
        const double* qip = AT(s, Q, i + 1, j, k);
        const double* qjm = AT(s, Q, i, j - 1, k);
        const double* qjp = AT(s, Q, i, j + 1, k);
        const double* qkm = AT(s, Q, i, j, k - 1);
        const double* qkp = AT(s, Q, i, j, k + 1);
        double* ox = AT(s, s->sx, i, j, k);
        double* oy = AT(s, s->sy, i, j, k);
        double* oz = AT(s, s->sz, i, j, k);
        for (int v = 0; v < 5; ++v) {
          double dL = q[v] - qim[v];
          double dR = qip[v] - q[v];
          double dU = q[v] - qjm[v];
          double dD = qjp[v] - q[v];
          double dF = qkp[v] - q[v];
          double dB = q[v] - qkm[v];
          ox[v] = minmod(dL, dR);
          oy[v] = minmod(dU, dD);
          oz[v] = minmod(dF, dB);
        }
      }
}

/* Update.h:14-33 */
static void reconstruct(const fvora_sim* s, const double* Q, const double* slopes, int i, int j, int k,
                        double sign, int dir, double* out) {
  const double* q = AT(s, Q, i, j, k);
  const double* sl = AT(s, slopes, i, j, k);
  double res[5];
  switch (s->p.reconstruction) {
    case FV_PLM:
      for (int v = 0; v < 5; ++v) res[v] = q[v] + sl[v] * sign * 0.5;
      break;
    case FV_PCM_WB:
      res[IR] = q[IR]; res[IU] = q[IU]; res[IV] = q[IV]; res[IW] = q[IW];
      res[IP] = (dir == IX || dir == IY ? q[IP] : q[IP] + sign * q[IR] * s->p.g * s->p.dz * 0.5);
      break;
    default:
      memcpy(res, q, sizeof(res));
  }
  swap_component(res, dir, out);
}

/* Update.h:90-162 */
static void compute_fluxes_and_update(fvora_sim* s, const double* Q, double* Unew, double dt) {
  range3 r = range_dom(s);
  const fv_params* P = &s->p;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = r.b[2]; k < r.e[2]; ++k)
    for (int j = r.b[1]; j < r.e[1]; ++j)
      for (int i = r.b[0]; i < r.e[0]; ++i) {
        for (int dir = 0; dir < 3; ++dir) {
          const double* slopes = (dir == IX ? s->sx : (dir == IY ? s->sy : s->sz));
          int dm[3] = {0, 0, 0}, dp[3] = {0, 0, 0};
          dm[dir] = -1;
          dp[dir] = 1;
          double qCL[5], qCR[5], qL[5], qR[5];
          reconstruct(s, Q, slopes, i, j, k, -1.0, dir, qCL);
          reconstruct(s, Q, slopes, i, j, k, 1.0, dir, qCR);
          reconstruct(s, Q, slopes, i + dm[IX], j + dm[IY], k + dm[IZ], 1.0, dir, qL);
          reconstruct(s, Q, slopes, i + dp[IX], j + dp[IY], k + dp[IZ], -1.0, dir, qR);
          double fluxL[5], fluxR[5], poutL, poutR;
          riemann(s, qL, qCL, fluxL, &poutL);
          riemann(s, qCR, qR, fluxR, &poutR);
          swap_component(fluxL, dir, fluxL);
          swap_component(fluxR, dir, fluxR);
          if (P->well_balanced_flux_at_z_bc && (k == s->kbeg || k == s->kend - 1) && dir == IZ) {
            const double rho = AT(s, Q, i, j, k)[IR];
            if (k == s->kbeg) {
              const double f[5] = {0.0, 0.0, 0.0, poutR - rho * P->g * P->dz, 0.0};
              memcpy(fluxL, f, sizeof(f));
            } else {
              const double f[5] = {0.0, 0.0, 0.0, poutL + rho * P->g * P->dz, 0.0};
              memcpy(fluxR, f, sizeof(f));
            }
          } else if (dir == IZ && (k == s->kbeg || k == s->kend - 1) && P->boundary_z == FV_BC_C91) {
            if (k == s->kbeg) {
              const double f[5] = {0.0, 0.0, 0.0, poutL, 0.0};
              memcpy(fluxL, f, sizeof(f));
            } else {
              const double f[5] = {0.0, 0.0, 0.0, poutR, 0.0};
              memcpy(fluxR, f, sizeof(f));
            }
          }
          double* un = AT(s, Unew, i, j, k);
          const double d = (dir == IX ? P->dx : (dir == IY ? P->dy : P->dz));
          for (int v = 0; v < 5; ++v) un[v] += (fluxL[v] - fluxR[v]) * dt / d;
          if (dir == IZ && P->gravity) {
            un[IW] += dt * AT(s, Q, i, j, k)[IR] * P->g;
            un[IE] += dt * 0.5 * (fluxL[IR] + fluxR[IR]) * P->g;
          }
        }
        double* un = AT(s, Unew, i, j, k);
        un[IR] = fmax(1.0e-6, un[IR]);
      }
}

/* ---------------- ThermalConduction.h ---------------- */

/* ThermalConduction.h:7-22 */
static double compute_kappa(const fv_params* P, double x, double y, double z) {
  (void)x; (void)y;
  if (P->thermal_conductivity_mode == FV_TCM_B02) {
    const double tr = (tanh((z - P->b02_zmid) / P->b02_thickness) + 1.0) * 0.5;
    return P->kappa * (P->b02_kappa1 * (1.0 - tr) + P->b02_kappa2 * tr);
  }
  return P->kappa;
}

/* ThermalConduction.h:32-97 */
static void apply_thermal_conduction(fvora_sim* s, const double* Q, double* Unew, double dt) {
  range3 r = range_dom(s);
  const fv_params* P = &s->p;
  const double dx = P->dx, dy = P->dy, dz = P->dz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = r.b[2]; k < r.e[2]; ++k)
    for (int j = r.b[1]; j < r.e[1]; ++j)
      for (int i = r.b[0]; i < r.e[0]; ++i) {
        double pos[3];
        get_pos(s, i, j, k, pos);
        const double x = pos[0], y = pos[1], z = pos[2];
        const double kc = compute_kappa(P, x, y, z);
        const double kappaL = 0.5 * (kc + compute_kappa(P, x - dx, y, z));
        const double kappaR = 0.5 * (kc + compute_kappa(P, x + dx, y, z));
        const double kappaU = 0.5 * (kc + compute_kappa(P, x, y - dy, z));
        const double kappaD = 0.5 * (kc + compute_kappa(P, x, y + dy, z));
        const double kappaF = 0.5 * (kc + compute_kappa(P, x, y, z - dz));
        const double kappaB = 0.5 * (kc + compute_kappa(P, x, y, z + dz));
#define TEMP(ii, jj, kk) (AT(s, Q, ii, jj, kk)[IP] / AT(s, Q, ii, jj, kk)[IR])
        const double TC = TEMP(i, j, k);
        const double TL = TEMP(i - 1, j, k);
        const double TR = TEMP(i + 1, j, k);
        const double TU = TEMP(i, j - 1, k);
        const double TD = TEMP(i, j + 1, k);
        const double TF = TEMP(i, j, k - 1);
        const double TB = TEMP(i, j, k + 1);
#undef TEMP
        const double FL = kappaL * (TC - TL) / dx;
        const double FR = kappaR * (TR - TC) / dx;
        const double FU = kappaU * (TC - TU) / dy;
        const double FD = kappaD * (TD - TC) / dy;
        double FF = kappaF * (TC - TF) / dz;
        double FB = kappaB * (TB - TC) / dz;
        if (k == s->kbeg && P->bctc_zmin != FV_BCTC_NONE) {
          if (P->bctc_zmin == FV_BCTC_FIXED_TEMPERATURE) FF = kappaF * 2.0 * (TC - P->bctc_zmin_value) / dz;
          else if (P->bctc_zmin == FV_BCTC_FIXED_GRADIENT) FF = kappaF * P->bctc_zmin_value;
        }
        if (k == s->kend - 1 && P->bctc_zmax != FV_BCTC_NONE) {
          if (P->bctc_zmax == FV_BCTC_FIXED_TEMPERATURE) FB = kappaB * 2.0 * (P->bctc_zmax_value - TC) / dz;
          else if (P->bctc_zmax == FV_BCTC_FIXED_GRADIENT) FB = kappaB * P->bctc_zmax_value;
        }
        AT(s, Unew, i, j, k)[IE] += dt / dx * (FR - FL) + dt / dy * (FD - FU) + dt / dz * (FB - FF);
      }
}

/* ---------------- Viscosity.h ---------------- */

/* Viscosity.h:22-155, written as the reference does it (including the
 * z-branch index/field mix-ups of Viscosity.h:221-228 and the missing 1/dx
 * on the flux divergence). */
static void apply_viscosity(fvora_sim* s, const double* Q, double* Unew, double dt) {
  range3 r = range_dom(s);
  const fv_params* P = &s->p;
  const double dx = P->dx, dy = P->dy, dz = P->dz;
  const double four_thirds = 4.0 / 3.0;
  const double two_thirds = 2.0 / 3.0;
  const int corrected = P->physics == FV_PHYS_CORRECTED;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = r.b[2]; k < r.e[2]; ++k)
    for (int j = r.b[1]; j < r.e[1]; ++j)
      for (int i = r.b[0]; i < r.e[0]; ++i) {
        double st[3][3][3][5]; /* [dk][dj][di][var] */
        for (int di = -1; di < 2; ++di)
          for (int dj = -1; dj < 2; ++dj)
            for (int dk = -1; dk < 2; ++dk)
              memcpy(st[dk + 1][dj + 1][di + 1], AT(s, Q, i + di, j + dj, k + dk), 5 * sizeof(double));
        const double one_over_dx = 1.0 / dx;
        const double one_over_dy = 1.0 / dy;
        const double one_over_dz = 1.0 / dz;
        const double mu = P->mu;
        double vf[3][5];
        for (int dir = 0; dir < 3; ++dir) {
          double flux[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
          for (int side = 1; side < 3; ++side) {
            const double sign = (side == 1 ? -1.0 : 1.0);
            double qi[5];
            if (dir == IX) {
              for (int v = 0; v < 5; ++v) qi[v] = (st[1][1][side][v] + st[1][1][side - 1][v]) * 0.5;
              double dudx = one_over_dx * (st[1][1][side][IU] - st[1][1][side - 1][IU]);
              double dvdx = one_over_dx * (st[1][1][side][IV] - st[1][1][side - 1][IV]);
              double dwdx = one_over_dx * (st[1][1][side][IW] - st[1][1][side - 1][IW]);
              double dudy = 0.25 * one_over_dy * (st[1][2][side][IU] - st[1][0][side][IU]
                                                + st[1][2][side - 1][IU] - st[1][0][side - 1][IU]);
              double dvdy = 0.25 * one_over_dy * (st[1][2][side][IV] - st[1][0][side][IV]
                                                + st[1][2][side - 1][IV] - st[1][0][side - 1][IV]);
              double dudz = 0.25 * one_over_dz * (st[2][1][side][IU] - st[0][1][side][IU]
                                                + st[2][1][side - 1][IU] - st[0][1][side - 1][IU]);
              double dwdz = 0.25 * one_over_dz * (st[2][1][side][IW] - st[0][1][side][IW]
                                                + st[2][1][side - 1][IW] - st[0][1][side - 1][IW]);
              const double tau_xx = four_thirds * dudx - two_thirds * (dvdy + dwdz);
              const double tau_xy = dvdx + dudy;
              const double tau_xz = dwdx + dudz;
              flux[IU] += sign * mu * tau_xx;
              flux[IV] += sign * mu * tau_xy;
              flux[IW] += sign * mu * tau_xz;
              flux[IE] += sign * mu * (tau_xx * qi[IU] + tau_xy * qi[IV] + tau_xz * qi[IW]);
            } else if (dir == IY) {
              for (int v = 0; v < 5; ++v) qi[v] = (st[1][side][1][v] + st[1][side - 1][1][v]) * 0.5;
              double dudy = one_over_dy * (st[1][side][1][IU] - st[1][side - 1][1][IU]);
              double dvdy = one_over_dy * (st[1][side][1][IV] - st[1][side - 1][1][IV]);
              double dwdy = one_over_dy * (st[1][side][1][IW] - st[1][side - 1][1][IW]);
              double dudx = 0.25 * one_over_dx * (st[1][side][2][IU] - st[1][side][0][IU]
                                                + st[1][side - 1][2][IU] - st[1][side - 1][0][IU]);
              double dvdx = 0.25 * one_over_dx * (st[1][side][2][IV] - st[1][side][0][IV]
                                                + st[1][side - 1][2][IV] - st[1][side - 1][0][IV]);
              double dwdz = 0.25 * one_over_dz * (st[2][side][1][IW] - st[0][side][1][IW]
                                                + st[2][side - 1][1][IW] - st[0][side - 1][1][IW]);
              double dvdz = 0.25 * one_over_dz * (st[2][side][1][IV] - st[0][side][1][IV]
                                                + st[2][side - 1][1][IV] - st[0][side - 1][1][IV]);
              const double tau_yy = four_thirds * dvdy - two_thirds * (dudx + dwdz);
              const double tau_xy = dvdx + dudy;
              const double tau_yz = dvdz + dwdy;
              flux[IU] += sign * mu * tau_xy;
              flux[IV] += sign * mu * tau_yy;
              flux[IW] += sign * mu * tau_yz;
              flux[IE] += sign * mu * (tau_xy * qi[IU] + tau_yy * qi[IV] + tau_yz * qi[IW]);
            } else if (corrected) {
              /* the mirror of the x / y branches (no counterpart in the reference) */
              for (int v = 0; v < 5; ++v) qi[v] = (st[side][1][1][v] + st[side - 1][1][1][v]) * 0.5;
              double dudz = one_over_dz * (st[side][1][1][IU] - st[side - 1][1][1][IU]);
              double dvdz = one_over_dz * (st[side][1][1][IV] - st[side - 1][1][1][IV]);
              double dwdz = one_over_dz * (st[side][1][1][IW] - st[side - 1][1][1][IW]);
              double dudx = 0.25 * one_over_dx * (st[side][1][2][IU] - st[side][1][0][IU]
                                                + st[side - 1][1][2][IU] - st[side - 1][1][0][IU]);
              double dwdx = 0.25 * one_over_dx * (st[side][1][2][IW] - st[side][1][0][IW]
                                                + st[side - 1][1][2][IW] - st[side - 1][1][0][IW]);
              double dvdy = 0.25 * one_over_dy * (st[side][2][1][IV] - st[side][0][1][IV]
                                                + st[side - 1][2][1][IV] - st[side - 1][0][1][IV]);
              double dwdy = 0.25 * one_over_dy * (st[side][2][1][IW] - st[side][0][1][IW]
                                                + st[side - 1][2][1][IW] - st[side - 1][0][1][IW]);
              const double tau_zz = four_thirds * dwdz - two_thirds * (dudx + dvdy);
              const double tau_xz = dudz + dwdx;
              const double tau_yz = dvdz + dwdy;
              flux[IU] += sign * mu * tau_xz;
              flux[IV] += sign * mu * tau_yz;
              flux[IW] += sign * mu * tau_zz;
              flux[IE] += sign * mu * (tau_xz * qi[IU] + tau_yz * qi[IV] + tau_zz * qi[IW]);
            } else {
              for (int v = 0; v < 5; ++v) qi[v] = (st[side][1][1][v] + st[side - 1][1][1][v]) * 0.5;
              double dudz = one_over_dz * (st[side][1][1][IU] - st[side - 1][1][1][IU]);
              double dvdz = one_over_dz * (st[side][1][1][IV] - st[side - 1][1][1][IV]);
              double dwdz = one_over_dz * (st[side][1][1][IW] - st[side - 1][1][1][IW]);
              double dudx = 0.25 * one_over_dx * (st[side][1][2][IU] - st[1][side][0][IU]
                                                + st[side - 1][1][2][IU] - st[1][side - 1][0][IU]);
              double dwdx = 0.25 * one_over_dx * (st[side][1][2][IV] - st[1][side][0][IW]
                                                + st[side - 1][1][2][IV] - st[1][side - 1][0][IW]);
              double dvdy = 0.25 * one_over_dz * (st[side][2][1][IW] - st[side][0][1][IV]
                                                + st[side - 1][2][1][IW] - st[side - 1][0][1][IV]);
              double dwdy = 0.25 * one_over_dz * (st[side][2][1][IV] - st[side][0][1][IW]
                                                + st[side - 1][2][1][IV] - st[side - 1][0][1][IW]);
              const double tau_zz = four_thirds * dwdz - two_thirds * (dudx + dvdy);
              const double tau_xz = dudz + dwdx;
              const double tau_yz = dvdz + dwdy;
              flux[IU] += sign * mu * tau_xz;
              flux[IV] += sign * mu * tau_yz;
              flux[IW] += sign * mu * tau_zz;
              flux[IE] += sign * mu * (tau_xz * qi[IU] + tau_yz * qi[IV] + tau_zz * qi[IW]);
            }
          }
          memcpy(vf[dir], flux, sizeof(flux));
        }
        double* un = AT(s, Unew, i, j, k);
        if (corrected)
          for (int v = 0; v < 5; ++v) un[v] += (vf[0][v] / dx + vf[1][v] / dy + vf[2][v] / dz) * dt;
        else
          for (int v = 0; v < 5; ++v) un[v] += (vf[0][v] + vf[1][v] + vf[2][v]) * dt;
      }
}

/* ---------------- Update.h: euler_step / update ---------------- */

/* Update.h:164-178 */
static void euler_step(fvora_sim* s, double* Q, double* Unew, double dt) {
  fill_boundaries(s, Q);
  if (s->p.reconstruction == FV_PLM) compute_slopes(s, Q);
  compute_fluxes_and_update(s, Q, Unew, dt);
  if (s->p.thermal_conductivity_active) apply_thermal_conduction(s, Q, Unew, dt);
  if (s->p.viscosity_active) apply_viscosity(s, Q, Unew, dt);
}

/* Update.h:187-204, with U0/Ustar sized like the other arrays */
static void rk2(fvora_sim* s, double dt) {
  const size_t bytes = s->ncell * 5 * sizeof(double);
  memcpy(s->U0, s->Unew, bytes);
  memcpy(s->Ustar, s->Unew, bytes);
  euler_step(s, s->Q, s->Ustar, dt);
  memcpy(s->Unew, s->Ustar, bytes);
  array_cons_to_prim(s, s->Ustar, s->Q);
  euler_step(s, s->Q, s->Unew, dt);
  range3 r = range_dom(s);
  double* U0 = s->U0;
  double* Unew = s->Unew;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = r.b[2]; k < r.e[2]; ++k)
    for (int j = r.b[1]; j < r.e[1]; ++j)
      for (int i = r.b[0]; i < r.e[0]; ++i)
        for (int v = 0; v < 5; ++v) AT(s, Unew, i, j, k)[v] = 0.5 * (AT(s, U0, i, j, k)[v] + AT(s, Unew, i, j, k)[v]);
}

/* ---------------- ComputeDt.h ---------------- */

/* ComputeDt.h:17-63 (computeKappa/computeMu of constant mode) */
static double compute_dt(fvora_sim* s, const double* Q, double inv_out[3]) {
  range3 r = range_dom(s);
  const fv_params* P = &s->p;
  double g0 = -INFINITY, g1 = -INFINITY, g2 = -INFINITY;
#pragma omp parallel
  {
    double l0 = -INFINITY, l1 = -INFINITY, l2 = -INFINITY;
#pragma omp for collapse(2) schedule(static)
    for (int k = r.b[2]; k < r.e[2]; ++k)
      for (int j = r.b[1]; j < r.e[1]; ++j)
        for (int i = r.b[0]; i < r.e[0]; ++i) {
          const double* q = AT(s, Q, i, j, k);
          const double cs = sound_speed(q, P->gamma0);
          const double hyp = (cs + fabs(q[IU])) / P->dx + (cs + fabs(q[IV])) / P->dy + (cs + fabs(q[IW])) / P->dz;
          double tc = P->epsilon;
          if (P->thermal_conductivity_active) {
            const double kap = compute_kappa(P, i, j, k);
            tc = fmax(fmax(2.0 * kap / (P->dx * P->dx), 2.0 * kap / (P->dy * P->dy)), 2.0 * kap / (P->dz * P->dz));
          }
          double vis = P->epsilon;
          if (P->viscosity_active)
            vis = fmax(fmax(2.0 * P->mu / (P->dx * P->dx), 2.0 * P->mu / (P->dy * P->dy)), 2.0 * P->mu / (P->dz * P->dz));
          l0 = fmax(l0, hyp);
          l1 = fmax(l1, tc);
          l2 = fmax(l2, vis);
        }
#pragma omp critical
    {
      if (l0 > g0) g0 = l0;
      if (l1 > g1) g1 = l1;
      if (l2 > g2) g2 = l2;
    }
  }
  if (inv_out) { inv_out[0] = g0; inv_out[1] = g1; inv_out[2] = g2; }
  double m = g0;
  if (g1 > m) m = g1;
  if (g2 > m) m = g2;
  return P->CFL / m;
}

/* ---------------- API ---------------- */

fvora_sim* fvora_create(const fv_params* p) {
  if (!p || p->Nx < 1 || p->Ny < 1 || p->Nz < 1 || p->Ng < 2) return NULL; /* slopes read i-2 */
  fvora_sim* s = (fvora_sim*)calloc(1, sizeof(fvora_sim));
  if (!s) return NULL;
  s->p = *p;
  s->Ntx = p->Nx + 2 * p->Ng;
  s->Nty = p->Ny + 2 * p->Ng;
  s->Ntz = p->Nz + 2 * p->Ng;
  s->ibeg = p->Ng; s->iend = p->Ng + p->Nx;
  s->jbeg = p->Ng; s->jend = p->Ng + p->Ny;
  s->kbeg = p->Ng; s->kend = p->Ng + p->Nz;
  s->ncell = (size_t)s->Ntx * s->Nty * s->Ntz;
  double** arrs[] = {&s->U, &s->Unew, &s->Q, &s->sx, &s->sy, &s->sz, &s->U0, &s->Ustar};
  for (size_t a = 0; a < sizeof(arrs) / sizeof(arrs[0]); ++a) {
    *arrs[a] = (double*)calloc(s->ncell * 5, sizeof(double));
    if (!*arrs[a]) { fvora_destroy(s); return NULL; }
  }
  return s;
}

void fvora_destroy(fvora_sim* s) {
  if (!s) return;
  free(s->U); free(s->Unew); free(s->Q); free(s->sx); free(s->sy); free(s->sz); free(s->U0); free(s->Ustar);
  free(s);
}

#define FOR_INTERIOR(s)                              \
  for (int k_ = 0; k_ < (s)->p.Nz; ++k_)             \
    for (int j_ = 0; j_ < (s)->p.Ny; ++j_)           \
      for (int i_ = 0; i_ < (s)->p.Nx; ++i_)

#define INTERIOR_N(s) (((size_t)k_ * (s)->p.Ny + j_) * (s)->p.Nx + i_)

/* Q interior <- fields, ghosts by the BC fill, U <- primToCons(Q) everywhere
 * (main.cpp:43-44 after Init.h:275-277). */
int fvora_set_prim(fvora_sim* s, const double* r, const double* u, const double* v, const double* w,
                   const double* p) {
  const double* f[5] = {r, u, v, w, p};
  FOR_INTERIOR(s) {
    double* q = AT(s, s->Q, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg);
    for (int var = 0; var < 5; ++var) q[var] = f[var] ? f[var][INTERIOR_N(s)] : 0.0;
  }
  fill_boundaries(s, s->Q);
  array_prim_to_cons(s, s->Q, s->U);
  return FV_OK;
}

/* ---------------- Init.h ---------------- */

/* Counter-based uniform in [0, 1): splitmix64 finaliser of key + golden *
 * (c + 1), top 53 bits, with key = splitmix64(seed + golden * (stream + 1)).
 * The H84 / C91 perturbations draw cell c = (k * Ny + j) * Nx + i of stream
 * 31 / 32 from it in place of Kokkos' XorShift64 pool (Init.h:13), whose
 * draws depend on which thread visits which cell; the product's generator
 * uses the same stream. */
static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double stream_uniform(uint64_t seed, uint64_t stream, uint64_t c) {
  const uint64_t golden = 0x9E3779B97F4A7C15ull;
  const uint64_t key = mix64(seed + golden * (stream + 1));
  return (double)(mix64(key + golden * (c + 1)) >> 11) * (1.0 / 9007199254740992.0);
}

/* One cell of the generator `problem` (Init.h:18-209); q in IR..IP order.
 * Returns 0 for an unknown problem (Init.h:241-242 throws). */
static int generate_cell(const fvora_sim* s, const char* problem, int i, int j, int k, uint64_t c, double* q) {
  const fv_params* P = &s->p;
  double pos[3];
  get_pos(s, i, j, k, pos);
  const double x = pos[IX], y = pos[IY], z = pos[IZ];
  q[IR] = q[IU] = q[IV] = q[IW] = q[IP] = 0.0;
  if (!strcmp(problem, "sod_x") || !strcmp(problem, "sod_y") || !strcmp(problem, "sod_z")) { /* Init.h:18-64 */
    const double d = problem[4] == 'x' ? x : problem[4] == 'y' ? y : z;
    q[IR] = d <= 0.5 ? 1.0 : 0.125;
    q[IP] = d <= 0.5 ? 1.0 : 0.1;
  } else if (!strcmp(problem, "blast")) { /* Init.h:69-98 */
    const double xr = 0.5 * (P->xmin + P->xmax) - x;
    const double yr = 0.5 * (P->ymin + P->ymax) - y;
    const double zr = 0.5 * (P->zmin + P->zmax) - z;
    const double r = sqrt(xr * xr + yr * yr + zr * zr);
    q[IR] = r < 0.2 ? 1.0 : 1.2;
    q[IP] = r < 0.2 ? 10.0 : 0.1;
  } else if (!strcmp(problem, "diffusion")) { /* Init.h:153-177 */
    const double x0 = x - 0.5 * (P->xmin + P->xmax);
    const double y0 = y - 0.5 * (P->ymin + P->ymax);
    const double z0 = z - 0.5 * (P->zmin + P->zmax);
    const double r = sqrt(x0 * x0 + y0 * y0 + z0 * z0);
    q[IR] = r < 0.2 ? 1.0 : 0.1;
    q[IP] = 1.0;
    q[IU] = q[IV] = q[IW] = 1.0;
  } else if (!strcmp(problem, "rayleigh-taylor")) { /* Init.h:182-206 */
    const double zmid = 0.5 * (P->zmin + P->zmax);
    q[IR] = z < zmid ? 1.0 : 2.0;
    q[IP] = 2.5 + 0.1 * P->g * z;
    if (z > -1.0 / 3.0 && z < 1.0 / 3.0)
      q[IW] = 0.01 * (1.0 + cos(4 * M_PI * x)) * (1.0 + cos(4.0 * M_PI * y)) * (1 + cos(3.0 * M_PI * z)) / 4.0;
  } else if (!strcmp(problem, "H84")) { /* Init.h:103-122 */
    q[IR] = pow(z, P->m1);
    q[IP] = pow(z, P->m1 + 1.0);
    q[IW] = P->h84_pert * (stream_uniform((uint64_t)(int64_t)P->seed, 31, c) - 0.5);
  } else if (!strcmp(problem, "C91")) { /* Init.h:127-148 */
    const double T = 1.0 + P->theta1 * z;
    q[IR] = pow(T, P->m1);
    const double prs = pow(T, P->m1 + 1.0);
    const double pert = P->c91_pert * (stream_uniform((uint64_t)(int64_t)P->seed, 32, c) - 0.5);
    q[IP] = prs * (1.0 + pert);
  } else {
    return 0;
  }
  return 1;
}

/* InitFunctor::init(Q) then primToCons (Init.h:247-279, main.cpp:42-44): Q's
 * interior from the generator, ghosts by the BC fill, U = primToCons(Q).
 * The generated interior primitives are returned when the arrays are given. */
int fvora_generate(fvora_sim* s, double* r, double* u, double* v, double* w, double* p) {
  double* f[5] = {r, u, v, w, p};
  int ok = 1;
  FOR_INTERIOR(s) {
    double* q = AT(s, s->Q, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg);
    ok &= generate_cell(s, s->p.problem, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg, (uint64_t)INTERIOR_N(s), q);
    for (int var = 0; var < 5; ++var)
      if (f[var]) f[var][INTERIOR_N(s)] = q[var];
  }
  if (!ok) return FV_ERR_PARAM;
  fill_boundaries(s, s->Q);
  array_prim_to_cons(s, s->Q, s->U);
  return FV_OK;
}

/* U interior <- fields; ghost cells of U get primToCons of BC-filled
 * consToPrim(U) so that every cell of U holds a finite state. */
int fvora_set_cons(fvora_sim* s, const double* r, const double* mx, const double* my, const double* mz,
                   const double* E) {
  const double* f[5] = {r, mx, my, mz, E};
  FOR_INTERIOR(s) {
    double* u = AT(s, s->U, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg);
    for (int var = 0; var < 5; ++var) u[var] = f[var] ? f[var][INTERIOR_N(s)] : 0.0;
    cons_to_prim(u, AT(s, s->Q, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg), s->p.gamma0);
  }
  fill_boundaries(s, s->Q);
  for (int k = 0; k < s->Ntz; ++k)
    for (int j = 0; j < s->Nty; ++j)
      for (int i = 0; i < s->Ntx; ++i) {
        const int interior = i >= s->ibeg && i < s->iend && j >= s->jbeg && j < s->jend && k >= s->kbeg && k < s->kend;
        if (!interior) prim_to_cons(AT(s, s->Q, i, j, k), AT(s, s->U, i, j, k), s->p.gamma0);
      }
  return FV_OK;
}

int fvora_get_prim(fvora_sim* s, double* r, double* u, double* v, double* w, double* p) {
  double* f[5] = {r, u, v, w, p};
  FOR_INTERIOR(s) {
    double q[5];
    cons_to_prim(AT(s, s->U, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg), q, s->p.gamma0);
    for (int var = 0; var < 5; ++var)
      if (f[var]) f[var][INTERIOR_N(s)] = q[var];
  }
  return FV_OK;
}

int fvora_get_cons(fvora_sim* s, double* r, double* mx, double* my, double* mz, double* E) {
  double* f[5] = {r, mx, my, mz, E};
  FOR_INTERIOR(s) {
    const double* u = AT(s, s->U, i_ + s->ibeg, j_ + s->jbeg, k_ + s->kbeg);
    for (int var = 0; var < 5; ++var)
      if (f[var]) f[var][INTERIOR_N(s)] = u[var];
  }
  return FV_OK;
}

/* main.cpp:55-57 */
double fvora_compute_dt(fvora_sim* s, double inv[3]) {
  array_cons_to_prim(s, s->U, s->Q);
  return compute_dt(s, s->Q, inv);
}

/* One pass of the main.cpp:51-74 loop body with the given dt (no I/O). */
int fvora_step(fvora_sim* s, double dt) {
  const size_t bytes = s->ncell * 5 * sizeof(double);
  memcpy(s->Unew, s->U, bytes);
  array_cons_to_prim(s, s->U, s->Q);
  if (s->p.time_stepping == FV_TS_RK2) rk2(s, dt);
  else euler_step(s, s->Q, s->Unew, dt);
  memcpy(s->U, s->Unew, bytes);
  return FV_OK;
}

/* main.cpp:51-74 */
int fvora_advance(fvora_sim* s, double tend, long max_steps, double* t, long* nsteps) {
  long n = 0;
  double tt = *t;
  while (tt + s->p.epsilon < tend && (max_steps <= 0 || n < max_steps)) {
    const double dt = fvora_compute_dt(s, NULL);
    fvora_step(s, dt);
    tt += dt;
    ++n;
  }
  *t = tt;
  if (nsteps) *nsteps = n;
  return FV_OK;
}

int fvora_riemann(int solver, double gamma0, long n, const double* qL, const double* qR, double* flux,
                  double* pout) {
  for (long c = 0; c < n; ++c) {
    if (solver == FV_HLL) hll(qL + 5 * c, qR + 5 * c, flux + 5 * c, pout + c, gamma0);
    else hllc(qL + 5 * c, qR + 5 * c, flux + 5 * c, pout + c, gamma0, 0);
  }
  return FV_OK;
}

int fvora_set_threads(int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
}
