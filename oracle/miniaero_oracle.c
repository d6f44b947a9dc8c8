/*
 * CPU oracle for the miniAero explicit RK4 residual path (test infrastructure;
 * see miniaero_oracle.h). Each function restates one reference functor, with
 * the same operand order, so that a serial run reproduces the reference's
 * Kokkos Serial arithmetic bit for bit when compiled with -ffp-contract=off.
 */
#include "miniaero_oracle.h"

#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- atomics (Kokkos::atomic_add / atomic_compare_exchange semantics) ---- */
static inline void atomic_add_d(double* p, double v, int par) {
  if (!par) { *p += v; return; }
#pragma omp atomic
  *p += v;
}

typedef union { double d; uint64_t u; } dbits;

/* CAS loop of StencilLimiter.h:156-161: new = op(*p, v) until the swap sticks. */
static inline void atomic_min_d(double* p, double v, int par) {
  if (!par) { double cur = *p; *p = (v < cur) ? v : cur; return; }
  uint64_t* pu = (uint64_t*)p;
  for (;;) {
    dbits oldv, newv;
    oldv.u = __atomic_load_n(pu, __ATOMIC_RELAXED);
    newv.d = (v < oldv.d) ? v : oldv.d;
    if (__atomic_compare_exchange_n(pu, &oldv.u, newv.u, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
  }
}

static inline void atomic_max_d(double* p, double v, int par) {
  if (!par) { double cur = *p; *p = (cur < v) ? v : cur; return; }
  uint64_t* pu = (uint64_t*)p;
  for (;;) {
    dbits oldv, newv;
    oldv.u = __atomic_load_n(pu, __ATOMIC_RELAXED);
    newv.d = (oldv.d < v) ? v : oldv.d;
    if (__atomic_compare_exchange_n(pu, &oldv.u, newv.u, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
  }
}

/* ---- gas model (GasModel.h) ---- */
static inline double pressure_of(const double* V) { return V[0] * 287.05 * V[4]; }
static inline double enthalpy_of(const double* V) { return 1004.0 * V[4]; }

/* GasModel.h:69-90 */
void oracle_primitives(const double* U, double* V) {
  const double gamma = 1.4, Rgas = 287.05;
  const double r = U[0];
  const double ri = 1.0 / r;
  const double u = U[1] * ri;
  const double v = U[2] * ri;
  const double w = U[3] * ri;
  const double k = 0.5 * (u * u + v * v + w * w);
  const double e = U[4] * ri - k;
  const double T = e * (gamma - 1.0) / Rgas;
  V[0] = r; V[1] = u; V[2] = v; V[3] = w; V[4] = T;
}

/* ---- Roe flux (Roe_Flux.h:50-265) ---- */
static void matvec5(const double A[25], const double x[5], double y[5]) {
  for (int i = 0; i < 5; ++i) {
    double acc = 0.0;
    for (int j = 0; j < 5; ++j) acc += 1.0 * A[5 * i + j] * x[j];
    y[i] = acc;
  }
}

void oracle_roe_flux(const double* pl, const double* pr, const double* n, const double* t,
                     const double* b, double* flux) {
  const double efix_u = 0.1, efix_c = 0.1, gm1 = 0.4;
  const double rl = pl[0], ul = pl[1], vl = pl[2], wl = pl[3];
  const double p_l = pressure_of(pl), h_l = enthalpy_of(pl);
  const double H_l = h_l + 0.5 * (ul * ul + vl * vl + wl * wl);
  const double mf_l = rl * (n[0] * ul + n[1] * vl + n[2] * wl);
  const double rr = pr[0], ur = pr[1], vr = pr[2], wr = pr[3];
  const double p_r = pressure_of(pr), h_r = enthalpy_of(pr);
  const double H_r = h_r + 0.5 * (ur * ur + vr * vr + wr * wr);
  const double mf_r = rr * (n[0] * ur + n[1] * vr + n[2] * wr);
  const double psum = p_l + p_r;

  flux[0] = 0.5 * (mf_l + mf_r);
  flux[1] = 0.5 * (mf_l * ul + mf_r * ur + n[0] * psum);
  flux[2] = 0.5 * (mf_l * vl + mf_r * vr + n[1] * psum);
  flux[3] = 0.5 * (mf_l * wl + mf_r * wr + n[2] * psum);
  flux[4] = 0.5 * (mf_l * H_l + mf_r * H_r);

  const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const double tn = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  const double bn = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  const double nu[3] = {n[0] / nn, n[1] / nn, n[2] / nn};
  const double tu[3] = {t[0] / tn, t[1] / tn, t[2] / tn};
  const double bu[3] = {b[0] / bn, b[1] / bn, b[2] / bn};

  const double denom = 1.0 / (sqrt(rl) + sqrt(rr));
  const double alpha = sqrt(rl) * denom;
  const double beta = 1.0 - alpha;
  const double uroe = alpha * ul + beta * ur;
  const double vroe = alpha * vl + beta * vr;
  const double wroe = alpha * wl + beta * wr;
  const double hroe = alpha * h_l + beta * h_r +
                      0.5 * alpha * beta *
                          ((ur - ul) * (ur - ul) + (vr - vl) * (vr - vl) + (wr - wl) * (wr - wl));
  const double c = sqrt(gm1 * hroe);

  const double nv = uroe * nu[0] + vroe * nu[1] + wroe * nu[2];
  const double tv = uroe * tu[0] + vroe * tu[1] + wroe * tu[2];
  const double bv = uroe * bu[0] + vroe * bu[1] + wroe * bu[2];
  const double ke = 0.5 * (uroe * uroe + vroe * vroe + wroe * wroe);
  const double cssi = 1.0 / (c * c);
  const double hcssi = 0.5 * cssi;

  double dq[5];
  dq[0] = rr - rl;
  dq[1] = rr * ur - rl * ul;
  dq[2] = rr * vr - rl * vl;
  dq[3] = rr * wr - rl * wl;
  dq[4] = (rr * H_r - p_r) - (rl * H_l - p_l);

  const double cbar = c * nn;
  const double ubar = uroe * n[0] + vroe * n[1] + wroe * n[2];
  const double cfl = fabs(ubar) + cbar;
  const double eig1 = ubar + cbar, eig2 = ubar - cbar, eig3 = ubar;
  double a1 = fabs(eig1), a2 = fabs(eig2), a3 = fabs(eig3);
  const double epuc = efix_u * cfl, epcc = efix_c * cfl;
  if (a1 < epcc) a1 = 0.5 * (eig1 * eig1 + epcc * epcc) / epcc;
  if (a2 < epcc) a2 = 0.5 * (eig2 * eig2 + epcc * epcc) / epcc;
  if (a3 < epuc) a3 = 0.5 * (eig3 * eig3 + epuc * epuc) / epuc;
  double eigp[5] = {0.5 * (eig1 + a1), 0.5 * (eig2 + a2), 0.5 * (eig3 + a3), 0.0, 0.0};
  eigp[3] = eigp[4] = eigp[2];
  double eigm[5] = {0.5 * (eig1 - a1), 0.5 * (eig2 - a2), 0.5 * (eig3 - a3), 0.0, 0.0};
  eigm[3] = eigm[4] = eigm[2];

  double M[25], ldq[5], rlldq[5];
  M[0] = gm1 * (ke - hroe) + c * (c - nv);
  M[1] = c * nu[0] - gm1 * uroe;
  M[2] = c * nu[1] - gm1 * vroe;
  M[3] = c * nu[2] - gm1 * wroe;
  M[4] = gm1;
  M[5] = gm1 * (ke - hroe) + c * (c + nv);
  M[6] = -c * nu[0] - gm1 * uroe;
  M[7] = -c * nu[1] - gm1 * vroe;
  M[8] = -c * nu[2] - gm1 * wroe;
  M[9] = gm1;
  M[10] = ke - hroe;
  M[11] = -uroe;
  M[12] = -vroe;
  M[13] = -wroe;
  M[14] = 1.0;
  M[15] = -tv;
  M[16] = tu[0];
  M[17] = tu[1];
  M[18] = tu[2];
  M[19] = 0.0;
  M[20] = -bv;
  M[21] = bu[0];
  M[22] = bu[1];
  M[23] = bu[2];
  M[24] = 0.0;
  matvec5(M, dq, ldq);
  for (int j = 0; j < 5; ++j) ldq[j] = (eigp[j] - eigm[j]) * ldq[j];

  M[0] = hcssi;
  M[1] = hcssi;
  M[2] = -gm1 * cssi;
  M[3] = 0.0;
  M[4] = 0.0;
  M[5] = (uroe + nu[0] * c) * hcssi;
  M[6] = (uroe - nu[0] * c) * hcssi;
  M[7] = -gm1 * uroe * cssi;
  M[8] = tu[0];
  M[9] = bu[0];
  M[10] = (vroe + nu[1] * c) * hcssi;
  M[11] = (vroe - nu[1] * c) * hcssi;
  M[12] = -gm1 * vroe * cssi;
  M[13] = tu[1];
  M[14] = bu[1];
  M[15] = (wroe + nu[2] * c) * hcssi;
  M[16] = (wroe - nu[2] * c) * hcssi;
  M[17] = -gm1 * wroe * cssi;
  M[18] = tu[2];
  M[19] = bu[2];
  M[20] = (hroe + ke + c * nv) * hcssi;
  M[21] = (hroe + ke - c * nv) * hcssi;
  M[22] = (c * c - gm1 * (hroe + ke)) * cssi;
  M[23] = tv;
  M[24] = bv;
  matvec5(M, ldq, rlldq);
  for (int i = 0; i < 5; ++i) flux[i] -= 0.5 * rlldq[i];
}

/* ---- Newtonian viscous flux (Viscous_Flux.h:66-98, GasModel.h:92-106) ---- */
void oracle_viscous_flux(const double g[5][3], const double* prim, const double* a,
                         int viscosity_model, double mu_const, double prandtl, double* vflux) {
  double mu, kcond;
  if (viscosity_model == 1) {
    mu = mu_const;
    kcond = mu * 1006.0 / prandtl;
  } else {
    const double T = prim[4];
    mu = 1.458e-6 * T * sqrt(T) / (T + 110.4);
    kcond = mu * 1006.0 / 0.71;
  }
  double div = 0;
  for (int i = 0; i < 5; ++i) vflux[i] = 0.0;
  for (int i = 0; i < 3; ++i) div += g[i + 1][i];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      const double delta = (i == j) ? 1 : 0;
      const double S = 0.5 * (g[i + 1][j] + g[j + 1][i]);
      const double tij = S - div * delta / 3.;
      vflux[1 + i] += (2 * mu * tij) * a[j];
      vflux[4] += (2 * mu * tij) * prim[i + 1] * a[j];
    }
    vflux[4] += kcond * g[4][i] * a[i];
  }
}

/* ---- limiter functions ---- */
/* VenkatLimiter.h:45-73 */
double oracle_venkat(double dumax, double dumin, double du, double deltax3) {
  const double beta = 1;
  const double eps2 = deltax3 * beta * beta * beta;
  double phi;
  if (du > 1e-40) {
    const double num = (dumax * dumax + eps2) * du + 2 * du * du * dumax;
    const double den = du * (dumax * dumax + 2 * du * du + dumax * du + eps2);
    phi = num / den;
  } else if (du < -1e-40) {
    const double num = (dumin * dumin + eps2) * du + 2 * du * du * dumin;
    const double den = du * (dumin * dumin + 2 * du * du + dumin * du + eps2);
    phi = num / den;
  } else {
    phi = 1;
  }
  return phi;
}

/* VanAlbadaLimiter.h:45-65 (serial MathTools min/max = std::min/std::max) */
double oracle_vanalbada(double dumax, double dumin, double du) {
  double y = 2;
  if (du > DBL_EPSILON) y = dumax / du;
  else if (du < -DBL_EPSILON) y = dumin / du;
  double phi = 1;
  if (y < 2) {
    phi = (4 * y - y * y) / (y * y - 4 * y + 8);
    phi = (phi < 0.0) ? 0.0 : phi;
    phi = (1.0 < phi) ? 1.0 : phi;
  }
  return phi;
}

/* ---- solver state ---- */
typedef struct {
  const oracle_mesh* m;
  const oracle_options* o;
  int par, nt;
  double *Un, *Unp1, *Utmp, *res;
  double *cell_flux;   /* [C*5]  (Cells.h cell_flux_(i,0,icomp)) */
  double *cell_grad;   /* [C*15] (cell_gradient_(i,0,icomp,idir)) */
  double *grad;        /* [C*15] summed gradients */
  double *smin, *smax; /* [C*5] stored and stencil min/max (ATOMICS layout) */
  double *slim;        /* [C*5] stored limiter */
  double *lim;         /* [C*5] limiter */
  /* CELL_FLUX storage, one entry per element-local face slot (Cells.h:70-73) */
  int cf;
  double *cf_flux;     /* [C*6*5] */
  double *cf_grad;     /* [C*6*15] */
  double *cf_min, *cf_max, *cf_lim;  /* [C*6*5] */
} ostate;

#define NSLOTS 6  /* Hexa8 faces per cell */
static inline size_t slot5(int c, int slot) { return ((size_t)c * NSLOTS + (size_t)slot) * 5; }
static inline size_t slot15(int c, int slot) { return ((size_t)c * NSLOTS + (size_t)slot) * 15; }

#define PFOR _Pragma("omp parallel for schedule(static) if(s->par) num_threads(s->nt)")

/* TimeSolverExplicitRK4.h:106-128 */
static void update(ostate* s, double alpha, const double* res, const double* src, double* dst) {
  const int C = s->m->ncells;
  PFOR
  for (int i = 0; i < C; ++i)
    for (int k = 0; k < 5; ++k) dst[5 * i + k] = src[5 * i + k] + alpha * res[5 * i + k];
}

/* Cells.h:83-120 */
static void zero_cell_flux(ostate* s) {
  const int C = s->m->ncells;
  PFOR
  for (int i = 0; i < C; ++i) {
    for (int k = 0; k < 5; ++k) {
      s->cell_flux[5 * i + k] = 0.0;
      for (int d = 0; d < 3; ++d) s->cell_grad[15 * i + 3 * k + d] = 0.0;
    }
    if (s->cf)
      for (int slot = 0; slot < NSLOTS; ++slot) {
        for (int k = 0; k < 5; ++k) s->cf_flux[slot5(i, slot) + k] = 0.0;
        for (int j = 0; j < 15; ++j) s->cf_grad[slot15(i, slot) + j] = 0.0;
      }
  }
}

/* GreenGauss.h:300-321 */
static void green_gauss(ostate* s) {
  const oracle_mesh* m = s->m;
  const oracle_faces* f = &m->internal;
  const double* U = s->Utmp;
  const double* vol = m->cell_volumes;
  PFOR
  for (int ii = 0; ii < f->nfaces; ++ii) {   /* green_gauss_face, GreenGauss.h:79-135 */
    const int i = f->permutation[ii];
    const int L = f->conn[2 * i], R = f->conn[2 * i + 1];
    double pl[5], pr[5];
    oracle_primitives(&U[5 * L], pl);
    oracle_primitives(&U[5 * R], pr);
    const double vl = vol[L], vr = vol[R];
    for (int d = 0; d < 3; ++d) {
      const double fn = f->normal[3 * i + d];
      for (int k = 0; k < 5; ++k) {
        const double g = 0.5 * (pl[k] + pr[k]) * fn;
        if (s->cf) {  /* GreenGauss.h:129-132 */
          s->cf_grad[slot15(L, f->flux_index[2 * i]) + 3 * k + d] = g / vl;
          s->cf_grad[slot15(R, f->flux_index[2 * i + 1]) + 3 * k + d] = -g / vr;
        } else {
          atomic_add_d(&s->cell_grad[15 * L + 3 * k + d], g / vl, s->par);
          atomic_add_d(&s->cell_grad[15 * R + 3 * k + d], -g / vr, s->par);
        }
      }
    }
  }
  for (int b = 0; b < m->nbc; ++b) {          /* green_gauss_boundary_face, :168-220 */
    const oracle_faces* bf = &m->bc[b];
    PFOR
    for (int i = 0; i < bf->nfaces; ++i) {
      const int c = bf->conn[2 * i];
      double p[5], g[5][3];
      oracle_primitives(&U[5 * c], p);
      for (int k = 0; k < 5; ++k)
        for (int d = 0; d < 3; ++d) g[k][d] = p[k] * bf->normal[3 * i + d];
      for (int k = 0; k < 5; ++k)
        for (int d = 0; d < 3; ++d) {
          if (s->cf)  /* GreenGauss.h:211-219 */
            s->cf_grad[slot15(c, bf->flux_index[2 * i]) + 3 * k + d] = g[k][d] / vol[c];
          else
            atomic_add_d(&s->cell_grad[15 * c + 3 * k + d], g[k][d] / vol[c], s->par);
        }
    }
  }
  const int C = m->ncells;
  PFOR
  for (int i = 0; i < C; ++i)                 /* green_gauss_gradient_sum, :244-269 */
    for (int j = 0; j < 15; ++j) {
      double acc = 0;
      if (s->cf)
        for (int slot = 0; slot < NSLOTS; ++slot) acc += s->cf_grad[slot15(i, slot) + j];
      else
        acc += s->cell_grad[15 * i + j];
      s->grad[15 * i + j] = acc;
    }
}

/* StencilLimiter.h:532-559 */
static void min_max(ostate* s) {
  const oracle_mesh* m = s->m;
  const double* U = s->Utmp;
  const int C = m->ncells;
  PFOR
  for (int i = 0; i < C; ++i)                  /* initialize_min_max, :227-236 */
    for (int k = 0; k < 5; ++k) {
      s->smin[5 * i + k] = 1.0e300;
      s->smax[5 * i + k] = -1.0e300;
      if (s->cf)
        for (int slot = 0; slot < NSLOTS; ++slot) {
          s->cf_min[slot5(i, slot) + k] = 1.0e300;
          s->cf_max[slot5(i, slot) + k] = -1.0e300;
        }
    }
  const oracle_faces* f = &m->internal;
  PFOR
  for (int ii = 0; ii < f->nfaces; ++ii) {   /* min_max_face<true>, :84-201 */
    const int i = f->permutation[ii];
    const int L = f->conn[2 * i], R = f->conn[2 * i + 1];
    double pl[5], pr[5];
    oracle_primitives(&U[5 * L], pl);
    oracle_primitives(&U[5 * R], pr);
    for (int k = 0; k < 5; ++k) {
      const double fmin_ = (pr[k] < pl[k]) ? pr[k] : pl[k];
      const double fmax_ = (pr[k] > pl[k]) ? pr[k] : pl[k];
      if (s->cf) {  /* :191-198 */
        s->cf_min[slot5(L, f->flux_index[2 * i]) + k] = fmin_;
        s->cf_max[slot5(L, f->flux_index[2 * i]) + k] = fmax_;
        s->cf_min[slot5(R, f->flux_index[2 * i + 1]) + k] = fmin_;
        s->cf_max[slot5(R, f->flux_index[2 * i + 1]) + k] = fmax_;
        continue;
      }
      atomic_min_d(&s->smin[5 * L + k], fmin_, s->par);
      atomic_max_d(&s->smax[5 * L + k], fmax_, s->par);
      atomic_min_d(&s->smin[5 * R + k], fmin_, s->par);
      atomic_max_d(&s->smax[5 * R + k], fmax_, s->par);
    }
  }
  for (int b = 0; b < m->nbc; ++b) {          /* min_max_face<false> */
    const oracle_faces* bf = &m->bc[b];
    PFOR
    for (int ii = 0; ii < bf->nfaces; ++ii) {
      const int i = bf->permutation[ii];
      const int L = bf->conn[2 * i];
      double pl[5];
      oracle_primitives(&U[5 * L], pl);
      for (int k = 0; k < 5; ++k) {
        if (s->cf) {
          s->cf_min[slot5(L, bf->flux_index[2 * i]) + k] = pl[k];
          s->cf_max[slot5(L, bf->flux_index[2 * i]) + k] = pl[k];
          continue;
        }
        atomic_min_d(&s->smin[5 * L + k], pl[k], s->par);
        atomic_max_d(&s->smax[5 * L + k], pl[k], s->par);
      }
    }
  }
  /* gather_min_max: ATOMICS_FLUX copies stored -> stencil (same buffers here);
     CELL_FLUX takes std::min / std::max over the slots in order (:274-279). */
  if (s->cf) {
    PFOR
    for (int i = 0; i < C; ++i)
      for (int k = 0; k < 5; ++k)
        for (int slot = 0; slot < NSLOTS; ++slot) {
          const double a = s->cf_min[slot5(i, slot) + k], b = s->cf_max[slot5(i, slot) + k];
          s->smin[5 * i + k] = (a < s->smin[5 * i + k]) ? a : s->smin[5 * i + k];
          s->smax[5 * i + k] = (s->smax[5 * i + k] < b) ? b : s->smax[5 * i + k];
        }
  }
}

static inline double limit_fn(const ostate* s, double dumax, double dumin, double du, double d2) {
  return s->o->limiter == 1 ? oracle_vanalbada(dumax, dumin, du) : oracle_venkat(dumax, dumin, du, d2);
}

/* One side of limiter_face (StencilLimiter.h:391-461). */
static void limiter_side(const ostate* s, const oracle_faces* f, int i, int c, const double* p, double* phi) {
  const double* xc = &s->m->cell_coords[3 * c];
  double disp[3], dist = 0;
  for (int d = 0; d < 3; ++d) {
    disp[d] = f->coords[3 * i + d] - xc[d];
    dist += disp[d] * disp[d];
  }
  for (int k = 0; k < 5; ++k) {
    double du = 0;
    for (int d = 0; d < 3; ++d) du += disp[d] * s->grad[15 * c + 3 * k + d];
    const double dumax = s->smax[5 * c + k] - p[k];
    const double dumin = s->smin[5 * c + k] - p[k];
    phi[k] = limit_fn(s, dumax, dumin, du, dist);
  }
}

/* StencilLimiter.h:591-616 */
static void limiter(ostate* s) {
  const oracle_mesh* m = s->m;
  const double* U = s->Utmp;
  const int C = m->ncells;
  PFOR
  for (int i = 0; i < C; ++i)                  /* initialize_limiter, :306-313 */
    for (int k = 0; k < 5; ++k) {
      s->slim[5 * i + k] = 1.0;
      if (s->cf)
        for (int slot = 0; slot < NSLOTS; ++slot) s->cf_lim[slot5(i, slot) + k] = 1.0;
    }
  const oracle_faces* f = &m->internal;
  PFOR
  for (int ii = 0; ii < f->nfaces; ++ii) {
    const int i = f->permutation[ii];
    const int L = f->conn[2 * i], R = f->conn[2 * i + 1];
    double pl[5], pr[5], phl[5], phr[5];
    oracle_primitives(&U[5 * L], pl);
    oracle_primitives(&U[5 * R], pr);
    limiter_side(s, f, i, L, pl, phl);
    limiter_side(s, f, i, R, pr, phr);
    for (int k = 0; k < 5; ++k) {
      if (s->cf) {  /* :489-497 */
        s->cf_lim[slot5(L, f->flux_index[2 * i]) + k] = phl[k];
        s->cf_lim[slot5(R, f->flux_index[2 * i + 1]) + k] = phr[k];
        continue;
      }
      atomic_min_d(&s->slim[5 * L + k], phl[k], s->par);
      atomic_min_d(&s->slim[5 * R + k], phr[k], s->par);
    }
  }
  for (int b = 0; b < m->nbc; ++b) {
    const oracle_faces* bf = &m->bc[b];
    PFOR
    for (int ii = 0; ii < bf->nfaces; ++ii) {
      const int i = bf->permutation[ii];
      const int L = bf->conn[2 * i];
      double pl[5], phl[5];
      oracle_primitives(&U[5 * L], pl);
      limiter_side(s, bf, i, L, pl, phl);
      for (int k = 0; k < 5; ++k) {
        if (s->cf)
          s->cf_lim[slot5(L, bf->flux_index[2 * i]) + k] = phl[k];
        else
          atomic_min_d(&s->slim[5 * L + k], phl[k], s->par);
      }
    }
  }
  PFOR
  for (int i = 0; i < C; ++i)                  /* gather_limiter, :336-349 */
    for (int k = 0; k < 5; ++k) {
      if (s->cf) {  /* limiter_ starts at 1.0; std::min over the slots in order */
        double l = 1.0;
        for (int slot = 0; slot < NSLOTS; ++slot) {
          const double v = s->cf_lim[slot5(i, slot) + k];
          l = (v < l) ? v : l;
        }
        s->lim[5 * i + k] = l;
      } else {
        s->lim[5 * i + k] = s->slim[5 * i + k];
      }
    }
}

/* compute_face_flux (Flux.h:89-180) */
static void internal_flux(ostate* s) {
  const oracle_mesh* m = s->m;
  const oracle_faces* f = &m->internal;
  const double* U = s->Utmp;
  const int second = s->o->second_order, visc = s->o->viscous;
  PFOR
  for (int ii = 0; ii < f->nfaces; ++ii) {
    const int i = f->permutation[ii];
    const int L = f->conn[2 * i], R = f->conn[2 * i + 1];
    double flux[5], pl[5], pr[5];
    oracle_primitives(&U[5 * L], pl);
    oracle_primitives(&U[5 * R], pr);
    if (second) {
      for (int k = 0; k < 5; ++k) {
        double tl = 0, tr = 0;
        for (int d = 0; d < 3; ++d) {
          tl += (f->coords[3 * i + d] - m->cell_coords[3 * L + d]) * s->grad[15 * L + 3 * k + d];
          tr += (f->coords[3 * i + d] - m->cell_coords[3 * R + d]) * s->grad[15 * R + 3 * k + d];
        }
        pl[k] += tl * s->lim[5 * L + k];
        pr[k] += tr * s->lim[5 * R + k];
      }
    }
    oracle_roe_flux(pl, pr, &f->normal[3 * i], &f->tangent[3 * i], &f->binormal[3 * i], flux);
    if (visc) {
      double pf[5], gf[5][3], vf[5];
      for (int k = 0; k < 5; ++k) {
        pf[k] = 0.5 * (pl[k] + pr[k]);
        for (int d = 0; d < 3; ++d) gf[k][d] = 0.5 * (s->grad[15 * L + 3 * k + d] + s->grad[15 * R + 3 * k + d]);
      }
      oracle_viscous_flux((const double(*)[3])gf, pf, &f->normal[3 * i], s->o->viscosity_model, s->o->mu,
                          s->o->prandtl, vf);
      for (int k = 0; k < 5; ++k) flux[k] -= vf[k];
    }
    for (int k = 0; k < 5; ++k) {
      if (s->cf) {  /* Flux.h:172-178 */
        s->cf_flux[slot5(L, f->flux_index[2 * i]) + k] = -flux[k];
        s->cf_flux[slot5(R, f->flux_index[2 * i + 1]) + k] = flux[k];
        continue;
      }
      atomic_add_d(&s->cell_flux[5 * L + k], -flux[k], s->par);
      atomic_add_d(&s->cell_flux[5 * R + k], flux[k], s->par);
    }
  }
}

/* Ghost state of Tangent_BC.h:86-102 / NoSlip_BC.h:93-109. */
static double reflect(const double* n, const double* pl, double* pr) {
  double area = 0;
  for (int d = 0; d < 3; ++d) area += n[d] * n[d];
  area = sqrt(area);
  double ub = 0.0;
  ub += pl[1] * n[0] / area;
  ub += pl[2] * n[1] / area;
  ub += pl[3] * n[2] / area;
  pr[0] = pl[0];
  pr[1] = pl[1] - 2 * ub * n[0] / area;
  pr[2] = pl[2] - 2 * ub * n[1] / area;
  pr[3] = pl[3] - 2 * ub * n[2] / area;
  pr[4] = pl[4];
  return area;
}

static void bc_flux(ostate* s, const oracle_faces* bf) {
  const oracle_mesh* m = s->m;
  const double* U = s->Utmp;
  PFOR
  for (int i = 0; i < bf->nfaces; ++i) {
    const int c = bf->conn[2 * i];
    const double* n = &bf->normal[3 * i];
    const double* t = &bf->tangent[3 * i];
    const double* b = &bf->binormal[3 * i];
    double pl[5], pr[5], flux[5], contrib[5];
    oracle_primitives(&U[5 * c], pl);
    if (bf->type == 0) {                       /* Extrapolate_BC.h:70-100 */
      oracle_roe_flux(pl, pl, n, t, b, flux);
      for (int k = 0; k < 5; ++k) contrib[k] = -flux[k];
    } else if (bf->type == 1) {                /* Tangent_BC.h:72-121 */
      reflect(n, pl, pr);
      oracle_roe_flux(pl, pr, n, t, b, flux);
      for (int k = 0; k < 5; ++k) contrib[k] = -flux[k];
    } else if (bf->type == 2) {                /* Inflow_BC.h:73-109 */
      oracle_primitives(s->o->inflow_state, pr);
      oracle_roe_flux(pl, pr, n, t, b, flux);
      for (int k = 0; k < 5; ++k) contrib[k] = -flux[k];
    } else {                                   /* NoSlip_BC.h:77-155 */
      double vflux[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      const double area = reflect(n, pl, pr);
      oracle_roe_flux(pl, pr, n, t, b, flux);
      double pf[5], gf[5][3], dist = 0, un[3];
      pf[0] = pl[0]; pf[1] = 0.0; pf[2] = 0.0; pf[3] = 0.0; pf[4] = pl[4];
      for (int d = 0; d < 3; ++d) {
        const double dx = bf->coords[3 * i + d] - m->cell_coords[3 * c + d];
        dist += dx * dx; /* std::pow(dx, 2) */
        un[d] = n[d] / area;
      }
      const double inv_d = 1.0 / sqrt(dist);
      for (int k = 0; k < 5; ++k)
        for (int d = 0; d < 3; ++d) gf[k][d] = (pf[k] - pl[k]) * un[d] * inv_d;
      oracle_viscous_flux((const double(*)[3])gf, pf, n, s->o->viscosity_model, s->o->mu, s->o->prandtl, vflux);
      for (int k = 0; k < 5; ++k) contrib[k] = -flux[k] + vflux[k];
    }
    for (int k = 0; k < 5; ++k) {
      if (s->cf)  /* Extrapolate_BC.h:94-99 and the other BC functors */
        s->cf_flux[slot5(c, bf->flux_index[2 * i]) + k] = contrib[k];
      else
        atomic_add_d(&s->cell_flux[5 * c + k], contrib[k], s->par);
    }
  }
}

/* Flux.h:188-229 */
static void apply_cell_flux(ostate* s) {
  const int C = s->m->ncells;
  const double dt = s->o->dt;
  PFOR
  for (int i = 0; i < C; ++i)
    for (int k = 0; k < 5; ++k) {
      double r = 0.0;
      if (s->cf)  /* one term per slot, in slot order */
        for (int slot = 0; slot < NSLOTS; ++slot) r = r + dt / s->m->cell_volumes[i] * s->cf_flux[slot5(i, slot) + k];
      else
        r = r + dt / s->m->cell_volumes[i] * s->cell_flux[5 * i + k];
      s->res[5 * i + k] = r;
    }
}

void oracle_free(oracle_state* h);

struct oracle_state {
  ostate s;
  double* pool;
  double* cf_pool;
  double* Un;
};

oracle_state* oracle_create(const oracle_mesh* m, const oracle_options* o, const double* U0, int nthreads) {
  if (!m || !o || !U0 || m->ncells <= 0) return NULL;
  const size_t C = (size_t)m->ncells;
  oracle_state* h = (oracle_state*)calloc(1, sizeof(oracle_state));
  if (!h) return NULL;
  h->pool = (double*)calloc(C * (5 * 10 + 15 * 2), sizeof(double));
  if (!h->pool) { free(h); return NULL; }
  ostate* s = &h->s;
  s->m = m;
  s->o = o;
  s->nt = nthreads > 0 ? nthreads : 1;
  s->par = s->nt > 1;
  double* q = h->pool;
  h->Un = q; q += 5 * C;
  s->Un = h->Un;
  s->Unp1 = q; q += 5 * C;
  s->Utmp = q; q += 5 * C;
  s->res = q; q += 5 * C;
  s->cell_flux = q; q += 5 * C;
  s->smin = q; q += 5 * C;
  s->smax = q; q += 5 * C;
  s->slim = q; q += 5 * C;
  s->lim = q; q += 5 * C;
  q += 5 * C;
  s->cell_grad = q; q += 15 * C;
  s->grad = q; q += 15 * C;
  memcpy(s->Un, U0, sizeof(double) * 5 * C);
  memcpy(s->Unp1, s->Un, sizeof(double) * 5 * C);    /* copy (TimeSolverExplicitRK4.h:335) */
  s->cf = o->cell_flux != 0;
  if (s->cf) {
    /* CELL_FLUX needs every non-empty face set's flux_index. */
    int missing = m->internal.nfaces > 0 && !m->internal.flux_index;
    for (int b = 0; b < m->nbc; ++b) missing |= m->bc[b].nfaces > 0 && !m->bc[b].flux_index;
    if (missing) { oracle_free(h); return NULL; }
    h->cf_pool = (double*)calloc(C * NSLOTS * (5 * 4 + 15), sizeof(double));
    if (!h->cf_pool) { oracle_free(h); return NULL; }
    double* r = h->cf_pool;
    s->cf_flux = r; r += NSLOTS * 5 * C;
    s->cf_min = r; r += NSLOTS * 5 * C;
    s->cf_max = r; r += NSLOTS * 5 * C;
    s->cf_lim = r; r += NSLOTS * 5 * C;
    s->cf_grad = r;
  }
  return h;
}

void oracle_step(oracle_state* h, int nsteps) {
  static const double alpha[4] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0};
  static const double beta[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
  static const int type_order[4] = {0, 1, 3, 2};  /* Extrapolate, Tangent, NoSlip, Inflow */
  ostate* s = &h->s;
  const oracle_mesh* m = s->m;
  const oracle_options* o = s->o;
  const size_t C = (size_t)m->ncells;
  for (int step = 1; step <= nsteps; ++step) {                 /* Solve loop, :340-491 */
    for (int irk = 0; irk < 4; ++irk) {
      update(s, alpha[irk], s->res, s->Un, s->Utmp);
      zero_cell_flux(s);
      if (o->second_order || o->viscous) green_gauss(s);
      if (o->second_order) {
        min_max(s);
        limiter(s);
      }
      internal_flux(s);
      for (int t = 0; t < 4; ++t)
        for (int b = 0; b < m->nbc; ++b)
          if (m->bc[b].type == type_order[t]) bc_flux(s, &m->bc[b]);
      apply_cell_flux(s);
      update(s, beta[irk], s->res, s->Unp1, s->Unp1);
    }
    memcpy(s->Un, s->Unp1, sizeof(double) * 5 * C);
  }
}

void oracle_get_state(const oracle_state* h, double* U, double* res) {
  const size_t C = (size_t)h->s.m->ncells;
  if (U) memcpy(U, h->s.Un, sizeof(double) * 5 * C);
  if (res) memcpy(res, h->s.res, sizeof(double) * 5 * C);
}

void oracle_free(oracle_state* h) {
  if (!h) return;
  free(h->pool);
  free(h->cf_pool);
  free(h);
}

int oracle_solve(const oracle_mesh* m, const oracle_options* o, double* U, double* res_out, int nthreads) {
  oracle_state* h = oracle_create(m, o, U, nthreads);
  if (!h) return 1;
  oracle_step(h, o->nsteps);
  oracle_get_state(h, U, res_out);
  oracle_free(h);
  return 0;
}

/* Initial_Conditions.h:38-96 */
void oracle_init_sod_reference(const oracle_mesh* m, double midx, double* U) {
  const double Rgas = 287.05, gamma = 1.4;
  const double Cv = Rgas / (gamma - 1.0);
  const double P1 = 68947.57, T1 = 288.889, P2 = 6894.757, T2 = 231.11;
  const double d1 = P1 / (Rgas * T1), e1 = d1 * (Cv * T1);
  const double d2 = P2 / (Rgas * T2), e2 = d2 * (Cv * T2);
  for (int i = 0; i < m->ncells; ++i) {
    const int left = m->cell_coords[3 * i] < midx;
    U[5 * i] = left ? d1 : d2;
    U[5 * i + 1] = 0.0;
    U[5 * i + 2] = 0.0;
    U[5 * i + 3] = 0.0;
    U[5 * i + 4] = left ? e1 : e2;
  }
}

void oracle_init_constant(const oracle_mesh* m, const double st[5], double* U) {
  for (int i = 0; i < m->ncells; ++i)
    for (int k = 0; k < 5; ++k) U[5 * i + k] = st[k];
}

/* ---- drivers one at a time (unit parity of the device operator entry points) ---- */
static const int bc_type_order[4] = {0, 1, 3, 2};  /* Extrapolate, Tangent, NoSlip, Inflow */

static oracle_state* field_state(const oracle_mesh* m, const oracle_options* o, oracle_options* serial,
                                 const double* U) {
  *serial = *o;
  serial->cell_flux = 0;
  oracle_state* h = oracle_create(m, serial, U, 1);
  if (!h) return NULL;
  memcpy(h->s.Utmp, U, sizeof(double) * 5 * (size_t)m->ncells);
  zero_cell_flux(&h->s);
  return h;
}

/* GreenGauss::compute_gradients (GreenGauss.h:300-321) */
int oracle_field_gradients(const oracle_mesh* m, const oracle_options* o, const double* U, double* grad) {
  oracle_options so;
  oracle_state* h = field_state(m, o, &so, U);
  if (!h) return 1;
  green_gauss(&h->s);
  memcpy(grad, h->s.grad, sizeof(double) * 15 * (size_t)m->ncells);
  oracle_free(h);
  return 0;
}

/* StencilLimiter::compute_min_max + compute_limiter (StencilLimiter.h:532-616) */
int oracle_field_limiter(const oracle_mesh* m, const oracle_options* o, const double* U, double* phi) {
  oracle_options so;
  oracle_state* h = field_state(m, o, &so, U);
  if (!h) return 1;
  green_gauss(&h->s);
  min_max(&h->s);
  limiter(&h->s);
  memcpy(phi, h->s.lim, sizeof(double) * 5 * (size_t)m->ncells);
  oracle_free(h);
  return 0;
}

/* The BC functors in Solve's order (TimeSolverExplicitRK4.h:428-475) */
int oracle_field_bc_flux(const oracle_mesh* m, const oracle_options* o, const double* U, double* cell_flux) {
  oracle_options so;
  oracle_state* h = field_state(m, o, &so, U);
  if (!h) return 1;
  for (int t = 0; t < 4; ++t)
    for (int b = 0; b < m->nbc; ++b)
      if (m->bc[b].type == bc_type_order[t]) bc_flux(&h->s, &m->bc[b]);
  memcpy(cell_flux, h->s.cell_flux, sizeof(double) * 5 * (size_t)m->ncells);
  oracle_free(h);
  return 0;
}
