/*
 * CPU oracle for the miniAero explicit RK4 residual path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * Kokkos functors (kokkos/Flux.h, Roe_Flux.h, Viscous_Flux.h, GreenGauss.h,
 * StencilLimiter.h, VenkatLimiter.h, VanAlbadaLimiter.h, *_BC.h,
 * TimeSolverExplicitRK4.h). It is the checker for the CUDA path and the timed
 * CPU baseline; nothing in the product links or calls it.
 *
 * Loop structure and accumulation order follow the reference face loops:
 * with nthreads == 1 every accumulator is summed in the serial order of the
 * reference's Kokkos Serial execution (the parity oracle); with nthreads > 1
 * the loops run under OpenMP with atomic updates, like the reference's
 * Kokkos OpenMP build (nondeterministic summation order, timing only).
 */
#ifndef MINIAERO_ORACLE_H_
#define MINIAERO_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* One face list, fields as in kokkos/Faces.h:42-71 (LayoutRight). */
typedef struct {
  int nfaces;
  int type;                 /* 0 Extrapolate, 1 Tangent, 2 Inflow, 3 NoSlip; -1 internal */
  const int* conn;          /* [nfaces*2] (left, right); right unused on boundaries */
  const double* coords;     /* [nfaces*3] */
  const double* normal;     /* [nfaces*3] area vector */
  const double* tangent;    /* [nfaces*3] */
  const double* binormal;   /* [nfaces*3] */
  const int* permutation;   /* [nfaces] iteration order */
  const int* flux_index;    /* [nfaces*2] element-local face slots of (left, right)
                               (Faces.h:109-110); read in CELL_FLUX mode only */
} oracle_faces;

typedef struct {
  int ncells;
  const double* cell_coords;   /* [ncells*3] */
  const double* cell_volumes;  /* [ncells] */
  oracle_faces internal;
  int nbc;
  const oracle_faces* bc;      /* in the reference's boundary_faces order */
} oracle_mesh;

typedef struct {
  int second_order;      /* Options::second_order_space */
  int viscous;           /* Options::viscous */
  int limiter;           /* 0 Venkatakrishnan (reference), 1 Van Albada */
  int viscosity_model;   /* 0 Sutherland (reference), 1 constant mu */
  double mu;             /* constant viscosity (model 1) */
  double prandtl;        /* Prandtl number (model 1) */
  double dt;
  int nsteps;
  double inflow_state[5];/* conserved inflow state (TimeSolverExplicitRK4.h:218-223) */
  int cell_flux;         /* 1: the reference's -DCELL_FLUX build (per-slot storage,
                            gathers in slot order); 0: its default -DATOMICS_FLUX */
} oracle_options;

/* Advances U (conserved, [ncells*5], in/out) by opts->nsteps RK4 steps.
 * res_out, when not NULL, receives the last stage residual [ncells*5].
 * Returns 0 on success, nonzero on bad arguments. */
int oracle_solve(const oracle_mesh* mesh, const oracle_options* opts, double* U, double* res_out,
                 int nthreads);

/* Persistent solver state for step-by-step use (timing). The mesh and options
 * must outlive the state. */
typedef struct oracle_state oracle_state;
oracle_state* oracle_create(const oracle_mesh* mesh, const oracle_options* opts, const double* U0, int nthreads);
void oracle_step(oracle_state* h, int nsteps);
void oracle_get_state(const oracle_state* h, double* U, double* res);
void oracle_free(oracle_state* h);

/* Reference Sod initial condition (Initial_Conditions.h:38-96) on U[ncells*5]. */
void oracle_init_sod_reference(const oracle_mesh* mesh, double midx, double* U);

/* Constant conserved state (Initial_Conditions.h:103-133). */
void oracle_init_constant(const oracle_mesh* mesh, const double state[5], double* U);

/* Scalar operators, exposed for unit checks. */
void oracle_roe_flux(const double* pl, const double* pr, const double* n, const double* t,
                     const double* b, double* flux);
void oracle_viscous_flux(const double grad[5][3], const double* prim, const double* a,
                         int viscosity_model, double mu, double prandtl, double* vflux);
double oracle_venkat(double dumax, double dumin, double du, double deltax2);
double oracle_vanalbada(double dumax, double dumin, double du);
void oracle_primitives(const double* U, double* V);

/* One RK stage's drivers taken one at a time on a state U ([ncells*5]; the
 * stage state U_tmp of Solve), in the serial ATOMICS_FLUX order. Return 0 on
 * success. grad [ncells*15] (cell, component, direction), phi and cell_flux
 * [ncells*5]. */
int oracle_field_gradients(const oracle_mesh* mesh, const oracle_options* opts, const double* U, double* grad);
int oracle_field_limiter(const oracle_mesh* mesh, const oracle_options* opts, const double* U, double* phi);
int oracle_field_bc_flux(const oracle_mesh* mesh, const oracle_options* opts, const double* U, double* cell_flux);

#ifdef __cplusplus
}
#endif
#endif
