/*
 * iemic_gb300.h -- C ABI of the GB300 THCM Newton-step engine.
 *
 * One opaque handle stands in for the reference's `Ocean` model object
 * (src/ocean/Ocean.H:169-250, a `Model` from src/utils/Model.H:54-145) and the
 * `THCM` singleton below it (src/ocean/THCM.H). Every call returns an int
 * status (0 = success, negative = error, see IEMIC_ERR_*), never aborts and
 * throws nothing across the boundary. Host arrays are borrowed for the
 * duration of a call; device buffers are owned by the handle. Calls on one
 * handle are serialised on its own CUDA stream; a handle is not thread-safe.
 *
 * Vector layout is the reference's: cell-interleaved unknowns
 * row = 6*(i + n*j + n*m*k) + (XX-1), 0-based i,j,k, XX in {u,v,w,p,T,S}
 * (src/ocean/matetc.F90:123-144; src/trios/THCMdefs.H FIND_ROW2).
 * The Jacobian is the reference's solver-facing matrix: the state-independent
 * "maximal graph" of src/ocean/THCM.C:2300-2580 (sorted columns, explicit
 * zeros) holding the Fortran `matrix` coefficients (src/ocean/usrc.F90:449-521)
 * that survive the |c| > 1e-10 drop rule of src/ocean/assemble.F90:115.
 */
#ifndef IEMIC_GB300_H
#define IEMIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    IEMIC_OK = 0,
    IEMIC_ERR_ARG = -1,            /* bad argument (null handle, size out of range) */
    IEMIC_ERR_CUDA = -2,           /* a CUDA runtime call failed */
    IEMIC_ERR_NOT_CONVERGED = -3,  /* Krylov/Newton iteration cap reached above tolerance */
    IEMIC_ERR_NAN = -4,            /* a NaN/Inf appeared in a residual or update */
    IEMIC_ERR_ZERO_PIVOT = -5,     /* factorisation met pivots it had to perturb beyond its budget */
    IEMIC_ERR_STATE = -6,          /* call order violated (e.g. solve before jacobian) */
    IEMIC_ERR_NOMEM = -7           /* device allocation failed */
};

/* THCM init keys used by this path (src/ocean/THCM.C:180-260 and the
 * "Starting Parameters" handled through iemic_set_par). */
typedef struct {
    int n, m, l;                   /* "Global Grid-Size n/m/l" */
    double xmin_deg, xmax_deg;     /* "Global Bound xmin/xmax" */
    double ymin_deg, ymax_deg;     /* "Global Bound ymin/ymax" */
    int periodic;                  /* "Periodic" */
    double hdim;                   /* "Depth hdim" */
    double qz;                     /* "Grid Stretching qz" */
    double alphaT, alphaS;         /* "Linear EOS: alpha T/S" */
    int ih;                        /* "Inhomogeneous Mixing" */
    int coriolis_on;               /* "Coriolis Force" */
    int tres, sres;                /* "Restoring Temperature/Salinity Profile" */
    int iza;                       /* "Wind Forcing Type": 2 idealized, else injected taux/tauy */
    int ite, its;                  /* "Levitus T/S": 1 idealized, else injected tatm/emip */
    int forcing_type;              /* "Forcing Type" */
    int vmix;                      /* "Mixing" (vmix_GLB, src/ocean/mix_imp.f): 0 off, 1 fixed partition,
                                      2 partition adapted to the T/S fields (Ocean::computeRHS and
                                      computeJacobian re-evaluate it every call). The implicit vertical
                                      mixing / convective adjustment (P_VC) and consistent vertical mixing
                                      (ALPC < 1) terms run on the GPU; neutral physics and Gent-McWilliams
                                      (MIXP, MKAP nonzero) are not implemented: rhs and jacobian return
                                      IEMIC_ERR_ARG while either is nonzero with Mixing >= 1. */
    int rho_mixing;                /* "Rho Mixing" */
    int tap;                       /* "Taper" (tap of src/ocean/usr.F90; used by neutral physics only) */
    int sint_sign;                 /* "Salinity Integral Sign" (-1 or 1; 0 is taken as -1). With sres = 0
                                      the S row of cell (intcon_i, intcon_j, l-1) holds the integral
                                      condition sint_sign * sum_cells cos(y_j) dfzT(k) S (THCM::intcond_S,
                                      src/ocean/THCM.C:2180-2257): a dense row of the Jacobian over every S
                                      unknown, F = sint_sign * (that sum), and the net salt flux of the
                                      forcing is removed (qint, src/ocean/forcing.F90:121-160). */
    int intcon_i, intcon_j;        /* "Integral row coordinate i/j" (0-based; -1: n-1, m-1); must be ocean */
    int fix_pressure_points;       /* "Fix Pressure Points": the continuity rows of the surface pressures
                                      (n-1, m-1) and (n-2, m-1) become identity rows, F = 0 there
                                      (THCM::fixPressurePoints, THCM.C:2260-2297) */
} iemic_config;

typedef struct iemic_ocean iemic_ocean;

/* Replaces THCM::THCM + Ocean::Ocean (src/ocean/THCM.C:180-795,
 * src/ocean/Ocean.C:63-213). landm: (n+2)(m+2)(l+2) ints in the readmask
 * layout of src/ocean/topo.F90:41-60 (i fastest, 0 ocean, 1 land, 3 periodic
 * border), or NULL for "Topography" = 1 (no continents). */
int iemic_create(const iemic_config* cfg, const int* landm, iemic_ocean** out);
int iemic_destroy(iemic_ocean* h);
int iemic_ndim(const iemic_ocean* h, int* ndim);
/* landm as the model uses it after THCM's init fix-ups (usrc.F90:79-107). */
int iemic_get_landm(const iemic_ocean* h, int* landm);

/* Ocean::setPar / THCM::setParameter -> Fortran setparcs (usrc.F90:163-181):
 * par(idx) = value, then forcing + lin are recomputed. idx is 1..30. */
int iemic_set_par(iemic_ocean* h, int idx, double value);
int iemic_get_par(const iemic_ocean* h, int idx, double* value);
/* m_inserts injection (src/ocean/inserts.F90:12-247; THCM::setTaux etc.):
 * n*m fields, i fastest; NULL leaves a field unchanged. */
int iemic_set_forcing(iemic_ocean* h, const double* taux, const double* tauy,
                      const double* tatm, const double* emip, const double* spert);

/* Ocean::computeRHS -> THCM::evaluate(rhs) (THCM.C:993-1042): F = -B of
 * Fortran rhs (usrc.F90:523-603). Host vectors of length ndim. */
int iemic_rhs(iemic_ocean* h, const double* x, double* F);
/* Ocean::computeJacobian -> THCM::evaluate(jac) (THCM.C:1043-1199). */
int iemic_jacobian(iemic_ocean* h, const double* x);
/* Same on device pointers (no host copies). */
int iemic_rhs_dev(iemic_ocean* h, const double* x_dev, double* F_dev);
int iemic_jacobian_dev(iemic_ocean* h, const double* x_dev);

/* iemic_rhs_dev without per-handle scratch (no reference counterpart): the
 * padded state fields live in one static device array of
 * IEMIC_NOALLOC_MAX_PADDED_CELLS cells per field; grids with
 * (n+2)(m+2)(l+2) above it are rejected (IEMIC_ERR_ARG). Allocates nothing.
 * The first call for a device looks the array up (cudaGetSymbolAddress, with
 * the handle's device made current) and must not run during stream capture.
 * Runs on the handle's stream and, like iemic_rhs_dev, returns after that
 * work has finished. Calls overlapping in time on one device (several host
 * threads) race on the shared array. */
#define IEMIC_NOALLOC_MAX_PADDED_CELLS 65536
int iemic_rhs_dev_noalloc(iemic_ocean* h, const double* x_dev, double* F_dev);

/* Ocean::getJacobian: the CSR of the maximal graph, 0- or 1-based. */
int iemic_graph_nnz(const iemic_ocean* h, int64_t* nnz);
int iemic_get_csr(iemic_ocean* h, int* row_ptr, int* col_idx, double* values, int index_base);
/* Ocean::applyMassMat diagonal, fillcolB (src/ocean/assemble.F90:18-54). */
int iemic_mass(iemic_ocean* h, double* diagB);
/* Ocean::applyMatrix: out = J v (FP64). */
int iemic_apply_matrix(iemic_ocean* h, const double* v, double* out);

/* Linear solve options / statistics (Ocean::solve, Ocean.C:1070-1147). */
enum { IEMIC_PREC_FP64 = 0, IEMIC_PREC_MIXED = 1 };
typedef struct {
    int precision;         /* IEMIC_PREC_FP64: FP64 GMRES + FP64 factors;
                              IEMIC_PREC_MIXED: FP64 GMRES + FP32 factors (compensated solves) */
    int restart;           /* GMRES restart length ("FGMRES iterations") */
    int max_iters;         /* cap on total inner iterations */
    double tol;            /* relative residual target ||b - J x|| / ||b|| */
    int transpose;         /* 0: J x = b, 1: J^T x = b (adjoint solve) */
    int reuse_preconditioner; /* 0: refactor when J changed since the last factorisation;
                                 1: keep the existing factorisation (the reference recomputes its
                                 preconditioner once per continuation step, Ocean::preProcess) */
} iemic_solve_opts;
typedef struct {
    int iters;             /* total inner Krylov iterations */
    int factorizations;    /* preconditioner (re)builds performed by this call */
    int perturbed_pivots;  /* pivots the last factorisation had to perturb */
    double relres;         /* final FP64 ||b - J x|| / ||b|| */
    double time_factor_ms; /* time spent (re)building the preconditioner */
    double time_solve_ms;  /* time spent in the Krylov solve */
} iemic_solve_stats;
void iemic_default_solve_opts(iemic_solve_opts* o);

/* Ocean::buildPreconditioner / BlockPreconditioner::Compute: factor the
 * current Jacobian (precision as in opts->precision; both if -1). */
int iemic_build_preconditioner(iemic_ocean* h, int precision);
/* Ocean::applyPrecon: out = M^{-1} v with the current factorisation. */
int iemic_apply_precon(iemic_ocean* h, int precision, const double* v, double* out);
/* The gauge of J's null space (no reference counterpart: the reference's
 * Belos/Ifpack solve leaves it implicit). J is singular (hydrostatic B-grid
 * pressure modes per basin); every solution the solver returns has exactly
 * zero pressure at these unknowns, and their (redundant) continuity rows are
 * satisfied through the others for consistent right-hand sides. With
 * capacity 0 only *count is set. */
int iemic_solver_gauge(iemic_ocean* h, int* idx, int capacity, int* count);
/* Size of the preconditioner's nested-dissection factorisation (no
 * reference counterpart). factor_entries: entries the triangular solves read
 * (the factor store; per precision multiply by 4 or 8 bytes); front_entries:
 * the dense F x F fronts of all levels together; work_entries: the working
 * area (fronts of the largest level); contrib_entries: the ring of
 * contribution blocks; factor_flops: flops of one LU (without the explicit
 * inverses). Device storage of one precision is about (factor_entries +
 * work_entries + contrib_entries) entries. */
typedef struct {
    int64_t unknowns, reduced_unknowns, fronts, levels, factor_entries, front_entries;
    double factor_flops;
    int64_t work_entries, contrib_entries;
} iemic_solver_info;
int iemic_get_solver_info(iemic_ocean* h, iemic_solver_info* out);
/* The same size report from the host-side symbolic analysis alone (no device
 * work, no handle): grid from cfg (n, m, l, periodic), the land mask as the
 * engine holds it ((n+2)(m+2)(l+2) entries, iemic_get_landm) and the 0-based
 * CSR pattern of J (row_ptr: 6nml + 1 entries). The plan's offsets and maps
 * are checked for consistency; IEMIC_ERR_STATE if one fails. */
int iemic_analyse_pattern(const iemic_config* cfg, const int* landm, const int* row_ptr, const int* col_idx,
                          iemic_solver_info* out);
/* Triangular solves of the preconditioner: a factorisation whose fronts have
 * at most `max_inverse_nf` own unknowns (default 12288) stores the whole
 * inverses of their diagonal triangles and applies them as GEMVs; a larger one
 * substitutes over inverted 256-row diagonal blocks (more sequential steps,
 * rounding bounded by the blocks' condition instead of the whole triangle's).
 * A change discards the current factorisations. */
int iemic_set_substitution_threshold(iemic_ocean* h, int max_inverse_nf);
/* The elimination tree of the nested-dissection factorisation: per front its
 * own unknowns nf, boundary unknowns nb, level (0 = leaves) and parent (-1 at
 * the root). Copies up to `cap` fronts; *count receives the number of fronts. */
int iemic_get_fronts(iemic_ocean* h, int cap, int* nf, int* nb, int* level, int* parent, int* count);
/* Ocean::solve(rhs): x = J^{-1} b (host vectors). */
int iemic_solve(iemic_ocean* h, const double* b, double* x, const iemic_solve_opts* o,
                iemic_solve_stats* st);
int iemic_solve_dev(iemic_ocean* h, const double* b_dev, double* x_dev, const iemic_solve_opts* o,
                    iemic_solve_stats* st);

/* Newton iteration at fixed parameters (Newton<Model>::Run / RunBackTracking,
 * src/newton/Newton.H:40-100): x += dx with J dx = -F until ||F||_2 < tol,
 * halving back-tracking whenever the residual norm grew. */
typedef struct {
    int max_iters;            /* maxNumIterations_ (10) */
    double tol;               /* toleranceRHS_ on ||F||_2 (1e-3) */
    int backtracking_steps;   /* numBackTrackingSteps_ (10) */
    iemic_solve_opts solve;
    int refactor_each_iter;   /* 1: new preconditioner every iteration; 0: the first one is kept;
                                 2: kept while the Krylov time it costs beyond its first solve stays
                                 below its own factorisation time, then rebuilt (see below) */
} iemic_newton_opts;
typedef struct {
    int iters, backtracks, linear_solves, krylov_iters, factorizations;
    double rhs_norm0, rhs_norm;
    double time_ms, time_assembly_ms, time_factor_ms, time_solve_ms;
} iemic_newton_stats;
void iemic_default_newton_opts(iemic_newton_opts* o);
int iemic_newton(iemic_ocean* h, double* x, const iemic_newton_opts* o, iemic_newton_stats* st);
int iemic_newton_dev(iemic_ocean* h, double* x_dev, const iemic_newton_opts* o, iemic_newton_stats* st);

/* One implicit time step of the theta method, ThetaModel<Ocean>
 * (src/transient/ThetaModel.H:64-140) solved by the transient Newton
 * iteration (src/transient/Newton.H:77-110). From x_old = x (in/out):
 *   G(x) = B (x_old - x) + dt theta F(x) + dt (1 - theta) F(x_old)
 *   J2   = J - B / (theta dt),   J2 dx = G / (theta dt),   x -= dx
 * with B the diagonal mass matrix (iemic_mass), until ||dx||_inf < tol and
 * ||G||_2 < tol; ||dx||_inf > 1e2 stops the iteration as diverging. The
 * preconditioner follows `refactor_policy` (0: rebuilt once per time step, as
 * ThetaModel::initStep calls Ocean::preProcess; 1: every iteration; 2: as
 * refactor_each_newton = 2). Each linear solve runs to the relative
 * tolerance solve.tol, relaxed to 0.1 tol / ||G||_2 when that is larger (the
 * Newton test needs no more; near convergence G is at round-off level).
 * theta must lie in (0, 1]: the explicit theta = 0
 * division by B is not offered (B vanishes on land and pressure rows). The
 * Jacobian left in the handle afterwards is J2 of the last iterate. */
typedef struct {
    double theta;             /* "theta" (1: backward Euler) */
    double dt;                /* time step (the reference's timestep_) */
    double tol;               /* "Newton tolerance" (1e-8) */
    int max_newton;           /* "maximum Newton iterations" (20) */
    iemic_solve_opts solve;
    int refactor_policy;      /* 0, 1 or 2 (default 2) */
} iemic_theta_opts;
typedef struct {
    int newton_iters, converged, linear_solves, krylov_iters, factorizations;
    double norm_G, norm_dx;   /* ||G||_2 and ||dx||_inf of the last iteration */
    double time_ms, time_assembly_ms, time_factor_ms, time_solve_ms;
} iemic_theta_stats;
void iemic_default_theta_opts(iemic_theta_opts* o);
/* IEMIC_ERR_NOT_CONVERGED: the iteration cap was reached or it diverged;
 * x then holds the last iterate. */
int iemic_theta_step(iemic_ocean* h, double* x, const iemic_theta_opts* o, iemic_theta_stats* st);
int iemic_theta_step_dev(iemic_ocean* h, double* x_dev, const iemic_theta_opts* o, iemic_theta_stats* st);

/* Pseudo-arclength continuation (Continuation<Model>::run,
 * src/continuation/Continuation.H:209-1115). Field names follow the
 * reference's "Continuation parameters" list; defaults
 * (iemic_default_continuation_opts) are those of getDefaultInitParameters.
 * The state advances in place; the model's parameter par_idx ends at the
 * last accepted point. Returns IEMIC_ERR_NOT_CONVERGED when the run aborted
 * at the minimum step size. */
typedef struct {
    int par_idx;              /* "continuation parameter": par(1..30), e.g. 15 "Salinity Forcing" */
    double ds, ds_min, ds_max;/* "initial/minimum/maximum step size" */
    double decrease;          /* "decrease step size": a failed step divides ds by it */
    double destination;       /* "destination 0" */
    double destination_tol;   /* "destination tolerance" */
    int max_steps;            /* "maximum number of steps" (-1: until the destination) */
    int max_newton;           /* "maximum Newton iterations" */
    int min_newton;           /* "minimum Newton iterations" */
    double opt_newton;        /* "optimal Newton iterations" (Seydel step control) */
    double newton_tol;        /* "Newton tolerance" */
    char residual_test;       /* "corrector residual test": 'R' ||F||_2, 'D' max(|dpar|, ||dx||_inf) */
    char normalize;           /* "normalize strategy": 'O' or 'N' */
    char tangent;             /* "tangent type": 'E' Euler, 'S' secant */
    char initial_tangent;     /* "initial tangent type": 'E' (solve) or 'A' (-dF/dpar) */
    double epsilon;           /* "epsilon increment" of the finite-difference dF/dpar */
    double tan_scaling;       /* "state tangent scaling" */
    double predictor_bound;   /* "predictor bound" on ||F||_2 */
    int backtracking_steps;   /* "backtracking steps" (0: off) */
    double backtracking_increase; /* "backtracking increase" */
    int newton_chord;         /* "enable Newton Chord hybrid solve" */
    int give_up_at_ds_min;    /* "give up at minimum step size" */
    iemic_solve_opts solve;
    int refactor_each_newton; /* 0: preconditioner rebuilt once per step (Ocean::preProcess);
                                 1: rebuilt after every new Jacobian;
                                 2: once per step, plus a rebuild on the current Jacobian as soon as
                                    the Krylov time spent beyond the first solve's iteration count
                                    exceeds the factorisation's own time; a solve on an older
                                    Jacobian's factors gets only the iterations that budget still
                                    pays for, and is repeated on fresh factors if it runs out; after
                                    such a failure the step's later Jacobians are factorised directly
                                    when fresh factors need >= 8 iterations (inexact FP32 factors).
                                 Setting IEMIC_SOLVE_TRACE=1 in the environment prints one line per
                                 solve and per step to stderr. */
} iemic_continuation_opts;
typedef struct {
    int steps, failed_steps, newton_iters, linear_solves, unconverged_solves, krylov_iters, factorizations;
    int reached_destination, aborted;
    double par, ds, rhs_norm;
    double time_ms, time_assembly_ms, time_factor_ms, time_solve_ms;
} iemic_continuation_stats;
void iemic_default_continuation_opts(iemic_continuation_opts* o);
int iemic_continuation_run(iemic_ocean* h, double* x, const iemic_continuation_opts* o,
                           iemic_continuation_stats* st);
int iemic_continuation_run_dev(iemic_ocean* h, double* x_dev, const iemic_continuation_opts* o,
                               iemic_continuation_stats* st);

/* ---- adjoint -----------------------------------------------------------
 * Ocean::getPsiM (src/ocean/Ocean.C:882-896; OceanGrid::recomputePsiM,
 * src/ocean/OceanGrid.C:268-340; compute_psim, src/ocean/thcm_utils.F90:95-118):
 * the meridional overturning streamfunction psi(j,k), (m+1)(l+1) values
 * psim[(m+1)k + j], and its extrema, in Sv. */
int iemic_psim(iemic_ocean* h, const double* x, double* psim, double* psi_min, double* psi_max);
/* No reference counterpart (the adjoint is new): g = max psi over the
 * longitude sector [i_begin, i_end) and dg/dx (device vector); jk[0..1] =
 * (j, k) of the maximum. */
int iemic_psim_max_grad_dev(iemic_ocean* h, const double* x_dev, int i_begin, int i_end, double* g, int* jk,
                            double* grad_dev);
/* -lambda^T dF/d(surface field) for the 5 fields taux, tauy, tatm, emip,
 * spert of iemic_set_forcing (5*n*m values, field-major, i fastest): the
 * gradient of g with respect to the forcing when J^T lambda = dg/dx. */
int iemic_forcing_adjoint_dev(iemic_ocean* h, const double* lambda_dev, double* grad_dev);
/* -lambda^T dF/dpar(par_idx) by central differences (step fd_rel max(1,|par|)). */
int iemic_par_adjoint_dev(iemic_ocean* h, const double* x_dev, const double* lambda_dev, int par_idx, double fd_rel,
                          double* out);
typedef struct {
    int i_begin, i_end;        /* longitude sector of the overturning sum; i_end < 0: to n */
    iemic_solve_opts solve;    /* the transposed solve (transpose is set by the call) */
    double fd_rel;             /* relative step of the parameter central differences */
} iemic_adjoint_opts;
typedef struct {
    double g;                  /* max psi (Sv) */
    int jmax, kmax;            /* where it is attained */
    int iters;                 /* Krylov iterations of the J^T solve */
    double relres;             /* its FP64 relative residual */
    double time_ms;
} iemic_adjoint_stats;
void iemic_default_adjoint_opts(iemic_adjoint_opts* o);
/* Gradient of g = max psi (Sv) at a steady state x (host, F(x) = 0) with
 * respect to the surface forcing fields (grad_fields: 5*n*m host values or
 * NULL) and the parameters par_idx[0..npar) (grad_par), by one transposed
 * solve J^T lambda = dg/dx preconditioned with the factorisation of J. */
int iemic_adjoint_psim(iemic_ocean* h, const double* x, const iemic_adjoint_opts* o, double* grad_fields,
                       const int* par_idx, int npar, double* grad_par, iemic_adjoint_stats* st);

/* Device timing of the instrumented kernel classes (no reference
 * counterpart; it plays the role of the reference's TIMER_START/STOP
 * profile, src/globaldefs/GlobalDefinitions.H:193-223). enable = 1 clears the
 * counters and starts recording CUDA events around every launch of the
 * classes below on the handle's stream; enable = 0 stops. bytes/flops are
 * the launches' algorithmic bytes and flops. */
enum {
    IEMIC_KC_FACTOR_GEMM = 0,   /* trailing-update GEMM of the block LU */
    IEMIC_KC_SOLVE_GEMV = 1,    /* triangular-solve GEMV sweeps of the preconditioner */
    IEMIC_KC_ASSEMBLY = 2,      /* Jacobian / residual assembly */
    IEMIC_KC_SPMV = 3,          /* CSR SpMV and residual of the Krylov solver */
    IEMIC_KC_FACTOR_PANEL = 4,  /* panel LU, row permutations and L21 of the block LU */
    IEMIC_KC_FACTOR_INVERSE = 5,/* explicit triangular inverses and G, H of the fronts */
    IEMIC_KC_FACTOR_SETUP = 6,  /* equilibration, front assembly and extend-add */
    IEMIC_KC_SOLVE_OTHER = 7,   /* gathers, reductions and scatter of the triangular solves */
    IEMIC_KC_COUNT = 8
};
typedef struct {
    long long launches;
    double ms, bytes, flops;
} iemic_kernel_stats;
int iemic_kernel_timing(iemic_ocean* h, int enable);
int iemic_kernel_stats_get(iemic_ocean* h, int kclass, iemic_kernel_stats* out);
/* Timing records the runtime could not time since timing was enabled. */
long long iemic_kernel_timing_failures(iemic_ocean* h);
/* Per-launch trace since timing was enabled, in completion order: kernel class,
 * device time (ms) and algorithmic bytes of each timed launch. Copies up to
 * `cap` entries; *count receives the number recorded (at most 2^20). */
int iemic_kernel_trace(iemic_ocean* h, int cap, int* kclass, float* ms, double* bytes, int* count);
/* Kernel launches this library has made in the process so far. */
long long iemic_launch_count(void);
/* The CUDA stream (cudaStream_t) every call on this handle runs on. */
int iemic_get_stream(iemic_ocean* h, void** stream);

#ifdef __cplusplus
}
#endif
#endif
