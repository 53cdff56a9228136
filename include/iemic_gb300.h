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
                              IEMIC_PREC_MIXED: FP32 GMRES + FP32 factors inside FP64 refinement */
    int restart;           /* GMRES restart length ("FGMRES iterations") */
    int max_iters;         /* cap on total inner iterations */
    double tol;            /* relative residual target ||b - J x|| / ||b|| */
    int max_refinements;   /* outer FP64 refinement steps (mixed only) */
    double inner_tol;      /* FP32 inner relative tolerance (mixed only) */
    int transpose;         /* 0: J x = b, 1: J^T x = b (adjoint solve) */
    int reuse_preconditioner; /* 0: refactor when J changed since the last factorisation;
                                 1: keep the existing factorisation (the reference recomputes its
                                 preconditioner once per continuation step, Ocean::preProcess) */
} iemic_solve_opts;
typedef struct {
    int iters;             /* total inner Krylov iterations */
    int factorizations;    /* preconditioner (re)builds performed by this call */
    int perturbed_pivots;  /* pivots the last factorisation had to perturb */
    int refinements;       /* outer refinement steps */
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
/* Ocean::solve(rhs): x = J^{-1} b (host vectors). */
int iemic_solve(iemic_ocean* h, const double* b, double* x, const iemic_solve_opts* o,
                iemic_solve_stats* st);
int iemic_solve_dev(iemic_ocean* h, const double* b_dev, double* x_dev, const iemic_solve_opts* o,
                    iemic_solve_stats* st);

#ifdef __cplusplus
}
#endif
#endif
