// CPU oracle for the THCM Newton-step path (TEST INFRASTRUCTURE ONLY).
//
// A plain C++17 FP64 restatement of the reference's Fortran THCM kernels
// (src/ocean/usrc.F90, spf.F90, boundary.F90, assemble.F90, matetc.F90,
// grid.F90, forcing.F90) and of the C++ glue that turns their CSR output into
// the solver-facing Jacobian (src/ocean/THCM.C: evaluate, CreateMaximalGraph).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
// it; the GPU product never links or calls it.
//
// Parity status: the reference cannot be compiled here (no Fortran compiler,
// no Trilinos/MPI), and it ships no golden values for J or F entries. The
// restatement is pinned to the reference's own known-answer tests
// (src/tests/test_ocean.C: F(0)=0 at zero forcing, exact mass-matrix values,
// salt-conservation column integrals; src/tests/TestDefinitions.H: analytic
// vs finite-difference Jacobian) and to the reference-produced state of
// test/ocean/ocean_reference.h5: the steady state the reference's
// src/tests/reft_ocean.C reaches by continuation on the 16x16x16 gateway mask
// with vertical mixing (Mixing = 2), checked through the u, v, T, S norms
// that test compares.
#pragma once
#include <cstdint>

extern "C" {

// Mirrors the THCM XML keys used by this path (src/ocean/THCM.C:180-260).
typedef struct {
    int n, m, l;              // "Global Grid-Size n/m/l"
    double xmin_deg, xmax_deg; // "Global Bound xmin/xmax" (degrees)
    double ymin_deg, ymax_deg; // "Global Bound ymin/ymax" (degrees)
    int periodic;             // "Periodic"
    double hdim;              // "Depth hdim" (m)
    double qz;                // "Grid Stretching qz"
    double alphaT, alphaS;    // "Linear EOS: alpha T/S"
    int ih;                   // "Inhomogeneous Mixing"
    int coriolis_on;          // "Coriolis Force"
    int tres, sres;           // "Restoring Temperature/Salinity Profile"
    int iza;                  // "Wind Forcing Type" (2 = idealized Bryan profile, else injected)
    int ite, its;             // "Levitus T/S" (1 = idealized profile, else injected)
    int forcing_type;         // "Forcing Type"
    int vmix;                 // "Mixing" (vmix_GLB): 0 off, 1 fixed partition, 2 adaptive
    int rho_mixing;           // "Rho Mixing"
    int tap;                  // "Taper" (tap in usr.F90)
    int sint_sign;            // "Salinity Integral Sign" (-1 or 1; 0 taken as -1)
    int intcon_i, intcon_j;   // "Integral row coordinate i/j" (-1: n-1, m-1)
    int fix_pressure_points;  // "Fix Pressure Points"
} iemic_oracle_config;

void* oracle_create(const iemic_oracle_config* cfg, const int* landm);
void oracle_destroy(void* h);
int oracle_ndim(void* h);
// landm as THCM sees it after init: (n+2)*(m+2)*(l+2), i fastest, 0..n+1.
void oracle_get_landm(void* h, int* out);
// Forcing fields (n*m, i fastest); a NULL pointer leaves that field unchanged.
// Recomputes forcing + lin like setparcs (src/ocean/usrc.F90:163-181).
void oracle_set_forcing(void* h, const double* taux, const double* tauy,
                        const double* tatm, const double* emip, const double* spert);
void oracle_set_par(void* h, int idx, double value);   // par(idx), 1-based, + forcing + lin
double oracle_get_par(void* h, int idx);
void oracle_get_frc(void* h, double* out);
// Grid metrics: x(n), y(0:m+1), xu(0:n), yv(0:m), z(l), zw(0:l), dfzT(l), dfzW(0:l)
void oracle_get_grid(void* h, double* x, double* y, double* xu, double* yv,
                     double* z, double* zw, double* dfzT, double* dfzW);

// F(x) with the C++ sign convention (src/ocean/THCM.C:993-1042).
void oracle_rhs(void* h, const double* x, double* F);
// Fortran-layout CSR of the last assembled matrix (1-based, unsorted, drop rule).
int oracle_fortran_nnz(void* h);
void oracle_fortran_csr(void* h, int* beg, int* jco, double* co);
// Builds A_rhs(x) (rhs branch: nlin_rhs + boundaries + fillcolA) into the Fortran CSR.
void oracle_assemble_rhs_matrix(void* h, const double* x);

// Maximal graph (src/ocean/THCM.C:2300-2580): 0-based, sorted columns.
int64_t oracle_graph_nnz(void* h);
void oracle_graph(void* h, int* row_ptr, int* col_idx);
// J(x) scattered into the maximal graph. Returns the number of Fortran entries
// that fell outside the graph (Epetra would report them as excluded).
int oracle_jacobian(void* h, const double* x, double* values);
void oracle_mass(void* h, double* diagB);   // fillcolB (src/ocean/assemble.F90:18-54)

// psi_M(j,k), j=0..m, k=0..l (src/ocean/thcm_utils.F90:95-118; OceanGrid.C:270-330).
void oracle_psim(void* h, const double* x, double* psim);
// Atom-level access for tests: An(kk,A,B,i,j,k) after the last assembly, 1-based.
double oracle_An(void* h, int kk, int A, int B, int i, int j, int k);

// CPU FP64 Krylov baseline (same preconditioner algorithm as the GPU FP64 path).
typedef struct {
    int restart, maxit;
    double tol;
    int precond;      // 0 none, 1 point ILU(0) with pivot floor, 2 cell-block ILU(0)
    int threads;
} iemic_oracle_solve_opts;
typedef struct { int iters; double relres; double explicit_relres; int status; } iemic_oracle_solve_stats;
int oracle_gmres(int ndim, const int* row_ptr, const int* col_idx, const double* val,
                 const double* b, double* x, const iemic_oracle_solve_opts* o,
                 iemic_oracle_solve_stats* st);
}
