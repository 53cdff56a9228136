// The engine object behind an iemic_ocean handle.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/iemic_gb300.h"
#include "ktimer.cuh"
#include "ocean_impl.cuh"

namespace iemic {

struct EngineError {
    int code;
    explicit EngineError(int c) : code(c) {}
};
inline void ck(cudaError_t e) {
    if (e != cudaSuccess) throw EngineError(IEMIC_ERR_CUDA);
}

struct NdLu;     // nested-dissection block factorisation (ndlu.cu)
struct NdPlan;   // its symbolic analysis
struct Krylov;   // Krylov workspace (krylov.cu)

struct Engine {
    iemic_config cfg{};
    size_t nc = 0;
    int ndim = 0;
    int64_t nnz = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;

    // host-side geometry
    double xmin = 0, xmax = 0, ymin = 0, ymax = 0, dx = 0, dy = 0, dz = 0, tdzi2 = 0;
    std::vector<double> y, yv, z, dfzT, dfzW, jt, kt, surf;
    std::vector<int> landm, row_ptr;
    std::vector<int8_t> slot;

    Params P{};
    ForcingScalars fs{};
    Geo geo{};
    Pattern pat{};

    // device buffers
    int8_t* d_lm = nullptr;
    int8_t* d_slot = nullptr;
    double *d_jt = nullptr, *d_kt = nullptr, *d_al = nullptr, *d_pads = nullptr, *d_surf = nullptr;
    double *d_x = nullptr, *d_F = nullptr, *d_v1 = nullptr, *d_v2 = nullptr, *d_B = nullptr;
    int* d_diagpos = nullptr;   // CSR position of each row's diagonal (theta method), built on first use
    int device = 0;           // the CUDA device the handle was created on
    // vertical mixing (Mixing >= 1): partition flags (device) and norm partials
    int* d_mixflags = nullptr;
    double* d_mixpart = nullptr;
    int any_ocean = 0;
    // SRES = 0: the integral condition on S in row `rowintcon` (dense over the
    // S unknowns); "Fix Pressure Points": identity rows rowPfix1/2; -1 if absent
    int rowintcon = -1, sint_sign = -1, rowPfix1 = -1, rowPfix2 = -1;
    double* d_intcoef = nullptr;   // cos(y_j) dfzT(k) per cell (0 on land), nc entries
    // Sherman-Morrison correction of the preconditioner for the dense row,
    // per factor precision [0] FP64, [1] FP32 factors: zr = M0^{-1} e_r, the
    // scalar (d.y - y_r) / alpha of the last correction, alpha itself, and
    // for transposed solves wt = M0^{-T}(d - e_r) with its generation
    double* d_zr[2] = {nullptr, nullptr};
    double* d_sm[2] = {nullptr, nullptr};   // [0] alpha, [1] scratch scalar, [2] transposed alpha
    double* d_wt[2] = {nullptr, nullptr};
    double* d_smtmp = nullptr;              // scratch vector of the set-up solves
    long fact_gen[2] = {0, 0}, wt_gen[2] = {-1, -1};
    int *d_rowptr = nullptr, *d_col = nullptr;
    double* d_val = nullptr;

    bool jac_valid = false;
    bool fact64_stale = true, fact32_stale = true;   // J changed since the last factorisation

    // solver state (krylov.cu / ndlu.cu)
    NdPlan* ndplan = nullptr;
    int subst_min_nf = 12288;  // fronts up to this size: whole inverses (ndlu_setup)
    NdLu* lu64 = nullptr;
    NdLu* lu32 = nullptr;
    Krylov* kry = nullptr;
    std::vector<int> h_col;   // host copy of the CSR column indices
    // transposed Jacobian for adjoint solves: pattern, slot map, values
    int *d_rowT = nullptr, *d_colT = nullptr, *d_permT = nullptr;
    double* d_valT = nullptr;
    bool jacT_stale = true;
    KTimer timer;             // optional per-kernel-class device timing

    ~Engine();
    void init(const iemic_config& c, const int* landm_in);
    void* dalloc(size_t bytes);
    void build_grid();
    void stpnt();
    void update_forcing();
    void lin();
    void build_pattern();
    void set_par(int idx, double value);
    void rhs_dev(const double* x, double* F);
    void jacobian_dev(const double* x);
    // mixing scalars of the current parameters; throws IEMIC_ERR_ARG for the
    // neutral-physics / Gent-McWilliams terms, which have no GPU kernels
    MixParams mix_params() const;
    // vmix_control before an rhs or jacobian (Mixing = 2); part: 2*152 doubles
    void mix_control(const double* x, double* part);
    // rows that the Fortran assembly does not produce: the integral condition
    // and the fixed pressure points (F values after the row kernels)
    void special_rows_rhs(const double* x, double* F);
    void zero_mass_rows();
    // the preconditioner of the dense-row Jacobian: M0^{-1} of the factors
    // (row rowintcon as an identity row), corrected by Sherman-Morrison
    void precond_apply(NdLu& lu, int prec, const double* v, double* z, bool transpose);
    void sm_setup(int prec);

    // linear algebra (krylov.cu)
    void spmv64(const double* x, double* y);
    void free_solver();
    void drop_factors();   // both factorisations and the Krylov workspace (keeps the plan)
    void ensure_solver();
    void build_preconditioner(int precision);
    int solve_dev(const double* b, double* x, const iemic_solve_opts& o, iemic_solve_stats& st);
    int solve_transpose_dev(const double* b, double* x, const iemic_solve_opts& o, iemic_solve_stats& st);
    void ensure_transpose();
    void apply_precon(int precision, const double* v, double* out);
    NdLu*& lu_for(int precision);
    const std::vector<int>& host_col_idx();
};

}  // namespace iemic

// the opaque handle of include/iemic_gb300.h
struct iemic_ocean {
    iemic::Engine e;
};
