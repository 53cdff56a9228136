// Internal definitions shared by the THCM engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "stencil.cuh"

namespace iemic {

// Process-wide count of kernel launches made by this library (read through
// iemic_launch_count); every launch site is followed by IEMIC_COUNT_LAUNCH().
long long& launch_counter();
#define IEMIC_COUNT_LAUNCH() (++::iemic::launch_counter())

// Geometry tables, computed once on the host from the grid exactly as the
// Fortran atoms compute them (src/ocean/spf.F90), and uploaded. The GPU
// kernels never call transcendental functions.
enum JTab {   // per latitude row j = 0..m+1
    JT_UXX, JT_UYY4, JT_UYY6, JT_UCSI, JT_UXS2, JT_UXS8, JT_CORV, JT_PXC,
    JT_VXX, JT_VXX5, JT_VYY4, JT_VYY6, JT_VCSI, JT_VXS2, JT_VXS8, JT_PYC,
    JT_UXC, JT_VYC4, JT_VYC2, JT_TXX, JT_TYY4, JT_TYY6,
    JT_CUX, JT_CUY, JT_COSYV, JT_TANYV, JT_CTX, JT_CTY, JT_COSY,
    NJT
};
enum KTab {   // per level k = 0..l+1
    KT_UZZ14, KT_UZZ23, KT_PZ5, KT_PZ23, KT_WZC5, KT_WZC14, KT_TZZ14, KT_TZZ23,
    KT_TDZ8, KT_DFZT, KT_ZHDIM, KT_DFZW,
    NKT
};

struct Geo {
    int n, m, l, periodic;
    const int8_t* lm;      // land mask (n+2)(m+2)(l+2)
    const double* jt;      // [NJT][m+2]
    const double* kt;      // [NKT][l+2]
    double tdzi2;          // 1/(2 dz)
    double dx, dz;
    __host__ __device__ int L(int i, int j, int k) const { return lm[i + (n + 2) * (j + (m + 2) * k)]; }
    __host__ __device__ double J(int t, int j) const { return jt[t * (m + 2) + j]; }
    __host__ __device__ double K(int t, int k) const { return kt[t * (l + 2) + k]; }
    __host__ __device__ size_t pad(int i, int j, int k) const {
        return size_t(i) + size_t(n + 2) * (size_t(j) + size_t(m + 2) * size_t(k));
    }
    __host__ __device__ size_t npad() const { return size_t(n + 2) * (m + 2) * (l + 2); }
};

struct Params {
    double par[NPAR + 1];
    int TRES, SRES;
};

// Vertical mixing and convective adjustment (src/ocean/mix_imp.f vmix_fun,
// Mixing >= 1): scalars of one call, and the device-resident state of the
// adaptive partition, flags[5] = {vmix_temp, vmix_salt, partition rows/columns
// T, partition rows/columns S, partition built (vmix_dim > 0)}.
struct MixParams {
    int on;                     // Mixing >= 1
    int rhomix;                 // Rho Mixing and a linear equation of state
    double lambda, xes, kvc, eps, fac;   // LAMB, NLES, P_VC, (1-ALPC) ENER PE_V, alphaT SPL1
    const int* flags;
};

// Scalars of the forcing routine (src/ocean/forcing.F90:4-218) for the
// uncoupled restoring path, computed on the host from par().
struct ForcingScalars {
    double sigma;   // COMB*WIND*AL_T
    double etabi;   // COMB*TEMP*(1-TRES+TRES*BIOT)
    double gamma;   // COMB*SALT*(1-SRES+SRES*BIOT)
    double hmtp, sper_fac;  // par(HMTP), par(SPER)*(1-SRES+SRES*BIOT)
    double temcor, salcor, adapted_salcor, spertcor;
};

// Stencil slot tables for the maximal graph: for each boundary class and
// canonical entry, the offset inside the row (or -1 when the neighbour falls
// outside the domain).
struct Pattern {
    const int* row_ptr;     // ndim+1
    const int* col_idx;     // nnz
    const int8_t* slot;     // [NCLASS][104]
};

// launchers (thcm_assembly.cu)
void launch_lin(const Geo& g, const Params& p, double* al_tab, cudaStream_t s);
void launch_usol(const Geo& g, const double* x, double* pads, cudaStream_t s);
void launch_dfdsurf_t(const Geo& g, const ForcingScalars& fs, const double* lambda, double* grad, cudaStream_t s);
void launch_pattern(const Geo& g, const Pattern& pat, int* col_idx, cudaStream_t s);
void launch_jacobian(const Geo& g, const Params& p, const MixParams& mp, const Pattern& pat, const double* al_tab,
                     const double* pads, double* val, float* val32, cudaStream_t s);
void launch_rhs(const Geo& g, const Params& p, const MixParams& mp, const ForcingScalars& fs, const double* al_tab,
                const double* pads, const double* x, const double* surf, double* F, cudaStream_t s);
// vmix_control (src/ocean/mix_imp.f:131-166) on the device: ||T||_2, ||S||_2
// of the state (part: 2 * 152 doubles of scratch) and the flag update.
void launch_mix_control(const Geo& g, const double* x, double* part, int* flags, int any_ocean, cudaStream_t s);
void launch_mass(const Geo& g, const Params& p, double* diagB, cudaStream_t s);
// the integral-condition row (SRES = 0) and the fixed pressure points
void launch_special_rhs(int nc, const double* coef, const double* x, double* F, int row, int sign, int pfix1, int pfix2,
                        cudaStream_t s);
void launch_special_jac(int nc, const int* rp, const int* ci, const double* coef, double* val, float* val32, int row,
                        int sign, int pfix1, int pfix2, cudaStream_t s);
void launch_dense_row_cols(int nc, int* cols, cudaStream_t s);

}  // namespace iemic
