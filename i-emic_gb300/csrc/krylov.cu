// Krylov solvers of the Newton step: SpMV, right-preconditioned restarted
// GMRES and FP64 iterative refinement around an FP32 GMRES.
//
// The reference solves J x = b with Belos block GMRES (block size 1,
// "Flexible Gmres", DGKS orthogonalisation, restart = "FGMRES iterations";
// src/ocean/Ocean.C:971-1030). Here the preconditioner is fixed during a
// solve, so right-preconditioned GMRES with x = x0 + M^{-1} V y gives the
// same iterates as the flexible variant without storing the M^{-1} V basis.
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2, the
// DGKS-style reorthogonalisation). Each pass fuses the (j+1) dot products
// into one sweep over the basis and the update into a second sweep. The
// Hessenberg least-squares problem (Givens rotations) is solved in FP64.
//
// Mixed precision (IEMIC_PREC_MIXED): the factorisation is computed and
// stored in FP32 (half the bytes, FP32 GEMM rate); its triangular solves
// accumulate in FP64 and GMRES, J and the convergence test are FP64. This is
// GMRES-based iterative refinement with a low-precision factorisation
// (Carson & Higham, SIAM J. Sci. Comput. 40 (2018) A817). An all-FP32 inner
// Krylov solve (J, basis and inner products in FP32 inside FP64 residual
// refinement) stalled on the 96x38x12 ocean, whose Jacobian has a condition
// number near 1e8, and is not offered.
//
// SpMV: rows hold 7..24 entries, so four lanes share a row and reduce with
// warp shuffles; a warp covers eight consecutive rows (contiguous loads of
// col_idx/values). The state vectors stay resident in the 126 MB L2.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "engine.cuh"
#include "ndlu.cuh"

namespace iemic {
namespace {

template <class T>
__global__ void __launch_bounds__(256) spmv_csr4(int nrows, const int* __restrict__ rp, const int* __restrict__ ci,
                                                 const T* __restrict__ v, const T* __restrict__ x, T* __restrict__ y,
                                                 int skip) {
    const int lane = threadIdx.x & 3;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; row < nrows; row += (gridDim.x * blockDim.x) >> 2) {
        if (row == skip) continue;   // the dense row: k_long_row
        const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
        T s = T(0);
        for (int q = b + lane; q < e; q += 4) s += __ldg(v + q) * __ldg(x + __ldg(ci + q));
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (lane == 0) y[row] = s;
    }
}

// y = b - J x in FP64
__global__ void __launch_bounds__(256) residual_csr4(int nrows, const int* __restrict__ rp, const int* __restrict__ ci,
                                                     const double* __restrict__ v, const double* __restrict__ x,
                                                     const double* __restrict__ b, double* __restrict__ y, int skip) {
    const int lane = threadIdx.x & 3;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; row < nrows; row += (gridDim.x * blockDim.x) >> 2) {
        if (row == skip) continue;
        const int s0 = __ldg(rp + row), e = __ldg(rp + row + 1);
        double s = 0.0;
        for (int q = s0 + lane; q < e; q += 4) s += __ldg(v + q) * __ldg(x + __ldg(ci + q));
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (lane == 0) y[row] = b[row] - s;
    }
}

// One long CSR row (the dense integral-condition row) as a block-wide
// reduction: y[row] = (b[row] if b) - sum_q v[q] x[ci[q]]... or + the sum.
template <class T>
__global__ void __launch_bounds__(1024) k_long_row(const int* __restrict__ rp, const int* __restrict__ ci,
                                                   const T* __restrict__ v, const T* __restrict__ x,
                                                   const double* __restrict__ b, T* __restrict__ y, int row) {
    __shared__ double red[1024];
    double sum = 0.0;
    for (int q = rp[row] + threadIdx.x; q < rp[row + 1]; q += blockDim.x) sum += double(v[q]) * double(x[ci[q]]);
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) y[row] = b ? T(b[row] - red[0]) : T(red[0]);
}
// Sherman-Morrison scalars of the dense row d (row `row` of J):
//   mode 0: out = (d.z - z_row) / sm[0]          (the forward correction)
//   mode 1: out = 1 + d.z - z_row                (alpha, from z = M0^{-1} e_row)
//   mode 2: out = z_row / sm[2]                  (the transposed correction)
//   mode 3: out = 1 + z_row                      (transposed alpha, z = M0^{-T}(d - e_row))
__global__ void __launch_bounds__(1024) k_sm_scalar(const int* __restrict__ rp, const int* __restrict__ ci,
                                                    const double* __restrict__ v, const double* __restrict__ z, int row,
                                                    const double* __restrict__ sm, double* __restrict__ out, int mode) {
    __shared__ double red[1024];
    double sum = 0.0;
    if (mode <= 1)
        for (int q = rp[row] + threadIdx.x; q < rp[row + 1]; q += blockDim.x) sum += v[q] * z[ci[q]];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double zr = z[row];
        if (mode == 0) out[0] = (red[0] - zr) / sm[0];
        else if (mode == 1) out[0] = 1.0 + red[0] - zr;
        else if (mode == 2) out[0] = zr / sm[2];
        else out[0] = 1.0 + zr;
    }
}
// z -= scal[0] * w
__global__ void k_axpy_scal(int n, const double* __restrict__ scal, const double* __restrict__ w, double* __restrict__ z) {
    const double a = scal[0];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) z[r] -= a * w[r];
}
// out = d - e_row as a vector (d: the entries of CSR row `row`)
__global__ void k_row_vector(const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v, int row,
                             double* __restrict__ out) {
    for (int q = rp[row] + blockIdx.x * blockDim.x + threadIdx.x; q < rp[row + 1]; q += gridDim.x * blockDim.x)
        out[ci[q]] = v[q] - (ci[q] == row ? 1.0 : 0.0);
}
__global__ void k_set_unit(double* __restrict__ v, int row) { v[row] = 1.0; }

// partial sums of dots[i] = <V_i, w>, i < nv, per block (double partials)
template <class T>
__global__ void __launch_bounds__(256) multidot(int n, int nv, const T* __restrict__ V, const T* __restrict__ w,
                                                double* __restrict__ part) {
    constexpr int MAXV = 8;   // basis vectors per sweep chunk
    __shared__ double red[MAXV][256 / 32];
    for (int i0 = 0; i0 < nv; i0 += MAXV) {
        const int cnt = min(MAXV, nv - i0);
        T acc[MAXV];
#pragma unroll
        for (int q = 0; q < MAXV; ++q) acc[q] = T(0);
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
            const T wr = w[r];
#pragma unroll
            for (int q = 0; q < MAXV; ++q)
                if (q < cnt) acc[q] += V[size_t(i0 + q) * n + r] * wr;
        }
#pragma unroll
        for (int q = 0; q < MAXV; ++q) {
            double a = double(acc[q]);
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = a;
        }
        __syncthreads();
        if (threadIdx.x < cnt) {
            double s = 0.0;
            for (int q = 0; q < 256 / 32; ++q) s += red[threadIdx.x][q];
            part[size_t(blockIdx.x) * nv + i0 + threadIdx.x] = s;
        }
        __syncthreads();
    }
}
// The sum of the nblocks partials of dot product i (part[b * ldp + i]) by one
// block of RT threads: strided per-thread sums, then a fixed-order tree in
// shared memory, so the result is deterministic. Every thread returns it.
constexpr int RT = 256;
__device__ __forceinline__ double sum_parts(int nblocks, int ldp, int i, const double* __restrict__ part) {
    __shared__ double red[RT];
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += RT) s += part[size_t(b) * ldp + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = RT / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    return red[0];
}
// dots[i] = sum over blocks of the partials, one CTA per dot product (grid nv,
// RT threads); also accumulates into h if given
__global__ void __launch_bounds__(RT) reduce_parts(int nblocks, int nv, const double* __restrict__ part,
                                                   double* __restrict__ dots, double* __restrict__ hacc, int first) {
    const int i = blockIdx.x;
    const double s = sum_parts(nblocks, nv, i, part);
    if (threadIdx.x == 0) {
        dots[i] = s;
        if (hacc) hacc[i] = first ? s : hacc[i] + s;
    }
}
// w -= sum_i h[i] V_i
template <class T>
__global__ void __launch_bounds__(256) basis_update(int n, int nv, const T* __restrict__ V, const double* __restrict__ h,
                                                    T* __restrict__ w) {
    __shared__ T hs[1024];
    for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = T(h[i]);
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        T s = w[r];
        for (int i = 0; i < nv; ++i) s -= hs[i] * V[size_t(i) * n + r];
        w[r] = s;
    }
}
// y = sum_i c[i] V_i
template <class T>
__global__ void combine(int n, int nv, const T* __restrict__ V, const double* __restrict__ c, T* __restrict__ y) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < nv; ++i) s += c[i] * double(V[size_t(i) * n + r]);
        y[r] = T(s);
    }
}
template <class A, class B>
__global__ void convert(int n, const A* __restrict__ x, B* __restrict__ y, double scale) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) y[r] = B(double(x[r]) * scale);
}
// x += alpha * d
template <class T>
__global__ void axpy_into(int n, double alpha, const T* __restrict__ d, double* __restrict__ x) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) x[r] += alpha * double(d[r]);
}

template <class T>
__global__ void sub_from(int n, const T* __restrict__ b, const T* __restrict__ a, T* __restrict__ out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) out[r] = b[r] - a[r];
}
template <class T>
__global__ void scale_by(int n, const T* __restrict__ x, double a, T* __restrict__ y) {
    const T aa = T(a);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) y[r] = x[r] * aa;
}
template <class T>
__global__ void add_to(int n, const T* __restrict__ d, T* __restrict__ x) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) x[r] += d[r];
}

// ---- device-driven Arnoldi cycle ------------------------------------------
// Control block: j = Hessenberg columns done in this cycle, it = inner
// iterations of the solve, stop = 0 running, 1 converged, 2 lucky breakdown
// (the new basis vector vanished), 3 cycle full or iteration cap, 4 a
// non-finite value.
}  // namespace
struct KryCtl {
    int j, it, maxit, m, stop, pad;
    double beta0, tol, relres, hn2, inv_hn;
};
namespace {
__global__ void k_cycle_init(KryCtl* __restrict__ ctl, double* __restrict__ g, int m, double beta, double beta0,
                             double tol, int it, int maxit) {
    for (int i = threadIdx.x; i <= m; i += blockDim.x) g[i] = i == 0 ? beta : 0.0;
    if (threadIdx.x == 0) {
        ctl->j = 0; ctl->it = it; ctl->maxit = maxit; ctl->m = m; ctl->stop = 0;
        ctl->beta0 = beta0; ctl->tol = tol; ctl->relres = beta / beta0; ctl->hn2 = 0.0; ctl->inv_hn = 0.0;
    }
}
// per-block partial sums of <V_i, w>, i <= ctl->j, into part[block * ldp + i]
__global__ void __launch_bounds__(256) multidot_ctl(int n, const KryCtl* __restrict__ ctl, int ldp,
                                                    const double* __restrict__ V, const double* __restrict__ w,
                                                    double* __restrict__ part) {
    constexpr int MAXV = 8;
    __shared__ double red[MAXV][256 / 32];
    const int nv = ctl->j + 1;
    for (int i0 = 0; i0 < nv; i0 += MAXV) {
        const int cnt = min(MAXV, nv - i0);
        double acc[MAXV];
#pragma unroll
        for (int q = 0; q < MAXV; ++q) acc[q] = 0.0;
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
            const double wr = w[r];
#pragma unroll
            for (int q = 0; q < MAXV; ++q)
                if (q < cnt) acc[q] += V[size_t(i0 + q) * n + r] * wr;
        }
#pragma unroll
        for (int q = 0; q < MAXV; ++q) {
            double a = acc[q];
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = a;
        }
        __syncthreads();
        if (threadIdx.x < cnt) {
            double sum = 0.0;
            for (int q = 0; q < 256 / 32; ++q) sum += red[threadIdx.x][q];
            part[size_t(blockIdx.x) * ldp + i0 + threadIdx.x] = sum;
        }
        __syncthreads();
    }
}
// dots = sum of the partials; column j of H gets them (first pass) or adds
// them. One CTA per possible dot product (grid m + 1, RT threads); CTAs past
// ctl->j return at once.
__global__ void __launch_bounds__(RT) reduce_parts_ctl(int nblocks, int ldp, const KryCtl* __restrict__ ctl,
                                                       const double* __restrict__ part, double* __restrict__ dots,
                                                       double* __restrict__ H, int first) {
    const int i = blockIdx.x;
    if (i > ctl->j) return;   // the same for every thread of the CTA
    const double sum = sum_parts(nblocks, ldp, i, part);
    if (threadIdx.x == 0) {
        double* col = H + size_t(ctl->m + 1) * ctl->j;
        dots[i] = sum;
        col[i] = first ? sum : col[i] + sum;
    }
}
// w -= sum_{i <= j} dots[i] V_i
__global__ void __launch_bounds__(256) basis_update_ctl(int n, const KryCtl* __restrict__ ctl, const double* __restrict__ V,
                                                        const double* __restrict__ h, double* __restrict__ w) {
    __shared__ double hs[1024];
    const int nv = ctl->j + 1;
    for (int i = threadIdx.x; i < nv; i += blockDim.x) hs[i] = h[i];
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double sum = w[r];
        for (int i = 0; i < nv; ++i) sum -= hs[i] * V[size_t(i) * n + r];
        w[r] = sum;
    }
}
// Givens rotations of column j (FP64), the residual estimate and the loop
// condition of the cycle's while-node
__global__ void k_givens(KryCtl* __restrict__ ctl, double* __restrict__ H, double* __restrict__ cs,
                         double* __restrict__ sn, double* __restrict__ g, cudaGraphConditionalHandle cond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int j = ctl->j, m = ctl->m;
    double* col = H + size_t(m + 1) * j;
    const double hn = sqrt(ctl->hn2);
    col[j + 1] = hn;
    for (int i = 0; i < j; ++i) {
        const double a = col[i], c = col[i + 1];
        col[i] = cs[i] * a + sn[i] * c;
        col[i + 1] = -sn[i] * a + cs[i] * c;
    }
    const double a = col[j], c = col[j + 1];
    const double d = hypot(a, c);
    cs[j] = d > 0 ? a / d : 1.0;
    sn[j] = d > 0 ? c / d : 0.0;
    col[j] = d;
    col[j + 1] = 0.0;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    const int jn = j + 1, it = ctl->it + 1;
    const double relres = fabs(g[jn]) / ctl->beta0;
    int stop = 0;
    if (!isfinite(hn) || !isfinite(relres)) stop = 4;
    else if (relres <= ctl->tol) stop = 1;
    else if (hn == 0.0) stop = 2;
    else if (jn >= m || it >= ctl->maxit) stop = 3;
    ctl->j = jn;
    ctl->it = it;
    ctl->relres = relres;
    ctl->stop = stop;
    ctl->inv_hn = (stop != 4 && hn > 0.0) ? 1.0 / hn : 0.0;
    cudaGraphSetConditional(cond, stop ? 0u : 1u);
}
// v_{j+1} = w / h(j+1, j) into the basis and into the preconditioner's input
__global__ void k_scale_next(int n, const KryCtl* __restrict__ ctl, const double* __restrict__ w, double* __restrict__ V,
                             double* __restrict__ vcur) {
    const double a = ctl->inv_hn;
    if (a == 0.0) return;
    double* vn = V + size_t(ctl->j) * n;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double v = w[r] * a;
        vn[r] = v;
        vcur[r] = v;
    }
}
// y = R^{-1} g for the j x j triangle R of the rotated Hessenberg (one warp).
// A zero diagonal (an exactly singular least-squares column) contributes a
// zero coefficient instead of a division by zero.
__global__ void k_backsolve(const KryCtl* __restrict__ ctl, const double* __restrict__ H, const double* __restrict__ g,
                            double* __restrict__ y) {
    const int j = ctl->j, ld = ctl->m + 1, lane = threadIdx.x;
    for (int i = j - 1; i >= 0; --i) {
        double part = 0.0;
        for (int q = i + 1 + lane; q < j; q += 32) part += H[i + size_t(ld) * q] * y[q];
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) {
            const double dgn = H[i + size_t(ld) * i];
            y[i] = dgn != 0.0 ? (g[i] - part) / dgn : 0.0;
        }
        __syncwarp();
    }
}

int vgrid(int n) {
    long b = (long(n) + 255) / 256;
    return int(b < 152 * 4 ? b : 152 * 4);
}
int spmv_grid(int nrows) {
    long blocks = (long(nrows) * 4 + 255) / 256;
    return int(blocks < 152 * 8 ? blocks : 152 * 8);
}

}  // namespace

// y = A x with A in CSR; row `skip` (a dense row, or -1) by a block-wide reduction
template <class T>
static void spmv_launch(int nrows, const int* rp, const int* ci, const T* v, const T* x, T* y, int skip, cudaStream_t s) {
    spmv_csr4<T><<<spmv_grid(nrows), 256, 0, s>>>(nrows, rp, ci, v, x, y, skip); IEMIC_COUNT_LAUNCH();
    if (skip >= 0) {
        k_long_row<T><<<1, 1024, 0, s>>>(rp, ci, v, x, nullptr, y, skip); IEMIC_COUNT_LAUNCH();
    }
}
// y = b - A x
static void residual_launch(int nrows, const int* rp, const int* ci, const double* v, const double* x, const double* b,
                            double* y, int skip, cudaStream_t s) {
    residual_csr4<<<spmv_grid(nrows), 256, 0, s>>>(nrows, rp, ci, v, x, b, y, skip); IEMIC_COUNT_LAUNCH();
    if (skip >= 0) {
        k_long_row<double><<<1, 1024, 0, s>>>(rp, ci, v, x, b, y, skip); IEMIC_COUNT_LAUNCH();
    }
}
void launch_spmv64(int nrows, const int* rp, const int* ci, const double* v, const double* x, double* y, int skip,
                   cudaStream_t s) {
    spmv_launch<double>(nrows, rp, ci, v, x, y, skip, s);
}

// Krylov workspace (both precisions share the layout)
struct Krylov {
    int n = 0, m = 0, nblk = 0;
    void* V = nullptr;       // (m+1) x n in the Krylov precision
    void* w = nullptr;       // n
    void* z = nullptr;       // n
    double* part = nullptr;  // nblk x (m+1)
    double* dots = nullptr;  // m+1
    double* h = nullptr;     // m+1 (current Hessenberg column)
    double* y = nullptr;     // m
    double* r64 = nullptr;   // n
    double* x64 = nullptr;   // n
    double* hpin = nullptr;  // pinned host copy of h
    void* rhsT = nullptr;    // n, Krylov precision: normalised rhs of an inner solve
    void* xT = nullptr;      // n, Krylov precision: inner solution
    int prec = -1;
    // device-driven Arnoldi cycle (FP64 Krylov): Hessenberg, rotations and
    // control block on the device, the cycle as one CUDA graph whose
    // conditional while-node runs the Arnoldi steps until the control kernel
    // stops it
    double *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *vcur = nullptr;
    KryCtl* ctl = nullptr;   // device
    KryCtl* ctl_pin = nullptr;
    cudaGraph_t cyc_graph = nullptr;
    cudaGraphExec_t cyc_exec = nullptr;
    const void* cyc_key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int cyc_full = -1;
    long long cyc_body_launches = 0;
    bool cyc_failed = false;   // the runtime refused the conditional graph: host-driven cycles
};

static void free_krylov(Krylov* k) {
    if (!k) return;
    if (k->cyc_exec) cudaGraphExecDestroy(k->cyc_exec);
    if (k->cyc_graph) cudaGraphDestroy(k->cyc_graph);
    cudaFree(k->V); cudaFree(k->w); cudaFree(k->z); cudaFree(k->part); cudaFree(k->dots);
    cudaFree(k->h); cudaFree(k->y); cudaFree(k->r64); cudaFree(k->x64);
    cudaFree(k->rhsT); cudaFree(k->xT);
    cudaFree(k->H); cudaFree(k->cs); cudaFree(k->sn); cudaFree(k->g); cudaFree(k->vcur); cudaFree(k->ctl);
    cudaFreeHost(k->hpin);
    cudaFreeHost(k->ctl_pin);
    delete k;
}

void Engine::spmv64(const double* x, double* y) {
    launch_spmv64(ndim, d_rowptr, d_col, d_val, x, y, rowintcon, stream);
    ck(cudaGetLastError());
}

void Engine::drop_factors() {
    // the Krylov workspace goes too: its captured Arnoldi cycle holds the
    // factorisation's buffers, and a new factorisation may reuse the address
    delete lu64;
    delete lu32;
    lu64 = lu32 = nullptr;
    free_krylov(kry);
    kry = nullptr;
    fact64_stale = fact32_stale = true;
}

void Engine::free_solver() {
    drop_factors();
    delete ndplan;
    ndplan = nullptr;
}

void Engine::ensure_solver() {
    if (!ndplan) {
        ndplan = new NdPlan();
        build_nd_plan(*ndplan, cfg.n, cfg.m, cfg.l, cfg.periodic ? 1 : 0, landm, row_ptr, host_col_idx(), 32,
                      {rowintcon, rowPfix1, rowPfix2}, {rowPfix1, rowPfix2});
    }
}

const std::vector<int>& Engine::host_col_idx() {
    if (h_col.empty()) {
        h_col.resize(size_t(nnz));
        ck(cudaMemcpyAsync(h_col.data(), d_col, sizeof(int) * size_t(nnz), cudaMemcpyDeviceToHost, stream));
        ck(cudaStreamSynchronize(stream));
    }
    return h_col;
}

static void ensure_krylov(Engine& e, int m, int prec) {
    Krylov*& k = e.kry;
    const size_t ts = prec ? sizeof(float) : sizeof(double);
    if (k && k->m >= m && k->prec == prec) return;
    free_krylov(k);
    k = nullptr;
    k = new Krylov();
    k->n = e.ndim;
    k->m = m;
    k->prec = prec;
    k->nblk = vgrid(e.ndim);
    auto A = [&](size_t bytes) {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) throw EngineError(IEMIC_ERR_NOMEM);
        return p;
    };
    k->V = A(ts * size_t(m + 1) * e.ndim);
    k->w = A(ts * e.ndim);
    k->z = A(ts * e.ndim);
    k->part = static_cast<double*>(A(sizeof(double) * size_t(k->nblk) * (m + 1)));
    k->dots = static_cast<double*>(A(sizeof(double) * (m + 2)));
    k->h = static_cast<double*>(A(sizeof(double) * (m + 2)));
    k->y = static_cast<double*>(A(sizeof(double) * (m + 2)));
    k->r64 = static_cast<double*>(A(sizeof(double) * e.ndim));
    k->x64 = static_cast<double*>(A(sizeof(double) * e.ndim));
    k->rhsT = A(ts * e.ndim);
    k->xT = A(ts * e.ndim);
    k->H = static_cast<double*>(A(sizeof(double) * size_t(m + 1) * m));
    k->cs = static_cast<double*>(A(sizeof(double) * (m + 1)));
    k->sn = static_cast<double*>(A(sizeof(double) * (m + 1)));
    k->g = static_cast<double*>(A(sizeof(double) * (m + 2)));
    k->vcur = static_cast<double*>(A(sizeof(double) * e.ndim));
    k->ctl = static_cast<KryCtl*>(A(sizeof(KryCtl)));
    ck(cudaMallocHost(&k->hpin, sizeof(double) * (m + 2)));
    ck(cudaMallocHost(&k->ctl_pin, sizeof(KryCtl)));
}

NdLu*& Engine::lu_for(int precision) { return precision == IEMIC_PREC_MIXED ? lu32 : lu64; }

void Engine::build_preconditioner(int precision) {
    if (!jac_valid) throw EngineError(IEMIC_ERR_STATE);
    ensure_solver();
    NdLu*& lu = lu_for(precision);
    if (!lu) {
        lu = new NdLu();
        ndlu_setup(*lu, *ndplan, precision == IEMIC_PREC_MIXED ? 1 : 0, subst_min_nf);
        lu->timer = &timer;
    }
    ndlu_factor(*lu, d_rowptr, d_col, d_val, stream);
    ck(cudaStreamSynchronize(stream));
    timer.drain();
    if (precision == IEMIC_PREC_MIXED) fact32_stale = false; else fact64_stale = false;
    sm_setup(precision == IEMIC_PREC_MIXED ? 1 : 0);
}

// Dense integral-condition row r (SRES = 0): the factorisation treats row r
// as the identity row e_r (J0 = J + e_r (e_r - d)^T, d = row r of J), which
// keeps its elimination tree local, and the preconditioner restores d by
// Sherman-Morrison:
//   J^{-1} v  = y - zr (d.y - y_r) / alpha,   y = M0^{-1} v, zr = M0^{-1} e_r,
//               alpha = 1 + d.zr - zr_r
//   J^{-T} v  = y - wt y_r / (1 + wt_r),       y = M0^{-T} v, wt = M0^{-T} (d - e_r)
// zr and alpha are refreshed after every factorisation, wt on the first
// transposed solve of a factorisation.
void Engine::sm_setup(int pi) {
    ++fact_gen[pi];
    if (rowintcon < 0) return;
    NdLu* lu = pi ? lu32 : lu64;
    if (!d_zr[pi]) {
        d_zr[pi] = static_cast<double*>(dalloc(sizeof(double) * ndim));
        d_sm[pi] = static_cast<double*>(dalloc(sizeof(double) * 4));
    }
    if (!d_smtmp) d_smtmp = static_cast<double*>(dalloc(sizeof(double) * ndim));
    ck(cudaMemsetAsync(d_smtmp, 0, sizeof(double) * ndim, stream));
    k_set_unit<<<1, 1, 0, stream>>>(d_smtmp, rowintcon); IEMIC_COUNT_LAUNCH();
    ndlu_apply(*lu, d_rowptr, d_col, d_val, d_smtmp, d_zr[pi], 0, stream);
    k_sm_scalar<<<1, 1024, 0, stream>>>(d_rowptr, d_col, d_val, d_zr[pi], rowintcon, d_sm[pi], d_sm[pi], 1); IEMIC_COUNT_LAUNCH();
    ck(cudaGetLastError());
}

void Engine::precond_apply(NdLu& lu, int pi, const double* v, double* z, bool transpose) {
    cudaStream_t s = stream;
    if (!transpose) {
        ndlu_apply(lu, d_rowptr, d_col, d_val, v, z, 0, s);
        if (rowintcon < 0) return;
        k_sm_scalar<<<1, 1024, 0, s>>>(d_rowptr, d_col, d_val, z, rowintcon, d_sm[pi], d_sm[pi] + 1, 0); IEMIC_COUNT_LAUNCH();
        k_axpy_scal<<<vgrid(ndim), 256, 0, s>>>(ndim, d_sm[pi] + 1, d_zr[pi], z); IEMIC_COUNT_LAUNCH();
        return;
    }
    if (rowintcon >= 0 && wt_gen[pi] != fact_gen[pi]) {
        if (!d_wt[pi]) d_wt[pi] = static_cast<double*>(dalloc(sizeof(double) * ndim));
        if (!d_smtmp) d_smtmp = static_cast<double*>(dalloc(sizeof(double) * ndim));
        ck(cudaMemsetAsync(d_smtmp, 0, sizeof(double) * ndim, s));
        k_row_vector<<<vgrid(ndim), 256, 0, s>>>(d_rowptr, d_col, d_val, rowintcon, d_smtmp); IEMIC_COUNT_LAUNCH();
        ndlu_apply_transpose(lu, d_smtmp, d_wt[pi], s);
        k_sm_scalar<<<1, 1024, 0, s>>>(d_rowptr, d_col, d_val, d_wt[pi], rowintcon, d_sm[pi], d_sm[pi] + 2, 3); IEMIC_COUNT_LAUNCH();
        wt_gen[pi] = fact_gen[pi];
    }
    ndlu_apply_transpose(lu, v, z, s);
    if (rowintcon < 0) return;
    k_sm_scalar<<<1, 1024, 0, s>>>(d_rowptr, d_col, d_val, z, rowintcon, d_sm[pi], d_sm[pi] + 3, 2); IEMIC_COUNT_LAUNCH();
    k_axpy_scal<<<vgrid(ndim), 256, 0, s>>>(ndim, d_sm[pi] + 3, d_wt[pi], z); IEMIC_COUNT_LAUNCH();
}

void Engine::apply_precon(int precision, const double* v, double* out) {
    NdLu* lu = lu_for(precision);
    if (!lu || !lu->factored) throw EngineError(IEMIC_ERR_STATE);
    // FP64 vectors in and out for both factor precisions (the mixed solve
    // applies its FP32 factors to FP64 Krylov vectors the same way)
    precond_apply(*lu, precision == IEMIC_PREC_MIXED ? 1 : 0, v, out, false);
    ck(cudaGetLastError());
}

// M^{-1} v (or M^{-T} v for the adjoint) in the Krylov precision T
template <class T>
static void precond(NdLu& lu, Engine& e, const T* v, T* z, bool transpose, cudaStream_t s) {
    if constexpr (sizeof(T) == 8) {
        e.precond_apply(lu, &lu == e.lu32 ? 1 : 0, v, z, transpose);
        return;
    }
    ndlu_apply(lu, e.d_rowptr, e.d_col, e.d_val, v, z, sizeof(T) == 4, s);
}

// One restarted-GMRES solve of J x = b in precision T, x0 = 0, right
// preconditioned by the factorisation `lu`. `b` must not alias the Krylov
// workspace. Returns the inner iterations used.
template <class T>
static int gmres(Engine& e, NdLu& lu, const int* rp, const int* ci, const T* vals, const T* b, T* x, int m, int maxit,
                 double tol, double* relres_out, bool transpose = false, int skip = -1) {
    Krylov& K = *e.kry;
    const int n = e.ndim;
    cudaStream_t s = e.stream;
    T* V = static_cast<T*>(K.V);
    T* w = static_cast<T*>(K.w);
    T* z = static_cast<T*>(K.z);
    const int G = vgrid(n);
    auto dot = [&](const T* a, const T* c) {
        multidot<T><<<G, 256, 0, s>>>(n, 1, a == c ? a : a, c, K.part); IEMIC_COUNT_LAUNCH();
        reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
        ck(cudaMemcpyAsync(K.hpin, K.dots, sizeof(double), cudaMemcpyDeviceToHost, s));
        ck(cudaStreamSynchronize(s));
        return K.hpin[0];
    };
    std::vector<double> H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    // CSR values + column indices + row pointers, x gathered once, y written
    const double spmv_bytes = double(e.nnz) * (sizeof(T) + 4) + 4.0 * (n + 1) + 2.0 * sizeof(T) * n;
    ck(cudaMemsetAsync(x, 0, sizeof(T) * n, s));
    const double beta0 = std::sqrt(dot(b, b));
    if (!(beta0 > 0.0)) {
        *relres_out = 0.0;
        return 0;
    }
    if (!std::isfinite(beta0)) throw EngineError(IEMIC_ERR_NAN);
    int it = 0;
    double relres = 1.0;
    bool first = true;
    while (true) {
        // r = b - J x  (x = 0 on the first cycle)
        if (first) {
            ck(cudaMemcpyAsync(w, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
        } else {
            spmv_launch<T>(n, rp, ci, vals, x, z, skip, s);
            sub_from<T><<<G, 256, 0, s>>>(n, b, z, w); IEMIC_COUNT_LAUNCH();
        }
        first = false;
        const double beta = std::sqrt(dot(w, w));
        if (!std::isfinite(beta)) throw EngineError(IEMIC_ERR_NAN);
        relres = beta / beta0;
        if (relres <= tol || it >= maxit) break;
        scale_by<T><<<G, 256, 0, s>>>(n, w, 1.0 / beta, V); IEMIC_COUNT_LAUNCH();
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        for (; j < m && it < maxit;) {
            precond(lu, e, V + size_t(j) * n, z, transpose, s);
            cudaEvent_t ev = e.timer.start(s);
            spmv_launch<T>(n, rp, ci, vals, z, w, skip, s);
            e.timer.stop(ev, s, IEMIC_KC_SPMV, spmv_bytes, 2.0 * double(e.nnz));
            for (int pass = 0; pass < 2; ++pass) {   // CGS2
                multidot<T><<<G, 256, 0, s>>>(n, j + 1, V, w, K.part); IEMIC_COUNT_LAUNCH();
                reduce_parts<<<j + 1, RT, 0, s>>>(G, j + 1, K.part, K.dots, K.h, pass == 0); IEMIC_COUNT_LAUNCH();
                basis_update<T><<<G, 256, 0, s>>>(n, j + 1, V, K.dots, w); IEMIC_COUNT_LAUNCH();
            }
            multidot<T><<<G, 256, 0, s>>>(n, 1, w, w, K.part); IEMIC_COUNT_LAUNCH();
            reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.h + j + 1, nullptr, 0); IEMIC_COUNT_LAUNCH();
            ck(cudaMemcpyAsync(K.hpin, K.h, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, s));
            ck(cudaStreamSynchronize(s));
            e.timer.drain();   // before the next replay re-records the graph's timing events
            const double hn = std::sqrt(K.hpin[j + 1]);
            if (!std::isfinite(hn)) throw EngineError(IEMIC_ERR_NAN);
            if (hn > 0.0) {
                scale_by<T><<<G, 256, 0, s>>>(n, w, 1.0 / hn, V + size_t(j + 1) * n); IEMIC_COUNT_LAUNCH();
            }
            for (int i = 0; i <= j; ++i) H[size_t(i) * m + j] = K.hpin[i];
            H[size_t(j + 1) * m + j] = hn;
            for (int i = 0; i < j; ++i) {   // apply the previous Givens rotations
                double a = H[size_t(i) * m + j], c = H[size_t(i + 1) * m + j];
                H[size_t(i) * m + j] = cs[i] * a + sn[i] * c;
                H[size_t(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
            }
            double a = H[size_t(j) * m + j], c = H[size_t(j + 1) * m + j];
            double d = std::hypot(a, c);
            cs[j] = d > 0 ? a / d : 1.0;
            sn[j] = d > 0 ? c / d : 0.0;
            H[size_t(j) * m + j] = d;
            H[size_t(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++j;
            ++it;
            relres = std::fabs(g[j]) / beta0;
            if (relres <= tol || hn == 0.0) break;
        }
        // y = H^{-1} g (FP64 back substitution), x += M^{-1} (V y)
        for (int i = j - 1; i >= 0; --i) {   // a zero diagonal contributes a zero coefficient
            double sum = g[i];
            for (int q = i + 1; q < j; ++q) sum -= H[size_t(i) * m + q] * y[q];
            const double dgn = H[size_t(i) * m + i];
            y[i] = dgn != 0.0 ? sum / dgn : 0.0;
        }
        ck(cudaMemcpyAsync(K.y, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        combine<T><<<G, 256, 0, s>>>(n, j, V, K.y, w); IEMIC_COUNT_LAUNCH();
        precond(lu, e, w, z, transpose, s);
        add_to<T><<<G, 256, 0, s>>>(n, z, x); IEMIC_COUNT_LAUNCH();
        ck(cudaStreamSynchronize(s));   // y is a host temporary
        e.timer.drain();
    }
    ck(cudaGetLastError());
    *relres_out = relres;
    return it;
}

// The device-driven cycle: one CUDA graph holding a conditional while-node
// whose body is one Arnoldi step (preconditioner sweeps, SpMV, CGS2, norm,
// Givens rotation, next basis vector). The step's control kernel updates the
// residual estimate and ends the loop, so a cycle runs with no host round
// trip between its iterations. Built once per (factorisation object, matrix,
// solve mode) and replayed for every cycle and solve.
static bool ensure_cycle_graph(Engine& e, NdLu& lu, const int* rp, const int* ci, const double* vals) {
    Krylov& K = *e.kry;
    const void* key[5] = {&lu, rp, ci, vals, lu.d_factor};
    const int full = lu.full_inverse ? 1 : 0;
    if (K.cyc_exec && std::equal(key, key + 5, K.cyc_key) && K.cyc_full == full) return true;
    if (K.cyc_exec) { cudaGraphExecDestroy(K.cyc_exec); K.cyc_exec = nullptr; }
    if (K.cyc_graph) { cudaGraphDestroy(K.cyc_graph); K.cyc_graph = nullptr; }
    cudaStream_t s = e.stream;
    const int n = e.ndim, G = vgrid(n), m = K.m;
    double* V = static_cast<double*>(K.V);
    double* w = static_cast<double*>(K.w);
    double* z = static_cast<double*>(K.z);
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
    cudaGraphConditionalHandle cond;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    cudaGraphNode_t node;
    if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
        cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return false;
    }
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess) {
        cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return false;
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    ck(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const long long n0 = launch_counter();
    bool captured = true;
    try {
        e.precond_apply(lu, &lu == e.lu32 ? 1 : 0, K.vcur, z, false);
        spmv_launch<double>(n, rp, ci, vals, z, w, e.rowintcon, s);
        for (int pass = 0; pass < 2; ++pass) {   // CGS2
            multidot_ctl<<<G, 256, 0, s>>>(n, K.ctl, m + 1, V, w, K.part); IEMIC_COUNT_LAUNCH();
            reduce_parts_ctl<<<m + 1, RT, 0, s>>>(G, m + 1, K.ctl, K.part, K.dots, K.H, pass == 0); IEMIC_COUNT_LAUNCH();
            basis_update_ctl<<<G, 256, 0, s>>>(n, K.ctl, V, K.dots, w); IEMIC_COUNT_LAUNCH();
        }
        multidot<double><<<G, 256, 0, s>>>(n, 1, w, w, K.part); IEMIC_COUNT_LAUNCH();
        reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, &K.ctl->hn2, nullptr, 0); IEMIC_COUNT_LAUNCH();
        k_givens<<<1, 32, 0, s>>>(K.ctl, K.H, K.cs, K.sn, K.g, cond); IEMIC_COUNT_LAUNCH();
        k_scale_next<<<G, 256, 0, s>>>(n, K.ctl, w, V, K.vcur); IEMIC_COUNT_LAUNCH();
    } catch (...) {
        captured = false;
    }
    cudaGraph_t out = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &out);
    K.cyc_body_launches = launch_counter() - n0;
    launch_counter() = n0;
    if (!captured || ec != cudaSuccess) {
        cudaGraphDestroy(g);
        (void)cudaGetLastError();
        if (!captured) throw EngineError(IEMIC_ERR_CUDA);
        return false;
    }
    if (cudaGraphInstantiate(&K.cyc_exec, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        K.cyc_exec = nullptr;
        (void)cudaGetLastError();
        return false;
    }
    K.cyc_graph = g;
    std::copy(key, key + 5, K.cyc_key);
    K.cyc_full = full;
    return true;
}

// Restarted GMRES (FP64 Krylov, right preconditioned, x0 = 0) with
// device-driven cycles; the same iteration as gmres<double> with the
// Hessenberg, the Givens rotations and the back substitution on the device
// (FP64). The host waits twice per cycle: for the restart residual and for
// the cycle's end. Returns false (and does nothing) when the runtime refuses
// the conditional graph.
static bool gmres_dev(Engine& e, NdLu& lu, const int* rp, const int* ci, const double* vals, const double* b,
                      double* x, int m, int maxit, double tol, double* relres_out, int* iters_out) {
    Krylov& K = *e.kry;
    if (K.cyc_failed) return false;
    // IEMIC_HOST_GMRES=1 steps the cycles from the host (the same iteration;
    // for profilers that cannot see kernels inside conditional graph nodes)
    static const bool host_only = [] {
        const char* v = std::getenv("IEMIC_HOST_GMRES");
        return v && *v && *v != '0';
    }();
    if (host_only) return false;
    if (!ensure_cycle_graph(e, lu, rp, ci, vals)) {
        K.cyc_failed = true;
        return false;
    }
    const int n = e.ndim, G = vgrid(n);
    cudaStream_t s = e.stream;
    double* V = static_cast<double*>(K.V);
    double* w = static_cast<double*>(K.w);
    double* z = static_cast<double*>(K.z);
    auto norm = [&](const double* a) {
        multidot<double><<<G, 256, 0, s>>>(n, 1, a, a, K.part); IEMIC_COUNT_LAUNCH();
        reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
        ck(cudaMemcpyAsync(K.hpin, K.dots, sizeof(double), cudaMemcpyDeviceToHost, s));
        ck(cudaStreamSynchronize(s));
        return std::sqrt(K.hpin[0]);
    };
    ck(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    const double beta0 = norm(b);
    *iters_out = 0;
    if (!(beta0 > 0.0)) {
        *relres_out = 0.0;
        return true;
    }
    if (!std::isfinite(beta0)) throw EngineError(IEMIC_ERR_NAN);
    int it = 0;
    double relres = 1.0;
    for (bool first = true;; first = false) {
        if (first) {
            ck(cudaMemcpyAsync(w, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        } else {
            spmv_launch<double>(n, rp, ci, vals, x, z, e.rowintcon, s);
            sub_from<double><<<G, 256, 0, s>>>(n, b, z, w); IEMIC_COUNT_LAUNCH();
        }
        const double beta = norm(w);
        if (!std::isfinite(beta)) throw EngineError(IEMIC_ERR_NAN);
        relres = beta / beta0;
        if (relres <= tol || it >= maxit) break;
        scale_by<double><<<G, 256, 0, s>>>(n, w, 1.0 / beta, V); IEMIC_COUNT_LAUNCH();
        ck(cudaMemcpyAsync(K.vcur, V, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        k_cycle_init<<<1, 256, 0, s>>>(K.ctl, K.g, m, beta, beta0, tol, it, maxit); IEMIC_COUNT_LAUNCH();
        ck(cudaGraphLaunch(K.cyc_exec, s));
        ck(cudaMemcpyAsync(K.ctl_pin, K.ctl, sizeof(KryCtl), cudaMemcpyDeviceToHost, s));
        ck(cudaStreamSynchronize(s));
        const KryCtl c = *K.ctl_pin;
        launch_counter() += K.cyc_body_launches * (c.it - it);
        it = c.it;
        if (c.stop == 4) throw EngineError(IEMIC_ERR_NAN);
        // y = R^{-1} g, x += M^{-1} (V y)
        k_backsolve<<<1, 32, 0, s>>>(K.ctl, K.H, K.g, K.y); IEMIC_COUNT_LAUNCH();
        combine<double><<<G, 256, 0, s>>>(n, c.j, V, K.y, w); IEMIC_COUNT_LAUNCH();
        e.precond_apply(lu, &lu == e.lu32 ? 1 : 0, w, z, false);
        add_to<double><<<G, 256, 0, s>>>(n, z, x); IEMIC_COUNT_LAUNCH();
    }
    ck(cudaGetLastError());
    *relres_out = relres;
    *iters_out = it;
    return true;
}

int Engine::solve_dev(const double* b, double* x, const iemic_solve_opts& o, iemic_solve_stats& st) {
    if (!jac_valid) return IEMIC_ERR_STATE;
    if (o.transpose) return solve_transpose_dev(b, x, o, st);
    // IEMIC_PREC_MIXED: FP32 factors under an FP64 Krylov solve
    const int prec = o.precision == IEMIC_PREC_FP64 ? IEMIC_PREC_FP64 : IEMIC_PREC_MIXED;
    auto t0 = std::chrono::steady_clock::now();
    ensure_solver();
    NdLu*& lu = lu_for(prec);
    bool stale = prec == IEMIC_PREC_MIXED ? fact32_stale : fact64_stale;
    if (!lu || !lu->factored || (stale && !o.reuse_preconditioner)) {
        build_preconditioner(prec);
        st.factorizations += 1;
    }
    st.perturbed_pivots = lu->npert;
    auto t1 = std::chrono::steady_clock::now();
    st.time_factor_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
    ensure_krylov(*this, o.restart, 0);
    Krylov& K = *kry;
    const int n = ndim;
    const int G = vgrid(n);
    cudaStream_t s = stream;
    // ||b||
    multidot<double><<<G, 256, 0, s>>>(n, 1, b, b, K.part); IEMIC_COUNT_LAUNCH();
    reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
    double bn2 = 0.0;
    ck(cudaMemcpyAsync(&bn2, K.dots, sizeof(double), cudaMemcpyDeviceToHost, s));
    ck(cudaStreamSynchronize(s));
    const double bnorm = std::sqrt(bn2);
    if (!std::isfinite(bnorm)) return IEMIC_ERR_NAN;
    ck(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    if (bnorm == 0.0) {
        st.relres = 0.0;
        return IEMIC_OK;
    }
    int rc = IEMIC_OK;
    scale_by<double><<<G, 256, 0, s>>>(n, b, 1.0 / bnorm, K.r64); IEMIC_COUNT_LAUNCH();
    double est = 1.0;
    int its = 0;
    if (!timer.on && gmres_dev(*this, *lu, d_rowptr, d_col, d_val, K.r64, K.x64, o.restart, o.max_iters, o.tol,
                               &est, &its))
        st.iters += its;
    else
        st.iters += gmres<double>(*this, *lu, d_rowptr, d_col, d_val, K.r64, K.x64, o.restart, o.max_iters, o.tol,
                                  &est, false, rowintcon);
    axpy_into<double><<<G, 256, 0, s>>>(n, bnorm, K.x64, x); IEMIC_COUNT_LAUNCH();
    residual_launch(n, d_rowptr, d_col, d_val, x, b, K.r64, rowintcon, s);
    multidot<double><<<G, 256, 0, s>>>(n, 1, K.r64, K.r64, K.part); IEMIC_COUNT_LAUNCH();
    reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
    double rn2 = 0.0;
    ck(cudaMemcpyAsync(&rn2, K.dots, sizeof(double), cudaMemcpyDeviceToHost, s));
    ck(cudaStreamSynchronize(s));
    const double relres = std::sqrt(rn2) / bnorm;
    st.relres = relres;
    timer.drain();
    auto t2 = std::chrono::steady_clock::now();
    st.time_solve_ms += std::chrono::duration<double, std::milli>(t2 - t1).count();
    if (relres > o.tol) rc = IEMIC_ERR_NOT_CONVERGED;
    return rc;
}

// J^T values in the transposed pattern (refreshed when J changed)
__global__ void k_gather_vals(int64_t nnz, const int* __restrict__ perm, const double* __restrict__ v,
                              double* __restrict__ vt) {
    for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < nnz; q += int64_t(gridDim.x) * blockDim.x)
        vt[q] = v[perm[q]];
}

void Engine::ensure_transpose() {
    if (!d_rowT) {
        const std::vector<int>& ci = host_col_idx();
        std::vector<int> rt(static_cast<size_t>(ndim) + 1, 0), ct(static_cast<size_t>(nnz)), pm(static_cast<size_t>(nnz));
        for (int64_t q = 0; q < nnz; ++q) rt[size_t(ci[q]) + 1] += 1;
        for (int r = 0; r < ndim; ++r) rt[r + 1] += rt[r];
        std::vector<int> fill(rt.begin(), rt.end() - 1);
        for (int r = 0; r < ndim; ++r)
            for (int q = row_ptr[r]; q < row_ptr[r + 1]; ++q) {
                const int d = fill[ci[q]]++;
                ct[d] = r;
                pm[d] = q;
            }
        d_rowT = static_cast<int*>(dalloc(sizeof(int) * rt.size()));
        d_colT = static_cast<int*>(dalloc(sizeof(int) * ct.size()));
        d_permT = static_cast<int*>(dalloc(sizeof(int) * pm.size()));
        d_valT = static_cast<double*>(dalloc(sizeof(double) * size_t(nnz)));
        ck(cudaMemcpyAsync(d_rowT, rt.data(), sizeof(int) * rt.size(), cudaMemcpyHostToDevice, stream));
        ck(cudaMemcpyAsync(d_colT, ct.data(), sizeof(int) * ct.size(), cudaMemcpyHostToDevice, stream));
        ck(cudaMemcpyAsync(d_permT, pm.data(), sizeof(int) * pm.size(), cudaMemcpyHostToDevice, stream));
        ck(cudaStreamSynchronize(stream));
        jacT_stale = true;
    }
    if (jacT_stale) {
        k_gather_vals<<<vgrid(int(std::min<int64_t>(nnz, 1 << 30))), 256, 0, stream>>>(nnz, d_permT, d_val, d_valT); IEMIC_COUNT_LAUNCH();
        ck(cudaGetLastError());
        jacT_stale = false;
    }
}

// Adjoint solve J^T x = b: FP64 GMRES on J^T, right preconditioned by M^{-T}
// from the same factorisation as the forward solve (FP64 or FP32 factors).
int Engine::solve_transpose_dev(const double* b, double* x, const iemic_solve_opts& o, iemic_solve_stats& st) {
    if (!jac_valid) return IEMIC_ERR_STATE;
    const int prec = o.precision == IEMIC_PREC_FP64 ? IEMIC_PREC_FP64 : IEMIC_PREC_MIXED;
    auto t0 = std::chrono::steady_clock::now();
    ensure_solver();
    NdLu*& lu = lu_for(prec);
    const bool stale = prec == IEMIC_PREC_MIXED ? fact32_stale : fact64_stale;
    if (!lu || !lu->factored || (stale && !o.reuse_preconditioner)) {
        build_preconditioner(prec);
        st.factorizations += 1;
    }
    st.perturbed_pivots = lu->npert;
    ensure_transpose();
    auto t1 = std::chrono::steady_clock::now();
    st.time_factor_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
    ensure_krylov(*this, o.restart, 0);
    Krylov& K = *kry;
    const int n = ndim, G = vgrid(n);
    cudaStream_t s = stream;
    multidot<double><<<G, 256, 0, s>>>(n, 1, b, b, K.part); IEMIC_COUNT_LAUNCH();
    reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
    double bn2 = 0.0;
    ck(cudaMemcpyAsync(&bn2, K.dots, sizeof(double), cudaMemcpyDeviceToHost, s));
    ck(cudaStreamSynchronize(s));
    const double bnorm = std::sqrt(bn2);
    if (!std::isfinite(bnorm)) return IEMIC_ERR_NAN;
    ck(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    if (bnorm == 0.0) {
        st.relres = 0.0;
        return IEMIC_OK;
    }
    scale_by<double><<<G, 256, 0, s>>>(n, b, 1.0 / bnorm, K.r64); IEMIC_COUNT_LAUNCH();
    double est = 1.0;
    st.iters += gmres<double>(*this, *lu, d_rowT, d_colT, d_valT, K.r64, K.x64, o.restart, o.max_iters, o.tol, &est,
                              true);
    axpy_into<double><<<G, 256, 0, s>>>(n, bnorm, K.x64, x); IEMIC_COUNT_LAUNCH();
    residual_launch(n, d_rowT, d_colT, d_valT, x, b, K.r64, -1, s);
    multidot<double><<<G, 256, 0, s>>>(n, 1, K.r64, K.r64, K.part); IEMIC_COUNT_LAUNCH();
    reduce_parts<<<1, RT, 0, s>>>(G, 1, K.part, K.dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
    double rn2 = 0.0;
    ck(cudaMemcpyAsync(&rn2, K.dots, sizeof(double), cudaMemcpyDeviceToHost, s));
    ck(cudaStreamSynchronize(s));
    st.relres = std::sqrt(rn2) / bnorm;
    timer.drain();
    st.time_solve_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
    return st.relres <= o.tol ? IEMIC_OK : IEMIC_ERR_NOT_CONVERGED;
}

}  // namespace iemic

// ---------------------------------------------------------------------------
// small device-vector helpers for the Newton / continuation drivers
// ---------------------------------------------------------------------------
namespace iemic {
namespace {
__global__ void k_axpby(int n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) y[r] = a * x[r] + b * y[r];
}
}  // namespace
double dev_dot(Engine& e, const double* a, const double* b) {
    ensure_krylov(e, e.kry ? e.kry->m : 100, e.kry ? e.kry->prec : 0);
    const int n = e.ndim, G = vgrid(n);
    multidot<double><<<G, 256, 0, e.stream>>>(n, 1, a, b, e.kry->part); IEMIC_COUNT_LAUNCH();
    reduce_parts<<<1, RT, 0, e.stream>>>(G, 1, e.kry->part, e.kry->dots, nullptr, 0); IEMIC_COUNT_LAUNCH();
    double v = 0.0;
    ck(cudaMemcpyAsync(&v, e.kry->dots, sizeof(double), cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    return v;
}
__global__ void k_absmax_part(int n, const double* __restrict__ x, double* __restrict__ part) {
    double m = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) m = fmax(m, fabs(x[r]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (blockDim.x >> 5); ++w) m = fmax(m, sm[w]);
        part[blockIdx.x] = m;
    }
}
double dev_norm_inf(Engine& e, const double* a) {
    ensure_krylov(e, e.kry ? e.kry->m : 100, e.kry ? e.kry->prec : 0);
    const int G = vgrid(e.ndim);
    k_absmax_part<<<G, 256, 0, e.stream>>>(e.ndim, a, e.kry->part); IEMIC_COUNT_LAUNCH();
    std::vector<double> h(size_t(G), 0.0);
    ck(cudaMemcpyAsync(h.data(), e.kry->part, sizeof(double) * G, cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    double m = 0.0;
    for (double v : h) m = std::max(m, v);
    return m;
}
void dev_axpby(Engine& e, double a, const double* x, double b, double* y) {
    k_axpby<<<vgrid(e.ndim), 256, 0, e.stream>>>(e.ndim, a, x, b, y); IEMIC_COUNT_LAUNCH();
    ck(cudaGetLastError());
}
}  // namespace iemic
