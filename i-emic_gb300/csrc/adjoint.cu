// Steady-state adjoint of the THCM ocean: the gradient of a scalar diagnostic
// g(x) at a steady state F(x, p) = 0 with respect to the surface forcing
// fields and the parameters,
//   dg/dtheta = -lambda^T dF/dtheta,   J(x)^T lambda = dg/dx,
// with the transposed solve preconditioned by the same factorisation as the
// forward solves (Engine::solve_transpose_dev).
//
// The diagnostic is the meridional overturning streamfunction of
// Ocean::getPsiM (src/ocean/Ocean.C:882-896) built by
// OceanGrid::recomputePsiM (src/ocean/OceanGrid.C:268-340) and
// compute_psim (src/ocean/thcm_utils.F90:95-118):
//   vs(j,k) = dx sum_i v(i,j,k),
//   psi(j,k) = -cos(yv_j) vs(j,k) dz dfzT(k) + psi(j,k-1) where z(k) hdim < -500 m, else 0,
// in Sv (times r0dim hdim udim 1e-6), and g = max over (j,k) of psi, with the
// sum over i optionally restricted to a longitude sector.
#include <chrono>
#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.cuh"

namespace iemic {
double dev_dot(Engine& e, const double* a, const double* b);
}  // namespace iemic

using namespace iemic;

namespace {
constexpr double kR0dim = 6.37e+06, kUdim = 0.1e+00;   // src/ocean/usr.F90:134-135

int grid_of(int n) { return std::max(1, std::min((n + 255) / 256, 152 * 8)); }

// vs(j,k) for j = 1..m, k = 1..l over the sector [i0, i1): one block per (j,k)
__global__ void k_psim_vs(int n, int m, int l, int i0, int i1, double dx, const double* __restrict__ x,
                          double* __restrict__ vs) {
    const int jk = blockIdx.x, j = jk % m, k = jk / m;   // 0-based
    double s = 0.0;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
        s += x[size_t(NUN) * (size_t(i) + size_t(n) * (size_t(j) + size_t(m) * k)) + (VV - 1)];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) t += ws[w];
        vs[jk] = t * dx;
    }
}

// dg/dx for g = psi(j*, k*): d psi / d v(i, j*, k') for k' <= k* (all levels
// up to k* lie deeper than 500 m, or psi(j*,k*) would be zero)
__global__ void k_psim_grad(int n, int m, int l, int i0, int i1, int js, int ks, const double* __restrict__ wk,
                            double* __restrict__ grad) {
    const size_t ndim = size_t(NUN) * n * m * l;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < ndim; q += size_t(gridDim.x) * blockDim.x) {
        double v = 0.0;
        if (int(q % NUN) == VV - 1) {
            const size_t c = q / NUN;
            const int i = int(c % n), j = int((c / n) % m), k = int(c / (size_t(n) * m));
            if (j + 1 == js && k + 1 <= ks && i >= i0 && i < i1) v = wk[k + 1];
        }
        grad[q] = v;
    }
}

struct Psim {
    std::vector<double> psi;   // (m+1) x (l+1), psi[(m+1)*k + j]
    double pmin = 0, pmax = 0;
    int jmax = 0, kmax = 0;
};

// psi from vs (host, FP64), in Sv
Psim psim_from_vs(const Engine& e, const std::vector<double>& vs) {
    const int m = e.cfg.m, l = e.cfg.l;
    const double scale = kR0dim * e.cfg.hdim * kUdim * 1e-6;
    Psim P;
    P.psi.assign(size_t(m + 1) * (l + 1), 0.0);
    for (int j = 1; j <= m; ++j) {
        const double cs = std::cos(e.yv[j]);
        for (int k = 1; k <= l; ++k)
            if (e.z[k] * e.cfg.hdim < -500)
                P.psi[size_t(m + 1) * k + j] =
                    -cs * vs[size_t(m) * (k - 1) + (j - 1)] * e.dz * e.dfzT[k] + P.psi[size_t(m + 1) * (k - 1) + j];
    }
    P.pmin = P.pmax = P.psi[0];
    for (int j = 0; j <= m; ++j)
        for (int k = 0; k <= l; ++k) {
            const double v = P.psi[size_t(m + 1) * k + j];
            if (v > P.pmax) {
                P.pmax = v;
                P.jmax = j;
                P.kmax = k;
            }
            P.pmin = std::min(P.pmin, v);
        }
    for (double& v : P.psi) v *= scale;
    P.pmin *= scale;
    P.pmax *= scale;
    return P;
}

Psim psim_dev(Engine& e, const double* x_dev, int i0, int i1) {
    const int n = e.cfg.n, m = e.cfg.m, l = e.cfg.l;
    double* vs_dev = e.d_v2;   // m*l <= ndim scratch
    k_psim_vs<<<m * l, 128, 0, e.stream>>>(n, m, l, i0, i1, e.dx, x_dev, vs_dev); IEMIC_COUNT_LAUNCH();
    std::vector<double> vs(size_t(m) * l);
    ck(cudaMemcpyAsync(vs.data(), vs_dev, sizeof(double) * vs.size(), cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    return psim_from_vs(e, vs);
}

// grad = d psi(j*, k*) / dx (Sv per unit state)
void psim_grad_dev(Engine& e, int i0, int i1, int js, int ks, double* grad) {
    const int n = e.cfg.n, m = e.cfg.m, l = e.cfg.l;
    const double scale = kR0dim * e.cfg.hdim * kUdim * 1e-6;
    std::vector<double> wk(size_t(l) + 1, 0.0);
    if (js >= 1 && ks >= 1) {
        const double cs = std::cos(e.yv[js]);
        for (int k = 1; k <= ks; ++k) wk[k] = -cs * e.dx * e.dz * e.dfzT[k] * scale;
    }
    double* wk_dev = e.d_v2;
    ck(cudaMemcpyAsync(wk_dev, wk.data(), sizeof(double) * wk.size(), cudaMemcpyHostToDevice, e.stream));
    k_psim_grad<<<grid_of(e.ndim), 256, 0, e.stream>>>(n, m, l, i0, i1, js, ks, wk_dev, grad); IEMIC_COUNT_LAUNCH();
    ck(cudaGetLastError());
}

// -lambda^T dF/dpar by central differences of the residual
double par_adjoint_dev(Engine& e, const double* x_dev, const double* lambda, int idx, double rel, double* w1,
                       double* w2) {
    const double p0 = e.P.par[idx];
    const double h = rel * std::max(1.0, std::fabs(p0));
    e.set_par(idx, p0 + h);
    e.rhs_dev(x_dev, w1);
    e.set_par(idx, p0 - h);
    e.rhs_dev(x_dev, w2);
    e.set_par(idx, p0);
    const double a = dev_dot(e, lambda, w1), b = dev_dot(e, lambda, w2);
    return -(a - b) / (2.0 * h);
}

bool sector_ok(const Engine& e, int i0, int i1) { return i0 >= 0 && i1 <= e.cfg.n && i0 < i1; }
}  // namespace

#define GUARD_BEGIN try {
#define GUARD_END                                              \
    }                                                          \
    catch (const EngineError& err) { return err.code; }        \
    catch (...) { return IEMIC_ERR_CUDA; }                     \
    return IEMIC_OK;

extern "C" {

int iemic_psim(iemic_ocean* h, const double* x, double* psim, double* psi_min, double* psi_max) {
    if (!h || !x) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    ck(cudaMemcpyAsync(e.d_v1, x, sizeof(double) * e.ndim, cudaMemcpyHostToDevice, e.stream));
    const Psim P = psim_dev(e, e.d_v1, 0, e.cfg.n);
    if (psim) std::copy(P.psi.begin(), P.psi.end(), psim);
    if (psi_min) *psi_min = P.pmin;
    if (psi_max) *psi_max = P.pmax;
    GUARD_END
}

int iemic_psim_max_grad_dev(iemic_ocean* h, const double* x_dev, int i_begin, int i_end, double* g, int* jk,
                            double* grad_dev) {
    if (!h || !x_dev || !grad_dev || !sector_ok(h->e, i_begin, i_end)) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    const Psim P = psim_dev(e, x_dev, i_begin, i_end);
    if (g) *g = P.pmax;
    if (jk) {
        jk[0] = P.jmax;
        jk[1] = P.kmax;
    }
    psim_grad_dev(e, i_begin, i_end, P.jmax, P.kmax, grad_dev);
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_forcing_adjoint_dev(iemic_ocean* h, const double* lambda_dev, double* grad_dev) {
    if (!h || !lambda_dev || !grad_dev) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    launch_dfdsurf_t(e.geo, e.fs, lambda_dev, grad_dev, e.stream);
    ck(cudaGetLastError());
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_par_adjoint_dev(iemic_ocean* h, const double* x_dev, const double* lambda_dev, int par_idx, double fd_rel,
                          double* out) {
    if (!h || !x_dev || !lambda_dev || !out || par_idx < 1 || par_idx > NPAR || !(fd_rel > 0)) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    *out = par_adjoint_dev(e, x_dev, lambda_dev, par_idx, fd_rel, e.d_v1, e.d_v2);
    GUARD_END
}

void iemic_default_adjoint_opts(iemic_adjoint_opts* o) {
    if (!o) return;
    o->i_begin = 0;
    o->i_end = -1;
    iemic_default_solve_opts(&o->solve);
    o->solve.precision = IEMIC_PREC_MIXED;
    o->solve.tol = 1e-10;
    o->fd_rel = 1e-6;
}

int iemic_adjoint_psim(iemic_ocean* h, const double* x, const iemic_adjoint_opts* opts, double* grad_fields,
                       const int* par_idx, int npar, double* grad_par, iemic_adjoint_stats* st) {
    if (!h || !x || npar < 0 || (npar > 0 && (!par_idx || !grad_par))) return IEMIC_ERR_ARG;
    iemic_adjoint_opts o;
    iemic_default_adjoint_opts(&o);
    if (opts) o = *opts;
    Engine& e = h->e;
    if (o.i_end < 0) o.i_end = e.cfg.n;
    if (!sector_ok(e, o.i_begin, o.i_end) || !(o.fd_rel > 0)) return IEMIC_ERR_ARG;
    for (int q = 0; q < npar; ++q)
        if (par_idx[q] < 1 || par_idx[q] > NPAR) return IEMIC_ERR_ARG;
    iemic_adjoint_stats s{};
    auto t0 = std::chrono::steady_clock::now();
    const size_t nb = sizeof(double) * size_t(e.ndim);
    double *xs = nullptr, *gx = nullptr, *lam = nullptr, *gf = nullptr, *w1 = nullptr, *w2 = nullptr;
    int rc = IEMIC_OK;
    try {
        double** bufs[] = {&xs, &gx, &lam, &w1, &w2};
        for (double** b : bufs)
            if (cudaMalloc(b, nb) != cudaSuccess) throw EngineError(IEMIC_ERR_NOMEM);
        if (cudaMalloc(&gf, sizeof(double) * 5 * size_t(e.cfg.n) * e.cfg.m) != cudaSuccess)
            throw EngineError(IEMIC_ERR_NOMEM);
        ck(cudaMemcpyAsync(xs, x, nb, cudaMemcpyHostToDevice, e.stream));
        // g and dg/dx
        const Psim P = psim_dev(e, xs, o.i_begin, o.i_end);
        s.g = P.pmax;
        s.jmax = P.jmax;
        s.kmax = P.kmax;
        psim_grad_dev(e, o.i_begin, o.i_end, P.jmax, P.kmax, gx);
        // J^T lambda = dg/dx with the forward solve's factorisation
        e.jacobian_dev(xs);
        iemic_solve_opts so = o.solve;
        so.transpose = 1;
        so.reuse_preconditioner = 0;
        iemic_solve_stats ss{};
        rc = e.solve_dev(gx, lam, so, ss);
        s.iters = ss.iters;
        s.relres = ss.relres;
        if (rc == IEMIC_OK || rc == IEMIC_ERR_NOT_CONVERGED) {
            const int rc_solve = rc;
            if (grad_fields) {
                launch_dfdsurf_t(e.geo, e.fs, lam, gf, e.stream);
                ck(cudaMemcpyAsync(grad_fields, gf, sizeof(double) * 5 * size_t(e.cfg.n) * e.cfg.m,
                                   cudaMemcpyDeviceToHost, e.stream));
            }
            for (int q = 0; q < npar; ++q) grad_par[q] = par_adjoint_dev(e, xs, lam, par_idx[q], o.fd_rel, w1, w2);
            ck(cudaStreamSynchronize(e.stream));
            rc = rc_solve;
        }
    } catch (const EngineError& err) {
        rc = err.code;
    } catch (...) {
        rc = IEMIC_ERR_CUDA;
    }
    for (double* b : {xs, gx, lam, gf, w1, w2})
        if (b) cudaFree(b);
    s.time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st) *st = s;
    return rc;
}

}  // extern "C"
