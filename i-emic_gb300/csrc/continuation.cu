// Newton solver and pseudo-arclength continuation on the GPU engine.
//
// Host-side control flow restating the reference drivers, with every vector
// on the device and only scalars on the host:
//  - Newton: src/newton/Newton.H:40-100 (Run, RunBackTracking): x += dx with
//    J dx = -F until ||F||_2 < tolerance, halving back-tracking when the
//    residual grew.
//  - Continuation: Continuation<Model> (src/continuation/Continuation.H):
//    run 209-246, step 250-320, createInitialTangent 324-376, computeDFDPar
//    412-442, createTangent 446-518, normalize 522-566, eulerPredictor
//    570-606, newtonCorrector 610-837, runBackTracking 841-878, detect
//    882-950, adjustStep 974-1003, reset 1030-1065, store/restore 1068-1115,
//    with the defaults of getDefaultInitParameters (1335-1395).
//    Ocean::preProcess (src/ocean/Ocean.C:799-808) asks for a new
//    preconditioner at the start of each step; the next solve builds it and
//    the rest of the step reuses it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>

#include "engine.cuh"

namespace iemic {
double dev_dot(Engine& e, const double* a, const double* b);
double dev_norm_inf(Engine& e, const double* a);
void dev_axpby(Engine& e, double a, const double* x, double b, double* y);
}  // namespace iemic

using namespace iemic;

namespace {
using clk = std::chrono::steady_clock;
double ms_since(clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); }
int sgn(double v) { return (v > 0) - (v < 0); }

// Device vectors owned by one driver call.
struct DevVecs {
    std::vector<double*> v;
    DevVecs(Engine& e, int count) : v(size_t(count), nullptr) {
        for (auto& p : v) {
            if (cudaMalloc(&p, sizeof(double) * e.ndim) != cudaSuccess) {
                release();
                throw EngineError(IEMIC_ERR_NOMEM);
            }
            ck(cudaMemsetAsync(p, 0, sizeof(double) * e.ndim, e.stream));
        }
    }
    void release() {
        for (auto& p : v) {
            if (p) cudaFree(p);
            p = nullptr;
        }
    }
    ~DevVecs() { release(); }
};

// The model side of the drivers: F, J and solves with the reference's
// preconditioner policy, plus timing.
//
// Preconditioner policy (`policy`):
//  0  rebuilt once per continuation step (Ocean::preProcess,
//     src/ocean/Ocean.C:799-808) and reused for every later Jacobian of the step;
//  1  rebuilt after every new Jacobian;
//  2  as 0, plus a cost-balanced rebuild: a factorisation is reused while the
//     Krylov time spent beyond the iteration count of its first solve stays
//     below the time the factorisation itself took (the break-even rule of
//     rent-or-buy); once it exceeds it, the next solve refactors the current
//     Jacobian. The same budget caps a solve that runs on the factors of an
//     older Jacobian: when it is spent before the solve converges, the solve
//     is repeated on a fresh factorisation of the current Jacobian. After
//     such a failure, the later Jacobians of the same continuation step are
//     factorised directly when fresh factors themselves need at least 8
//     iterations: inexact (FP32) factors have little margin, and near a fold,
//     where the Jacobian moves fast, the next attempts on old factors fail as
//     well. Exact (FP64) factors, a few iterations when fresh and expensive to
//     rebuild, keep the budget rule.
struct ModelOps {
    Engine& e;
    iemic_solve_opts solve_opts;
    int policy = 0;
    bool recompute = true;   // set by pre_process
    long jac_gen = 0, fact_gen = -1;
    double t_asm = 0, t_fac = 0, t_sol = 0;
    int solves = 0, krylov = 0, facts = 0, unconverged = 0, retries = 0;
    double fact_ms = 0.0, excess_ms = 0.0;   // cost of the current factorisation, Krylov time beyond its first solve
    int base_iters = 0;                      // iterations of the first solve on the current factorisation
    double iter_ms = 0.0;                    // time of one Krylov iteration, from the last solve
    bool stale_failed = false;               // a solve on older factors failed in this step
    bool trace = false;

    ModelOps(Engine& en, const iemic_solve_opts& o, int pol) : e(en), solve_opts(o), policy(pol) {
        const char* t = std::getenv("IEMIC_SOLVE_TRACE");
        trace = t && *t && *t != '0';
    }
    void rhs(const double* x, double* F) {
        auto t = clk::now();
        e.rhs_dev(x, F);
        ck(cudaStreamSynchronize(e.stream));
        t_asm += ms_since(t);
    }
    void jacobian(const double* x) {
        auto t = clk::now();
        e.jacobian_dev(x);
        ck(cudaStreamSynchronize(e.stream));
        t_asm += ms_since(t);
        ++jac_gen;
    }
    void pre_process() {
        recompute = true;
        stale_failed = false;
    }
    int solve_once(const double* b, double* x, bool refactor, int cap) {
        iemic_solve_opts o = solve_opts;
        o.reuse_preconditioner = refactor ? 0 : 1;
        if (cap > 0 && cap < o.max_iters) o.max_iters = cap;
        iemic_solve_stats st{};
        int rc = e.solve_dev(b, x, o, st);
        if (rc != IEMIC_OK && rc != IEMIC_ERR_NOT_CONVERGED) throw EngineError(rc);
        if (refactor) {
            recompute = false;
            fact_gen = jac_gen;
        }
        if (st.factorizations > 0) {
            fact_ms = st.time_factor_ms;
            base_iters = st.iters;
            excess_ms = 0.0;
        } else if (st.iters > base_iters) {
            excess_ms += double(st.iters - base_iters) * st.time_solve_ms / double(st.iters);
        }
        if (st.iters > 0) iter_ms = st.time_solve_ms / double(st.iters);
        t_fac += st.time_factor_ms;
        t_sol += st.time_solve_ms;
        ++solves;
        krylov += st.iters;
        facts += st.factorizations;
        if (trace)
            std::fprintf(stderr, "iemic solve: jac %ld fact %ld iters %d relres %.3e factor_ms %.1f solve_ms %.1f%s\n",
                         jac_gen, fact_gen, st.iters, st.relres, st.time_factor_ms, st.time_solve_ms,
                         rc == IEMIC_OK ? "" : " NOT CONVERGED");
        return rc;
    }
    void solve(const double* b, double* x) {
        const bool newer = fact_gen != jac_gen;
        const bool need = recompute || (policy == 1 && newer) ||
                          (policy == 2 && newer && (excess_ms >= fact_ms || (stale_failed && base_iters >= 8)));
        const bool stale = policy == 2 && !need && newer;
        int cap = 0;
        if (stale && iter_ms > 0.0)   // iterations the remaining rebuild budget pays for
            cap = base_iters + std::max(10, int(std::ceil((fact_ms - excess_ms) / iter_ms)));
        int rc = solve_once(b, x, need, cap);
        if (rc == IEMIC_ERR_NOT_CONVERGED && stale) {
            ++retries;
            stale_failed = true;
            rc = solve_once(b, x, true, 0);
        }
        if (rc == IEMIC_ERR_NOT_CONVERGED) ++unconverged;
    }
    double dot(const double* a, const double* b) { return dev_dot(e, a, b); }
    double norm(const double* a) { return std::sqrt(dev_dot(e, a, a)); }
    double norm_inf(const double* a) { return dev_norm_inf(e, a); }
    void axpby(double a, const double* x, double b, double* y) { dev_axpby(e, a, x, b, y); }
    void copy(double* dst, const double* src) {
        ck(cudaMemcpyAsync(dst, src, sizeof(double) * e.ndim, cudaMemcpyDeviceToDevice, e.stream));
    }
    void set_par(int idx, double v) { e.set_par(idx, v); }
};

// Continuation<Model> state and algorithm.
struct Continuation {
    ModelOps& M;
    const iemic_continuation_opts& o;
    double* x;                                   // model state (device, in/out)
    double *x0, *x00, *xdot, *xdot0, *F, *Fc, *dFdPar, *y, *z, *diff;
    double par, ds, zeta = 1.0, pardot = 1.0;
    double par0, par00, ds0, ds00, pardot0 = 0.0;
    double ds_start;
    int newton_iter = 0, sum_newton = 0, step = 0, resets = 0;
    bool secant = false, fix_step = false, reached = false, abort_flag = false;
    int sign_monitor = 0;
    double norm_rhs = 0.0, norm_rhs_test = 0.0, last_res = 0.0;

    Continuation(ModelOps& m, const iemic_continuation_opts& opts, double* state, DevVecs& V)
        : M(m), o(opts), x(state) {
        double** ps[] = {&x0, &x00, &xdot, &xdot0, &F, &Fc, &dFdPar, &y, &z, &diff};
        for (size_t i = 0; i < sizeof(ps) / sizeof(ps[0]); ++i) *ps[i] = V.v[i];
        par = M.e.P.par[o.par_idx];
        ds = o.ds;
        ds_start = ds;
        ds0 = ds00 = ds;
        par0 = par00 = par;
        M.copy(x0, x);
        M.copy(x00, x);
        const double n = double(M.e.ndim);
        zeta = (o.normalize == 'O') ? 1.0 / n : o.tan_scaling / n;
    }

    // dFdPar = (F(par + eps) - F(par)) / eps and Fc = F(par); fresh (mode
    // 'F') recomputes F(par) first, otherwise F already holds it. F(par + eps)
    // goes straight into dFdPar, so F keeps F(par).
    void compute_dfdpar(bool fresh) {
        if (fresh) M.rhs(x, F);
        M.copy(Fc, F);
        M.set_par(o.par_idx, par + o.epsilon);
        M.rhs(x, dFdPar);
        M.set_par(o.par_idx, par);
        M.axpby(-1.0 / o.epsilon, Fc, 1.0 / o.epsilon, dFdPar);
    }

    void normalize() {
        if (o.normalize == 'O') {
            const double nx = M.norm(xdot);
            zeta = o.tan_scaling / nx;
            M.axpby(0.0, xdot, zeta, xdot);
            const double nrm = M.norm(xdot);
            const double comb = std::sqrt(nrm * nrm + 1.0);
            M.axpby(0.0, xdot, 1.0 / comb, xdot);
            pardot = 1.0 / comb;
        } else {
            const double nrm = M.norm(xdot);
            const double comb = std::sqrt(zeta * nrm * nrm + 1.0);
            pardot = 1.0 / comb;
            M.axpby(0.0, xdot, pardot, xdot);
        }
    }

    void initial_tangent() {
        compute_dfdpar(true);
        if (o.initial_tangent == 'A') {
            M.axpby(-1.0, dFdPar, 0.0, xdot);
        } else {
            M.pre_process();
            M.jacobian(x);
            M.axpby(-1.0, dFdPar, 0.0, diff);
            M.solve(diff, xdot);
        }
        normalize();
    }

    void create_tangent(char mode) {
        if (mode == 'S') {
            M.copy(xdot, x);
            M.axpby(-1.0 / ds0, x0, 1.0 / ds0, xdot);
            pardot = (par - par0) / ds0;
        } else {
            if (o.newton_chord) {
                compute_dfdpar(true);
                M.jacobian(x);
                M.axpby(-1.0, dFdPar, 0.0, diff);
                M.solve(diff, xdot);
            } else {
                M.axpby(0.0, xdot, -1.0, xdot);   // xdot holds y of the corrector
            }
            normalize();
        }
    }

    void store() {
        std::swap(x00, x0);
        M.copy(x0, x);
        M.copy(xdot0, xdot);
        par00 = par0;
        par0 = par;
        ds00 = ds0;
        ds0 = ds;
        pardot0 = pardot;
    }

    void restore() {
        M.copy(x, x0);
        par = par0;
        M.set_par(o.par_idx, par);
        ds = ds0;
        M.copy(xdot, xdot0);
        std::swap(x0, x00);   // state0 <- state00
        M.copy(x00, x);       // state00 <- current model state
        par0 = par00;
        ds0 = ds00;
    }

    int euler_predictor() {
        M.axpby(ds, xdot, 1.0, x);
        par = par + ds * pardot;
        M.set_par(o.par_idx, par);
        M.rhs(x, F);
        const double r = M.norm(F);
        if (!std::isfinite(r)) return 1;
        return r > o.predictor_bound ? 1 : 0;
    }

    int newton_corrector() {
        double res = 100.0;
        const double nx0 = M.norm(x0);
        newton_iter = 0;
        while (newton_iter < o.max_newton) {
            compute_dfdpar(newton_iter == 0);
            norm_rhs = M.norm(Fc);
            M.axpby(-1.0, Fc, 0.0, Fc);           // R = -F(par)
            M.copy(diff, x);
            M.axpby(-1.0, x0, 1.0, diff);         // state - state0
            const double pdiff = par - par0;
            double rbp;
            if (o.normalize == 'O')
                rbp = ds - M.dot(xdot, diff) * zeta - pardot * pdiff;
            else
                rbp = ds * ds - M.dot(diff, diff) * zeta - pdiff * pdiff;
            M.jacobian(x);
            if (!o.newton_chord) M.solve(dFdPar, y);
            M.solve(Fc, z);
            double pdir;
            if (o.normalize == 'O') {
                if (o.newton_chord)
                    pdir = (rbp - zeta * M.dot(xdot, z)) / (pardot + zeta * M.dot(xdot, xdot));
                else
                    pdir = (rbp - zeta * M.dot(xdot, z)) / (pardot - zeta * M.dot(xdot, y));
            } else {
                if (o.newton_chord)
                    pdir = (rbp - 2 * zeta * M.dot(diff, z)) /
                           (2 * pdiff + 2 * (zeta / pdiff) * M.dot(diff, diff));
                else
                    pdir = (rbp - 2 * zeta * M.dot(diff, z)) / (2 * pdiff - 2 * zeta * M.dot(diff, y));
            }
            if (o.newton_chord)
                M.axpby(pdir, xdot, 1.0, z);
            else
                M.axpby(-pdir, y, 1.0, z);
            M.axpby(1.0, z, 1.0, x);
            par = par + pdir;
            M.set_par(o.par_idx, par);
            ++newton_iter;
            ++sum_newton;
            M.rhs(x, F);
            norm_rhs_test = M.norm(F);
            if (!std::isfinite(norm_rhs_test) || !std::isfinite(par)) return 1;
            if (norm_rhs_test > o.predictor_bound) return 1;
            if (o.backtracking_steps > 0 && norm_rhs < norm_rhs_test) {
                if (back_tracking(z, pdir)) return 1;
            }
            const double ndx = M.norm(z);
            if (ndx > 1e3 * nx0 && nx0 > 0) return 1;
            if (o.residual_test == 'R')
                res = norm_rhs_test;
            else
                res = std::max(std::fabs(pdir), M.norm_inf(z));
            if (res < o.newton_tol && newton_iter >= o.min_newton) break;
        }
        if (!o.newton_chord) M.copy(xdot, y);   // stateDot = y for createTangent('E')
        last_res = res;
        return res > o.newton_tol ? 1 : 0;
    }

    int back_tracking(const double* dir, double pdir) {
        double reduction = -0.5;
        for (int b = 0; b < o.backtracking_steps; ++b) {
            if (norm_rhs_test < norm_rhs * o.backtracking_increase) break;
            M.axpby(reduction, dir, 1.0, x);
            par = par + reduction * pdir;
            M.set_par(o.par_idx, par);
            M.rhs(x, F);
            norm_rhs_test = M.norm(F);
            reduction /= 2.0;
        }
        return norm_rhs_test > norm_rhs * o.backtracking_increase ? 1 : 0;
    }

    int do_step() {
        M.pre_process();
        if (euler_predictor()) return 1;
        if (newton_corrector()) return 1;
        create_tangent(o.tangent);
        return 0;
    }

    void reset() {
        restore();
        const int s = sgn(ds) ? sgn(ds) : 1;
        ds = s * std::max(std::fabs(ds) / o.decrease, std::fabs(o.ds_min));
        ++resets;
        fix_step = true;
        if (std::fabs(ds) <= std::fabs(o.ds_min) && (resets >= 100 || o.give_up_at_ds_min)) abort_flag = true;
    }

    void detect() {
        const double f0 = par0 - o.destination, f1 = par - o.destination;
        if (sign_monitor == 0) sign_monitor = sgn(f1);
        if (sign_monitor != sgn(f1) && !secant) {
            secant = true;
            ds_start = ds;
        } else {
            sign_monitor = sgn(f1);
        }
        if (secant) {
            ds = -f1 * ds / (f1 - f0);
            create_tangent('S');
        }
        if (secant && std::fabs(f1) < o.destination_tol) {
            secant = false;
            ds = ds_start;
            fix_step = true;
            reached = true;   // one destination
        }
    }

    void adjust_step() {
        if (secant || fix_step) {
            fix_step = false;
            return;
        }
        double factor = o.opt_newton / double(newton_iter);
        factor = std::min(2.0, std::max(0.5, factor));
        ds *= factor;
        if (std::fabs(ds) > std::fabs(o.ds_max)) ds = sgn(ds) * std::fabs(o.ds_max);
        if (std::fabs(ds) < std::fabs(o.ds_min)) ds = sgn(ds) * std::fabs(o.ds_min);
    }

    void run(iemic_continuation_stats& s) {
        initial_tangent();
        int failed = 0;
        while (!reached && step != o.max_steps && !abort_flag) {
            ++step;
            store();
            if (do_step()) {
                if (M.trace)
                    std::fprintf(stderr, "iemic step %d FAILED: par %.9g newton %d res %.3e\n", step, par,
                                 newton_iter, last_res);
                reset();
                ++failed;
                continue;
            }
            if (M.trace)
                std::fprintf(stderr, "iemic step %d: par %.9g ds %.3e newton %d res %.3e\n", step, par, ds,
                             newton_iter, last_res);
            detect();
            adjust_step();
        }
        s.steps = step;
        s.failed_steps = failed;
        s.newton_iters = sum_newton;
        s.par = par;
        s.ds = ds;
        s.rhs_norm = M.norm(F);
        s.reached_destination = reached ? 1 : 0;
        s.aborted = abort_flag ? 1 : 0;
    }
};

// ---- theta method (ThetaModel<Ocean>, src/transient/ThetaModel.H:64-140) ----
// G = B (x_old - x) + (dt (1 - theta) F_old + dt theta F), in the order of the
// Epetra updates of ThetaModel::computeRHS (unfused products and sums)
__global__ void k_theta_rhs(int n, const double* __restrict__ B, const double* __restrict__ xold,
                            const double* __restrict__ x, const double* __restrict__ Fold, double a, double b,
                            double* __restrict__ FG) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double bxdot = __dmul_rn(B[r], __dadd_rn(-x[r], xold[r]));
        const double f = __dadd_rn(__dmul_rn(a, Fold[r]), __dmul_rn(b, FG[r]));
        FG[r] = __dadd_rn(bxdot, f);
    }
}
// J2 = J - B / (theta dt) on the diagonal (ThetaModel::computeJacobian)
__global__ void k_theta_diag(int n, const int* __restrict__ diagpos, const double* __restrict__ B, double dt,
                             double theta, double* __restrict__ val) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int q = diagpos[r];
        if (q >= 0) val[q] = __dadd_rn(val[q], -B[r] / dt / theta);
    }
}
__global__ void k_scale(int n, double s, const double* __restrict__ x, double* __restrict__ y) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) y[r] = __dmul_rn(x[r], s);
}
int vblocks(int n) { return std::min((n + 255) / 256, 152 * 8); }

// CSR position of each row's diagonal entry (-1 if the maximal graph has none)
const int* diag_positions(Engine& e) {
    if (!e.d_diagpos) {
        const std::vector<int>& ci = e.host_col_idx();
        std::vector<int> pos(size_t(e.ndim), -1);
        for (int r = 0; r < e.ndim; ++r)
            for (int q = e.row_ptr[r]; q < e.row_ptr[r + 1]; ++q)
                if (ci[q] == r) pos[r] = q;
        e.d_diagpos = static_cast<int*>(e.dalloc(sizeof(int) * pos.size()));
        ck(cudaMemcpyAsync(e.d_diagpos, pos.data(), sizeof(int) * pos.size(), cudaMemcpyHostToDevice, e.stream));
        ck(cudaStreamSynchronize(e.stream));
    }
    return e.d_diagpos;
}

}  // namespace

extern "C" {

void iemic_default_newton_opts(iemic_newton_opts* o) {
    if (!o) return;
    o->max_iters = 10;             // Newton::maxNumIterations_
    o->tol = 1.0e-3;               // Newton::toleranceRHS_ on ||F||_2
    o->backtracking_steps = 10;    // Newton::numBackTrackingSteps_
    iemic_default_solve_opts(&o->solve);
    o->refactor_each_iter = 1;
}

int iemic_newton_dev(iemic_ocean* h, double* x, const iemic_newton_opts* opts, iemic_newton_stats* st) {
    if (!h || !x) return IEMIC_ERR_ARG;
    iemic_newton_opts o;
    iemic_default_newton_opts(&o);
    if (opts) o = *opts;
    if (o.max_iters < 0 || o.backtracking_steps < 0) return IEMIC_ERR_ARG;
    iemic_newton_stats s{};
    Engine& e = h->e;
    int rc = IEMIC_OK;
    auto t0 = clk::now();
    try {
        DevVecs V(e, 3);
        double *F = V.v[0], *dx = V.v[1], *b = V.v[2];
        ModelOps M(e, o.solve, o.refactor_each_iter);
        M.rhs(x, F);
        double norm_rhs = M.norm(F), test = norm_rhs;
        s.rhs_norm0 = norm_rhs;
        if (!std::isfinite(norm_rhs)) throw EngineError(IEMIC_ERR_NAN);
        bool converged = false;
        for (s.iters = 0; s.iters < o.max_iters; ++s.iters) {
            M.jacobian(x);
            M.pre_process();
            M.axpby(-1.0, F, 0.0, b);
            M.solve(b, dx);
            M.axpby(1.0, dx, 1.0, x);
            M.rhs(x, F);
            test = M.norm(F);
            if (!std::isfinite(test)) throw EngineError(IEMIC_ERR_NAN);
            if (test < o.tol) {
                converged = true;
                ++s.iters;
                break;
            }
            if (norm_rhs < test) {   // RunBackTracking
                double reduction = -0.5;
                for (int bt = 0; bt < o.backtracking_steps; ++bt) {
                    if (test < norm_rhs) break;
                    M.axpby(reduction, dx, 1.0, x);
                    M.rhs(x, F);
                    test = M.norm(F);
                    reduction /= 2.0;
                    ++s.backtracks;
                }
            }
            norm_rhs = test;
        }
        if (!converged) rc = IEMIC_ERR_NOT_CONVERGED;
        s.rhs_norm = test;
        s.linear_solves = M.solves;
        s.krylov_iters = M.krylov;
        s.factorizations = M.facts;
        s.time_assembly_ms = M.t_asm;
        s.time_factor_ms = M.t_fac;
        s.time_solve_ms = M.t_sol;
    } catch (const EngineError& err) {
        rc = err.code;
    } catch (...) {
        rc = IEMIC_ERR_CUDA;
    }
    s.time_ms = ms_since(t0);
    if (st) *st = s;
    return rc;
}

static int with_device_state(iemic_ocean* h, double* x, const std::function<int(double*)>& fn) {
    Engine& e = h->e;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * e.ndim) != cudaSuccess) return IEMIC_ERR_NOMEM;
    int rc = IEMIC_OK;
    if (cudaMemcpy(d, x, sizeof(double) * e.ndim, cudaMemcpyHostToDevice) != cudaSuccess) rc = IEMIC_ERR_CUDA;
    if (rc == IEMIC_OK) rc = fn(d);
    if (cudaMemcpy(x, d, sizeof(double) * e.ndim, cudaMemcpyDeviceToHost) != cudaSuccess && rc == IEMIC_OK)
        rc = IEMIC_ERR_CUDA;
    cudaFree(d);
    return rc;
}

int iemic_newton(iemic_ocean* h, double* x, const iemic_newton_opts* opts, iemic_newton_stats* st) {
    if (!h || !x) return IEMIC_ERR_ARG;
    return with_device_state(h, x, [&](double* d) { return iemic_newton_dev(h, d, opts, st); });
}

void iemic_default_continuation_opts(iemic_continuation_opts* o) {
    if (!o) return;
    // getDefaultInitParameters (src/continuation/Continuation.H:1335-1395)
    o->par_idx = 19;   // "Combined Forcing"
    o->ds = 1.0e-2;
    o->ds_min = 1.0e-8;
    o->ds_max = 1.0e3;
    o->decrease = 2.0;
    o->destination = 1.0;
    o->destination_tol = 1.0e-7;
    o->max_steps = -1;
    o->max_newton = 7;
    o->min_newton = 1;
    o->opt_newton = 3.5;
    o->newton_tol = 1.0e-4;
    o->residual_test = 'D';
    o->normalize = 'N';
    o->tangent = 'S';
    o->initial_tangent = 'E';
    o->epsilon = 1.0e-5;
    o->tan_scaling = 1.0;
    o->predictor_bound = 1.0e3;
    o->backtracking_steps = 0;
    o->backtracking_increase = 0.0;
    o->newton_chord = 0;
    o->give_up_at_ds_min = 1;
    iemic_default_solve_opts(&o->solve);
    o->refactor_each_newton = 0;
}

int iemic_continuation_run_dev(iemic_ocean* h, double* x, const iemic_continuation_opts* opts,
                               iemic_continuation_stats* st) {
    if (!h || !x) return IEMIC_ERR_ARG;
    iemic_continuation_opts o;
    iemic_default_continuation_opts(&o);
    if (opts) o = *opts;
    if (o.par_idx < 1 || o.par_idx > NPAR || !(o.epsilon != 0.0) || !(o.decrease > 0.0) || o.max_newton < 1 ||
        (o.normalize != 'O' && o.normalize != 'N') || (o.tangent != 'E' && o.tangent != 'S') ||
        (o.initial_tangent != 'E' && o.initial_tangent != 'A' && o.initial_tangent != 'S') ||
        (o.residual_test != 'R' && o.residual_test != 'D') || !(o.ds != 0.0))
        return IEMIC_ERR_ARG;
    iemic_continuation_stats s{};
    Engine& e = h->e;
    int rc = IEMIC_OK;
    auto t0 = clk::now();
    try {
        DevVecs V(e, 10);
        ModelOps M(e, o.solve, o.refactor_each_newton);
        Continuation C(M, o, x, V);
        C.run(s);
        if (C.abort_flag) rc = IEMIC_ERR_NOT_CONVERGED;
        s.linear_solves = M.solves;
        s.unconverged_solves = M.unconverged;
        s.krylov_iters = M.krylov;
        s.factorizations = M.facts;
        s.time_assembly_ms = M.t_asm;
        s.time_factor_ms = M.t_fac;
        s.time_solve_ms = M.t_sol;
    } catch (const EngineError& err) {
        rc = err.code;
    } catch (...) {
        rc = IEMIC_ERR_CUDA;
    }
    s.time_ms = ms_since(t0);
    if (st) *st = s;
    return rc;
}

int iemic_continuation_run(iemic_ocean* h, double* x, const iemic_continuation_opts* opts,
                           iemic_continuation_stats* st) {
    if (!h || !x) return IEMIC_ERR_ARG;
    return with_device_state(h, x, [&](double* d) { return iemic_continuation_run_dev(h, d, opts, st); });
}

void iemic_default_theta_opts(iemic_theta_opts* o) {
    if (!o) return;
    o->theta = 1.0;        // ThetaModel "theta"
    o->dt = 1.0e-3;        // ThetaModel::timestep_ before initStep
    o->tol = 1.0e-8;       // transient Newton "Newton tolerance"
    o->max_newton = 20;    // "maximum Newton iterations"
    iemic_default_solve_opts(&o->solve);
    o->refactor_policy = 2;
}

// ThetaModel::initStep + Newton<ThetaModel>::run (src/transient/Newton.H:77-110)
int iemic_theta_step_dev(iemic_ocean* h, double* x, const iemic_theta_opts* opts, iemic_theta_stats* st) {
    if (!h || !x) return IEMIC_ERR_ARG;
    iemic_theta_opts o;
    iemic_default_theta_opts(&o);
    if (opts) o = *opts;
    if (!(o.theta > 0.0 && o.theta <= 1.0) || !(o.dt > 0.0) || o.max_newton < 0 || o.refactor_policy < 0 ||
        o.refactor_policy > 2)
        return IEMIC_ERR_ARG;
    iemic_theta_stats s{};
    Engine& e = h->e;
    int rc = IEMIC_OK;
    auto t0 = clk::now();
    try {
        DevVecs V(e, 4);
        double *xold = V.v[0], *Fold = V.v[1], *G = V.v[2], *dx = V.v[3];
        ModelOps M(e, o.solve, o.refactor_policy);
        const int* diagpos = diag_positions(e);
        const int n = e.ndim, nb = vblocks(n);
        const double a = o.dt * (1.0 - o.theta), b = o.dt * o.theta, scale = 1.0 / o.dt / o.theta;
        // initStep: the old state, Ocean::preProcess, F(x_old)
        M.copy(xold, x);
        M.pre_process();
        M.rhs(xold, Fold);
        auto residual = [&](const double* xc) {   // G(xc), ThetaModel::computeRHS
            M.rhs(xc, G);
            k_theta_rhs<<<nb, 256, 0, e.stream>>>(n, e.d_B, xold, xc, Fold, a, b, G); IEMIC_COUNT_LAUNCH();
            ck(cudaGetLastError());
        };
        residual(x);
        s.norm_G = -1.0;
        double gnorm = M.norm(G);
        for (s.newton_iters = 0; s.newton_iters < o.max_newton;) {
            // Jsol: J2 at x, J2 dx = G / (theta dt). The linear tolerance is
            // relaxed to what the Newton test needs: a linear residual below
            // 0.1 tol in G's units; near convergence G is at round-off level
            // and a 1e-8 relative solve of it is neither reachable nor needed.
            M.solve_opts.tol = gnorm > 0.0 ? std::max(o.solve.tol, 0.1 * o.tol / gnorm) : o.solve.tol;
            M.jacobian(x);
            k_theta_diag<<<nb, 256, 0, e.stream>>>(n, diagpos, e.d_B, o.dt, o.theta, e.d_val); IEMIC_COUNT_LAUNCH();
            k_scale<<<nb, 256, 0, e.stream>>>(n, scale, G, G); IEMIC_COUNT_LAUNCH();
            M.solve(G, dx);
            s.norm_dx = M.norm_inf(dx);
            M.axpby(-1.0, dx, 1.0, x);
            residual(x);
            s.norm_G = gnorm = M.norm(G);
            ++s.newton_iters;
            if (!std::isfinite(s.norm_G) || !std::isfinite(s.norm_dx)) throw EngineError(IEMIC_ERR_NAN);
            if (s.norm_dx < o.tol && s.norm_G < o.tol) {
                s.converged = 1;
                break;
            }
            if (s.norm_dx > 1e2) break;   // "Norm exploding"
        }
        if (!s.converged) rc = IEMIC_ERR_NOT_CONVERGED;
        s.linear_solves = M.solves;
        s.krylov_iters = M.krylov;
        s.factorizations = M.facts;
        s.time_assembly_ms = M.t_asm;
        s.time_factor_ms = M.t_fac;
        s.time_solve_ms = M.t_sol;
    } catch (const EngineError& err) {
        rc = err.code;
    } catch (...) {
        rc = IEMIC_ERR_CUDA;
    }
    s.time_ms = ms_since(t0);
    if (st) *st = s;
    return rc;
}

int iemic_theta_step(iemic_ocean* h, double* x, const iemic_theta_opts* opts, iemic_theta_stats* st) {
    if (!h || !x) return IEMIC_ERR_ARG;
    return with_device_state(h, x, [&](double* d) { return iemic_theta_step_dev(h, d, opts, st); });
}

}  // extern "C"
