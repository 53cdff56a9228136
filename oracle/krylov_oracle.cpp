// CPU FP64 Krylov solver (TEST INFRASTRUCTURE and CPU BASELINE ONLY).
//
// Right-preconditioned restarted GMRES with Givens-rotated Hessenberg least
// squares (the scheme of src/gmressolver/GMRESSolverDecl.H and of Belos
// BlockGmresSolMgr with block size 1 used by src/ocean/Ocean.C:971-1030),
// preconditioned by an incomplete LU factorisation of the Jacobian in the
// maximal-graph CSR layout. Zero or tiny pivots are replaced by a floor,
// the rule MRILU documents for its ILDU (mrilu/precon/incldup.F90).
// Loaded only by tests/ and by bench.py's CPU-baseline leg.
#include "thcm_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Csr {
    int n;
    const int* rp;
    const int* ci;
    const double* v;
};

void spmv(const Csr& A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A.n; ++i) {
        double s = 0.0;
        for (int q = A.rp[i]; q < A.rp[i + 1]; ++q) s += A.v[q] * x[A.ci[q]];
        y[i] = s;
    }
}
double dot(int n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

// Point ILU(0) in natural ordering (IKJ variant) with a relative pivot floor.
struct Ilu0 {
    int n;
    std::vector<int> rp, ci, diag;
    std::vector<double> lu;
    void factor(const Csr& A) {
        n = A.n;
        rp.assign(A.rp, A.rp + n + 1);
        ci.assign(A.ci, A.ci + rp[n]);
        lu.assign(A.v, A.v + rp[n]);
        diag.assign(n, -1);
        std::vector<int> pos(n, -1);
        for (int i = 0; i < n; ++i) {
            double rowmax = 0.0;
            for (int q = rp[i]; q < rp[i + 1]; ++q) {
                pos[ci[q]] = q;
                rowmax = std::max(rowmax, std::fabs(lu[q]));
                if (ci[q] == i) diag[i] = q;
            }
            for (int q = rp[i]; q < rp[i + 1] && ci[q] < i; ++q) {
                int k = ci[q];
                double lik = lu[q] / lu[diag[k]];
                lu[q] = lik;
                for (int r = diag[k] + 1; r < rp[k + 1]; ++r) {
                    int p = pos[ci[r]];
                    if (p >= 0) lu[p] -= lik * lu[r];
                }
            }
            double floor_ = 1e-8 * (rowmax > 0 ? rowmax : 1.0);
            double& d = lu[diag[i]];
            if (std::fabs(d) < floor_) d = (d < 0 ? -floor_ : floor_);
            for (int q = rp[i]; q < rp[i + 1]; ++q) pos[ci[q]] = -1;
        }
    }
    void apply(const double* r, double* z) const {
        for (int i = 0; i < n; ++i) {
            double s = r[i];
            for (int q = rp[i]; q < diag[i]; ++q) s -= lu[q] * z[ci[q]];
            z[i] = s;
        }
        for (int i = n - 1; i >= 0; --i) {
            double s = z[i];
            for (int q = diag[i] + 1; q < rp[i + 1]; ++q) s -= lu[q] * z[ci[q]];
            z[i] = s / lu[diag[i]];
        }
    }
};

// Block ILU(0) on 6x6 cell blocks (all unknowns of one grid cell), natural
// cell ordering; diagonal blocks inverted by Gauss-Jordan with partial
// pivoting and a relative pivot floor.
struct Bilu0 {
    static constexpr int B = 6;
    int nb;
    std::vector<int> brp, bci, bdiag;
    std::vector<double> blk;   // 36 doubles per block, row-major
    std::vector<double> dinv;  // inverted diagonal blocks
    static void inv6(const double* a, double* out) {
        double m[B][2 * B];
        double amax = 0.0;
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) {
                m[r][c] = a[r * B + c];
                m[r][B + c] = (r == c);
                amax = std::max(amax, std::fabs(a[r * B + c]));
            }
        double floor_ = 1e-8 * (amax > 0 ? amax : 1.0);
        for (int c = 0; c < B; ++c) {
            int piv = c;
            for (int r = c + 1; r < B; ++r)
                if (std::fabs(m[r][c]) > std::fabs(m[piv][c])) piv = r;
            if (piv != c)
                for (int q = 0; q < 2 * B; ++q) std::swap(m[c][q], m[piv][q]);
            if (std::fabs(m[c][c]) < floor_) m[c][c] = (m[c][c] < 0 ? -floor_ : floor_);
            double d = 1.0 / m[c][c];
            for (int q = 0; q < 2 * B; ++q) m[c][q] *= d;
            for (int r = 0; r < B; ++r)
                if (r != c && m[r][c] != 0.0) {
                    double f = m[r][c];
                    for (int q = 0; q < 2 * B; ++q) m[r][q] -= f * m[c][q];
                }
        }
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) out[r * B + c] = m[r][B + c];
    }
    static void mm(const double* a, const double* b, double* c) {   // c = a*b
        for (int r = 0; r < B; ++r)
            for (int q = 0; q < B; ++q) {
                double s = 0.0;
                for (int k = 0; k < B; ++k) s += a[r * B + k] * b[k * B + q];
                c[r * B + q] = s;
            }
    }
    void factor(const Csr& A) {
        nb = A.n / B;
        brp.assign(nb + 1, 0);
        bci.clear();
        std::vector<int> mark(nb, -1);
        for (int I = 0; I < nb; ++I) {
            std::vector<int> cols;
            for (int r = 0; r < B; ++r)
                for (int q = A.rp[I * B + r]; q < A.rp[I * B + r + 1]; ++q) {
                    int J = A.ci[q] / B;
                    if (mark[J] != I) { mark[J] = I; cols.push_back(J); }
                }
            std::sort(cols.begin(), cols.end());
            bci.insert(bci.end(), cols.begin(), cols.end());
            brp[I + 1] = int(bci.size());
        }
        blk.assign(bci.size() * 36, 0.0);
        bdiag.assign(nb, -1);
        for (int I = 0; I < nb; ++I) {
            for (int q = brp[I]; q < brp[I + 1]; ++q) if (bci[q] == I) bdiag[I] = q;
            for (int r = 0; r < B; ++r)
                for (int q = A.rp[I * B + r]; q < A.rp[I * B + r + 1]; ++q) {
                    int J = A.ci[q] / B, c = A.ci[q] % B;
                    int p = int(std::lower_bound(bci.begin() + brp[I], bci.begin() + brp[I + 1], J) - bci.begin());
                    blk[size_t(p) * 36 + r * B + c] = A.v[q];
                }
        }
        dinv.assign(size_t(nb) * 36, 0.0);
        std::vector<int> pos(nb, -1);
        double tmp[36];
        for (int I = 0; I < nb; ++I) {
            for (int q = brp[I]; q < brp[I + 1]; ++q) pos[bci[q]] = q;
            for (int q = brp[I]; q < brp[I + 1] && bci[q] < I; ++q) {
                int K = bci[q];
                mm(&blk[size_t(q) * 36], &dinv[size_t(K) * 36], tmp);   // L_IK = A_IK * D_K^{-1}
                std::memcpy(&blk[size_t(q) * 36], tmp, sizeof tmp);
                for (int r = bdiag[K] + 1; r < brp[K + 1]; ++r) {
                    int p = pos[bci[r]];
                    if (p < 0) continue;
                    double t2[36];
                    mm(&blk[size_t(q) * 36], &blk[size_t(r) * 36], t2);
                    for (int e = 0; e < 36; ++e) blk[size_t(p) * 36 + e] -= t2[e];
                }
            }
            inv6(&blk[size_t(bdiag[I]) * 36], &dinv[size_t(I) * 36]);
            for (int q = brp[I]; q < brp[I + 1]; ++q) pos[bci[q]] = -1;
        }
    }
    void apply(const double* r, double* z) const {
        double t[B];
        for (int I = 0; I < nb; ++I) {
            for (int a = 0; a < B; ++a) t[a] = r[I * B + a];
            for (int q = brp[I]; q < bdiag[I]; ++q) {
                const double* L = &blk[size_t(q) * 36];
                const double* zz = &z[bci[q] * B];
                for (int a = 0; a < B; ++a) for (int c = 0; c < B; ++c) t[a] -= L[a * B + c] * zz[c];
            }
            for (int a = 0; a < B; ++a) z[I * B + a] = t[a];
        }
        for (int I = nb - 1; I >= 0; --I) {
            for (int a = 0; a < B; ++a) t[a] = z[I * B + a];
            for (int q = bdiag[I] + 1; q < brp[I + 1]; ++q) {
                const double* U = &blk[size_t(q) * 36];
                const double* zz = &z[bci[q] * B];
                for (int a = 0; a < B; ++a) for (int c = 0; c < B; ++c) t[a] -= U[a * B + c] * zz[c];
            }
            const double* D = &dinv[size_t(I) * 36];
            for (int a = 0; a < B; ++a) {
                double s = 0.0;
                for (int c = 0; c < B; ++c) s += D[a * B + c] * t[c];
                z[I * B + a] = s;
            }
        }
    }
};

}  // namespace

extern "C" int oracle_gmres(int n, const int* rp, const int* ci, const double* v, const double* b,
                            double* x, const iemic_oracle_solve_opts* o, iemic_oracle_solve_stats* st) {
#ifdef _OPENMP
    if (o->threads > 0) omp_set_num_threads(o->threads);
#endif
    Csr A{n, rp, ci, v};
    Ilu0 ilu;
    Bilu0 bilu;
    if (o->precond == 1) ilu.factor(A);
    if (o->precond == 2) bilu.factor(A);
    auto prec = [&](const double* r, double* z) {
        if (o->precond == 1) ilu.apply(r, z);
        else if (o->precond == 2) bilu.apply(r, z);
        else std::memcpy(z, r, sizeof(double) * n);
    };
    const int m = o->restart;
    std::vector<double> V(size_t(m + 1) * n), Z(size_t(m) * n), H(size_t(m + 1) * m), cs(m), sn(m), g(m + 1);
    std::vector<double> r(n), w(n);
    double bnorm = std::sqrt(dot(n, b, b));
    if (bnorm == 0.0) bnorm = 1.0;
    int it = 0;
    double relres = 1.0;
    st->status = 1;
    while (it < o->maxit) {
        spmv(A, x, r.data());
        for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
        double beta = std::sqrt(dot(n, r.data(), r.data()));
        relres = beta / bnorm;
        if (relres <= o->tol) { st->status = 0; break; }
        for (int i = 0; i < n; ++i) V[i] = r[i] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        for (; j < m && it < o->maxit; ++j, ++it) {
            prec(&V[size_t(j) * n], &Z[size_t(j) * n]);
            spmv(A, &Z[size_t(j) * n], w.data());
            // classical Gram-Schmidt with one reorthogonalisation pass (CGS2)
            for (int pass = 0; pass < 2; ++pass)
                for (int i = 0; i <= j; ++i) {
                    double h = dot(n, &V[size_t(i) * n], w.data());
                    if (pass == 0) H[size_t(i) * m + j] = h; else H[size_t(i) * m + j] += h;
                    const double* vi = &V[size_t(i) * n];
                    for (int q = 0; q < n; ++q) w[q] -= h * vi[q];
                }
            double hn = std::sqrt(dot(n, w.data(), w.data()));
            H[size_t(j + 1) * m + j] = hn;
            if (hn > 0) for (int q = 0; q < n; ++q) V[size_t(j + 1) * n + q] = w[q] / hn;
            for (int i = 0; i < j; ++i) {
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
            relres = std::fabs(g[j + 1]) / bnorm;
            if (relres <= o->tol || hn == 0.0) { ++j; ++it; break; }
        }
        // back substitution and update with the preconditioned basis
        std::vector<double> y(j);
        for (int i = j - 1; i >= 0; --i) {
            double s = g[i];
            for (int q = i + 1; q < j; ++q) s -= H[size_t(i) * m + q] * y[q];
            y[i] = s / H[size_t(i) * m + i];
        }
        for (int i = 0; i < j; ++i) {
            const double* zi = &Z[size_t(i) * n];
            for (int q = 0; q < n; ++q) x[q] += y[i] * zi[q];
        }
        if (relres <= o->tol) {
            st->status = 0;
            break;
        }
    }
    spmv(A, x, r.data());
    for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
    st->explicit_relres = std::sqrt(dot(n, r.data(), r.data())) / bnorm;
    st->iters = it;
    st->relres = relres;
    if (st->explicit_relres > o->tol * 10) st->status = 1;
    return st->status;
}
