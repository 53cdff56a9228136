// THCM Jacobian / residual assembly kernels (GB300, sm_103a).
//
// One thread evaluates one matrix row (one unknown of one cell). Its
// coefficients live in registers, one per canonical maximal-graph entry
// (stencil.cuh). The thread then applies the land-mask surgery of
// src/ocean/boundary.F90 and the |c| > 1e-10 drop rule of
// src/ocean/assemble.F90:115. It writes the row straight into its
// precomputed CSR slots (Jacobian), or accumulates A_rhs(x)*x in the Fortran
// CSR order (residual). The dense 27x6x6 An array of the reference is never
// formed.
//
// Every coefficient is built with the operation order of the Fortran
// expression it restates (src/ocean/usrc.F90 lin / nlin_jac / nlin_rhs,
// src/ocean/spf.F90 atoms). This file is compiled with -fmad=false, so the
// FP64 results are bit-identical to an unfused evaluation of the reference's
// arithmetic on the same host-computed metric tables.
#include "ocean_impl.cuh"

namespace iemic {
namespace {

constexpr double ALPT1 = 2.93, ALPT2 = 8.3e-02, ALPT3 = 6.6e-04;

// ---------------------------------------------------------------------------
// lin: state-independent coefficients Al(kk,A,B) for one (j,k, surface-land)
// class (src/ocean/usrc.F90:605-789, uncoupled branch). Within a latitude row
// and level, Al depends on i only through landm(i,j,l) (spf.F90 tderiv 3-6).
// ---------------------------------------------------------------------------
__device__ double al_value(const Geo& g, const Params& P, int A, int kk, int B, int j, int k, double lm) {
    const double EV = P.par[EK_V], EH = P.par[EK_H];
    const double ph = (1 - P.par[MIXP]) * P.par[PE_H], pv = P.par[PE_V];
    const double lambda = P.par[LAMB], xes = P.par[NLES], bi = P.par[BIOT], Ra = P.par[RAYL];
    if ((A == UU && B == UU) || (A == VV && B == VV)) {
        double xx, yy, cs;
        if (A == UU) {   // uderiv 2,3,5
            double a = g.J(JT_UXX, j);
            xx = (kk == 2 || kk == 8) ? a : (kk == 5 ? -(a + a) : 0.0);
            double a4 = g.J(JT_UYY4, j), a6 = g.J(JT_UYY6, j);
            yy = kk == 4 ? a4 : (kk == 6 ? a6 : (kk == 5 ? -(a4 + a6) : 0.0));
            cs = kk == 5 ? g.J(JT_UCSI, j) : 0.0;
        } else {         // vderiv 2,3,5
            xx = (kk == 2 || kk == 8) ? g.J(JT_VXX, j) : (kk == 5 ? g.J(JT_VXX5, j) : 0.0);
            double a4 = g.J(JT_VYY4, j), a6 = g.J(JT_VYY6, j);
            yy = kk == 4 ? a4 : (kk == 6 ? a6 : (kk == 5 ? -(a4 + a6) : 0.0));
            cs = kk == 5 ? g.J(JT_VCSI, j) : 0.0;
        }
        double z14 = g.K(KT_UZZ14, k), z23 = g.K(KT_UZZ23, k);   // u/vderiv 4
        double zz = kk == 14 ? z14 : (kk == 23 ? z23 : (kk == 5 ? -(z14 + z23) : 0.0));
        return -EH * (xx + yy + cs) - EV * zz;
    }
    if (A == UU && B == VV) {   // -fv - EH*vxs
        double fv = kk == 5 ? g.J(JT_CORV, j) : 0.0;
        double vxs = kk == 2 ? g.J(JT_UXS2, j) : (kk == 8 ? g.J(JT_UXS8, j) : 0.0);
        return -fv - EH * vxs;
    }
    if (A == VV && B == UU) {   // fu - EH*uxs
        double fu = kk == 5 ? g.J(JT_CORV, j) : 0.0;
        double uxs = kk == 2 ? g.J(JT_VXS2, j) : (kk == 8 ? g.J(JT_VXS8, j) : 0.0);
        return fu - EH * uxs;
    }
    if (A == UU && B == PP) {   // gradp 1
        double c = g.J(JT_PXC, j);
        return (kk == 5 || kk == 6) ? -c : ((kk == 8 || kk == 9) ? c : 0.0);
    }
    if (A == VV && B == PP) {   // gradp 2
        double c = g.J(JT_PYC, j);
        return (kk == 5 || kk == 8) ? -c : ((kk == 6 || kk == 9) ? c : 0.0);
    }
    if (A == WW && B == PP)     // gradp 3
        return kk == 5 ? g.K(KT_PZ5, k) : (kk == 23 ? g.K(KT_PZ23, k) : 0.0);
    if (A == WW && (B == TT || B == SS)) {   // tderiv 6
        double tbc = (kk == 5 || kk == 23) ? 1.0 * lm : 0.0;
        if (B == TT) return -Ra * (1. + xes * ALPT1) * tbc / 2.;
        return lambda * Ra * tbc / 2.;
    }
    if (A == PP && B == UU) {   // pderiv 1
        double c = g.J(JT_UXC, j);
        return (kk == 2 || kk == 1) ? -c : ((kk == 4 || kk == 5) ? c : 0.0);
    }
    if (A == PP && B == VV)     // pderiv 2
        return (kk == 4 || kk == 1) ? g.J(JT_VYC4, j) : ((kk == 2 || kk == 5) ? g.J(JT_VYC2, j) : 0.0);
    if (A == PP && B == WW)     // pderiv 3
        return kk == 5 ? g.K(KT_WZC5, k) : (kk == 14 ? g.K(KT_WZC14, k) : 0.0);
    if ((A == TT && B == TT) || (A == SS && B == SS)) {   // tderiv 1/2,3,4,5
        double c = g.J(JT_TXX, j);
        double tx = (kk == 2 || kk == 8) ? c * lm : (kk == 5 ? -(2 * c * lm) : 0.0);
        double a4 = g.J(JT_TYY4, j) * lm, a6 = g.J(JT_TYY6, j) * lm;
        double ty = kk == 4 ? a4 : (kk == 6 ? a6 : (kk == 5 ? -(a4 + a6) : 0.0));
        double a14 = g.K(KT_TZZ14, k) * lm, a23 = (k < g.l) ? g.K(KT_TZZ23, k) * lm : 0.0;
        double tz = kk == 14 ? a14 : (kk == 23 ? a23 : (kk == 5 ? -(a14 + a23) : 0.0));
        double tc = (kk == 5 && k == g.l) ? 1.0 : 0.0;
        int RES = (A == TT) ? P.TRES : P.SRES;
        return -ph * (tx + ty) - pv * tz + RES * bi * tc;
    }
    return 0.0;
}

__global__ void lin_kernel(Geo g, Params P, double* al_tab) {
    // one thread per (j, k, Ls, e)
    const int total = g.m * g.l * 2 * CELL_ENTRIES;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        int e = t % CELL_ENTRIES;
        int rest = t / CELL_ENTRIES;
        int ls = rest % 2;
        int jk = rest / 2;
        int j = jk % g.m + 1, k = jk / g.m + 1;
        int A = row_of_cell_entry(e);
        Ent en = entry(A, e - rowoff(A));
        al_tab[t] = al_value(g, P, A, en.kk, en.B, j, k, ls ? 0.0 : 1.0);
    }
}

// ---------------------------------------------------------------------------
// usol (src/ocean/usrc.F90:1014-1121): halo-padded u,v,w,t,s in one
// (n+2)(m+2)(l+2) layout each. The Fortran sequence of boundary assignments is
// evaluated per padded point; stage order is kept (the k-halo copies are taken
// before land zeroing, as in the reference).
// ---------------------------------------------------------------------------
__device__ double xval(const double* x, const Geo& g, int i, int j, int k, int XX) {
    return x[size_t(NUN) * (size_t(i - 1) + size_t(g.n) * (size_t(j - 1) + size_t(g.m) * (k - 1))) + XX - 1];
}
// u or v after the i-, j- and k-boundary stages, before land zeroing
__device__ double uv_bc(const double* x, const Geo& g, int i, int j, int k, int XX) {
    const int n = g.n, m = g.m, l = g.l;
    if (k == 0 || k == l + 1) {
        if (i < 1 || i > n || j < 1 || j > m) return 0.0;
        return uv_bc(x, g, i, j, k == 0 ? 1 : l, XX);
    }
    if (k < 1 || k > l) return 0.0;
    if (j >= 1 && j <= m && i >= 1 && i <= n && (j == m)) return 0.0;   // j-stage: u(i,M,k) = 0
    if (i >= 1 && i <= n && (j == 0)) return 0.0;                       // j-stage: u(i,0,k) = 0
    if (j < 1 || j > m) return 0.0;
    if (g.periodic) {
        if (i == 0) return xval(x, g, n, j, k, XX);
        if (i >= 1 && i <= n) return xval(x, g, i, j, k, XX);
        return 0.0;
    }
    if (i == 0 || i == n) return 0.0;
    if (i >= 1 && i <= n) return xval(x, g, i, j, k, XX);
    return 0.0;
}
__device__ bool uv_land_zero(const Geo& g, int i, int j, int k) {
    // zeroed by a land cell (I,J,k) with (I,J) in {(i,j),(i+1,j),(i,j+1),(i+1,j+1)}
    if (k < 1 || k > g.l) return false;
    for (int dj = 0; dj <= 1; ++dj)
        for (int di = 0; di <= 1; ++di) {
            int I = i + di, J = j + dj;
            if (I >= 1 && I <= g.n && J >= 1 && J <= g.m && g.L(I, J, k) == 1) return true;
        }
    return false;
}
__device__ double w_bc(const double* x, const Geo& g, int i, int j, int k) {
    const int n = g.n, m = g.m, l = g.l;
    if (k < 1 || k > l || j < 1 || j > m) return 0.0;
    if (k == l && i >= 1 && i <= n) return 0.0;                 // w(i,j,l) = 0
    if (i >= 1 && i <= n) return xval(x, g, i, j, k, WW);
    if (g.periodic) {
        if (i == n + 1) return xval(x, g, 1, j, k, WW);
        if (i == 0) return xval(x, g, n, j, k, WW);
    }
    return 0.0;
}
__device__ double ts_bc(const double* x, const Geo& g, int i, int j, int k, int XX) {
    const int n = g.n, m = g.m, l = g.l;
    if (k == 0 || k == l + 1) {
        if (i < 1 || i > n || j < 1 || j > m) return 0.0;
        return xval(x, g, i, j, k == 0 ? 1 : l, XX);
    }
    if (j == 0 || j == m + 1) {
        if (i < 1 || i > n) return 0.0;
        return xval(x, g, i, j == 0 ? 1 : m, k, XX);
    }
    if (i >= 1 && i <= n) return xval(x, g, i, j, k, XX);
    if (g.periodic) return xval(x, g, i == 0 ? n : 1, j, k, XX);
    return xval(x, g, i == 0 ? 1 : n, j, k, XX);
}

__global__ void usol_kernel(Geo g, const double* __restrict__ x, double* __restrict__ pads) {
    const size_t np = g.npad();
    for (size_t p = size_t(blockIdx.x) * blockDim.x + threadIdx.x; p < np; p += size_t(gridDim.x) * blockDim.x) {
        int i = int(p % (g.n + 2));
        size_t r = p / (g.n + 2);
        int j = int(r % (g.m + 2));
        int k = int(r / (g.m + 2));
        bool lz = uv_land_zero(g, i, j, k);
        double u = (i <= g.n) ? uv_bc(x, g, i, j, k, UU) : 0.0;
        double v = (i <= g.n) ? uv_bc(x, g, i, j, k, VV) : 0.0;
        if (lz) { u = 0.0; v = 0.0; }
        pads[p] = u;
        pads[np + p] = v;
        pads[2 * np + p] = (k <= g.l) ? w_bc(x, g, i, j, k) : 0.0;
        pads[3 * np + p] = ts_bc(x, g, i, j, k, TT);
        pads[4 * np + p] = ts_bc(x, g, i, j, k, SS);
    }
}

// ---------------------------------------------------------------------------
// Per-cell context for the nonlinear atoms (src/ocean/spf.F90:362-790)
// ---------------------------------------------------------------------------
struct Cell {
    int i, j, k;          // 1-based
    double lm;            // 1 - landm(i,j,l)
    const double* f[5];   // padded u, v, w, t, s
    const Geo* g;
    __device__ double at(int q, int di, int dj, int dk) const { return f[q][g->pad(i + di, j + dj, k + dk)]; }
    __device__ double U(int a, int b, int c) const { return at(0, a, b, c); }
    __device__ double V(int a, int b, int c) const { return at(1, a, b, c); }
    __device__ double W(int a, int b, int c) const { return at(2, a, b, c); }
};

// uwz / vwz (unlin 5, vnlin 5)
__device__ __forceinline__ double atom_wz(int kk, const Cell& c) {
    const Geo& g = *c.g;
    double t = g.K(KT_TDZ8, c.k);
    double a23 = (c.W(0, 0, 0) + c.W(0, 1, 0) + c.W(1, 0, 0) + c.W(1, 1, 0)) * t;
    double a14 = -(c.W(0, 0, -1) + c.W(0, 1, -1) + c.W(1, 0, -1) + c.W(1, 1, -1)) * t;
    return kk == 23 ? a23 : (kk == 14 ? a14 : (kk == 5 ? a14 + a23 : 0.0));
}
// Urwz / Vrwz (unlin 6, vnlin 6) with q = 0 (u) or 1 (v)
__device__ __forceinline__ double atom_rwz(int kk, const Cell& c, int q) {
    const Geo& g = *c.g;
    double t = g.K(KT_TDZ8, c.k);
    if (kk == 5 || kk == 6 || kk == 8 || kk == 9) return (c.at(q, 0, 0, 0) + c.at(q, 0, 0, 1)) * t;
    if (kk == 14 || kk == 15 || kk == 17 || kk == 18) return -(c.at(q, 0, 0, 0) + c.at(q, 0, 0, -1)) * t;
    return 0.0;
}
// x-advection atoms: value*cux at kk=8 (i<=n-1), -value*cux at kk=2 (i>=2), field q,
// scaled by `two` (uux/uvx: 1, Urux: 2)
__device__ __forceinline__ double atom_x(int kk, const Cell& c, int q, bool two) {
    const Geo& g = *c.g;
    double cx = g.J(JT_CUX, c.j);
    if (kk == 8 && c.i <= g.n - 1) return (two ? 2 * c.at(q, 1, 0, 0) : c.at(q, 1, 0, 0)) * cx;
    if (kk == 2 && c.i >= 2) return -(two ? 2 * c.at(q, -1, 0, 0) : c.at(q, -1, 0, 0)) * cx;
    return 0.0;
}
// y-advection atoms (uvy1/Urvy1/vvry/Vrvy)
__device__ __forceinline__ double atom_y(int kk, const Cell& c, int q, bool two) {
    const Geo& g = *c.g;
    double cy = g.J(JT_CUY, c.j);
    if (kk == 6 && c.j <= g.m - 1)
        return (two ? 2 * c.at(q, 0, 1, 0) : c.at(q, 0, 1, 0)) * g.J(JT_COSYV, c.j + 1) * cy;
    if (kk == 4 && c.j >= 2)
        return -(two ? 2 * c.at(q, 0, -1, 0) : c.at(q, 0, -1, 0)) * g.J(JT_COSYV, c.j - 1) * cy;
    return 0.0;
}
// metric atoms u*tan(yv) (uvy2 q=1, Urvy2/wvrz q=0, Urt2 q=0 two)
__device__ __forceinline__ double atom_tan(int kk, const Cell& c, int q, bool two) {
    if (kk != 5) return 0.0;
    double v = c.at(q, 0, 0, 0);
    return (two ? 2 * v : v) * c.g->J(JT_TANYV, c.j);
}
// tracer advection atoms, tnlin types 2..7, tracer field q (3 = T, 4 = S)
__device__ __forceinline__ double atom_urTx(int kk, const Cell& c, int q) {   // type 2
    const Geo& g = *c.g;
    double cx = g.J(JT_CTX, c.j);
    if (kk == 2 || kk == 1) return -(c.at(q, 0, 0, 0) + c.at(q, -1, 0, 0)) * cx * c.lm;
    if (kk == 4 || kk == 5) return (c.at(q, 1, 0, 0) + c.at(q, 0, 0, 0)) * cx * c.lm;
    return 0.0;
}
__device__ __forceinline__ double atom_Utrx(int kk, const Cell& c) {   // type 3
    const Geo& g = *c.g;
    double cx = g.J(JT_CTX, c.j);
    double a2 = -(c.U(-1, 0, 0) + c.U(-1, -1, 0)) * cx * c.lm;
    double a8 = (c.U(0, 0, 0) + c.U(0, -1, 0)) * cx * c.lm;
    return kk == 2 ? a2 : (kk == 8 ? a8 : (kk == 5 ? a2 + a8 : 0.0));
}
__device__ __forceinline__ double atom_vrTy(int kk, const Cell& c, int q) {   // type 4
    const Geo& g = *c.g;
    double cy = g.J(JT_CTY, c.j);
    if (kk == 4 || kk == 1)
        return -cy * (c.at(q, 0, 0, 0) + c.at(q, 0, -1, 0)) * g.J(JT_COSYV, c.j - 1) * c.lm;
    if (kk == 5 || kk == 2)
        return cy * (c.at(q, 0, 1, 0) + c.at(q, 0, 0, 0)) * g.J(JT_COSYV, c.j) * c.lm;
    return 0.0;
}
__device__ __forceinline__ double atom_Vtry(int kk, const Cell& c) {   // type 5
    const Geo& g = *c.g;
    double cy = g.J(JT_CTY, c.j);
    double a4 = -(c.V(0, -1, 0) + c.V(-1, -1, 0)) * cy * g.J(JT_COSYV, c.j - 1) * c.lm;
    double a6 = (c.V(0, 0, 0) + c.V(-1, 0, 0)) * cy * g.J(JT_COSYV, c.j) * c.lm;
    return kk == 4 ? a4 : (kk == 6 ? a6 : (kk == 5 ? a4 + a6 : 0.0));
}
__device__ __forceinline__ double atom_wrTz(int kk, const Cell& c, int q) {   // type 6
    const Geo& g = *c.g;
    double d = g.K(KT_DFZT, c.k);
    if (kk == 14) return -g.tdzi2 * c.lm * (c.at(q, 0, 0, 0) + c.at(q, 0, 0, -1)) / d;
    if (kk == 5 && c.k <= g.l - 1) return g.tdzi2 * c.lm * (c.at(q, 0, 0, 1) + c.at(q, 0, 0, 0)) / d;
    return 0.0;
}
__device__ __forceinline__ double atom_Wtrz(int kk, const Cell& c) {   // type 7
    const Geo& g = *c.g;
    double d = g.K(KT_DFZT, c.k);
    double a14 = -c.W(0, 0, -1) * c.lm * g.tdzi2 / d;
    double a23 = c.W(0, 0, 0) * c.lm * g.tdzi2 / d;
    return kk == 14 ? a14 : (kk == 23 ? a23 : (kk == 5 ? a14 + a23 : 0.0));
}
// wnlin types 1..4 (src/ocean/spf.F90:486-542)
__device__ __forceinline__ double atom_wnlin(int type, int kk, const Cell& c) {
    if (c.k > c.g->l - 1 || (kk != 5 && kk != 23)) return 0.0;
    double t0 = c.at(3, 0, 0, 0), t1 = c.at(3, 0, 0, 1);
    switch (type) {
    case 1: return (t0 + t1) / 2.;
    case 2: return kk == 23 ? t1 / 4. : (t0 + 2 * t1) / 4.;
    case 3: { double q = t0 + t1; return 0.375 * (q * q); }
    default: return kk == 5 ? 0.125 * (t0 * t0 + 3 * t1 * t0 + 3 * t1 * t1) : 0.125 * t1 * t1;
    }
}

// An(kk,A,B) for the Jacobian: Al + nlin_jac terms (src/ocean/usrc.F90:890-1012)
template <int A, int B>
__device__ __forceinline__ double an_jac(double al, int kk, const Cell& c, const Params& P) {
    const double epsr = P.par[ROSB];
    if constexpr (A == UU && B == UU)
        return al + epsr * (atom_x(kk, c, 0, true) + atom_y(kk, c, 1, false) + atom_wz(kk, c) + atom_tan(kk, c, 1, false));
    else if constexpr (A == UU && B == VV)
        return al + epsr * (atom_y(kk, c, 0, false) + atom_tan(kk, c, 0, false));
    else if constexpr (A == UU && B == WW)
        return al + epsr * atom_rwz(kk, c, 0);
    else if constexpr (A == VV && B == UU)
        return al + epsr * (atom_tan(kk, c, 0, true) + atom_x(kk, c, 1, false));
    else if constexpr (A == VV && B == VV)
        return al + epsr * (atom_x(kk, c, 0, false) + atom_y(kk, c, 1, true) + atom_wz(kk, c));
    else if constexpr (A == VV && B == WW)
        return al + epsr * atom_rwz(kk, c, 1);
    else if constexpr (A == WW && B == TT) {
        const double Ra = P.par[RAYL], xes = P.par[NLES];
        return al - Ra * xes * ALPT2 * atom_wnlin(1, kk, c) + Ra * xes * ALPT3 * atom_wnlin(3, kk, c);
    } else if constexpr ((A == TT || A == SS) && B == UU)
        return al + atom_urTx(kk, c, A == TT ? 3 : 4);
    else if constexpr ((A == TT || A == SS) && B == VV)
        return al + atom_vrTy(kk, c, A == TT ? 3 : 4);
    else if constexpr ((A == TT || A == SS) && B == WW)
        return al + atom_wrTz(kk, c, A == TT ? 3 : 4);
    else if constexpr ((A == TT && B == TT) || (A == SS && B == SS))
        return al + atom_Utrx(kk, c) + atom_Vtry(kk, c) + atom_Wtrz(kk, c);
    else
        return al;
}
// An(kk,A,B) for the residual: Al + nlin_rhs terms (src/ocean/usrc.F90:792-887).
// The tracer atoms (tnlin 3,5,7) read only u, v, w, so T and S share them.
template <int A, int B>
__device__ __forceinline__ double an_rhs(double al, int kk, const Cell& c, const Params& P) {
    const double epsr = P.par[ROSB];
    if constexpr (A == UU && B == UU)
        return al + epsr * (atom_x(kk, c, 0, false) + atom_y(kk, c, 1, false) + atom_wz(kk, c) + atom_tan(kk, c, 1, false));
    else if constexpr (A == VV && B == UU)
        return al + epsr * atom_tan(kk, c, 0, false);
    else if constexpr (A == VV && B == VV)
        return al + epsr * (atom_x(kk, c, 0, false) + atom_y(kk, c, 1, false) + atom_wz(kk, c));
    else if constexpr (A == WW && B == TT) {
        const double Ra = P.par[RAYL], xes = P.par[NLES];
        return al - Ra * xes * ALPT2 * atom_wnlin(2, kk, c) + Ra * xes * ALPT3 * atom_wnlin(4, kk, c);
    } else if constexpr ((A == TT && B == TT) || (A == SS && B == SS))
        return al + atom_Utrx(kk, c) + atom_Vtry(kk, c) + atom_Wtrz(kk, c);
    else
        return al;
}

// ---------------------------------------------------------------------------
// Vertical mixing and convective adjustment (src/ocean/mix_imp.f, Mixing >= 1)
// of one water column: the implicit vertical mixing Ftimp/Fsimp (P_VC) and
// the consistent vertical mixing Ftzt/Fszt (ALPC < 1) at the top faces
// k-1 and k of cell (i,j,k), and the T/S divergence terms of vmix_fun
// (mix_imp.f:231-562) in its operation order. The horizontal neutral-physics
// and Gent-McWilliams fluxes are zero (MIXP = MKAP = 0, checked on the host),
// so their two divergence stages leave mix(row) = +0.0 exactly.
// ---------------------------------------------------------------------------
// tanh by one explicit algorithm, shared operation for operation with the
// oracle (the platform tanh's last bit is implementation-defined): |y| < 2^-27
// gives y, |y| > 22 gives +-1, otherwise e/(e+2) with e = expm1(2|y|) from a
// degree-13 Taylor series, after Cody-Waite reduction by ln2 above ln2/2.
__device__ __forceinline__ double expm1_taylor(double r) {
    const double c[13] = {0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26,
                          0x1.27e4fb7789f5cp-22, 0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16,
                          0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7,
                          0x1.5555555555555p-5,  0x1.5555555555555p-3,  0x1.0p-1,
                          0x1.0p+0};   // 1/13!, ..., 1/1!
    double p = c[0];
#pragma unroll
    for (int q = 1; q < 13; ++q) p = p * r + c[q];
    return p * r;
}
__device__ __forceinline__ double tanh_x(double y) {
    const double a = fabs(y);
    if (!(a >= 0x1p-27)) return y;
    if (a > 22.0) return y > 0 ? 1.0 : -1.0;
    const double x = 2.0 * a;
    double e;
    if (x <= 0x1.62e42fefa39efp-2) {
        e = expm1_taylor(x);
    } else {
        const double kf = rint(x / 0x1.62e42fefa39efp-1);
        const double r = (x - kf * 0x1.62e42fee00000p-1) - kf * 0x1.a39ef35793c76p-33;
        e = ldexp(expm1_taylor(r) + 1.0, int(kf)) - 1.0;
    }
    const double t = e / (e + 2.0);
    return y < 0 ? -t : t;
}
// tprstb (mix_imp.f:835-856): max(tanh((-grad fac)^3), 0)
__device__ __forceinline__ double tprstb(double grad, double fac) {
    const double q = -grad * fac;
    const double t = tanh_x(q * q * q);
    return t < 0.0 ? 0.0 : t;
}
__device__ __forceinline__ double rho_of(const MixParams& M, double t, double s) {
    return M.lambda * s - t - M.xes * (ALPT1 * t + ALPT2 * t * t - ALPT3 * t * t * t);
}
struct MixFace { double ti, si, tz, sz; };   // Ftimp, Fsimp, Ftzt, Fszt at one top face
// fluxes through the top face kf of column (i,j) from the values below (0) and above (1)
__device__ __forceinline__ MixFace mix_face(const Geo& g, const MixParams& M, int kf, double t0, double t1,
                                            double s0, double s1, double iso0, double iso1) {
    MixFace f{0.0, 0.0, 0.0, 0.0};
    if (kf < 1) return f;                      // Ftimp(:,:,0), Ftzt(:,:,0) stay zero
    const double w = iso1 * iso0;
    const double den = g.dz * g.K(KT_DFZW, kf);
    const double dt = w * (t1 - t0) / den, ds = w * (s1 - s0) / den;
    const double dr = w * (rho_of(M, t1, s1) - rho_of(M, t0, s0)) / den;
    if (M.eps != 0.0) {
        const double tp = tprstb(dr, M.fac);
        f.tz = 0.0 + tp * M.eps * dt / (dr - 1.0e-20);
        f.sz = 0.0 + tp * M.eps * ds / (dr - 1.0e-20);
    }
    if (M.kvc != 0.0) {
        const double tp = tprstb(-dr, M.fac);
        f.ti = -(tp * M.kvc * dt);
        f.si = -(tp * M.kvc * ds);
    }
    return f;
}
// mix(row) of the T (q = 0) or S (q = 1) row of cell (i,j,k) from the column
// values at levels k-1, k, k+1 (the padded-field halo values at levels 0 and
// l+1) and isoc of those levels
__device__ __forceinline__ double mix_value(const Geo& g, const MixParams& M, int q, int k, const double* t,
                                            const double* s, const double* iso) {
    const MixFace lo = mix_face(g, M, k - 1, t[0], t[1], s[0], s[1], iso[0], iso[1]);
    const MixFace up = mix_face(g, M, k, t[1], t[2], s[1], s[2], iso[1], iso[2]);
    const double d = g.dz * g.K(KT_DFZT, k);
    double m = 0.0;
    if (q == 0) {
        m = (up.tz - lo.tz) / d + m;
        if (M.rhomix) m = ((up.ti - lo.ti) - (up.si - lo.si) * M.lambda) / (2.0 * g.dz * g.K(KT_DFZT, k)) + m;
        else m = (up.ti - lo.ti) / d + m;
    } else {
        m = (up.sz - lo.sz) / d + m;
        if (M.rhomix) m = ((up.si - lo.si) - (up.ti - lo.ti) / M.lambda) / (2.0 * g.dz * g.K(KT_DFZT, k)) + m;
        else m = (up.si - lo.si) / d + m;
    }
    return m;
}
__device__ __forceinline__ double isoc(const Geo& g, int i, int j, int k) {
    const int v = g.L(i, j, k);
    return (v == OCEAN || v == PERIO) ? 1.0 : 0.0;
}
// the column of cell c: T, S and isoc at levels k-1, k, k+1
__device__ __forceinline__ void mix_column(const Cell& c, double* t, double* s, double* iso) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        t[d] = c.at(3, 0, 0, d - 1);
        s[d] = c.at(4, 0, 0, d - 1);
        iso[d] = isoc(*c.g, c.i, c.j, c.k + d - 1);
    }
}
// mix(row) of row A (TT or SS) at the current state, with vmix_fun's row flags
template <int A>
__device__ __forceinline__ double mix_row(const Cell& c, const MixParams& M) {
    if (!M.on) return 0.0;
    const int* fl = M.flags;
    if (!((fl[0] == 1 || fl[1] == 1) && fl[4])) return 0.0;
    if ((A == TT && fl[0] != 1) || (A == SS && fl[1] != 1)) return 0.0;
    double t[3], s[3], iso[3];
    mix_column(c, t, s, iso);
    return mix_value(*c.g, M, A == TT ? 0 : 1, c.k, t, s, iso);
}
// vmix_jac (mix_imp.f:729-815) for row A: forward differences with step
// 1e-8 of mix(row) in the T and S unknowns of the cells below, at and above
// (the only ones it depends on), added to An at stencil positions 14, 5, 23.
// The reference perturbs a whole DSM colour group at once; no other column of
// a group touches this row, so each difference is this single-column one.
template <int A>
__device__ __forceinline__ void mix_jacobian(double* a, const Cell& c, const MixParams& M) {
    if (!M.on) return;
    const int* fl = M.flags;
    if (!((fl[0] == 1 || fl[1] == 1) && fl[4])) return;
    if (c.g->L(c.i, c.j, c.k) != OCEAN) return;
    if ((A == TT && !fl[2]) || (A == SS && !fl[3])) return;
    const bool rowon = (A == TT) ? fl[0] == 1 : fl[1] == 1;   // vmix_fun's flag for this row
    if (!rowon) return;                                       // mixd - mix = 0 for every column
    const Geo& g = *c.g;
    const int q = A == TT ? 0 : 1;
    double t[3], s[3], iso[3];
    mix_column(c, t, s, iso);
    const double f0 = mix_value(g, M, q, c.k, t, s, iso);
    const double eps = 1.0e-08;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int kn = c.k + d - 1;
        if (kn < 1 || kn > g.l || g.L(c.i, c.j, kn) != OCEAN) continue;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if ((b == 0 && !fl[2]) || (b == 1 && !fl[3])) continue;
            double tp[3], sp[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) { tp[e] = t[e]; sp[e] = s[e]; }
            // und = un + d: the unknown of level kn, and every halo copy of it
            const double pv = (b == 0 ? t[d] : s[d]) + eps;
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const int ke = c.k + e - 1;
                const int src = ke < 1 ? 1 : (ke > g.l ? g.l : ke);
                if (src == kn) { if (b == 0) tp[e] = pv; else sp[e] = pv; }
            }
            const double fj = (mix_value(g, M, q, c.k, tp, sp, iso) - f0) / eps;
            const int kk = d == 0 ? 14 : (d == 1 ? 5 : 23);
            if (b == 0) {
                constexpr int e0 = idx(A, 14, TT), e1 = idx(A, 5, TT), e2 = idx(A, 23, TT);
                const int e = kk == 14 ? e0 : (kk == 5 ? e1 : e2);
                a[e] = a[e] + fj;
            } else {
                constexpr int e0 = idx(A, 14, SS), e1 = idx(A, 5, SS), e2 = idx(A, 23, SS);
                const int e = kk == 14 ? e0 : (kk == 5 ? e1 : e2);
                a[e] = a[e] + fj;
            }
        }
    }
}

__global__ void mix_norm_part(Geo g, const double* __restrict__ x, double* __restrict__ part) {
    const int nc = g.n * g.m * g.l;
    double st = 0.0, ss = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const double t = x[size_t(NUN) * c + TT - 1], s = x[size_t(NUN) * c + SS - 1];
        st += t * t;
        ss += s * s;
    }
    __shared__ double red[2][256];
    red[0][threadIdx.x] = st;
    red[1][threadIdx.x] = ss;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            red[0][threadIdx.x] += red[0][threadIdx.x + h];
            red[1][threadIdx.x] += red[1][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = red[0][0];
        part[2 * blockIdx.x + 1] = red[1][0];
    }
}
// vmix_control (mix_imp.f:131-166): flags follow ||T||_2, ||S||_2 > 1e-12;
// on a change the partition is rebuilt, but only when the temperature flag is
// on (the reference tests vmix_temp twice, so a salinity-only change keeps
// the old partition)
__global__ void mix_control(const double* __restrict__ part, int nblocks, int* __restrict__ flags, int any_ocean) {
    if (threadIdx.x != 0) return;
    double st = 0.0, ss = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        st += part[2 * b];
        ss += part[2 * b + 1];
    }
    const int tt = sqrt(st) > 1.0e-12 ? 1 : 0, ts = sqrt(ss) > 1.0e-12 ? 1 : 0;
    if (flags[0] != tt || flags[1] != ts) {
        flags[0] = tt;
        flags[1] = ts;
        if (tt != 0) {
            flags[2] = tt;
            flags[3] = ts;
            flags[4] = any_ocean;
        }
    }
}

// ---------------------------------------------------------------------------
// boundaries (src/ocean/boundary.F90:2-393) applied to one row
// ---------------------------------------------------------------------------
struct Nb {
    int8_t c[28];   // c[kk] = landm at stencil position kk (1..27)
    int8_t southee, easteast, northee, nnorthee, nnorth;
    bool ilt, jlt;  // i < n, j < m
};
__device__ __forceinline__ Nb load_nb(const Geo& g, int i, int j, int k) {
    Nb nb;
    nb.c[0] = 0;
#pragma unroll
    for (int kk = 1; kk <= 27; ++kk) nb.c[kk] = int8_t(g.L(i + di_of(kk), j + dj_of(kk), k + dk_of(kk)));
    nb.ilt = i < g.n;
    nb.jlt = j < g.m;
    nb.southee = nb.easteast = nb.northee = nb.nnorthee = nb.nnorth = -1;
    if (nb.ilt) {
        nb.southee = int8_t(g.L(i + 2, j - 1, k));
        nb.easteast = int8_t(g.L(i + 2, j, k));
        nb.northee = int8_t(g.L(i + 2, j + 1, k));
        if (nb.jlt) nb.nnorthee = int8_t(g.L(i + 2, j + 2, k));
    }
    if (nb.jlt) nb.nnorth = int8_t(g.L(i, j + 2, k));
    return nb;
}

#define E_(kk, B) idx(A, kk, B)
#define ZC(kk, B) do { if constexpr (E_(kk, B) >= 0) a[E_(kk, B)] = 0.0; } while (0)
#define ZCUV(kk) do { ZC(kk, UU); ZC(kk, VV); } while (0)
#define ZP(kk) do { ZC(kk, UU); ZC(kk, VV); ZC(kk, WW); ZC(kk, PP); ZC(kk, TT); ZC(kk, SS); } while (0)
#define FOLD(dst, src, B) do { if constexpr (E_(src, B) >= 0) { static_assert(E_(dst, B) >= 0, "fold"); \
        a[E_(dst, B)] = a[E_(dst, B)] + a[E_(src, B)]; } } while (0)
#define DIR(X) do { if constexpr (A == X) { for (int e_ = 0; e_ < N; ++e_) a[e_] = 0.0; a[E_(5, X)] = 1.0; } \
        else { ZC(5, X); } } while (0)
#define SETC(kk, B, val) do { if constexpr (E_(kk, B) >= 0) a[E_(kk, B)] = (val); } while (0)

template <int A>
__device__ __forceinline__ void surgery(double* a, const Nb& nb) {
    constexpr int N = rowlen(A);
    const int8_t* L = nb.c;
    if (L[5] == OCEAN) {
        if (L[14] == LAND) {   // bottom
            if (L[11] == LAND && L[10] == LAND && L[13] == LAND) { FOLD(1, 10, UU); FOLD(1, 10, VV); }
            ZCUV(10);
            if (L[11] == LAND && L[18] == LAND && L[15] == LAND) { FOLD(2, 11, UU); FOLD(2, 11, VV); }
            ZCUV(11);
            if (L[17] == LAND && L[16] == LAND && L[13] == LAND) { FOLD(4, 13, UU); FOLD(4, 13, VV); }
            ZCUV(13);
            if (L[17] == LAND && L[18] == LAND && L[15] == LAND) { FOLD(5, 14, UU); FOLD(5, 14, VV); }
            FOLD(5, 14, TT); FOLD(5, 14, SS);
            ZP(14);
        }
        if (L[10] == LAND) ZP(10);
        if (L[11] == LAND) ZP(11);
        if (L[12] == LAND) ZP(12);
        if (L[13] == LAND) ZP(13);
        if (L[15] == LAND) ZP(15);
        if (L[16] == LAND) ZP(16);
        if (L[17] == LAND) ZP(17);
        if (L[18] == LAND) ZP(18);
        if (L[23] == LAND) {   // top
            if (L[20] == LAND && L[19] == LAND && L[22] == LAND) { FOLD(1, 19, UU); FOLD(1, 19, VV); }
            ZCUV(19);
            if (L[20] == LAND && L[21] == LAND && L[24] == LAND) { FOLD(2, 20, UU); FOLD(2, 20, VV); }
            ZCUV(20);
            if (L[26] == LAND && L[25] == LAND && L[22] == LAND) { FOLD(4, 22, UU); FOLD(4, 22, VV); }
            ZCUV(22);
            if (L[26] == LAND && L[27] == LAND && L[24] == LAND) { FOLD(5, 23, UU); FOLD(5, 23, VV); }
            FOLD(5, 23, TT); FOLD(5, 23, SS);
            ZP(23);
            if constexpr (A == WW) { for (int e = 0; e < N; ++e) a[e] = 0.0; }
            SETC(5, WW, 1.0e-10); SETC(6, WW, 1.0e-10); SETC(8, WW, 1.0e-10); SETC(9, WW, 1.0e-10);
            if constexpr (A == WW) a[E_(5, WW)] = 1.0;
        }
        if (L[19] == LAND) ZP(19);
        if (L[20] == LAND) ZP(20);
        if (L[21] == LAND) ZP(21);
        if (L[22] == LAND) ZP(22);
        if (L[24] == LAND) ZP(24);
        if (L[25] == LAND) ZP(25);
        if (L[26] == LAND) ZP(26);
        if (L[27] == LAND) ZP(27);
        if (L[1] == LAND) ZCUV(1);
        if (L[2] == LAND) {   // west
            FOLD(5, 2, TT); FOLD(5, 2, SS);
            ZP(2);
            ZCUV(1);
        }
        if (L[3] == LAND) {   // nwest
            ZCUV(2); ZCUV(3);
        } else if (nb.jlt) {
            if (nb.nnorth == LAND) ZCUV(3);
        }
        if (L[4] == LAND) {   // south
            FOLD(5, 4, SS); FOLD(5, 4, TT);
            ZP(4);
            ZCUV(1);
        }
        if (L[6] == LAND) {   // north
            ZCUV(2);
            if constexpr (A == PP) { ZC(2, UU); ZC(2, VV); ZC(5, UU); ZC(5, VV); }
            DIR(VV);
            DIR(UU);
            FOLD(5, 6, SS); FOLD(5, 6, TT);
            ZP(6);
        } else if (nb.jlt) {
            if (nb.nnorth == LAND) { ZCUV(3); ZCUV(6); }
        }
        if (L[7] == LAND) {   // southe
            ZCUV(4); ZCUV(7);
        } else if (nb.ilt) {
            if (nb.southee == LAND) ZCUV(7);
        }
        if (L[8] == LAND) {   // east
            ZCUV(4);
            if constexpr (A == PP) { ZC(4, UU); ZC(4, VV); ZC(5, UU); ZC(5, VV); }
            DIR(UU);
            DIR(VV);
            FOLD(5, 8, SS); FOLD(5, 8, TT);
            ZP(8);
            ZCUV(7);
        } else if (nb.ilt) {
            if (nb.easteast == LAND) { ZCUV(7); ZCUV(8); }
        }
        if (L[9] == LAND) {   // neast
            DIR(UU);
            DIR(VV);
            ZCUV(7);
        } else if (nb.ilt || nb.jlt) {
            if (nb.ilt) {
                if (nb.northee == LAND) { ZCUV(8); ZCUV(9); }
                else if (nb.jlt) { if (nb.nnorthee == LAND) ZCUV(9); }
            }
            if (nb.jlt) {
                if (nb.nnorth == LAND) { ZCUV(6); ZCUV(9); }
            }
        }
    } else {
        for (int e = 0; e < N; ++e) a[e] = 0.0;
        a[E_(5, A)] = 1.0;
    }
}
#undef E_
#undef ZC
#undef ZCUV
#undef ZP
#undef FOLD
#undef DIR
#undef SETC

// Fortran rhs forcing of one row after the boundaries() zeroing
// (src/ocean/forcing.F90:4-218; boundary.F90 Frc assignments).
template <int A>
__device__ __forceinline__ double forcing_row(const Geo& g, const Params& P, const ForcingScalars& fs,
                                              const double* surf, int i, int j, int k, const Nb& nb) {
    if (nb.c[5] != OCEAN) return 0.0;
    const size_t ij = size_t(i - 1) + size_t(g.n) * (j - 1);
    const size_t nm = size_t(g.n) * g.m;
    if constexpr (A == UU || A == VV) {
        if (nb.c[6] == LAND || nb.c[8] == LAND || nb.c[9] == LAND) return 0.0;
        if (k != g.l || j > g.m - 1) return 0.0;
        return fs.sigma * surf[(A == UU ? 0 : 1) * nm + ij];
    } else if constexpr (A == WW) {
        if (nb.c[23] == LAND || k > g.l - 1) return 0.0;
        double lmk = double(1 - g.L(i, j, k));
        return -(P.par[COMB] * lmk * P.par[RAYL] * (P.par[LAMB] * (0.0 + 0.0) / 2. - (0.0 + 0.0) / 2.));
    } else if constexpr (A == TT) {
        if (k != g.l) return 0.0;
        return fs.etabi * (surf[2 * nm + ij] - fs.temcor);
    } else if constexpr (A == SS) {
        if (k != g.l) return 0.0;
        return fs.gamma * (1 - fs.hmtp) * (surf[3 * nm + ij] - fs.salcor) +
               fs.gamma * fs.hmtp * (0.0 - fs.adapted_salcor) +
               fs.sper_fac * (surf[4 * nm + ij] - fs.spertcor);
    } else {
        return 0.0;
    }
}

__device__ __forceinline__ bool keep(double c) {
    // abs(c) > 1.0e-10 evaluated on the bit pattern (no FP64 pipe instruction)
    const unsigned long long mag = __double_as_longlong(c) & 0x7fffffffffffffffULL;
    return mag > 0x3ddb7cdfd9d7bdbbULL;   // bit pattern of 1.0e-10
}

// neighbour column of canonical entry (kk,B), or -1 outside the domain
__device__ __forceinline__ int col_of(const Geo& g, int i, int j, int k, int kk, int B) {
    int ii = i + di_of(kk), jj = j + dj_of(kk), k2 = k + dk_of(kk);
    if (g.periodic) { if (ii == 0) ii = g.n; else if (ii == g.n + 1) ii = 1; }
    if (ii < 1 || ii > g.n || jj < 1 || jj > g.m || k2 < 1 || k2 > g.l) return -1;
    return NUN * ((ii - 1) + g.n * ((jj - 1) + g.m * (k2 - 1))) + B - 1;
}

template <int A, bool JAC>
__device__ __forceinline__ void eval_row(double* a, const Cell& c, const Params& P, const double* al_row) {
    static_for<0, rowlen(A)>([&](auto E) {
        constexpr Ent en = entry(A, decltype(E)::value);
        double al = al_row[rowoff(A) + decltype(E)::value];
        if constexpr (JAC) a[decltype(E)::value] = an_jac<A, en.B>(al, en.kk, c, P);
        else a[decltype(E)::value] = an_rhs<A, en.B>(al, en.kk, c, P);
    });
}

template <int A>
__device__ void jac_row(const Geo& g, const Params& P, const MixParams& M, const Pattern& pat, const double* al_tab,
                        const Cell& c, const Nb& nb, int cell, int cls, double* val, float* val32) {
    double a[rowlen(A)];
    const size_t jk = size_t(c.j - 1) + size_t(g.m) * (c.k - 1);
    const double* al_row = al_tab + (jk * 2 + (c.lm == 0.0 ? 1 : 0)) * CELL_ENTRIES;
    eval_row<A, true>(a, c, P, al_row);
    if constexpr (A == TT || A == SS) mix_jacobian<A>(a, c, M);
    surgery<A>(a, nb);
    const int row = NUN * cell + A - 1;
    const int base = pat.row_ptr[row];
    const int8_t* sl = pat.slot + cls * CELL_ENTRIES + rowoff(A);
#pragma unroll
    for (int e = 0; e < rowlen(A); ++e) {
        int s = sl[e];
        if (s >= 0) {
            double v = keep(a[e]) ? a[e] : 0.0;
            val[base + s] = v;
            if (val32) val32[base + s] = float(v);
        }
    }
}

template <int A>
__device__ void rhs_row(const Geo& g, const Params& P, const MixParams& M, const ForcingScalars& fs,
                        const double* al_tab, const Cell& c, const Nb& nb, int cell, const double* x,
                        const double* surf, double* F) {
    double a[rowlen(A)];
    const size_t jk = size_t(c.j - 1) + size_t(g.m) * (c.k - 1);
    const double* al_row = al_tab + (jk * 2 + (c.lm == 0.0 ? 1 : 0)) * CELL_ENTRIES;
    eval_row<A, false>(a, c, P, al_row);
    surgery<A>(a, nb);
    // matAvec (src/ocean/matetc.F90:147-166): accumulate in fillcolA order
    double acc = 0.0;
    static_for<0, rowlen(A)>([&](auto R) {
        constexpr int r = decltype(R)::value;
        constexpr int e = [] {
            for (int q = 0; q < rowlen(A); ++q) if (fortran_rank(A, q) == r) return q;
            return -1;
        }();
        constexpr Ent en = entry(A, e);
        if (keep(a[e])) {
            int col = col_of(g, c.i, c.j, c.k, en.kk, en.B);
            if (col >= 0) acc = a[e] * x[col] + acc;
        }
    });
    double frc = forcing_row<A>(g, P, fs, surf, c.i, c.j, c.k, nb);
    double mix = 0.0;
    if constexpr (A == TT || A == SS) mix = mix_row<A>(c, M);
    double B = -acc - mix + frc - 0.0 * (1 - P.par[RESC]) * 0.0;
    B = B * double(1 - g.L(c.i, c.j, c.k));
    F[NUN * cell + A - 1] = -B;
}

__device__ __forceinline__ Cell make_cell(const Geo& g, const double* pads, int cell) {
    Cell c;
    c.i = cell % g.n + 1;
    int r = cell / g.n;
    c.j = r % g.m + 1;
    c.k = r / g.m + 1;
    c.lm = double(1 - g.L(c.i, c.j, g.l));
    const size_t np = g.npad();
    for (int q = 0; q < 5; ++q) c.f[q] = pads + q * np;
    c.g = &g;
    return c;
}

// block = 6 warps; warp w evaluates row type w+1 for 32 consecutive cells
__global__ void __launch_bounds__(192) jacobian_kernel(Geo g, Params P, MixParams M, Pattern pat,
                                                       const double* __restrict__ al_tab,
                                                       const double* __restrict__ pads, double* __restrict__ val,
                                                       float* __restrict__ val32) {
    const int nc = g.n * g.m * g.l;
    const int A = threadIdx.x / 32 + 1;
    for (int cb = blockIdx.x * 32; cb < nc; cb += gridDim.x * 32) {
        int cell = cb + (threadIdx.x & 31);
        if (cell >= nc) continue;
        Cell c = make_cell(g, pads, cell);
        Nb nb = load_nb(g, c.i, c.j, c.k);
        int cls = cell_class(c.i - 1, c.j - 1, c.k - 1, g.n, g.m, g.l);
        switch (A) {
        case UU: jac_row<UU>(g, P, M, pat, al_tab, c, nb, cell, cls, val, val32); break;
        case VV: jac_row<VV>(g, P, M, pat, al_tab, c, nb, cell, cls, val, val32); break;
        case WW: jac_row<WW>(g, P, M, pat, al_tab, c, nb, cell, cls, val, val32); break;
        case PP: jac_row<PP>(g, P, M, pat, al_tab, c, nb, cell, cls, val, val32); break;
        case TT: jac_row<TT>(g, P, M, pat, al_tab, c, nb, cell, cls, val, val32); break;
        default: jac_row<SS>(g, P, M, pat, al_tab, c, nb, cell, cls, val, val32); break;
        }
    }
}

__global__ void __launch_bounds__(192) rhs_kernel(Geo g, Params P, MixParams M, ForcingScalars fs,
                                                  const double* __restrict__ al_tab,
                                                  const double* __restrict__ pads, const double* __restrict__ x,
                                                  const double* __restrict__ surf, double* __restrict__ F) {
    const int nc = g.n * g.m * g.l;
    const int A = threadIdx.x / 32 + 1;
    for (int cb = blockIdx.x * 32; cb < nc; cb += gridDim.x * 32) {
        int cell = cb + (threadIdx.x & 31);
        if (cell >= nc) continue;
        Cell c = make_cell(g, pads, cell);
        Nb nb = load_nb(g, c.i, c.j, c.k);
        switch (A) {
        case UU: rhs_row<UU>(g, P, M, fs, al_tab, c, nb, cell, x, surf, F); break;
        case VV: rhs_row<VV>(g, P, M, fs, al_tab, c, nb, cell, x, surf, F); break;
        case WW: rhs_row<WW>(g, P, M, fs, al_tab, c, nb, cell, x, surf, F); break;
        case PP: rhs_row<PP>(g, P, M, fs, al_tab, c, nb, cell, x, surf, F); break;
        case TT: rhs_row<TT>(g, P, M, fs, al_tab, c, nb, cell, x, surf, F); break;
        default: rhs_row<SS>(g, P, M, fs, al_tab, c, nb, cell, x, surf, F); break;
        }
    }
}

// column indices of the maximal graph (src/ocean/THCM.C:2300-2580)
__global__ void pattern_kernel(Geo g, Pattern pat, int* __restrict__ col_idx) {
    const int nc = g.n * g.m * g.l;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nc * CELL_ENTRIES; t += gridDim.x * blockDim.x) {
        int cell = t / CELL_ENTRIES, e = t % CELL_ENTRIES;
        int A = row_of_cell_entry(e);
        int i = cell % g.n + 1, r = cell / g.n, j = r % g.m + 1, k = r / g.m + 1;
        int cls = cell_class(i - 1, j - 1, k - 1, g.n, g.m, g.l);
        int s = pat.slot[cls * CELL_ENTRIES + e];
        if (s < 0) continue;
        Ent en = entry(A, e - rowoff(A));
        col_idx[pat.row_ptr[NUN * cell + A - 1] + s] = col_of(g, i, j, k, en.kk, en.B);
    }
}

// fillcolB (src/ocean/assemble.F90:18-54)
__global__ void mass_kernel(Geo g, double rosb, double* __restrict__ B) {
    const int nc = g.n * g.m * g.l;
    for (int cell = blockIdx.x * blockDim.x + threadIdx.x; cell < nc; cell += gridDim.x * blockDim.x) {
        int i = cell % g.n + 1, r = cell / g.n, j = r % g.m + 1, k = r / g.m + 1;
        double* b = B + NUN * size_t(cell);
        for (int q = 0; q < NUN; ++q) b[q] = 0.0;
        if (g.L(i, j, k) == OCEAN) {
            if (g.L(i + 1, j, k) != LAND) b[0] = -rosb;
            if (g.L(i, j + 1, k) != LAND) b[1] = -rosb;
            b[4] = -1.0;
            b[5] = -1.0;
        }
    }
}

int grid_for(size_t work, int block) {
    size_t b = (work + block - 1) / block;
    return int(b < 152 * 16 ? (b == 0 ? 1 : b) : 152 * 16);
}

}  // namespace

void launch_lin(const Geo& g, const Params& p, double* al_tab, cudaStream_t s) {
    size_t work = size_t(g.m) * g.l * 2 * CELL_ENTRIES;
    lin_kernel<<<grid_for(work, 256), 256, 0, s>>>(g, p, al_tab); IEMIC_COUNT_LAUNCH();
}
void launch_usol(const Geo& g, const double* x, double* pads, cudaStream_t s) {
    usol_kernel<<<grid_for(g.npad(), 256), 256, 0, s>>>(g, x, pads); IEMIC_COUNT_LAUNCH();
}
void launch_pattern(const Geo& g, const Pattern& pat, int* col_idx, cudaStream_t s) {
    size_t work = size_t(g.n) * g.m * g.l * CELL_ENTRIES;
    pattern_kernel<<<grid_for(work, 256), 256, 0, s>>>(g, pat, col_idx); IEMIC_COUNT_LAUNCH();
}
void launch_jacobian(const Geo& g, const Params& p, const MixParams& mp, const Pattern& pat, const double* al_tab,
                     const double* pads, double* val, float* val32, cudaStream_t s) {
    size_t nc = size_t(g.n) * g.m * g.l;
    size_t blocks = (nc + 31) / 32;
    jacobian_kernel<<<int(blocks), 192, 0, s>>>(g, p, mp, pat, al_tab, pads, val, val32); IEMIC_COUNT_LAUNCH();
}
void launch_rhs(const Geo& g, const Params& p, const MixParams& mp, const ForcingScalars& fs, const double* al_tab,
                const double* pads, const double* x, const double* surf, double* F, cudaStream_t s) {
    size_t nc = size_t(g.n) * g.m * g.l;
    size_t blocks = (nc + 31) / 32;
    rhs_kernel<<<int(blocks), 192, 0, s>>>(g, p, mp, fs, al_tab, pads, x, surf, F); IEMIC_COUNT_LAUNCH();
}
// Rows the Fortran assembly does not produce (THCM::evaluate, src/ocean/THCM.C:
// 1014-1041): the integral condition F_r = sign * sum_cells coef_c S_c
// (one block; tree reduction in shared memory, no global scratch) and the
// fixed pressure points F = 0.
__global__ void __launch_bounds__(1024) k_special_rhs(int nc, const double* __restrict__ coef,
                                                      const double* __restrict__ x, double* __restrict__ F, int row,
                                                      int sign, int pfix1, int pfix2) {
    __shared__ double red[1024];
    double sum = 0.0;
    if (row >= 0)
        for (int c = threadIdx.x; c < nc; c += blockDim.x) sum += coef[c] * x[size_t(NUN) * c + SS - 1];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (row >= 0) F[row] = sign * (red[0] - 0.0);
        if (pfix1 >= 0) F[pfix1] = 0.0;
        if (pfix2 >= 0) F[pfix2] = 0.0;
    }
}
// Jacobian rows the assembly does not produce: the dense integral-condition
// row (its columns are the S unknowns of every cell, in order) and the
// identity rows of the fixed pressure points.
__global__ void k_special_jac(int nc, const int* __restrict__ rp, const int* __restrict__ ci,
                              const double* __restrict__ coef, double* __restrict__ val, float* __restrict__ val32,
                              int row, int sign, int pfix1, int pfix2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= 0)
        for (int c = t; c < nc; c += gridDim.x * blockDim.x) {
            const double v = sign * coef[c];
            val[rp[row] + c] = v;
            if (val32) val32[rp[row] + c] = float(v);
        }
    const int pf[2] = {pfix1, pfix2};
    if (t == 0)
        for (int k = 0; k < 2; ++k) {
            const int r = pf[k];
            if (r < 0) continue;
            for (int q = rp[r]; q < rp[r + 1]; ++q) {
                const double v = ci[q] == r ? 1.0 : 0.0;
                val[q] = v;
                if (val32) val32[q] = float(v);
            }
        }
}
__global__ void k_dense_row_cols(int nc, int* __restrict__ cols) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
        cols[c] = NUN * c + SS - 1;
}
void launch_mix_control(const Geo& g, const double* x, double* part, int* flags, int any_ocean, cudaStream_t s) {
    mix_norm_part<<<152, 256, 0, s>>>(g, x, part); IEMIC_COUNT_LAUNCH();
    mix_control<<<1, 32, 0, s>>>(part, 152, flags, any_ocean); IEMIC_COUNT_LAUNCH();
}
void launch_special_rhs(int nc, const double* coef, const double* x, double* F, int row, int sign, int pfix1, int pfix2,
                        cudaStream_t s) {
    if (row < 0 && pfix1 < 0 && pfix2 < 0) return;
    k_special_rhs<<<1, 1024, 0, s>>>(nc, coef, x, F, row, sign, pfix1, pfix2); IEMIC_COUNT_LAUNCH();
}
void launch_special_jac(int nc, const int* rp, const int* ci, const double* coef, double* val, float* val32, int row,
                        int sign, int pfix1, int pfix2, cudaStream_t s) {
    if (row < 0 && pfix1 < 0 && pfix2 < 0) return;
    k_special_jac<<<grid_for(size_t(nc), 256), 256, 0, s>>>(nc, rp, ci, coef, val, val32, row, sign, pfix1, pfix2); IEMIC_COUNT_LAUNCH();
}
void launch_dense_row_cols(int nc, int* cols, cudaStream_t s) {
    k_dense_row_cols<<<grid_for(size_t(nc), 256), 256, 0, s>>>(nc, cols); IEMIC_COUNT_LAUNCH();
}

void launch_mass(const Geo& g, const Params& p, double* diagB, cudaStream_t s) {
    size_t nc = size_t(g.n) * g.m * g.l;
    mass_kernel<<<grid_for(nc, 256), 256, 0, s>>>(g, p.par[ROSB], diagB); IEMIC_COUNT_LAUNCH();
}


// ---------------------------------------------------------------------------
// Adjoint of the surface forcing: grad[f][i,j] = -lambda^T dF/d(field f)(i,j)
// for f = taux, tauy, tatm, emip, spert. F is affine in these fields and
// every field value enters one row only, the row forcing_row fills (with the
// same land and boundary conditions): F_row = -(frc_row - acc) (1 - landm).
// ---------------------------------------------------------------------------
__global__ void dfdsurf_t_kernel(Geo g, ForcingScalars fs, const double* __restrict__ lambda,
                                 double* __restrict__ grad) {
    const int nm = g.n * g.m;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 5 * nm; q += gridDim.x * blockDim.x) {
        const int f = q / nm, ij = q % nm;
        const int i = ij % g.n + 1, j = ij / g.n + 1, k = g.l;
        const Nb nb = load_nb(g, i, j, k);
        double coef = 0.0;
        int A = 0;
        if (nb.c[5] == OCEAN) {
            if (f <= 1) {
                if (!(nb.c[6] == LAND || nb.c[8] == LAND || nb.c[9] == LAND) && j <= g.m - 1) {
                    coef = fs.sigma;
                    A = f == 0 ? UU : VV;
                }
            } else if (f == 2) {
                coef = fs.etabi;
                A = TT;
            } else {
                coef = f == 3 ? fs.gamma * (1 - fs.hmtp) : fs.sper_fac;
                A = SS;
            }
        }
        double v = 0.0;
        if (A) {
            const size_t row = size_t(NUN) * (size_t(i - 1) + size_t(g.n) * (size_t(j - 1) + size_t(g.m) * (k - 1))) + A - 1;
            // dF_row / dfield = -coef (1 - landm); dg/dfield = -lambda_row dF_row/dfield
            v = lambda[row] * coef * double(1 - g.L(i, j, k));
        }
        grad[q] = v;
    }
}
void launch_dfdsurf_t(const Geo& g, const ForcingScalars& fs, const double* lambda, double* grad, cudaStream_t s) {
    dfdsurf_t_kernel<<<grid_for(size_t(5) * g.n * g.m, 256), 256, 0, s>>>(g, fs, lambda, grad); IEMIC_COUNT_LAUNCH();
}

}  // namespace iemic
