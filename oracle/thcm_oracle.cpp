// CPU oracle for the THCM Newton-step path (TEST INFRASTRUCTURE ONLY).
//
// FP64 restatement of the reference's Fortran physics. Each routine cites the
// reference routine it follows. Whole-array Fortran expressions are evaluated
// element by element in the same left-to-right order, and this file must be
// compiled with -ffp-contract=off so no fused multiply-adds change rounding
// (the reference's gfortran -O3 build on x86-64 emits none either).
// Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
#include "thcm_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

// ---- constants: src/ocean/par.F90:11-83, usr.F90:130-171, atm.F90 ----------
constexpr double PI = 3.14159265358979323846;
constexpr int NUN = 6, NP = 27, NPAR = 30;
enum { UU = 1, VV = 2, WW = 3, PP = 4, TT = 5, SS = 6 };
enum { OCEAN = 0, LAND = 1, WATER = 2, PERIO = 3 };
enum {
    AL_T = 1, RAYL, EK_V, EK_H, ROSB, MIXP, RESC, SPL1, HMTP, SUNP, PE_H, PE_V, P_VC,
    LAMB, SALT, WIND, TEMP, BIOT, COMB, ARCL, NLES, IFRICB, CONT, ENER, ALPC, CMPR,
    FPER, SPER, MKAP, SPL2
};
constexpr double omegadim = 7.292e-05, r0dim = 6.37e+06, udim = 0.1e+00,
                 gdim = 9.8e+00, rhodim = 1.024e+03, deltas = 1.0, s0 = 35.0,
                 cp0 = 4.2e+03, alpt1 = 2.93, alpt2 = 8.3e-02, alpt3 = 6.6e-04,
                 ah = 2.5e+05, av = 1.0e-03, kappah = 1.0e+03, kappav = 1.0e-04;
constexpr double zmin = -1.0, zmax = 0.0;

// Fortran-style array with arbitrary lower bounds, column-major.
struct Arr3 {
    int i0, i1, j0, j1, k0, k1, ni, nj;
    std::vector<double> d;
    Arr3() = default;
    Arr3(int a0, int a1, int b0, int b1, int c0, int c1)
        : i0(a0), i1(a1), j0(b0), j1(b1), k0(c0), k1(c1), ni(a1 - a0 + 1), nj(b1 - b0 + 1),
          d(size_t(ni) * nj * (c1 - c0 + 1), 0.0) {}
    double& operator()(int i, int j, int k) {
        return d[size_t(i - i0) + size_t(ni) * (size_t(j - j0) + size_t(nj) * size_t(k - k0))];
    }
    void zero() { std::fill(d.begin(), d.end(), 0.0); }
};

struct Model {
    // configuration
    int n, m, l, ndim;
    bool periodic;
    double xmin, xmax, ymin, ymax, hdim, qz, alphaT, alphaS;
    int ih, coriolis_on, TRES, SRES, iza, ite, its, forcing_type;
    int vmix = 0, rho_mixing = 0, tap = 1;   // "Mixing", "Rho Mixing", "Taper"
    // SRES = 0: integral condition on S (THCM::intcond_S, src/ocean/THCM.C:2180-2257)
    int sint_sign = -1, rowintcon = -1;      // 0-based row of the condition
    double intCorrection = 0.0;              // THCM::setIntCondCorrection
    std::vector<double> intcoef;             // cos(y_j) dfzT(k) at S of ocean cells (intcond_scaling)
    // "Fix Pressure Points" (THCM::fixPressurePoints, THCM.C:2260-2297)
    int rowPfix1 = -1, rowPfix2 = -1;
    const int coupled_T = 0, coupled_S = 0;
    // grid (src/ocean/grid.F90)
    double dx, dy, dz;
    std::vector<double> x, y, xu, yv, z, zw, ze, zwe, dfzT, dfzW;  // offset storage below
    std::vector<int> landm;
    double par[NPAR + 1];
    double QTnd, QSnd;
    std::vector<double> Frc, taux, tauy, tatm, emip, spert, adapted_emip, internal_temp,
        internal_salt;
    std::vector<double> Al, An;
    std::vector<int> begA, jcoA;
    std::vector<double> coA, coB;
    // maximal graph
    std::vector<int> g_ptr, g_col;

    // ---- index helpers ----
    double& Y(int j) { return y[j]; }            // y(0:m+1)
    double& YV(int j) { return yv[j]; }          // yv(0:m)
    double& XU(int i) { return xu[i]; }          // xu(0:n)
    double& DFZT(int k) { return dfzT[k - 1]; }  // dfzT(1:l)
    double& DFZW(int k) { return dfzW[k]; }      // dfzW(0:l)
    double& ZW(int k) { return zw[k]; }          // zw(0:l)
    double& Z(int k) { return z[k - 1]; }
    int& LM(int i, int j, int k) { return landm[i + (n + 2) * (j + (m + 2) * k)]; }
    int find_row2(int i, int j, int k, int XX) const {
        return NUN * ((k - 1) * n * m + n * (j - 1) + i - 1) + XX;
    }
    size_t cell(int i, int j, int k) const {
        return size_t(i - 1) + size_t(n) * (size_t(j - 1) + size_t(m) * size_t(k - 1));
    }
    size_t aidx(int kk, int A, int B, int i, int j, int k) const {
        return size_t(kk - 1) + NP * (size_t(A - 1) + NUN * (size_t(B - 1) + NUN * cell(i, j, k)));
    }
    double& AN(int kk, int A, int B, int i, int j, int k) { return An[aidx(kk, A, B, i, j, k)]; }
    double& AL(int kk, int A, int B, int i, int j, int k) { return Al[aidx(kk, A, B, i, j, k)]; }
    double& F2(std::vector<double>& f, int i, int j) { return f[size_t(i - 1) + size_t(n) * (j - 1)]; }
    double& F3(std::vector<double>& f, int i, int j, int k) {
        return f[size_t(i - 1) + size_t(n) * (size_t(j - 1) + size_t(m) * (k - 1))];
    }

    // atom(np,n,m,l)
    struct Atom {
        int n, m, l;
        std::vector<double> d;
        Atom(int n_, int m_, int l_) : n(n_), m(m_), l(l_), d(size_t(NP) * n_ * m_ * l_, 0.0) {}
        double& operator()(int kk, int i, int j, int k) {
            return d[size_t(kk - 1) + NP * (size_t(i - 1) + size_t(n) * (size_t(j - 1) + size_t(m) * (k - 1)))];
        }
        void zero() { std::fill(d.begin(), d.end(), 0.0); }
    };
    Atom mk() { return Atom(n, m, l); }

    // ---- src/ocean/spf.F90:792-854 ----
    double amh(double yy) const { return ih == 0 ? 1.0 : 1. + 10.0 * std::exp(-5 * yy * yy); }
    double bmh(double yy) const { return ih == 0 ? 1.0 : 1.0 + 10.0 * std::exp(-5 * yy * yy); }
    double bmhy(double yy) const { return ih == 0 ? 0.0 : -10. * 10.0 * yy * std::exp(-5 * yy * yy); }

    // ---- grid: src/ocean/grid.F90:2-95 ----
    static double fz(double zz, double q) {
        double th = std::tanh(q * (zz + 1));
        double tth = std::tanh(q);
        if (q > 1.0) return -1 + th / tth;
        return zz + (1. - q) * zz * (1 - zz);
    }
    static double dfdz(double zz, double q) {
        double ch = std::cosh(q * (zz + 1));
        double tth = std::tanh(q);
        if (q > 1.0) return q / (tth * ch * ch);
        return 1.0 + (1. - q) * (1. - 2. * zz);
    }
    void grid() {
        dx = (xmax - xmin) / n;
        dy = (ymax - ymin) / m;
        dz = (zmax - zmin) / l;
        x.assign(n, 0);
        xu.assign(n + 1, 0);
        y.assign(m + 2, 0);
        yv.assign(m + 1, 0);
        z.assign(l, 0);
        zw.assign(l + 1, 0);
        ze.assign(l, 0);
        zwe.assign(l, 0);
        dfzT.assign(l, 0);
        dfzW.assign(l + 1, 0);
        for (int i = 1; i <= n; ++i) {
            x[i - 1] = (double(i) - 0.5) * dx + xmin;
            xu[i] = (double(i)) * dx + xmin;
        }
        xu[0] = xmin;
        for (int j = 1; j <= m; ++j) {
            y[j] = (double(j) - 0.5) * dy + ymin;
            yv[j] = (double(j)) * dy + ymin;
        }
        y[0] = y[1] - dy;
        y[m + 1] = y[m] + dy;
        yv[0] = ymin;
        for (int k = 1; k <= l; ++k) {
            ze[k - 1] = (double(k) - 0.5) * dz + zmin;
            zwe[k - 1] = (double(k)) * dz + zmin;
            z[k - 1] = fz(ze[k - 1], qz);
            zw[k] = fz(zwe[k - 1], qz);
            dfzT[k - 1] = dfdz(ze[k - 1], qz);
            dfzW[k] = dfdz(zwe[k - 1], qz);
        }
        zw[0] = zmin;
        dfzW[0] = dfdz(zmin, qz);
    }

    // ---- stpnt: src/ocean/usrc.F90:1153-1197 (+ vmix_par with vmix=0) ----
    void stpnt() {
        for (int i = 0; i <= NPAR; ++i) par[i] = 0.0;
        par[AL_T] = 0.1 / (2 * omegadim * rhodim * hdim * udim * dz * DFZT(l));
        par[RAYL] = alphaT * gdim * hdim / (2 * omegadim * udim * r0dim);
        par[EK_V] = av / (2 * omegadim * hdim * hdim);
        par[EK_H] = ah / (2 * omegadim * r0dim * r0dim);
        par[ROSB] = udim / (2 * omegadim * r0dim);
        par[HMTP] = 0.0;
        par[SUNP] = 0.0;
        par[PE_H] = kappah / (udim * r0dim);
        par[PE_V] = kappav * r0dim / (udim * hdim * hdim);
        par[P_VC] = 2.5e+04 * par[PE_V];
        par[LAMB] = alphaS / alphaT;
        par[SALT] = 0.0;
        par[WIND] = 0.0;
        par[TEMP] = 0.0;
        par[BIOT] = r0dim / (75. * 3600. * 24. * udim);
        par[COMB] = 0.0;
        par[NLES] = 0.0;
        par[CMPR] = 0.0;
        par[ALPC] = 1.0;
        par[ENER] = 1.0e+02;
        par[MIXP] = 0.0;
        par[MKAP] = 0.0;
        par[SPL1] = 2.0e+03;
        par[SPL2] = 0.01;
        // vmix_par (src/ocean/mix_imp.f:113-128): only Mixing = 0 clears them
        if (vmix == 0) {
            par[MIXP] = 0.0;
            par[P_VC] = 0.0;
            par[ALPC] = 1.0;
            par[ENER] = 1.0e+2;
            par[MKAP] = 0.0;
        }
    }

    // ---- forcing profiles: src/ocean/forcing.F90:405-449 ----
    double wfun(double yy, int v1) const {
        if (v1 == 1)
            return 0.2 - 0.8 * std::sin(6 * std::fabs(yy)) - 0.5 * (1 - std::tanh(10 * std::fabs(yy))) -
                   0.5 * (1 - std::tanh(10 * (PI / 2 - std::fabs(yy))));
        return 0.0;
    }
    double temfun(double yy) {
        if (forcing_type == 2) return std::cos(PI * (yy - ymin) / (ymax - ymin));
        return std::cos(PI * yy / ymax) + par[CMPR] * std::sin(PI * yy / ymax);
    }
    double salfun(double yy) {
        if (forcing_type == 2) return std::cos(PI * (yy - ymin) / (ymax - ymin));
        if (forcing_type == 1) return (std::cos(PI * yy / ymax) + par[FPER] * yy / ymax) / std::cos(yy);
        return std::cos(PI * yy / ymax) + par[FPER] * yy / ymax;
    }

    // ---- qint (src/ocean/forcing.F90:452-464) through thcm_forcing_integral
    // (src/ocean/THCM.C:2653-2686): area mean of a surface field over ocean ----
    double qint(std::vector<double>& f) {
        double lfsint = 0.0, lsint = 0.0;
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n; ++i) {
                const int lmv = LM(i + 1, j + 1, l);
                lfsint = f[size_t(i) + size_t(n) * j] * std::cos(Y(j + 1)) * double(1 - lmv) + lfsint;
                lsint = std::cos(Y(j + 1)) * double(1 - lmv) + lsint;
            }
        return lfsint / lsint;
    }

    // ---- forcing: src/ocean/forcing.F90:4-218 (uncoupled, restoring branches) ----
    void forcing() {
        std::fill(Frc.begin(), Frc.end(), 0.0);
        double sigma = par[COMB] * par[WIND] * par[AL_T];
        if (iza == 2) {
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= n; ++i) {
                    F2(taux, i, j) = wfun(YV(j), 1);
                    F2(tauy, i, j) = wfun(YV(j), 2);
                }
        }
        for (int j = 1; j <= m - 1; ++j)
            for (int i = 1; i <= n; ++i) {
                Frc[find_row2(i, j, l, UU) - 1] = sigma * F2(taux, i, j);
                Frc[find_row2(i, j, l, VV) - 1] = sigma * F2(tauy, i, j);
            }
        double etabi = par[COMB] * par[TEMP] * (double(1 - TRES) + TRES * par[BIOT]);
        double temcor = 0.0;
        if (ite == 1 && coupled_T == 0) {
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= n; ++i) F2(tatm, i, j) = temfun(Y(j));
            if (TRES == 0) temcor = qint(tatm);
        }
        for (int j = 1; j <= m; ++j)
            for (int i = 1; i <= n; ++i)
                Frc[find_row2(i, j, l, TT) - 1] = etabi * (F2(tatm, i, j) - temcor);

        double gamma = par[COMB] * par[SALT] * (double(1 - SRES) + SRES * par[BIOT]);
        double salcor = 0.0;
        if (its == 1) {
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= n; ++i) F2(emip, i, j) = salfun(Y(j)) * double(1 - LM(i, j, l));
            if (SRES == 0) salcor = qint(emip);
        }
        double adapted_salcor = 0.0, spertcor = 0.0;
        if (SRES == 0) {   // correct for a nonzero net flux
            adapted_salcor = qint(adapted_emip);
            spertcor = qint(spert);
        }
        for (int j = 1; j <= m; ++j)
            for (int i = 1; i <= n; ++i)
                Frc[find_row2(i, j, l, SS) - 1] =
                    gamma * (1 - par[HMTP]) * (F2(emip, i, j) - salcor) +
                    gamma * par[HMTP] * (F2(adapted_emip, i, j) - adapted_salcor) +
                    par[SPER] * (double(1 - SRES) + SRES * par[BIOT]) * (F2(spert, i, j) - spertcor);
        for (int k = 1; k <= l - 1; ++k)
            for (int j = 1; j <= m; ++j)
                for (int i = 1; i <= n; ++i)
                    Frc[find_row2(i, j, k, WW) - 1] =
                        -(par[COMB] * double(1 - LM(i, j, k)) * par[RAYL] *
                          (par[LAMB] * (F3(internal_salt, i, j, k) + F3(internal_salt, i, j, k + 1)) / 2. -
                           (F3(internal_temp, i, j, k) + F3(internal_temp, i, j, k + 1)) / 2.));
    }

    // ---- spf.F90 derivative atoms ----
    void uderiv(int type, Atom& a) {
        a.zero();
        switch (type) {
        case 1:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) a(5, i, j, k) = 1.0;
            break;
        case 2: {
            std::vector<double> c(m + 1);
            for (int j = 0; j <= m; ++j) { double t = 1.0 / (std::cos(YV(j)) * dx); c[j] = t * t; }
            for (int j = 1; j <= m - 1; ++j) for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) {
                a(2, i, j, k) = amh(YV(j)) * c[j];
                a(8, i, j, k) = amh(YV(j)) * c[j];
                a(5, i, j, k) = -(a(2, i, j, k) + a(8, i, j, k));
            }
        } break;
        case 3: {
            double t = 1.0 / dy, r = t * t;
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m - 1; ++j) for (int k = 1; k <= l; ++k) {
                a(4, i, j, k) = r * bmh(Y(j)) * std::cos(Y(j)) / std::cos(YV(j));
                a(6, i, j, k) = r * bmh(Y(j + 1)) * std::cos(Y(j + 1)) / std::cos(YV(j));
                a(5, i, j, k) = -(a(4, i, j, k) + a(6, i, j, k));
            }
        } break;
        case 4: {
            double t = 1.0 / dz, r = t * t;
            for (int k = 1; k <= l; ++k) {
                double h1 = 1. / (DFZT(k) * DFZW(k));
                double h2 = 1. / (DFZT(k) * DFZW(k - 1));
                for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                    a(14, i, j, k) = h2 * r;
                    a(23, i, j, k) = h1 * r;
                    a(5, i, j, k) = -(a(14, i, j, k) + a(23, i, j, k));
                }
            }
        } break;
        case 5:
            for (int j = 1; j <= m - 1; ++j) {
                double tv = std::tan(YV(j));
                double tand2 = 1 - tv * tv;
                double val = bmh(YV(j)) * tand2 + std::tan(YV(j)) * bmhy(YV(j));
                for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) a(5, i, j, k) = val;
            }
            break;
        case 6:
            for (int j = 1; j <= m - 1; ++j) {
                double tand2 = std::tan(YV(j)), cosd2 = std::cos(YV(j));
                double num = bmhy(YV(j)) - (amh(YV(j)) + bmh(YV(j))) * tand2;
                double v2 = num / (dx * cosd2);
                double v8 = -(num / (dx * cosd2));
                for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) { a(2, i, j, k) = v2; a(8, i, j, k) = v8; }
            }
            break;
        }
    }
    void vderiv(int type, Atom& a) {
        a.zero();
        switch (type) {
        case 1:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) a(5, i, j, k) = 1.0;
            break;
        case 2: {
            std::vector<double> c(m + 1);
            for (int j = 0; j <= m; ++j) { double t = 1.0 / (std::cos(YV(j)) * dx); c[j] = t * t; }
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m - 1; ++j) for (int k = 1; k <= l; ++k) {
                a(2, i, j, k) = bmh(YV(j)) * c[j];
                a(5, i, j, k) = -(2 * bmh(YV(j)) * c[j]);
                a(8, i, j, k) = bmh(YV(j)) * c[j];
            }
        } break;
        case 3: {
            double t = 1.0 / dy, r = t * t;
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m - 1; ++j) for (int k = 1; k <= l; ++k) {
                a(4, i, j, k) = r * amh(Y(j)) * std::cos(Y(j)) / std::cos(YV(j));
                a(6, i, j, k) = r * amh(Y(j + 1)) * std::cos(Y(j + 1)) / std::cos(YV(j));
                a(5, i, j, k) = -(a(4, i, j, k) + a(6, i, j, k));
            }
        } break;
        case 4:
            uderiv(4, a);
            break;
        case 5:
            for (int j = 1; j <= m - 1; ++j) {
                double tv = std::tan(YV(j));
                double val = bmh(YV(j)) - amh(YV(j)) * tv * tv + bmhy(YV(j)) * tv;
                for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) a(5, i, j, k) = val;
            }
            break;
        case 6:
            for (int j = 1; j <= m - 1; ++j) {
                double tand2 = std::tan(YV(j)), cosd2 = std::cos(YV(j));
                double num = (amh(YV(j)) + bmh(YV(j))) * tand2 - bmhy(YV(j));
                double v2 = -(num / (dx * cosd2));
                double v8 = num / (dx * cosd2);
                for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) { a(2, i, j, k) = v2; a(8, i, j, k) = v8; }
            }
            break;
        }
    }
    void pderiv(int type, Atom& a) {
        a.zero();
        switch (type) {
        case 1:
            for (int j = 1; j <= m; ++j) {
                double c = 1.0 / (2 * std::cos(Y(j)) * dx);
                for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) {
                    a(2, i, j, k) = -c; a(4, i, j, k) = c; a(1, i, j, k) = -c; a(5, i, j, k) = c;
                }
            }
            break;
        case 2:
            for (int j = 1; j <= m; ++j) {
                double c = 1. / (2 * std::cos(Y(j)) * dy);
                double cm = std::cos(YV(j - 1)), cc = std::cos(YV(j));
                for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) {
                    a(4, i, j, k) = -(cm * c);
                    a(2, i, j, k) = cc * c;
                    a(1, i, j, k) = -(cm * c);
                    a(5, i, j, k) = cc * c;
                }
            }
            break;
        case 3: {
            double dzi = 1.0 / dz;
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                a(5, i, j, k) = dzi / DFZT(k);
                a(14, i, j, k) = -(dzi / DFZT(k));
            }
        } break;
        }
    }
    void tderiv(int type, Atom& a) {
        a.zero();
        switch (type) {
        case 1:
        case 2:
            for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) a(5, i, j, l) = 1.0;
            break;
        case 3:
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m; ++j) {
                double t = 1.0 / (std::cos(Y(j)) * dx), c = t * t;
                double lm = double(1 - LM(i, j, l));
                for (int k = 1; k <= l; ++k) {
                    a(2, i, j, k) = c * lm;
                    a(5, i, j, k) = -(2 * c * lm);
                    a(8, i, j, k) = c * lm;
                }
            }
            break;
        case 4: {
            double t = 1.0 / dy, d = t * t;
            for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) {
                double lm = double(1 - LM(i, j, l));
                a(4, i, j, k) = (d * std::cos(YV(j - 1)) / std::cos(Y(j))) * lm;
                a(6, i, j, k) = (d * std::cos(YV(j)) / std::cos(Y(j))) * lm;
                a(5, i, j, k) = -(a(4, i, j, k) + a(6, i, j, k));
            }
        } break;
        case 5: {
            double t = 1.0 / dz, d = t * t;
            for (int k = 1; k <= l - 1; ++k) {
                double h1 = 1. / (DFZT(k) * DFZW(k));
                double h2 = 1. / (DFZT(k) * DFZW(k - 1));
                for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                    double lm = double(1 - LM(i, j, l));
                    a(14, i, j, k) = h2 * d * lm;
                    a(23, i, j, k) = h1 * d * lm;
                    a(5, i, j, k) = -(a(14, i, j, k) + a(23, i, j, k));
                }
            }
            int k = l;
            double h2 = 1. / (DFZT(k) * DFZW(k - 1));
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m; ++j) {
                double lm = double(1 - LM(i, j, l));
                a(14, i, j, k) = h2 * d * lm;
                a(23, i, j, k) = 0.0;
                a(5, i, j, k) = -(a(14, i, j, k) + a(23, i, j, k));
            }
        } break;
        case 6:
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m; ++j) for (int k = 1; k <= l; ++k) {
                double lm = double(1 - LM(i, j, l));
                a(23, i, j, k) = 1.0 * lm;
                a(5, i, j, k) = 1.0 * lm;
            }
            break;
        case 7:
            for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) a(5, i, j, 1) = 1.0;
            break;
        }
    }
    void coriolis(int /*type*/, Atom& a) {
        a.zero();
        for (int j = 1; j <= m - 1; ++j) {
            double corv = std::sin(YV(j)) * coriolis_on;
            for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) a(5, i, j, k) = corv;
        }
    }
    void gradp(int type, Atom& a) {
        a.zero();
        switch (type) {
        case 1:
            for (int j = 1; j <= m - 1; ++j) {
                double c = 1. / (2 * std::cos(YV(j)) * dx);
                for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) {
                    a(5, i, j, k) = -c; a(6, i, j, k) = -c; a(8, i, j, k) = c; a(9, i, j, k) = c;
                }
            }
            break;
        case 2: {
            double dyi = 1. / (2 * dy);
            for (int i = 1; i <= n; ++i) for (int j = 1; j <= m - 1; ++j) for (int k = 1; k <= l; ++k) {
                a(5, i, j, k) = -dyi; a(8, i, j, k) = -dyi; a(6, i, j, k) = dyi; a(9, i, j, k) = dyi;
            }
        } break;
        case 3: {
            double dzi = 1. / dz;
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                a(5, i, j, k) = -(dzi / DFZW(k));
                a(23, i, j, k) = dzi / DFZW(k);
            }
        } break;
        }
    }

    // Writes Al(:,A,B,:,:,1:l) = value(kk,i,j,k) for all entries.
    template <class F>
    void setAl(int A, int B, F f) {
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
            for (int kk = 1; kk <= NP; ++kk) AL(kk, A, B, i, j, k) = f(kk, i, j, k);
    }
    template <class F>
    void addAn(int A, int B, F f) {
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
            for (int kk = 1; kk <= NP; ++kk) {
                double& r = AN(kk, A, B, i, j, k);
                r = f(r, kk, i, j, k);
            }
    }

    // ---- lin: src/ocean/usrc.F90:605-789 (uncoupled branch) ----
    void lin() {
        Atom ucsi = mk(), uxx = mk(), uyy = mk(), uzz = mk(), uxs = mk(), fu = mk(), px = mk(), sc = mk(),
             tcb = mk();
        double EV = par[EK_V], EH = par[EK_H], ph = (1 - par[MIXP]) * par[PE_H], pv = par[PE_V],
               lambda = par[LAMB], xes = par[NLES], bi = par[BIOT], Ra = par[RAYL];
        std::fill(Al.begin(), Al.end(), 0.0);
        // u-equation
        uderiv(2, uxx); uderiv(3, uyy); uderiv(4, uzz); uderiv(5, ucsi); uderiv(6, uxs);
        coriolis(1, fu); gradp(1, px);
        setAl(UU, UU, [&](int kk, int i, int j, int k) {
            return -EH * (uxx(kk, i, j, k) + uyy(kk, i, j, k) + ucsi(kk, i, j, k)) - EV * uzz(kk, i, j, k);
        });
        setAl(UU, VV, [&](int kk, int i, int j, int k) { return -fu(kk, i, j, k) - EH * uxs(kk, i, j, k); });
        setAl(UU, PP, [&](int kk, int i, int j, int k) { return px(kk, i, j, k); });
        // v-equation
        vderiv(2, uxx); vderiv(3, uyy); vderiv(4, uzz); vderiv(5, ucsi); vderiv(6, uxs);
        coriolis(2, fu); gradp(2, px);
        setAl(VV, UU, [&](int kk, int i, int j, int k) { return fu(kk, i, j, k) - EH * uxs(kk, i, j, k); });
        setAl(VV, VV, [&](int kk, int i, int j, int k) {
            return -EH * (uxx(kk, i, j, k) + uyy(kk, i, j, k) + ucsi(kk, i, j, k)) - EV * uzz(kk, i, j, k);
        });
        setAl(VV, PP, [&](int kk, int i, int j, int k) { return px(kk, i, j, k); });
        // w-equation
        gradp(3, px); tderiv(6, uxs);
        setAl(WW, PP, [&](int kk, int i, int j, int k) { return px(kk, i, j, k); });
        setAl(WW, TT, [&](int kk, int i, int j, int k) { return -Ra * (1. + xes * alpt1) * uxs(kk, i, j, k) / 2.; });
        setAl(WW, SS, [&](int kk, int i, int j, int k) { return lambda * Ra * uxs(kk, i, j, k) / 2.; });
        // p-equation
        pderiv(1, uxx); pderiv(2, uyy); pderiv(3, uzz);
        setAl(PP, UU, [&](int kk, int i, int j, int k) { return uxx(kk, i, j, k); });
        setAl(PP, VV, [&](int kk, int i, int j, int k) { return uyy(kk, i, j, k); });
        setAl(PP, WW, [&](int kk, int i, int j, int k) { return uzz(kk, i, j, k); });
        // T-equation
        tderiv(1, fu); tderiv(2, sc); tderiv(3, uxx); tderiv(4, uyy); tderiv(5, uzz); tderiv(7, tcb);
        setAl(TT, TT, [&](int kk, int i, int j, int k) {
            return -ph * (uxx(kk, i, j, k) + uyy(kk, i, j, k)) - pv * uzz(kk, i, j, k) + TRES * bi * fu(kk, i, j, k);
        });
        // S-equation
        setAl(SS, SS, [&](int kk, int i, int j, int k) {
            return -ph * (uxx(kk, i, j, k) + uyy(kk, i, j, k)) - pv * uzz(kk, i, j, k) + SRES * bi * sc(kk, i, j, k);
        });
    }

    // ---- usol: src/ocean/usrc.F90:1014-1121 ----
    Arr3 u, v, w, p, t, s;
    void usol(const double* un) {
        u = Arr3(0, n, 0, m, 0, l + 1); v = Arr3(0, n, 0, m, 0, l + 1);
        w = Arr3(0, n + 1, 0, m + 1, 0, l); p = Arr3(0, n + 1, 0, m + 1, 0, l + 1);
        t = Arr3(0, n + 1, 0, m + 1, 0, l + 1); s = Arr3(0, n + 1, 0, m + 1, 0, l + 1);
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
            u(i, j, k) = un[find_row2(i, j, k, UU) - 1];
            v(i, j, k) = un[find_row2(i, j, k, VV) - 1];
            w(i, j, k) = un[find_row2(i, j, k, WW) - 1];
            p(i, j, k) = un[find_row2(i, j, k, PP) - 1];
            t(i, j, k) = un[find_row2(i, j, k, TT) - 1];
            s(i, j, k) = un[find_row2(i, j, k, SS) - 1];
        }
        const int N = n, M = m;
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) {
            if (periodic) {
                u(0, j, k) = u(N, j, k); v(0, j, k) = v(N, j, k);
                w(N + 1, j, k) = w(1, j, k); w(0, j, k) = w(N, j, k);
                p(N + 1, j, k) = p(1, j, k); p(0, j, k) = p(N, j, k);
                t(N + 1, j, k) = t(1, j, k); t(0, j, k) = t(N, j, k);
                s(N + 1, j, k) = s(1, j, k); s(0, j, k) = s(N, j, k);
            } else {
                u(0, j, k) = 0.0; u(N, j, k) = 0.0; v(0, j, k) = 0.0; v(N, j, k) = 0.0;
                p(0, j, k) = 0.0; p(N + 1, j, k) = 0.0;
                t(0, j, k) = t(1, j, k); t(N + 1, j, k) = t(N, j, k);
                s(0, j, k) = s(1, j, k); s(N + 1, j, k) = s(N, j, k);
            }
        }
        for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) {
            u(i, 0, k) = 0.0; u(i, M, k) = 0.0; v(i, 0, k) = 0.0; v(i, M, k) = 0.0;
            p(i, 0, k) = 0.0; p(i, M + 1, k) = 0.0;
            t(i, 0, k) = t(i, 1, k); t(i, M + 1, k) = t(i, M, k);
            s(i, 0, k) = s(i, 1, k); s(i, M + 1, k) = s(i, M, k);
        }
        for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
            u(i, j, 0) = u(i, j, 1); u(i, j, l + 1) = u(i, j, l);
            v(i, j, 0) = v(i, j, 1); v(i, j, l + 1) = v(i, j, l);
            w(i, j, l) = 0.0; w(i, j, 0) = 0.0;
            p(i, j, l + 1) = 0.0; p(i, j, 0) = 0.0;
            t(i, j, l + 1) = t(i, j, l); t(i, j, 0) = t(i, j, 1);
            s(i, j, l + 1) = s(i, j, l); s(i, j, 0) = s(i, j, 1);
        }
        for (int i = 1; i <= n; ++i) for (int j = 1; j <= m; ++j) for (int k = 1; k <= l; ++k)
            if (LM(i, j, k) == 1) {
                u(i, j, k) = 0.0; v(i, j, k) = 0.0; u(i - 1, j, k) = 0.0; v(i - 1, j, k) = 0.0;
                u(i, j - 1, k) = 0.0; v(i, j - 1, k) = 0.0; u(i - 1, j - 1, k) = 0.0; v(i - 1, j - 1, k) = 0.0;
            }
    }

    // ---- tnlin: src/ocean/spf.F90:362-484 ----
    void tnlin(int type, Atom& a, Arr3& U, Arr3& V, Arr3& W, Arr3& T) {
        a.zero();
        switch (type) {
        case 2:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                double c = 1.0 / (4 * std::cos(Y(j)) * dx), lm = double(1 - LM(i, j, l));
                a(2, i, j, k) = -(T(i, j, k) + T(i - 1, j, k)) * c * lm;
                a(4, i, j, k) = (T(i + 1, j, k) + T(i, j, k)) * c * lm;
                a(1, i, j, k) = -(T(i, j, k) + T(i - 1, j, k)) * c * lm;
                a(5, i, j, k) = (T(i + 1, j, k) + T(i, j, k)) * c * lm;
            }
            break;
        case 3:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                double c = 1.0 / (4 * std::cos(Y(j)) * dx), lm = double(1 - LM(i, j, l));
                a(2, i, j, k) = -(U(i - 1, j, k) + U(i - 1, j - 1, k)) * c * lm;
                a(8, i, j, k) = (U(i, j, k) + U(i, j - 1, k)) * c * lm;
                a(5, i, j, k) = a(2, i, j, k) + a(8, i, j, k);
            }
            break;
        case 4:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                double c = 1.0 / (4 * std::cos(Y(j)) * dy), lm = double(1 - LM(i, j, l));
                a(4, i, j, k) = -c * (T(i, j, k) + T(i, j - 1, k)) * std::cos(YV(j - 1)) * lm;
                a(1, i, j, k) = -c * (T(i, j, k) + T(i, j - 1, k)) * std::cos(YV(j - 1)) * lm;
                a(5, i, j, k) = c * (T(i, j + 1, k) + T(i, j, k)) * std::cos(YV(j)) * lm;
                a(2, i, j, k) = c * (T(i, j + 1, k) + T(i, j, k)) * std::cos(YV(j)) * lm;
            }
            break;
        case 5:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                double c = 1.0 / (4 * std::cos(Y(j)) * dy), lm = double(1 - LM(i, j, l));
                a(4, i, j, k) = -(V(i, j - 1, k) + V(i - 1, j - 1, k)) * c * std::cos(YV(j - 1)) * lm;
                a(6, i, j, k) = (V(i, j, k) + V(i - 1, j, k)) * c * std::cos(YV(j)) * lm;
                a(5, i, j, k) = a(4, i, j, k) + a(6, i, j, k);
            }
            break;
        case 6: {
            double tdzi = 1.0 / (2 * dz);
            for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                double lm = double(1 - LM(i, j, l));
                for (int k = 1; k <= l - 1; ++k) {
                    a(14, i, j, k) = -tdzi * lm * (T(i, j, k) + T(i, j, k - 1)) / DFZT(k);
                    a(5, i, j, k) = tdzi * lm * (T(i, j, k + 1) + T(i, j, k)) / DFZT(k);
                }
                int k = l;
                a(14, i, j, k) = -tdzi * lm * (T(i, j, k) + T(i, j, k - 1)) / DFZT(k);
                a(5, i, j, k) = 0.0;
            }
        } break;
        case 7: {
            double tdzi = 1.0 / (2 * dz);
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                double lm = double(1 - LM(i, j, l));
                a(14, i, j, k) = -W(i, j, k - 1) * lm * tdzi / DFZT(k);
                a(23, i, j, k) = W(i, j, k) * lm * tdzi / DFZT(k);
                a(5, i, j, k) = a(14, i, j, k) + a(23, i, j, k);
            }
        } break;
        }
    }
    // ---- wnlin: src/ocean/spf.F90:486-542 ----
    void wnlin(int type, Atom& a, Arr3& T) {
        a.zero();
        for (int k = 1; k <= l - 1; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
            double t0 = T(i, j, k), t1 = T(i, j, k + 1);
            switch (type) {
            case 1: a(23, i, j, k) = (t0 + t1) / 2.; a(5, i, j, k) = (t0 + t1) / 2.; break;
            case 2: a(23, i, j, k) = t1 / 4.; a(5, i, j, k) = (t0 + 2 * t1) / 4.; break;
            case 3: {
                double q = t0 + t1;
                a(5, i, j, k) = 0.375 * (q * q);
                a(23, i, j, k) = 0.375 * (q * q);
            } break;
            case 4:
                a(5, i, j, k) = 0.125 * (t0 * t0 + 3 * t1 * t0 + 3 * t1 * t1);
                a(23, i, j, k) = 0.125 * t1 * t1;
                break;
            }
        }
    }
    // ---- unlin: src/ocean/spf.F90:544-665 ----
    void unlin(int type, Atom& a, Arr3& U, Arr3& V, Arr3& W) {
        a.zero();
        switch (type) {
        case 1:
        case 2: {
            double f = (type == 2) ? 2.0 : 1.0;
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) {
                double c = 1.0 / (2 * std::cos(YV(j)) * dx);
                for (int i = 1; i <= n - 1; ++i) a(8, i, j, k) = (type == 2 ? f * U(i + 1, j, k) : U(i + 1, j, k)) * c;
                for (int i = 2; i <= n; ++i) a(2, i, j, k) = -(type == 2 ? f * U(i - 1, j, k) : U(i - 1, j, k)) * c;
            }
        } break;
        case 3:
        case 4: {
            Arr3& Q = (type == 3) ? V : U;
            for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) {
                for (int j = 2; j <= m; ++j) {
                    double c = 1.0 / (2 * std::cos(YV(j)) * dy);
                    a(4, i, j, k) = -Q(i, j - 1, k) * std::cos(YV(j - 1)) * c;
                }
                for (int j = 1; j <= m - 1; ++j) {
                    double c = 1.0 / (2 * std::cos(YV(j)) * dy);
                    a(6, i, j, k) = Q(i, j + 1, k) * std::cos(YV(j + 1)) * c;
                }
            }
        } break;
        case 5:
            for (int k = 1; k <= l; ++k) {
                double tdzi = 1.0 / (8 * DFZT(k) * dz);
                for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                    a(23, i, j, k) = (W(i, j, k) + W(i, j + 1, k) + W(i + 1, j, k) + W(i + 1, j + 1, k)) * tdzi;
                    a(14, i, j, k) = -(W(i, j, k - 1) + W(i, j + 1, k - 1) + W(i + 1, j, k - 1) + W(i + 1, j + 1, k - 1)) * tdzi;
                    a(5, i, j, k) = a(14, i, j, k) + a(23, i, j, k);
                }
            }
            break;
        case 6:
            for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) for (int k = 1; k <= l; ++k) {
                double tdzi = 1.0 / (8 * DFZT(k) * dz);
                double up = (U(i, j, k) + U(i, j, k + 1)) * tdzi;
                double dn = -(U(i, j, k) + U(i, j, k - 1)) * tdzi;
                a(5, i, j, k) = up; a(6, i, j, k) = up; a(8, i, j, k) = up; a(9, i, j, k) = up;
                a(14, i, j, k) = dn; a(15, i, j, k) = dn; a(17, i, j, k) = dn; a(18, i, j, k) = dn;
            }
            break;
        case 7:
        case 8: {
            Arr3& Q = (type == 7) ? V : U;
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
                a(5, i, j, k) = Q(i, j, k) * std::tan(YV(j));
        } break;
        }
    }
    // ---- vnlin: src/ocean/spf.F90:667-790 ----
    void vnlin(int type, Atom& a, Arr3& U, Arr3& V, Arr3& W) {
        a.zero();
        switch (type) {
        case 1:
        case 2: {
            Arr3& Q = (type == 1) ? U : V;
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) {
                double c = 1.0 / (2 * std::cos(YV(j)) * dx);
                for (int i = 1; i <= n - 1; ++i) a(8, i, j, k) = Q(i + 1, j, k) * c;
                for (int i = 2; i <= n; ++i) a(2, i, j, k) = -Q(i - 1, j, k) * c;
            }
        } break;
        case 3:
        case 4: {
            for (int k = 1; k <= l; ++k) for (int i = 1; i <= n; ++i) {
                for (int j = 1; j <= m - 1; ++j) {
                    double c = 1.0 / (2 * std::cos(YV(j)) * dy);
                    a(6, i, j, k) = (type == 4 ? 2 * V(i, j + 1, k) : V(i, j + 1, k)) * std::cos(YV(j + 1)) * c;
                }
                for (int j = 2; j <= m; ++j) {
                    double c = 1.0 / (2 * std::cos(YV(j)) * dy);
                    a(4, i, j, k) = -(type == 4 ? 2 * V(i, j - 1, k) : V(i, j - 1, k)) * std::cos(YV(j - 1)) * c;
                }
            }
        } break;
        case 5:
            unlin(5, a, U, V, W);
            break;
        case 6:
            unlin(6, a, V, V, W);
            break;
        case 7:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
                a(5, i, j, k) = U(i, j, k) * std::tan(YV(j));
            break;
        case 8:
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
                a(5, i, j, k) = 2 * U(i, j, k) * std::tan(YV(j));
            break;
        }
    }

    // ---- nlin_rhs: src/ocean/usrc.F90:792-887 ----
    void nlin_rhs(const double* un) {
        double lambda = par[LAMB], epsr = par[ROSB], Ra = par[RAYL], xes = par[NLES];
        (void)lambda;
        usol(un);
        Atom a1 = mk(), a2 = mk(), a3 = mk(), a4 = mk();
        unlin(1, a1, u, v, w); unlin(3, a2, u, v, w); unlin(5, a3, u, v, w); unlin(7, a4, u, v, w);
        addAn(UU, UU, [&](double r, int kk, int i, int j, int k) {
            return r + epsr * (a1(kk, i, j, k) + a2(kk, i, j, k) + a3(kk, i, j, k) + a4(kk, i, j, k));
        });
        vnlin(1, a1, u, v, w); vnlin(3, a2, u, v, w); vnlin(5, a3, u, v, w); vnlin(7, a4, u, v, w);
        addAn(VV, UU, [&](double r, int kk, int i, int j, int k) { return r + epsr * a4(kk, i, j, k); });
        addAn(VV, VV, [&](double r, int kk, int i, int j, int k) {
            return r + epsr * (a1(kk, i, j, k) + a2(kk, i, j, k) + a3(kk, i, j, k));
        });
        wnlin(2, a1, t); wnlin(4, a2, t);
        addAn(WW, TT, [&](double r, int kk, int i, int j, int k) {
            return r - Ra * xes * alpt2 * a1(kk, i, j, k) + Ra * xes * alpt3 * a2(kk, i, j, k);
        });
        tnlin(3, a1, u, v, w, t); tnlin(5, a2, u, v, w, t); tnlin(7, a3, u, v, w, t);
        addAn(TT, TT, [&](double r, int kk, int i, int j, int k) {
            return r + a1(kk, i, j, k) + a2(kk, i, j, k) + a3(kk, i, j, k);
        });
        tnlin(3, a1, u, v, w, s); tnlin(5, a2, u, v, w, s); tnlin(7, a3, u, v, w, s);
        addAn(SS, SS, [&](double r, int kk, int i, int j, int k) {
            return r + a1(kk, i, j, k) + a2(kk, i, j, k) + a3(kk, i, j, k);
        });
    }

    // ---- nlin_jac: src/ocean/usrc.F90:890-1012 ----
    void nlin_jac(const double* un) {
        double epsr = par[ROSB], Ra = par[RAYL], xes = par[NLES];
        usol(un);
        Atom a1 = mk(), a2 = mk(), a3 = mk(), a4 = mk(), a5 = mk(), a6 = mk(), a7 = mk();
        // u-equation
        unlin(2, a1, u, v, w); unlin(3, a2, u, v, w); unlin(4, a3, u, v, w); unlin(5, a4, u, v, w);
        unlin(6, a5, u, v, w); unlin(7, a6, u, v, w); unlin(8, a7, u, v, w);
        addAn(UU, UU, [&](double r, int kk, int i, int j, int k) {
            return r + epsr * (a1(kk, i, j, k) + a2(kk, i, j, k) + a4(kk, i, j, k) + a6(kk, i, j, k));
        });
        addAn(UU, VV, [&](double r, int kk, int i, int j, int k) { return r + epsr * (a3(kk, i, j, k) + a7(kk, i, j, k)); });
        addAn(UU, WW, [&](double r, int kk, int i, int j, int k) { return r + epsr * a5(kk, i, j, k); });
        // v-equation
        vnlin(1, a1, u, v, w); vnlin(2, a2, u, v, w); vnlin(4, a3, u, v, w); vnlin(5, a4, u, v, w);
        vnlin(6, a5, u, v, w); vnlin(8, a6, u, v, w);
        addAn(VV, UU, [&](double r, int kk, int i, int j, int k) { return r + epsr * (a6(kk, i, j, k) + a2(kk, i, j, k)); });
        addAn(VV, VV, [&](double r, int kk, int i, int j, int k) {
            return r + epsr * (a1(kk, i, j, k) + a3(kk, i, j, k) + a4(kk, i, j, k));
        });
        addAn(VV, WW, [&](double r, int kk, int i, int j, int k) { return r + epsr * a5(kk, i, j, k); });
        // w-equation
        wnlin(1, a1, t); wnlin(3, a2, t);
        addAn(WW, TT, [&](double r, int kk, int i, int j, int k) {
            return r - Ra * xes * alpt2 * a1(kk, i, j, k) + Ra * xes * alpt3 * a2(kk, i, j, k);
        });
        // T and S equations
        for (int q = 0; q < 2; ++q) {
            Arr3& X = q == 0 ? t : s;
            int A = q == 0 ? TT : SS;
            tnlin(2, a1, u, v, w, X); tnlin(3, a2, u, v, w, X); tnlin(4, a3, u, v, w, X);
            tnlin(5, a4, u, v, w, X); tnlin(6, a5, u, v, w, X); tnlin(7, a6, u, v, w, X);
            addAn(A, UU, [&](double r, int kk, int i, int j, int k) { return r + a1(kk, i, j, k); });
            addAn(A, VV, [&](double r, int kk, int i, int j, int k) { return r + a3(kk, i, j, k); });
            addAn(A, WW, [&](double r, int kk, int i, int j, int k) { return r + a5(kk, i, j, k); });
            addAn(A, A, [&](double r, int kk, int i, int j, int k) {
                return r + a2(kk, i, j, k) + a4(kk, i, j, k) + a6(kk, i, j, k);
            });
        }
    }

    // ---- boundaries: src/ocean/boundary.F90:2-393 ----
    void boundaries() {
        auto A = [&](int kk, int a, int b, int i, int j, int k) -> double& { return AN(kk, a, b, i, j, k); };
        auto zeroPos = [&](int kk, int i, int j, int k) {
            for (int b = 1; b <= NUN; ++b) for (int a = 1; a <= NUN; ++a) A(kk, a, b, i, j, k) = 0.0;
        };
        auto zeroPosCol = [&](int kk, int b, int i, int j, int k) {
            for (int a = 1; a <= NUN; ++a) A(kk, a, b, i, j, k) = 0.0;
        };
        auto foldCol = [&](int dst, int src, int b, int i, int j, int k) {
            for (int a = 1; a <= NUN; ++a) A(dst, a, b, i, j, k) = A(dst, a, b, i, j, k) + A(src, a, b, i, j, k);
        };
        auto dirRow = [&](int a, int i, int j, int k) {   // An(:,a,:) = 0; An(5,:,a) = 0; An(5,a,a) = 1
            for (int b = 1; b <= NUN; ++b) for (int kk = 1; kk <= NP; ++kk) A(kk, a, b, i, j, k) = 0.0;
            zeroPosCol(5, a, i, j, k);
            A(5, a, a, i, j, k) = 1.0;
        };
        for (int i = 1; i <= n; ++i) for (int j = 1; j <= m; ++j) for (int k = 1; k <= l; ++k) {
            int southw = LM(i - 1, j - 1, k), west = LM(i - 1, j, k), nwest = LM(i - 1, j + 1, k);
            int south = LM(i, j - 1, k), center = LM(i, j, k), north = LM(i, j + 1, k);
            int southe = LM(i + 1, j - 1, k), east = LM(i + 1, j, k), neast = LM(i + 1, j + 1, k);
            int southwb = LM(i - 1, j - 1, k - 1), westb = LM(i - 1, j, k - 1), nwestb = LM(i - 1, j + 1, k - 1);
            int southb = LM(i, j - 1, k - 1), bottom = LM(i, j, k - 1), northb = LM(i, j + 1, k - 1);
            int southeb = LM(i + 1, j - 1, k - 1), eastb = LM(i + 1, j, k - 1), neastb = LM(i + 1, j + 1, k - 1);
            int southwt = LM(i - 1, j - 1, k + 1), westt = LM(i - 1, j, k + 1), nwestt = LM(i - 1, j + 1, k + 1);
            int southt = LM(i, j - 1, k + 1), top = LM(i, j, k + 1), northt = LM(i, j + 1, k + 1);
            int southet = LM(i + 1, j - 1, k + 1), eastt = LM(i + 1, j, k + 1), neastt = LM(i + 1, j + 1, k + 1);
            int southee = -1, easteast = -1, northee = -1, nnorthee = -1, nnwest = -1, nnorth = -1, nneast = -1;
            if (i < n) {
                southee = LM(i + 2, j - 1, k);
                easteast = LM(i + 2, j, k);
                northee = LM(i + 2, j + 1, k);
                if (j < m) nnorthee = LM(i + 2, j + 2, k);
            }
            if (j < m) { nnwest = LM(i, j + 2, k); nnorth = LM(i, j + 2, k); nneast = LM(i, j + 2, k); }

            if (center == OCEAN) {
                if (bottom == LAND) {
                    if (westb == LAND && southwb == LAND && southb == LAND) { foldCol(1, 10, UU, i, j, k); foldCol(1, 10, VV, i, j, k); }
                    zeroPosCol(10, UU, i, j, k); zeroPosCol(10, VV, i, j, k);
                    if (westb == LAND && neastb == LAND && northb == LAND) { foldCol(2, 11, UU, i, j, k); foldCol(2, 11, VV, i, j, k); }
                    zeroPosCol(11, UU, i, j, k); zeroPosCol(11, VV, i, j, k);
                    if (eastb == LAND && southeb == LAND && southb == LAND) { foldCol(4, 13, UU, i, j, k); foldCol(4, 13, VV, i, j, k); }
                    zeroPosCol(13, UU, i, j, k); zeroPosCol(13, VV, i, j, k);
                    if (eastb == LAND && neastb == LAND && northb == LAND) { foldCol(5, 14, UU, i, j, k); foldCol(5, 14, VV, i, j, k); }
                    foldCol(5, 14, TT, i, j, k); foldCol(5, 14, SS, i, j, k);
                    zeroPos(14, i, j, k);
                }
                if (southwb == LAND) zeroPos(10, i, j, k);
                if (westb == LAND) zeroPos(11, i, j, k);
                if (nwestb == LAND) zeroPos(12, i, j, k);
                if (southb == LAND) zeroPos(13, i, j, k);
                if (northb == LAND) zeroPos(15, i, j, k);
                if (southeb == LAND) zeroPos(16, i, j, k);
                if (eastb == LAND) zeroPos(17, i, j, k);
                if (neastb == LAND) zeroPos(18, i, j, k);
                if (top == LAND) {
                    if (westt == LAND && southwt == LAND && southt == LAND) { foldCol(1, 19, UU, i, j, k); foldCol(1, 19, VV, i, j, k); }
                    zeroPosCol(19, UU, i, j, k); zeroPosCol(19, VV, i, j, k);
                    if (westt == LAND && nwestt == LAND && northt == LAND) { foldCol(2, 20, UU, i, j, k); foldCol(2, 20, VV, i, j, k); }
                    zeroPosCol(20, UU, i, j, k); zeroPosCol(20, VV, i, j, k);
                    if (eastt == LAND && southet == LAND && southt == LAND) { foldCol(4, 22, UU, i, j, k); foldCol(4, 22, VV, i, j, k); }
                    zeroPosCol(22, UU, i, j, k); zeroPosCol(22, VV, i, j, k);
                    if (eastt == LAND && neastt == LAND && northt == LAND) { foldCol(5, 23, UU, i, j, k); foldCol(5, 23, VV, i, j, k); }
                    foldCol(5, 23, TT, i, j, k); foldCol(5, 23, SS, i, j, k);
                    zeroPos(23, i, j, k);
                    Frc[find_row2(i, j, k, WW) - 1] = 0.0;
                    for (int b = 1; b <= NUN; ++b) for (int kk = 1; kk <= NP; ++kk) A(kk, WW, b, i, j, k) = 0.0;
                    for (int a = 1; a <= NUN; ++a) {
                        A(5, a, WW, i, j, k) = 1.0e-10; A(6, a, WW, i, j, k) = 1.0e-10;
                        A(8, a, WW, i, j, k) = 1.0e-10; A(9, a, WW, i, j, k) = 1.0e-10;
                    }
                    A(5, WW, WW, i, j, k) = 1.0;
                }
                if (southwt == LAND) zeroPos(19, i, j, k);
                if (westt == LAND) zeroPos(20, i, j, k);
                if (nwestt == LAND) zeroPos(21, i, j, k);
                if (southt == LAND) zeroPos(22, i, j, k);
                if (northt == LAND) zeroPos(24, i, j, k);
                if (southet == LAND) zeroPos(25, i, j, k);
                if (eastt == LAND) zeroPos(26, i, j, k);
                if (neastt == LAND) zeroPos(27, i, j, k);
                if (southw == LAND) { zeroPosCol(1, UU, i, j, k); zeroPosCol(1, VV, i, j, k); }
                if (west == LAND) {
                    foldCol(5, 2, TT, i, j, k); foldCol(5, 2, SS, i, j, k);
                    zeroPos(2, i, j, k);
                    zeroPosCol(1, UU, i, j, k); zeroPosCol(1, VV, i, j, k);
                }
                if (nwest == LAND) {
                    zeroPosCol(2, UU, i, j, k); zeroPosCol(2, VV, i, j, k);
                    zeroPosCol(3, UU, i, j, k); zeroPosCol(3, VV, i, j, k);
                } else if (j < m) {
                    if (nnwest == LAND) { zeroPosCol(3, UU, i, j, k); zeroPosCol(3, VV, i, j, k); }
                }
                if (south == LAND) {
                    foldCol(5, 4, SS, i, j, k); foldCol(5, 4, TT, i, j, k);
                    zeroPos(4, i, j, k);
                    zeroPosCol(1, UU, i, j, k); zeroPosCol(1, VV, i, j, k);
                }
                if (north == LAND) {
                    zeroPosCol(2, UU, i, j, k); zeroPosCol(2, VV, i, j, k);
                    A(2, PP, UU, i, j, k) = 0.0; A(2, PP, VV, i, j, k) = 0.0;
                    A(5, PP, UU, i, j, k) = 0.0; A(5, PP, VV, i, j, k) = 0.0;
                    Frc[find_row2(i, j, k, VV) - 1] = 0.0;
                    dirRow(VV, i, j, k);
                    Frc[find_row2(i, j, k, UU) - 1] = 0.0;
                    dirRow(UU, i, j, k);
                    foldCol(5, 6, SS, i, j, k); foldCol(5, 6, TT, i, j, k);
                    zeroPos(6, i, j, k);
                } else if (j < m) {
                    if (nnorth == LAND) {
                        zeroPosCol(3, UU, i, j, k); zeroPosCol(3, VV, i, j, k);
                        zeroPosCol(6, UU, i, j, k); zeroPosCol(6, VV, i, j, k);
                    }
                }
                if (southe == LAND) {
                    zeroPosCol(4, UU, i, j, k); zeroPosCol(4, VV, i, j, k);
                    zeroPosCol(7, UU, i, j, k); zeroPosCol(7, VV, i, j, k);
                } else if (i < n) {
                    if (southee == LAND) { zeroPosCol(7, UU, i, j, k); zeroPosCol(7, VV, i, j, k); }
                }
                if (east == LAND) {
                    zeroPosCol(4, UU, i, j, k); zeroPosCol(4, VV, i, j, k);
                    A(4, PP, UU, i, j, k) = 0.0; A(4, PP, VV, i, j, k) = 0.0;
                    A(5, PP, UU, i, j, k) = 0.0; A(5, PP, VV, i, j, k) = 0.0;
                    Frc[find_row2(i, j, k, UU) - 1] = 0.0;
                    dirRow(UU, i, j, k);
                    Frc[find_row2(i, j, k, VV) - 1] = 0.0;
                    dirRow(VV, i, j, k);
                    foldCol(5, 8, SS, i, j, k); foldCol(5, 8, TT, i, j, k);
                    zeroPos(8, i, j, k);
                    zeroPosCol(7, UU, i, j, k); zeroPosCol(7, VV, i, j, k);
                } else if (i < n) {
                    if (easteast == LAND) {
                        zeroPosCol(7, UU, i, j, k); zeroPosCol(7, VV, i, j, k);
                        zeroPosCol(8, UU, i, j, k); zeroPosCol(8, VV, i, j, k);
                    }
                }
                if (neast == LAND) {
                    Frc[find_row2(i, j, k, UU) - 1] = 0.0;
                    dirRow(UU, i, j, k);
                    Frc[find_row2(i, j, k, VV) - 1] = 0.0;
                    dirRow(VV, i, j, k);
                    zeroPosCol(7, UU, i, j, k); zeroPosCol(7, VV, i, j, k);
                } else if (i < n || j < m) {
                    if (i < n) {
                        if (northee == LAND) {
                            zeroPosCol(8, UU, i, j, k); zeroPosCol(8, VV, i, j, k);
                            zeroPosCol(9, UU, i, j, k); zeroPosCol(9, VV, i, j, k);
                        } else if (j < m) {
                            if (nnorthee == LAND) { zeroPosCol(9, UU, i, j, k); zeroPosCol(9, VV, i, j, k); }
                        }
                    }
                    if (j < m) {
                        if (nneast == LAND) {
                            zeroPosCol(6, UU, i, j, k); zeroPosCol(6, VV, i, j, k);
                            zeroPosCol(9, UU, i, j, k); zeroPosCol(9, VV, i, j, k);
                        }
                    }
                }
            } else {
                for (int b = 1; b <= NUN; ++b) for (int a = 1; a <= NUN; ++a) for (int kk = 1; kk <= NP; ++kk)
                    A(kk, a, b, i, j, k) = 0.0;
                for (int ii = 1; ii <= NUN; ++ii) {
                    Frc[find_row2(i, j, k, ii) - 1] = 0.0;
                    A(5, ii, ii, i, j, k) = 1.0;
                }
            }
        }
    }

    // ---- shift: src/ocean/assemble.F90:142-179 ----
    void shift(int i, int j, int k, int& i2, int& j2, int& k2, int kk) const {
        if (kk < 10) { k2 = k; j2 = j - 1 + (kk + 2) % 3; i2 = i - 1 + (kk - 1) / 3; }
        else if (kk < 19) { k2 = k - 1; j2 = j - 1 + (kk + 2) % 3; i2 = i - 1 + (kk - 10) / 3; }
        else { k2 = k + 1; j2 = j - 1 + (kk + 2) % 3; i2 = i - 1 + (kk - 19) / 3; }
        if (periodic) {
            if (i2 == 0) i2 = n;
            else if (i2 == n + 1) i2 = 1;
        }
    }
    // ---- fillcolA: src/ocean/assemble.F90:57-139 (drop rule abs(c) > 1e-10) ----
    std::vector<char> inDomain;   // per Fortran entry: neighbour inside 1..n,1..m,1..l
    void fillcolA() {
        begA.assign(ndim + 1, 0);
        jcoA.clear(); coA.clear(); inDomain.clear();
        int v = 1, row = 1;
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
            for (int ii = 1; ii <= NUN; ++ii) {
                begA[row - 1] = v;
                for (int kk = 1; kk <= NP; ++kk) for (int jj = 1; jj <= NUN; ++jj) {
                    double c = AN(kk, ii, jj, i, j, k);
                    if (std::fabs(c) > 1.0e-10) {
                        coA.push_back(c);
                        int i2, j2, k2;
                        shift(i, j, k, i2, j2, k2, kk);
                        jcoA.push_back(find_row2(i2, j2, k2, jj));
                        inDomain.push_back(i2 >= 1 && i2 <= n && j2 >= 1 && j2 <= m && k2 >= 1 && k2 <= l);
                        ++v;
                    }
                }
                ++row;
            }
        begA[ndim] = v;
    }
    // ---- fillcolB: src/ocean/assemble.F90:18-54 ----
    void fillcolB() {
        coB.assign(ndim, 0.0);
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
            if (LM(i, j, k) == OCEAN) {
                if (LM(i + 1, j, k) != LAND) coB[find_row2(i, j, k, UU) - 1] = -par[ROSB];
                if (LM(i, j + 1, k) != LAND) coB[find_row2(i, j, k, VV) - 1] = -par[ROSB];
                coB[find_row2(i, j, k, TT) - 1] = -1.0;
                coB[find_row2(i, j, k, SS) - 1] = -1.0;
            }
        if (rowintcon >= 0) coB[rowintcon] = 0.0;   // assemble.F90:49; THCM.C:1233-1238
        if (rowPfix1 >= 0) coB[rowPfix1] = 0.0;     // THCM.C:1220-1230
        if (rowPfix2 >= 0) coB[rowPfix2] = 0.0;
    }
    // ---- matAvec: src/ocean/matetc.F90:147-166 ----
    void matAvec(const double* v1, double* v2) const {
        for (int i = 0; i < ndim; ++i) {
            double acc = 0.0;
            for (int q = begA[i]; q < begA[i + 1]; ++q) acc = coA[q - 1] * v1[jcoA[q - 1] - 1] + acc;
            v2[i] = acc;
        }
    }

    // =====================================================================
    // Vertical mixing and convective adjustment (src/ocean/mix_imp.f,
    // Mixing >= 1): vmix_init 57-111, vmix_control 131-166, vmix_part
    // 168-228 (the partition is recorded as its row/column flags), vmix_fun
    // 231-562 with dCdxt/dCdyt/dCdzt/drhodC/tprslp 564-727, vmix_jac
    // 729-815, isoc 817-833, tprstb 835-856, vmix_el_1/vmix_el_2 858-1050.
    // =====================================================================
    int vmix_flag = 0, vmix_temp = 0, vmix_salt = 0, vmix_fix = 1;
    int part_temp = 0, part_salt = 0;   // row/column sets of the current partition
    long vmix_dim = 0;                  // NPAIRS of the current partition

    void vmix_init() {
        if (vmix == 0) { vmix_flag = 0; vmix_fix = 1; }
        else if (vmix == 1) { vmix_flag = 1; vmix_fix = 1; }
        else if (vmix == 2) { vmix_flag = 2; vmix_fix = 0; }
        else vmix_flag = -1;
        if (vmix_flag == 0) { vmix_temp = 0; vmix_salt = 0; }
        else if (vmix_flag == 1) { vmix_temp = 1; vmix_salt = 1; vmix_part(); }
        else if (vmix_flag == 2) { vmix_temp = 0; vmix_salt = 0; }
    }
    static double l2nrm_stride(const double* f, int count, int stride) {   // matetc.F90:22-36
        double nrm = 0.0;
        for (int i = 0; i < count; ++i) nrm = f[size_t(i) * stride] * f[size_t(i) * stride] + nrm;
        return std::sqrt(nrm);
    }
    void vmix_control(const double* un) {
        int test_temp = l2nrm_stride(un + TT - 1, n * m * l, NUN) > 1.0e-12 ? 1 : 0;
        int test_salt = l2nrm_stride(un + SS - 1, n * m * l, NUN) > 1.0e-12 ? 1 : 0;
        if (vmix_temp != test_temp || vmix_salt != test_salt) {
            vmix_temp = test_temp;
            vmix_salt = test_salt;
            if (vmix_temp != 0 && vmix_temp != 0) vmix_part();   // (sic) the reference tests vmix_temp twice
        }
        vmix_fix = 1;
    }
    // vmix_el_1 (flag 1: T and S rows, T and S columns) / vmix_el_2 (flag 2:
    // rows and columns of the fields switched on). Only the flags and the
    // count matter here: the pairs themselves are enumerated again in vmix_jac.
    void vmix_part() {
        part_temp = vmix_flag == 1 ? 1 : vmix_temp;
        part_salt = vmix_flag == 1 ? 1 : vmix_salt;
        long p = 0;
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
            if (LM(i, j, k) != OCEAN) continue;
            for (int h = 0; h < 27; ++h) {
                const int kind = LM(i + ST[h][0], j + ST[h][1], k + ST[h][2]);
                if (kind == OCEAN || kind == PERIO) p += long(part_temp + part_salt) * (part_temp + part_salt);
            }
        }
        vmix_dim = p;
    }
    // st(27,:) of vmix_el_1 / vmix_el_2: (di, dj, dk) per stencil point
    static constexpr int ST[27][3] = {
        {-1, -1, -1}, {-1, 0, -1}, {-1, 1, -1}, {0, -1, -1}, {0, 0, -1}, {0, 1, -1}, {1, -1, -1}, {1, 0, -1},
        {1, 1, -1},   {-1, -1, 0}, {-1, 0, 0},  {-1, 1, 0},  {0, -1, 0}, {0, 0, 0},  {0, 1, 0},  {1, -1, 0},
        {1, 0, 0},    {1, 1, 0},   {-1, -1, 1}, {-1, 0, 1},  {-1, 1, 1}, {0, -1, 1}, {0, 0, 1},  {0, 1, 1},
        {1, -1, 1},   {1, 0, 1},   {1, 1, 1}};

    double isoc(int i, int j, int k) { return (LM(i, j, k) == OCEAN || LM(i, j, k) == PERIO) ? 1.0 : 0.0; }

    // tanh(y) by one explicit algorithm, the same operation sequence as the
    // GPU kernels': the reference calls the platform libm, whose last bit is
    // implementation-defined (glibc and CUDA differ). |y| < 2^-27 returns y,
    // |y| > 22 returns +-1 (tanh is 1 to the last bit there); otherwise
    // tanh(y) = e / (e + 2) with e = expm1(2|y|): a Taylor series of degree 13
    // below ln2/2, else Cody-Waite reduction x = k ln2 + r (ln2 split into a
    // 32-bit head and a tail) and 2^k (1 + expm1(r)) - 1.
    static double expm1_taylor(double r) {
        static const double c[13] = {0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26,
                                     0x1.27e4fb7789f5cp-22, 0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16,
                                     0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7,
                                     0x1.5555555555555p-5,  0x1.5555555555555p-3,  0x1.0p-1,
                                     0x1.0p+0};   // 1/13!, 1/12!, ..., 1/1!
        double p = c[0];
        for (int q = 1; q < 13; ++q) p = p * r + c[q];
        return p * r;
    }
    static double tanh_x(double y) {
        const double a = std::fabs(y);
        if (!(a >= 0x1p-27)) return y;
        if (a > 22.0) return y > 0 ? 1.0 : -1.0;
        const double x = 2.0 * a;
        double e;
        if (x <= 0x1.62e42fefa39efp-2) {
            e = expm1_taylor(x);
        } else {
            const double kf = std::nearbyint(x / 0x1.62e42fefa39efp-1);
            const double r = (x - kf * 0x1.62e42fee00000p-1) - kf * 0x1.a39ef35793c76p-33;
            e = std::ldexp(expm1_taylor(r) + 1.0, int(kf)) - 1.0;
        }
        const double t = e / (e + 2.0);
        return y < 0 ? -t : t;
    }
    double tprstb(double grad, double spl) const {   // mix_imp.f:835-856
        const double fac = alphaT * spl;
        const double q = -grad * fac;
        return std::max(tanh_x(q * q * q), 0.0);
    }
    void tprslp(double drdh, double drdz, double spl, double& slp, double& tpr) const {   // mix_imp.f:660-727
        const double width = 1.0, epsln = 1.0e-20;
        if (drdz == 0.0) drdz = epsln;
        slp = -drdh / drdz;
        const double absslp = std::sqrt(slp * slp);
        const double delta = (r0dim / hdim) * spl;
        const double sd = width * delta;
        if (tap == 1) {
            if (absslp > delta) { const double q = delta / absslp; tpr = q * q; }
            else tpr = 1.0;
        } else if (tap == 2) {
            tpr = 0.5 * (1.0 - tanh_x((absslp - delta) / sd));
        } else if (tap == 3) {
            if (absslp < delta - sd && drdz < 0.0) tpr = 1.0;
            else if (absslp >= delta - sd && absslp < delta && drdz < 0.0) {
                const double dum = (absslp - (delta - sd)) / sd;
                tpr = 1.0 - 3.0 * (dum * dum) + 2.0 * (dum * dum * dum);
            } else tpr = 0.0;
        } else {
            tpr = 1.0;
        }
    }

    // vmix_fun (mix_imp.f:231-562): divergence of the diffusive T/S fluxes
    void vmix_fun(const double* un, double* mix) {
        usol(un);
        Arr3 T = t, S = s;
        const double xes = par[NLES], lambda = par[LAMB];
        const double piso = par[MIXP] * par[PE_H], pgm = par[MKAP] * par[PE_H];
        const double eps = (1.0 - par[ALPC]) * par[ENER] * par[PE_V];
        const double kvc = par[P_VC], sp1 = par[SPL1], sp2 = par[SPL2];
        const double epsln = 1.0e-20;
        auto dCdxt = [&](Arr3& C) {
            Arr3 d(0, n, 0, m + 1, 0, l + 1);
            for (int k = 0; k <= l + 1; ++k) for (int j = 0; j <= m + 1; ++j) for (int i = 0; i <= n; ++i)
                d(i, j, k) = isoc(i + 1, j, k) * isoc(i, j, k) * (C(i + 1, j, k) - C(i, j, k)) / (dx * std::cos(Y(j)));
            return d;
        };
        auto dCdyt = [&](Arr3& C) {
            Arr3 d(0, n + 1, 0, m, 0, l + 1);
            for (int k = 0; k <= l + 1; ++k) for (int j = 0; j <= m; ++j) for (int i = 0; i <= n + 1; ++i)
                d(i, j, k) = isoc(i, j + 1, k) * isoc(i, j, k) * (C(i, j + 1, k) - C(i, j, k)) / dy;
            return d;
        };
        auto dCdzt = [&](Arr3& C) {
            Arr3 d(0, n + 1, 0, m + 1, 0, l);
            for (int k = 0; k <= l; ++k) for (int j = 0; j <= m + 1; ++j) for (int i = 0; i <= n + 1; ++i)
                d(i, j, k) = isoc(i, j, k + 1) * isoc(i, j, k) * (C(i, j, k + 1) - C(i, j, k)) / (dz * DFZW(k));
            return d;
        };
        Arr3 dtdxe = dCdxt(T), dsdxe = dCdxt(S), dtdyn = dCdyt(T), dsdyn = dCdyt(S);
        Arr3 dtdzt = dCdzt(T), dsdzt = dCdzt(S);
        Arr3 rho(0, n + 1, 0, m + 1, 0, l + 1), drhodt(0, n + 1, 0, m + 1, 0, l + 1), drhods(0, n + 1, 0, m + 1, 0, l + 1);
        for (size_t q = 0; q < rho.d.size(); ++q) {
            const double tt = T.d[q], ss = S.d[q];
            rho.d[q] = lambda * ss - tt - xes * (alpt1 * tt + alpt2 * tt * tt - alpt3 * tt * tt * tt);
            drhodt.d[q] = -1.0 - xes * (alpt1 + 2.0 * alpt2 * tt - 3.0 * alpt3 * (tt * tt));
            drhods.d[q] = lambda;
        }
        Arr3 drhodzt = dCdzt(rho);
        Arr3 Ftxe(0, n, 1, m, 1, l), Fsxe(0, n, 1, m, 1, l), Ftyn(1, n, 0, m, 1, l), Fsyn(1, n, 0, m, 1, l);
        Arr3 Ftzt(1, n, 1, m, 0, l), Fszt(1, n, 1, m, 0, l), Ftimp(1, n, 1, m, 0, l), Fsimp(1, n, 1, m, 0, l);
        const bool np_gm = piso != 0.0 || pgm != 0.0;
        auto east_face = [&](int i, int j, int k) {
            double dumt = 0.0, dums = 0.0;
            for (int kr = 0; kr <= 1; ++kr) for (int ip = 0; ip <= 1; ++ip) {
                const double drdh = drhodt(i + ip, j, k) * dtdxe(i, j, k) + drhods(i + ip, j, k) * dsdxe(i, j, k);
                const double drdz = drhodt(i + ip, j, k) * dtdzt(i + ip, j, k - 1 + kr) +
                                    drhods(i + ip, j, k) * dsdzt(i + ip, j, k - 1 + kr);
                double slp, tpr;
                tprslp(drdh, drdz, sp2, slp, tpr);
                dumt = dumt + DFZW(k - 1 + kr) * (tpr * (piso)*dtdxe(i, j, k) + tpr * (piso - pgm) * slp * dtdzt(i + ip, j, k - 1 + kr));
                dums = dums + DFZW(k - 1 + kr) * (tpr * (piso)*dsdxe(i, j, k) + tpr * (piso - pgm) * slp * dsdzt(i + ip, j, k - 1 + kr));
            }
            Ftxe(i, j, k) = Ftxe(i, j, k) - dumt / (4 * DFZT(k));
            Fsxe(i, j, k) = Fsxe(i, j, k) - dums / (4 * DFZT(k));
        };
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) {
            if (np_gm) east_face(0, j, k);
            for (int i = 1; i <= n; ++i) {
                if (np_gm) {
                    east_face(i, j, k);
                    double dumt = 0.0, dums = 0.0;   // north face
                    for (int kr = 0; kr <= 1; ++kr) for (int jq = 0; jq <= 1; ++jq) {
                        const double drdh = drhodt(i, j + jq, k) * dtdyn(i, j, k) + drhods(i, j + jq, k) * dsdyn(i, j, k);
                        const double drdz = drhodt(i, j + jq, k) * dtdzt(i, j + jq, k - 1 + kr) +
                                            drhods(i, j + jq, k) * dsdzt(i, j + jq, k - 1 + kr);
                        double slp, tpr;
                        tprslp(drdh, drdz, sp2, slp, tpr);
                        dumt = dumt + DFZW(k - 1 + kr) * std::cos(Y(j + jq)) *
                                          (tpr * (piso)*dtdyn(i, j, k) + tpr * (piso - pgm) * slp * dtdzt(i, j + jq, k - 1 + kr));
                        dums = dums + DFZW(k - 1 + kr) * std::cos(Y(j + jq)) *
                                          (tpr * (piso)*dsdyn(i, j, k) + tpr * (piso - pgm) * slp * dsdzt(i, j + jq, k - 1 + kr));
                    }
                    Ftyn(i, j, k) = Ftyn(i, j, k) - dumt / (4 * DFZT(k) * std::cos(YV(j)));
                    Fsyn(i, j, k) = Fsyn(i, j, k) - dums / (4 * DFZT(k) * std::cos(YV(j)));
                    dumt = 0.0; dums = 0.0;   // top face, zonal variations
                    for (int ip = 0; ip <= 1; ++ip) for (int kr = 0; kr <= 1; ++kr) {
                        const double drdh = drhodt(i, j, k + kr) * dtdxe(i - 1 + ip, j, k + kr) +
                                            drhods(i, j, k + kr) * dsdxe(i - 1 + ip, j, k + kr);
                        const double drdz = drhodt(i, j, k + kr) * dtdzt(i, j, k) + drhods(i, j, k + kr) * dsdzt(i, j, k);
                        double slp, tpr;
                        tprslp(drdh, drdz, sp2, slp, tpr);
                        dumt = dumt + (tpr * (piso)*slp * slp * dtdzt(i, j, k) + tpr * (piso + pgm) * slp * dtdxe(i - 1 + ip, j, k + kr));
                        dums = dums + (tpr * (piso)*slp * slp * dsdzt(i, j, k) + tpr * (piso + pgm) * slp * dsdxe(i - 1 + ip, j, k + kr));
                    }
                    Ftzt(i, j, k) = Ftzt(i, j, k) - dumt / 4;
                    Fszt(i, j, k) = Fszt(i, j, k) - dums / 4;
                    dumt = 0.0; dums = 0.0;   // top face, meridional variations
                    for (int jq = 0; jq <= 1; ++jq) for (int kr = 0; kr <= 1; ++kr) {
                        const double drdh = drhodt(i, j, k + kr) * dtdyn(i, j - 1 + jq, k + kr) +
                                            drhods(i, j, k + kr) * dsdyn(i, j - 1 + jq, k + kr);
                        const double drdz = drhodt(i, j, k + kr) * dtdzt(i, j, k) + drhods(i, j, k + kr) * dsdzt(i, j, k);
                        double slp, tpr;
                        tprslp(drdh, drdz, sp2, slp, tpr);
                        dumt = dumt + (tpr * (piso)*slp * slp * dtdzt(i, j, k) + tpr * (piso + pgm) * slp * dtdyn(i, j - 1 + jq, k + kr));
                        dums = dums + (tpr * (piso)*slp * slp * dsdzt(i, j, k) + tpr * (piso + pgm) * slp * dsdyn(i, j - 1 + jq, k + kr));
                    }
                    Ftzt(i, j, k) = Ftzt(i, j, k) - dumt / 4;
                    Fszt(i, j, k) = Fszt(i, j, k) - dums / 4;
                }
                if (eps != 0.0) {   // consistent vertical mixing
                    const double d = drhodzt(i, j, k);
                    Ftzt(i, j, k) = Ftzt(i, j, k) + tprstb(d, sp1) * eps * dtdzt(i, j, k) / (d - epsln);
                    Fszt(i, j, k) = Fszt(i, j, k) + tprstb(d, sp1) * eps * dsdzt(i, j, k) / (d - epsln);
                }
                if (kvc != 0.0) {   // implicit vertical mixing (convective adjustment)
                    Ftimp(i, j, k) = -(tprstb(-drhodzt(i, j, k), sp1) * kvc * dtdzt(i, j, k));
                    Fsimp(i, j, k) = -(tprstb(-drhodzt(i, j, k), sp1) * kvc * dsdzt(i, j, k));
                }
            }
        }
        const bool rhomix = rho_mixing != 0 && xes == 0.0;
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
            const double cy = std::cos(Y(j));
            int row = find_row2(i, j, k, TT) - 1;
            mix[row] = 0.0;
            if (vmix_temp == 1) {
                mix[row] = (Ftxe(i, j, k) - Ftxe(i - 1, j, k)) / (dx * cy) + mix[row];
                mix[row] = (Ftyn(i, j, k) * std::cos(YV(j)) - Ftyn(i, j - 1, k) * std::cos(YV(j - 1))) / (dy * cy) + mix[row];
                mix[row] = (Ftzt(i, j, k) - Ftzt(i, j, k - 1)) / (dz * DFZT(k)) + mix[row];
                if (rhomix)
                    mix[row] = ((Ftimp(i, j, k) - Ftimp(i, j, k - 1)) - (Fsimp(i, j, k) - Fsimp(i, j, k - 1)) * lambda) /
                                   (2.0 * dz * DFZT(k)) + mix[row];
                else
                    mix[row] = (Ftimp(i, j, k) - Ftimp(i, j, k - 1)) / (dz * DFZT(k)) + mix[row];
            }
            row = find_row2(i, j, k, SS) - 1;
            mix[row] = 0.0;
            if (vmix_salt == 1) {
                mix[row] = (Fsxe(i, j, k) - Fsxe(i - 1, j, k)) / (dx * cy) + mix[row];
                mix[row] = (Fsyn(i, j, k) * std::cos(YV(j)) - Fsyn(i, j - 1, k) * std::cos(YV(j - 1))) / (dy * cy) + mix[row];
                mix[row] = (Fszt(i, j, k) - Fszt(i, j, k - 1)) / (dz * DFZT(k)) + mix[row];
                if (rhomix)
                    mix[row] = ((Fsimp(i, j, k) - Fsimp(i, j, k - 1)) - (Ftimp(i, j, k) - Ftimp(i, j, k - 1)) / lambda) /
                                   (2.0 * dz * DFZT(k)) + mix[row];
                else
                    mix[row] = (Fsimp(i, j, k) - Fsimp(i, j, k - 1)) / (dz * DFZT(k)) + mix[row];
            }
        }
    }

    // vmix_jac (mix_imp.f:729-815): forward differences (eps = 1e-8) over a
    // column partition, added into An at the stencil position of each pair.
    // The partition here colours columns by (i mod 3 or i, j mod 3, k mod 3,
    // field); any partition in which no two columns of a group share a row
    // of the 27-point pattern (such as DSM's) yields the same values: each
    // row's difference then sees exactly one perturbed column of its group.
    void vmix_jac(const double* un) {
        const double eps = 1.0e-08;
        std::vector<double> mix(ndim, 0.0), mixd(ndim, 0.0), und(ndim);
        vmix_fun(un, mix.data());
        const bool wrap3 = periodic && (n % 3 != 0);
        auto group_of = [&](int i, int j, int k, int XX) {
            const int ci = wrap3 ? i : (i % 3);
            return ((ci * 3 + j % 3) * 3 + k % 3) * 2 + (XX == SS ? 1 : 0);
        };
        const int ngroups = (wrap3 ? n + 1 : 3) * 9 * 2;
        // fjac per (row cell, h, row field, column field)
        std::vector<double> fj(size_t(n) * m * l * 27 * 4, 0.0);
        auto fjx = [&](int i, int j, int k, int h, int a, int b) -> double& {
            return fj[(((cell(i, j, k) * 27 + h) * 2 + a) * 2 + b)];
        };
        for (int g = 0; g < ngroups; ++g) {
            bool any = false;
            for (int r = 0; r < ndim; ++r) und[r] = un[r];
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
                for (int XX : {TT, SS}) {
                    if ((XX == TT && !part_temp) || (XX == SS && !part_salt)) continue;
                    if (group_of(i, j, k, XX) != g) continue;
                    const int c = find_row2(i, j, k, XX) - 1;
                    und[c] = un[c] + eps;
                    any = true;
                }
            if (!any) continue;
            vmix_fun(und.data(), mixd.data());
            for (int r = 0; r < ndim; ++r) mixd[r] = mixd[r] - mix[r];
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
                if (LM(i, j, k) != OCEAN) continue;
                for (int a = 0; a < 2; ++a) {
                    if ((a == 0 && !part_temp) || (a == 1 && !part_salt)) continue;
                    const int row = find_row2(i, j, k, a == 0 ? TT : SS) - 1;
                    for (int h = 0; h < 27; ++h) {
                        const int I = i + ST[h][0], J = j + ST[h][1], K = k + ST[h][2];
                        const int kind = LM(I, J, K);
                        if (kind != OCEAN && kind != PERIO) continue;
                        const int ci = kind == PERIO ? i - ST[h][0] * (n - 1) : I;
                        for (int b = 0; b < 2; ++b) {
                            if ((b == 0 && !part_temp) || (b == 1 && !part_salt)) continue;
                            if (group_of(ci, J, K, b == 0 ? TT : SS) != g) continue;
                            fjx(i, j, k, h, a, b) = mixd[row] / eps;
                        }
                    }
                }
            }
        }
        // scatter into An(s, ie, je, ix, iy, iz)
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
            if (LM(i, j, k) != OCEAN) continue;
            for (int h = 0; h < 27; ++h) {
                const int I = i + ST[h][0], J = j + ST[h][1], K = k + ST[h][2];
                const int kind = LM(I, J, K);
                if (kind != OCEAN && kind != PERIO) continue;
                const int jx = kind == PERIO ? i - ST[h][0] * (n - 1) : I;
                int sidx = 0;
                if (K - k == -1) sidx += 9;
                if (K - k == 1) sidx += 18;
                if (jx - i == 0) sidx += 3;
                if (jx - i == 1) sidx += 6;
                if (jx - i == 1 - n) sidx += 6;
                if (J - j == -1) sidx += 1;
                if (J - j == 0) sidx += 2;
                if (J - j == 1) sidx += 3;
                for (int a = 0; a < 2; ++a) {
                    if ((a == 0 && !part_temp) || (a == 1 && !part_salt)) continue;
                    for (int b = 0; b < 2; ++b) {
                        if ((b == 0 && !part_temp) || (b == 1 && !part_salt)) continue;
                        double& an = AN(sidx, a == 0 ? TT : SS, b == 0 ? TT : SS, i, j, k);
                        an = an + fjx(i, j, k, h, a, b);
                    }
                }
            }
        }
    }

    // ---- rhs: src/ocean/usrc.F90:523-603, sign flip of THCM.C:1008-1011 ----
    void rhs(const double* un, double* F) {
        std::vector<double> mix(ndim, 0.0);
        An = Al;
        nlin_rhs(un);
        boundaries();
        fillcolA();
        std::vector<double> Au(ndim);
        matAvec(un, Au.data());
        if (vmix_flag >= 1) {   // usrc.F90:551-569
            if (vmix_fix == 0 && vmix_flag >= 2) vmix_control(un);
            if ((vmix_temp == 1 || vmix_salt == 1) && vmix_dim > 0) vmix_fun(un, mix.data());
        }
        for (int r = 0; r < ndim; ++r) {
            double B = -Au[r] - mix[r] + Frc[r] - 0.0 * (1 - par[RESC]) * 0.0;
            F[r] = B;
        }
        for (int i = 1; i <= n; ++i) for (int j = 1; j <= m; ++j) for (int k = 1; k <= l; ++k)
            for (int k1 = 1; k1 <= NUN; ++k1) {
                int row = find_row2(i, j, k, k1) - 1;
                F[row] = F[row] * double(1 - LM(i, j, k));
            }
        for (int r = 0; r < ndim; ++r) F[r] = -F[r];   // Epetra Scale(-1.0)
        if (rowintcon >= 0) {   // THCM::evaluate (THCM.C:1014-1026): intSign (c . x - correction)
            double dot = 0.0;
            for (int q = 0; q < ndim; ++q) dot += intcoef[q] * un[q];
            F[rowintcon] = sint_sign * (dot - intCorrection);
        }
        if (rowPfix1 >= 0) F[rowPfix1] = 0.0;   // THCM.C:1028-1041
        if (rowPfix2 >= 0) F[rowPfix2] = 0.0;
    }
    void assemble_rhs_matrix(const double* un) {
        An = Al;
        nlin_rhs(un);
        boundaries();
        fillcolA();
    }
    // ---- matrix: src/ocean/usrc.F90:449-521 ----
    void matrix(const double* un) {
        An = Al;
        fillcolB();
        nlin_jac(un);
        if (vmix_flag >= 1) {   // usrc.F90:488-508
            if (vmix_fix == 0 && vmix_flag >= 2) vmix_control(un);
            if ((vmix_temp == 1 || vmix_salt == 1) && vmix_dim > 0) vmix_jac(un);
        }
        boundaries();
        fillcolA();
    }

    // ---- CreateMaximalGraph: src/ocean/THCM.C:2300-2580 (SRES = 1 path) ----
    void build_graph() {
        g_ptr.assign(ndim + 1, 0);
        g_col.clear();
        const int N = n, M = m, L = l;
        auto fr = [&](int i, int j, int k, int xx) { return NUN * (k * N * M + N * j + i) + xx - 1; };
        std::vector<int> idx;
        auto ins = [&](int i, int j, int k, int xx) {
            int ii = i;
            if (periodic) ii = ((i % N) + N) % N;
            if (ii >= 0 && j >= 0 && k >= 0 && ii < N && j < M && k < L) idx.push_back(fr(ii, j, k, xx));
        };
        std::vector<std::vector<int>> rows(ndim);
        for (int k = 0; k < L; ++k) for (int j = 0; j < M; ++j) for (int i = 0; i < N; ++i) {
            int g0 = fr(i, j, k, UU) - 0;   // row of UU (0-based)
            idx.clear();
            ins(i, j, k, UU); ins(i - 1, j, k, UU); ins(i + 1, j, k, UU); ins(i, j - 1, k, UU); ins(i, j + 1, k, UU);
            ins(i, j, k - 1, UU); ins(i, j, k + 1, UU);
            ins(i, j, k, VV); ins(i - 1, j, k, VV); ins(i + 1, j, k, VV); ins(i, j - 1, k, VV); ins(i, j + 1, k, VV);
            ins(i, j, k, WW); ins(i + 1, j, k, WW); ins(i + 1, j + 1, k, WW); ins(i, j + 1, k, WW);
            ins(i, j, k - 1, WW); ins(i + 1, j, k - 1, WW); ins(i + 1, j + 1, k - 1, WW); ins(i, j + 1, k - 1, WW);
            ins(i, j, k, PP); ins(i + 1, j, k, PP); ins(i, j + 1, k, PP); ins(i + 1, j + 1, k, PP);
            rows[g0 + 0] = idx;
            idx.clear();
            ins(i, j, k, VV); ins(i - 1, j, k, VV); ins(i + 1, j, k, VV); ins(i, j - 1, k, VV); ins(i, j + 1, k, VV);
            ins(i, j, k - 1, VV); ins(i, j, k + 1, VV);
            ins(i, j, k, UU); ins(i - 1, j, k, UU); ins(i + 1, j, k, UU);
            ins(i, j, k, WW); ins(i + 1, j, k, WW); ins(i + 1, j + 1, k, WW); ins(i, j + 1, k, WW);
            ins(i, j, k - 1, WW); ins(i + 1, j, k - 1, WW); ins(i + 1, j + 1, k - 1, WW); ins(i, j + 1, k - 1, WW);
            ins(i, j, k, PP); ins(i + 1, j, k, PP); ins(i, j + 1, k, PP); ins(i + 1, j + 1, k, PP);
            rows[g0 + 1] = idx;
            idx.clear();
            ins(i, j, k, WW); ins(i, j, k, PP); ins(i, j, k + 1, PP); ins(i, j, k, TT); ins(i, j, k + 1, TT);
            ins(i, j, k, SS); ins(i, j, k + 1, SS);
            rows[g0 + 2] = idx;
            idx.clear();
            ins(i, j, k, PP);
            ins(i, j, k, UU); ins(i - 1, j, k, UU); ins(i, j - 1, k, UU); ins(i - 1, j - 1, k, UU);
            ins(i, j, k, VV); ins(i - 1, j, k, VV); ins(i, j - 1, k, VV); ins(i - 1, j - 1, k, VV);
            ins(i, j, k, WW); ins(i, j, k - 1, WW);
            rows[g0 + 3] = idx;
            for (int q = 0; q < 2; ++q) {
                int A = q == 0 ? TT : SS, O = q == 0 ? SS : TT;
                idx.clear();
                ins(i, j, k, A); ins(i - 1, j, k, A); ins(i + 1, j, k, A); ins(i, j - 1, k, A); ins(i, j + 1, k, A);
                ins(i, j, k - 1, A); ins(i, j, k + 1, A);
                ins(i, j, k, UU); ins(i - 1, j, k, UU); ins(i - 1, j - 1, k, UU); ins(i, j - 1, k, UU);
                ins(i, j, k, VV); ins(i - 1, j, k, VV); ins(i - 1, j - 1, k, VV); ins(i, j - 1, k, VV);
                ins(i, j, k, WW); ins(i, j, k - 1, WW);
                ins(i, j, k, O); ins(i, j, k - 1, O); ins(i, j, k + 1, O);
                rows[g0 + 4 + q] = idx;
            }
        }
        if (rowintcon >= 0) {   // CreateMaximalGraph(useSRES) with SRES = 0 (THCM.C:2542-2577)
            auto& rr = rows[rowintcon];
            rr.clear();
            for (int k = 0; k < L; ++k) for (int j = 0; j < M; ++j) for (int i = 0; i < N; ++i) rr.push_back(fr(i, j, k, SS));
        }
        for (int r = 0; r < ndim; ++r) {
            auto& rr = rows[r];
            std::sort(rr.begin(), rr.end());
            rr.erase(std::unique(rr.begin(), rr.end()), rr.end());   // Epetra merges duplicates
            g_ptr[r + 1] = g_ptr[r] + int(rr.size());
            g_col.insert(g_col.end(), rr.begin(), rr.end());
        }
    }
    // Scatter of THCM::evaluate (src/ocean/THCM.C:1082-1162): ReplaceGlobalValues
    // into the zeroed maximal-graph matrix, entry by entry in Fortran order.
    int scatter(double* values) const {
        std::fill(values, values + g_col.size(), 0.0);
        int excluded = 0;
        for (int r = 0; r < ndim; ++r) {
            const int* b = g_col.data() + g_ptr[r];
            const int* e = g_col.data() + g_ptr[r + 1];
            if (r == rowintcon) {   // intcond_S replaces the row (THCM.C:1085, 2191-2230)
                for (int q = g_ptr[r]; q < g_ptr[r + 1]; ++q) values[q] = sint_sign * intcoef[g_col[q]];
                continue;
            }
            for (int q = begA[r]; q < begA[r + 1]; ++q) {
                int col = jcoA[q - 1] - 1;
                const int* f = std::lower_bound(b, e, col);
                if (f != e && *f == col) values[g_ptr[r] + (f - b)] = coA[q - 1];
                else ++excluded;
            }
        }
        for (int r : {rowPfix1, rowPfix2}) {   // fixPressurePoints: identity rows
            if (r < 0) continue;
            for (int q = g_ptr[r]; q < g_ptr[r + 1]; ++q) values[q] = g_col[q] == r ? 1.0 : 0.0;
        }
        return excluded;
    }

    // ---- compute_psim: src/ocean/thcm_utils.F90:95-118, OceanGrid.C:270-330 ----
    void psim(const double* un, double* out) {
        usol(un);
        std::vector<double> vs((m + 1) * l);
        for (int k = 1; k <= l; ++k) for (int j = 0; j <= m; ++j) {
            double sum = 0.0;
            for (int i = 1; i <= n; ++i) sum += v(i, j, k);
            vs[(m + 1) * (k - 1) + j] = sum * dx;
        }
        std::fill(out, out + (m + 1) * (l + 1), 0.0);
        for (int j = 1; j <= m; ++j) {
            double cs = std::cos(YV(j));
            for (int k = 1; k <= l; ++k)
                if (Z(k) * hdim < -500)
                    out[(m + 1) * k + j] = -cs * vs[(m + 1) * (k - 1) + j] * dz * DFZT(k) + out[(m + 1) * (k - 1) + j];
        }
    }

    // ---- init: src/ocean/usrc.F90:6-139 ----
    void init(const iemic_oracle_config& c, const int* lm) {
        n = c.n; m = c.m; l = c.l; ndim = n * m * l * NUN;
        periodic = c.periodic != 0;
        xmin = c.xmin_deg * PI / 180.0; xmax = c.xmax_deg * PI / 180.0;
        ymin = c.ymin_deg * PI / 180.0; ymax = c.ymax_deg * PI / 180.0;
        hdim = c.hdim; qz = c.qz; alphaT = c.alphaT; alphaS = c.alphaS;
        ih = c.ih; coriolis_on = c.coriolis_on; TRES = c.tres; SRES = c.sres;
        iza = c.iza; ite = c.ite; its = c.its; forcing_type = c.forcing_type;
        vmix = c.vmix; rho_mixing = c.rho_mixing; tap = c.tap;
        landm.assign(size_t(n + 2) * (m + 2) * (l + 2), OCEAN);
        if (lm) {
            for (size_t q = 0; q < landm.size(); ++q) landm[q] = lm[q];
        } else {   // Topography = 1: no continents (src/ocean/topo.F90 depth3land case 1)
            std::fill(landm.begin(), landm.end(), LAND);
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) LM(i, j, k) = OCEAN;
        }
        for (int k = 0; k <= l + 1; ++k) for (int j = 0; j <= m + 1; ++j) for (int i = 0; i <= n + 1; ++i)
            if (!periodic && LM(i, j, k) == PERIO) LM(i, j, k) = OCEAN;
        if (!periodic)
            for (int k = 0; k <= l + 1; ++k) for (int j = 0; j <= m + 1; ++j) { LM(0, j, k) = LAND; LM(n + 1, j, k) = LAND; }
        for (int k = 0; k <= l + 1; ++k) for (int i = 0; i <= n + 1; ++i) { LM(i, 0, k) = LAND; LM(i, m + 1, k) = LAND; }
        for (int j = 0; j <= m + 1; ++j) for (int i = 0; i <= n + 1; ++i) { LM(i, j, 0) = LAND; LM(i, j, l + 1) = LAND; }
        size_t nm = size_t(n) * m;
        taux.assign(nm, 0); tauy.assign(nm, 0); tatm.assign(nm, 0); emip.assign(nm, 0);
        spert.assign(nm, double(SRES)); adapted_emip.assign(nm, 0);
        internal_temp.assign(nm * l, 0); internal_salt.assign(nm * l, 0);
        Frc.assign(ndim, 0.0);
        Al.assign(size_t(NP) * NUN * NUN * n * m * l, 0.0);
        An = Al;
        grid();
        double dzne = dz * DFZT(l);
        QTnd = r0dim / (udim * cp0 * rhodim * hdim * dzne);
        QSnd = s0 * r0dim / (deltas * udim * hdim * dzne);
        if (SRES == 0) {   // location of the integral condition (THCM.C:651-697)
            const int Nic = c.intcon_i >= 0 ? c.intcon_i : n - 1, Mic = c.intcon_j >= 0 ? c.intcon_j : m - 1;
            if (Nic >= n || Mic >= m || LM(Nic + 1, Mic + 1, l) != OCEAN) throw 1;
            rowintcon = NUN * ((l - 1) * n * m + n * Mic + Nic) + SS - 1;
            sint_sign = c.sint_sign == 0 ? -1 : c.sint_sign;
            intcoef.assign(ndim, 0.0);   // intcond_scaling (thcm_utils.F90:285-312)
            for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
                if (LM(i, j, k) == OCEAN) intcoef[find_row2(i, j, k, SS) - 1] = std::cos(Y(j)) * DFZT(k);
        }
        if (c.fix_pressure_points) {   // THCM.C:749-758
            rowPfix1 = NUN * ((l - 1) * n * m + n * (m - 1) + (n - 1)) + PP - 1;
            rowPfix2 = NUN * ((l - 1) * n * m + n * (m - 1) + (n - 2)) + PP - 1;
        }
        stpnt();
        forcing();
        lin();
        vmix_init();   // usrc.F90:133
        build_graph();
    }
};

}  // namespace

extern "C" {

void* oracle_create(const iemic_oracle_config* cfg, const int* landm) {
    Model* M = new Model();
    try {
        M->init(*cfg, landm);
    } catch (...) {   // the integral-condition row is on land (THCM.C:671-690)
        delete M;
        return nullptr;
    }
    return M;
}
void oracle_destroy(void* h) { delete static_cast<Model*>(h); }
int oracle_ndim(void* h) { return static_cast<Model*>(h)->ndim; }
void oracle_get_landm(void* h, int* out) {
    Model* M = static_cast<Model*>(h);
    std::copy(M->landm.begin(), M->landm.end(), out);
}
void oracle_set_forcing(void* h, const double* taux, const double* tauy, const double* tatm,
                        const double* emip, const double* spert) {
    Model* M = static_cast<Model*>(h);
    size_t nm = size_t(M->n) * M->m;
    if (taux) std::copy(taux, taux + nm, M->taux.begin());
    if (tauy) std::copy(tauy, tauy + nm, M->tauy.begin());
    if (tatm) std::copy(tatm, tatm + nm, M->tatm.begin());
    if (emip) std::copy(emip, emip + nm, M->emip.begin());
    if (spert) std::copy(spert, spert + nm, M->spert.begin());
    M->forcing();
    M->lin();
}
void oracle_set_par(void* h, int idx, double value) {
    Model* M = static_cast<Model*>(h);
    if (idx >= 1 && idx <= NPAR) M->par[idx] = value;
    M->forcing();
    M->lin();
}
double oracle_get_par(void* h, int idx) {
    Model* M = static_cast<Model*>(h);
    return (idx >= 1 && idx <= NPAR) ? M->par[idx] : 0.0;
}
void oracle_get_frc(void* h, double* out) {
    Model* M = static_cast<Model*>(h);
    std::copy(M->Frc.begin(), M->Frc.end(), out);
}
void oracle_get_grid(void* h, double* x, double* y, double* xu, double* yv, double* z, double* zw,
                     double* dfzT, double* dfzW) {
    Model* M = static_cast<Model*>(h);
    std::copy(M->x.begin(), M->x.end(), x);
    std::copy(M->y.begin(), M->y.end(), y);
    std::copy(M->xu.begin(), M->xu.end(), xu);
    std::copy(M->yv.begin(), M->yv.end(), yv);
    std::copy(M->z.begin(), M->z.end(), z);
    std::copy(M->zw.begin(), M->zw.end(), zw);
    std::copy(M->dfzT.begin(), M->dfzT.end(), dfzT);
    std::copy(M->dfzW.begin(), M->dfzW.end(), dfzW);
}
void oracle_rhs(void* h, const double* x, double* F) {
    Model* M = static_cast<Model*>(h);
    if (M->vmix == 2) M->vmix_fix = 0;   // Ocean::computeRHS -> THCM::fixMixing(0) (Ocean.C:1281; THCM.C:2640-2647)
    // forcing() is re-run because boundaries() zeroes Frc entries in place,
    // exactly like the reference, where Frc persists across calls.
    M->rhs(x, F);
}
int oracle_fortran_nnz(void* h) { return int(static_cast<Model*>(h)->coA.size()); }
void oracle_fortran_csr(void* h, int* beg, int* jco, double* co) {
    Model* M = static_cast<Model*>(h);
    std::copy(M->begA.begin(), M->begA.end(), beg);
    std::copy(M->jcoA.begin(), M->jcoA.end(), jco);
    std::copy(M->coA.begin(), M->coA.end(), co);
}
void oracle_assemble_rhs_matrix(void* h, const double* x) { static_cast<Model*>(h)->assemble_rhs_matrix(x); }
int64_t oracle_graph_nnz(void* h) { return int64_t(static_cast<Model*>(h)->g_col.size()); }
void oracle_graph(void* h, int* row_ptr, int* col_idx) {
    Model* M = static_cast<Model*>(h);
    std::copy(M->g_ptr.begin(), M->g_ptr.end(), row_ptr);
    std::copy(M->g_col.begin(), M->g_col.end(), col_idx);
}
int oracle_jacobian(void* h, const double* x, double* values) {
    Model* M = static_cast<Model*>(h);
    if (M->vmix == 2) M->vmix_fix = 0;   // Ocean::computeJacobian -> THCM::fixMixing(0) (Ocean.C:1302)
    M->matrix(x);
    return M->scatter(values);
}
void oracle_mass(void* h, double* diagB) {
    Model* M = static_cast<Model*>(h);
    M->fillcolB();
    std::copy(M->coB.begin(), M->coB.end(), diagB);
}
void oracle_psim(void* h, const double* x, double* psim) { static_cast<Model*>(h)->psim(x, psim); }
double oracle_An(void* h, int kk, int A, int B, int i, int j, int k) {
    return static_cast<Model*>(h)->AN(kk, A, B, i, j, k);
}

}  // extern "C"
