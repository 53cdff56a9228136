// Handle, set-up and C ABI of the THCM engine (host side).
//
// Set-up mirrors the reference's initialisation chain THCM::THCM ->
// Fortran init (src/ocean/usrc.F90:6-139): land-mask fix-ups, grid
// (src/ocean/grid.F90), stpnt (usrc.F90:1153-1197), forcing
// (src/ocean/forcing.F90), lin (usrc.F90:605-789), and the maximal graph of
// src/ocean/THCM.C:2300-2580. Geometry-only metric tables are evaluated here
// with the host libm exactly as the Fortran atoms evaluate them; everything
// that depends on the state or on the parameters runs on the GPU.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/iemic_gb300.h"
#include "engine.cuh"

using namespace iemic;

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double omegadim = 7.292e-05, r0dim = 6.37e+06, udim = 0.1e+00, gdim = 9.8e+00,
                 rhodim = 1.024e+03, av = 1.0e-03, ah = 2.5e+05, kappah = 1.0e+03, kappav = 1.0e-04;

double amh(double y, int ih) { return ih == 0 ? 1.0 : 1. + 10.0 * std::exp(-5 * y * y); }
double bmh(double y, int ih) { return ih == 0 ? 1.0 : 1.0 + 10.0 * std::exp(-5 * y * y); }
double bmhy(double y, int ih) { return ih == 0 ? 0.0 : -10. * 10.0 * y * std::exp(-5 * y * y); }
double fz(double z, double q) {
    double th = std::tanh(q * (z + 1)), tth = std::tanh(q);
    if (q > 1.0) return -1 + th / tth;
    return z + (1. - q) * z * (1 - z);
}
double dfdz(double z, double q) {
    double ch = std::cosh(q * (z + 1)), tth = std::tanh(q);
    if (q > 1.0) return q / (tth * ch * ch);
    return 1.0 + (1. - q) * (1. - 2. * z);
}

}  // namespace

// ---------------------------------------------------------------------------
// grid + geometry tables
// ---------------------------------------------------------------------------
void Engine::build_grid() {
    const int n = cfg.n, m = cfg.m, l = cfg.l;
    xmin = cfg.xmin_deg * PI / 180.0; xmax = cfg.xmax_deg * PI / 180.0;
    ymin = cfg.ymin_deg * PI / 180.0; ymax = cfg.ymax_deg * PI / 180.0;
    dx = (xmax - xmin) / n;
    dy = (ymax - ymin) / m;
    dz = (0.0 - (-1.0)) / l;
    y.assign(m + 2, 0.0); yv.assign(m + 1, 0.0);
    z.assign(l + 1, 0.0); dfzT.assign(l + 1, 0.0); dfzW.assign(l + 1, 0.0);
    for (int j = 1; j <= m; ++j) {
        y[j] = (double(j) - 0.5) * dy + ymin;
        yv[j] = (double(j)) * dy + ymin;
    }
    y[0] = y[1] - dy;
    y[m + 1] = y[m] + dy;
    yv[0] = ymin;
    for (int k = 1; k <= l; ++k) {
        double ze = (double(k) - 0.5) * dz + (-1.0);
        double zwe = (double(k)) * dz + (-1.0);
        z[k] = fz(ze, cfg.qz);
        dfzT[k] = dfdz(ze, cfg.qz);
        dfzW[k] = dfdz(zwe, cfg.qz);
    }
    dfzW[0] = dfdz(-1.0, cfg.qz);

    const int ih = cfg.ih;
    jt.assign(size_t(NJT) * (m + 2), 0.0);
    kt.assign(size_t(NKT) * (l + 2), 0.0);
    auto J = [&](int t, int j) -> double& { return jt[size_t(t) * (m + 2) + j]; };
    auto K = [&](int t, int k) -> double& { return kt[size_t(t) * (l + 2) + k]; };
    const double rdy2 = (1.0 / dy) * (1.0 / dy);
    for (int j = 1; j <= m - 1; ++j) {   // spf.F90 u/vderiv, coriolis, gradp 1/2 (j = 1..m-1)
        double yy = yv[j];
        double t = 1.0 / (std::cos(yy) * dx), cosdx2i = t * t;
        J(JT_UXX, j) = amh(yy, ih) * cosdx2i;
        J(JT_UYY4, j) = rdy2 * bmh(y[j], ih) * std::cos(y[j]) / std::cos(yy);
        J(JT_UYY6, j) = rdy2 * bmh(y[j + 1], ih) * std::cos(y[j + 1]) / std::cos(yy);
        double tv = std::tan(yy);
        double tand2 = 1 - tv * tv;
        J(JT_UCSI, j) = bmh(yy, ih) * tand2 + std::tan(yy) * bmhy(yy, ih);
        double num = bmhy(yy, ih) - (amh(yy, ih) + bmh(yy, ih)) * tv;
        J(JT_UXS2, j) = num / (dx * std::cos(yy));
        J(JT_UXS8, j) = -(num / (dx * std::cos(yy)));
        J(JT_CORV, j) = std::sin(yy) * cfg.coriolis_on;
        J(JT_PXC, j) = 1. / (2 * std::cos(yy) * dx);
        J(JT_VXX, j) = bmh(yy, ih) * cosdx2i;
        J(JT_VXX5, j) = -(2 * bmh(yy, ih) * cosdx2i);
        J(JT_VYY4, j) = rdy2 * amh(y[j], ih) * std::cos(y[j]) / std::cos(yy);
        J(JT_VYY6, j) = rdy2 * amh(y[j + 1], ih) * std::cos(y[j + 1]) / std::cos(yy);
        J(JT_VCSI, j) = bmh(yy, ih) - amh(yy, ih) * tv * tv + bmhy(yy, ih) * tv;
        double num2 = (amh(yy, ih) + bmh(yy, ih)) * tv - bmhy(yy, ih);
        J(JT_VXS2, j) = -(num2 / (dx * std::cos(yy)));
        J(JT_VXS8, j) = num2 / (dx * std::cos(yy));
        J(JT_PYC, j) = 1. / (2 * dy);
    }
    for (int j = 1; j <= m; ++j) {   // pderiv 1/2, tderiv 3/4 (j = 1..m)
        J(JT_UXC, j) = 1.0 / (2 * std::cos(y[j]) * dx);
        double c = 1. / (2 * std::cos(y[j]) * dy);
        J(JT_VYC4, j) = -(std::cos(yv[j - 1]) * c);
        J(JT_VYC2, j) = std::cos(yv[j]) * c;
        double t = 1.0 / (std::cos(y[j]) * dx);
        J(JT_TXX, j) = t * t;
        J(JT_TYY4, j) = rdy2 * std::cos(yv[j - 1]) / std::cos(y[j]);
        J(JT_TYY6, j) = rdy2 * std::cos(yv[j]) / std::cos(y[j]);
    }
    for (int j = 0; j <= m; ++j) {   // unlin/vnlin metric factors on yv(0:m)
        J(JT_CUX, j) = 1.0 / (2 * std::cos(yv[j]) * dx);
        J(JT_CUY, j) = 1.0 / (2 * std::cos(yv[j]) * dy);
        J(JT_COSYV, j) = std::cos(yv[j]);
        J(JT_TANYV, j) = std::tan(yv[j]);
    }
    for (int j = 0; j <= m + 1; ++j) {   // tnlin metric factors on y(0:m+1)
        J(JT_CTX, j) = 1.0 / (4 * std::cos(y[j]) * dx);
        J(JT_CTY, j) = 1.0 / (4 * std::cos(y[j]) * dy);
        J(JT_COSY, j) = std::cos(y[j]);
    }
    const double rdz2 = (1.0 / dz) * (1.0 / dz), dzi = 1.0 / dz;
    for (int k = 1; k <= l; ++k) {
        double h1 = 1. / (dfzT[k] * dfzW[k]);
        double h2 = 1. / (dfzT[k] * dfzW[k - 1]);
        K(KT_UZZ14, k) = h2 * rdz2;
        K(KT_UZZ23, k) = h1 * rdz2;
        K(KT_PZ5, k) = -(dzi / dfzW[k]);
        K(KT_PZ23, k) = dzi / dfzW[k];
        K(KT_WZC5, k) = dzi / dfzT[k];
        K(KT_WZC14, k) = -(dzi / dfzT[k]);
        K(KT_TZZ14, k) = h2 * rdz2;
        K(KT_TZZ23, k) = (k < l) ? h1 * rdz2 : 0.0;
        K(KT_TDZ8, k) = 1.0 / (8 * dfzT[k] * dz);
        K(KT_DFZT, k) = dfzT[k];
        K(KT_ZHDIM, k) = z[k] * cfg.hdim;
    }
    for (int k = 0; k <= l; ++k) K(KT_DFZW, k) = dfzW[k];
    tdzi2 = 1.0 / (2 * dz);
}

// stpnt (src/ocean/usrc.F90:1153-1197); vmix_par (src/ocean/mix_imp.f:113-128)
// clears MIXP, P_VC, MKAP only for Mixing = 0
void Engine::stpnt() {
    double* p = P.par;
    for (int i = 0; i <= NPAR; ++i) p[i] = 0.0;
    const double hdim = cfg.hdim;
    p[AL_T] = 0.1 / (2 * omegadim * rhodim * hdim * udim * dz * dfzT[cfg.l]);
    p[RAYL] = cfg.alphaT * gdim * hdim / (2 * omegadim * udim * r0dim);
    p[EK_V] = av / (2 * omegadim * hdim * hdim);
    p[EK_H] = ah / (2 * omegadim * r0dim * r0dim);
    p[ROSB] = udim / (2 * omegadim * r0dim);
    p[PE_H] = kappah / (udim * r0dim);
    p[PE_V] = kappav * r0dim / (udim * hdim * hdim);
    p[LAMB] = cfg.alphaS / cfg.alphaT;
    p[BIOT] = r0dim / (75. * 3600. * 24. * udim);
    p[ALPC] = 1.0;
    p[ENER] = 1.0e+02;
    p[SPL1] = 2.0e+03;
    p[SPL2] = 0.01;
    if (cfg.vmix != 0) p[P_VC] = 2.5e+04 * p[PE_V];
    P.TRES = cfg.tres;
    P.SRES = cfg.sres;
}

// forcing fields and scalars (src/ocean/forcing.F90:4-218, 405-449)
void Engine::update_forcing() {
    const int n = cfg.n, m = cfg.m, l = cfg.l;
    const double* p = P.par;
    const size_t nm = size_t(n) * m;
    auto LMs = [&](int i, int j) { return landm[i + (n + 2) * (j + (m + 2) * l)]; };
    if (cfg.iza == 2) {   // Bryan (1987) idealized wind, wfun
        for (int j = 1; j <= m; ++j) {
            double yy = yv[j];
            double tx = 0.2 - 0.8 * std::sin(6 * std::fabs(yy)) - 0.5 * (1 - std::tanh(10 * std::fabs(yy))) -
                        0.5 * (1 - std::tanh(10 * (PI / 2 - std::fabs(yy))));
            for (int i = 1; i <= n; ++i) {
                surf[0 * nm + (i - 1) + size_t(n) * (j - 1)] = tx;
                surf[1 * nm + (i - 1) + size_t(n) * (j - 1)] = 0.0;
            }
        }
    }
    if (cfg.ite == 1) {   // temfun
        for (int j = 1; j <= m; ++j) {
            double yy = y[j];
            double v = cfg.forcing_type == 2 ? std::cos(PI * (yy - ymin) / (ymax - ymin))
                                             : std::cos(PI * yy / ymax) + p[CMPR] * std::sin(PI * yy / ymax);
            for (int i = 1; i <= n; ++i) surf[2 * nm + (i - 1) + size_t(n) * (j - 1)] = v;
        }
    }
    if (cfg.its == 1) {   // salfun * (1 - landm(i,j,l))
        for (int j = 1; j <= m; ++j) {
            double yy = y[j], v;
            if (cfg.forcing_type == 2) v = std::cos(PI * (yy - ymin) / (ymax - ymin));
            else if (cfg.forcing_type == 1) v = (std::cos(PI * yy / ymax) + p[FPER] * yy / ymax) / std::cos(yy);
            else v = std::cos(PI * yy / ymax) + p[FPER] * yy / ymax;
            for (int i = 1; i <= n; ++i)
                surf[3 * nm + (i - 1) + size_t(n) * (j - 1)] = v * double(1 - LMs(i, j));
        }
    }
    fs.sigma = p[COMB] * p[WIND] * p[AL_T];
    fs.etabi = p[COMB] * p[TEMP] * (double(1 - cfg.tres) + cfg.tres * p[BIOT]);
    fs.gamma = p[COMB] * p[SALT] * (double(1 - cfg.sres) + cfg.sres * p[BIOT]);
    fs.hmtp = p[HMTP];
    fs.sper_fac = p[SPER] * (double(1 - cfg.sres) + cfg.sres * p[BIOT]);
    fs.temcor = fs.salcor = fs.adapted_salcor = fs.spertcor = 0.0;
    // qint (src/ocean/forcing.F90:452-464, THCM.C:2653-2686): with no
    // restoring the area mean of the surface flux is removed
    auto qint = [&](int f) {
        double lfsint = 0.0, lsint = 0.0;
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n; ++i) {
                const int lmv = LMs(i + 1, j + 1);
                lfsint = surf[size_t(f) * nm + size_t(i) + size_t(n) * j] * std::cos(y[j + 1]) * double(1 - lmv) + lfsint;
                lsint = std::cos(y[j + 1]) * double(1 - lmv) + lsint;
            }
        return lfsint / lsint;
    };
    if (cfg.ite == 1 && cfg.tres == 0) fs.temcor = qint(2);
    if (cfg.sres == 0) {
        if (cfg.its == 1) fs.salcor = qint(3);
        fs.adapted_salcor = 0.0;   // adapted_emip is zero here: its mean is zero
        fs.spertcor = qint(4);
    }
    ck(cudaMemcpyAsync(d_surf, surf.data(), sizeof(double) * surf.size(), cudaMemcpyHostToDevice, stream));
}

void Engine::lin() { launch_lin(geo, P, d_al, stream); }

// Slot tables of the maximal graph: each boundary class of cells shares the
// same sorted order of its row entries.
void Engine::build_pattern() {
    const int n = cfg.n, m = cfg.m, l = cfg.l;
    slot.assign(size_t(NCLASS) * CELL_ENTRIES, int8_t(-1));
    std::vector<int> len(size_t(NCLASS) * 7, 0);
    auto rep = [](int cls_bits, int N) { return (cls_bits & 1) ? 0 : ((cls_bits & 2) ? N - 1 : 1); };
    for (int cls = 0; cls < NCLASS; ++cls) {
        int ic = cls & 3, jc = (cls >> 2) & 3, kc = (cls >> 4) & 3;
        int i = rep(ic, n), j = rep(jc, m), k = rep(kc, l);
        if (i >= n || j >= m || k >= l) continue;
        if (cell_class(i, j, k, n, m, l) != cls) continue;   // class not realised by this grid
        for (int A = 1; A <= 6; ++A) {
            std::vector<std::pair<long, int>> cols;
            for (int e = 0; e < rowlen(A); ++e) {
                Ent en = entry(A, e);
                int ii = i + di_of(en.kk), jj = j + dj_of(en.kk), k2 = k + dk_of(en.kk);
                if (cfg.periodic) ii = (ii + n) % n;
                if (ii < 0 || ii >= n || jj < 0 || jj >= m || k2 < 0 || k2 >= l) continue;
                long col = long(NUN) * (ii + long(n) * (jj + long(m) * k2)) + en.B - 1;
                cols.push_back({col, e});
            }
            std::sort(cols.begin(), cols.end());
            for (size_t q = 0; q < cols.size(); ++q) slot[size_t(cls) * CELL_ENTRIES + rowoff(A) + cols[q].second] = int8_t(q);
            len[size_t(cls) * 7 + A] = int(cols.size());
        }
    }
    row_ptr.assign(size_t(ndim) + 1, 0);
    for (int k = 0; k < l; ++k)
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n; ++i) {
                int cls = cell_class(i, j, k, n, m, l);
                size_t r0 = size_t(NUN) * (i + size_t(n) * (j + size_t(m) * k));
                for (int A = 1; A <= 6; ++A) row_ptr[r0 + A] = len[size_t(cls) * 7 + A];
            }
    if (rowintcon >= 0) row_ptr[size_t(rowintcon) + 1] = int(nc);   // the dense integral-condition row
    for (size_t r = 0; r < size_t(ndim); ++r) row_ptr[r + 1] += row_ptr[r];
    nnz = row_ptr[ndim];
}

Engine::~Engine() {
    free_solver();
    for (void* p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
}

void* Engine::dalloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) throw EngineError(IEMIC_ERR_NOMEM);
    allocs.push_back(p);
    return p;
}

void Engine::init(const iemic_config& c, const int* lm_in) {
    cfg = c;
    const int n = c.n, m = c.m, l = c.l;
    nc = size_t(n) * m * l;
    ndim = int(NUN * nc);
    ck(cudaGetDevice(&device));
    ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    // land mask as src/ocean/usrc.F90:79-107 leaves it
    const size_t nl = size_t(n + 2) * (m + 2) * (l + 2);
    landm.assign(nl, OCEAN);
    auto LM = [&](int i, int j, int k) -> int& { return landm[i + (n + 2) * (j + (m + 2) * k)]; };
    if (lm_in) {
        for (size_t q = 0; q < nl; ++q) landm[q] = lm_in[q];
    } else {   // "Topography" = 1: no continents
        std::fill(landm.begin(), landm.end(), LAND);
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) LM(i, j, k) = OCEAN;
    }
    for (size_t q = 0; q < nl; ++q)
        if (!c.periodic && landm[q] == PERIO) landm[q] = OCEAN;
    if (!c.periodic)
        for (int k = 0; k <= l + 1; ++k) for (int j = 0; j <= m + 1; ++j) { LM(0, j, k) = LAND; LM(n + 1, j, k) = LAND; }
    for (int k = 0; k <= l + 1; ++k) for (int i = 0; i <= n + 1; ++i) { LM(i, 0, k) = LAND; LM(i, m + 1, k) = LAND; }
    for (int j = 0; j <= m + 1; ++j) for (int i = 0; i <= n + 1; ++i) { LM(i, j, 0) = LAND; LM(i, j, l + 1) = LAND; }
    for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i) {
        int v = LM(i, j, k);
        if (v != OCEAN && v != LAND) throw EngineError(IEMIC_ERR_ARG);
    }
    build_grid();
    if (c.sres == 0) {   // location of the integral condition (THCM.C:651-697)
        const int Nic = c.intcon_i >= 0 ? c.intcon_i : n - 1, Mic = c.intcon_j >= 0 ? c.intcon_j : m - 1;
        if (Nic >= n || Mic >= m || LM(Nic + 1, Mic + 1, l) != OCEAN) throw EngineError(IEMIC_ERR_ARG);
        rowintcon = NUN * ((l - 1) * n * m + n * Mic + Nic) + SS - 1;
        sint_sign = c.sint_sign == 0 ? -1 : c.sint_sign;
    }
    if (c.fix_pressure_points) {   // THCM.C:749-758
        rowPfix1 = NUN * ((l - 1) * n * m + n * (m - 1) + (n - 1)) + PP - 1;
        rowPfix2 = NUN * ((l - 1) * n * m + n * (m - 1) + (n - 2)) + PP - 1;
    }
    stpnt();
    // device data
    std::vector<int8_t> lm8(nl);
    for (size_t q = 0; q < nl; ++q) lm8[q] = int8_t(landm[q]);
    d_lm = static_cast<int8_t*>(dalloc(nl));
    d_jt = static_cast<double*>(dalloc(sizeof(double) * jt.size()));
    d_kt = static_cast<double*>(dalloc(sizeof(double) * kt.size()));
    ck(cudaMemcpyAsync(d_lm, lm8.data(), nl, cudaMemcpyHostToDevice, stream));
    ck(cudaMemcpyAsync(d_jt, jt.data(), sizeof(double) * jt.size(), cudaMemcpyHostToDevice, stream));
    ck(cudaMemcpyAsync(d_kt, kt.data(), sizeof(double) * kt.size(), cudaMemcpyHostToDevice, stream));
    geo.n = n; geo.m = m; geo.l = l; geo.periodic = c.periodic ? 1 : 0;
    geo.lm = d_lm; geo.jt = d_jt; geo.kt = d_kt;
    geo.tdzi2 = tdzi2; geo.dx = dx; geo.dz = dz;
    d_al = static_cast<double*>(dalloc(sizeof(double) * size_t(m) * l * 2 * CELL_ENTRIES));
    d_pads = static_cast<double*>(dalloc(sizeof(double) * 5 * geo.npad()));
    surf.assign(5 * size_t(n) * m, 0.0);
    for (size_t q = 4 * size_t(n) * m; q < surf.size(); ++q) surf[q] = double(c.sres);   // get_spert default
    d_surf = static_cast<double*>(dalloc(sizeof(double) * surf.size()));
    d_x = static_cast<double*>(dalloc(sizeof(double) * ndim));
    d_F = static_cast<double*>(dalloc(sizeof(double) * ndim));
    d_v1 = static_cast<double*>(dalloc(sizeof(double) * ndim));
    d_v2 = static_cast<double*>(dalloc(sizeof(double) * ndim));
    d_B = static_cast<double*>(dalloc(sizeof(double) * ndim));
    // pattern
    build_pattern();
    d_rowptr = static_cast<int*>(dalloc(sizeof(int) * (size_t(ndim) + 1)));
    d_col = static_cast<int*>(dalloc(sizeof(int) * size_t(nnz)));
    d_slot = static_cast<int8_t*>(dalloc(slot.size()));
    d_val = static_cast<double*>(dalloc(sizeof(double) * size_t(nnz)));
    ck(cudaMemcpyAsync(d_rowptr, row_ptr.data(), sizeof(int) * row_ptr.size(), cudaMemcpyHostToDevice, stream));
    ck(cudaMemcpyAsync(d_slot, slot.data(), slot.size(), cudaMemcpyHostToDevice, stream));
    pat.row_ptr = d_rowptr; pat.col_idx = d_col; pat.slot = d_slot;
    launch_pattern(geo, pat, d_col, stream);
    if (rowintcon >= 0) launch_dense_row_cols(int(nc), d_col + row_ptr[rowintcon], stream);
    // intcond_scaling (src/ocean/thcm_utils.F90:285-312): cos(y_j) dfzT(k) on ocean cells
    d_intcoef = static_cast<double*>(dalloc(sizeof(double) * nc));
    {
        std::vector<double> coef(nc, 0.0);
        for (int k = 1; k <= l; ++k) for (int j = 1; j <= m; ++j) for (int i = 1; i <= n; ++i)
            if (LM(i, j, k) == OCEAN)
                coef[size_t(i - 1) + size_t(n) * (size_t(j - 1) + size_t(m) * (k - 1))] = std::cos(y[j]) * dfzT[k];
        ck(cudaMemcpyAsync(d_intcoef, coef.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, stream));
        ck(cudaStreamSynchronize(stream));
    }
    ck(cudaGetLastError());
    ck(cudaMemsetAsync(d_val, 0, sizeof(double) * size_t(nnz), stream));
    update_forcing();
    lin();
    launch_mass(geo, P, d_B, stream);
    zero_mass_rows();
    ck(cudaGetLastError());
    // vmix_init (src/ocean/mix_imp.f:57-111): Mixing = 1 fixes the partition
    // of T and S rows and columns; Mixing = 2 starts with both fields off
    for (int k = 1; k <= l && !any_ocean; ++k)
        for (int j = 1; j <= m && !any_ocean; ++j)
            for (int i = 1; i <= n && !any_ocean; ++i) any_ocean = LM(i, j, k) == OCEAN ? 1 : 0;
    int flags[5] = {0, 0, 0, 0, 0};
    if (c.vmix == 1) { flags[0] = flags[1] = flags[2] = flags[3] = 1; flags[4] = any_ocean; }
    d_mixflags = static_cast<int*>(dalloc(sizeof(flags)));
    d_mixpart = static_cast<double*>(dalloc(sizeof(double) * 2 * 152));
    ck(cudaMemcpyAsync(d_mixflags, flags, sizeof(flags), cudaMemcpyHostToDevice, stream));
    ck(cudaStreamSynchronize(stream));
}

MixParams Engine::mix_params() const {
    MixParams M{};
    M.on = (cfg.vmix == 1 || cfg.vmix == 2) ? 1 : 0;
    if (M.on && (P.par[MIXP] != 0.0 || P.par[MKAP] != 0.0)) throw EngineError(IEMIC_ERR_ARG);
    M.rhomix = (cfg.rho_mixing != 0 && P.par[NLES] == 0.0) ? 1 : 0;
    M.lambda = P.par[LAMB];
    M.xes = P.par[NLES];
    M.kvc = P.par[P_VC];
    M.eps = (1.0 - P.par[ALPC]) * P.par[ENER] * P.par[PE_V];
    M.fac = cfg.alphaT * P.par[SPL1];
    M.flags = d_mixflags;
    return M;
}

void Engine::special_rows_rhs(const double* x, double* F) {
    launch_special_rhs(int(nc), d_intcoef, x, F, rowintcon, sint_sign, rowPfix1, rowPfix2, stream);
}

// Ocean::computeRHS / computeJacobian call THCM::fixMixing(0) (Ocean.C:1281,
// 1302), so with Mixing = 2 every evaluation re-runs vmix_control.
void Engine::mix_control(const double* x, double* part) {
    if (cfg.vmix == 2) launch_mix_control(geo, x, part, d_mixflags, any_ocean, stream);
}

// B is zero in the rows that carry no time derivative: the integral
// condition (assemble.F90:49, THCM.C:1233-1238) and the fixed pressure points
void Engine::zero_mass_rows() {
    for (int r : {rowintcon, rowPfix1, rowPfix2})
        if (r >= 0) ck(cudaMemsetAsync(d_B + r, 0, sizeof(double), stream));
}

void Engine::set_par(int idx, double value) {
    if (idx >= 1 && idx <= NPAR) P.par[idx] = value;
    update_forcing();
    lin();
    launch_mass(geo, P, d_B, stream);
    zero_mass_rows();
    ck(cudaGetLastError());
    jac_valid = false;
}

// Algorithmic bytes: the state read and the padded fields written and read
// back (usol), plus the residual (3 vectors) or the CSR values written (FP64
// and FP32 copies) for the Jacobian.
void Engine::rhs_dev(const double* x, double* F) {
    const MixParams mp = mix_params();
    cudaEvent_t ev = timer.start(stream);
    launch_usol(geo, x, d_pads, stream);
    mix_control(x, d_mixpart);
    launch_rhs(geo, P, mp, fs, d_al, d_pads, x, d_surf, F, stream);
    special_rows_rhs(x, F);
    timer.stop(ev, stream, IEMIC_KC_ASSEMBLY, 8.0 * 4.0 * ndim, 0.0);
    ck(cudaGetLastError());
}

void Engine::jacobian_dev(const double* x) {
    const MixParams mp = mix_params();
    cudaEvent_t ev = timer.start(stream);
    launch_usol(geo, x, d_pads, stream);
    mix_control(x, d_mixpart);
    launch_jacobian(geo, P, mp, pat, d_al, d_pads, d_val, nullptr, stream);
    launch_special_jac(int(nc), d_rowptr, d_col, d_intcoef, d_val, nullptr, rowintcon, sint_sign, rowPfix1, rowPfix2,
                       stream);
    timer.stop(ev, stream, IEMIC_KC_ASSEMBLY, 8.0 * double(nnz) + 8.0 * 3.0 * ndim, 0.0);
    ck(cudaGetLastError());
    jac_valid = true;
    fact64_stale = fact32_stale = true;
    jacT_stale = true;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

#define GUARD_BEGIN try {
#define GUARD_END                                   \
    }                                               \
    catch (const EngineError& err) { return err.code; } \
    catch (const std::bad_alloc&) { return IEMIC_ERR_NOMEM; } \
    catch (...) { return IEMIC_ERR_CUDA; }          \
    return IEMIC_OK;

extern "C" {

int iemic_create(const iemic_config* cfg, const int* landm, iemic_ocean** out) {
    if (!cfg || !out) return IEMIC_ERR_ARG;
    *out = nullptr;
    if (cfg->n < 3 || cfg->m < 2 || cfg->l < 2) return IEMIC_ERR_ARG;
    if (int64_t(cfg->n) * cfg->m * cfg->l * NUN >= (int64_t(1) << 30)) return IEMIC_ERR_ARG;
    iemic_ocean* h = new (std::nothrow) iemic_ocean();
    if (!h) return IEMIC_ERR_NOMEM;
    try {
        h->e.init(*cfg, landm);
    } catch (const EngineError& err) {
        delete h;
        return err.code;
    } catch (...) {
        delete h;
        return IEMIC_ERR_CUDA;
    }
    *out = h;
    return IEMIC_OK;
}

int iemic_destroy(iemic_ocean* h) {
    if (!h) return IEMIC_ERR_ARG;
    delete h;
    return IEMIC_OK;
}

int iemic_ndim(const iemic_ocean* h, int* ndim) {
    if (!h || !ndim) return IEMIC_ERR_ARG;
    *ndim = h->e.ndim;
    return IEMIC_OK;
}

int iemic_get_landm(const iemic_ocean* h, int* landm) {
    if (!h || !landm) return IEMIC_ERR_ARG;
    std::copy(h->e.landm.begin(), h->e.landm.end(), landm);
    return IEMIC_OK;
}

int iemic_set_par(iemic_ocean* h, int idx, double value) {
    if (!h || idx < 1 || idx > NPAR) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    h->e.set_par(idx, value);
    GUARD_END
}

int iemic_get_par(const iemic_ocean* h, int idx, double* value) {
    if (!h || !value || idx < 1 || idx > NPAR) return IEMIC_ERR_ARG;
    *value = h->e.P.par[idx];
    return IEMIC_OK;
}

int iemic_set_forcing(iemic_ocean* h, const double* taux, const double* tauy, const double* tatm,
                      const double* emip, const double* spert) {
    if (!h) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    const size_t nm = size_t(e.cfg.n) * e.cfg.m;
    const double* f[5] = {taux, tauy, tatm, emip, spert};
    for (int q = 0; q < 5; ++q)
        if (f[q]) std::copy(f[q], f[q] + nm, e.surf.begin() + q * nm);
    e.update_forcing();
    e.lin();
    ck(cudaGetLastError());
    e.jac_valid = false;
    GUARD_END
}

int iemic_rhs_dev(iemic_ocean* h, const double* x, double* F) {
    if (!h || !x || !F) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    h->e.rhs_dev(x, F);
    ck(cudaStreamSynchronize(h->e.stream));
    GUARD_END
}

int iemic_rhs(iemic_ocean* h, const double* x, double* F) {
    if (!h || !x || !F) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    ck(cudaMemcpyAsync(e.d_x, x, sizeof(double) * e.ndim, cudaMemcpyHostToDevice, e.stream));
    e.rhs_dev(e.d_x, e.d_F);
    ck(cudaMemcpyAsync(F, e.d_F, sizeof(double) * e.ndim, cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_jacobian_dev(iemic_ocean* h, const double* x) {
    if (!h || !x) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    h->e.jacobian_dev(x);
    ck(cudaStreamSynchronize(h->e.stream));
    GUARD_END
}

int iemic_jacobian(iemic_ocean* h, const double* x) {
    if (!h || !x) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    ck(cudaMemcpyAsync(e.d_x, x, sizeof(double) * e.ndim, cudaMemcpyHostToDevice, e.stream));
    e.jacobian_dev(e.d_x);
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_graph_nnz(const iemic_ocean* h, int64_t* nnz) {
    if (!h || !nnz) return IEMIC_ERR_ARG;
    *nnz = h->e.nnz;
    return IEMIC_OK;
}

int iemic_get_csr(iemic_ocean* h, int* row_ptr, int* col_idx, double* values, int index_base) {
    if (!h || (index_base != 0 && index_base != 1)) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    if (row_ptr)
        for (size_t r = 0; r < e.row_ptr.size(); ++r) row_ptr[r] = e.row_ptr[r] + index_base;
    if (col_idx) {
        ck(cudaMemcpyAsync(col_idx, e.d_col, sizeof(int) * size_t(e.nnz), cudaMemcpyDeviceToHost, e.stream));
        ck(cudaStreamSynchronize(e.stream));
        if (index_base)
            for (int64_t q = 0; q < e.nnz; ++q) col_idx[q] += 1;
    }
    if (values) {
        if (!e.jac_valid) return IEMIC_ERR_STATE;
        ck(cudaMemcpyAsync(values, e.d_val, sizeof(double) * size_t(e.nnz), cudaMemcpyDeviceToHost, e.stream));
    }
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_mass(iemic_ocean* h, double* diagB) {
    if (!h || !diagB) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    ck(cudaMemcpyAsync(diagB, e.d_B, sizeof(double) * e.ndim, cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_apply_matrix(iemic_ocean* h, const double* v, double* out) {
    if (!h || !v || !out) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    if (!e.jac_valid) return IEMIC_ERR_STATE;
    ck(cudaMemcpyAsync(e.d_v1, v, sizeof(double) * e.ndim, cudaMemcpyHostToDevice, e.stream));
    e.spmv64(e.d_v1, e.d_v2);
    ck(cudaMemcpyAsync(out, e.d_v2, sizeof(double) * e.ndim, cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

}  // extern "C"
