"""CPU oracle for the THCM Newton-step path -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper around ``thcm_oracle.cpp`` / ``krylov_oracle.cpp``, a plain
C++ FP64 restatement of the reference's Fortran THCM kernels
(src/ocean/usrc.F90, spf.F90, boundary.F90, assemble.F90, matetc.F90,
grid.F90, forcing.F90) and of the maximal-graph scatter in src/ocean/THCM.C.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker / CPU baseline. The GPU
product never imports, links or calls it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libthcm_oracle.so")
SOURCES = ["thcm_oracle.cpp", "krylov_oracle.cpp"]

# Parameter indices of par(1..30) (src/ocean/par.F90:41-70)
PAR = dict(AL_T=1, RAYL=2, EK_V=3, EK_H=4, ROSB=5, MIXP=6, RESC=7, SPL1=8, HMTP=9,
           SUNP=10, PE_H=11, PE_V=12, P_VC=13, LAMB=14, SALT=15, WIND=16, TEMP=17,
           BIOT=18, COMB=19, ARCL=20, NLES=21, IFRICB=22, CONT=23, ENER=24, ALPC=25,
           CMPR=26, FPER=27, SPER=28, MKAP=29, SPL2=30)


def build(force=False):
    """Compile the oracle with g++ (-ffp-contract=off keeps FP64 rounding
    identical to an unfused evaluation of the Fortran expressions)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "thcm_oracle.h")])
        if os.path.getmtime(LIB) >= newest:
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
           "-o", tmp] + srcs
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class Config(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("m", ctypes.c_int), ("l", ctypes.c_int),
                ("xmin_deg", ctypes.c_double), ("xmax_deg", ctypes.c_double),
                ("ymin_deg", ctypes.c_double), ("ymax_deg", ctypes.c_double),
                ("periodic", ctypes.c_int), ("hdim", ctypes.c_double), ("qz", ctypes.c_double),
                ("alphaT", ctypes.c_double), ("alphaS", ctypes.c_double),
                ("ih", ctypes.c_int), ("coriolis_on", ctypes.c_int),
                ("tres", ctypes.c_int), ("sres", ctypes.c_int),
                ("iza", ctypes.c_int), ("ite", ctypes.c_int), ("its", ctypes.c_int),
                ("forcing_type", ctypes.c_int), ("vmix", ctypes.c_int), ("rho_mixing", ctypes.c_int),
                ("tap", ctypes.c_int), ("sint_sign", ctypes.c_int), ("intcon_i", ctypes.c_int),
                ("intcon_j", ctypes.c_int), ("fix_pressure_points", ctypes.c_int)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("restart", ctypes.c_int), ("maxit", ctypes.c_int), ("tol", ctypes.c_double),
                ("precond", ctypes.c_int), ("threads", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("relres", ctypes.c_double),
                ("explicit_relres", ctypes.c_double), ("status", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [ctypes.POINTER(Config), ip]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_ndim.restype = ctypes.c_int
        L.oracle_ndim.argtypes = [vp]
        L.oracle_get_landm.argtypes = [vp, ip]
        L.oracle_set_forcing.argtypes = [vp, dp, dp, dp, dp, dp]
        L.oracle_set_par.argtypes = [vp, ctypes.c_int, ctypes.c_double]
        L.oracle_get_par.restype = ctypes.c_double
        L.oracle_get_par.argtypes = [vp, ctypes.c_int]
        L.oracle_get_frc.argtypes = [vp, dp]
        L.oracle_get_grid.argtypes = [vp] + [dp] * 8
        L.oracle_rhs.argtypes = [vp, dp, dp]
        L.oracle_fortran_nnz.restype = ctypes.c_int
        L.oracle_fortran_nnz.argtypes = [vp]
        L.oracle_fortran_csr.argtypes = [vp, ip, ip, dp]
        L.oracle_assemble_rhs_matrix.argtypes = [vp, dp]
        L.oracle_graph_nnz.restype = ctypes.c_int64
        L.oracle_graph_nnz.argtypes = [vp]
        L.oracle_graph.argtypes = [vp, ip, ip]
        L.oracle_jacobian.restype = ctypes.c_int
        L.oracle_jacobian.argtypes = [vp, dp, dp]
        L.oracle_mass.argtypes = [vp, dp]
        L.oracle_psim.argtypes = [vp, dp, dp]
        L.oracle_An.restype = ctypes.c_double
        L.oracle_An.argtypes = [vp] + [ctypes.c_int] * 6
        L.oracle_gmres.restype = ctypes.c_int
        L.oracle_gmres.argtypes = [ctypes.c_int, ip, ip, dp, dp, dp, ctypes.POINTER(SolveOpts),
                                   ctypes.POINTER(SolveStats)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class Oracle:
    """The reference's THCM model restated on the CPU (FP64)."""

    def __init__(self, cfg, landm=None):
        self.L = lib()
        self.cfg = cfg
        c = Config(**cfg)
        lm = None
        if landm is not None:
            self._landm_in = np.ascontiguousarray(landm, dtype=np.int32).ravel()
            lm = _ip(self._landm_in)
        self.h = self.L.oracle_create(ctypes.byref(c), lm)
        if not self.h:
            raise ValueError("oracle_create: the integral-condition row lies on land")
        self.n, self.m, self.l = cfg["n"], cfg["m"], cfg["l"]
        self.ndim = self.L.oracle_ndim(self.h)

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def landm(self):
        out = np.zeros((self.l + 2) * (self.m + 2) * (self.n + 2), dtype=np.int32)
        self.L.oracle_get_landm(self.h, _ip(out))
        return out

    def set_forcing(self, taux=None, tauy=None, tatm=None, emip=None, spert=None):
        arrs = []
        ptrs = []
        for a in (taux, tauy, tatm, emip, spert):
            if a is None:
                ptrs.append(None)
            else:
                a = np.ascontiguousarray(a, dtype=np.float64).ravel()
                arrs.append(a)
                ptrs.append(_dp(a))
        self.L.oracle_set_forcing(self.h, *ptrs)

    def set_par(self, idx, value):
        if isinstance(idx, str):
            idx = PAR[idx]
        self.L.oracle_set_par(self.h, idx, float(value))

    def get_par(self, idx):
        if isinstance(idx, str):
            idx = PAR[idx]
        return self.L.oracle_get_par(self.h, idx)

    def frc(self):
        out = np.zeros(self.ndim)
        self.L.oracle_get_frc(self.h, _dp(out))
        return out

    def grid(self):
        n, m, l = self.n, self.m, self.l
        g = dict(x=np.zeros(n), y=np.zeros(m + 2), xu=np.zeros(n + 1), yv=np.zeros(m + 1),
                 z=np.zeros(l), zw=np.zeros(l + 1), dfzT=np.zeros(l), dfzW=np.zeros(l + 1))
        self.L.oracle_get_grid(self.h, *[_dp(g[k]) for k in ("x", "y", "xu", "yv", "z", "zw", "dfzT", "dfzW")])
        return g

    def rhs(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        F = np.zeros(self.ndim)
        self.L.oracle_rhs(self.h, _dp(x), _dp(F))
        return F

    def graph(self):
        nnz = self.L.oracle_graph_nnz(self.h)
        rp = np.zeros(self.ndim + 1, dtype=np.int32)
        ci = np.zeros(nnz, dtype=np.int32)
        self.L.oracle_graph(self.h, _ip(rp), _ip(ci))
        return rp, ci

    def jacobian(self, x):
        """Values of J(x) in the maximal graph; also returns the excluded count."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        nnz = self.L.oracle_graph_nnz(self.h)
        vals = np.zeros(nnz)
        excl = self.L.oracle_jacobian(self.h, _dp(x), _dp(vals))
        return vals, excl

    def fortran_csr(self):
        nnz = self.L.oracle_fortran_nnz(self.h)
        beg = np.zeros(self.ndim + 1, dtype=np.int32)
        jco = np.zeros(nnz, dtype=np.int32)
        co = np.zeros(nnz)
        self.L.oracle_fortran_csr(self.h, _ip(beg), _ip(jco), _dp(co))
        return beg, jco, co

    def assemble_rhs_matrix(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.L.oracle_assemble_rhs_matrix(self.h, _dp(x))
        return self.fortran_csr()

    def mass(self):
        out = np.zeros(self.ndim)
        self.L.oracle_mass(self.h, _dp(out))
        return out

    def psim(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros((self.m + 1) * (self.l + 1))
        self.L.oracle_psim(self.h, _dp(x), _dp(out))
        return out

    def An(self, kk, A, B, i, j, k):
        return self.L.oracle_An(self.h, kk, A, B, i, j, k)


def gmres(row_ptr, col_idx, val, b, restart=100, maxit=1000, tol=1e-8, precond=1, threads=1, x0=None):
    """CPU FP64 right-preconditioned GMRES(restart) on a CSR matrix."""
    L = lib()
    ndim = len(row_ptr) - 1
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_idx, dtype=np.int32)
    va = np.ascontiguousarray(val, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(ndim) if x0 is None else np.array(x0, dtype=np.float64)
    o = SolveOpts(restart, maxit, tol, precond, threads)
    st = SolveStats()
    L.oracle_gmres(ndim, _ip(rp), _ip(ci), _dp(va), _dp(bb), _dp(x), ctypes.byref(o), ctypes.byref(st))
    return x, dict(iters=st.iters, relres=st.relres, explicit_relres=st.explicit_relres, status=st.status)
