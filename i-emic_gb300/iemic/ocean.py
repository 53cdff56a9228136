"""Host-side mirror of the reference's ``Ocean`` model API.

Method names, argument meaning and the parameter names follow
src/ocean/Ocean.H:169-250 and src/utils/Model.H:54-145:
``computeRHS``, ``computeJacobian``, ``solve``, ``applyMatrix``,
``applyPrecon``, ``applyMassMat``, ``getState/getRHS/getSolution(mode)``,
``setPar/getPar(name)``. Errors from the C ABI raise ``IemicError`` (the
reference throws ``std::runtime_error`` through its ``ERROR`` macro).
"""
import ctypes
import os

import numpy as np

from . import build as _build

# Parameter names of THCM::par2int (src/ocean/THCM.C:1841-1886)
PARAMETER_NAMES = {
    "AL_T": 1, "Rayleigh-Number": 2, "Vertical Ekman-Number": 3, "Horizontal Ekman-Number": 4,
    "Rossby-Number": 5, "MIXP": 6, "RESC": 7, "SPL1": 8, "Salinity Homotopy": 9,
    "Solar Forcing": 10, "Horizontal Peclet-Number": 11, "Vertical Peclet-Number": 12,
    "P_VC": 13, "LAMB": 14, "Salinity Forcing": 15, "Wind Forcing": 16,
    "Temperature Forcing": 17, "Nonlinear Factor": 18, "Combined Forcing": 19, "ARCL": 20,
    "NLES": 21, "IFRICB": 22, "CONT": 23, "Energy": 24, "ALPC": 25, "CMPR": 26,
    "Flux Perturbation": 27, "Salinity Perturbation": 28, "MKAP": 29, "SPL2": 30,
}

ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "not converged", -4: "NaN/Inf",
          -5: "zero pivot", -6: "call order", -7: "device allocation failed"}

PREC_FP64, PREC_MIXED = 0, 1


class IemicError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        super().__init__("%s failed: %s (%d)" % (where, ERRORS.get(code, "error"), code))


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
    _fields_ = [("precision", ctypes.c_int), ("restart", ctypes.c_int), ("max_iters", ctypes.c_int),
                ("tol", ctypes.c_double), ("transpose", ctypes.c_int),
                ("reuse_preconditioner", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("factorizations", ctypes.c_int), ("perturbed_pivots", ctypes.c_int),
                ("relres", ctypes.c_double),
                ("time_factor_ms", ctypes.c_double), ("time_solve_ms", ctypes.c_double)]


class NewtonOpts(ctypes.Structure):
    _fields_ = [("max_iters", ctypes.c_int), ("tol", ctypes.c_double), ("backtracking_steps", ctypes.c_int),
                ("solve", SolveOpts), ("refactor_each_iter", ctypes.c_int)]


class NewtonStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("backtracks", ctypes.c_int), ("linear_solves", ctypes.c_int),
                ("krylov_iters", ctypes.c_int), ("factorizations", ctypes.c_int),
                ("rhs_norm0", ctypes.c_double), ("rhs_norm", ctypes.c_double),
                ("time_ms", ctypes.c_double), ("time_assembly_ms", ctypes.c_double),
                ("time_factor_ms", ctypes.c_double), ("time_solve_ms", ctypes.c_double)]


class ThetaOpts(ctypes.Structure):
    _fields_ = [("theta", ctypes.c_double), ("dt", ctypes.c_double), ("tol", ctypes.c_double),
                ("max_newton", ctypes.c_int), ("solve", SolveOpts), ("refactor_policy", ctypes.c_int)]


class ThetaStats(ctypes.Structure):
    _fields_ = [("newton_iters", ctypes.c_int), ("converged", ctypes.c_int), ("linear_solves", ctypes.c_int),
                ("krylov_iters", ctypes.c_int), ("factorizations", ctypes.c_int),
                ("norm_G", ctypes.c_double), ("norm_dx", ctypes.c_double),
                ("time_ms", ctypes.c_double), ("time_assembly_ms", ctypes.c_double),
                ("time_factor_ms", ctypes.c_double), ("time_solve_ms", ctypes.c_double)]


class ContinuationOpts(ctypes.Structure):
    _fields_ = [("par_idx", ctypes.c_int), ("ds", ctypes.c_double), ("ds_min", ctypes.c_double),
                ("ds_max", ctypes.c_double), ("decrease", ctypes.c_double),
                ("destination", ctypes.c_double), ("destination_tol", ctypes.c_double),
                ("max_steps", ctypes.c_int), ("max_newton", ctypes.c_int), ("min_newton", ctypes.c_int),
                ("opt_newton", ctypes.c_double), ("newton_tol", ctypes.c_double),
                ("residual_test", ctypes.c_char), ("normalize", ctypes.c_char), ("tangent", ctypes.c_char),
                ("initial_tangent", ctypes.c_char), ("epsilon", ctypes.c_double),
                ("tan_scaling", ctypes.c_double), ("predictor_bound", ctypes.c_double),
                ("backtracking_steps", ctypes.c_int), ("backtracking_increase", ctypes.c_double),
                ("newton_chord", ctypes.c_int), ("give_up_at_ds_min", ctypes.c_int),
                ("solve", SolveOpts), ("refactor_each_newton", ctypes.c_int)]


class ContinuationStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("failed_steps", ctypes.c_int), ("newton_iters", ctypes.c_int),
                ("linear_solves", ctypes.c_int), ("unconverged_solves", ctypes.c_int),
                ("krylov_iters", ctypes.c_int), ("factorizations", ctypes.c_int),
                ("reached_destination", ctypes.c_int), ("aborted", ctypes.c_int),
                ("par", ctypes.c_double), ("ds", ctypes.c_double), ("rhs_norm", ctypes.c_double),
                ("time_ms", ctypes.c_double), ("time_assembly_ms", ctypes.c_double),
                ("time_factor_ms", ctypes.c_double), ("time_solve_ms", ctypes.c_double)]


class KernelStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_longlong), ("ms", ctypes.c_double), ("bytes", ctypes.c_double),
                ("flops", ctypes.c_double)]


class AdjointOpts(ctypes.Structure):
    _fields_ = [("i_begin", ctypes.c_int), ("i_end", ctypes.c_int), ("solve", SolveOpts), ("fd_rel", ctypes.c_double)]


class AdjointStats(ctypes.Structure):
    _fields_ = [("g", ctypes.c_double), ("jmax", ctypes.c_int), ("kmax", ctypes.c_int), ("iters", ctypes.c_int),
                ("relres", ctypes.c_double), ("time_ms", ctypes.c_double)]


FORCING_FIELDS = ("taux", "tauy", "tatm", "emip", "spert")


class SolverInfo(ctypes.Structure):
    _fields_ = [("unknowns", ctypes.c_int64), ("reduced_unknowns", ctypes.c_int64), ("fronts", ctypes.c_int64),
                ("levels", ctypes.c_int64), ("factor_entries", ctypes.c_int64), ("front_entries", ctypes.c_int64),
                ("factor_flops", ctypes.c_double), ("work_entries", ctypes.c_int64),
                ("contrib_entries", ctypes.c_int64)]


KERNEL_CLASSES = {"factor_gemm": 0, "solve_gemv": 1, "assembly": 2, "spmv": 3, "factor_panel": 4,
                  "factor_inverse": 5, "factor_setup": 6, "solve_other": 7}


def _asdict(st):
    return {k: getattr(st, k) for k, _ in st._fields_}


# Every entry point of include/iemic_gb300.h with its ctypes signature.
_VP = ctypes.c_void_p
_IP = ctypes.POINTER(ctypes.c_int)
_DP = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "iemic_create": [ctypes.POINTER(Config), _IP, ctypes.POINTER(_VP)],
    "iemic_destroy": [_VP],
    "iemic_ndim": [_VP, _IP],
    "iemic_get_landm": [_VP, _IP],
    "iemic_set_par": [_VP, ctypes.c_int, ctypes.c_double],
    "iemic_get_par": [_VP, ctypes.c_int, _DP],
    "iemic_set_forcing": [_VP, _DP, _DP, _DP, _DP, _DP],
    "iemic_rhs": [_VP, _DP, _DP],
    "iemic_jacobian": [_VP, _DP],
    "iemic_rhs_dev": [_VP, _VP, _VP],
    "iemic_rhs_dev_noalloc": [_VP, _VP, _VP],
    "iemic_jacobian_dev": [_VP, _VP],
    "iemic_graph_nnz": [_VP, ctypes.POINTER(ctypes.c_int64)],
    "iemic_get_csr": [_VP, _IP, _IP, _DP, ctypes.c_int],
    "iemic_mass": [_VP, _DP],
    "iemic_apply_matrix": [_VP, _DP, _DP],
    "iemic_default_solve_opts": [ctypes.POINTER(SolveOpts)],
    "iemic_build_preconditioner": [_VP, ctypes.c_int],
    "iemic_apply_precon": [_VP, ctypes.c_int, _DP, _DP],
    "iemic_solve": [_VP, _DP, _DP, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats)],
    "iemic_solve_dev": [_VP, _VP, _VP, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats)],
    "iemic_solver_gauge": [_VP, _IP, ctypes.c_int, _IP],
    "iemic_get_solver_info": [_VP, ctypes.POINTER(SolverInfo)],
    "iemic_psim": [_VP, _DP, _DP, _DP, _DP],
    "iemic_psim_max_grad_dev": [_VP, _VP, ctypes.c_int, ctypes.c_int, _DP, _IP, _VP],
    "iemic_forcing_adjoint_dev": [_VP, _VP, _VP],
    "iemic_par_adjoint_dev": [_VP, _VP, _VP, ctypes.c_int, ctypes.c_double, _DP],
    "iemic_default_adjoint_opts": [ctypes.POINTER(AdjointOpts)],
    "iemic_adjoint_psim": [_VP, _DP, ctypes.POINTER(AdjointOpts), _DP, _IP, ctypes.c_int, _DP,
                           ctypes.POINTER(AdjointStats)],
    "iemic_kernel_timing": [_VP, ctypes.c_int],
    "iemic_kernel_stats_get": [_VP, ctypes.c_int, ctypes.POINTER(KernelStats)],
    "iemic_get_stream": [_VP, ctypes.POINTER(_VP)],
    "iemic_default_newton_opts": [ctypes.POINTER(NewtonOpts)],
    "iemic_newton": [_VP, _DP, ctypes.POINTER(NewtonOpts), ctypes.POINTER(NewtonStats)],
    "iemic_newton_dev": [_VP, _VP, ctypes.POINTER(NewtonOpts), ctypes.POINTER(NewtonStats)],
    "iemic_default_theta_opts": [ctypes.POINTER(ThetaOpts)],
    "iemic_theta_step": [_VP, _DP, ctypes.POINTER(ThetaOpts), ctypes.POINTER(ThetaStats)],
    "iemic_theta_step_dev": [_VP, _VP, ctypes.POINTER(ThetaOpts), ctypes.POINTER(ThetaStats)],
    "iemic_default_continuation_opts": [ctypes.POINTER(ContinuationOpts)],
    "iemic_continuation_run": [_VP, _DP, ctypes.POINTER(ContinuationOpts), ctypes.POINTER(ContinuationStats)],
    "iemic_continuation_run_dev": [_VP, _VP, ctypes.POINTER(ContinuationOpts),
                                   ctypes.POINTER(ContinuationStats)],
    "iemic_launch_count": [],
    "iemic_kernel_timing_failures": [_VP],
    "iemic_set_substitution_threshold": [_VP, ctypes.c_int],
    "iemic_analyse_pattern": [ctypes.POINTER(Config), _IP, _IP, _IP, ctypes.POINTER(SolverInfo)],
    "iemic_get_fronts": [_VP, ctypes.c_int, _IP, _IP, _IP, _IP, _IP],
    "iemic_kernel_trace": [_VP, ctypes.c_int, _IP, ctypes.POINTER(ctypes.c_float), _DP, _IP],
}
_VOID_RETURN = {"iemic_default_solve_opts", "iemic_default_newton_opts", "iemic_default_continuation_opts",
                "iemic_default_adjoint_opts", "iemic_default_theta_opts"}

_lib = None


def load_library(path=None, build_if_missing=True):
    """Load libiemic_gb300.so (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    if path is None:
        path = _build.LIB
        if build_if_missing and not os.path.exists(path):
            _build.build()
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = None if name in _VOID_RETURN else ctypes.c_int
        if name in ("iemic_launch_count", "iemic_kernel_timing_failures"):
            fn.restype = ctypes.c_longlong
    if path == _build.LIB:
        _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(_DP)


def _ip(a):
    return a.ctypes.data_as(_IP)


def analyse_pattern(cfg, landm, row_ptr, col_idx):
    """Host-side symbolic analysis of the preconditioner for a grid, the
    engine's land mask and J's 0-based CSR pattern (no GPU needed): the size
    report of iemic_get_solver_info, after the plan's consistency checks."""
    L = load_library()
    lm = np.ascontiguousarray(landm, dtype=np.int32)
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_idx, dtype=np.int32)
    st = SolverInfo()
    rc = L.iemic_analyse_pattern(ctypes.byref(Config(**{k: cfg[k] for k, _ in Config._fields_})),
                                 lm.ctypes.data_as(_IP), rp.ctypes.data_as(_IP), ci.ctypes.data_as(_IP),
                                 ctypes.byref(st))
    if rc != 0:
        raise IemicError(rc, "analyse_pattern")
    return _asdict(st)


class Ocean:
    """The THCM ocean model on one GPU (mirror of the reference ``Ocean``)."""

    def __init__(self, config, landm=None, forcing=None, starting_parameters=()):
        self.L = load_library()
        self.config = dict(config)
        c = Config(**{k: config[k] for k, _ in Config._fields_})
        self._h = _VP()
        lm = None
        if landm is not None:
            self._landm_in = np.ascontiguousarray(landm, dtype=np.int32).ravel()
            lm = _ip(self._landm_in)
        self._check(self.L.iemic_create(ctypes.byref(c), lm, ctypes.byref(self._h)), "iemic_create")
        nd = ctypes.c_int()
        self._check(self.L.iemic_ndim(self._h, ctypes.byref(nd)), "iemic_ndim")
        self.ndim = nd.value
        self.n, self.m, self.l = config["n"], config["m"], config["l"]
        self.state = np.zeros(self.ndim)
        self.rhs = np.zeros(self.ndim)
        self.sol = np.zeros(self.ndim)
        self._jac_state = None
        if forcing:
            self.setForcing(**forcing)
        for name, val in starting_parameters:
            self.setPar(name, val)

    # ---- lifecycle ------------------------------------------------------
    def _check(self, rc, where):
        if rc != 0:
            raise IemicError(rc, where)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.L.iemic_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ---- parameters and forcing ------------------------------------------
    @staticmethod
    def par2int(name):
        if isinstance(name, int):
            return name
        if name not in PARAMETER_NAMES:
            raise KeyError("unknown THCM parameter %r" % name)
        return PARAMETER_NAMES[name]

    def setPar(self, name, value):
        self._check(self.L.iemic_set_par(self._h, self.par2int(name), float(value)), "setPar")

    def getPar(self, name):
        v = ctypes.c_double()
        self._check(self.L.iemic_get_par(self._h, self.par2int(name), ctypes.byref(v)), "getPar")
        return v.value

    def setForcing(self, taux=None, tauy=None, tatm=None, emip=None, spert=None):
        keep, ptrs = [], []
        for a in (taux, tauy, tatm, emip, spert):
            if a is None:
                ptrs.append(None)
            else:
                a = np.ascontiguousarray(a, dtype=np.float64).ravel()
                if a.size != self.n * self.m:
                    raise ValueError("forcing field must have n*m entries")
                keep.append(a)
                ptrs.append(_dp(a))
        self._check(self.L.iemic_set_forcing(self._h, *ptrs), "setForcing")

    def getLandMask(self):
        out = np.zeros((self.l + 2) * (self.m + 2) * (self.n + 2), dtype=np.int32)
        self._check(self.L.iemic_get_landm(self._h, _ip(out)), "getLandMask")
        return out

    # ---- Model API -------------------------------------------------------
    def getState(self, mode="C"):
        return self.state if mode == "V" else self.state.copy()

    def getRHS(self, mode="C"):
        return self.rhs if mode == "V" else self.rhs.copy()

    def getSolution(self, mode="C"):
        return self.sol if mode == "V" else self.sol.copy()

    def setState(self, x):
        self.state[:] = np.asarray(x, dtype=np.float64)

    def computeRHS(self, x=None):
        x = self.state if x is None else np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(self.ndim)
        self._check(self.L.iemic_rhs(self._h, _dp(x), _dp(out)), "computeRHS")
        if x is self.state:
            self.rhs[:] = out
        return out

    def computeJacobian(self, x=None):
        x = self.state if x is None else np.ascontiguousarray(x, dtype=np.float64)
        self._check(self.L.iemic_jacobian(self._h, _dp(x)), "computeJacobian")

    def graph_nnz(self):
        v = ctypes.c_int64()
        self._check(self.L.iemic_graph_nnz(self._h, ctypes.byref(v)), "graph_nnz")
        return v.value

    def getJacobian(self, index_base=0, values=True):
        """(row_ptr, col_idx, values) of the maximal-graph CSR."""
        nnz = self.graph_nnz()
        rp = np.zeros(self.ndim + 1, dtype=np.int32)
        ci = np.zeros(nnz, dtype=np.int32)
        va = np.zeros(nnz) if values else None
        self._check(self.L.iemic_get_csr(self._h, _ip(rp), _ip(ci), _dp(va) if values else None, index_base),
                    "getJacobian")
        return rp, ci, va

    def getMassMat(self):
        out = np.zeros(self.ndim)
        self._check(self.L.iemic_mass(self._h, _dp(out)), "getMassMat")
        return out

    def applyMassMat(self, v):
        return self.getMassMat() * np.asarray(v, dtype=np.float64)

    def applyMatrix(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.zeros(self.ndim)
        self._check(self.L.iemic_apply_matrix(self._h, _dp(v), _dp(out)), "applyMatrix")
        return out

    def default_solve_opts(self, precision=PREC_MIXED):
        o = SolveOpts()
        self.L.iemic_default_solve_opts(ctypes.byref(o))
        o.precision = precision
        return o

    def buildPreconditioner(self, precision=-1):
        self._check(self.L.iemic_build_preconditioner(self._h, precision), "buildPreconditioner")

    def applyPrecon(self, v, precision=PREC_FP64):
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.zeros(self.ndim)
        self._check(self.L.iemic_apply_precon(self._h, precision, _dp(v), _dp(out)), "applyPrecon")
        return out

    def getGauge(self):
        """Pressure unknowns the solver holds at zero (gauge of J's null space)."""
        cnt = ctypes.c_int()
        self._check(self.L.iemic_solver_gauge(self._h, None, 0, ctypes.byref(cnt)), "getGauge")
        out = np.zeros(max(cnt.value, 1), dtype=np.int32)
        self._check(self.L.iemic_solver_gauge(self._h, _ip(out), cnt.value, ctypes.byref(cnt)), "getGauge")
        return out[:cnt.value].copy()

    def solve(self, rhs=None, opts=None, **kw):
        """Ocean::solve: x = J^{-1} rhs (default rhs: the stored RHS)."""
        b = self.rhs if rhs is None else np.ascontiguousarray(rhs, dtype=np.float64)
        o = opts if opts is not None else self.default_solve_opts(kw.pop("precision", PREC_MIXED))
        for k, v in kw.items():
            setattr(o, k, v)
        x = np.zeros(self.ndim)
        st = SolveStats()
        rc = self.L.iemic_solve(self._h, _dp(b), _dp(x), ctypes.byref(o), ctypes.byref(st))
        stats = dict(iters=st.iters, relres=st.relres,
                     factorizations=st.factorizations, perturbed_pivots=st.perturbed_pivots,
                     time_factor_ms=st.time_factor_ms, time_solve_ms=st.time_solve_ms, status=rc)
        if rc not in (0, -3):
            raise IemicError(rc, "solve")
        self.sol[:] = x
        return x, stats

    # ---- Newton and continuation (src/newton/Newton.H, src/continuation/Continuation.H)
    def default_newton_opts(self, precision=PREC_MIXED):
        o = NewtonOpts()
        self.L.iemic_default_newton_opts(ctypes.byref(o))
        o.solve.precision = precision
        return o

    def newton(self, x=None, opts=None, **kw):
        """Newton iteration at fixed parameters from x (default: the stored state).
        Returns (x, stats); the converged state also becomes the stored state."""
        x = np.array(self.state if x is None else x, dtype=np.float64)
        o = opts if opts is not None else self.default_newton_opts(kw.pop("precision", PREC_MIXED))
        for k, v in kw.items():
            setattr(o, k, v)
        st = NewtonStats()
        rc = self.L.iemic_newton(self._h, _dp(x), ctypes.byref(o), ctypes.byref(st))
        stats = _asdict(st)
        stats["status"] = rc
        if rc not in (0, -3):
            raise IemicError(rc, "newton")
        self.state[:] = x
        return x, stats

    # ---- implicit time stepping (src/transient/ThetaModel.H, src/transient/Newton.H)
    def default_theta_opts(self, precision=PREC_MIXED):
        o = ThetaOpts()
        self.L.iemic_default_theta_opts(ctypes.byref(o))
        o.solve.precision = precision
        return o

    def thetaStep(self, x=None, dt=None, theta=None, opts=None, **kw):
        """One implicit theta-method step of size dt from x (default: the
        stored state), ThetaModel<Ocean>::initStep + Newton::run. Returns
        (x_new, stats); x_new also becomes the stored state."""
        x = np.array(self.state if x is None else x, dtype=np.float64)
        o = opts if opts is not None else self.default_theta_opts(kw.pop("precision", PREC_MIXED))
        if dt is not None:
            o.dt = dt
        if theta is not None:
            o.theta = theta
        for k, v in kw.items():
            setattr(o, k, v)
        st = ThetaStats()
        rc = self.L.iemic_theta_step(self._h, _dp(x), ctypes.byref(o), ctypes.byref(st))
        stats = _asdict(st)
        stats["status"] = rc
        if rc not in (0, -3):
            raise IemicError(rc, "thetaStep")
        self.state[:] = x
        return x, stats

    def default_continuation_opts(self, par="Combined Forcing", precision=PREC_MIXED):
        o = ContinuationOpts()
        self.L.iemic_default_continuation_opts(ctypes.byref(o))
        o.par_idx = self.par2int(par)
        o.solve.precision = precision
        return o

    def continuation(self, x=None, opts=None, **kw):
        """Continuation<Ocean>::run from x (default: the stored state).
        Returns (x, stats) with stats["par"] the final parameter value."""
        x = np.array(self.state if x is None else x, dtype=np.float64)
        par = kw.pop("par", "Combined Forcing")
        o = opts if opts is not None else self.default_continuation_opts(par, kw.pop("precision", PREC_MIXED))
        for k, v in kw.items():
            if k in ("residual_test", "normalize", "tangent", "initial_tangent") and isinstance(v, str):
                v = v.encode()
            setattr(o, k, v)
        st = ContinuationStats()
        rc = self.L.iemic_continuation_run(self._h, _dp(x), ctypes.byref(o), ctypes.byref(st))
        stats = _asdict(st)
        stats["status"] = rc
        if rc not in (0, -3):
            raise IemicError(rc, "continuation")
        self.state[:] = x
        return x, stats

    def solverInfo(self):
        """Size of the nested-dissection factorisation (fronts, entries, flops)."""
        st = SolverInfo()
        self._check(self.L.iemic_get_solver_info(self._h, ctypes.byref(st)), "solverInfo")
        return _asdict(st)

    # ---- device timing of the instrumented kernel classes -------------------
    def kernelTiming(self, enable=True):
        self._check(self.L.iemic_kernel_timing(self._h, 1 if enable else 0), "kernelTiming")

    def kernelStats(self):
        out = {}
        for name, k in KERNEL_CLASSES.items():
            st = KernelStats()
            self._check(self.L.iemic_kernel_stats_get(self._h, k, ctypes.byref(st)), "kernelStats")
            out[name] = _asdict(st)
        return out

    def setSubstitutionThreshold(self, max_inverse_nf):
        """Fronts up to this many own unknowns use whole inverses; larger plans substitute over 256-row blocks."""
        self._check(self.L.iemic_set_substitution_threshold(self._h, int(max_inverse_nf)), "setSubstitutionThreshold")

    def fronts(self):
        """Elimination tree of the factorisation: arrays nf, nb, level, parent per front."""
        cnt = ctypes.c_int(0)
        self._check(self.L.iemic_get_fronts(self._h, 0, None, None, None, None, ctypes.byref(cnt)), "fronts")
        out = {k: np.zeros(cnt.value, np.int32) for k in ("nf", "nb", "level", "parent")}
        self._check(self.L.iemic_get_fronts(self._h, cnt.value, *(out[k].ctypes.data_as(_IP)
                                                                  for k in ("nf", "nb", "level", "parent")),
                                            ctypes.byref(cnt)), "fronts")
        return out

    def kernelTrace(self):
        """Per-launch (class name, device ms, algorithmic bytes) since timing was enabled."""
        cnt = ctypes.c_int(0)
        self._check(self.L.iemic_kernel_trace(self._h, 0, None, None, None, ctypes.byref(cnt)), "kernelTrace")
        n = cnt.value
        cls = np.zeros(n, np.int32)
        ms = np.zeros(n, np.float32)
        nb = np.zeros(n, np.float64)
        if n:
            self._check(self.L.iemic_kernel_trace(self._h, n, cls.ctypes.data_as(_IP),
                                                  ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                  nb.ctypes.data_as(_DP), ctypes.byref(cnt)), "kernelTrace")
        names = {v: k for k, v in KERNEL_CLASSES.items()}
        return [(names[int(c)], float(t), float(b)) for c, t, b in zip(cls, ms, nb)]

    def kernelTimingFailures(self):
        """Timing records the runtime could not time (0 when every launch was timed)."""
        return int(self.L.iemic_kernel_timing_failures(self._h))

    def stream(self):
        """The cudaStream_t (as an int) all calls on this handle run on."""
        p = _VP()
        self._check(self.L.iemic_get_stream(self._h, ctypes.byref(p)), "stream")
        return p.value or 0

    # ---- diagnostics and adjoint ---------------------------------------------
    def getPsiM(self, x=None):
        """Ocean::getPsiM: (psi (l+1, m+1) in Sv, psiMin, psiMax)."""
        x = np.ascontiguousarray(self.state if x is None else x, dtype=np.float64)
        psi = np.zeros((self.l + 1) * (self.m + 1))
        lo, hi = ctypes.c_double(), ctypes.c_double()
        self._check(self.L.iemic_psim(self._h, _dp(x), _dp(psi), ctypes.byref(lo), ctypes.byref(hi)), "getPsiM")
        return psi.reshape(self.l + 1, self.m + 1), lo.value, hi.value

    def default_adjoint_opts(self, precision=PREC_MIXED):
        o = AdjointOpts()
        self.L.iemic_default_adjoint_opts(ctypes.byref(o))
        o.solve.precision = precision
        return o

    def adjointPsiM(self, x, pars=(), sector=None, opts=None, **kw):
        """Gradient of g = max psi_M (Sv) at the steady state x: returns
        (g, {field: (m, n) gradient}, {par: gradient}, stats)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        o = opts if opts is not None else self.default_adjoint_opts(kw.pop("precision", PREC_MIXED))
        if sector is not None:
            o.i_begin, o.i_end = sector
        for k, v in kw.items():
            setattr(o.solve, k, v)
        idx = np.array([self.par2int(p) for p in pars], dtype=np.int32)
        gp = np.zeros(max(len(idx), 1))
        gf = np.zeros(5 * self.n * self.m)
        st = AdjointStats()
        rc = self.L.iemic_adjoint_psim(self._h, _dp(x), ctypes.byref(o), _dp(gf), _ip(idx) if len(idx) else None,
                                       len(idx), _dp(gp), ctypes.byref(st))
        stats = _asdict(st)
        stats["status"] = rc
        if rc not in (0, -3):
            raise IemicError(rc, "adjointPsiM")
        fields = {name: gf[q * self.n * self.m:(q + 1) * self.n * self.m].reshape(self.m, self.n)
                  for q, name in enumerate(FORCING_FIELDS)}
        return st.g, fields, {p: gp[q] for q, p in enumerate(pars)}, stats
