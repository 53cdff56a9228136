"""Newton and pseudo-arclength continuation on the CPU oracle -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's drivers, used as the checker of the
GPU drivers behind ``iemic_newton`` / ``iemic_continuation_run``:

- ``newton``: Newton<Model>::Run and RunBackTracking (src/newton/Newton.H:40-100).
- ``Continuation``: Continuation<Model> (src/continuation/Continuation.H):
  run 209-246, step 250-320, createInitialTangent 324-376, computeDFDPar
  412-442, createTangent 446-518, normalize 522-566, eulerPredictor 570-606,
  newtonCorrector 610-837, runBackTracking 841-878, detect 882-950,
  adjustStep 974-1003, reset 1030-1065, store/restore 1068-1115.

``OracleModel`` supplies F and J from the C++ THCM oracle and solves J x = b
exactly (scipy sparse LU). J is singular (pressure null modes, consistent
right-hand sides); the solve fixes the gauge by setting the given pinned
pressure unknowns to zero and dropping their (redundant) rows, the gauge the
GPU solver uses, so states can be compared entry by entry.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import PAR


class OracleModel:
    def __init__(self, oracle, pins):
        self.o = oracle
        self.rp, self.ci = oracle.graph()
        n = oracle.ndim
        self.keep = np.setdiff1d(np.arange(n), np.asarray(pins, dtype=np.int64))
        self.J = None
        self.lu = None
        self.solves = 0

    def rhs(self, x):
        return self.o.rhs(x)

    def jacobian(self, x):
        vals, _ = self.o.jacobian(x)
        n = self.o.ndim
        self.J = sp.csr_matrix((vals, self.ci, self.rp), shape=(n, n))
        self.lu = None

    def solve(self, b):
        if self.lu is None:
            Jr = self.J[self.keep][:, self.keep].tocsc()
            self.lu = spla.splu(Jr)
        x = np.zeros(self.o.ndim)
        x[self.keep] = self.lu.solve(np.asarray(b)[self.keep])
        self.solves += 1
        return x

    def set_par(self, idx, v):
        self.o.set_par(idx, v)

    def get_par(self, idx):
        return self.o.get_par(idx)


class MultifrontalModel:
    """F and J from the C++ oracle, solves with the FP64 multifrontal LU of
    oracle.multifrontal (all host cores; sizes where SuperLU is too slow).

    policy "each": every new Jacobian is factorised and solved exactly.
    policy "step": the reference's own preconditioner policy
    (Ocean::preProcess, src/ocean/Ocean.C:799-808, and Ocean::solve,
    Ocean.C:971-1147): the factorisation is rebuilt once per continuation step
    (``pre_process``) and later Jacobians of the step are solved by GMRES
    (restart 100) to ``tol`` preconditioned with it."""

    def __init__(self, oracle, plan, policy="each", tol=1e-8):
        self.o = oracle
        self.plan = plan
        self.rp, self.ci = oracle.graph()
        self.policy = policy
        self.tol = tol
        self.J = None
        self.vals = None
        self.fact = None
        self.fresh = False
        self.solves = 0
        self.factorizations = 0
        self.krylov = 0

    def rhs(self, x):
        return self.o.rhs(x)

    def jacobian(self, x):
        from .multifrontal import Factorization   # noqa: F401
        self.vals, _ = self.o.jacobian(x)
        n = self.o.ndim
        self.J = sp.csr_matrix((self.vals, self.ci, self.rp), shape=(n, n))
        self.fresh = False
        if self.policy == "each":
            self.fact = None

    def pre_process(self):
        self.fact = None

    def solve(self, b):
        from .multifrontal import Factorization
        b = np.asarray(b, dtype=np.float64)
        self.solves += 1
        if self.fact is None:
            self.fact = Factorization(self.plan, self.rp, self.ci, self.vals)
            self.factorizations += 1
            self.fresh = True
        if self.fresh:
            return self.fact.solve(b)
        n = self.o.ndim
        M = spla.LinearOperator((n, n), matvec=self.fact.solve, dtype=np.float64)
        count = [0]

        def cb(_):
            count[0] += 1

        kw = dict(M=M, atol=0.0, restart=100, maxiter=10, callback=cb, callback_type="pr_norm")
        try:
            x, info = spla.gmres(self.J, b, rtol=self.tol, **kw)
        except TypeError:   # scipy < 1.12 names the relative tolerance `tol`
            x, info = spla.gmres(self.J, b, tol=self.tol, **kw)
        self.krylov += count[0]
        return x

    def set_par(self, idx, v):
        self.o.set_par(idx, v)

    def get_par(self, idx):
        return self.o.get_par(idx)


def newton(model, x, max_iters=10, tol=1e-3, backtracking_steps=10):
    """Newton<Model>::Run: returns (x, iters, ||F||, converged)."""
    x = np.array(x, dtype=np.float64)
    F = model.rhs(x)
    norm_rhs = np.linalg.norm(F)
    test = norm_rhs
    for it in range(max_iters):
        model.jacobian(x)
        dx = model.solve(-F)
        x += dx
        F = model.rhs(x)
        test = np.linalg.norm(F)
        if test < tol:
            return x, it + 1, test, True
        if norm_rhs < test:
            reduction = -0.5
            for _ in range(backtracking_steps):
                if test < norm_rhs:
                    break
                x += reduction * dx
                F = model.rhs(x)
                test = np.linalg.norm(F)
                reduction /= 2.0
        norm_rhs = test
    return x, max_iters, test, False


DEFAULTS = dict(par="COMB", ds=1.0e-2, ds_min=1.0e-8, ds_max=1.0e3, decrease=2.0, destination=1.0,
                destination_tol=1.0e-7, max_steps=-1, max_newton=7, min_newton=1, opt_newton=3.5,
                newton_tol=1.0e-4, residual_test="D", normalize="N", tangent="S", initial_tangent="E",
                epsilon=1.0e-5, tan_scaling=1.0, predictor_bound=1.0e3, backtracking_steps=0,
                backtracking_increase=0.0, newton_chord=False, give_up_at_ds_min=True)


class Continuation:
    def __init__(self, model, x, **opts):
        o = dict(DEFAULTS)
        o.update(opts)
        self.o = o
        self.M = model
        self.pidx = PAR[o["par"]] if isinstance(o["par"], str) else int(o["par"])
        self.x = np.array(x, dtype=np.float64)
        self.par = model.get_par(self.pidx)
        self.ds = o["ds"]
        self.ds_start = self.ds
        self.ds0 = self.ds00 = self.ds
        self.par0 = self.par00 = self.par
        self.x0 = self.x.copy()
        self.x00 = self.x.copy()
        n = self.x.size
        self.zeta = 1.0 / n if o["normalize"] == "O" else o["tan_scaling"] / n
        self.pardot = 1.0
        self.pardot0 = 0.0
        self.xdot = np.zeros(n)
        self.xdot0 = np.zeros(n)
        self.F = np.zeros(n)
        self.newton_iter = 0
        self.sum_newton = 0
        self.step = 0
        self.resets = 0
        self.secant = False
        self.fix_step = False
        self.reached = False
        self.abort = False
        self.sign_monitor = 0
        self.history = []   # (par, ||x||) of accepted steps

    def _set_par(self, v):
        self.M.set_par(self.pidx, v)

    def compute_dfdpar(self, fresh):
        if fresh:
            self.F = self.M.rhs(self.x)
        Fc = self.F.copy()
        self._set_par(self.par + self.o["epsilon"])
        Fe = self.M.rhs(self.x)
        self._set_par(self.par)
        return Fc, (Fe - Fc) / self.o["epsilon"]

    def normalize(self):
        if self.o["normalize"] == "O":
            self.zeta = self.o["tan_scaling"] / np.linalg.norm(self.xdot)
            self.xdot = self.xdot * self.zeta
            nrm = np.linalg.norm(self.xdot)
            comb = np.sqrt(nrm * nrm + 1.0)
            self.xdot = self.xdot / comb
            self.pardot = 1.0 / comb
        else:
            nrm = np.linalg.norm(self.xdot)
            comb = np.sqrt(self.zeta * nrm * nrm + 1.0)
            self.pardot = 1.0 / comb
            self.xdot = self.xdot * self.pardot

    def initial_tangent(self):
        _, dfdp = self.compute_dfdpar(True)
        if self.o["initial_tangent"] == "A":
            self.xdot = -dfdp
        else:
            self.M.jacobian(self.x)
            self.xdot = self.M.solve(-dfdp)
        self.normalize()

    def create_tangent(self, mode):
        if mode == "S":
            self.xdot = (self.x - self.x0) / self.ds0
            self.pardot = (self.par - self.par0) / self.ds0
        else:
            if self.o["newton_chord"]:
                _, dfdp = self.compute_dfdpar(True)
                self.M.jacobian(self.x)
                self.xdot = self.M.solve(-dfdp)
            else:
                self.xdot = -self.xdot
            self.normalize()

    def store(self):
        self.x00 = self.x0
        self.x0 = self.x.copy()
        self.xdot0 = self.xdot.copy()
        self.par00, self.par0 = self.par0, self.par
        self.ds00, self.ds0 = self.ds0, self.ds
        self.pardot0 = self.pardot

    def restore(self):
        self.x = self.x0.copy()
        self.par = self.par0
        self._set_par(self.par)
        self.ds = self.ds0
        self.xdot = self.xdot0.copy()
        self.x0 = self.x00
        self.x00 = self.x.copy()
        self.par0 = self.par00
        self.ds0 = self.ds00

    def euler_predictor(self):
        self.x = self.x + self.ds * self.xdot
        self.par = self.par + self.ds * self.pardot
        self._set_par(self.par)
        self.F = self.M.rhs(self.x)
        r = np.linalg.norm(self.F)
        return 1 if (not np.isfinite(r) or r > self.o["predictor_bound"]) else 0

    def newton_corrector(self):
        o = self.o
        res = 100.0
        nx0 = np.linalg.norm(self.x0)
        self.newton_iter = 0
        y = None
        while self.newton_iter < o["max_newton"]:
            Fc, dfdp = self.compute_dfdpar(self.newton_iter == 0)
            norm_rhs = np.linalg.norm(Fc)
            R = -Fc
            diff = self.x - self.x0
            pdiff = self.par - self.par0
            if o["normalize"] == "O":
                rbp = self.ds - np.dot(self.xdot, diff) * self.zeta - self.pardot * pdiff
            else:
                rbp = self.ds * self.ds - np.dot(diff, diff) * self.zeta - pdiff * pdiff
            self.M.jacobian(self.x)
            if not o["newton_chord"]:
                y = self.M.solve(dfdp)
            z = self.M.solve(R)
            if o["normalize"] == "O":
                if o["newton_chord"]:
                    pdir = (rbp - self.zeta * np.dot(self.xdot, z)) / (self.pardot + self.zeta * np.dot(self.xdot, self.xdot))
                else:
                    pdir = (rbp - self.zeta * np.dot(self.xdot, z)) / (self.pardot - self.zeta * np.dot(self.xdot, y))
            else:
                if o["newton_chord"]:
                    pdir = (rbp - 2 * self.zeta * np.dot(diff, z)) / (2 * pdiff + 2 * (self.zeta / pdiff) * np.dot(diff, diff))
                else:
                    pdir = (rbp - 2 * self.zeta * np.dot(diff, z)) / (2 * pdiff - 2 * self.zeta * np.dot(diff, y))
            if o["newton_chord"]:
                z = z + pdir * self.xdot
            else:
                z = z - pdir * y
            self.x = self.x + z
            self.par = self.par + pdir
            self._set_par(self.par)
            self.newton_iter += 1
            self.sum_newton += 1
            self.F = self.M.rhs(self.x)
            test = np.linalg.norm(self.F)
            if not np.isfinite(test) or not np.isfinite(self.par) or test > o["predictor_bound"]:
                return 1
            if o["backtracking_steps"] > 0 and norm_rhs < test:
                reduction = -0.5
                for _ in range(o["backtracking_steps"]):
                    if test < norm_rhs * o["backtracking_increase"]:
                        break
                    self.x = self.x + reduction * z
                    self.par = self.par + reduction * pdir
                    self._set_par(self.par)
                    self.F = self.M.rhs(self.x)
                    test = np.linalg.norm(self.F)
                    reduction /= 2.0
                if test > norm_rhs * o["backtracking_increase"]:
                    return 1
            if np.linalg.norm(z) > 1e3 * nx0 and nx0 > 0:
                return 1
            if o["residual_test"] == "R":
                res = test
            else:
                res = max(abs(pdir), np.max(np.abs(z)))
            if res < o["newton_tol"] and self.newton_iter >= o["min_newton"]:
                break
        if not o["newton_chord"]:
            self.xdot = y
        return 1 if res > o["newton_tol"] else 0

    def do_step(self):
        if hasattr(self.M, "pre_process"):
            self.M.pre_process()   # Ocean::preProcess: a new preconditioner once per step
        if self.euler_predictor():
            return 1
        if self.newton_corrector():
            return 1
        self.create_tangent(self.o["tangent"])
        return 0

    def reset(self):
        self.restore()
        s = np.sign(self.ds) or 1.0
        self.ds = s * max(abs(self.ds) / self.o["decrease"], abs(self.o["ds_min"]))
        self.resets += 1
        self.fix_step = True
        if abs(self.ds) <= abs(self.o["ds_min"]) and (self.resets >= 100 or self.o["give_up_at_ds_min"]):
            self.abort = True

    def detect(self):
        dest = self.o["destination"]
        f0, f1 = self.par0 - dest, self.par - dest
        if self.sign_monitor == 0:
            self.sign_monitor = int(np.sign(f1))
        if self.sign_monitor != int(np.sign(f1)) and not self.secant:
            self.secant = True
            self.ds_start = self.ds
        else:
            self.sign_monitor = int(np.sign(f1))
        if self.secant:
            self.ds = -f1 * self.ds / (f1 - f0)
            self.create_tangent("S")
        if self.secant and abs(f1) < self.o["destination_tol"]:
            self.secant = False
            self.ds = self.ds_start
            self.fix_step = True
            self.reached = True

    def adjust_step(self):
        if self.secant or self.fix_step:
            self.fix_step = False
            return
        factor = min(2.0, max(0.5, self.o["opt_newton"] / self.newton_iter))
        self.ds *= factor
        if abs(self.ds) > abs(self.o["ds_max"]):
            self.ds = np.sign(self.ds) * abs(self.o["ds_max"])
        if abs(self.ds) < abs(self.o["ds_min"]):
            self.ds = np.sign(self.ds) * abs(self.o["ds_min"])

    def run(self):
        self.initial_tangent()
        failed = 0
        while not self.reached and self.step != self.o["max_steps"] and not self.abort:
            self.step += 1
            self.store()
            if self.do_step():
                self.reset()
                failed += 1
                continue
            self.history.append((self.par, float(np.linalg.norm(self.x)), self.newton_iter))
            self.detect()
            self.adjust_step()
        return dict(steps=self.step, failed_steps=failed, newton_iters=self.sum_newton, par=self.par,
                    ds=self.ds, reached_destination=int(self.reached), aborted=int(self.abort))
