"""CPU nested-dissection multifrontal LU of the THCM Jacobian -- TEST INFRASTRUCTURE ONLY.

The CPU side of the linear solve, for the CPU baseline and as an exact
reference solver at sizes where scipy's SuperLU is too slow: an FP64
multifrontal LU over water columns with LAPACK (getrf with partial pivoting
inside each front's fully summed block, trsm/gemm for the Schur complement)
on all host cores through numpy/scipy.

Ordering: every water column's unknowns (levels k, then u,v,w,p,T,S) stay
together; the horizontal grid is bisected recursively (the longer side
first, down to leaves of at most 4 columns); a periodic domain is cut first
by the columns i = 0 and i = n/2. Identity rows (land, Dirichlet velocities,
boundary.F90) pass the right-hand side through, the gauge pressures of
``gauge.gauge_pins`` are held at zero with their rows dropped, and the
surface pressure of every other water column is ordered into the root front
so that no subdomain block inherits a barotropic null mode.
"""
import numpy as np
import scipy.linalg as sla

from .gauge import gauge_pins

OCEAN, LAND = 0, 1


class Plan:
    def __init__(self, landm, n, m, l, periodic, leaf=4):
        self.n, self.m, self.l = n, m, l
        ndim = 6 * n * m * l
        self.ndim = ndim
        LM = np.asarray(landm).reshape(l + 2, m + 2, n + 2)

        def g(i, j, k, t):
            return 6 * (i + n * (j + m * k)) + t

        dry = np.zeros(ndim, dtype=bool)
        for k in range(1, l + 1):
            for j in range(1, m + 1):
                for i in range(1, n + 1):
                    b = g(i - 1, j - 1, k - 1, 0)
                    if LM[k, j, i] != OCEAN:
                        dry[b:b + 6] = True
                        continue
                    if LM[k, j + 1, i] == LAND or LM[k, j, i + 1] == LAND or LM[k, j + 1, i + 1] == LAND:
                        dry[b] = dry[b + 1] = True
                    if LM[k + 1, j, i] == LAND:
                        dry[b + 2] = True
        self.identity = np.nonzero(dry)[0]
        self.pins = np.array(gauge_pins(landm, n, m, l, periodic), dtype=np.int64)
        dry[self.pins] = True
        ocean = LM[l, 1:m + 1, 1:n + 1] == OCEAN
        surf = set(g(i, j, l - 1, 3) for j in range(m) for i in range(n) if ocean[j, i] and not dry[g(i, j, l - 1, 3)])
        colvars = {}
        for j in range(m):
            for i in range(n):
                colvars[i + n * j] = [g(i, j, k, t) for k in range(l) for t in range(6)
                                      if not dry[g(i, j, k, t)] and g(i, j, k, t) not in surf]
        nodes = []

        def rec(i0, i1, j0, j1):
            W, H = i1 - i0, j1 - j0
            if W <= 0 or H <= 0:
                return -1
            ch = []
            if W * H <= leaf:
                cols = [(i % n) + n * j for j in range(j0, j1) for i in range(i0, i1)]
            elif W >= H:
                im = i0 + W // 2
                ch = [rec(i0, im, j0, j1), rec(im + 1, i1, j0, j1)]
                cols = [(im % n) + n * j for j in range(j0, j1)]
            else:
                jm = j0 + H // 2
                ch = [rec(i0, i1, j0, jm), rec(i0, i1, jm + 1, j1)]
                cols = [(i % n) + n * jm for i in range(i0, i1)]
            ch = [c for c in ch if c >= 0]
            nodes.append(dict(cols=cols, reg=(i0, i1, j0, j1), ch=ch))
            return len(nodes) - 1

        if periodic:
            h = n // 2
            kids = [c for c in (rec(1, h, 0, m), rec(h + 1, n, 0, m)) if c >= 0]
            nodes.append(dict(cols=[n * j for j in range(m)] + [h + n * j for j in range(m)], reg=(0, n, 0, m),
                              ch=kids))
        else:
            rec(0, n, 0, m)
        root = len(nodes) - 1
        g2r = -np.ones(ndim, dtype=np.int64)
        r2g = []
        for f, nd in enumerate(nodes):
            nd["red0"] = len(r2g)
            own = [gg for c in nd["cols"] for gg in colvars[c]]
            if f == root:
                own += sorted(surf)
            for gg in own:
                g2r[gg] = len(r2g)
                r2g.append(gg)
            nd["nf"] = len(r2g) - nd["red0"]
        for f, nd in enumerate(nodes):
            if f == root:
                nd["B"] = np.zeros(0, dtype=np.int64)
                continue
            i0, i1, j0, j1 = nd["reg"]
            ring, region = set(), set()
            for j in range(j0 - 1, j1 + 1):
                for i in range(i0 - 1, i1 + 1):
                    if j < 0 or j >= m:
                        continue
                    if periodic:
                        ii = i % n
                    elif i < 0 or i >= n:
                        continue
                    else:
                        ii = i
                    (region if (i0 <= i < i1 and j0 <= j < j1) else ring).add(ii + n * j)
            B = [g2r[gg] for c in ring for gg in colvars[c]]
            B += [g2r[g(c % n, c // n, l - 1, 3)] for c in region | ring if g(c % n, c // n, l - 1, 3) in surf]
            nd["B"] = np.array(sorted(set(B)), dtype=np.int64)
        self.nodes = nodes
        self.g2r = g2r
        self.r2g = np.array(r2g, dtype=np.int64)
        self.nred = len(r2g)
        self.owner = np.empty(self.nred, dtype=np.int64)
        for f, nd in enumerate(nodes):
            self.owner[nd["red0"]:nd["red0"] + nd["nf"]] = f
        self.flops = sum(2.0 / 3 * nd["nf"] ** 3 + 2.0 * nd["nf"] ** 2 * len(nd["B"]) + 2.0 * nd["nf"] * len(nd["B"]) ** 2
                         for nd in nodes)


def _perm_of(piv):
    """Row order after LAPACK's sequential interchanges i <-> piv[i]."""
    perm = np.arange(len(piv))
    for i, p in enumerate(piv):
        if p != i:
            perm[i], perm[p] = perm[p], perm[i]
    return perm


class Factorization:
    """FP64 multifrontal LU of the pinned, wet part of J (CSR arrays)."""

    def __init__(self, plan, row_ptr, col_idx, values):
        P = self.plan = plan
        rp = np.asarray(row_ptr, dtype=np.int64)
        ci = np.asarray(col_idx, dtype=np.int64)
        va = np.asarray(values, dtype=np.float64)
        self.rp, self.ci, self.va = rp, ci, va
        rows = np.repeat(np.arange(P.ndim), np.diff(rp))
        rr, rc = P.g2r[rows], P.g2r[ci]
        keep = (rr >= 0) & (rc >= 0)
        rr, rc, vv = rr[keep], rc[keep], va[keep]
        f_of = P.owner[np.minimum(rr, rc)]
        order = np.argsort(f_of, kind="stable")
        rr, rc, vv, f_of = rr[order], rc[order], vv[order], f_of[order]
        bounds = np.searchsorted(f_of, np.arange(len(P.nodes) + 1))
        self.lu, self.piv, self.L21, self.U12 = [], [], [], []
        schur = [None] * len(P.nodes)
        for f, nd in enumerate(P.nodes):
            nf, B = nd["nf"], nd["B"]
            Fd = nf + len(B)
            A = np.zeros((Fd, Fd))
            s0, s1 = bounds[f], bounds[f + 1]
            A[self._local(nd, rr[s0:s1]), self._local(nd, rc[s0:s1])] = vv[s0:s1]
            for c in nd["ch"]:
                em = self._local(nd, P.nodes[c]["B"])
                A[np.ix_(em, em)] += schur[c]
                schur[c] = None
            lu, piv = sla.lu_factor(A[:nf, :nf], check_finite=False)
            # U12 = L11^{-1} P^T A12 and L21 = A21 U11^{-1}
            perm = _perm_of(piv)
            U12 = sla.solve_triangular(lu, A[:nf, nf:][perm], lower=True, unit_diagonal=True, check_finite=False)
            L21 = sla.solve_triangular(lu, A[nf:, :nf].T, trans="T", lower=False, check_finite=False).T
            S = A[nf:, nf:]
            S -= L21 @ U12
            schur[f] = S
            self.lu.append(lu)
            self.piv.append(perm)
            self.L21.append(L21)
            self.U12.append(U12)

    @staticmethod
    def _local(nd, red):
        red = np.asarray(red, dtype=np.int64)
        own = (red >= nd["red0"]) & (red < nd["red0"] + nd["nf"])
        out = np.empty(red.shape, dtype=np.int64)
        out[own] = red[own] - nd["red0"]
        if (~own).any():
            out[~own] = nd["nf"] + np.searchsorted(nd["B"], red[~own])
        return out

    def solve(self, b):
        """x with J x = b (consistent b), pins at zero, identity rows x = b."""
        P = self.plan
        b = np.asarray(b, dtype=np.float64)
        x = np.zeros(P.ndim)
        x[P.identity] = b[P.identity]
        # r = b - J[:, identity] b[identity] on the reduced unknowns
        rows = np.repeat(np.arange(P.ndim), np.diff(self.rp))
        isid = np.zeros(P.ndim, dtype=bool)
        isid[P.identity] = True
        sel = isid[self.ci]
        corr = np.bincount(rows[sel], weights=self.va[sel] * b[self.ci[sel]], minlength=P.ndim)
        red = (b - corr)[P.r2g]
        for f, nd in enumerate(P.nodes):
            s = slice(nd["red0"], nd["red0"] + nd["nf"])
            y = red[s][self.piv[f]]
            y = sla.solve_triangular(self.lu[f], y, lower=True, unit_diagonal=True, check_finite=False)
            red[s] = y
            if len(nd["B"]):
                red[nd["B"]] -= self.L21[f] @ y
        for f in range(len(P.nodes) - 1, -1, -1):
            nd = P.nodes[f]
            s = slice(nd["red0"], nd["red0"] + nd["nf"])
            y = red[s]
            if len(nd["B"]):
                y = y - self.U12[f] @ red[nd["B"]]
            red[s] = sla.solve_triangular(self.lu[f], y, lower=False, check_finite=False)
        x[P.r2g] = red
        return x
