"""Gauge of the THCM Jacobian's pressure null space -- TEST INFRASTRUCTURE ONLY.

Restates, for CPU-side exact solves, the rule by which the GPU solver picks
the pressure unknowns it holds at zero: per horizontally connected water
component (columns joined by an active u/v point at any level), two adjacent
surface pressures (a single surface pressure for a one-column component).
Dry u/v points are those boundaries() turns into identity rows
(src/ocean/boundary.F90): land cells, and velocities next to land to the
north/east/north-east.
"""
import numpy as np

OCEAN, LAND = 0, 1


def gauge_pins(landm, n, m, l, periodic):
    LM = np.asarray(landm).reshape(l + 2, m + 2, n + 2)    # [k][j][i]
    wet = LM[1:l + 1, 1:m + 1, 1:n + 1] == OCEAN               # [k][j][i], 0-based
    land_n = LM[1:l + 1, 2:m + 2, 1:n + 1] == LAND
    land_e = LM[1:l + 1, 1:m + 1, 2:n + 2] == LAND
    land_ne = LM[1:l + 1, 2:m + 2, 2:n + 2] == LAND
    uv_active = wet & ~(land_n | land_e | land_ne)
    ocean_col = wet[l - 1]                                      # [j][i]
    uv_col = uv_active.any(axis=0)
    parent = np.arange(n * m)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for j in range(m):
        for i in range(n):
            if not uv_col[j, i]:
                continue
            for di, dj in ((1, 0), (0, 1), (1, 1)):
                ii, jj = i + di, j + dj
                if periodic:
                    ii %= n
                if ii >= n or jj >= m or not ocean_col[jj, ii]:
                    continue
                parent[find(i + n * j)] = find(ii + n * jj)
    comps = {}
    for j in range(m - 1, -1, -1):
        for i in range(n - 1, -1, -1):
            if ocean_col[j, i]:
                comps.setdefault(find(i + n * j), []).append(i + n * j)
    order = sorted(comps, key=lambda r: r)   # the GPU walks components by root index

    def grow(i, j, k):
        return 6 * (i + n * (j + m * k)) + 3

    pins = []
    for r in order:
        K = comps[r]
        inset = set(K)
        done = False
        for c in K:
            i, j = c % n, c // n
            iw = (i - 1 + n) % n if periodic else i - 1
            if iw >= 0 and (iw + n * j) in inset:
                pins += [grow(i, j, l - 1), grow(iw, j, l - 1)]
                done = True
                break
        if not done:
            for c in K:
                i, j = c % n, c // n
                if j > 0 and (i + n * (j - 1)) in inset:
                    pins += [grow(i, j, l - 1), grow(i, j - 1, l - 1)]
                    done = True
                    break
        if not done:
            pins.append(grow(K[0] % n, K[0] // n, l - 1))
    return pins
