"""Gauge of the THCM Jacobian's pressure null space -- TEST INFRASTRUCTURE ONLY.

Restates, for CPU-side exact solves, the rule by which the GPU solver picks
the pressure unknowns it holds at zero: per horizontally connected water
component (columns joined by an active u/v point at any level), two adjacent
surface pressures (a single surface pressure for a one-column component),
plus one surface pressure for every further component of the diagonal
links (i,j)-(i+1,j+1), (i+1,j)-(i,j+1) of active velocity points (a region
joined to its basin through a single velocity point keeps a checkerboard
mode of its own).
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

    # diagonal components: the B-grid pressure gradient at an active velocity
    # point vanishes iff p(i,j) = p(i+1,j+1) and p(i+1,j) = p(i,j+1), so the
    # null modes are constant on the components of these diagonal links
    dparent = np.arange(n * m)

    def dfind(a):
        while dparent[a] != a:
            dparent[a] = dparent[dparent[a]]
            a = dparent[a]
        return a

    uv_point = uv_active.any(axis=0)                            # [j][i]: NE corner of cell (i, j)
    for j in range(m):
        for i in range(n):
            ie = (i + 1) % n if periodic else i + 1
            if ie >= n or j + 1 >= m or not uv_point[j, i]:
                continue
            dparent[dfind(i + n * j)] = dfind(ie + n * (j + 1))
            dparent[dfind(ie + n * j)] = dfind(i + n * (j + 1))

    pins = []
    pinned = set()

    def pin(c):
        r = dfind(c)
        if r not in pinned:
            pinned.add(r)
            pins.append(grow(c % n, c // n, l - 1))

    for r in order:
        K = comps[r]
        inset = set(K)
        done = False
        for c in K:
            i, j = c % n, c // n
            iw = (i - 1 + n) % n if periodic else i - 1
            if iw >= 0 and (iw + n * j) in inset:
                pin(c)
                pin(iw + n * j)
                done = True
                break
        if not done:
            for c in K:
                i, j = c % n, c // n
                if j > 0 and (i + n * (j - 1)) in inset:
                    pin(c)
                    pin(i + n * (j - 1))
                    done = True
                    break
        if not done:
            pin(K[0])
        for c in K:          # diagonal components the pair left unpinned
            pin(c)
    return pins
