// Nested-dissection multilevel block LU of the THCM Jacobian.
//
// The reference preconditions its FGMRES with an ILU/MRILU-based block
// scheme (src/trios/TRIOS_BlockPreconditioner.C, src/mrilucpp). On the full
// saddle-point Jacobian, zero-fill ILU variants do not converge (W and P rows
// have zero diagonals, and the B-grid pressure has constant and checkerboard
// null modes). This preconditioner therefore follows MRILU's multilevel idea
// with drop tolerance 0: eliminate an independent set, form the Schur
// complement, recurse. The independent sets come from a nested dissection of
// the grid's water columns. Each elimination tree node is a dense frontal
// matrix: batched panel LU with block-local partial pivoting, tiled GEMM
// Schur updates and extend-add into the parent.
//
// Three kinds of unknowns are left out of the factorisation: unknowns whose
// Jacobian rows are identities (land cells, velocity points next to land,
// surface w; src/ocean/boundary.F90), and two pinned pressures per surface
// basin, the rows src/ocean/THCM.C:2260-2297 (fixPressurePoints) would
// replace. So the factor preconditions the original, singular-but-consistent
// J.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <numeric>
#include <unordered_map>

#include "engine.cuh"
#include "ndlu.cuh"
#include "ktimer.cuh"
#include "stencil.cuh"

namespace iemic {

// ===========================================================================
// symbolic analysis (host, once per land mask)
// ===========================================================================
namespace {

struct Node {
    std::vector<int> cols;        // own water columns (i + n*j)
    int i0, i1, j0, j1;           // region of the subtree
    int child[2] = {-1, -1};
    int nchild = 0;
    int parent = -1;
    int height = 0;
};

}  // namespace

void build_nd_plan(NdPlan& plan, int n, int m, int l, int periodic, const std::vector<int>& landm,
                   const std::vector<int>& row_ptr, const std::vector<int>& col_idx, int panel,
                   const std::vector<int>& identity_rows, const std::vector<int>& fixed_pressures) {
    plan = NdPlan();
    plan.panel = panel;
    const int ndim = NUN * n * m * l;
    plan.ndim = ndim;
    auto LM = [&](int i, int j, int k) { return landm[i + (n + 2) * (j + (m + 2) * k)]; };
    auto grow = [&](int i, int j, int k, int t) { return NUN * (i + n * (j + m * k)) + t; };   // 0-based

    // 1. dry unknowns: identity rows made by boundaries() (src/ocean/boundary.F90)
    std::vector<char> dry(ndim, 0);
    for (int k = 1; k <= l; ++k)
        for (int j = 1; j <= m; ++j)
            for (int i = 1; i <= n; ++i) {
                int base = grow(i - 1, j - 1, k - 1, 0);
                if (LM(i, j, k) != OCEAN) {
                    for (int t = 0; t < NUN; ++t) dry[base + t] = 1;
                    continue;
                }
                if (LM(i, j + 1, k) == LAND || LM(i + 1, j, k) == LAND || LM(i + 1, j + 1, k) == LAND) {
                    dry[base + 0] = 1;
                    dry[base + 1] = 1;
                }
                if (LM(i, j, k + 1) == LAND) dry[base + 2] = 1;
            }
    // rows the factorisation takes as identity rows: the integral condition
    // (its dense row is restored by the solve phase's Sherman-Morrison step)
    for (int r : identity_rows)
        if (r >= 0 && r < ndim) dry[r] = 1;
    // 2. barotropic pressure of every water column. A column's pressures are
    //    tied together by its hydrostatic w rows, so one pressure per column (at
    //    the surface) carries its depth-independent mode; that mode couples
    //    only through horizontal velocity points. Columns are connected when
    //    an active velocity point (any level) touches both. Per connected
    //    component, two adjacent surface pressures (one for a single column)
    //    are pinned, as THCM's fixPressurePoints rows would pin them
    //    (src/ocean/THCM.C:2260-2297): this removes the constant and
    //    checkerboard null modes of J from the preconditioner.
    //    The B-grid gradient at an active velocity point vanishes exactly when
    //    the two diagonal pairs of its four columns carry equal pressures, so
    //    the null modes are the functions constant on the components of the
    //    "diagonal" graph (edges (i,j)-(i+1,j+1) and (i+1,j)-(i,j+1) per active
    //    point). A basin usually splits into two such components (constant and
    //    checkerboard); where a region hangs on through a single velocity point
    //    its checkerboard is separate, and any component the adjacent pair
    //    leaves unpinned gets a pin of its own.
    std::vector<char> ocean_col(size_t(n) * m, 0), uv_col(size_t(n) * m, 0);
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
            ocean_col[i + n * j] = LM(i + 1, j + 1, l) == OCEAN;
            for (int k = 0; k < l; ++k)
                if (!dry[grow(i, j, k, 0)] || !dry[grow(i, j, k, 1)]) uv_col[i + n * j] = 1;
        }
    {
        std::vector<int> uf(size_t(n) * m);
        std::iota(uf.begin(), uf.end(), 0);
        std::function<int(int)> find = [&](int a) {
            while (uf[a] != a) { uf[a] = uf[uf[a]]; a = uf[a]; }
            return a;
        };
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n; ++i) {
                if (!uv_col[i + n * j]) continue;
                const int di[3] = {1, 0, 1}, dj[3] = {0, 1, 1};
                for (int d = 0; d < 3; ++d) {
                    int ii = i + di[d], jj = j + dj[d];
                    if (periodic) ii %= n;
                    if (ii >= n || jj >= m || !ocean_col[ii + n * jj]) continue;
                    uf[find(i + n * j)] = find(ii + n * jj);
                }
            }
        // diagonal components
        std::vector<int> dg(size_t(n) * m);
        std::iota(dg.begin(), dg.end(), 0);
        std::function<int(int)> dfind = [&](int a) {
            while (dg[a] != a) { dg[a] = dg[dg[a]]; a = dg[a]; }
            return a;
        };
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < n; ++i) {
                int ie = i + 1;
                if (periodic) ie %= n;
                if (ie >= n || j + 1 >= m) continue;
                bool active = false;
                for (int k = 0; k < l && !active; ++k) active = !dry[grow(i, j, k, 0)];
                if (!active) continue;
                dg[dfind(i + n * j)] = dfind(ie + n * (j + 1));
                dg[dfind(ie + n * j)] = dfind(i + n * (j + 1));
            }
        std::vector<char> dpinned(size_t(n) * m, 0);
        auto pin = [&](int c) {
            if (dpinned[dfind(c)]) return;
            dpinned[dfind(c)] = 1;
            plan.pins.push_back(grow(c % n, c / n, l - 1, PP - 1));
        };
        // surface pressures the model itself fixes ("Fix Pressure Points":
        // identity rows of J, passed in identity_rows) already remove the
        // null modes of their components: no gauge pin there
        for (int r : fixed_pressures) {
            if (r < 0 || r >= ndim || r % NUN != PP - 1) continue;
            const int cell = r / NUN, ci0 = cell % n, cj0 = (cell / n) % m, ck0 = cell / (n * m);
            if (ck0 != l - 1 || !ocean_col[ci0 + n * cj0]) continue;
            dpinned[dfind(ci0 + n * cj0)] = 1;
        }
        std::vector<std::vector<int>> comps(size_t(n) * m);
        for (int j = m - 1; j >= 0; --j)      // scan from the north-east corner
            for (int i = n - 1; i >= 0; --i)
                if (ocean_col[i + n * j]) comps[find(i + n * j)].push_back(i + n * j);
        for (auto& K : comps) {
            if (K.empty()) continue;
            std::vector<char> in(size_t(n) * m, 0);
            for (int c : K) in[c] = 1;
            bool done = false;
            for (int c : K) {   // a horizontally adjacent pair first
                int i = c % n, j = c / n, iw = periodic ? (i - 1 + n) % n : i - 1;
                if (iw >= 0 && in[iw + n * j]) {
                    pin(c);
                    pin(iw + n * j);
                    done = true;
                    break;
                }
            }
            for (size_t q = 0; q < K.size() && !done; ++q) {
                int i = K[q] % n, j = K[q] / n;
                if (j > 0 && in[i + n * (j - 1)]) {
                    pin(K[q]);
                    pin(i + n * (j - 1));
                    done = true;
                }
            }
            if (!done) pin(K[0]);
            for (int c : K) pin(c);   // components the pair left unpinned
        }
        for (int p : plan.pins) dry[p] = 1;
    }
    for (int r = 0; r < ndim; ++r)
        if (dry[r]) plan.dry_rows.push_back(r);
    // deferred unknowns: the surface pressure of every (unpinned) water column
    // is eliminated in the root front, so no subdomain block contains a
    // floating barotropic pressure mode. (Deferring only a coarse lattice of
    // them leaves subdomain blocks that block-local pivoting cannot factor:
    // their pivots break down even in FP64.)
    std::vector<char> deferred(ndim, 0);
    std::vector<int> deferred_list;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
            int g = grow(i, j, l - 1, PP - 1);
            if (ocean_col[i + n * j] && !dry[g]) {
                deferred[g] = 1;
                deferred_list.push_back(g);
            }
        }

    // 3. wet unknowns per water column, ordered (k, t)
    std::vector<std::vector<int>> colvars(size_t(n) * m);
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < l; ++k)
                for (int t = 0; t < NUN; ++t) {
                    int g = grow(i, j, k, t);
                    if (!dry[g] && !deferred[g]) colvars[i + n * j].push_back(g);
                }

    // 4. nested dissection of the column grid (postorder)
    std::vector<Node> nodes;
    const int LEAF = 4;
    std::function<int(int, int, int, int)> rec = [&](int i0, int i1, int j0, int j1) -> int {
        int W = i1 - i0, H = j1 - j0;
        if (W <= 0 || H <= 0) return -1;
        Node nd;
        nd.i0 = i0; nd.i1 = i1; nd.j0 = j0; nd.j1 = j1;
        int c0 = -1, c1 = -1;
        if (W * H <= LEAF) {
            for (int j = j0; j < j1; ++j)
                for (int i = i0; i < i1; ++i) nd.cols.push_back(((i % n) + n) % n + n * j);
        } else if (W >= H) {
            int im = i0 + W / 2;
            c0 = rec(i0, im, j0, j1);
            c1 = rec(im + 1, i1, j0, j1);
            for (int j = j0; j < j1; ++j) nd.cols.push_back(((im % n) + n) % n + n * j);
        } else {
            int jm = j0 + H / 2;
            c0 = rec(i0, i1, j0, jm);
            c1 = rec(i0, i1, jm + 1, j1);
            for (int i = i0; i < i1; ++i) nd.cols.push_back(((i % n) + n) % n + n * jm);
        }
        for (int c : {c0, c1})
            if (c >= 0) nd.child[nd.nchild++] = c;
        nodes.push_back(nd);
        int id = int(nodes.size()) - 1;
        for (int q = 0; q < nodes[id].nchild; ++q) nodes[nodes[id].child[q]].parent = id;
        return id;
    };
    int root = -1;
    if (periodic) {
        int h = n / 2;
        int c0 = rec(1, h, 0, m);
        int c1 = rec(h + 1, n, 0, m);
        Node nd;
        nd.i0 = 0; nd.i1 = n; nd.j0 = 0; nd.j1 = m;
        for (int j = 0; j < m; ++j) nd.cols.push_back(0 + n * j);
        for (int j = 0; j < m; ++j) nd.cols.push_back(h + n * j);
        for (int c : {c0, c1})
            if (c >= 0) nd.child[nd.nchild++] = c;
        nodes.push_back(nd);
        root = int(nodes.size()) - 1;
        for (int q = 0; q < nodes[root].nchild; ++q) nodes[nodes[root].child[q]].parent = root;
    } else {
        root = rec(0, n, 0, m);
    }
    const int NF = int(nodes.size());
    for (int f = 0; f < NF; ++f) {   // postorder: children precede parents
        int h = 0;
        for (int q = 0; q < nodes[f].nchild; ++q) h = std::max(h, nodes[nodes[f].child[q]].height + 1);
        nodes[f].height = h;
    }

    // 5. reduced ordering: own unknowns of the fronts in postorder
    plan.g2r.assign(ndim, -1);
    plan.fronts.resize(NF);
    std::vector<int> owner;
    for (int f = 0; f < NF; ++f) {
        FrontDev& fr = plan.fronts[f];
        fr.red0 = int(plan.r2g.size());
        std::vector<int> own;
        for (int c : nodes[f].cols)
            for (int g : colvars[c]) own.push_back(g);
        if (f == root) own.insert(own.end(), deferred_list.begin(), deferred_list.end());
        for (int g : own) {
            plan.g2r[g] = int(plan.r2g.size());
            plan.r2g.push_back(g);
            owner.push_back(f);
        }
        fr.nf = int(plan.r2g.size()) - fr.red0;
        fr.parent = nodes[f].parent;
    }
    plan.nred = int(plan.r2g.size());
    // couplings of the reduced rows to identity (dry, unpinned) unknowns, in
    // CSR order: the right-hand side reduction subtracts only these
    {
        std::vector<char> ident(ndim, 0);
        for (int r : plan.dry_rows) ident[r] = 1;
        for (int p : plan.pins) ident[p] = 0;
        plan.dry_ptr.assign(1, 0);
        for (int q = 0; q < plan.nred; ++q) {
            const int g = plan.r2g[q];
            for (int e = row_ptr[g]; e < row_ptr[g + 1]; ++e)
                if (ident[col_idx[e]]) {
                    plan.dry_e.push_back(e);
                    plan.dry_c.push_back(col_idx[e]);
                }
            plan.dry_ptr.push_back(int(plan.dry_e.size()));
        }
    }

    // 6. boundary unknowns: the non-deferred unknowns of the ring of columns
    //    around the subtree region, plus the deferred surface pressures of the
    //    region and the ring (all owned by ancestors), sorted by reduced index
    std::vector<std::vector<int>> bvars(NF);
    for (int f = 0; f < NF; ++f) {
        if (nodes[f].parent < 0) continue;
        const Node& nd = nodes[f];
        std::vector<int> ring, region;
        for (int j = nd.j0 - 1; j <= nd.j1; ++j)
            for (int i = nd.i0 - 1; i <= nd.i1; ++i) {
                if (j < 0 || j >= m) continue;
                int ii = i;
                if (periodic) ii = (i % n + n) % n;
                else if (i < 0 || i >= n) continue;
                bool inside = i >= nd.i0 && i < nd.i1 && j >= nd.j0 && j < nd.j1;
                (inside ? region : ring).push_back(ii + n * j);
            }
        std::sort(ring.begin(), ring.end());
        ring.erase(std::unique(ring.begin(), ring.end()), ring.end());
        for (int c : ring)
            for (int g : colvars[c]) bvars[f].push_back(plan.g2r[g]);
        for (auto* cols : {&region, &ring})
            for (int c : *cols) {
                int g = grow(c % n, c / n, l - 1, PP - 1);
                if (deferred[g]) bvars[f].push_back(plan.g2r[g]);
            }
        std::sort(bvars[f].begin(), bvars[f].end());
        bvars[f].erase(std::unique(bvars[f].begin(), bvars[f].end()), bvars[f].end());
    }
    auto local = [&](int f, int red) -> int {
        const FrontDev& fr = plan.fronts[f];
        if (red >= fr.red0 && red < fr.red0 + fr.nf) return red - fr.red0;
        auto it = std::lower_bound(bvars[f].begin(), bvars[f].end(), red);
        if (it == bvars[f].end() || *it != red) return -1;
        return fr.nf + int(it - bvars[f].begin());
    };

    // 7. offsets, var lists, extend-add maps
    int64_t off = 0, dinv = 0, voff = 0, eoff = 0, woff = 0;
    plan.child_slot.assign(NF, -1);
    for (int f = 0; f < NF; ++f) {
        FrontDev& fr = plan.fronts[f];
        fr.nb = int(bvars[f].size());
        fr.F = fr.nf + fr.nb;
        fr.lvl = nodes[f].height;
        off += int64_t(fr.F) * fr.F;
        fr.foff = plan.factor_entries;   // before this front's entries are counted below
        fr.dinv_off = dinv;
        dinv += int64_t((fr.nf + panel - 1) / panel) * 2 * panel * panel;
        fr.voff = voff;
        voff += fr.F;
        for (int q = 0; q < fr.nf; ++q) plan.vars.push_back(fr.red0 + q);
        for (int r : bvars[f]) plan.vars.push_back(r);
        fr.woff = woff;
        woff += fr.F;
        fr.emap_off = eoff;
        for (int q = 0; q < nodes[f].nchild; ++q) plan.child_slot[nodes[f].child[q]] = q;
        const double a = fr.nf, b = fr.nb;
        plan.flops += 2.0 / 3.0 * a * a * a + 2.0 * a * a * b + 2.0 * a * b * b;
        plan.factor_entries += int64_t(fr.nf) * fr.nf + 2 * int64_t(fr.nf) * fr.nb;
    }
    for (int f = 0; f < NF; ++f) {
        FrontDev& fr = plan.fronts[f];
        fr.emap_off = eoff;
        if (fr.parent >= 0)
            for (int r : bvars[f]) {
                int loc = local(fr.parent, r);
                if (loc < 0) throw EngineError(IEMIC_ERR_STATE);   // broken tree invariant
                plan.emap.push_back(loc);
                ++eoff;
            }
    }
    plan.front_entries = off;
    plan.dinv_entries = dinv;
    plan.emap_entries = eoff;
    plan.w_entries = woff;
    plan.nfronts = NF;

    // 8. levels by height; children lists per parent level and slot
    int H = 0;
    for (int f = 0; f < NF; ++f) H = std::max(H, nodes[f].height + 1);
    plan.nlevels = H;
    plan.level_fronts.assign(H, {});
    plan.level_children[0].assign(H, {});
    plan.level_children[1].assign(H, {});
    for (int f = 0; f < NF; ++f) plan.level_fronts[nodes[f].height].push_back(f);
    for (int f = 0; f < NF; ++f)
        if (nodes[f].parent >= 0)
            plan.level_children[plan.child_slot[f]][nodes[nodes[f].parent].height].push_back(f);
    plan.level_maxnf.assign(H, 0);
    plan.level_maxF.assign(H, 0);
    for (int h = 0; h < H; ++h)
        for (int f : plan.level_fronts[h]) {
            plan.level_maxnf[h] = std::max(plan.level_maxnf[h], plan.fronts[f].nf);
            plan.level_maxF[h] = std::max(plan.level_maxF[h], plan.fronts[f].F);
        }
    // working offsets (per level, from 0) and contribution-ring offsets
    int gap = 1;
    for (int f = 0; f < NF; ++f)
        if (plan.fronts[f].parent >= 0) gap = std::max(gap, plan.fronts[plan.fronts[f].parent].lvl - plan.fronts[f].lvl);
    plan.contrib_ring = gap + 1;
    plan.level_work.assign(H, 0);
    std::vector<int64_t> level_contrib(H, 0);
    for (int h = 0; h < H; ++h)
        for (int f : plan.level_fronts[h]) {
            FrontDev& fr = plan.fronts[f];
            fr.off = plan.level_work[h];
            plan.level_work[h] += int64_t(fr.F) * fr.F;
            fr.soff = level_contrib[h];
            level_contrib[h] += int64_t(fr.nb) * fr.nb;
        }
    for (int h = 0; h < H; ++h) {
        plan.work_entries = std::max(plan.work_entries, plan.level_work[h]);
        plan.contrib_slot_entries = std::max(plan.contrib_slot_entries, level_contrib[h]);
    }
    for (int f = 0; f < NF; ++f) plan.fronts[f].soff += (plan.fronts[f].lvl % plan.contrib_ring) * plan.contrib_slot_entries;

    // 9. assembly map: entry (r, c) goes to the front that eliminates the
    //    earlier of its two unknowns; entries grouped by level (each level
    //    is assembled into the working area when its turn comes)
    std::vector<int64_t> per_level(H, 0);
    std::vector<int> ent_front;
    std::vector<int> ent_q, ent_r;
    std::vector<int64_t> ent_dst;
    for (int r = 0; r < ndim; ++r) {
        int rr = plan.g2r[r];
        if (rr < 0) continue;
        for (int q = row_ptr[r]; q < row_ptr[r + 1]; ++q) {
            int rc = plan.g2r[col_idx[q]];
            if (rc < 0) continue;
            int f = owner[std::min(rr, rc)];
            int lr = local(f, rr), lc = local(f, rc);
            if (lr < 0 || lc < 0) throw EngineError(IEMIC_ERR_STATE);
            const FrontDev& fr = plan.fronts[f];
            ent_q.push_back(q);
            ent_r.push_back(r);
            ent_dst.push_back(fr.off + int64_t(lc) * fr.F + lr);
            ent_front.push_back(fr.lvl);
            per_level[fr.lvl] += 1;
        }
    }
    plan.asm_level_start.assign(H + 1, 0);
    for (int h = 0; h < H; ++h) plan.asm_level_start[h + 1] = plan.asm_level_start[h] + per_level[h];
    const size_t na = ent_q.size();
    plan.asm_src.resize(na);
    plan.asm_row.resize(na);
    plan.asm_dst.resize(na);
    std::vector<int64_t> fill(plan.asm_level_start.begin(), plan.asm_level_start.end() - 1);
    for (size_t e = 0; e < na; ++e) {
        const int64_t d = fill[ent_front[e]]++;
        plan.asm_src[d] = ent_q[e];
        plan.asm_row[d] = ent_r[e];
        plan.asm_dst[d] = ent_dst[e];
    }
    check_nd_plan(plan);
}

// Every offset and index the numeric kernels derive from the plan stays
// inside its buffer: fronts in the working area of their level, the factor
// store and the contribution ring, solve vectors, inverse panel blocks,
// extend-add maps in the parent, assembly targets, the reduced ordering.
// Throws IEMIC_ERR_STATE otherwise.
void check_nd_plan(const NdPlan& P) {
    auto req = [](bool ok) {
        if (!ok) throw EngineError(IEMIC_ERR_STATE);
    };
    int64_t fsum = 0;
    int roots = 0;
    req(int(P.fronts.size()) == P.nfronts && int(P.level_work.size()) == P.nlevels);
    req(int(P.asm_level_start.size()) == P.nlevels + 1 && P.contrib_ring >= 1);
    for (int q = 0; q < P.nfronts; ++q) {
        const FrontDev& fr = P.fronts[q];
        req(fr.nf >= 0 && fr.nb >= 0 && fr.F == fr.nf + fr.nb && fr.lvl >= 0 && fr.lvl < P.nlevels);
        req(fr.foff == fsum);
        fsum += int64_t(fr.nf) * fr.nf + 2 * int64_t(fr.nf) * fr.nb;
        req(fr.off >= 0 && fr.off + int64_t(fr.F) * fr.F <= P.level_work[fr.lvl]);
        req(P.level_work[fr.lvl] <= P.work_entries);
        req(fr.soff >= 0 && fr.soff + int64_t(fr.nb) * fr.nb <= int64_t(P.contrib_ring) * P.contrib_slot_entries);
        req(fr.red0 >= 0 && fr.red0 + fr.nf <= P.nred);
        req(fr.voff >= 0 && fr.voff + fr.F <= int64_t(P.vars.size()));
        for (int a = 0; a < fr.F; ++a) req(P.vars[fr.voff + a] >= 0 && P.vars[fr.voff + a] < P.nred);
        req(fr.woff >= 0 && fr.woff + fr.F <= P.w_entries);
        req(fr.dinv_off + int64_t((fr.nf + P.panel - 1) / P.panel) * 2 * P.panel * P.panel <= P.dinv_entries);
        if (fr.parent >= 0) {
            req(fr.parent < P.nfronts);
            const FrontDev& pa = P.fronts[fr.parent];
            req(pa.lvl > fr.lvl && pa.lvl - fr.lvl < P.contrib_ring);
            req(fr.emap_off >= 0 && fr.emap_off + fr.nb <= int64_t(P.emap.size()));
            for (int a = 0; a < fr.nb; ++a) req(P.emap[fr.emap_off + a] >= 0 && P.emap[fr.emap_off + a] < pa.F);
        } else {
            req(fr.nb == 0);
            ++roots;
        }
    }
    req(roots == 1 && fsum == P.factor_entries);
    for (int h = 0; h < P.nlevels; ++h)
        for (int64_t d = P.asm_level_start[h]; d < P.asm_level_start[h + 1]; ++d)
            req(P.asm_dst[d] >= 0 && P.asm_dst[d] < P.level_work[h]);
    req(int(P.r2g.size()) == P.nred && int(P.g2r.size()) == P.ndim);
    for (int q = 0; q < P.nred; ++q) req(P.r2g[q] >= 0 && P.r2g[q] < P.ndim && P.g2r[P.r2g[q]] == q);
    req(int(P.dry_ptr.size()) == P.nred + 1);
}

// ===========================================================================
// numeric kernels
// ===========================================================================
namespace {

constexpr int NT = 256;    // threads of the per-front solve kernels
constexpr int OB = 128;   // outer panel width of the two-level blocked LU
constexpr int NTP = 512;   // threads of the panel kernel

__device__ __forceinline__ double atomic_max_pos(double* a, double v) {
    // non-negative doubles order like their bit patterns
    unsigned long long* p = reinterpret_cast<unsigned long long*>(a);
    return __longlong_as_double(atomicMax(p, __double_as_longlong(v)));
}

// Ruiz equilibration of the wet block: one pass of row then column scaling
// by the square root of the largest scaled magnitude.
__global__ void k_rowmax(int ndim, const int* __restrict__ g2r, const int* __restrict__ rp, const int* __restrict__ ci,
                         const double* __restrict__ v, const double* __restrict__ dc, double* __restrict__ dr) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ndim; r += gridDim.x * blockDim.x) {
        if (g2r[r] < 0) continue;
        double mx = 0.0;
        for (int q = rp[r]; q < rp[r + 1]; ++q)
            if (g2r[ci[q]] >= 0) mx = fmax(mx, fabs(v[q]) * dc[ci[q]]);
        mx *= dr[r];
        if (mx > 0.0) dr[r] /= sqrt(mx);
    }
}
__global__ void k_colmax(int ndim, const int* __restrict__ g2r, const int* __restrict__ rp, const int* __restrict__ ci,
                         const double* __restrict__ v, const double* __restrict__ dr, const double* __restrict__ dc,
                         double* __restrict__ cmax) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ndim; r += gridDim.x * blockDim.x) {
        if (g2r[r] < 0) continue;
        for (int q = rp[r]; q < rp[r + 1]; ++q) {
            int c = ci[q];
            if (g2r[c] >= 0) atomic_max_pos(cmax + c, fabs(dr[r] * v[q] * dc[c]));
        }
    }
}
__global__ void k_colscale(int ndim, const int* __restrict__ g2r, const double* __restrict__ cmax,
                           double* __restrict__ dc) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ndim; c += gridDim.x * blockDim.x)
        if (g2r[c] >= 0 && cmax[c] > 0.0) dc[c] /= sqrt(cmax[c]);
}

template <class T>
__global__ void k_assemble(int64_t n, const int* __restrict__ src, const int64_t* __restrict__ dst,
                           const int* __restrict__ rowof, const int* __restrict__ ci, const double* __restrict__ val,
                           const double* __restrict__ dr, const double* __restrict__ dc, T* __restrict__ front) {
    for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < n; q += int64_t(gridDim.x) * blockDim.x) {
        const int e = src[q];
        front[dst[q]] = T(dr[rowof[q]] * val[e] * dc[ci[e]]);
    }
}

// front[parent] += S[child] for the children in `list` (one slot at a time);
// the children's contribution blocks come from the ring
template <class T>
__global__ void k_extend_add(const FrontDev* __restrict__ fronts, const int* __restrict__ list,
                             const int* __restrict__ emap, const T* __restrict__ contrib, T* __restrict__ front) {
    // blocks stride over the columns b of S, threads over its rows a
    const FrontDev c = fronts[list[blockIdx.y]];
    const FrontDev p = fronts[c.parent];
    const int nb = c.nb;
    const int* em = emap + c.emap_off;
    const T* S = contrib + c.soff;
    T* P = front + p.off;
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        T* pc = P + int64_t(em[b]) * p.F;
        const T* sc = S + int64_t(b) * nb;
        for (int a = threadIdx.x; a < nb; a += blockDim.x) pc[em[a]] += sc[a];
    }
}

// End of a level: each front's factors move from the working area to the
// factor store (its first nf columns as they are, ld F; then rows [0, nf) of
// columns [nf, F), ld nf) and its contribution block (rows and columns
// [nf, F)) to the ring (ld nb). Blocks stride over the columns, threads over
// the rows, four rows in flight per thread.
template <class T>
__global__ void __launch_bounds__(256) k_spill(const FrontDev* __restrict__ fronts, const int* __restrict__ lf,
                                               const T* __restrict__ front, T* __restrict__ factor,
                                               T* __restrict__ contrib) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    const int F = fr.F, nf = fr.nf, nb = fr.nb;
    for (int c = blockIdx.x; c < F; c += gridDim.x) {
        const T* src = front + fr.off + int64_t(c) * F;
        // rows [0, nf) go to lo + r; rows [nf, F) to hi + (r - nf)
        T* lo = c < nf ? factor + fr.foff + int64_t(c) * F : factor + fr.foff + int64_t(F) * nf + int64_t(c - nf) * nf;
        T* hi = c < nf ? lo + nf : contrib + fr.soff + int64_t(c - nf) * nb;
        for (int r0 = threadIdx.x; r0 < F; r0 += 4 * blockDim.x) {
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = r0 + u * blockDim.x;
                v[u] = r < F ? src[r] : T(0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = r0 + u * blockDim.x;
                if (r < nf) lo[r] = v[u];
                else if (r < F) hi[r - nf] = v[u];
            }
        }
    }
}

// Panel p of every front of a level: LU with partial pivoting inside the
// bb x bb diagonal block (block-local pivoting), plus the inverses of its
// unit-lower and upper factors. With the barotropic pressures deferred to the
// root, no fully-summed block is singular and local pivots suffice.
template <class T, int B>
__global__ void __launch_bounds__(32) k_panel_diag(const FrontDev* __restrict__ fronts, const int* __restrict__ lf,
                                                   int p, T* __restrict__ front, T* __restrict__ dinv,
                                                   int* __restrict__ piv, T tau, int* __restrict__ npert) {
    // One warp per front; lane r keeps row r of the block in registers for
    // the whole elimination (rows are not exchanged: `pos` records the step at
    // which a row became the pivot, and the rows are written out in that
    // order). Each step finds the pivot by warp shuffles, the pivot lane
    // publishes its row in shared memory, and every lane reads it back with
    // vector loads. The step loop is not unrolled, to keep the kernel small.
    static_assert(B == 32, "one lane per row");
    const FrontDev fr = fronts[lf[blockIdx.x]];
    if (fr.nf <= p) return;
    const int bb = min(B, fr.nf - p), F = fr.F, lane = threadIdx.x;
    const unsigned full = 0xffffffffu;
    __shared__ __align__(16) T prow[B];        // the current pivot row
    __shared__ T S[B][B + 1];                   // the factored block in pivot order (padded rows)
    T* A = front + fr.off + int64_t(p) * F + p;
    T row[B];
#pragma unroll
    for (int c = 0; c < B; ++c) row[c] = (lane < bb && c < bb) ? A[int64_t(c) * F + lane] : (lane == c ? T(1) : T(0));
    int pos = lane < bb ? -1 : lane;            // padding rows keep their place
#pragma unroll 1
    for (int j = 0; j < bb; ++j) {
        T a = T(0);
#pragma unroll
        for (int c = 0; c < B; ++c)
            if (c == j) a = row[c];
        // pivot: largest |a| over the rows not yet used, smallest lane on ties;
        // a NaN ranks below every number (and is counted), so that every lane
        // agrees on the pivot and it stays inside the block
        T bv = pos < 0 ? abs(a) : T(-1);
        if (bv != bv) {
            bv = T(-0.5);
            atomicAdd(npert + 1, 1);
        }
        int br = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const T ov = __shfl_xor_sync(full, bv, o);
            const int orr = __shfl_xor_sync(full, br, o);
            if (ov > bv || (ov == bv && orr < br)) { bv = ov; br = orr; }
        }
        const int pr = br;
        if (lane == pr) {
            pos = j;
            // pivot row maximum from column j on, perturbation of a tiny pivot
            T sc = T(0);
#pragma unroll
            for (int c = 0; c < B; ++c)
                if (c >= j) sc = max(sc, abs(row[c]));
            T d = a;
            if (!(abs(d) > tau * sc)) {
                d = (d < T(0) ? -tau : tau) * (sc > T(0) ? sc : T(1));
                atomicAdd(npert, 1);
#pragma unroll
                for (int c = 0; c < B; ++c)
                    if (c == j) row[c] = d;
            }
#pragma unroll
            for (int c = 0; c < B; ++c) prow[c] = row[c];
        }
        __syncwarp();
        if (pos < 0) {   // eliminate below the pivot: l = a / d, row -= l * prow (columns > j)
            T u[B];
#pragma unroll
            for (int c = 0; c < B; c += 16 / sizeof(T)) {
                if (sizeof(T) == 4) {
                    const float4 v = *reinterpret_cast<const float4*>(&prow[c]);
                    u[c] = T(v.x); u[c + 1] = T(v.y); u[c + 2] = T(v.z); u[c + 3] = T(v.w);
                } else {
                    const double2 v = *reinterpret_cast<const double2*>(&prow[c]);
                    u[c] = T(v.x); u[c + 1] = T(v.y);
                }
            }
            T d = T(0);
#pragma unroll
            for (int c = 0; c < B; ++c)
                if (c == j) d = u[c];
            const T l = a / d;
#pragma unroll
            for (int c = 0; c < B; ++c) {
                if (c > j) row[c] -= l * u[c];
                else if (c == j) row[c] = l;
            }
        }
        __syncwarp();
    }
    // rows in pivot order: S[pos] = row; the factors go back to the front
#pragma unroll
    for (int c = 0; c < B; ++c) S[pos][c] = row[c];
    __syncwarp();
    if (lane < bb) {
#pragma unroll
        for (int c = 0; c < B; ++c)
            if (c < bb) A[int64_t(c) * F + pos] = row[c];
        piv[fr.red0 + p + pos] = lane;
    }
    // inverses: lane c computes column c of Linv (unit lower) and of Uinv
    T* Di = dinv + fr.dinv_off + int64_t(p / B) * 2 * B * B;
    T x[B];
#pragma unroll
    for (int r = 0; r < B; ++r) {
        T t = (r == lane) ? T(1) : T(0);
#pragma unroll
        for (int q = 0; q < r; ++q) t -= S[r][q] * x[q];
        x[r] = (r > lane) ? t : (r == lane ? T(1) : T(0));
    }
#pragma unroll
    for (int r = 0; r < B; ++r) Di[r * B + lane] = (r < bb && lane < bb) ? x[r] : T(0);
#pragma unroll
    for (int r = B - 1; r >= 0; --r) {
        T t = (r == lane) ? T(1) : T(0);
#pragma unroll
        for (int q = r + 1; q < B; ++q) t -= S[r][q] * x[q];
        x[r] = (r <= lane && r < bb && lane < bb) ? t / S[r][r] : T(0);
    }
#pragma unroll
    for (int r = 0; r < B; ++r) Di[B * B + r * B + lane] = (r < bb && lane < bb) ? x[r] : T(0);
}

// The block row permutation of panel p applied to every column outside the
// diagonal block (left columns: row order of L becomes final; right columns:
// followed by U12 = Linv * A(p:p+bb, c)).
template <class T, int B>
__global__ void k_rowperm_u12(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, int p, int P0,
                              T* __restrict__ front, const T* __restrict__ dinv, const int* __restrict__ piv) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    if (fr.nf <= p) return;
    const int cend = min(P0 + OB, fr.nf);   // columns past the outer panel: permuted only
    const int bb = min(B, fr.nf - p), F = fr.F;
    __shared__ T Li[B][B];
    __shared__ int perm[B];
    const T* Di = dinv + fr.dinv_off + int64_t(p / B) * 2 * B * B;
    for (int e = threadIdx.x; e < B * B; e += blockDim.x) Li[e / B][e % B] = Di[e];
    if (threadIdx.x < bb) perm[threadIdx.x] = min(max(piv[fr.red0 + p + threadIdx.x], 0), bb - 1);
    __syncthreads();
    int c = blockIdx.x * blockDim.x + threadIdx.x;   // skip the diagonal block
    if (c >= p) c += bb;
    if (c >= F) return;
    T* col = front + fr.off + int64_t(c) * F + p;
    T v[B];
#pragma unroll
    for (int r = 0; r < B; ++r) v[r] = r < bb ? col[perm[r]] : T(0);
    if (c < p || c >= cend) {
#pragma unroll
        for (int r = 0; r < B; ++r)
            if (r < bb) col[r] = v[r];
        return;
    }
#pragma unroll
    for (int r = B - 1; r >= 0; --r) {
        if (r < bb) {
            T s = v[r];
#pragma unroll
            for (int q = 0; q < r; ++q) s += Li[r][q] * v[q];
            col[r] = s;
        }
    }
}

// L21 = A(p+bb:F, p:p+bb) * Uinv
template <class T, int B>
__global__ void k_l21(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, int p, T* __restrict__ front,
                      const T* __restrict__ dinv) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    if (fr.nf <= p) return;
    const int bb = min(B, fr.nf - p), F = fr.F;
    __shared__ T Ui[B][B];
    const T* Di = dinv + fr.dinv_off + int64_t(p / B) * 2 * B * B + B * B;
    for (int e = threadIdx.x; e < B * B; e += blockDim.x) Ui[e / B][e % B] = Di[e];
    __syncthreads();
    const int r = p + bb + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= F) return;
    T* A = front + fr.off;
    T v[B];
#pragma unroll
    for (int c = 0; c < B; ++c) v[c] = c < bb ? A[int64_t(p + c) * F + r] : T(0);
#pragma unroll
    for (int c = 0; c < B; ++c) {
        if (c < bb) {
            T s = T(0);
#pragma unroll
            for (int q = 0; q <= c; ++q) s += v[q] * Ui[q][c];
            A[int64_t(p + c) * F + r] = s;
        }
    }
}

// Band rows [p, p+bb) of the columns past the outer panel: U12 = Linv_pp * A
// (their rows were already permuted by k_rowperm_u12)
template <class T, int B>
__global__ void k_band_u12(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, int p, int P0,
                           T* __restrict__ front, const T* __restrict__ dinv) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    if (fr.nf <= p) return;
    const int bb = min(B, fr.nf - p), F = fr.F, cend = min(P0 + OB, fr.nf);
    __shared__ T Li[B][B];
    const T* Di = dinv + fr.dinv_off + int64_t(p / B) * 2 * B * B;
    for (int e = threadIdx.x; e < B * B; e += blockDim.x) Li[e / B][e % B] = Di[e];
    __syncthreads();
    const int c = cend + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= F) return;
    T* col = front + fr.off + int64_t(c) * F + p;
    T v[B];
#pragma unroll
    for (int r = 0; r < B; ++r) v[r] = r < bb ? col[r] : T(0);
#pragma unroll
    for (int r = B - 1; r >= 0; --r) {
        if (r < bb) {
            T s = v[r];
#pragma unroll
            for (int q = 0; q < r; ++q) s += Li[r][q] * v[q];
            col[r] = s;
        }
    }
}

// Front-local GEMM updates of the two-level blocked LU (outer panels of OB
// columns starting at P0, inner panels of B columns starting at p):
//   STRIP: A[p+bb:F, p+bb:cend] -= A[p+bb:F, p:p+bb] * A[p:p+bb, p+bb:cend]
//   BAND:  A[p+bb:cend, cend:F] -= A[p+bb:cend, p:p+bb] * A[p:p+bb, cend:F]
//   TRAIL: A[cend:F, cend:F]    -= A[cend:F, P0:cend] * A[P0:cend, cend:F]
// with cend = min(P0 + OB, nf). TM x TM tiles per CTA of 256 threads, the K
// range staged through shared memory in chunks of 32.
enum { GM_STRIP = 0, GM_BAND = 1, GM_TRAIL = 2 };
template <class T, int MODE, int TM>
__global__ void __launch_bounds__(256) k_fgemm(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, int p,
                                               int P0, T* __restrict__ front) {
    constexpr int TT = TM / 16;   // outputs per thread and dimension
    const FrontDev fr = fronts[lf[blockIdx.y]];
    const int nf = fr.nf, F = fr.F;
    const int cend = min(P0 + OB, nf);
    int r0, r1, c0, c1, k0, k1;
    if (MODE == GM_STRIP) {
        if (nf <= p) return;
        const int bb = min(32, nf - p);
        r0 = p + bb; r1 = F; c0 = p + bb; c1 = cend; k0 = p; k1 = p + bb;
    } else if (MODE == GM_BAND) {
        if (nf <= p) return;
        const int bb = min(32, nf - p);
        r0 = p + bb; r1 = cend; c0 = cend; c1 = F; k0 = p; k1 = p + bb;
    } else {
        if (nf <= P0) return;
        r0 = cend; r1 = F; c0 = cend; c1 = F; k0 = P0; k1 = cend;
    }
    const int M = r1 - r0, N = c1 - c0;
    if (M <= 0 || N <= 0) return;
    const int tm = (M + TM - 1) / TM, tn = (N + TM - 1) / TM;
    if (int(blockIdx.x) >= tm * tn) return;
    const int row0 = r0 + (blockIdx.x % tm) * TM, col0 = c0 + (blockIdx.x / tm) * TM;
    T* A = front + fr.off;
    __shared__ T As[32][TM];
    __shared__ T Bs[32][TM + 1];
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    T acc[TT][TT];
#pragma unroll
    for (int a = 0; a < TT; ++a)
#pragma unroll
        for (int b = 0; b < TT; ++b) acc[a][b] = T(0);
    for (int kb = k0; kb < k1; kb += 32) {
        const int kc = min(32, k1 - kb);
#pragma unroll 4
        for (int e = tid; e < 32 * TM; e += 256) {
            const int i = e % TM, k = e / TM, r = row0 + i;
            As[k][i] = (k < kc && r < r1) ? A[int64_t(kb + k) * F + r] : T(0);
        }
#pragma unroll 4
        for (int e = tid; e < 32 * TM; e += 256) {
            const int k = e % 32, j = e / 32, c = col0 + j;
            Bs[k][j] = (k < kc && c < c1) ? A[int64_t(c) * F + kb + k] : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            T av[TT], bv[TT];
#pragma unroll
            for (int a = 0; a < TT; ++a) av[a] = As[k][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < TT; ++b) bv[b] = Bs[k][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < TT; ++a)
#pragma unroll
                for (int b = 0; b < TT; ++b) acc[a][b] += av[a] * bv[b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < TT; ++b) {
        const int c = col0 + ty + 16 * b;
        if (c >= c1) continue;
        T* col = A + int64_t(c) * F;
#pragma unroll
        for (int a = 0; a < TT; ++a) {
            const int r = row0 + tx + 16 * a;
            if (r < r1) col[r] -= acc[a][b];
        }
    }
}

// FP32 version of k_fgemm: 128 x 128 tiles, 8 x 8 outputs per thread in two
// 4 x 4 quadrants (rows tx*4 + {0..3} and 64 + tx*4 + {0..3}, likewise for
// the columns) so that every operand read from shared memory is a float4.
// Operands are staged with cp.async (zero-filled outside the block) into three
// buffers in dynamic shared memory: the copies of the next two 32-deep K
// chunks are in flight while the current one is multiplied. B is stored k-major with
// its 4-column groups XOR-swizzled by (k & 7) to spread the transposing
// copies over the banks.
constexpr int FG_TM = 128;
constexpr int FG_NBUF = 3;
constexpr size_t FG_SMEM = sizeof(float) * FG_NBUF * 2 * 32 * FG_TM;   // 96 KiB: two CTAs per SM
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::); }
template <int MODE>
__global__ void __launch_bounds__(256, 2) k_fgemm_f32(const FrontDev* __restrict__ fronts, const int* __restrict__ lf,
                                                      int p, int P0, float* __restrict__ front) {
    constexpr int TM = FG_TM;
    const FrontDev fr = fronts[lf[blockIdx.y]];
    const int nf = fr.nf, F = fr.F;
    const int cend = min(P0 + OB, nf);
    int r0, r1, c0, c1, k0, k1;
    if (MODE == GM_STRIP) {
        if (nf <= p) return;
        const int bb = min(32, nf - p);
        r0 = p + bb; r1 = F; c0 = p + bb; c1 = cend; k0 = p; k1 = p + bb;
    } else if (MODE == GM_BAND) {
        if (nf <= p) return;
        const int bb = min(32, nf - p);
        r0 = p + bb; r1 = cend; c0 = cend; c1 = F; k0 = p; k1 = p + bb;
    } else {
        if (nf <= P0) return;
        r0 = cend; r1 = F; c0 = cend; c1 = F; k0 = P0; k1 = cend;
    }
    const int M = r1 - r0, N = c1 - c0;
    if (M <= 0 || N <= 0) return;
    const int tm = (M + TM - 1) / TM, tn = (N + TM - 1) / TM;
    if (int(blockIdx.x) >= tm * tn) return;
    const int row0 = r0 + (blockIdx.x % tm) * TM, col0 = c0 + (blockIdx.x / tm) * TM;
    float* A = front + fr.off;
    extern __shared__ __align__(16) float fg_smem[];
    auto As = [&](int buf, int k) { return fg_smem + (buf * 32 + k) * TM; };
    auto Bs = [&](int buf, int k) { return fg_smem + FG_NBUF * 32 * TM + (buf * 32 + k) * TM; };
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    auto issue = [&](int kb, int buf) {
        const int kc = min(32, k1 - kb);
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
            const int e = tid + 256 * q, i = e % TM, k = e / TM, r = row0 + i;
            const bool v = k < kc && r < r1;
            cp_async4(As(buf, k) + i, v ? A + int64_t(kb + k) * F + r : A, v);
        }
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
            const int e = tid + 256 * q, k = e % 32, j = e / 32, c = col0 + j;
            const bool v = k < kc && c < c1;
            cp_async4(Bs(buf, k) + ((((j >> 2) ^ (k & 7)) << 2) | (j & 3)), v ? A + int64_t(c) * F + kb + k : A, v);
        }
        cp_async_commit();
    };
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    issue(k0, 0);
    if (k0 + 32 < k1) issue(k0 + 32, 1);
    int buf = 0;
    for (int kb = k0; kb < k1; kb += 32) {
        if (kb + 32 < k1) cp_async_wait_one();   // this thread's copies of chunk kb have landed
        else cp_async_wait_all();
        __syncthreads();                 // chunk kb is in buffer buf; the buffer read before it is free
        if (kb + 64 < k1) issue(kb + 64, (buf + 2) % FG_NBUF);
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            const float* ar = As(buf, k);
            const float* br = Bs(buf, k);
            const float4 a0 = *reinterpret_cast<const float4*>(ar + tx * 4);
            const float4 a1 = *reinterpret_cast<const float4*>(ar + 64 + tx * 4);
            const int sw = k & 7;
            const float4 b0 = *reinterpret_cast<const float4*>(br + ((ty ^ sw) << 2));
            const float4 b1 = *reinterpret_cast<const float4*>(br + (((16 + ty) ^ sw) << 2));
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
        }
        buf = (buf + 1) % FG_NBUF;
    }
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int c = col0 + (b < 4 ? ty * 4 + b : 64 + ty * 4 + b - 4);
        if (c >= c1) continue;
        float* col = A + int64_t(c) * F;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int r = row0 + (a < 4 ? tx * 4 + a : 64 + tx * 4 + a - 4);
            if (r < r1) col[r] -= acc[a][b];
        }
    }
}

// ---------------------------------------------------------------------------
// explicit inverses for the solve phase: after its LU, every front's 256-row
//   diagonal super-blocks of L11 (strict lower part, unit diagonal) and U11
//   (upper part) are replaced by their inverses; plans whose fronts stay at
//   or below the substitution threshold then complete the whole inverses
//   Linv11 / Uinv11, so the triangular solves become dense GEMVs. L21 and
//   U12 are kept as they are (two dependent GEMV stages per level and sweep).
// ---------------------------------------------------------------------------

// write the inverted diagonal blocks (Linv_jj strict lower, Uinv_jj upper)
template <class T, int B>
__global__ void k_put_diag_inv(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, T* __restrict__ factor,
                               const T* __restrict__ dinv) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    const int nblk = (fr.nf + B - 1) / B;
    if (int(blockIdx.x) >= nblk) return;
    const int p = blockIdx.x * B, bb = min(B, fr.nf - p);
    const T* Di = dinv + fr.dinv_off + int64_t(blockIdx.x) * 2 * B * B;
    T* A = factor + fr.foff;   // the first nf columns keep ld F in the factor store
    for (int e = threadIdx.x; e < bb * bb; e += blockDim.x) {
        int r = e / bb, c = e % bb;
        A[int64_t(p + c) * fr.F + p + r] = r > c ? Di[r * B + c] : Di[B * B + r * B + c];
    }
}

// Triangular inversion in two parts, all fronts of a level and both triangles
// in the same launches, each step two batched GEMMs (a product into scratch,
// then the second product in place):
//  (1) inside every 256-row super-block, pairs of neighbouring inverted
//      diagonal blocks A (first) and D (second) of size s = 32, 64, 128 merge:
//        lower:  X21 = -Dinv * (L21blk * Ainv)    upper:  X12 = -(Ainv * U12blk) * Dinv
//  (2) over the super-blocks, block-row steps of the row-oriented method
//      (lower top down, upper bottom up), whose rounding errors carry one
//      large inverse per product instead of the two of a merge (Du Croz and
//      Higham, IMA J. Numer. Anal. 12 (1992) 1-19), which the FP32
//      preconditioner's quality depends on for ill-conditioned factors.
// Triangular operands are read in place through masks (unit lower / upper)
// and the K loop skips their zero part.
enum { OP_DENSE = 0, OP_LOWER_UNIT = 1, OP_UPPER = 2 };
constexpr int TRI_SB = 256;   // super-block rows of the row-oriented steps
constexpr int TRI_KS = 512;   // K piece of a split-K product
// The solves apply L11 / U11 of a plan whose fronts have at most 12288 own
// unknowns (the default of iemic_set_substitution_threshold)
// as whole inverses, one GEMV stage per triangle; a larger plan substitutes
// over the inverted 256-row diagonal super-blocks. The whole inverses need one GEMV stage per triangle, but their
// rounding grows with the condition of the whole triangle, which block-local
// pivoting leaves large: on a 5,005-unknown root front FP32 solves with them
// reach a relative residual of 0.5 (1e-4 by substitution), and on the
// 59,470-unknown root of the 360 x 160 x 20 ocean the preconditioner fails.

struct TriTask {
    int64_t a_off, b_off, c_off;   // element offsets: base 0 = front storage, 1 = scratch
    int lda, ldb, ldc, M, N, K;
    int opA, opB, a_base, b_base, c_base;
    float alpha;
    int k0 = 0, k1 = 1 << 30;      // K sub-range of a split-K part
};
// Split-K partial sums of one product: part s (s = 1..nsplit-1) lies at
// off + s * len and is added into part 0 at off.
struct SplitGroup {
    int64_t off, len;
    int nsplit;
};
template <class T>
__global__ void k_split_reduce(const SplitGroup* __restrict__ groups, int ngroups, T* __restrict__ scr) {
    for (int g = blockIdx.y; g < ngroups; g += gridDim.y) {
        const SplitGroup sg = groups[g];
        for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < sg.len; q += int64_t(gridDim.x) * blockDim.x) {
            T v = scr[sg.off + q];
            for (int sp = 1; sp < sg.nsplit; ++sp) v += scr[sg.off + sp * sg.len + q];
            scr[sg.off + q] = v;
        }
    }
}
struct TriTile {
    int task, i0, j0;
};
template <class T>
__device__ __forceinline__ T tri_ld(const T* P, int ld, int r, int c, int op) {
    if (op == OP_LOWER_UNIT) return r > c ? P[int64_t(c) * ld + r] : (r == c ? T(1) : T(0));
    if (op == OP_UPPER) return r <= c ? P[int64_t(c) * ld + r] : T(0);
    return P[int64_t(c) * ld + r];
}
template <class T>
__global__ void __launch_bounds__(256) k_tri_gemm(const TriTask* __restrict__ tasks, const TriTile* __restrict__ tiles,
                                                  T* __restrict__ front, T* __restrict__ scr) {
    const TriTile tl = tiles[blockIdx.x];
    const TriTask t = tasks[tl.task];
    const T* A = (t.a_base ? scr : front) + t.a_off;
    const T* Bm = (t.b_base ? scr : front) + t.b_off;
    T* C = (t.c_base ? scr : front) + t.c_off;
    const int i0 = tl.i0, j0 = tl.j0;
    int kb = max(0, t.k0), ke = min(t.K, t.k1);
    if (t.opA == OP_LOWER_UNIT) ke = min(ke, i0 + 64);
    if (t.opA == OP_UPPER) kb = max(kb, i0);
    if (t.opB == OP_LOWER_UNIT) kb = max(kb, j0);
    if (t.opB == OP_UPPER) ke = min(ke, j0 + 64);
    __shared__ T As[32][65];
    __shared__ T Bs[32][65];
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
    for (int k0 = kb; k0 < ke; k0 += 32) {
        for (int e = tid; e < 32 * 64; e += 256) {
            const int ii = e % 64, kk = e / 64, r = i0 + ii, k = k0 + kk;
            As[kk][ii] = (r < t.M && k < ke) ? tri_ld(A, t.lda, r, k, t.opA) : T(0);
        }
        for (int e = tid; e < 32 * 64; e += 256) {
            const int kk = e % 32, jj = e / 32, k = k0 + kk, c = j0 + jj;
            Bs[kk][jj] = (c < t.N && k < ke) ? tri_ld(Bm, t.ldb, k, c, t.opB) : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            T av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[kk][tx * 4 + a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][ty * 4 + b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
        }
        __syncthreads();
    }
    const T alpha = T(t.alpha);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int c = j0 + ty * 4 + b;
        if (c >= t.N) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int r = i0 + tx * 4 + a;
            if (r < t.M) C[int64_t(c) * t.ldc + r] = alpha * acc[a][b];
        }
    }
}

// FP32 task GEMM (triangular inversion): C = alpha op(A) op(B) over
// 128 x 128 tiles with the staging of k_fgemm_f32 (cp.async double buffering,
// float4 operands, swizzled B). Masked triangular entries are zero-filled by
// the copy; the implicit unit diagonal of OP_LOWER_UNIT operands is written
// into shared memory by the thread that issued its copy, after its copies
// completed and before the barrier that publishes the chunk.
__device__ __forceinline__ bool tri_mask(int op, int r, int c) {
    return op == OP_DENSE || (op == OP_LOWER_UNIT ? r > c : r <= c);
}
__global__ void __launch_bounds__(256, 2) k_task_gemm_f32(const TriTask* __restrict__ tasks,
                                                          const TriTile* __restrict__ tiles,
                                                          float* __restrict__ front, float* __restrict__ scr) {
    constexpr int TM = FG_TM;
    const TriTile tl = tiles[blockIdx.x];
    const TriTask t = tasks[tl.task];
    const float* A = (t.a_base ? scr : front) + t.a_off;
    const float* Bm = (t.b_base ? scr : front) + t.b_off;
    float* C = (t.c_base ? scr : front) + t.c_off;
    const int i0 = tl.i0, j0 = tl.j0;
    int kb = max(0, t.k0), ke = min(t.K, t.k1);
    if (t.opA == OP_LOWER_UNIT) ke = min(ke, i0 + TM);
    if (t.opA == OP_UPPER) kb = max(kb, i0);
    if (t.opB == OP_LOWER_UNIT) kb = max(kb, j0);
    if (t.opB == OP_UPPER) ke = min(ke, j0 + TM);
    extern __shared__ __align__(16) float fg_smem[];
    auto As = [&](int buf, int k) { return fg_smem + (buf * 32 + k) * TM; };
    auto Bs = [&](int buf, int k) { return fg_smem + FG_NBUF * 32 * TM + (buf * 32 + k) * TM; };
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    auto issue = [&](int k0c, int buf) {
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
            const int e = tid + 256 * q, i = e % TM, k = e / TM, r = i0 + i, kk = k0c + k;
            const bool v = r < t.M && kk < ke && tri_mask(t.opA, r, kk);
            cp_async4(As(buf, k) + i, v ? A + int64_t(kk) * t.lda + r : A, v);
        }
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
            const int e = tid + 256 * q, k = e % 32, j = e / 32, c = j0 + j, kk = k0c + k;
            const bool v = c < t.N && kk < ke && tri_mask(t.opB, kk, c);
            cp_async4(Bs(buf, k) + ((((j >> 2) ^ (k & 7)) << 2) | (j & 3)), v ? Bm + int64_t(c) * t.ldb + kk : Bm, v);
        }
        cp_async_commit();
    };
    auto unit_diag = [&](int k0c, int buf) {   // after this thread's copies of the chunk completed
        if (t.opA == OP_LOWER_UNIT) {
#pragma unroll 4
            for (int q = 0; q < 16; ++q) {
                const int e = tid + 256 * q, i = e % TM, k = e / TM, r = i0 + i, kk = k0c + k;
                if (r == kk && r < t.M && kk < ke) As(buf, k)[i] = 1.f;
            }
        }
        if (t.opB == OP_LOWER_UNIT) {
#pragma unroll 4
            for (int q = 0; q < 16; ++q) {
                const int e = tid + 256 * q, k = e % 32, j = e / 32, c = j0 + j, kk = k0c + k;
                if (kk == c && c < t.N && kk < ke) Bs(buf, k)[(((j >> 2) ^ (k & 7)) << 2) | (j & 3)] = 1.f;
            }
        }
    };
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    if (kb < ke) issue(kb, 0);
    if (kb + 32 < ke) issue(kb + 32, 1);
    int buf = 0;
    for (int k0c = kb; k0c < ke; k0c += 32) {
        if (k0c + 32 < ke) cp_async_wait_one();
        else cp_async_wait_all();
        unit_diag(k0c, buf);
        __syncthreads();
        if (k0c + 64 < ke) issue(k0c + 64, (buf + 2) % FG_NBUF);
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            const float* ar = As(buf, k);
            const float* br = Bs(buf, k);
            const float4 a0 = *reinterpret_cast<const float4*>(ar + tx * 4);
            const float4 a1 = *reinterpret_cast<const float4*>(ar + 64 + tx * 4);
            const int sw = k & 7;
            const float4 b0 = *reinterpret_cast<const float4*>(br + ((ty ^ sw) << 2));
            const float4 b1 = *reinterpret_cast<const float4*>(br + (((16 + ty) ^ sw) << 2));
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
        }
        buf = (buf + 1) % FG_NBUF;
    }
    const float alpha = t.alpha;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int c = j0 + (b < 4 ? ty * 4 + b : 64 + ty * 4 + b - 4);
        if (c >= t.N) continue;
        float* col = C + int64_t(c) * t.ldc;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int r = i0 + (a < 4 ? tx * 4 + a : 64 + tx * 4 + a - 4);
            if (r < t.M) col[r] = alpha * acc[a][b];
        }
    }
}

// ---------------------------------------------------------------------------
// solve phase
// ---------------------------------------------------------------------------
// reduced, row-scaled rhs: wet rows minus the couplings to the eliminated
// (dry) unknowns
// (the solve phase works in FP64 for both factor precisions: FP32 factors are
// read and upcast, so the accumulation error is FP64's, not FP32's)
template <class TV>
__global__ void k_reduce_rhs(int nred, const int* __restrict__ r2g, const int* __restrict__ dry_ptr,
                             const int* __restrict__ dry_e, const int* __restrict__ dry_c,
                             const double* __restrict__ val, const double* __restrict__ dr, const TV* __restrict__ r,
                             double* __restrict__ red) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nred; q += gridDim.x * blockDim.x) {
        const int g = r2g[q];
        double s = double(r[g]);
        for (int k = dry_ptr[q]; k < dry_ptr[q + 1]; ++k) s -= val[dry_e[k]] * double(r[dry_c[k]]);
        red[q] = dr[g] * s;
    }
}
// Identity rows (isdry 1) pass r through; pinned pressures (isdry 2) are the
// gauge of J's null space and come out as exact zeros, so every solution the
// solver returns has zero pressure at the pins.
template <class TV>
__global__ void k_expand(int ndim, const int* __restrict__ g2r, const char* __restrict__ isdry,
                         const double* __restrict__ dc, const double* __restrict__ red, const TV* __restrict__ r,
                         TV* __restrict__ z) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ndim; g += gridDim.x * blockDim.x) {
        int q = g2r[g];
        z[g] = q >= 0 ? TV(dc[g] * red[q]) : (isdry[g] == 2 ? TV(0) : r[g]);
    }
}

// Solve phase, one level at a time (all fronts of the level together), two
// GEMV stages per level and sweep:
//   forward:  y = Linv11 (P w_own);           u_B = w_B - L21 y
//   backward: t = y - U12 x_B;                x_own = Uinv11 t
// (Linv11 / Uinv11 applied as whole inverses or by block substitution).
// Work items split every block into (64-row tile, 256-column chunk) pieces
// so the GEMVs spread over all SMs; partial sums per chunk are reduced in a
// second pass (deterministic order), each stage into its own zero-initialised
// buffer so that skipped empty tiles contribute exact zeros.
struct WorkItem {
    int front, row0, col0, chunk, stage;
};
// solve GEMV tiles: GT rows x GC columns per block of GR threads; the
// block's threads form GR / GT column groups of GC * GT / GR columns each, so
// a thread walks one row of one column group (a short dependent chain of
// loads) and a tile's column groups are summed in shared memory
constexpr int GR = 256, GC = 256, GT = 64, NCG = GR / GT, CGW = GC / NCG;
enum { ST_LINV = 0, ST_UINV = 1, ST_L21 = 2, ST_U12 = 3, NSTAGE = 4 };
// work-item stage codes of the product blocks L21 Linv11 and Uinv11 U12 (the
// blocks and partial buffers of ST_L21 / ST_U12, read from the product store)
enum { ST_P21 = 4, ST_Q12 = 5 };
// rows and columns of a stage's block inside a front
__host__ __device__ inline void stage_block(int st, int nf, int F, int& r0, int& r1, int& c0, int& c1) {
    r0 = st == ST_L21 ? nf : 0;
    r1 = st == ST_L21 ? F : nf;
    c0 = st == ST_U12 ? nf : 0;
    c1 = st == ST_U12 ? F : nf;
}

// front-local row that row q of the own block takes after the block-local
// pivoting (clamped into its block)
__device__ __forceinline__ int piv_row(const int* __restrict__ piv, const FrontDev& fr, int q, int B) {
    const int p = (q / B) * B;
    return p + min(max(piv[fr.red0 + q], 0), min(B, fr.nf - p) - 1);
}
// forward prologue: w = [red_C ; 0] + children's update vectors, then the
// block-local row permutations applied to the own part (into wp). A thread
// per row: the inverse extend-add map gives each row its children's update
// rows, added in slot order (the order of a scatter child by child).
__device__ __forceinline__ double fwd_row(const FrontDev& fr, int q, const double* __restrict__ red,
                                          const int2* __restrict__ einv, const double* __restrict__ u0,
                                          const double* __restrict__ u1) {
    double w = q < fr.nf ? red[fr.red0 + q] : 0.0;
    const int2 a = einv[fr.woff + q];
    if (a.x >= 0) w += u0[a.x];
    if (a.y >= 0) w += u1[a.y];
    return w;
}
__global__ void __launch_bounds__(NT) k_fwd_gather(const FrontDev* __restrict__ fronts, const int* __restrict__ lf,
                                                   const int* __restrict__ child_of, const int2* __restrict__ einv,
                                                   const int* __restrict__ piv, const double* __restrict__ red,
                                                   double* __restrict__ W, double* __restrict__ WP, int B) {
    const int f = lf[blockIdx.y];
    const FrontDev fr = fronts[f];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= fr.F) return;
    const double* u[2] = {nullptr, nullptr};
    for (int sl = 0; sl < 2; ++sl) {
        const int c = child_of[2 * f + sl];
        if (c >= 0) {
            const FrontDev ch = fronts[c];
            u[sl] = WP + ch.woff + ch.nf;   // child's update vector
        }
    }
    const double wq = fwd_row(fr, q, red, einv, u[0], u[1]);
    W[fr.woff + q] = wq;
    WP[fr.woff + q] = q < fr.nf ? fwd_row(fr, piv_row(piv, fr, q, B), red, einv, u[0], u[1]) : wq;
}
// Compensated (double-float) accumulation of a * (xh + xl) into (s, c) with
// FP32 instructions only: the product's rounding error comes from an FMA and
// the sum's from TwoSum (Knuth), so the result carries about 2 x 24 bits.
// GB300 runs FP32 at 64x its FP64 rate, and FP32 factors applied with plain
// FP32 sums lose the accuracy the refinement needs; this keeps FP64-level
// accumulation at FP32 throughput. Intrinsics keep the compiler from fusing.
__device__ __forceinline__ void dd_acc(float& s, float& c, float a, float xh, float xl) {
    const float p = __fmul_rn(a, xh);
    float e = __fmaf_rn(a, xh, -p);
    e = __fmaf_rn(a, xl, e);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
}

// sg * sum_{c0 <= c < c1} A[c * ld] x[c - col0] with x staged in shared
// memory (xs: FP64; xs2: its hi/lo FP32 split for FP32 factors). FP32
// factors accumulate in compensated double-float, FP64 factors in FP64.
// The factors are read-only while a sweep runs: loads take the
// non-coherent path explicitly (kernels that also write, fence or use
// atomics would otherwise get coherent loads).
template <class T>
__device__ __forceinline__ double row_dot(const T* __restrict__ A, int64_t ld, int c0, int c1, int col0,
                                          const double* xs, const float2* xs2, float sg) {
    if (sizeof(T) == 4) {
        float sh = 0.f, sl = 0.f;
        // loads are issued 16 columns ahead of the accumulation chain so that
        // each thread keeps 16 independent HBM reads in flight
        int c = c0;
        for (; c + 16 <= c1; c += 16) {
            float a[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) a[u] = float(A[int64_t(c + u) * ld]);
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const float2 xv = xs2[c + u - col0];
                dd_acc(sh, sl, sg * a[u], xv.x, xv.y);
            }
        }
        for (; c < c1; ++c) {
            const float2 xv = xs2[c - col0];
            dd_acc(sh, sl, sg * float(A[int64_t(c) * ld]), xv.x, xv.y);
        }
        return double(sh) + double(sl);
    }
    double acc = 0.0;
#pragma unroll 4
    for (int c = c0; c < c1; ++c) acc += double(A[int64_t(c) * ld]) * xs[c - col0];
    return double(sg) * acc;
}
__device__ __forceinline__ void stage_x(double v, double* xs, float2* xs2, int q, bool fp32) {
    if (fp32) {
        const float h = __double2float_rn(v);
        xs2[q] = make_float2(h, __double2float_rn(v - double(h)));
    } else {
        xs[q] = v;
    }
}

// Partial GEMV products of one stage over a (GT-row, GC-column) tile;
// ST_LINV uses the strict lower part plus the unit diagonal, ST_UINV the
// upper part, ST_L21 and ST_U12 the dense blocks with a minus sign. Partial
// sums go to part[off + chunk * rows + (r - r0)], the column groups of a tile
// added in order.
struct StageBufs {
    double* part[4];
    const int64_t* off[4];
};
template <class T, int ST>
__device__ __forceinline__ void gemv_stage(const WorkItem& it, const FrontDev& fr, const T* __restrict__ front,
                                           const double* __restrict__ X, const StageBufs& sb) {
    // front: the factor store, or for ST_L21 / ST_U12 the product store
    double* __restrict__ part = sb.part[ST];
    const int64_t* __restrict__ part_off = sb.off[ST];
    const int F = fr.F, nf = fr.nf;
    int br0, br1, bc0, bc1;
    stage_block(ST, nf, F, br0, br1, bc0, bc1);
    const int rl = threadIdx.x % GT, cg = threadIdx.x / GT;
    const int r = it.row0 + rl;
    __shared__ double xs[GC];
    __shared__ float2 xs2[GC];
    __shared__ double gsum[NCG - 1][GT];
    const double* x = X + fr.woff;
    for (int q = threadIdx.x; q < GC; q += GR) {
        const double v = it.col0 + q < bc1 ? x[it.col0 + q] : 0.0;
        if (sizeof(T) == 4) {
            const float h = __double2float_rn(v);
            xs2[q] = make_float2(h, __double2float_rn(v - double(h)));
        } else {
            xs[q] = v;
        }
    }
    __syncthreads();
    const bool live = r < br1;
    // factor store: columns [0, nf) with ld F; the U12/H block (columns
    // [nf, F), rows [0, nf)) follows them with ld nf
    const int64_t ld = ST == ST_U12 ? nf : F;
    const T* A = ST == ST_U12 ? front + fr.foff + int64_t(F - nf) * nf + r : front + fr.foff + r;
    const int g0 = it.col0 + cg * CGW;
    int c0 = g0, c1 = min(bc1, g0 + CGW);
    if (ST == ST_LINV) c1 = min(c1, r);
    else if (ST == ST_UINV) c0 = max(c0, r);
    if (!live) c1 = c0;
    const float sg = (ST == ST_L21 || ST == ST_U12) ? -1.f : 1.f;
    double out = row_dot<T>(A, ld, c0, c1, it.col0, xs, xs2, sg);
    if (cg > 0) gsum[cg - 1][rl] = out;
    __syncthreads();
    if (cg > 0 || !live) return;
    for (int k = 0; k < NCG - 1; ++k) out += gsum[k][rl];
    if (ST == ST_LINV && r >= it.col0 && r < min(bc1, it.col0 + GC))   // unit diagonal
        out += sizeof(T) == 4 ? xs2[r - it.col0].x + double(xs2[r - it.col0].y) : xs[r - it.col0];
    part[part_off[it.front] + int64_t(it.chunk) * (br1 - br0) + (r - br0)] = out;
}
// Block substitution over the inverted 256-row diagonal super-blocks of a
// front's L11 / U11 (the forward solves): for super-block s,
//   lower (forward sweep):  y_s = Linv_ss (w_s - L(s, 0:s) y)
//   upper (backward sweep): x_s = Uinv_ss (t_s - U(s, s+1:) x)
// Only the 256 x 256 diagonal blocks are inverted, so rounding errors grow
// with their condition, not with that of the whole triangle (which
// block-local pivoting leaves large). One sub-step per super-block: the
// off-diagonal products of every front of the level as tiled partial GEMVs
// (k_sub_gemv), then the diagonal blocks (k_sub_diag, one CTA per front).
constexpr int SB = 256;
static_assert(SB == GC, "a GEMV column chunk is one super-block");
struct SubDiag {
    int front, s, pbase, nch;   // super-block s; its nch partial chunks at part[pbase + c * SB + r]
};
// off-diagonal partials of one sub-step: an item is a (GT-row, GC-column)
// tile, `stage` holds the front's partial base; x (y or x of the
// super-blocks already done) is read from the front's solve vector W
template <class T, bool UP>
__global__ void __launch_bounds__(GR) k_sub_gemv(const FrontDev* __restrict__ fronts, const WorkItem* __restrict__ items,
                                                 const T* __restrict__ factor, const double* __restrict__ W,
                                                 double* __restrict__ part) {
    const WorkItem it = items[blockIdx.x];
    const FrontDev fr = fronts[it.front];
    const int F = fr.F, nf = fr.nf;
    const int s = it.row0 / SB, r1 = min(nf, (s + 1) * SB);
    const int cend = UP ? nf : s * SB;
    const int rl = threadIdx.x % GT, cg = threadIdx.x / GT;
    const int r = it.row0 + rl;
    __shared__ double xs[GC];
    __shared__ float2 xs2[GC];
    __shared__ double gsum[NCG - 1][GT];
    const double* x = W + fr.woff;
    for (int q = threadIdx.x; q < GC; q += GR) stage_x(it.col0 + q < cend ? x[it.col0 + q] : 0.0, xs, xs2, q, sizeof(T) == 4);
    __syncthreads();
    const bool live = r < r1;
    const int g0 = it.col0 + cg * CGW;
    const int c0 = g0, c1 = live ? min(cend, g0 + CGW) : g0;
    double out = row_dot<T>(factor + fr.foff + r, F, c0, c1, it.col0, xs, xs2, -1.f);
    if (cg > 0) gsum[cg - 1][rl] = out;
    __syncthreads();
    if (cg > 0 || !live) return;
    for (int k = 0; k < NCG - 1; ++k) out += gsum[k][rl];
    part[it.stage + int64_t(it.chunk) * SB + (r - s * SB)] = out;
}
// diagonal super-block: t = rhs + partials, then y = Linv_ss t (unit lower)
// or x = Uinv_ss t; 1024 threads = 256 rows x 4 column groups of 64
constexpr int SDT = 1024, SDG = SDT / SB, SDW = SB / SDG;
template <class T, bool UP>
__global__ void __launch_bounds__(SDT) k_sub_diag(const FrontDev* __restrict__ fronts, const SubDiag* __restrict__ items,
                                                  const T* __restrict__ factor, const double* __restrict__ part,
                                                  double* __restrict__ W, double* __restrict__ WP,
                                                  double* __restrict__ xred) {
    const SubDiag it = items[blockIdx.x];
    const FrontDev fr = fronts[it.front];
    const int F = fr.F, s0 = it.s * SB, ns = min(SB, fr.nf - s0);
    const int rl = threadIdx.x % SB, cg = threadIdx.x / SB;
    __shared__ double ts[SB];
    __shared__ float2 ts2[SB];
    __shared__ double gsum[SDG - 1][SB];
    if (cg == 0) {
        double t = 0.0;
        if (rl < ns) {
            t = WP[fr.woff + s0 + rl];
            const double* p = part + it.pbase + rl;
            for (int c = 0; c < it.nch; ++c) t += p[int64_t(c) * SB];
        }
        ts[rl] = t;
        if (sizeof(T) == 4) stage_x(t, ts, ts2, rl, true);
    }
    __syncthreads();
    const bool live = rl < ns;
    int c0 = cg * SDW, c1 = min(ns, c0 + SDW);
    if (UP) c0 = max(c0, rl);   // upper part incl. the diagonal
    else c1 = min(c1, rl);      // strict lower part (unit diagonal added below)
    if (!live) c1 = c0;
    double out = row_dot<T>(factor + fr.foff + int64_t(s0) * F + s0 + rl, F, c0, max(c0, c1), 0, ts, ts2, 1.f);
    if (cg > 0) gsum[cg - 1][rl] = out;
    __syncthreads();
    if (cg > 0 || !live) return;
    for (int k = 0; k < SDG - 1; ++k) out += gsum[k][rl];
    if (!UP) out += ts[rl];
    W[fr.woff + s0 + rl] = out;
    if (UP) xred[fr.red0 + s0 + rl] = out;
    else WP[fr.woff + s0 + rl] = out;
}

template <class T>
__global__ void __launch_bounds__(GR) k_gemv_part(const FrontDev* __restrict__ fronts, const WorkItem* __restrict__ items,
                                                  const T* __restrict__ front, const T* __restrict__ prod,
                                                  const double* __restrict__ X, StageBufs sb) {
    const WorkItem it = items[blockIdx.x];
    const FrontDev fr = fronts[it.front];
    switch (it.stage) {
        case ST_LINV: gemv_stage<T, ST_LINV>(it, fr, front, X, sb); break;
        case ST_UINV: gemv_stage<T, ST_UINV>(it, fr, front, X, sb); break;
        case ST_L21: gemv_stage<T, ST_L21>(it, fr, front, X, sb); break;
        case ST_U12: gemv_stage<T, ST_U12>(it, fr, front, X, sb); break;
        case ST_P21: gemv_stage<T, ST_L21>(it, fr, prod, X, sb); break;
        default: gemv_stage<T, ST_U12>(it, fr, prod, X, sb); break;
    }
}

// Stage epilogues (one thread per row of the stage's block):
//   ST_LINV: y -> W (kept for the backward sweep) and WP (input of ST_L21)
//   ST_L21:  WP[B] += partials (the update vector u_B for the parent)
//   ST_U12:  WP[own] = y + partials (t)
//   ST_UINV: x_own -> xred
__device__ __forceinline__ double stage_sum(int st, int f, const FrontDev& fr, int r, const StageBufs& sb) {
    int br0, br1, bc0, bc1;
    stage_block(st, fr.nf, fr.F, br0, br1, bc0, bc1);
    const int rows = br1 - br0, nch = (bc1 - bc0 + GC - 1) / GC;
    const double* p = sb.part[st] + sb.off[st][f] + (r - br0);
    double s = 0.0;
    for (int c = 0; c < nch; ++c) s += p[int64_t(c) * rows];
    return s;
}
template <int ST>
__global__ void k_stage_reduce(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, StageBufs sb,
                               double* __restrict__ W, double* __restrict__ WP, double* __restrict__ xred) {
    const int f = lf[blockIdx.y];
    const FrontDev fr = fronts[f];
    int br0, br1, bc0, bc1;
    stage_block(ST, fr.nf, fr.F, br0, br1, bc0, bc1);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= br1 - br0) return;
    const int r = br0 + q;
    const double s = stage_sum(ST, f, fr, r, sb);
    if (ST == ST_LINV) {
        W[fr.woff + r] = s;
        WP[fr.woff + r] = s;
    } else if (ST == ST_L21) {
        WP[fr.woff + r] += s;
    } else if (ST == ST_U12) {
        WP[fr.woff + r] += s;
    } else {
        xred[fr.red0 + r] = s;
    }
}

// Level links of the product sweeps: the epilogue of level h and the gather
// of the next level in one launch (grid.y: the fronts of level h, then those
// of the next level). The next level's gather adds a child's pending partial
// sums itself when the child is at level h, so the two parts never touch the
// same rows.
//   forward, levels h -> h + 1:
//     level h:      y -> W, WP (own rows); u_B = w_B + partials -> WP[B] only
//                   for fronts whose parent is not at level h + 1 (those are
//                   gathered later, from WP);
//     level h + 1:  w = [red_own ; 0] + the children's update vectors, W = w,
//                   WP = P w (own rows), as k_fwd_gather;
//   backward, levels h -> h - 1:
//     level h:      x_own = partials -> xred;
//     level h - 1:  WP = [y ; x_B] as k_bwd_gather, x_B of an ancestor at
//                   level h summed from its partials.
// Sums are formed in the same order as the separate kernels', so results are
// bit-identical to them.
__device__ __forceinline__ double link_update(const FrontDev* __restrict__ fronts, int c, int a, int h,
                                              const double* __restrict__ WP, const StageBufs& sb) {
    const FrontDev ch = fronts[c];
    const double u = WP[ch.woff + ch.nf + a];
    return ch.lvl == h ? u + stage_sum(ST_L21, c, ch, ch.nf + a, sb) : u;
}
__device__ __forceinline__ double link_row(const FrontDev* __restrict__ fronts, const FrontDev& fr, int f, int q, int h,
                                           const double* __restrict__ red, const int* __restrict__ child_of,
                                           const int2* __restrict__ einv, const double* __restrict__ WP,
                                           const StageBufs& sb) {
    double w = q < fr.nf ? red[fr.red0 + q] : 0.0;
    const int2 a = einv[fr.woff + q];
    if (a.x >= 0) w += link_update(fronts, child_of[2 * f], a.x, h, WP, sb);
    if (a.y >= 0) w += link_update(fronts, child_of[2 * f + 1], a.y, h, WP, sb);
    return w;
}
__global__ void k_fwd_link(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, int nfr, const int* __restrict__ lfn,
                           int h, StageBufs sb, const int* __restrict__ child_of, const int2* __restrict__ einv,
                           const int* __restrict__ piv, const double* __restrict__ red, double* __restrict__ W,
                           double* __restrict__ WP, int B) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (int(blockIdx.y) < nfr) {
        const int f = lf[blockIdx.y];
        const FrontDev fr = fronts[f];
        if (q < fr.nf) {
            const double y = stage_sum(ST_LINV, f, fr, q, sb);
            W[fr.woff + q] = y;
            WP[fr.woff + q] = y;
        } else if (q < fr.F && (fr.parent < 0 || fronts[fr.parent].lvl != h + 1)) {
            WP[fr.woff + q] += stage_sum(ST_L21, f, fr, q, sb);
        }
        return;
    }
    const int f = lfn[blockIdx.y - nfr];
    const FrontDev fr = fronts[f];
    if (q >= fr.F) return;
    const double wq = link_row(fronts, fr, f, q, h, red, child_of, einv, WP, sb);
    W[fr.woff + q] = wq;
    WP[fr.woff + q] = q < fr.nf ? link_row(fronts, fr, f, piv_row(piv, fr, q, B), h, red, child_of, einv, WP, sb) : wq;
}
__global__ void k_bwd_link(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, int nfr, const int* __restrict__ lfn,
                           int h, StageBufs sb, const int* __restrict__ vars, const int* __restrict__ owner,
                           const double* __restrict__ W, double* __restrict__ xred, double* __restrict__ WP) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (int(blockIdx.y) < nfr) {
        const int f = lf[blockIdx.y];
        const FrontDev fr = fronts[f];
        if (q < fr.nf) xred[fr.red0 + q] = stage_sum(ST_UINV, f, fr, q, sb) + stage_sum(ST_U12, f, fr, q, sb);
        return;
    }
    const FrontDev fr = fronts[lfn[blockIdx.y - nfr]];
    if (q >= fr.F) return;
    if (q < fr.nf) {
        WP[fr.woff + q] = W[fr.woff + q];
        return;
    }
    const int v = vars[fr.voff + q];
    const int o = owner[v];
    const FrontDev an = fronts[o];
    WP[fr.woff + q] = an.lvl == h ? stage_sum(ST_UINV, o, an, v - an.red0, sb) + stage_sum(ST_U12, o, an, v - an.red0, sb)
                                  : xred[v];
}

// backward prologue: X = [y ; x_B]
__global__ void k_bwd_gather(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, const int* __restrict__ vars,
                             const double* __restrict__ W, const double* __restrict__ xred, double* __restrict__ WP) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= fr.F) return;
    WP[fr.woff + q] = q < fr.nf ? W[fr.woff + q] : xred[vars[fr.voff + q]];
}
// ---------------------------------------------------------------------------
// transposed solve phase (A^T y = c with the same factors; A = P^T L U per
// front):
//   leaves -> root: v_o = Uinv11^T c_o;  u_B = c_B - U12^T v_o
//   root -> leaves: t = v_o - L21^T y_B; y_o = P^T Linv11^T t
// Each stage reads one stored block column-wise: a warp owns a column, its
// lanes stride down the rows (coalesced), and a tile of 64 columns x 256 rows
// writes one partial sum per column.
// ---------------------------------------------------------------------------
constexpr int TCOLS = 64, TROWS = 256;
enum { TS_UINV = 0, TS_U12 = 1, TS_LINV = 2, TS_L21 = 3 };
// rows summed over and columns produced by a transposed stage
__host__ __device__ inline void tstage_block(int st, int nf, int F, int& r0, int& r1, int& c0, int& c1) {
    r0 = st == TS_L21 ? nf : 0;
    r1 = st == TS_L21 ? F : nf;
    c0 = st == TS_U12 ? nf : 0;
    c1 = st == TS_U12 ? F : nf;
}
struct TStageBufs {
    double* part[4];
    const int64_t* off[4];
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}
template <class T, int ST>
__device__ __forceinline__ void tgemv_stage(const WorkItem& it, const FrontDev& fr, const T* __restrict__ front,
                                            const double* __restrict__ X, const TStageBufs& sb) {
    const int F = fr.F, nf = fr.nf;
    int br0, br1, bc0, bc1;
    tstage_block(ST, nf, F, br0, br1, bc0, bc1);
    __shared__ double txs[TROWS];
    __shared__ float2 txs2[TROWS];
    const double* x = X + fr.woff;
    for (int q = threadIdx.x; q < TROWS; q += blockDim.x) {
        const int r = it.row0 + q;
        const double v = r < br1 ? x[r] : 0.0;
        if (sizeof(T) == 4) {
            const float h = __double2float_rn(v);
            txs2[q] = make_float2(h, __double2float_rn(v - double(h)));
        } else {
            txs[q] = v;
        }
    }
    __syncthreads();
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int rend = min(br1, it.row0 + TROWS);
    for (int cc = warp; cc < TCOLS; cc += blockDim.x / 32) {
        const int c = it.col0 + cc;
        if (c >= bc1) break;
        const T* col = ST == TS_U12 ? front + fr.foff + int64_t(F) * nf + int64_t(c - nf) * nf
                                    : front + fr.foff + int64_t(c) * F;
        // rows of this column that the stage uses
        int rb = it.row0, re = rend;
        if (ST == TS_UINV) re = min(re, c + 1);          // upper incl. diagonal: r <= c
        if (ST == TS_LINV) rb = max(rb, c + 1);          // strict lower: r > c
        double out;
        if (sizeof(T) == 4) {
            float sh = 0.f, sl = 0.f;
            for (int r = rb + lane; r < re; r += 32) {
                const float2 xv = txs2[r - it.row0];
                dd_acc(sh, sl, float(col[r]), xv.x, xv.y);
            }
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, sh, o), ol = __shfl_xor_sync(0xffffffffu, sl, o);
                float t, e;
                two_sum(sh, oh, t, e);
                sh = t;
                sl = __fadd_rn(__fadd_rn(sl, ol), e);
            }
            out = double(sh) + double(sl);
        } else {
            double acc = 0.0;
            for (int r = rb + lane; r < re; r += 32) acc += double(col[r]) * txs[r - it.row0];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            out = acc;
        }
        if (ST == TS_LINV && c >= it.row0 && c < rend)   // unit diagonal
            out += sizeof(T) == 4 ? txs2[c - it.row0].x + double(txs2[c - it.row0].y) : txs[c - it.row0];
        if (ST == TS_U12 || ST == TS_L21) out = -out;
        if (lane == 0) sb.part[ST][sb.off[ST][it.front] + int64_t(it.chunk) * (bc1 - bc0) + (c - bc0)] = out;
    }
}
template <class T>
__global__ void __launch_bounds__(256) k_tgemv_part(const FrontDev* __restrict__ fronts,
                                                    const WorkItem* __restrict__ items, const T* __restrict__ front,
                                                    const double* __restrict__ X, TStageBufs sb) {
    const WorkItem it = items[blockIdx.x];
    const FrontDev fr = fronts[it.front];
    switch (it.stage) {
        case TS_UINV: tgemv_stage<T, TS_UINV>(it, fr, front, X, sb); break;
        case TS_U12: tgemv_stage<T, TS_U12>(it, fr, front, X, sb); break;
        case TS_LINV: tgemv_stage<T, TS_LINV>(it, fr, front, X, sb); break;
        default: tgemv_stage<T, TS_L21>(it, fr, front, X, sb); break;
    }
}
__device__ __forceinline__ double tstage_sum(int st, int f, const FrontDev& fr, int c, const TStageBufs& sb) {
    int br0, br1, bc0, bc1;
    tstage_block(st, fr.nf, fr.F, br0, br1, bc0, bc1);
    const int cols = bc1 - bc0, nch = (br1 - br0 + TROWS - 1) / TROWS;
    const double* p = sb.part[st] + sb.off[st][f] + (c - bc0);
    double s = 0.0;
    for (int q = 0; q < nch; ++q) s += p[int64_t(q) * cols];
    return s;
}
// leaves -> root prologue: W = [c_own ; 0] + children's update vectors (no permutation)
__global__ void __launch_bounds__(NT) k_tfwd_gather(const FrontDev* __restrict__ fronts, const int* __restrict__ lf,
                                                    const int* __restrict__ child_of, const int2* __restrict__ einv,
                                                    const double* __restrict__ red, double* __restrict__ W,
                                                    double* __restrict__ WP) {
    // a thread per front row: own rhs (or 0), then the children's update
    // vectors (kept in W) added in slot order through the inverse map
    const int f = lf[blockIdx.y];
    const FrontDev fr = fronts[f];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= fr.F) return;
    double w = q < fr.nf ? red[fr.red0 + q] : 0.0;
    const int2 a = einv[fr.woff + q];
    if (a.x >= 0) {
        const FrontDev ch = fronts[child_of[2 * f]];
        w += W[ch.woff + ch.nf + a.x];
    }
    if (a.y >= 0) {
        const FrontDev ch = fronts[child_of[2 * f + 1]];
        w += W[ch.woff + ch.nf + a.y];
    }
    WP[fr.woff + q] = w;
}
// leaves -> root epilogues: MODE 0 (after UINV^T) v -> W[own], WP[own];
// MODE 1 (after U12^T) W[B] = c_B + sums
template <int MODE>
__global__ void k_tfwd_reduce(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, TStageBufs sb,
                              double* __restrict__ W, double* __restrict__ WP) {
    const int f = lf[blockIdx.y];
    const FrontDev fr = fronts[f];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= fr.F) return;
    if (q < fr.nf) {
        if (MODE != 1) {
            const double v = tstage_sum(TS_UINV, f, fr, q, sb);
            W[fr.woff + q] = v;
            WP[fr.woff + q] = v;
        }
    } else if (MODE != 0) {
        W[fr.woff + q] = WP[fr.woff + q] + tstage_sum(TS_U12, f, fr, q, sb);
    }
}
// root -> leaves prologue: WP = [v_own ; y_B]
__global__ void k_tbwd_gather(const FrontDev* __restrict__ fronts, const int* __restrict__ lf,
                              const int* __restrict__ vars, const double* __restrict__ W,
                              const double* __restrict__ yred, double* __restrict__ WP) {
    const FrontDev fr = fronts[lf[blockIdx.y]];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= fr.F) return;
    WP[fr.woff + q] = q < fr.nf ? W[fr.woff + q] : yred[vars[fr.voff + q]];
}
// root -> leaves epilogues: MODE 0 (after L21^T) WP[own] = v + sum;
// MODE 1 (after LINV^T) y_o = P^T (sum) scattered to yred
template <int MODE>
__global__ void k_tbwd_reduce(const FrontDev* __restrict__ fronts, const int* __restrict__ lf, TStageBufs sb,
                              const int* __restrict__ piv, double* __restrict__ WP, double* __restrict__ yred,
                              int B) {
    const int f = lf[blockIdx.y];
    const FrontDev fr = fronts[f];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= fr.nf) return;
    if (MODE == 0) {
        WP[fr.woff + q] += tstage_sum(TS_L21, f, fr, q, sb);
    } else {
        yred[fr.red0 + piv_row(piv, fr, q, B)] = tstage_sum(TS_LINV, f, fr, q, sb);
    }
}
// reduced transposed right-hand side: column-scaled wet entries
template <class TV>
__global__ void k_treduce_rhs(int nred, const int* __restrict__ r2g, const double* __restrict__ dc,
                              const TV* __restrict__ r, double* __restrict__ red) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nred; q += gridDim.x * blockDim.x) {
        const int g = r2g[q];
        red[q] = dc[g] * double(r[g]);
    }
}
// transposed expansion: row-scaled solution, identity unknowns pass r, gauge zero
template <class TV>
__global__ void k_texpand(int ndim, const int* __restrict__ g2r, const char* __restrict__ isdry,
                          const double* __restrict__ dr, const double* __restrict__ red, const TV* __restrict__ r,
                          TV* __restrict__ z) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ndim; g += gridDim.x * blockDim.x) {
        const int q = g2r[g];
        z[g] = q >= 0 ? TV(dr[g] * red[q]) : (isdry[g] == 2 ? TV(0) : r[g]);
    }
}

__global__ void k_fill(int n, double v, double* __restrict__ a) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) a[q] = v;
}

int blocks_for(int64_t work, int per = NT) {
    int64_t b = (work + per - 1) / per;
    return int(std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32)));
}

}  // namespace

// ===========================================================================
// drivers
// ===========================================================================
NdLu::~NdLu() {
    for (int k = 0; k < 3; ++k) {
        if (sweep_exec[k]) cudaGraphExecDestroy(sweep_exec[k]);
        if (sweep_exec_timed[k]) cudaGraphExecDestroy(sweep_exec_timed[k]);
    }
    if (factor_exec) cudaGraphExecDestroy(factor_exec);
    if (factor_exec_timed) cudaGraphExecDestroy(factor_exec_timed);
    for (auto* t : {&factor_tmpl, &sweep_tmpl[0], &sweep_tmpl[1], &sweep_tmpl[2]})
        for (const KTimer::Rec& r : *t) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
    for (cudaEvent_t e : fork_ev)
        if (e) cudaEventDestroy(e);
    if (join_ev) cudaEventDestroy(join_ev);
    if (side) cudaStreamDestroy(side);
    for (void* p : allocs) cudaFree(p);
}

template <class X>
static X* upload(NdLu& lu, const std::vector<X>& v, cudaStream_t s) {
    X* d = nullptr;
    size_t bytes = sizeof(X) * std::max<size_t>(v.size(), 1);
    if (cudaMalloc(&d, bytes) != cudaSuccess) throw EngineError(IEMIC_ERR_NOMEM);
    lu.allocs.push_back(d);
    if (!v.empty()) ck(cudaMemcpyAsync(d, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice, s));
    return d;
}
static void* dmalloc(NdLu& lu, size_t bytes) {
    void* d = nullptr;
    if (cudaMalloc(&d, std::max<size_t>(bytes, 16)) != cudaSuccess) throw EngineError(IEMIC_ERR_NOMEM);
    lu.allocs.push_back(d);
    return d;
}

void ndlu_setup(NdLu& lu, const NdPlan& plan, int prec, int subst_min_nf) {
    cudaStream_t s = 0;
    ck(cudaFuncSetAttribute(k_fgemm_f32<GM_TRAIL>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(FG_SMEM)));
    ck(cudaFuncSetAttribute(k_task_gemm_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, int(FG_SMEM)));
    lu.prec = prec;
    lu.plan = &plan;
    const size_t ts = prec ? sizeof(float) : sizeof(double);
    lu.d_fronts = upload(lu, plan.fronts, s);
    std::vector<int> lf;
    lu.level_start.clear();
    for (auto& L : plan.level_fronts) {
        lu.level_start.push_back(int(lf.size()));
        lf.insert(lf.end(), L.begin(), L.end());
    }
    lu.level_start.push_back(int(lf.size()));
    lu.d_level_fronts = upload(lu, lf, s);
    for (int sl = 0; sl < 2; ++sl) {
        std::vector<int> cl;
        lu.child_start[sl].clear();
        for (auto& L : plan.level_children[sl]) {
            lu.child_start[sl].push_back(int(cl.size()));
            cl.insert(cl.end(), L.begin(), L.end());
        }
        lu.child_start[sl].push_back(int(cl.size()));
        lu.d_level_children[sl] = upload(lu, cl, s);
    }
    std::vector<int> child_of(2 * size_t(plan.nfronts), -1);
    for (int f = 0; f < plan.nfronts; ++f) {
        int par = plan.fronts[f].parent;
        if (par >= 0) child_of[2 * size_t(par) + plan.child_slot[f]] = f;
    }
    lu.d_vars = upload(lu, plan.vars, s);
    lu.d_emap = upload(lu, plan.emap, s);
    lu.d_r2g = upload(lu, plan.r2g, s);
    lu.d_g2r = upload(lu, plan.g2r, s);
    std::vector<char> isdry(plan.ndim, 0);
    for (int r : plan.dry_rows) isdry[r] = 1;
    for (int r : plan.pins) isdry[r] = 2;
    lu.d_isdry = upload(lu, isdry, s);
    lu.d_dry_ptr = upload(lu, plan.dry_ptr, s);
    lu.d_dry_e = upload(lu, plan.dry_e, s);
    lu.d_dry_c = upload(lu, plan.dry_c, s);
    // inverse extend-add maps: for each row of a front's solve vector, the
    // update-vector row of the child in slot 0 (.x) and slot 1 (.y), or -1
    {
        std::vector<int2> einv(size_t(std::max<int64_t>(plan.w_entries, 1)), make_int2(-1, -1));
        for (int f = 0; f < plan.nfronts; ++f) {
            const FrontDev& ch = plan.fronts[f];
            if (ch.parent < 0) continue;
            const FrontDev& pa = plan.fronts[ch.parent];
            for (int a = 0; a < ch.nb; ++a) {
                const int q = plan.emap[ch.emap_off + a];
                int& slot = plan.child_slot[f] == 0 ? einv[pa.woff + q].x : einv[pa.woff + q].y;
                if (q < 0 || q >= pa.F || slot != -1) throw EngineError(IEMIC_ERR_STATE);
                slot = a;
            }
        }
        lu.d_einv = upload(lu, einv, s);
    }
    lu.d_asm_src = upload(lu, plan.asm_src, s);
    lu.d_asm_dst = upload(lu, plan.asm_dst, s);
    lu.d_asm_row = upload(lu, plan.asm_row, s);
    lu.d_child_of = upload(lu, child_of, s);
    {
        std::vector<int> owner(size_t(std::max(plan.nred, 1)), -1);
        for (int f = 0; f < plan.nfronts; ++f)
            for (int q = 0; q < plan.fronts[f].nf; ++q) owner[size_t(plan.fronts[f].red0) + q] = f;
        lu.d_owner = upload(lu, owner, s);
    }
    lu.d_piv = static_cast<int*>(dmalloc(lu, sizeof(int) * size_t(std::max(plan.nred, 1))));
    lu.d_front = dmalloc(lu, ts * size_t(plan.work_entries));
    lu.d_factor = dmalloc(lu, ts * size_t(std::max<int64_t>(plan.factor_entries, 1)));
    lu.d_contrib = dmalloc(lu, ts * size_t(std::max<int64_t>(plan.contrib_ring * plan.contrib_slot_entries, 1)));
    lu.d_dinv = dmalloc(lu, ts * size_t(plan.dinv_entries));
    lu.d_w = dmalloc(lu, sizeof(double) * size_t(plan.w_entries));
    lu.d_red = dmalloc(lu, sizeof(double) * size_t(std::max(plan.nred, 1)));
    lu.d_dr = static_cast<double*>(dmalloc(lu, sizeof(double) * size_t(plan.ndim)));
    lu.d_dc = static_cast<double*>(dmalloc(lu, sizeof(double) * size_t(plan.ndim)));
    lu.d_cmax = static_cast<double*>(dmalloc(lu, sizeof(double) * size_t(plan.ndim)));
    lu.d_npert = static_cast<int*>(dmalloc(lu, 2 * sizeof(int)));
    lu.d_wp = dmalloc(lu, sizeof(double) * size_t(plan.w_entries));
    // solve-phase partial-sum buffers (per stage) and work items (one launch
    // group per stage)
    std::vector<WorkItem> items[NSTAGE];
    for (int st = 0; st < NSTAGE; ++st) {
        std::vector<int64_t> off(plan.nfronts, 0);
        int64_t poff = 0;
        for (int f = 0; f < plan.nfronts; ++f) {
            const FrontDev& fr = plan.fronts[f];
            int r0, r1, c0, c1;
            stage_block(st, fr.nf, fr.F, r0, r1, c0, c1);
            off[f] = poff;
            poff += int64_t(r1 - r0) * ((c1 - c0 + GC - 1) / GC);
        }
        lu.d_stage_off[st] = upload(lu, off, s);
        const size_t pb = sizeof(double) * size_t(std::max<int64_t>(poff, 1));
        lu.d_stage_part[st] = static_cast<double*>(dmalloc(lu, pb));
        ck(cudaMemsetAsync(lu.d_stage_part[st], 0, pb, s));
    }
    const int group_of[NSTAGE] = {0, 3, 1, 2};   // by stage
    std::vector<WorkItem> gitems[4];
    for (int g = 0; g < 4; ++g) {
        lu.group_start[g].assign(1, 0);
        lu.group_bytes[g].assign(plan.nlevels, 0.0);
    }
    for (int h = 0; h < plan.nlevels; ++h) {
        for (int st = 0; st < NSTAGE; ++st) {
            const int g = group_of[st];
            for (int f : plan.level_fronts[h]) {
                const FrontDev& fr = plan.fronts[f];
                const double nf = fr.nf, nb = fr.nb;
                lu.group_bytes[g][h] += double(ts) * (st == ST_LINV ? nf * (nf - 1) / 2
                                                      : st == ST_UINV ? nf * (nf + 1) / 2 : nf * nb);
                int r0, r1, c0, c1;
                stage_block(st, fr.nf, fr.F, r0, r1, c0, c1);
                for (int c = c0, ch = 0; c < c1; c += GC, ++ch)
                    for (int r = r0; r < r1; r += GT) {
                        // tiles holding no entry of a triangular part are skipped
                        if (st == ST_LINV && r + GT <= fr.nf && c >= r + GT) continue;
                        if (st == ST_UINV && c + GC <= r) continue;
                        gitems[g].push_back(WorkItem{f, r, c, ch, st});
                    }
            }
        }
        for (int g = 0; g < 4; ++g) lu.group_start[g].push_back(int(gitems[g].size()));
    }
    for (int g = 0; g < 4; ++g) lu.d_group_items[g] = upload(lu, gitems[g], s);
    // product sweeps: per level one launch group per sweep, [0] Linv11 and
    // L21 Linv11 (both read P w_own), [1] Uinv11 and Uinv11 U12 (read y and x_B)
    {
        const int mgroup_of[NSTAGE] = {0, 1, 0, 1};
        const int mcode[NSTAGE] = {ST_LINV, ST_UINV, ST_P21, ST_Q12};
        std::vector<WorkItem> mitems[2];
        for (int g = 0; g < 2; ++g) {
            lu.mgroup_start[g].assign(1, 0);
            lu.mgroup_bytes[g].assign(plan.nlevels, 0.0);
        }
        for (int h = 0; h < plan.nlevels; ++h) {
            for (int st = 0; st < NSTAGE; ++st) {
                const int mg = mgroup_of[st];
                for (int f : plan.level_fronts[h]) {
                    const FrontDev& fr = plan.fronts[f];
                    const double nf = fr.nf, nb = fr.nb;
                    lu.mgroup_bytes[mg][h] += double(ts) * (st == ST_LINV ? nf * (nf - 1) / 2
                                                            : st == ST_UINV ? nf * (nf + 1) / 2 : nf * nb);
                    int r0, r1, c0, c1;
                    stage_block(st, fr.nf, fr.F, r0, r1, c0, c1);
                    for (int c = c0, ch = 0; c < c1; c += GC, ++ch)
                        for (int r = r0; r < r1; r += GT) {
                            if (st == ST_LINV && r + GT <= fr.nf && c >= r + GT) continue;
                            if (st == ST_UINV && c + GC <= r) continue;
                            mitems[mg].push_back(WorkItem{f, r, c, ch, mcode[st]});
                        }
                }
            }
            for (int g = 0; g < 2; ++g) lu.mgroup_start[g].push_back(int(mitems[g].size()));
        }
        for (int g = 0; g < 2; ++g) lu.d_mgroup_items[g] = upload(lu, mitems[g], s);
    }
    // block substitution: per level and sub-step k, the fronts with more than
    // k super-blocks take super-block s = k (lower) or s = nsb - 1 - k (upper)
    {
        int64_t pmax = 0;
        for (int up = 0; up < 2; ++up) {
            std::vector<WorkItem> its;
            std::vector<SubDiag> dgs;
            lu.sub_item_start[up].assign(plan.nlevels, {});
            lu.sub_diag_start[up].assign(plan.nlevels, {});
            lu.sub_bytes[up].assign(plan.nlevels, {});
            for (int h = 0; h < plan.nlevels; ++h) {
                const int nk = (plan.level_maxnf[h] + SB - 1) / SB;
                for (int k = 0; k < nk; ++k) {
                    lu.sub_item_start[up][h].push_back(int(its.size()));
                    lu.sub_diag_start[up][h].push_back(int(dgs.size()));
                    int64_t pb = 0;
                    double by = 0.0;
                    for (int f : plan.level_fronts[h]) {
                        const FrontDev& fr = plan.fronts[f];
                        const int nsb = (fr.nf + SB - 1) / SB;
                        if (k >= nsb) continue;
                        const int sblk = up ? nsb - 1 - k : k;
                        const int r0 = sblk * SB, r1 = std::min(fr.nf, r0 + SB);
                        const int cb = up ? r1 : 0, ce = up ? fr.nf : r0;   // off-diagonal columns
                        const int nch = (ce - cb + SB - 1) / SB;
                        if (pb + int64_t(SB) * nch > INT32_MAX) throw EngineError(IEMIC_ERR_NOMEM);
                        for (int ch = 0; ch < nch; ++ch)
                            for (int r = r0; r < r1; r += GT) its.push_back(WorkItem{f, r, cb + ch * SB, ch, int(pb)});
                        dgs.push_back(SubDiag{f, sblk, int(pb), nch});
                        pb += int64_t(SB) * nch;
                        const double m = r1 - r0;
                        by += double(ts) * (m * (ce - cb) + m * (m + (up ? 1 : -1)) / 2);
                    }
                    pmax = std::max(pmax, pb);
                    lu.sub_bytes[up][h].push_back(by);
                }
                lu.sub_item_start[up][h].push_back(int(its.size()));
                lu.sub_diag_start[up][h].push_back(int(dgs.size()));
            }
            lu.d_sub_items[up] = upload(lu, its, s);
            lu.d_sub_diag[up] = upload(lu, dgs, s);
        }
        lu.d_sub_part = static_cast<double*>(dmalloc(lu, sizeof(double) * size_t(std::max<int64_t>(pmax, 1))));
    }
    // transposed solve: partial buffers per stage (columns x row chunks) and
    // work items, one launch group per stage
    for (int st = 0; st < 4; ++st) {
        std::vector<int64_t> off(plan.nfronts, 0);
        int64_t poff = 0;
        for (int f = 0; f < plan.nfronts; ++f) {
            const FrontDev& fr = plan.fronts[f];
            int r0, r1, c0, c1;
            tstage_block(st, fr.nf, fr.F, r0, r1, c0, c1);
            off[f] = poff;
            poff += int64_t(c1 - c0) * ((r1 - r0 + TROWS - 1) / TROWS);
        }
        lu.d_tstage_off[st] = upload(lu, off, s);
        const size_t pb = sizeof(double) * size_t(std::max<int64_t>(poff, 1));
        lu.d_tstage_part[st] = static_cast<double*>(dmalloc(lu, pb));
        ck(cudaMemsetAsync(lu.d_tstage_part[st], 0, pb, s));
    }
    {
        const int tgroup_of[4] = {0, 1, 2, 3};   // TS_UINV, TS_U12, TS_LINV, TS_L21
        std::vector<WorkItem> titems[4];
        for (int g = 0; g < 4; ++g) lu.tgroup_start[g].assign(1, 0);
        for (int h = 0; h < plan.nlevels; ++h) {
            for (int st = 0; st < 4; ++st) {
                const int g = tgroup_of[st];
                for (int f : plan.level_fronts[h]) {
                    const FrontDev& fr = plan.fronts[f];
                    int r0, r1, c0, c1;
                    tstage_block(st, fr.nf, fr.F, r0, r1, c0, c1);
                    for (int r = r0, ch = 0; r < r1; r += TROWS, ++ch)
                        for (int c = c0; c < c1; c += TCOLS) {
                            // skip tiles with no entry of a triangular part
                            if (st == TS_UINV && r > c + TCOLS - 1) continue;        // needs r <= c
                            if (st == TS_LINV && r + TROWS <= c) continue;           // needs r >= c (diag: r == c)
                            titems[g].push_back(WorkItem{f, r, c, ch, st});
                        }
                }
            }
            for (int g = 0; g < 4; ++g) lu.tgroup_start[g].push_back(int(titems[g].size()));
        }
        for (int g = 0; g < 4; ++g) lu.d_tgroup_items[g] = upload(lu, titems[g], s);
    }
    // recursive triangular inversion: tasks and 64x64 tiles per (level, merge
    // size, phase); phase-1 products go to a scratch area of their own
    {
        std::vector<TriTask> tasks;
        std::vector<TriTile> tiles;
        std::vector<SplitGroup> groups;
        const int tile = prec ? FG_TM : 64;   // k_task_gemm_f32 / k_tri_gemm tile size
        int64_t tmax = 0, tmax2 = 0;
        int maxnf = 0;
        for (int h = 0; h < plan.nlevels; ++h) maxnf = std::max(maxnf, plan.level_maxnf[h]);
        lu.subst = maxnf > subst_min_nf;
        lu.products = !lu.subst;
        lu.tri_ranges.clear();
        lu.inv2_ranges.clear();
        lu.prod_ranges.clear();
        for (int h = 0; h < plan.nlevels; ++h) {
            std::vector<std::pair<int, int>> lv, lv2, lv3;
            auto emit = [&](const TriTask& t) {
                const int id = int(tasks.size());
                tasks.push_back(t);
                for (int j = 0; j < t.N; j += tile)
                    for (int i = 0; i < t.M; i += tile) tiles.push_back(TriTile{id, i, j});
            };
            // (1) merges inside the 256-row super-blocks: sz = 32, 64, 128
            for (int sz = plan.panel; sz < TRI_SB && sz < plan.level_maxnf[h]; sz *= 2) {
                for (int phase = 0; phase < 2; ++phase) {
                    const int tb = int(tiles.size());
                    int64_t toff = 0;
                    for (int f : plan.level_fronts[h]) {
                        const FrontDev& fr = plan.fronts[f];
                        const int nf = fr.nf, F = fr.F;
                        for (int a0 = 0; a0 + sz < nf; a0 += 2 * sz) {
                            const int a1 = a0 + sz, d0 = a1, d1 = std::min(nf, a1 + sz);
                            const int na = a1 - a0, nd = d1 - d0;
                            for (int up = 0; up < 2; ++up) {
                                const int64_t tcur = toff;
                                toff += int64_t(na) * nd;
                                if (!up && phase == 0)            // T = L21blk * Ainv   (nd x na)
                                    emit(TriTask{fr.foff + int64_t(a0) * F + d0, fr.foff + int64_t(a0) * F + a0, tcur,
                                                 F, F, nd, nd, na, na, OP_DENSE, OP_LOWER_UNIT, 0, 0, 1, 1.f});
                                else if (!up)                     // X21 = -Dinv * T
                                    emit(TriTask{fr.foff + int64_t(d0) * F + d0, tcur, fr.foff + int64_t(a0) * F + d0,
                                                 F, nd, F, nd, na, nd, OP_LOWER_UNIT, OP_DENSE, 0, 1, 0, -1.f});
                                else if (phase == 0)              // T = Ainv * U12blk   (na x nd)
                                    emit(TriTask{fr.foff + int64_t(a0) * F + a0, fr.foff + int64_t(d0) * F + a0, tcur,
                                                 F, F, na, na, nd, na, OP_UPPER, OP_DENSE, 0, 0, 1, 1.f});
                                else                              // X12 = -T * Dinv
                                    emit(TriTask{tcur, fr.foff + int64_t(d0) * F + d0, fr.foff + int64_t(d0) * F + a0,
                                                 na, F, F, na, nd, nd, OP_DENSE, OP_UPPER, 1, 0, 0, -1.f});
                            }
                        }
                    }
                    tmax = std::max(tmax, toff);
                    lv.push_back({tb, int(tiles.size())});
                }
            }
            // (2) block-row steps over the super-blocks (row-oriented inversion,
            //     run on demand in the factor store, for transposed solves,
            //     whose rounding involves one large inverse per product):
            //     lower, top down:  X[Ri, 0:i0] = -Linv_ii (L[Ri, 0:i0] X[0:i0, 0:i0])
            //     upper, bottom up: Y[Ri, i1:nf] = -Uinv_ii (U[Ri, i1:nf] Y[i1:nf, i1:nf])
            const int nsb_max = (plan.level_maxnf[h] + TRI_SB - 1) / TRI_SB;
            // long products (w > TRI_KS) are split along K into TRI_KS pieces
            auto nsplit = [](int w) { return w > 2 * TRI_KS ? (w + TRI_KS - 1) / TRI_KS : 1; };
            for (int t = 1; t < nsb_max; ++t) {
                for (int phase = 0; phase < 2; ++phase) {
                    const int tb = int(tiles.size());
                    const int gb = int(groups.size());
                    int64_t toff = 0;
                    for (int f : plan.level_fronts[h]) {
                        const FrontDev& fr = plan.fronts[f];
                        const int nf = fr.nf, F = fr.F;
                        const int nsb = (nf + TRI_SB - 1) / TRI_SB;
                        if (t >= nsb) continue;
                        {   // lower, super-block row i = t
                            const int r0 = t * TRI_SB, r1 = std::min(nf, r0 + TRI_SB), m = r1 - r0, w = r0;
                            const int ns = nsplit(w);
                            const int64_t tcur = toff;
                            toff += int64_t(m) * w * ns;
                            if (phase == 0) {   // T = L[Ri, 0:r0] * X[0:r0, 0:r0]   (m x w), split along K
                                for (int sp = 0; sp < ns; ++sp) {
                                    TriTask tk{fr.foff + r0, fr.foff, tcur + int64_t(sp) * m * w, F, F, m, m, w, w,
                                               OP_DENSE, OP_LOWER_UNIT, 0, 0, 1, 1.f};
                                    tk.k0 = sp * TRI_KS;
                                    tk.k1 = ns > 1 ? std::min(w, (sp + 1) * TRI_KS) : w;
                                    emit(tk);
                                }
                                if (ns > 1) groups.push_back(SplitGroup{tcur, int64_t(m) * w, ns});
                            } else {            // X[Ri, 0:r0] = -Linv_ii * T
                                emit(TriTask{fr.foff + int64_t(r0) * F + r0, tcur, fr.foff + r0, F, m, F, m, w, m,
                                             OP_LOWER_UNIT, OP_DENSE, 0, 1, 0, -1.f});
                            }
                        }
                        {   // upper, super-block row i = nsb - 1 - t
                            const int i = nsb - 1 - t;
                            const int r0 = i * TRI_SB, r1 = r0 + TRI_SB, m = r1 - r0, w = nf - r1;
                            const int ns = nsplit(w);
                            const int64_t tcur = toff;
                            toff += int64_t(m) * w * ns;
                            if (phase == 0) {   // T = U[Ri, r1:nf] * Y[r1:nf, r1:nf]   (m x w), split along K
                                for (int sp = 0; sp < ns; ++sp) {
                                    TriTask tk{fr.foff + int64_t(r1) * F + r0, fr.foff + int64_t(r1) * F + r1,
                                               tcur + int64_t(sp) * m * w, F, F, m, m, w, w, OP_DENSE, OP_UPPER,
                                               0, 0, 1, 1.f};
                                    tk.k0 = sp * TRI_KS;
                                    tk.k1 = ns > 1 ? std::min(w, (sp + 1) * TRI_KS) : w;
                                    emit(tk);
                                }
                                if (ns > 1) groups.push_back(SplitGroup{tcur, int64_t(m) * w, ns});
                            } else {            // Y[Ri, r1:nf] = -Uinv_ii * T
                                emit(TriTask{fr.foff + int64_t(r0) * F + r0, tcur, fr.foff + int64_t(r1) * F + r0,
                                             F, m, F, m, w, m, OP_UPPER, OP_DENSE, 0, 1, 0, -1.f});
                            }
                        }
                    }
                    tmax2 = std::max(tmax2, toff);
                    lv2.push_back({tb, int(tiles.size())});
                    if (int(groups.size()) > gb) lv2.push_back({-1 - gb, -1 - int(groups.size())});   // split-K reduce
                }
            }
            // (3) whole-inverse plans: the products of the solve sweeps, into
            //     the product store (the tasks' scratch) at the offsets of the
            //     blocks they replace:  L21 Linv11 (nb x nf)  and  Uinv11 U12 (nf x nb)
            if (lu.products) {
                const int tb = int(tiles.size());
                for (int f : plan.level_fronts[h]) {
                    const FrontDev& fr = plan.fronts[f];
                    const int nf = fr.nf, nb = fr.nb, F = fr.F;
                    if (nf == 0 || nb == 0) continue;
                    const int64_t l21 = fr.foff + nf, u12 = fr.foff + int64_t(F) * nf;
                    emit(TriTask{l21, fr.foff, l21, F, F, F, nb, nf, nf, OP_DENSE, OP_LOWER_UNIT, 0, 0, 1, 1.f});
                    emit(TriTask{fr.foff, u12, u12, F, nf, nf, nf, nb, nf, OP_UPPER, OP_DENSE, 0, 0, 1, 1.f});
                }
                if (int(tiles.size()) > tb) lv3.push_back({tb, int(tiles.size())});
            }
            lu.tri_ranges.push_back(lv);
            lu.inv2_ranges.push_back(lv2);
            lu.prod_ranges.push_back(lv3);
        }
        lu.d_tri_tasks = upload(lu, tasks, s);
        lu.d_tri_tiles = upload(lu, tiles, s);
        lu.d_tri_groups = upload(lu, groups, s);
        lu.d_tri_scratch = dmalloc(lu, ts * size_t(std::max<int64_t>(tmax, 1)));
        lu.inv2_scratch_entries = tmax2;
        if (!lu.subst) lu.d_inv2_scratch = dmalloc(lu, ts * size_t(std::max<int64_t>(tmax2, 1)));
        if (lu.products) {
            const size_t pb = ts * size_t(std::max<int64_t>(plan.factor_entries, 1));
            lu.d_prod = dmalloc(lu, pb);
            ck(cudaMemsetAsync(lu.d_prod, 0, pb, s));
        }
        ck(cudaStreamCreateWithFlags(&lu.side, cudaStreamNonBlocking));
        lu.fork_ev.assign(plan.nlevels, nullptr);
        for (auto& e : lu.fork_ev) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ck(cudaEventCreateWithFlags(&lu.join_ev, cudaEventDisableTiming));
        lu.tri_flops = 0.0;
        for (const TriTask& t : tasks) lu.tri_flops += double(t.M) * t.N * t.K;   // ~ half are structural zeros
    }

    ck(cudaStreamSynchronize(s));
}

// Ruiz equilibration (FP64) of the wet block of J: each sweep divides rows and
// then columns by the square roots of their largest magnitudes
constexpr int kRuizSweeps = 8;
static void equilibrate(NdLu& lu, const int* rp, const int* ci, const double* val, cudaStream_t s) {
    const NdPlan& P = *lu.plan;
    const int nd = P.ndim, G = blocks_for(nd);
    k_fill<<<G, NT, 0, s>>>(nd, 1.0, lu.d_dr); IEMIC_COUNT_LAUNCH();
    k_fill<<<G, NT, 0, s>>>(nd, 1.0, lu.d_dc); IEMIC_COUNT_LAUNCH();
    for (int it = 0; it < kRuizSweeps; ++it) {
        k_rowmax<<<G, NT, 0, s>>>(nd, lu.d_g2r, rp, ci, val, lu.d_dc, lu.d_dr); IEMIC_COUNT_LAUNCH();
        ck(cudaMemsetAsync(lu.d_cmax, 0, sizeof(double) * nd, s));
        k_colmax<<<G, NT, 0, s>>>(nd, lu.d_g2r, rp, ci, val, lu.d_dr, lu.d_dc, lu.d_cmax); IEMIC_COUNT_LAUNCH();
        k_colscale<<<G, NT, 0, s>>>(nd, lu.d_g2r, lu.d_cmax, lu.d_dc); IEMIC_COUNT_LAUNCH();
    }
}

// One launch range of the triangular-inversion tasks (k >= 0: task tiles;
// negative: the split-K reduce of a group range); `base` is the storage the
// tasks' offsets refer to (working area or factor store).
template <class T>
static void tri_range(NdLu& lu, const std::pair<int, int>& rg, T* base, T* scr, cudaStream_t s) {
    if (rg.first < 0) {   // split-K reduce of groups [-1-first, -1-second)
        const int g0 = -1 - rg.first, g1 = -1 - rg.second;
        k_split_reduce<T><<<dim3(64, std::min(g1 - g0, 65535)), 256, 0, s>>>(
            static_cast<const SplitGroup*>(lu.d_tri_groups) + g0, g1 - g0, scr); IEMIC_COUNT_LAUNCH();
        return;
    }
    if (rg.second <= rg.first) return;
    const TriTask* tk = static_cast<const TriTask*>(lu.d_tri_tasks);
    const TriTile* tl = static_cast<const TriTile*>(lu.d_tri_tiles) + rg.first;
    if constexpr (sizeof(T) == 4)
        k_task_gemm_f32<<<rg.second - rg.first, 256, FG_SMEM, s>>>(tk, tl, reinterpret_cast<float*>(base),
                                                                   reinterpret_cast<float*>(scr));
    else
        k_tri_gemm<T><<<rg.second - rg.first, 256, 0, s>>>(tk, tl, base, scr);
    IEMIC_COUNT_LAUNCH();
}

// Whole-block inverses Linv11 / Uinv11 in the factor store (the row-oriented
// steps over the super-blocks), for the transposed sweeps; run once per
// factorisation, when the first transposed solve needs them.
template <class T>
static void to_full_inverse(NdLu& lu, cudaStream_t s) {
    if (lu.full_inverse) return;
    if (!lu.d_inv2_scratch)
        lu.d_inv2_scratch = dmalloc(lu, sizeof(T) * size_t(std::max<int64_t>(lu.inv2_scratch_entries, 1)));
    cudaEvent_t ev = lu.timer ? lu.timer->start(s) : nullptr;
    for (const auto& lv : lu.inv2_ranges)
        for (const auto& rg : lv) tri_range<T>(lu, rg, static_cast<T*>(lu.d_factor), static_cast<T*>(lu.d_inv2_scratch), s);
    if (ev) lu.timer->stop(ev, s, IEMIC_KC_FACTOR_INVERSE, 0.0, 0.0);
    ck(cudaGetLastError());
    lu.full_inverse = true;
}

template <class T, int B>
static void factor_body(NdLu& lu, const int* rp, const int* ci, const double* values, cudaStream_t s) {
    const NdPlan& P = *lu.plan;
    T* front = static_cast<T*>(lu.d_front);
    T* dinv = static_cast<T*>(lu.d_dinv);
    const T tau = sizeof(T) == 4 ? T(1e-7) : T(1e-15);
    T* factor = static_cast<T*>(lu.d_factor);
    T* contrib = static_cast<T*>(lu.d_contrib);
    cudaEvent_t ev_fs = lu.timer ? lu.timer->start(s) : nullptr;
    equilibrate(lu, rp, ci, values, s);
    ck(cudaMemsetAsync(lu.d_npert, 0, 2 * sizeof(int), s));
    if (ev_fs) lu.timer->stop(ev_fs, s, IEMIC_KC_FACTOR_SETUP, 0.0, 0.0);
    for (int h = 0; h < P.nlevels; ++h) {
        const int nfr = lu.level_start[h + 1] - lu.level_start[h];
        const int* lf = lu.d_level_fronts + lu.level_start[h];
        cudaEvent_t ev_ea = lu.timer ? lu.timer->start(s) : nullptr;
        // the level's fronts in the working area: J's entries, then the children's contributions
        ck(cudaMemsetAsync(front, 0, sizeof(T) * size_t(P.level_work[h]), s));
        {
            const int64_t a0 = P.asm_level_start[h], na = P.asm_level_start[h + 1] - a0;
            if (na > 0) {
                k_assemble<T><<<blocks_for(na), NT, 0, s>>>(na, lu.d_asm_src + a0, lu.d_asm_dst + a0, lu.d_asm_row + a0,
                                                            ci, values, lu.d_dr, lu.d_dc, front); IEMIC_COUNT_LAUNCH();
            }
        }
        for (int sl = 0; sl < 2; ++sl) {
            int nc = lu.child_start[sl][h + 1] - lu.child_start[sl][h];
            if (nc == 0) continue;
            int mx = 1;
            for (int c : P.level_children[sl][h]) mx = std::max(mx, P.fronts[c].nb);
            dim3 g(std::max(1, std::min(mx, (152 * 16 + nc - 1) / nc)), nc);
            k_extend_add<T><<<g, NT, 0, s>>>(lu.d_fronts, lu.d_level_children[sl] + lu.child_start[sl][h], lu.d_emap,
                                             contrib, front); IEMIC_COUNT_LAUNCH();
        }
        if (ev_ea) lu.timer->stop(ev_ea, s, IEMIC_KC_FACTOR_SETUP, 0.0, 0.0);
        const int maxnf = P.level_maxnf[h], maxF = P.level_maxF[h];
        constexpr int TM = sizeof(T) == 4 ? 128 : 64;
        auto tiles = [](int n) { return (std::max(n, 1) + TM - 1) / TM; };
        // host-side flop and byte counts of a GEMM launch (timing only)
        auto gemm_cost = [&](int mode, int p, int P0, double& fl, double& by) {
            fl = by = 0.0;
            for (int f : P.level_fronts[h]) {
                const FrontDev& fr = P.fronts[f];
                if (fr.nf <= (mode == GM_TRAIL ? P0 : p)) continue;
                const int cend = std::min(P0 + OB, fr.nf), bb = std::min(B, fr.nf - p);
                double Mr, Nc, K;
                if (mode == GM_STRIP) { Mr = fr.F - p - bb; Nc = cend - p - bb; K = bb; }
                else if (mode == GM_BAND) { Mr = cend - p - bb; Nc = fr.F - cend; K = bb; }
                else { Mr = fr.F - cend; Nc = fr.F - cend; K = cend - P0; }
                if (Mr <= 0 || Nc <= 0) continue;
                fl += 2.0 * Mr * Nc * K;
                by += double(sizeof(T)) * (2.0 * Mr * Nc + Mr * K + K * Nc);
            }
        };
        constexpr int TS = 64;   // tile of the strip and band updates
        auto tiles_s = [](int n) { return (std::max(n, 1) + TS - 1) / TS; };
        auto fgemm = [&](int mode, dim3 grid, int p, int P0) {
            if constexpr (sizeof(T) == 4) {
                float* fp = reinterpret_cast<float*>(front);
                // the K = 32 strip and band updates are skinny (one side <= OB):
                // 64 x 64 tiles give them four times the CTAs of 128 x 128
                if (mode == GM_STRIP) k_fgemm<float, GM_STRIP, TS><<<grid, 256, 0, s>>>(lu.d_fronts, lf, p, P0, fp);
                else if (mode == GM_BAND) k_fgemm<float, GM_BAND, TS><<<grid, 256, 0, s>>>(lu.d_fronts, lf, p, P0, fp);
                else k_fgemm_f32<GM_TRAIL><<<grid, 256, FG_SMEM, s>>>(lu.d_fronts, lf, p, P0, fp);
            } else {
                if (mode == GM_STRIP) k_fgemm<T, GM_STRIP, TM><<<grid, 256, 0, s>>>(lu.d_fronts, lf, p, P0, front);
                else if (mode == GM_BAND) k_fgemm<T, GM_BAND, TM><<<grid, 256, 0, s>>>(lu.d_fronts, lf, p, P0, front);
                else k_fgemm<T, GM_TRAIL, TM><<<grid, 256, 0, s>>>(lu.d_fronts, lf, p, P0, front);
            }
            IEMIC_COUNT_LAUNCH();
        };
        auto timed_gemm = [&](int mode, int p, int P0, auto launch) {
            cudaEvent_t ev = lu.timer ? lu.timer->start(s) : nullptr;
            launch();
            if (ev) {
                double fl, by;
                gemm_cost(mode, p, P0, fl, by);
                lu.timer->stop(ev, s, IEMIC_KC_FACTOR_GEMM, by, fl);
            }
        };
        // two-level blocked LU: outer panels of OB columns, inner panels of B
        for (int P0 = 0; P0 < maxnf; P0 += OB) {
            const int pend = std::min(P0 + OB, maxnf);
            for (int p = P0; p < pend; p += B) {
                cudaEvent_t ev_pn = lu.timer ? lu.timer->start(s) : nullptr;
                k_panel_diag<T, B><<<nfr, 32, 0, s>>>(lu.d_fronts, lf, p, front, dinv, lu.d_piv, tau, lu.d_npert); IEMIC_COUNT_LAUNCH();
                dim3 g1((maxF + NT - 1) / NT, nfr);
                k_rowperm_u12<T, B><<<g1, NT, 0, s>>>(lu.d_fronts, lf, p, P0, front, dinv, lu.d_piv); IEMIC_COUNT_LAUNCH();
                dim3 g3((maxF - p + NT - 1) / NT, nfr);
                k_l21<T, B><<<g3, NT, 0, s>>>(lu.d_fronts, lf, p, front, dinv); IEMIC_COUNT_LAUNCH();
                if (ev_pn) lu.timer->stop(ev_pn, s, IEMIC_KC_FACTOR_PANEL, 0.0, 0.0);
                if (p + B < pend) {   // update inside the outer panel
                    timed_gemm(GM_STRIP, p, P0, [&] {
                        fgemm(GM_STRIP, dim3(tiles_s(maxF - p) * tiles_s(OB), nfr), p, P0);
                    });
                }
            }
            // band rows of the columns past the outer panel
            for (int p = P0; p < pend; p += B) {
                cudaEvent_t ev_pn = lu.timer ? lu.timer->start(s) : nullptr;
                k_band_u12<T, B><<<dim3((maxF - P0 + NT - 1) / NT, nfr), NT, 0, s>>>(lu.d_fronts, lf, p, P0, front,
                                                                                      dinv); IEMIC_COUNT_LAUNCH();
                if (ev_pn) lu.timer->stop(ev_pn, s, IEMIC_KC_FACTOR_PANEL, 0.0, 0.0);
                if (p + B < pend) {
                    timed_gemm(GM_BAND, p, P0, [&] {
                        fgemm(GM_BAND, dim3(tiles_s(OB) * tiles_s(maxF - P0), nfr), p, P0);
                    });
                }
            }
            timed_gemm(GM_TRAIL, P0, P0, [&] {
                fgemm(GM_TRAIL, dim3(tiles(maxF - P0) * tiles(maxF - P0), nfr), P0, P0);
            });
        }
        cudaEvent_t ev_sp = lu.timer ? lu.timer->start(s) : nullptr;
        const int gx = std::max(1, std::min(maxF, (152 * 16 + nfr - 1) / nfr));
        k_spill<T><<<dim3(gx, nfr), 256, 0, s>>>(lu.d_fronts, lf, front, factor, contrib); IEMIC_COUNT_LAUNCH();
        if (ev_sp) lu.timer->stop(ev_sp, s, IEMIC_KC_FACTOR_SETUP, 2.0 * sizeof(T) * double(P.level_work[h]), 0.0);
        // explicit inverses for the solve phase, in the factor store, on the
        // side stream: they touch only this level's nf x nf blocks and their
        // own scratch, so the next levels factor meanwhile. The inverted
        // diagonal panel blocks, then merges inside the 256-row super-blocks
        // (each diagonal super-block of L11 / U11 then holds its inverse), then
        // for whole-inverse plans the row-oriented steps over the super-blocks.
        ck(cudaEventRecord(lu.fork_ev[h], s));
        ck(cudaStreamWaitEvent(lu.side, lu.fork_ev[h], 0));
        cudaEvent_t ev_inv = lu.timer ? lu.timer->start(lu.side) : nullptr;
        const int maxblk = (maxnf + B - 1) / B;
        k_put_diag_inv<T, B><<<dim3(std::max(maxblk, 1), nfr), NT, 0, lu.side>>>(lu.d_fronts, lf, factor, dinv); IEMIC_COUNT_LAUNCH();
        for (const auto& rg : lu.tri_ranges[h]) tri_range<T>(lu, rg, factor, static_cast<T*>(lu.d_tri_scratch), lu.side);
        if (!lu.subst)
            for (const auto& rg : lu.inv2_ranges[h])
                tri_range<T>(lu, rg, factor, static_cast<T*>(lu.d_inv2_scratch), lu.side);
        if (lu.products)
            for (const auto& rg : lu.prod_ranges[h]) tri_range<T>(lu, rg, factor, static_cast<T*>(lu.d_prod), lu.side);
        if (ev_inv) lu.timer->stop(ev_inv, lu.side, IEMIC_KC_FACTOR_INVERSE, 0.0, 0.0);
    }
    // the factorisation ends when the side stream's inverses are done
    ck(cudaEventRecord(lu.join_ev, lu.side));
    ck(cudaStreamWaitEvent(s, lu.join_ev, 0));
}

// Captures the launches of body() on stream s into a new graph. If body()
// throws, the capture is ended and its partial graph destroyed before the
// exception propagates, so the stream is never left capturing.
template <class F>
static cudaGraph_t capture_graph(cudaStream_t s, F body) {
    ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        body();
    } catch (...) {
        cudaGraph_t partial = nullptr;
        if (cudaStreamEndCapture(s, &partial) == cudaSuccess && partial) cudaGraphDestroy(partial);
        (void)cudaGetLastError();
        throw;
    }
    cudaGraph_t g = nullptr;
    ck(cudaStreamEndCapture(s, &g));
    return g;
}
// The factorisation is a fixed sequence of ~1,400 launches over buffers that
// do not move (the CSR arrays of the engine and the factor storage), so it is
// captured once into a CUDA graph and replayed; with kernel timing on it runs
// eagerly so that every launch can be timed.
// Capture `body` into a graph whose launches are timed by event nodes
// (records into `tmpl`), once, then replay it and queue its records.
template <class F>
static void timed_graph(NdLu& lu, cudaGraphExec_t& exec, std::vector<KTimer::Rec>& tmpl, long long& nlaunch,
                        cudaStream_t s, F body) {
    if (!exec) {
        const long long n0 = launch_counter();
        cudaGraph_t g = capture_graph(s, [&] {
            lu.timer->sink = &tmpl;
            try {
                body();
            } catch (...) {
                lu.timer->sink = nullptr;
                throw;
            }
            lu.timer->sink = nullptr;
        });
        nlaunch = launch_counter() - n0;
        launch_counter() = n0;
        const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        ck(e);
    }
    ck(cudaGraphLaunch(exec, s));
    launch_counter() += nlaunch;
    lu.timer->replayed(tmpl);
}

template <class T, int B>
static void factor_t(NdLu& lu, const int* rp, const int* ci, const double* values, cudaStream_t s) {
    if (lu.timer && lu.timer->on) {
        if (lu.factor_exec_timed && (lu.fg_rp != rp || lu.fg_ci != ci || lu.fg_val != values)) {
            // new CSR buffers: recapture, as the untimed path does; the old
            // template's events are retired once their records are drained
            ck(cudaStreamSynchronize(s));
            lu.timer->drain();
            cudaGraphExecDestroy(lu.factor_exec_timed);
            lu.factor_exec_timed = nullptr;
            for (const KTimer::Rec& r : lu.factor_tmpl) {
                cudaEventDestroy(r.a);
                cudaEventDestroy(r.b);
            }
            lu.factor_tmpl.clear();
        }
        lu.fg_rp = rp;
        lu.fg_ci = ci;
        lu.fg_val = values;
        timed_graph(lu, lu.factor_exec_timed, lu.factor_tmpl, lu.factor_launches_timed, s,
                    [&] { factor_body<T, B>(lu, rp, ci, values, s); });
    } else {
        if (lu.factor_exec && (lu.fg_rp != rp || lu.fg_ci != ci || lu.fg_val != values)) {
            cudaGraphExecDestroy(lu.factor_exec);
            lu.factor_exec = nullptr;
        }
        if (!lu.factor_exec) {
            const long long n0 = launch_counter();
            cudaGraph_t g = capture_graph(s, [&] { factor_body<T, B>(lu, rp, ci, values, s); });
            lu.factor_launches = launch_counter() - n0;
            launch_counter() = n0;
            const cudaError_t e = cudaGraphInstantiate(&lu.factor_exec, g, 0);
            cudaGraphDestroy(g);
            ck(e);
            lu.fg_rp = rp;
            lu.fg_ci = ci;
            lu.fg_val = values;
        }
        ck(cudaGraphLaunch(lu.factor_exec, s));
        launch_counter() += lu.factor_launches;
    }
    ck(cudaGetLastError());
    int cnt[2] = {0, 0};
    ck(cudaMemcpyAsync(cnt, lu.d_npert, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    ck(cudaStreamSynchronize(s));
    lu.npert = cnt[0];
    lu.nnan = cnt[1];
    lu.full_inverse = !lu.subst;
    lu.factored = lu.nnan == 0;
    if (!lu.factored) throw EngineError(IEMIC_ERR_NAN);   // the factors overflowed
}

void ndlu_factor(NdLu& lu, const int* rp, const int* ci, const double* values, cudaStream_t s) {
    if (lu.prec) factor_t<float, 32>(lu, rp, ci, values, s);
    else factor_t<double, 32>(lu, rp, ci, values, s);
}

static StageBufs stage_bufs(NdLu& lu) {
    StageBufs sb;
    for (int st = 0; st < NSTAGE; ++st) {
        sb.part[st] = lu.d_stage_part[st];
        sb.off[st] = lu.d_stage_off[st];
    }
    return sb;
}
template <class T>
static void launch_group(NdLu& lu, int g, int h, const T* front, double* WP, cudaStream_t s) {
    const int ni = lu.group_start[g][h + 1] - lu.group_start[g][h];
    if (!ni) return;
    cudaEvent_t ev = lu.timer ? lu.timer->start(s) : nullptr;
    k_gemv_part<T><<<ni, GR, 0, s>>>(lu.d_fronts, static_cast<const WorkItem*>(lu.d_group_items[g]) +
                                         lu.group_start[g][h], front, front, WP, stage_bufs(lu)); IEMIC_COUNT_LAUNCH();
    if (ev) lu.timer->stop(ev, s, IEMIC_KC_SOLVE_GEMV, lu.group_bytes[g][h], 2.0 * lu.group_bytes[g][h] / sizeof(T));
}
// one GEMV launch of the product sweeps (g = 0 forward, 1 backward) over
// level h: both stages of the level
template <class T>
static void launch_mgemv(NdLu& lu, int g, int h, double* WP, cudaStream_t s) {
    KTimer* kt = lu.timer;
    const int ni = lu.mgroup_start[g][h + 1] - lu.mgroup_start[g][h];
    if (ni <= 0) return;
    cudaEvent_t ev = kt ? kt->start(s) : nullptr;
    k_gemv_part<T><<<ni, GR, 0, s>>>(lu.d_fronts, static_cast<const WorkItem*>(lu.d_mgroup_items[g]) +
                                         lu.mgroup_start[g][h], static_cast<const T*>(lu.d_factor),
                                     static_cast<const T*>(lu.d_prod), WP, stage_bufs(lu)); IEMIC_COUNT_LAUNCH();
    if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_GEMV, lu.mgroup_bytes[g][h], 2.0 * lu.mgroup_bytes[g][h] / sizeof(T));
}
// the level link after level h's GEMV: its epilogue and the gather of the
// next level hn (forward h + 1, backward h - 1; -1: none, the sweep's end)
static void launch_link(NdLu& lu, bool up, int h, int hn, double* W, double* WP, double* red, int B, cudaStream_t s) {
    const NdPlan& P = *lu.plan;
    KTimer* kt = lu.timer;
    const int nfr = lu.level_start[h + 1] - lu.level_start[h];
    const int* lf = lu.d_level_fronts + lu.level_start[h];
    const int nfn = hn >= 0 ? lu.level_start[hn + 1] - lu.level_start[hn] : 0;
    const int* lfn = hn >= 0 ? lu.d_level_fronts + lu.level_start[hn] : nullptr;
    const int rows = std::max(up ? P.level_maxnf[h] : P.level_maxF[h], hn >= 0 ? P.level_maxF[hn] : 0);
    if (rows <= 0 || nfr + nfn <= 0) return;
    cudaEvent_t ev = kt ? kt->start(s) : nullptr;
    const dim3 grid((rows + NT - 1) / NT, nfr + nfn);
    if (up)
        k_bwd_link<<<grid, NT, 0, s>>>(lu.d_fronts, lf, nfr, lfn, h, stage_bufs(lu), lu.d_vars, lu.d_owner, W, red, WP);
    else
        k_fwd_link<<<grid, NT, 0, s>>>(lu.d_fronts, lf, nfr, lfn, h, stage_bufs(lu), lu.d_child_of, lu.d_einv, lu.d_piv,
                                       red, W, WP, B);
    IEMIC_COUNT_LAUNCH();
    if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_OTHER, 0.0, 0.0);
}
template <int ST>
static void launch_reduce(NdLu& lu, int h, double* W, double* WP, double* red, cudaStream_t s) {
    const NdPlan& P = *lu.plan;
    const int nfr = lu.level_start[h + 1] - lu.level_start[h];
    const int* lf = lu.d_level_fronts + lu.level_start[h];
    const int rows = ST == ST_L21 ? P.level_maxF[h] : P.level_maxnf[h];
    if (rows <= 0) return;
    KTimer* kt = lu.timer;
    cudaEvent_t ev = kt ? kt->start(s) : nullptr;
    k_stage_reduce<ST><<<dim3((rows + NT - 1) / NT, nfr), NT, 0, s>>>(lu.d_fronts, lf, stage_bufs(lu), W, WP, red); IEMIC_COUNT_LAUNCH();
    if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_OTHER, 0.0, 0.0);
}
// the sub-steps of the block substitution of level h (UP: backward sweep)
template <class T, bool UP>
static void sub_steps(NdLu& lu, int h, const T* factor, double* W, double* WP, double* red, cudaStream_t s) {
    const auto& is = lu.sub_item_start[UP][h];
    const auto& ds = lu.sub_diag_start[UP][h];
    KTimer* kt = lu.timer;
    for (size_t k = 0; k + 1 < is.size(); ++k) {
        cudaEvent_t ev = kt ? kt->start(s) : nullptr;
        const int ni = is[k + 1] - is[k], nd = ds[k + 1] - ds[k];
        if (ni > 0) {
            k_sub_gemv<T, UP><<<ni, GR, 0, s>>>(lu.d_fronts, static_cast<const WorkItem*>(lu.d_sub_items[UP]) + is[k],
                                                factor, W, lu.d_sub_part); IEMIC_COUNT_LAUNCH();
        }
        if (nd > 0) {
            k_sub_diag<T, UP><<<nd, SDT, 0, s>>>(lu.d_fronts, static_cast<const SubDiag*>(lu.d_sub_diag[UP]) + ds[k],
                                                 factor, lu.d_sub_part, W, WP, red); IEMIC_COUNT_LAUNCH();
        }
        const double by = lu.sub_bytes[UP][h][k];
        if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_GEMV, by, 2.0 * by / sizeof(T));
    }
}

// The forward and backward sweeps over the levels: internal buffers only
// (red -> red), so they can be captured once into a CUDA graph. Modes:
// 0: L11 / U11 applied by block substitution (plans with large fronts);
// 1: their whole inverses as GEMVs (such a plan after a transposed solve);
// 2: whole inverses and the product store: per level and sweep one GEMV
//    launch, whose two stages read the same gathered vector, and one epilogue
//      forward:  [y ; u_B] = [Linv11 ; -(L21 Linv11)] P w_own  (+ [0 ; w_B])
//      backward: x_own = Uinv11 y - (Uinv11 U12) x_B
template <class T, int B>
static void sweeps_t(NdLu& lu, int mode, cudaStream_t s) {
    const bool full = mode >= 1, prod = mode == 2;
    const NdPlan& P = *lu.plan;
    double* red = static_cast<double*>(lu.d_red);
    double* W = static_cast<double*>(lu.d_w);
    double* WP = static_cast<double*>(lu.d_wp);
    const T* front = static_cast<const T*>(lu.d_factor);
    KTimer* kt = lu.timer;
    const int top = P.nlevels - 1;
    for (int h = 0; h < P.nlevels; ++h) {
        const int nfr = lu.level_start[h + 1] - lu.level_start[h];
        const int* lf = lu.d_level_fronts + lu.level_start[h];
        if (!prod || h == 0) {
            cudaEvent_t ev = kt ? kt->start(s) : nullptr;
            k_fwd_gather<<<dim3((P.level_maxF[h] + NT - 1) / NT, nfr), NT, 0, s>>>(lu.d_fronts, lf, lu.d_child_of,
                                                                                lu.d_einv, lu.d_piv, red, W, WP, B); IEMIC_COUNT_LAUNCH();
            if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_OTHER, 0.0, 0.0);
        }
        if (prod) {   // both stages in one launch, then the link to the next level
            launch_mgemv<T>(lu, 0, h, WP, s);
            launch_link(lu, false, h, h < top ? h + 1 : -1, W, WP, red, B, s);
            continue;
        }
        if (full) {
            launch_group<T>(lu, 0, h, front, WP, s);
            launch_reduce<ST_LINV>(lu, h, W, WP, red, s);
        } else {
            sub_steps<T, false>(lu, h, front, W, WP, red, s);
        }
        launch_group<T>(lu, 1, h, front, WP, s);
        launch_reduce<ST_L21>(lu, h, W, WP, red, s);
    }
    for (int h = P.nlevels - 1; h >= 0; --h) {
        const int nfr = lu.level_start[h + 1] - lu.level_start[h];
        const int* lf = lu.d_level_fronts + lu.level_start[h];
        if (!prod || h == top) {
            cudaEvent_t ev = kt ? kt->start(s) : nullptr;
            k_bwd_gather<<<dim3((P.level_maxF[h] + NT - 1) / NT, nfr), NT, 0, s>>>(lu.d_fronts, lf, lu.d_vars, W, red, WP); IEMIC_COUNT_LAUNCH();
            if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_OTHER, 0.0, 0.0);
        }
        if (prod) {   // both stages in one launch, then the link to the next level
            launch_mgemv<T>(lu, 1, h, WP, s);
            launch_link(lu, true, h, h > 0 ? h - 1 : -1, W, WP, red, B, s);
            continue;
        }
        launch_group<T>(lu, 2, h, front, WP, s);
        launch_reduce<ST_U12>(lu, h, W, WP, red, s);
        if (full) {
            launch_group<T>(lu, 3, h, front, WP, s);
            launch_reduce<ST_UINV>(lu, h, W, WP, red, s);
        } else {
            sub_steps<T, true>(lu, h, front, W, WP, red, s);
        }
    }
}

template <class T, int B, class TV>
static void apply_t(NdLu& lu, const int* rp, const int* ci, const double* val, const TV* r, TV* z, cudaStream_t s) {
    const NdPlan& P = *lu.plan;
    double* red = static_cast<double*>(lu.d_red);
    KTimer* kt = lu.timer;
    {
        cudaEvent_t ev = kt ? kt->start(s) : nullptr;
        k_reduce_rhs<TV><<<blocks_for(P.nred), NT, 0, s>>>(P.nred, lu.d_r2g, lu.d_dry_ptr, lu.d_dry_e, lu.d_dry_c, val,
                                                            lu.d_dr, r, red); IEMIC_COUNT_LAUNCH();
        if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_OTHER, 0.0, 0.0);
    }
    const int fm = lu.products ? 2 : lu.full_inverse ? 1 : 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    ck(cudaStreamIsCapturing(s, &cap));
    if (cap == cudaStreamCaptureStatusActive) {
        // captured into the caller's graph (the device-driven GMRES cycle):
        // the sweep kernels themselves, not a launch of the sweep graph
        sweeps_t<T, B>(lu, fm, s);
    } else if (kt && kt->on) {
        timed_graph(lu, lu.sweep_exec_timed[fm], lu.sweep_tmpl[fm], lu.sweep_launches_timed[fm], s,
                    [&] { sweeps_t<T, B>(lu, fm, s); });
    } else {
        if (!lu.sweep_exec[fm]) {
            const long long n0 = launch_counter();
            cudaGraph_t g = capture_graph(s, [&] { sweeps_t<T, B>(lu, fm, s); });
            lu.sweep_launches[fm] = launch_counter() - n0;
            launch_counter() = n0;
            const cudaError_t e = cudaGraphInstantiate(&lu.sweep_exec[fm], g, 0);
            cudaGraphDestroy(g);
            ck(e);
        }
        ck(cudaGraphLaunch(lu.sweep_exec[fm], s));
        launch_counter() += lu.sweep_launches[fm];
    }
    {
        cudaEvent_t ev = kt ? kt->start(s) : nullptr;
        k_expand<TV><<<blocks_for(P.ndim), NT, 0, s>>>(P.ndim, lu.d_g2r, lu.d_isdry, lu.d_dc, red, r, z); IEMIC_COUNT_LAUNCH();
        if (ev) kt->stop(ev, s, IEMIC_KC_SOLVE_OTHER, 0.0, 0.0);
    }
    ck(cudaGetLastError());
}

static TStageBufs tstage_bufs(NdLu& lu) {
    TStageBufs sb;
    for (int st = 0; st < 4; ++st) {
        sb.part[st] = lu.d_tstage_part[st];
        sb.off[st] = lu.d_tstage_off[st];
    }
    return sb;
}
template <class T>
static void launch_tgroup(NdLu& lu, int g, int h, const T* front, double* WP, cudaStream_t s) {
    const int ni = lu.tgroup_start[g][h + 1] - lu.tgroup_start[g][h];
    if (!ni) return;
    k_tgemv_part<T><<<ni, 256, 0, s>>>(lu.d_fronts, static_cast<const WorkItem*>(lu.d_tgroup_items[g]) +
                                           lu.tgroup_start[g][h], front, WP, tstage_bufs(lu)); IEMIC_COUNT_LAUNCH();
}
template <class T, int B, class TV>
static void apply_transpose_t(NdLu& lu, const TV* r, TV* z, cudaStream_t s) {
    const NdPlan& P = *lu.plan;
    double* red = static_cast<double*>(lu.d_red);
    double* W = static_cast<double*>(lu.d_w);
    double* WP = static_cast<double*>(lu.d_wp);
    to_full_inverse<T>(lu, s);
    const T* front = static_cast<const T*>(lu.d_factor);
    const TStageBufs sb = tstage_bufs(lu);
    k_treduce_rhs<TV><<<blocks_for(P.nred), NT, 0, s>>>(P.nred, lu.d_r2g, lu.d_dc, r, red); IEMIC_COUNT_LAUNCH();
    for (int h = 0; h < P.nlevels; ++h) {
        const int nfr = lu.level_start[h + 1] - lu.level_start[h];
        const int* lf = lu.d_level_fronts + lu.level_start[h];
        const dim3 gF((P.level_maxF[h] + NT - 1) / NT, nfr);
        k_tfwd_gather<<<gF, NT, 0, s>>>(lu.d_fronts, lf, lu.d_child_of, lu.d_einv, red, W, WP); IEMIC_COUNT_LAUNCH();
        launch_tgroup<T>(lu, 0, h, front, WP, s);   // v = UINV^T c
        k_tfwd_reduce<0><<<gF, NT, 0, s>>>(lu.d_fronts, lf, sb, W, WP); IEMIC_COUNT_LAUNCH();
        launch_tgroup<T>(lu, 1, h, front, WP, s);   // -U12^T v
        k_tfwd_reduce<1><<<gF, NT, 0, s>>>(lu.d_fronts, lf, sb, W, WP); IEMIC_COUNT_LAUNCH();
    }
    for (int h = P.nlevels - 1; h >= 0; --h) {
        const int nfr = lu.level_start[h + 1] - lu.level_start[h];
        const int* lf = lu.d_level_fronts + lu.level_start[h];
        const dim3 gF((P.level_maxF[h] + NT - 1) / NT, nfr), gN((P.level_maxnf[h] + NT - 1) / NT, nfr);
        k_tbwd_gather<<<gF, NT, 0, s>>>(lu.d_fronts, lf, lu.d_vars, W, red, WP); IEMIC_COUNT_LAUNCH();
        launch_tgroup<T>(lu, 2, h, front, WP, s);   // -L21^T y_B
        k_tbwd_reduce<0><<<gN, NT, 0, s>>>(lu.d_fronts, lf, sb, lu.d_piv, WP, red, B); IEMIC_COUNT_LAUNCH();
        launch_tgroup<T>(lu, 3, h, front, WP, s);   // LINV^T t
        k_tbwd_reduce<1><<<gN, NT, 0, s>>>(lu.d_fronts, lf, sb, lu.d_piv, WP, red, B); IEMIC_COUNT_LAUNCH();
    }
    k_texpand<TV><<<blocks_for(P.ndim), NT, 0, s>>>(P.ndim, lu.d_g2r, lu.d_isdry, lu.d_dr, red, r, z); IEMIC_COUNT_LAUNCH();
    ck(cudaGetLastError());
}

void ndlu_apply_transpose(NdLu& lu, const double* r, double* z, cudaStream_t s) {
    if (!lu.factored) throw EngineError(IEMIC_ERR_STATE);
    if (lu.prec) apply_transpose_t<float, 32, double>(lu, r, z, s);
    else apply_transpose_t<double, 32, double>(lu, r, z, s);
}

void ndlu_apply(NdLu& lu, const int* rp, const int* ci, const double* values, const void* r, void* z, int vec_fp32,
                cudaStream_t s) {
    if (!lu.factored) throw EngineError(IEMIC_ERR_STATE);
    if (lu.prec) {
        if (vec_fp32)
            apply_t<float, 32, float>(lu, rp, ci, values, static_cast<const float*>(r), static_cast<float*>(z), s);
        else
            apply_t<float, 32, double>(lu, rp, ci, values, static_cast<const double*>(r), static_cast<double*>(z), s);
    } else {
        if (vec_fp32)
            apply_t<double, 32, float>(lu, rp, ci, values, static_cast<const float*>(r), static_cast<float*>(z), s);
        else
            apply_t<double, 32, double>(lu, rp, ci, values, static_cast<const double*>(r), static_cast<double*>(z), s);
    }
}

}  // namespace iemic
