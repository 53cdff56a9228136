// C ABI of the linear-solve path (Ocean::solve / applyPrecon /
// buildPreconditioner, src/ocean/Ocean.C:1070-1147, 1377-1404).
#include "engine.cuh"
#include "ndlu.cuh"

using namespace iemic;


#define GUARD_BEGIN try {
#define GUARD_END                                            \
    }                                                        \
    catch (const EngineError& err) { return err.code; }      \
    catch (...) { return IEMIC_ERR_CUDA; }                   \
    return IEMIC_OK;

namespace iemic {
long long& launch_counter() {
    static long long count = 0;
    return count;
}
}  // namespace iemic

extern "C" {

long long iemic_launch_count(void) { return iemic::launch_counter(); }

void iemic_default_solve_opts(iemic_solve_opts* o) {
    if (!o) return;
    o->precision = IEMIC_PREC_MIXED;
    o->restart = 100;          // Belos "Num Blocks" (FGMRES iterations)
    o->max_iters = 1000;
    o->tol = 1e-8;
    o->transpose = 0;
    o->reuse_preconditioner = 0;
}

int iemic_solver_gauge(iemic_ocean* h, int* idx, int capacity, int* count) {
    if (!h || !count || capacity < 0 || (capacity > 0 && !idx)) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    h->e.ensure_solver();
    const std::vector<int>& pins = h->e.ndplan->pins;
    *count = int(pins.size());
    if (capacity < int(pins.size())) return capacity == 0 ? IEMIC_OK : IEMIC_ERR_ARG;
    for (size_t q = 0; q < pins.size(); ++q) idx[q] = pins[q];
    GUARD_END
}

int iemic_build_preconditioner(iemic_ocean* h, int precision) {
    if (!h || precision < -1 || precision > 1) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    if (!h->e.jac_valid) return IEMIC_ERR_STATE;
    if (precision == -1 || precision == IEMIC_PREC_FP64) h->e.build_preconditioner(IEMIC_PREC_FP64);
    if (precision == -1 || precision == IEMIC_PREC_MIXED) h->e.build_preconditioner(IEMIC_PREC_MIXED);
    ck(cudaStreamSynchronize(h->e.stream));
    GUARD_END
}

int iemic_apply_precon(iemic_ocean* h, int precision, const double* v, double* out) {
    if (!h || !v || !out || precision < 0 || precision > 1) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    Engine& e = h->e;
    ck(cudaMemcpyAsync(e.d_v1, v, sizeof(double) * e.ndim, cudaMemcpyHostToDevice, e.stream));
    e.apply_precon(precision, e.d_v1, e.d_v2);
    ck(cudaMemcpyAsync(out, e.d_v2, sizeof(double) * e.ndim, cudaMemcpyDeviceToHost, e.stream));
    ck(cudaStreamSynchronize(e.stream));
    GUARD_END
}

int iemic_solve_dev(iemic_ocean* h, const double* b, double* x, const iemic_solve_opts* o, iemic_solve_stats* st) {
    if (!h || !b || !x) return IEMIC_ERR_ARG;
    iemic_solve_opts oo;
    iemic_default_solve_opts(&oo);
    if (o) oo = *o;
    if (oo.restart < 1 || oo.restart > 1000 || oo.max_iters < 1 || !(oo.tol > 0)) return IEMIC_ERR_ARG;
    if (oo.precision < 0 || oo.precision > 1) return IEMIC_ERR_ARG;
    iemic_solve_stats s{};
    int rc;
    try {
        rc = h->e.solve_dev(b, x, oo, s);
        ck(cudaStreamSynchronize(h->e.stream));
    } catch (const EngineError& err) {
        rc = err.code;
    } catch (...) {
        rc = IEMIC_ERR_CUDA;
    }
    if (st) *st = s;
    return rc;
}

int iemic_solve(iemic_ocean* h, const double* b, double* x, const iemic_solve_opts* o, iemic_solve_stats* st) {
    if (!h || !b || !x) return IEMIC_ERR_ARG;
    Engine& e = h->e;
    try {
        ck(cudaMemcpyAsync(e.d_v1, b, sizeof(double) * e.ndim, cudaMemcpyHostToDevice, e.stream));
    } catch (...) {
        return IEMIC_ERR_CUDA;
    }
    int rc = iemic_solve_dev(h, e.d_v1, e.d_v2, o, st);
    try {
        ck(cudaMemcpyAsync(x, e.d_v2, sizeof(double) * e.ndim, cudaMemcpyDeviceToHost, e.stream));
        ck(cudaStreamSynchronize(e.stream));
    } catch (...) {
        return IEMIC_ERR_CUDA;
    }
    return rc;
}

int iemic_get_solver_info(iemic_ocean* h, iemic_solver_info* out) {
    if (!h || !out) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    h->e.ensure_solver();
    const NdPlan& P = *h->e.ndplan;
    out->unknowns = P.ndim;
    out->reduced_unknowns = P.nred;
    out->fronts = P.nfronts;
    out->levels = P.nlevels;
    out->factor_entries = P.factor_entries;
    out->front_entries = P.front_entries;
    out->factor_flops = P.flops;
    out->work_entries = P.work_entries;
    out->contrib_entries = int64_t(P.contrib_ring) * P.contrib_slot_entries;
    GUARD_END
}

int iemic_set_substitution_threshold(iemic_ocean* h, int max_inverse_nf) {
    if (!h || max_inverse_nf < 0) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    if (max_inverse_nf != h->e.subst_min_nf) {
        ck(cudaStreamSynchronize(h->e.stream));
        h->e.drop_factors();
        h->e.subst_min_nf = max_inverse_nf;
    }
    GUARD_END
}

int iemic_get_fronts(iemic_ocean* h, int cap, int* nf, int* nb, int* level, int* parent, int* count) {
    if (!h || !count || cap < 0 || (cap > 0 && (!nf || !nb || !level || !parent))) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    h->e.ensure_solver();
    const NdPlan& P = *h->e.ndplan;
    for (int lv = 0; lv < P.nlevels; ++lv)
        for (int f : P.level_fronts[lv]) {
            if (f >= cap) continue;
            nf[f] = P.fronts[f].nf;
            nb[f] = P.fronts[f].nb;
            level[f] = lv;
            parent[f] = P.fronts[f].parent;
        }
    *count = P.nfronts;
    GUARD_END
}

int iemic_analyse_pattern(const iemic_config* cfg, const int* landm, const int* row_ptr, const int* col_idx,
                          iemic_solver_info* out) {
    if (!cfg || !landm || !row_ptr || !col_idx || !out || cfg->n < 1 || cfg->m < 1 || cfg->l < 1)
        return IEMIC_ERR_ARG;
    GUARD_BEGIN
    const int64_t ndim = int64_t(6) * cfg->n * cfg->m * cfg->l;
    const int64_t nmask = int64_t(cfg->n + 2) * (cfg->m + 2) * (cfg->l + 2);
    if (ndim > INT32_MAX || row_ptr[0] != 0 || row_ptr[ndim] < 0) return IEMIC_ERR_ARG;
    std::vector<int> lm(landm, landm + nmask), rp(row_ptr, row_ptr + ndim + 1), ci(col_idx, col_idx + row_ptr[ndim]);
    for (int64_t r = 0; r < ndim; ++r)
        if (rp[r + 1] < rp[r]) return IEMIC_ERR_ARG;
    for (int c : ci)
        if (c < 0 || c >= ndim) return IEMIC_ERR_ARG;
    NdPlan P;
    build_nd_plan(P, cfg->n, cfg->m, cfg->l, cfg->periodic ? 1 : 0, lm, rp, ci, 32);   // checks the plan
    out->unknowns = P.ndim;
    out->reduced_unknowns = P.nred;
    out->fronts = P.nfronts;
    out->levels = P.nlevels;
    out->factor_entries = P.factor_entries;
    out->front_entries = P.front_entries;
    out->factor_flops = P.flops;
    out->work_entries = P.work_entries;
    out->contrib_entries = int64_t(P.contrib_ring) * P.contrib_slot_entries;
    GUARD_END
}

int iemic_kernel_timing(iemic_ocean* h, int enable) {
    if (!h) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    ck(cudaStreamSynchronize(h->e.stream));
    h->e.timer.drain();
    if (enable) h->e.timer.reset();
    h->e.timer.on = enable != 0;
    GUARD_END
}

int iemic_kernel_stats_get(iemic_ocean* h, int kclass, iemic_kernel_stats* out) {
    if (!h || !out || kclass < 0 || kclass >= IEMIC_KC_COUNT) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    ck(cudaStreamSynchronize(h->e.stream));
    KTimer& t = h->e.timer;
    t.drain();
    out->launches = t.launches[kclass];
    out->ms = t.ms[kclass];
    out->bytes = t.bytes[kclass];
    out->flops = t.flops[kclass];
    GUARD_END
}

long long iemic_kernel_timing_failures(iemic_ocean* h) { return h ? h->e.timer.failed : -1; }

int iemic_kernel_trace(iemic_ocean* h, int cap, int* kclass, float* ms, double* bytes, int* count) {
    if (!h || !count || cap < 0 || (cap > 0 && (!kclass || !ms || !bytes))) return IEMIC_ERR_ARG;
    GUARD_BEGIN
    ck(cudaStreamSynchronize(h->e.stream));
    h->e.timer.drain();
    const auto& tr = h->e.timer.trace;
    const int n = static_cast<int>(tr.size());
    for (int i = 0; i < n && i < cap; ++i) {
        kclass[i] = tr[i].cls;
        ms[i] = tr[i].ms;
        bytes[i] = tr[i].bytes;
    }
    *count = n;
    GUARD_END
}

int iemic_get_stream(iemic_ocean* h, void** stream) {
    if (!h || !stream) return IEMIC_ERR_ARG;
    *stream = static_cast<void*>(h->e.stream);
    return IEMIC_OK;
}

}  // extern "C"
