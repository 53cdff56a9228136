// Nested-dissection multilevel block LU of the THCM Jacobian (preconditioner).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "ktimer.cuh"

namespace iemic {

// One frontal matrix of the elimination tree: `nf` own ("fully summed")
// unknowns followed by `nb` boundary unknowns owned by ancestors.
struct FrontDev {
    int nf, nb, F;          // F = nf + nb, leading dimension of the dense front
    int parent;             // -1 at the root
    int red0;               // reduced index of the first own unknown
    int lvl;                // level (height in the elimination tree)
    int64_t off;            // offset of the column-major F x F front in the working area of its level
    int64_t foff;           // offset in the factor store: F x nf (ld F), then the nf x nb block (ld nf)
    int64_t soff;           // offset of its nb x nb contribution block (ld nb) in the contribution ring
    int64_t voff;           // offset into `vars` (F reduced indices)
    int64_t dinv_off;       // offset of the per-panel inverse diagonal blocks
    int64_t emap_off;       // offset into `emap` (nb parent-local indices)
    int64_t woff;           // offset of the front's solve vector (F entries)
};

// Host-side symbolic analysis, built once per land mask.
struct NdPlan {
    int ndim = 0, nred = 0, nfronts = 0, nlevels = 0, panel = 32;
    std::vector<FrontDev> fronts;
    std::vector<std::vector<int>> level_fronts;   // fronts by height (leaves first)
    std::vector<int> level_maxnf, level_maxF;
    std::vector<std::vector<int>> level_children[2];   // per level, children in slot s of its fronts
    std::vector<int> r2g, g2r;      // reduced <-> global unknown
    std::vector<int> vars;          // per front: reduced indices of its F unknowns
    std::vector<int> emap;          // per front: parent-local index of its nb boundary unknowns
    std::vector<int> child_slot;    // slot of each front in its parent
    std::vector<int> dry_rows;      // unknowns the factorisation leaves out (identity rows, pins)
    std::vector<int> pins;          // pinned pressure unknowns
    std::vector<int> dry_ptr, dry_e, dry_c;   // per reduced row: CSR entries (and columns) on identity unknowns
    std::vector<int> asm_src;       // CSR entry index
    std::vector<int> asm_row;       // its row
    std::vector<int64_t> asm_dst;   // offset in the front storage
    int64_t front_entries = 0, dinv_entries = 0, emap_entries = 0, w_entries = 0;
    // storage: one working area sized for the largest level (its F x F
    // fronts), the factor store, and a ring of `contrib_ring` slots of
    // contribution blocks (a level's blocks live in slot level % ring until
    // every parent has added them)
    int64_t work_entries = 0, contrib_slot_entries = 0;
    int contrib_ring = 1;
    std::vector<int64_t> level_work;      // per level: its working entries
    std::vector<int64_t> asm_level_start; // per level: range of its assembly entries
    double flops = 0.0;             // factorisation flop count
    int64_t factor_entries = 0;     // entries the solve phase reads
};

// consistency of a plan's offsets and indices (throws IEMIC_ERR_STATE)
void check_nd_plan(const NdPlan& plan);
void build_nd_plan(NdPlan& plan, int n, int m, int l, int periodic, const std::vector<int>& landm,
                   const std::vector<int>& row_ptr, const std::vector<int>& col_idx, int panel,
                   const std::vector<int>& identity_rows = {}, const std::vector<int>& fixed_pressures = {});

// Device-resident factorisation for one precision.
struct NdLu {
    int prec = 0;   // 0 FP64, 1 FP32
    const NdPlan* plan = nullptr;
    KTimer* timer = nullptr;                // optional launch timing (owned by the engine)
    // device copies of the plan
    FrontDev* d_fronts = nullptr;
    int* d_level_fronts = nullptr;          // concatenated per level
    std::vector<int> level_start;           // offsets into d_level_fronts
    int* d_level_children[2] = {nullptr, nullptr};
    std::vector<int> child_start[2];
    int *d_vars = nullptr, *d_emap = nullptr, *d_r2g = nullptr, *d_g2r = nullptr, *d_child_of = nullptr;
    char* d_isdry = nullptr;                // 1 for unknowns left out of the factorisation
    int *d_dry_ptr = nullptr, *d_dry_e = nullptr, *d_dry_c = nullptr;   // NdPlan::dry_*
    int2* d_einv = nullptr;                 // per solve-vector row: child update rows (slot 0, slot 1) or -1
    int* d_owner = nullptr;                 // per reduced unknown: the front whose own unknown it is
    int* d_asm_src = nullptr;
    int* d_asm_row = nullptr;
    double *d_dr = nullptr, *d_dc = nullptr, *d_cmax = nullptr;   // equilibration scalings
    int64_t* d_asm_dst = nullptr;
    int* d_piv = nullptr;                   // per reduced unknown: block-local pivot source
    void* d_front = nullptr;                // working area: the F x F fronts of one level (T)
    void* d_factor = nullptr;               // factor store read by the solves (T)
    void* d_contrib = nullptr;              // contribution-block ring (T)
    void* d_dinv = nullptr;                 // inverse diagonal panel blocks (T)
    void* d_w = nullptr;                    // solve vectors (T)
    void* d_red = nullptr;                  // reduced rhs / solution (T)
    int* d_npert = nullptr;                 // counters: perturbed pivots, NaN pivot candidates
    void* d_wp = nullptr;                   // permuted / gathered solve vectors (FP64)
    // solve phase: partial-sum buffers and per-front offsets per GEMV stage
    // (Linv11, Uinv11, L21, U12), work items per launch group
    double* d_stage_part[4] = {nullptr, nullptr, nullptr, nullptr};
    int64_t* d_stage_off[4] = {nullptr, nullptr, nullptr, nullptr};
    void* d_group_items[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<int> group_start[4];        // per level offsets into d_group_items
    std::vector<double> group_bytes[4];     // per level: factor bytes the group reads
    // block substitution over the inverted 256-row diagonal super-blocks
    // (forward solves), [0] lower (forward sweep), [1] upper (backward sweep):
    // per level and sub-step the off-diagonal GEMV tiles and the per-front
    // diagonal items; one partial-sum buffer reused by every sub-step
    void* d_sub_items[2] = {nullptr, nullptr};
    void* d_sub_diag[2] = {nullptr, nullptr};
    std::vector<std::vector<int>> sub_item_start[2], sub_diag_start[2];   // [level][sub-step], one past the end
    std::vector<std::vector<double>> sub_bytes[2];                        // factor bytes per sub-step
    double* d_sub_part = nullptr;
    // transposed solve: partial buffers per transposed stage, items per group
    double* d_tstage_part[4] = {nullptr, nullptr, nullptr, nullptr};
    int64_t* d_tstage_off[4] = {nullptr, nullptr, nullptr, nullptr};
    void* d_tgroup_items[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<int> tgroup_start[4];
    // recursive triangular inversion: tasks, tiles, per level the tile ranges
    // of its launches, and the scratch of the first product of each merge
    void *d_tri_tasks = nullptr, *d_tri_tiles = nullptr, *d_tri_scratch = nullptr, *d_tri_groups = nullptr;
    std::vector<std::vector<std::pair<int, int>>> tri_ranges;    // merges (factorisation)
    std::vector<std::vector<std::pair<int, int>>> inv2_ranges;   // whole-block inverses (on demand)
    int64_t inv2_scratch_entries = 0;
    void* d_inv2_scratch = nullptr;
    bool subst = false;                     // solves substitute over super-blocks (large fronts)
    // the whole-inverse steps of a level run on a second stream (forked and
    // joined inside the captured factorisation) while the next level factors
    cudaStream_t side = nullptr;
    std::vector<cudaEvent_t> fork_ev;       // per level
    cudaEvent_t join_ev = nullptr;
    bool full_inverse = false;              // L11 / U11 replaced by their whole inverses
    // whole-inverse plans: the products L21 Linv11 and Uinv11 U12 in a store
    // laid out like the factor store (the same offsets; the nf x nf squares
    // unused), computed with the inverses. The two GEMV stages of a level and
    // sweep then read the same gathered vector and run as one launch with one
    // epilogue (product sweeps)
    void* d_prod = nullptr;
    bool products = false;
    std::vector<std::vector<std::pair<int, int>>> prod_ranges;   // product tasks per level
    void* d_mgroup_items[2] = {nullptr, nullptr};   // [0] Linv11 + L21 Linv11, [1] Uinv11 + Uinv11 U12
    std::vector<int> mgroup_start[2];               // per level offsets
    std::vector<double> mgroup_bytes[2];            // per level: factor bytes the launch reads
    double tri_flops = 0.0;
    cudaGraphExec_t factor_exec = nullptr;  // captured factorisation
    // captured forward + backward level sweeps, [0] block substitution,
    // [1] whole inverses, [2] whole inverses with the products (one GEMV
    // launch per level and sweep)
    cudaGraphExec_t sweep_exec[3] = {nullptr, nullptr, nullptr};
    // the same graphs with timing event nodes (kernel timing on)
    cudaGraphExec_t factor_exec_timed = nullptr, sweep_exec_timed[3] = {nullptr, nullptr, nullptr};
    std::vector<KTimer::Rec> factor_tmpl, sweep_tmpl[3];
    long long factor_launches_timed = 0, sweep_launches_timed[3] = {0, 0, 0};
    long long factor_launches = 0;
    const void *fg_rp = nullptr, *fg_ci = nullptr, *fg_val = nullptr;   // arrays the factor graph reads
    long long sweep_launches[3] = {0, 0, 0};   // kernels in the captured sweeps
    int npert = 0;
    int nnan = 0;
    bool factored = false;
    std::vector<void*> allocs;
    ~NdLu();
};

// subst_min_nf: fronts up to this many own unknowns keep whole inverses of
// L11 / U11; a plan with a larger front substitutes over 256-row super-blocks
void ndlu_setup(NdLu& lu, const NdPlan& plan, int prec, int subst_min_nf);
// values: FP64 CSR values of J (equilibrated in FP64, then cast to the factor precision)
void ndlu_factor(NdLu& lu, const int* row_ptr, const int* col_idx, const double* values, cudaStream_t s);
// z = M^{-1} r on global-indexed vectors (float if vec_fp32, else double);
// `values` are the FP64 CSR values (used for the eliminated columns). The
// triangular solves accumulate in FP64 whatever the factor precision.
void ndlu_apply(NdLu& lu, const int* row_ptr, const int* col_idx, const double* values, const void* r, void* z,
                int vec_fp32, cudaStream_t s);
// z = M^{-T} r with the same factors (FP64 vectors): the transposed
// preconditioner of J^T for adjoint solves.
void ndlu_apply_transpose(NdLu& lu, const double* r, double* z, cudaStream_t s);

}  // namespace iemic
