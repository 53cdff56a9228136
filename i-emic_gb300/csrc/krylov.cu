// Sparse matrix-vector products on the maximal-graph CSR (FP64 and FP32).
//
// Rows hold 7..24 entries, so four lanes share a row: each lane walks every
// fourth entry and the partial sums are reduced with warp shuffles. A warp
// covers eight consecutive rows, so its loads of col_idx/values are
// contiguous. The state vector is at most a few tens of MB and stays resident
// in the 126 MB L2, so the gathers of x hit L2; DRAM traffic is the matrix.
#include "engine.cuh"

namespace iemic {
namespace {

template <class T>
__global__ void __launch_bounds__(256) spmv_csr4(int nrows, const int* __restrict__ rp, const int* __restrict__ ci,
                                                 const T* __restrict__ v, const T* __restrict__ x, T* __restrict__ y) {
    const int lane = threadIdx.x & 3;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; row < nrows; row += (gridDim.x * blockDim.x) >> 2) {
        const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
        T s = T(0);
        for (int q = b + lane; q < e; q += 4) s += __ldg(v + q) * __ldg(x + __ldg(ci + q));
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (lane == 0) y[row] = s;
    }
}

int spmv_grid(int nrows) {
    long blocks = (long(nrows) * 4 + 255) / 256;
    return int(blocks < 152 * 8 ? blocks : 152 * 8);
}

}  // namespace

void launch_spmv64(int nrows, const int* rp, const int* ci, const double* v, const double* x, double* y, cudaStream_t s) {
    spmv_csr4<double><<<spmv_grid(nrows), 256, 0, s>>>(nrows, rp, ci, v, x, y);
}
void launch_spmv32(int nrows, const int* rp, const int* ci, const float* v, const float* x, float* y, cudaStream_t s) {
    spmv_csr4<float><<<spmv_grid(nrows), 256, 0, s>>>(nrows, rp, ci, v, x, y);
}

void Engine::spmv64(const double* x, double* y) {
    launch_spmv64(ndim, d_rowptr, d_col, d_val, x, y, stream);
    ck(cudaGetLastError());
}
void Engine::spmv32(const float* x, float* y) {
    launch_spmv32(ndim, d_rowptr, d_col, d_val32, x, y, stream);
    ck(cudaGetLastError());
}

void Engine::free_solver() {}
void Engine::ensure_solver() {}
void Engine::build_preconditioner(int) { throw EngineError(IEMIC_ERR_STATE); }
int Engine::solve_dev(const double*, double*, const iemic_solve_opts&, iemic_solve_stats&) { return IEMIC_ERR_STATE; }
void Engine::apply_precon(int, const double*, double*) { throw EngineError(IEMIC_ERR_STATE); }

}  // namespace iemic
