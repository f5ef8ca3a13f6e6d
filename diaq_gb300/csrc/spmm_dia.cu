// C = A B with A in the row-aligned DIA format and B, C dense, all arrays already on the device:
// the reference's spmm_dia_device (src/spMM_device_gpu.cu:44-127, bound at
// include/pythonWrappers.cpp:622-633).
//
// Format: offsets int64[n_diags]; vals[k * n_rows + r] = A[r, r + offsets[k]] (entries whose
// column falls outside [0, n_cols) are ignored); B is n_cols x n_right and C n_rows x n_right,
// both row-major; float64 or interleaved complex128.  C is overwritten; diagonals are summed in
// the order given (duplicates add).
//
// Work split: thread e computes C's element e = r * n_right + j, so a warp's stores to C and its
// loads of B (at e + offset * n_right) are contiguous whatever n_right is, and the lanes of one
// row share the diagonal value (an L1 broadcast).  Offsets are staged in shared memory in chunks;
// the diagonal loop is unrolled by 4 with predicated loads, so four diagonals' loads are in flight
// per thread.  A grid-stride loop covers any size with a grid of a few waves of the SMs.
#include <algorithm>

#include "diaq_internal.cuh"

namespace diaq_gb300 {

namespace {

constexpr int kSpmmThreads = 256;
constexpr int kOffChunk = 1024;
constexpr int kUnroll = 4;

struct Real {
    using V = double;
    static __device__ __forceinline__ V zero() { return 0.0; }
    static __device__ __forceinline__ V mac(V acc, V a, V b) { return fma(a, b, acc); }
};

struct Cplx {
    using V = double2;
    static __device__ __forceinline__ V zero() { return make_double2(0.0, 0.0); }
    static __device__ __forceinline__ V mac(V acc, V a, V b) {
        acc.x = fma(-a.y, b.y, fma(a.x, b.x, acc.x));
        acc.y = fma(a.y, b.x, fma(a.x, b.y, acc.y));
        return acc;
    }
};

template <class T>
__global__ void __launch_bounds__(kSpmmThreads)
    spmm_dia_kernel(const int64_t *__restrict__ offsets, int nd, const typename T::V *__restrict__ vals,
                    int64_t M, int64_t K, const typename T::V *__restrict__ B, int64_t R,
                    typename T::V *__restrict__ C) {
    using V = typename T::V;
    __shared__ int64_t so[kOffChunk];
    const int64_t total = M * R;
    const int64_t stride = (int64_t)gridDim.x * kSpmmThreads;
    // every thread runs the same number of outer iterations, so the block can sync inside
    const int64_t iters = (total + stride - 1) / stride;
    for (int64_t it = 0; it < iters; ++it) {
        const int64_t e = it * stride + (int64_t)blockIdx.x * kSpmmThreads + threadIdx.x;
        const bool live = e < total;
        const int64_t r = live ? e / R : 0;
        V acc = T::zero();
        for (int c0 = 0; c0 < nd; c0 += kOffChunk) {
            const int cn = min(kOffChunk, nd - c0);
            __syncthreads();
            for (int i = threadIdx.x; i < cn; i += kSpmmThreads) so[i] = offsets[c0 + i];
            __syncthreads();
            if (!live) continue;
            int k = 0;
            for (; k + kUnroll <= cn; k += kUnroll) {
                V a[kUnroll], b[kUnroll];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) {
                    const int64_t c = r + so[k + u];
                    const bool ok = c >= 0 && c < K;
                    a[u] = ok ? vals[(int64_t)(c0 + k + u) * M + r] : T::zero();
                    b[u] = ok ? __ldg(B + e + so[k + u] * R) : T::zero();
                }
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) acc = T::mac(acc, a[u], b[u]);
            }
            for (; k < cn; ++k) {
                const int64_t c = r + so[k];
                if (c >= 0 && c < K) acc = T::mac(acc, vals[(int64_t)(c0 + k) * M + r], __ldg(B + e + so[k] * R));
            }
        }
        if (live) C[e] = acc;
    }
}

}  // namespace

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" int diaq_spmm_dia_device(const int64_t *offsets, const void *vals, int n_diags, int64_t n_rows,
                                    int64_t n_cols, const void *B, int64_t n_right, void *C, int is_complex,
                                    void *stream) {
    if (n_diags < 0 || n_rows < 0 || n_cols < 0 || n_right < 0)
        return set_error(DIAQ_ERR_INVALID, "spmm_dia_device: sizes must be non-negative");
    if (n_rows == 0 || n_right == 0) return DIAQ_OK;
    if (!C || (n_diags > 0 && (!offsets || !vals || (n_cols > 0 && !B))))
        return set_error(DIAQ_ERR_INVALID, "spmm_dia_device: NULL array");
    const int64_t total = n_rows * n_right;
    const int64_t want = (total + kSpmmThreads - 1) / kSpmmThreads;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, 16 * (int64_t)num_sms()));
    const cudaStream_t s = (cudaStream_t)stream;
    if (is_complex)
        spmm_dia_kernel<Cplx><<<grid, kSpmmThreads, 0, s>>>(offsets, n_diags, (const double2 *)vals, n_rows, n_cols,
                                                            (const double2 *)B, n_right, (double2 *)C);
    else
        spmm_dia_kernel<Real><<<grid, kSpmmThreads, 0, s>>>(offsets, n_diags, (const double *)vals, n_rows, n_cols,
                                                           (const double *)B, n_right, (double *)C);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}
