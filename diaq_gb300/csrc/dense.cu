// Dense <-> DiaQ on the device: the conversions either side of the path, which the reference runs
// on the host (from_numpy: src/dense_to_diagonals.hpp:20-58 via include/pythonWrappers.cpp:146-193;
// to_numpy and the device matrix's host staging: src/deviceMatrix_gpu.cu:62-113).
//
// from_dense: pass 1 flags every diagonal holding a value other than exact zero (one thread per
// element, row-major and coalesced; a flag is only ever set to 1, so racing writes agree); the
// host turns the flags into the ascending offset list, lays the matrix out, and pass 2 gathers
// each stored diagonal's values into the row-phase aligned arrays.  Dense input is interleaved
// complex128, row-major (numpy / torch complex128), on the device or the host.
// to_dense: zero the output, then scatter every stored value to (r, r + d).
#include <algorithm>
#include <vector>

#include "diaq_internal.cuh"

namespace diaq_gb300 {

namespace {

__global__ void dense_flags_kernel(const double2 *__restrict__ a, int64_t rows, int64_t cols, int *__restrict__ flags) {
    const int64_t n = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = a[e];
        if (v.x != 0.0 || v.y != 0.0) {
            const int64_t r = e / cols, c = e - r * cols;
            flags[c - r + rows - 1] = 1;
        }
    }
}

template <typename T>
__global__ void dense_gather_kernel(const DiagMeta *__restrict__ meta, int nd, const double2 *__restrict__ a,
                                    int64_t cols, T *__restrict__ re, T *__restrict__ im) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        for (int64_t r = m.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m.hi;
             r += (int64_t)gridDim.x * blockDim.x) {
            const double2 v = a[r * cols + r + m.off];
            re[m.base + r] = (T)v.x;
            im[m.base + r] = (T)v.y;
        }
    }
}

template <typename T>
__global__ void dense_scatter_kernel(const DiagMeta *__restrict__ meta, int nd, const T *__restrict__ re,
                                     const T *__restrict__ im, int64_t cols, double2 *__restrict__ a) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        for (int64_t r = m.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m.hi;
             r += (int64_t)gridDim.x * blockDim.x)
            a[r * cols + r + m.off] = make_double2((double)re[m.base + r], (double)im[m.base + r]);
    }
}

dim3 diag_grid(const Matrix &M) {
    int64_t maxlen = 1;
    for (const auto &m : M.meta) maxlen = std::max(maxlen, m.hi - m.lo);
    return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>((maxlen + 255) / 256, 4 * num_sms())),
                (unsigned)std::min<int64_t>(std::max<int32_t>(M.nd, 1), 65535));
}

// A device buffer freed on every exit path.
struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace

int from_dense(int64_t rows, int64_t cols, const double *dense, bool on_device, int prec, cudaStream_t s,
               Matrix **out) {
    if (rows < 0 || cols < 0) return set_error(DIAQ_ERR_INVALID, "from_dense: negative shape");
    if (rows > 0 && cols > 0 && !dense) return set_error(DIAQ_ERR_INVALID, "from_dense: NULL array");
    if (prec != DIAQ_C128 && prec != DIAQ_C64 && prec != DIAQ_C128F2)
        return set_error(DIAQ_ERR_INVALID, "from_dense: unknown precision");
    const int64_t n = rows * cols;
    if (n == 0) return make_zero(rows, cols, 0, nullptr, prec, s, out);
    if (prec == DIAQ_C128F2) {  // float64 first, then split into float pairs
        Matrix *D = nullptr;
        DQ_TRY(from_dense(rows, cols, dense, on_device, DIAQ_C128, s, &D));
        const int st = copy_as(*D, DIAQ_C128F2, s, out);
        cudaStreamSynchronize(s);
        destroy(D);
        return st;
    }
    DevBuf staged, flags;
    const double2 *a = reinterpret_cast<const double2 *>(dense);
    if (!on_device) {
        DQ_CUDA(dev_malloc(&staged.p, sizeof(double2) * (size_t)n));
        DQ_CUDA(cudaMemcpyAsync(staged.p, dense, sizeof(double2) * (size_t)n, cudaMemcpyHostToDevice, s));
        a = static_cast<const double2 *>(staged.p);
    }
    const int64_t ndiag = rows + cols - 1;
    DQ_CUDA(dev_malloc(&flags.p, sizeof(int) * (size_t)ndiag));
    DQ_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int) * (size_t)ndiag, s));
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 16 * num_sms()));
    dense_flags_kernel<<<g, 256, 0, s>>>(a, rows, cols, static_cast<int *>(flags.p));
    DQ_CUDA(cudaGetLastError());
    std::vector<int> hf((size_t)ndiag);
    DQ_CUDA(cudaMemcpyAsync(hf.data(), flags.p, sizeof(int) * (size_t)ndiag, cudaMemcpyDeviceToHost, s));
    DQ_CUDA(cudaStreamSynchronize(s));
    std::vector<int32_t> off;
    for (int64_t i = 0; i < ndiag; ++i)
        if (hf[(size_t)i]) off.push_back((int32_t)(i - (rows - 1)));
    Matrix *M = nullptr;
    DQ_TRY(make_zero(rows, cols, (int32_t)off.size(), off.data(), prec, s, &M));
    if (M->nd > 0) {
        if (prec == DIAQ_C128)
            dense_gather_kernel<double><<<diag_grid(*M), 256, 0, s>>>(M->d_meta, M->nd, a, cols, (double *)M->re,
                                                                    (double *)M->im);
        else
            dense_gather_kernel<float><<<diag_grid(*M), 256, 0, s>>>(M->d_meta, M->nd, a, cols, (float *)M->re,
                                                                   (float *)M->im);
        const cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) cudaStreamSynchronize(s);  // the staged input is freed on return
        if (e != cudaSuccess) {
            destroy(M);
            return cuda_status(e, "from_dense", __FILE__, __LINE__);
        }
    }
    *out = M;
    return DIAQ_OK;
}

int to_dense(const Matrix &A, double *dense, bool on_device, cudaStream_t s) {
    const int64_t n = A.rows * A.cols;
    if (n == 0) return DIAQ_OK;
    if (!dense) return set_error(DIAQ_ERR_INVALID, "to_dense: NULL array");
    if (A.prec == DIAQ_C128F2) {
        Matrix *D = nullptr;
        DQ_TRY(copy_as(A, DIAQ_C128, s, &D));
        const int st = to_dense(*D, dense, on_device, s);
        cudaStreamSynchronize(s);
        destroy(D);
        return st;
    }
    DevBuf staged;
    double2 *a = reinterpret_cast<double2 *>(dense);
    if (!on_device) {
        DQ_CUDA(dev_malloc(&staged.p, sizeof(double2) * (size_t)n));
        a = static_cast<double2 *>(staged.p);
    }
    DQ_CUDA(cudaMemsetAsync(a, 0, sizeof(double2) * (size_t)n, s));
    if (A.nd > 0) {
        if (A.prec == DIAQ_C128)
            dense_scatter_kernel<double><<<diag_grid(A), 256, 0, s>>>(A.d_meta, A.nd, (const double *)A.re,
                                                                    (const double *)A.im, A.cols, a);
        else
            dense_scatter_kernel<float><<<diag_grid(A), 256, 0, s>>>(A.d_meta, A.nd, (const float *)A.re,
                                                                   (const float *)A.im, A.cols, a);
        DQ_CUDA(cudaGetLastError());
    }
    if (!on_device) {
        DQ_CUDA(cudaMemcpyAsync(dense, a, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost, s));
        DQ_CUDA(cudaStreamSynchronize(s));
    }
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_matrix_from_dense(int64_t rows, int64_t cols, const double *dense, int on_device, int precision,
                           void *stream, diaq_matrix_t *out) {
    if (!out) return set_error(DIAQ_ERR_INVALID, "NULL output handle");
    Matrix *M = nullptr;
    DQ_TRY(from_dense(rows, cols, dense, on_device != 0, precision, (cudaStream_t)stream, &M));
    *out = handle(M);
    return DIAQ_OK;
}

int diaq_matrix_to_dense(diaq_matrix_t A, double *dense, int on_device, void *stream) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    return to_dense(*A, dense, on_device != 0, (cudaStream_t)stream);
}

}  // extern "C"
