// Device matrices: layout, allocation, upload/download, copy, precision conversion, prune.
// Replaces deviceDiaQMatrix (src/deviceMatrix_gpu.hpp:37-68, src/deviceMatrix_gpu.cu:30-113)
// and diaQMatrix::pruneMatrix (src/diaQMatrix.hpp:1543-1604).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_set>

#include "diaq_internal.cuh"

namespace diaq_gb300 {

// ---- error state ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

int set_error(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

int cuda_status(cudaError_t e, const char *what, const char *file, int line) {
    const char *base = std::strrchr(file, '/');
    char buf[512];
    std::snprintf(buf, sizeof(buf), "CUDA error: %s (%s:%d) in %s", cudaGetErrorString(e),
                  base ? base + 1 : file, line, what);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // clear the sticky-free allocation error
        return set_error(DIAQ_ERR_OOM, buf);
    }
    return set_error(DIAQ_ERR_CUDA, buf);
}

size_t alloc_limit() {
    const char *v = std::getenv("DIAQ_DEVICE_ALLOC_LIMIT");
    if (!v || !*v) return SIZE_MAX;
    char *end = nullptr;
    const unsigned long long n = std::strtoull(v, &end, 10);
    return (end && *end == '\0') ? (size_t)n : SIZE_MAX;
}

int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// ---- geometry --------------------------------------------------------------------------------
int64_t diag_len(int64_t rows, int64_t cols, int64_t d) {
    // src/diaQMatrix.hpp:390-409 for offsets inside the matrix
    int64_t len;
    if (d < 0) len = rows + d;
    else if (d > 0) len = cols - d;
    else len = rows < cols ? rows : cols;
    if (len > rows) len = rows;
    else if (len > cols) len = cols;
    return len < 0 ? 0 : len;
}

int plan_layout(Matrix &M, int64_t rows, int64_t cols, int32_t nd, const int32_t *off) {
    if (rows < 0 || cols < 0) return set_error(DIAQ_ERR_INVALID, "matrix shape must be non-negative");
    // the kernels keep row indices, offsets and row ranges in 32 bits (the reference's are 32-bit too)
    if (rows >= ((int64_t)1 << 31) || cols >= ((int64_t)1 << 31))
        return set_error(DIAQ_ERR_UNSUPPORTED, "matrix dimensions must be below 2^31");
    if (nd < 0) return set_error(DIAQ_ERR_INVALID, "diagonal count must be non-negative");
    if (nd > 0 && !off) return set_error(DIAQ_ERR_INVALID, "offsets pointer is NULL");
    M.rows = rows;
    M.cols = cols;
    M.nd = nd;
    M.off.assign(off, off + nd);
    M.meta.resize(nd);
    std::unordered_set<int32_t> seen;
    seen.reserve(nd * 2 + 1);
    int64_t cursor = kAlign, pstart = 0;
    for (int32_t k = 0; k < nd; ++k) {
        const int64_t d = off[k];
        if (d <= -rows || d >= cols)
            return set_error(DIAQ_ERR_INVALID, "diagonal offset " + std::to_string(d) +
                                                   " lies outside a " + std::to_string(rows) + " x " +
                                                   std::to_string(cols) + " matrix");
        if (!seen.insert(off[k]).second)
            return set_error(DIAQ_ERR_INVALID, "diagonal offset " + std::to_string(d) + " appears twice");
        const int64_t len = diag_len(rows, cols, d);
        const int64_t lo = d < 0 ? -d : 0;
        const int64_t gap = ((lo - cursor) % kAlign + kAlign) % kAlign;
        const int64_t s = cursor + gap;  // s == lo (mod kAlign)
        DiagMeta &m = M.meta[k];
        m.base = s - lo;
        m.lo = lo;
        m.hi = lo + len;
        m.pstart = pstart;
        m.off = off[k];
        m.slot = k;
        m.pad = 0;
        cursor = s + len;
        pstart += len;
    }
    // a multiple of kAlign, so that a second plane (C128F2) starts aligned as well
    M.capacity = (cursor + 2 * kAlign - 1) / kAlign * kAlign;
    M.total = pstart;
    return DIAQ_OK;
}

int allocate(Matrix &M, cudaStream_t s, bool zero) {
    cudaGetDevice(&M.device);
    const size_t bytes = (size_t)M.capacity * M.elem();
    DQ_CUDA(dev_malloc(&M.re, bytes));
    DQ_CUDA(dev_malloc(&M.im, bytes));
    if (zero) {
        DQ_CUDA(cudaMemsetAsync(M.re, 0, bytes, s));
        DQ_CUDA(cudaMemsetAsync(M.im, 0, bytes, s));
    }
    if (M.nd > 0) {
        // the zero-tile mask's storage, so that SpMV calls never allocate (it is filled on first use)
        DQ_CUDA(dev_malloc(&M.tmask, sizeof(uint32_t) * (size_t)M.nd * (size_t)((M.rows + 1023) / 1024)));
        DQ_CUDA(dev_malloc(&M.d_meta, sizeof(DiagMeta) * M.nd));
        DQ_CUDA(cudaMemcpyAsync(M.d_meta, M.meta.data(), sizeof(DiagMeta) * M.nd,
                                cudaMemcpyHostToDevice, s));
        // the host vector may be reallocated later; finish the copy before returning
        DQ_CUDA(cudaStreamSynchronize(s));
    }
    return DIAQ_OK;
}

void release(Matrix &M) {
    if (M.re) cudaFree(M.re);
    if (M.im) cudaFree(M.im);
    if (M.d_meta) cudaFree(M.d_meta);
    if (M.tmask) cudaFree(M.tmask);
    M.re = M.im = nullptr;
    M.d_meta = nullptr;
    M.tmask = nullptr;
    M.tmask_ok = false;
}

int make_zero(int64_t rows, int64_t cols, int32_t nd, const int32_t *off, int prec,
              cudaStream_t s, Matrix **out, bool zero) {
    if (prec != DIAQ_C128 && prec != DIAQ_C64 && prec != DIAQ_C128F2)
        return set_error(DIAQ_ERR_INVALID, "precision must be DIAQ_C128, DIAQ_C64 or DIAQ_C128F2");
    Matrix *M = new diaq_matrix_s();
    M->prec = prec;
    int st = plan_layout(*M, rows, cols, nd, off);
    if (st == DIAQ_OK) st = allocate(*M, s, zero);
    if (st != DIAQ_OK) {
        destroy(M);
        return st;
    }
    *out = M;
    return DIAQ_OK;
}

// Block j zeroes gap j: [0, start of diagonal 0) for j = 0, [end of j - 1, start of j) between
// diagonals, [end of the last, capacity) for j = nd -- in each of the `planes` planes of
// `capacity` elements of size esz in re and im.
__global__ void zero_gaps_kernel(const DiagMeta *__restrict__ meta, int nd, int64_t capacity, int esz, int planes,
                                 unsigned char *re, unsigned char *im) {
    const int j = blockIdx.x;
    const int64_t a = j == 0 ? 0 : meta[j - 1].base + meta[j - 1].hi;
    const int64_t b = j == nd ? capacity : meta[j].base + meta[j].lo;
    for (int p = 0; p < planes; ++p)
        for (int64_t e = a + threadIdx.x; e < b; e += blockDim.x)
            for (int k = 0; k < esz; ++k) {
                re[(p * capacity + e) * esz + k] = 0;
                im[(p * capacity + e) * esz + k] = 0;
            }
}

int zero_gaps(const Matrix &M, cudaStream_t s) {
    const int planes = M.prec == DIAQ_C128F2 ? 2 : 1;
    const int esz = M.prec == DIAQ_C128 ? 8 : 4;
    zero_gaps_kernel<<<M.nd + 1, 64, 0, s>>>(M.d_meta, M.nd, M.capacity, esz, planes, (unsigned char *)M.re,
                                             (unsigned char *)M.im);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

void destroy(Matrix *M) {
    if (!M) return;
    release(*M);
    delete static_cast<diaq_matrix_s *>(M);
}

// ---- copy kernels ------------------------------------------------------------------------------
// One y-row of the grid per diagonal (strided when there are more diagonals than grid rows),
// x over the diagonal's rows.

template <typename TS, typename TD>
__global__ void scatter_kernel(const DiagMeta *__restrict__ meta, int nd, const TS *__restrict__ sre,
                               const TS *__restrict__ sim, TD *__restrict__ dre,
                               TD *__restrict__ dim) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        const int64_t len = m.hi - m.lo;
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < len;
             j += (int64_t)gridDim.x * blockDim.x) {
            dre[m.base + m.lo + j] = (TD)sre[m.pstart + j];
            dim[m.base + m.lo + j] = (TD)sim[m.pstart + j];
        }
    }
}

template <typename TS>
__global__ void gather_kernel(const DiagMeta *__restrict__ meta, int nd, const TS *__restrict__ sre,
                              const TS *__restrict__ sim, double *__restrict__ dre,
                              double *__restrict__ dim) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        const int64_t len = m.hi - m.lo;
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < len;
             j += (int64_t)gridDim.x * blockDim.x) {
            dre[m.pstart + j] = (double)sre[m.base + m.lo + j];
            dim[m.pstart + j] = (double)sim[m.base + m.lo + j];
        }
    }
}

// dst diagonal k <- src diagonal map[k] (same offset, so same rows), with conversion.
template <typename TS, typename TD>
__global__ void remap_kernel(const DiagMeta *__restrict__ smeta, const TS *__restrict__ sre,
                             const TS *__restrict__ sim, const DiagMeta *__restrict__ dmeta,
                             TD *__restrict__ dre, TD *__restrict__ dim, const int32_t *__restrict__ map,
                             int nd) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta dm = dmeta[k];
        const DiagMeta sm = smeta[map ? map[k] : k];
        for (int64_t r = dm.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < dm.hi;
             r += (int64_t)gridDim.x * blockDim.x) {
            dre[dm.base + r] = (TD)sre[sm.base + r];
            dim[dm.base + r] = (TD)sim[sm.base + r];
        }
    }
}

// Per diagonal: does it hold a value other than exact zero?
template <typename T>
__global__ void nonzero_kernel(const DiagMeta *__restrict__ meta, int nd, const T *__restrict__ re,
                               const T *__restrict__ im, int32_t *__restrict__ flag) {
    for (int k = blockIdx.x; k < nd; k += gridDim.x) {
        const DiagMeta m = meta[k];
        int nz = 0;
        for (int64_t r = m.lo + threadIdx.x; r < m.hi && !nz; r += blockDim.x)
            nz = (re[m.base + r] != (T)0) || (im[m.base + r] != (T)0);
        nz = __syncthreads_or(nz);
        if (threadIdx.x == 0) flag[k] = nz;
    }
}

static dim3 diag_grid(const Matrix &M) {
    int64_t maxlen = 1;
    for (const auto &m : M.meta) maxlen = std::max(maxlen, m.hi - m.lo);
    int64_t gx = (maxlen + 1023) / 1024;
    gx = std::min<int64_t>(gx, 4 * num_sms());
    const int64_t gy = std::min<int64_t>(std::max<int32_t>(M.nd, 1), 65535);
    return dim3((unsigned)std::max<int64_t>(gx, 1), (unsigned)gy);
}

int scatter_packed(Matrix &M, const double *re, const double *im, cudaStream_t s) {
    M.tmask_ok = false;
    if (M.nd == 0 || M.total == 0) return DIAQ_OK;
    if (M.prec == DIAQ_C128F2) return f2_scatter(M, re, im, s);
    const dim3 g = diag_grid(M);
    if (M.prec == DIAQ_C128)
        scatter_kernel<double, double><<<g, 256, 0, s>>>(M.d_meta, M.nd, re, im, (double *)M.re, (double *)M.im);
    else
        scatter_kernel<double, float><<<g, 256, 0, s>>>(M.d_meta, M.nd, re, im, (float *)M.re, (float *)M.im);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

int gather_packed(const Matrix &M, double *re, double *im, cudaStream_t s) {
    if (M.nd == 0 || M.total == 0) return DIAQ_OK;
    if (M.prec == DIAQ_C128F2) return f2_gather(M, re, im, s);
    const dim3 g = diag_grid(M);
    if (M.prec == DIAQ_C128)
        gather_kernel<double><<<g, 256, 0, s>>>(M.d_meta, M.nd, (const double *)M.re, (const double *)M.im, re, im);
    else
        gather_kernel<float><<<g, 256, 0, s>>>(M.d_meta, M.nd, (const float *)M.re, (const float *)M.im, re, im);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// Copy the values of src into dst (dst's offsets are a subset of src's; map[k] = src slot of
// dst slot k, NULL when the slots coincide).
static int remap(const Matrix &src, Matrix &dst, const int32_t *d_map, cudaStream_t s) {
    dst.tmask_ok = false;
    if (dst.nd == 0) return DIAQ_OK;
    const dim3 g = diag_grid(dst);
    if (src.prec == DIAQ_C128 && dst.prec == DIAQ_C128)
        remap_kernel<double, double><<<g, 256, 0, s>>>(src.d_meta, (const double *)src.re, (const double *)src.im,
                                                       dst.d_meta, (double *)dst.re, (double *)dst.im, d_map, dst.nd);
    else if (src.prec == DIAQ_C128 && dst.prec == DIAQ_C64)
        remap_kernel<double, float><<<g, 256, 0, s>>>(src.d_meta, (const double *)src.re, (const double *)src.im,
                                                      dst.d_meta, (float *)dst.re, (float *)dst.im, d_map, dst.nd);
    else if (src.prec == DIAQ_C64 && dst.prec == DIAQ_C128)
        remap_kernel<float, double><<<g, 256, 0, s>>>(src.d_meta, (const float *)src.re, (const float *)src.im,
                                                      dst.d_meta, (double *)dst.re, (double *)dst.im, d_map, dst.nd);
    else
        remap_kernel<float, float><<<g, 256, 0, s>>>(src.d_meta, (const float *)src.re, (const float *)src.im,
                                                     dst.d_meta, (float *)dst.re, (float *)dst.im, d_map, dst.nd);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

int copy_as(const Matrix &A, int prec, cudaStream_t s, Matrix **out) {
    Matrix *C = nullptr;
    DQ_TRY(make_zero(A.rows, A.cols, A.nd, A.off.data(), prec, s, &C));
    int st = DIAQ_OK;
    if (A.prec == DIAQ_C128F2 && prec == DIAQ_C128F2) {
        cudaError_t e = cudaMemcpyAsync(C->re, A.re, A.capacity * A.elem(), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(C->im, A.im, A.capacity * A.elem(), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) st = cuda_status(e, "copy", __FILE__, __LINE__);
    } else if (A.prec == DIAQ_C128F2 || prec == DIAQ_C128F2) {
        st = f2_convert(A, *C, s);
    } else {
        st = remap(A, *C, nullptr, s);
    }
    if (st == DIAQ_OK) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_status(e, "cudaStreamSynchronize", __FILE__, __LINE__);
    }
    if (st != DIAQ_OK) {
        destroy(C);
        return st;
    }
    *out = C;
    return DIAQ_OK;
}

int prune_matrix(const Matrix &A, cudaStream_t s, Matrix **out) {
    if (A.prec == DIAQ_C128F2) return set_error(DIAQ_ERR_UNSUPPORTED, "prune: convert a c128f2 matrix to c128 first");
    std::vector<int32_t> flag(A.nd, 1);
    if (A.nd > 0) {
        int32_t *d_flag = nullptr;
        DQ_CUDA(dev_malloc(&d_flag, sizeof(int32_t) * A.nd));
        const int grid = (int)std::min<int64_t>(A.nd, 65535);
        if (A.prec == DIAQ_C128)
            nonzero_kernel<double><<<grid, 256, 0, s>>>(A.d_meta, A.nd, (const double *)A.re, (const double *)A.im, d_flag);
        else
            nonzero_kernel<float><<<grid, 256, 0, s>>>(A.d_meta, A.nd, (const float *)A.re, (const float *)A.im, d_flag);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(flag.data(), d_flag, sizeof(int32_t) * A.nd, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFree(d_flag);
        if (e != cudaSuccess) return cuda_status(e, "prune flags", __FILE__, __LINE__);
    }
    std::vector<int32_t> keep_off, map;
    for (int32_t k = 0; k < A.nd; ++k)
        if (flag[k]) {
            keep_off.push_back(A.off[k]);
            map.push_back(k);
        }
    Matrix *C = nullptr;
    DQ_TRY(make_zero(A.rows, A.cols, (int32_t)keep_off.size(), keep_off.data(), A.prec, s, &C));
    int st = DIAQ_OK;
    if (C->nd > 0) {
        int32_t *d_map = nullptr;
        cudaError_t e = dev_malloc(&d_map, sizeof(int32_t) * C->nd);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_map, map.data(), sizeof(int32_t) * C->nd, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) st = remap(A, *C, d_map, s);
        else st = cuda_status(e, "prune map", __FILE__, __LINE__);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (d_map) cudaFree(d_map);
        if (st == DIAQ_OK && e != cudaSuccess) st = cuda_status(e, "prune copy", __FILE__, __LINE__);
    }
    if (st != DIAQ_OK) {
        destroy(C);
        return st;
    }
    *out = C;
    return DIAQ_OK;
}

}  // namespace diaq_gb300

// ---- C ABI -------------------------------------------------------------------------------------
using namespace diaq_gb300;

extern "C" {

const char *diaq_last_error(void) { return g_last_error.c_str(); }

const char *diaq_version(void) { return "diaq_gb300 0.1 (sm_103a)"; }

int diaq_matrix_create(int64_t rows, int64_t cols, int32_t ndiag, const int32_t *offsets,
                       const double *re, const double *im, int values_on_device, int precision,
                       void *stream, diaq_matrix_t *out) {
    if (!out) return set_error(DIAQ_ERR_INVALID, "out pointer is NULL");
    *out = nullptr;
    if ((re == nullptr) != (im == nullptr))
        return set_error(DIAQ_ERR_INVALID, "re and im must both be given or both be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    Matrix *M = nullptr;
    DQ_TRY(make_zero(rows, cols, ndiag, offsets, precision, s, &M));
    if (re && M->total > 0) {
        const double *dre = re, *dim = im;
        double *stage = nullptr;
        int st = DIAQ_OK;
        if (!values_on_device) {
            const size_t bytes = sizeof(double) * (size_t)M->total;
            cudaError_t e = dev_malloc(&stage, 2 * bytes);
            if (e == cudaSuccess) e = cudaMemcpyAsync(stage, re, bytes, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(stage + M->total, im, bytes, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) st = cuda_status(e, "upload", __FILE__, __LINE__);
            dre = stage;
            dim = stage + M->total;
        }
        if (st == DIAQ_OK) st = scatter_packed(*M, dre, dim, s);
        if (st == DIAQ_OK) {
            cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) st = cuda_status(e, "cudaStreamSynchronize", __FILE__, __LINE__);
        }
        if (stage) cudaFree(stage);
        if (st != DIAQ_OK) {
            destroy(M);
            return st;
        }
    }
    *out = handle(M);
    return DIAQ_OK;
}

int diaq_matrix_destroy(diaq_matrix_t A) {
    destroy(A);
    return DIAQ_OK;
}

int diaq_matrix_info(diaq_matrix_t A, int64_t *rows, int64_t *cols, int32_t *ndiag,
                     int64_t *total, int *precision) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (rows) *rows = A->rows;
    if (cols) *cols = A->cols;
    if (ndiag) *ndiag = A->nd;
    if (total) *total = A->total;
    if (precision) *precision = A->prec;
    return DIAQ_OK;
}

int diaq_matrix_offsets(diaq_matrix_t A, int32_t *offsets) {
    if (!A || (!offsets && A->nd > 0)) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    if (A->nd) std::memcpy(offsets, A->off.data(), sizeof(int32_t) * A->nd);
    return DIAQ_OK;
}

int diaq_matrix_download(diaq_matrix_t A, double *re, double *im, int dst_on_device, void *stream) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (A->total == 0) return DIAQ_OK;
    if (!re || !im) return set_error(DIAQ_ERR_INVALID, "destination pointer is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (dst_on_device) {
        DQ_TRY(gather_packed(*A, re, im, s));
        DQ_CUDA(cudaStreamSynchronize(s));
        return DIAQ_OK;
    }
    double *stage = nullptr;
    const size_t bytes = sizeof(double) * (size_t)A->total;
    DQ_CUDA(dev_malloc(&stage, 2 * bytes));
    int st = gather_packed(*A, stage, stage + A->total, s);
    cudaError_t e = cudaSuccess;
    if (st == DIAQ_OK) e = cudaMemcpyAsync(re, stage, bytes, cudaMemcpyDeviceToHost, s);
    if (st == DIAQ_OK && e == cudaSuccess) e = cudaMemcpyAsync(im, stage + A->total, bytes, cudaMemcpyDeviceToHost, s);
    if (st == DIAQ_OK && e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(stage);
    if (st == DIAQ_OK && e != cudaSuccess) st = cuda_status(e, "download", __FILE__, __LINE__);
    return st;
}

int diaq_matrix_copy(diaq_matrix_t A, void *stream, diaq_matrix_t *out) {
    if (!A || !out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    Matrix *C = nullptr;
    DQ_TRY(copy_as(*A, A->prec, (cudaStream_t)stream, &C));
    *out = handle(C);
    return DIAQ_OK;
}

int diaq_matrix_convert(diaq_matrix_t A, int precision, void *stream, diaq_matrix_t *out) {
    if (!A || !out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    Matrix *C = nullptr;
    DQ_TRY(copy_as(*A, precision, (cudaStream_t)stream, &C));
    *out = handle(C);
    return DIAQ_OK;
}

int diaq_matrix_prune(diaq_matrix_t A, void *stream, diaq_matrix_t *out) {
    if (!A || !out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    Matrix *C = nullptr;
    DQ_TRY(prune_matrix(*A, (cudaStream_t)stream, &C));
    *out = handle(C);
    return DIAQ_OK;
}

}  // extern "C"
