// Internal declarations shared by the translation units of libdiaq_gb300.so.
//
// Device layout of a DiaQ matrix ("row-phase aligned"): the diagonals keep the reference's
// slot order and are stored back to back in two SoA arrays (re, im) of float64 (c128) or
// float32 (c64).  Diagonal k with offset d holds rows [lo, hi), lo = max(0, -d), hi = lo + len;
// the value of row r sits at re[base + r].  Each diagonal's first value is placed at the next
// index s >= cursor with s == lo (mod kAlign), so base = s - lo is a multiple of kAlign: the
// values of rows r .. r+V-1 (r a multiple of V) form one aligned 16-byte vector on every
// diagonal.  The gap this costs is < kAlign values per diagonal (the reference pads diagonal
// starts to the SIMD width on the host in the same spirit, src/diaQMatrix.hpp:313-327).  A
// guard of kAlign zero values sits before the first and after the last diagonal, so a vector
// that straddles a diagonal's first or last row stays inside the allocation; the kernels mask
// the rows outside [lo, hi).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/diaq_gb300.h"

namespace diaq_gb300 {

constexpr int64_t kAlign = 32;  // values; 256 B for c128, 128 B for c64

struct DiagMeta {
    int64_t base;    // element index of (virtual) row 0: value of row r at vals[base + r]
    int64_t lo, hi;  // rows [lo, hi) are stored
    int64_t pstart;  // start of this diagonal in the reference's packed layout
    int32_t off;     // diagonal offset d (column = row + d)
    int32_t slot;    // slot index
    int64_t pad;
};
static_assert(sizeof(DiagMeta) == 48, "DiagMeta layout");

struct Matrix {
    int64_t rows = 0, cols = 0;
    int32_t nd = 0;
    int prec = DIAQ_C128;                  // DIAQ_C128 (double), DIAQ_C64 (float), DIAQ_C128F2 (float pairs)
    std::vector<int32_t> off;              // host copies, slot order
    std::vector<DiagMeta> meta;
    int64_t capacity = 0;                  // values allocated per array
    int64_t total = 0;                     // stored values (sum of lengths, no gaps)
    void *re = nullptr, *im = nullptr;     // device value arrays
    DiagMeta *d_meta = nullptr;            // device copy of meta
    int device = 0;
    // zero-tile mask of the values (see spmv_kernel.cuh), built on first use by the SpMV entry
    // points; every function that writes values into an existing matrix clears tmask_ok
    mutable uint32_t *tmask = nullptr;
    mutable bool tmask_ok = false;

    // bytes per stored value and array (C128F2: a hi and a lo float, in two planes)
    size_t elem() const { return prec == DIAQ_C64 ? sizeof(float) : sizeof(double); }
};

// ---- error state -------------------------------------------------------------------------
int set_error(int status, const std::string &msg);
int cuda_status(cudaError_t e, const char *what, const char *file, int line);
#define DQ_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t _e = (call);                                                        \
        if (_e != cudaSuccess) return ::diaq_gb300::cuda_status(_e, #call, __FILE__, __LINE__); \
    } while (0)
#define DQ_TRY(call)                 \
    do {                             \
        int _s = (call);             \
        if (_s != DIAQ_OK) return _s; \
    } while (0)

// ---- device allocation -------------------------------------------------------------------------
// Every device allocation of the library goes through dev_malloc / dev_malloc_async.  A single
// allocation larger than the byte count in the environment variable DIAQ_DEVICE_ALLOC_LIMIT
// (read at every call; unset, empty or unparsable = no limit) fails as cudaErrorMemoryAllocation
// without reaching the driver, which the entry points report as DIAQ_ERR_OOM: a host-side way to
// drive the out-of-memory paths (the reference maps a failed cudaMalloc to a runtime error,
// src/cuda_check.hpp:11-18).
size_t alloc_limit();
template <typename T>
inline cudaError_t dev_malloc(T **p, size_t bytes) {
    if (bytes > alloc_limit()) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}
template <typename T>
inline cudaError_t dev_malloc_async(T **p, size_t bytes, cudaStream_t s) {
    if (bytes > alloc_limit()) return cudaErrorMemoryAllocation;
    return cudaMallocAsync(p, bytes, s);
}

// ---- geometry ----------------------------------------------------------------------------
int64_t diag_len(int64_t rows, int64_t cols, int64_t d);
// Lay out a matrix of these offsets (fills meta, capacity, total); validates the offsets.
int plan_layout(Matrix &M, int64_t rows, int64_t cols, int32_t nd, const int32_t *off);
// Allocate device storage for a planned matrix (zeroed unless zero == false) and upload its
// metadata.
int allocate(Matrix &M, cudaStream_t s, bool zero = true);
void release(Matrix &M);

// A new matrix with these offsets, all values zero; zero == false leaves the storage
// uninitialised for a caller that writes every stored value and then calls zero_gaps.
int make_zero(int64_t rows, int64_t cols, int32_t nd, const int32_t *off, int prec,
              cudaStream_t s, Matrix **out, bool zero = true);
// Zero what lies outside the stored rows: the guard before the first diagonal, the alignment gaps
// between diagonals and the tail of the allocation (every plane).
int zero_gaps(const Matrix &M, cudaStream_t s);

// Packed (reference layout) float64 values <-> device layout.
int scatter_packed(Matrix &M, const double *re, const double *im, cudaStream_t s);
int gather_packed(const Matrix &M, double *re, double *im, cudaStream_t s);

// ---- kernels used across units ------------------------------------------------------------
int spmv_launch(const Matrix &A, const void *xr, const void *xi, int64_t ldx, void *yr, void *yi,
                int64_t ldy, int nrhs, cudaStream_t s);

// Taylor term of the time evolution: term_out = (-i * scale) * (A term_in); acc += term_out
// (acc = init + term_out when init is given).  Vectors in the matrix's precision.  tmask: A's
// zero-tile mask, or NULL.
int taylor_term_launch(const Matrix &A, const void *tin_r, const void *tin_i, void *tout_r,
                       void *tout_i, void *acc_r, void *acc_i, const void *init_r,
                       const void *init_i, double scale, int nrhs, int64_t ld, cudaStream_t s,
                       const uint32_t *tmask);

int num_sms();

// DIAQ_C128F2 (spmv_f2.cu)
int f2_scatter(Matrix &M, const double *re, const double *im, cudaStream_t s);
int f2_gather(const Matrix &M, double *re, double *im, cudaStream_t s);
int f2_convert(const Matrix &src, Matrix &dst, cudaStream_t s);
int f2_spmv(const Matrix &A, const double *xr, const double *xi, double *yr, double *yi, cudaStream_t s);

// Copy of A in precision prec / A without its exact-zero diagonals (new matrices).
int copy_as(const Matrix &A, int prec, cudaStream_t s, Matrix **out);
int prune_matrix(const Matrix &A, cudaStream_t s, Matrix **out);
void destroy(Matrix *M);

}  // namespace diaq_gb300

// The public handle is a Matrix; every Matrix is allocated as one (make_zero).
struct diaq_matrix_s : public diaq_gb300::Matrix {};

namespace diaq_gb300 {
inline diaq_matrix_t handle(Matrix *m) { return static_cast<diaq_matrix_t>(m); }
}  // namespace diaq_gb300
