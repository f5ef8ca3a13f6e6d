// SpMV entry points: y = A x on device vectors, one or several right-hand sides.
// Replaces spmv_device / spmv_row_kernel / spmv_single_diag_kernel (src/spMV_gpu.cu:17-168).
#include <algorithm>

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

int spmv_launch(const Matrix &A, const void *xr, const void *xi, int64_t ldx, void *yr, void *yi,
                int64_t ldy, int nrhs, cudaStream_t s) {
    if (A.rows == 0 || nrhs <= 0) return DIAQ_OK;
    if (!xr || !xi || !yr || !yi) return set_error(DIAQ_ERR_INVALID, "vector pointer is NULL");
    if (nrhs > 1 && (ldx < A.cols || ldy < A.rows))
        return set_error(DIAQ_ERR_INVALID, "leading dimension smaller than the vector length");
    if (A.prec == DIAQ_C128F2) {  // float64 vectors, float-pair arithmetic; one state per launch
        for (int q = 0; q < nrhs; ++q)
            DQ_TRY(f2_spmv(A, (const double *)xr + q * ldx, (const double *)xi + q * ldx, (double *)yr + q * ldy,
                           (double *)yi + q * ldy, s));
        return DIAQ_OK;
    }
    if (A.prec == DIAQ_C128) {
        EpiStoreRhs<double> e;
        e.yr = (double *)yr;
        e.yi = (double *)yi;
        e.ldy = ldy;
        return launch_dia_spmv_rhs<double>(A, (const double *)xr, (const double *)xi, ldx, nrhs, e, s);
    }
    EpiStoreRhs<float> e;
    e.yr = (float *)yr;
    e.yi = (float *)yi;
    e.ldy = ldy;
    return launch_dia_spmv_rhs<float>(A, (const float *)xr, (const float *)xi, ldx, nrhs, e, s);
}

int taylor_term_launch(const Matrix &A, const void *tin_r, const void *tin_i, void *tout_r,
                       void *tout_i, void *acc_r, void *acc_i, const void *init_r,
                       const void *init_i, double scale, int nrhs, int64_t ld, cudaStream_t s,
                       const uint32_t *tmask) {
    if (A.prec == DIAQ_C128) {
        EpiTaylorRhs<double> e;
        e.tr = (double *)tout_r;
        e.ti = (double *)tout_i;
        e.accr = (double *)acc_r;
        e.acci = (double *)acc_i;
        e.initr = (const double *)init_r;
        e.initi = (const double *)init_i;
        e.ld = ld;
        e.scale = scale;
        return launch_dia_spmv_rhs_cfg<double, EpiTaylorRhs<double>, VecOf<double>::V>(
            A, (const double *)tin_r, (const double *)tin_i, ld, nrhs, e, s, SpmvCfg{}, tmask);
    }
    EpiTaylorRhs<float> e;
    e.tr = (float *)tout_r;
    e.ti = (float *)tout_i;
    e.accr = (float *)acc_r;
    e.acci = (float *)acc_i;
    e.initr = (const float *)init_r;
    e.initi = (const float *)init_i;
    e.ld = ld;
    e.scale = (float)scale;
    return launch_dia_spmv_rhs_cfg<float, EpiTaylorRhs<float>, VecOf<float>::V>(
        A, (const float *)tin_r, (const float *)tin_i, ld, nrhs, e, s, SpmvCfg{}, tmask);
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_spmv_z(diaq_matrix_t A, const double *x_re, const double *x_im, double *y_re,
                double *y_im, void *stream) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (A->prec != DIAQ_C128 && A->prec != DIAQ_C128F2)
        return set_error(DIAQ_ERR_INVALID, "diaq_spmv_z needs a c128 or c128f2 matrix");
    return spmv_launch(*A, x_re, x_im, A->cols, y_re, y_im, A->rows, 1, (cudaStream_t)stream);
}

int diaq_spmv_c(diaq_matrix_t A, const float *x_re, const float *x_im, float *y_re, float *y_im,
                void *stream) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (A->prec != DIAQ_C64) return set_error(DIAQ_ERR_INVALID, "diaq_spmv_c needs a c64 matrix");
    return spmv_launch(*A, x_re, x_im, A->cols, y_re, y_im, A->rows, 1, (cudaStream_t)stream);
}

int diaq_spmm(diaq_matrix_t A, int nrhs, const void *x_re, const void *x_im, int64_t ldx,
              void *y_re, void *y_im, int64_t ldy, void *stream) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (nrhs < 0) return set_error(DIAQ_ERR_INVALID, "nrhs must be non-negative");
    return spmv_launch(*A, x_re, x_im, ldx, y_re, y_im, ldy, nrhs, (cudaStream_t)stream);
}

}  // extern "C"

namespace {
// Device scratch for host-vector calls, released on scope exit.
struct Scratch {
    double *p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
};
}  // namespace

extern "C" {

int diaq_spmv_host(diaq_matrix_t A, const double *x_re, const double *x_im, double *y_re,
                   double *y_im) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (A->prec != DIAQ_C128 && A->prec != DIAQ_C128F2) return set_error(DIAQ_ERR_INVALID, "spmv_cuda: needs a c128 matrix");
    if (A->rows == 0) return DIAQ_OK;
    if (!x_re || !x_im || !y_re || !y_im) return set_error(DIAQ_ERR_INVALID, "vector pointer is NULL");
    Scratch w;
    const int64_t M = A->rows, N = A->cols;
    DQ_CUDA(dev_malloc(&w.p, sizeof(double) * (size_t)(2 * N + 2 * M)));
    double *xr = w.p, *xi = w.p + N, *yr = w.p + 2 * N, *yi = w.p + 2 * N + M;
    DQ_CUDA(cudaMemcpy(xr, x_re, sizeof(double) * N, cudaMemcpyHostToDevice));
    DQ_CUDA(cudaMemcpy(xi, x_im, sizeof(double) * N, cudaMemcpyHostToDevice));
    DQ_TRY(spmv_launch(*A, xr, xi, N, yr, yi, M, 1, 0));
    DQ_CUDA(cudaMemcpy(y_re, yr, sizeof(double) * M, cudaMemcpyDeviceToHost));
    DQ_CUDA(cudaMemcpy(y_im, yi, sizeof(double) * M, cudaMemcpyDeviceToHost));
    return DIAQ_OK;
}

int diaq_spmv_ntimes_host(diaq_matrix_t A, const double *x_re, const double *x_im, int n,
                          double *y_re, double *y_im) {
    if (!A) return set_error(DIAQ_ERR_INVALID, "matrix handle is NULL");
    if (A->prec != DIAQ_C128) return set_error(DIAQ_ERR_INVALID, "spmv_ntimes_cuda: needs a c128 matrix");
    if (n < 0) return set_error(DIAQ_ERR_INVALID, "spmv_ntimes_cuda: num_times must be >= 0");
    const int64_t M = A->rows, N = A->cols;
    if (n == 0) {
        if (M != N)
            return set_error(DIAQ_ERR_INVALID,
                             "spmv_ntimes_cuda: num_times==0 requires square matrix (M==N) to copy x -> y");
        std::copy(x_re, x_re + M, y_re);
        std::copy(x_im, x_im + M, y_im);
        return DIAQ_OK;
    }
    if (n > 1 && M != N)
        return set_error(DIAQ_ERR_INVALID,
                         "spmv_ntimes_cuda: repeated SpMV requires square matrix (M==N) for num_times > 1");
    if (M == 0) return DIAQ_OK;
    Scratch w;
    const int64_t L = std::max(M, N);
    DQ_CUDA(dev_malloc(&w.p, sizeof(double) * (size_t)(4 * L)));
    double *ar = w.p, *ai = w.p + L, *br = w.p + 2 * L, *bi = w.p + 3 * L;
    DQ_CUDA(cudaMemcpy(ar, x_re, sizeof(double) * N, cudaMemcpyHostToDevice));
    DQ_CUDA(cudaMemcpy(ai, x_im, sizeof(double) * N, cudaMemcpyHostToDevice));
    for (int t = 0; t < n; ++t) {
        DQ_TRY(spmv_launch(*A, ar, ai, N, br, bi, M, 1, 0));
        std::swap(ar, br);
        std::swap(ai, bi);
    }
    DQ_CUDA(cudaMemcpy(y_re, ar, sizeof(double) * M, cudaMemcpyDeviceToHost));
    DQ_CUDA(cudaMemcpy(y_im, ai, sizeof(double) * M, cudaMemcpyDeviceToHost));
    return DIAQ_OK;
}

}  // extern "C"
