// ref_harness.cpp -- a C-ABI wrapper around the reference's own CPU code (built unmodified from
// its sources by oracle/Makefile into oracle/_ref/).  TEST INFRASTRUCTURE ONLY: it pins the C
// restatement in diaq_oracle.c and generates golden fixtures; the product never links it.
//
// Matrices cross this boundary packed (diagonals back to back, no padding).  They are built on
// the reference side with diaQMatrix(shape, dIndices) + setContiguousData
// (src/diaQMatrix.hpp:708-745), which avoids the 32-bit kron helpers.
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "diaq.hpp"

using diaq::diaQMatrix;
using diaq::valType;

namespace {
thread_local std::string g_err;

std::shared_ptr<diaQMatrix> build(int64_t rows, int64_t cols, int32_t nd, const int32_t *off,
                                  const double *re, const double *im) {
    std::array<unsigned int, 2> shape{(unsigned int)rows, (unsigned int)cols};
    std::vector<int> d(off, off + nd);
    auto A = std::make_shared<diaQMatrix>(shape, d);
    size_t total = 0;
    for (int32_t k = 0; k < nd; ++k) total += A->getDiagonalLengthInternal(d[k]);
    std::vector<valType> r(re, re + total), i(im, im + total);
    if (nd > 0) A->setContiguousData(r, i);
    return A;
}

struct Held {
    std::shared_ptr<diaQMatrix> m;
};
}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

int ref_threads() { return omp_get_max_threads(); }
void ref_set_threads(int n) { omp_set_num_threads(n); }

// y = A x through diaq::spMV (src/spMV.cpp:27-322).
int ref_spmv(int64_t rows, int64_t cols, int32_t nd, const int32_t *off, const double *re,
             const double *im, const double *xr, const double *xi, double *yr, double *yi) {
    try {
        auto A = build(rows, cols, nd, off, re, im);
        auto x = std::make_shared<diaq::vector>((unsigned int)cols);
        auto y = std::make_shared<diaq::vector>((unsigned int)rows);
        std::memcpy(x->realValues, xr, sizeof(double) * cols);
        std::memcpy(x->imagValues, xi, sizeof(double) * cols);
        diaq::spMV(A, x, y);
        std::memcpy(yr, y->realValues, sizeof(double) * rows);
        std::memcpy(yi, y->imagValues, sizeof(double) * rows);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

// A matrix handle built on the reference side, so that timing loops exclude construction.
void *ref_matrix_new(int64_t rows, int64_t cols, int32_t nd, const int32_t *off,
                     const double *re, const double *im) {
    try {
        return new Held{build(rows, cols, nd, off, re, im)};
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}
void ref_matrix_free(void *h) { delete static_cast<Held *>(h); }

// Shape, diagonal count and packed (unpadded) value count of a handle.
void ref_matrix_info(void *h, int64_t *rows, int64_t *cols, int32_t *nd, int64_t *total) {
    auto &A = *static_cast<Held *>(h)->m;
    *rows = A.matrix_shape[0];
    *cols = A.matrix_shape[1];
    *nd = (int32_t)A.dIndices.size();
    int64_t t = 0;
    for (int d : A.dIndices) t += A.getDiagonalLengthInternal(d);
    *total = t;
}

// Offsets in slot order and packed values of a handle.
void ref_matrix_export(void *h, int32_t *off, double *re, double *im) {
    auto &A = *static_cast<Held *>(h)->m;
    int64_t s = 0;
    for (size_t k = 0; k < A.dIndices.size(); ++k) {
        off[k] = A.dIndices[k];
        const unsigned int len = A.getDiagonalLengthInternal(A.dIndices[k]);
        std::memcpy(re + s, A.realData + A.diagOffsets[k], sizeof(double) * len);
        std::memcpy(im + s, A.imagData + A.diagOffsets[k], sizeof(double) * len);
        s += len;
    }
}

// y = A x on a prebuilt handle (for timing).
int ref_spmv_h(void *h, const double *xr, const double *xi, double *yr, double *yi) {
    try {
        auto &A = static_cast<Held *>(h)->m;
        const unsigned int rows = A->matrix_shape[0], cols = A->matrix_shape[1];
        auto x = std::make_shared<diaq::vector>(cols);
        auto y = std::make_shared<diaq::vector>(rows);
        std::memcpy(x->realValues, xr, sizeof(double) * cols);
        std::memcpy(x->imagValues, xi, sizeof(double) * cols);
        diaq::spMV(A, x, y);
        std::memcpy(yr, y->realValues, sizeof(double) * rows);
        std::memcpy(yi, y->imagValues, sizeof(double) * rows);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

// C = A B through diaq::product (src/spGEMM.cpp:303-538, pruned as the reference prunes).
void *ref_product(void *a, void *b) {
    try {
        return new Held{diaq::product(static_cast<Held *>(a)->m, static_cast<Held *>(b)->m)};
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

// A^n through diaq::pow (src/spPow.cpp:19-56).
void *ref_pow(void *a, int n) {
    try {
        return new Held{diaq::pow(static_cast<Held *>(a)->m, n)};
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

// exp(-i t A) through diaq::expm_negative_taylor_scaled (src/spME.cpp:230-295).
void *ref_expm_negative(void *a, double t, int max_it, double cutoff, double tol) {
    try {
        return new Held{diaq::expm_negative_taylor_scaled(static_cast<Held *>(a)->m, t, max_it,
                                                          cutoff, tol)};
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

// exp(-i t A) through diaq::expm_negative_pade (src/spME.cpp:298-445, its inverse :447-589).
void *ref_expm_negative_pade(void *a, double t, int max_it, double cutoff, double tol) {
    try {
        return new Held{diaq::expm_negative_pade(static_cast<Held *>(a)->m, t, max_it, cutoff, tol)};
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

// exp(A) through diaq::expm_taylor_scaled (src/spME.cpp:13-80).
void *ref_expm(void *a, int max_it, double cutoff, double tol) {
    try {
        return new Held{diaq::expm_taylor_scaled(static_cast<Held *>(a)->m, max_it, cutoff, tol)};
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

double ref_norm1_est(void *a) { return static_cast<Held *>(a)->m->estimate_1norm(); }
double ref_frobenius(void *a) { return static_cast<Held *>(a)->m->norm(); }

// The time-evolution action on the reference's own CPU spMV: the reference has no CPU routine
// for it, so this restates src/spHamSim_gpu_all_fused.cu:235-277 and :347 (dt = t / r, exactly
// m Taylor terms per step, no scaling) with diaq::spMV for every term.
int ref_ham_sim(void *h, const double *pr, const double *pi, double t, int64_t r, int m,
                double *outr, double *outi) {
    try {
        auto &H = static_cast<Held *>(h)->m;
        const unsigned int n = H->matrix_shape[0];
        std::memcpy(outr, pr, sizeof(double) * n);
        std::memcpy(outi, pi, sizeof(double) * n);
        if (r == 0) return 0;
        auto a = std::make_shared<diaq::vector>(n), b = std::make_shared<diaq::vector>(n),
             term = std::make_shared<diaq::vector>(n), tmp = std::make_shared<diaq::vector>(n);
        std::memcpy(a->realValues, pr, sizeof(double) * n);
        std::memcpy(a->imagValues, pi, sizeof(double) * n);
        const double dt = t / (double)r;
        for (int64_t step = 0; step < r; ++step) {
            std::memcpy(b->realValues, a->realValues, sizeof(double) * n);
            std::memcpy(b->imagValues, a->imagValues, sizeof(double) * n);
            std::memcpy(term->realValues, a->realValues, sizeof(double) * n);
            std::memcpy(term->imagValues, a->imagValues, sizeof(double) * n);
            for (int k = 1; k <= m; ++k) {
                diaq::spMV(H, term, tmp);
                const double scale = dt / (double)k;
                double *tr = term->realValues, *ti = term->imagValues;
                const double *wr = tmp->realValues, *wi = tmp->imagValues;
                double *br = b->realValues, *bi = b->imagValues;
#pragma omp parallel for schedule(static)
                for (long long i = 0; i < (long long)n; ++i) {
                    tr[i] = wi[i] * scale;
                    ti[i] = -wr[i] * scale;
                    br[i] += tr[i];
                    bi[i] += ti[i];
                }
            }
            std::swap(a, b);
        }
        std::memcpy(outr, a->realValues, sizeof(double) * n);
        std::memcpy(outi, a->imagValues, sizeof(double) * n);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

}  // extern "C"
