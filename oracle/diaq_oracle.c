/*
 * diaq_oracle.c -- CPU restatement of DiaQ's diagonal-sparse hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: it is imported by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / reference leg, and never by the
 * product path (diaq_gb300/), which has no CPU fallback.
 *
 * Storage convention (the DiaQ format as the reference packs it on the device,
 * src/deviceMatrix_gpu.cu:30-55): a matrix is (rows, cols, ndiag, off[ndiag]) plus two value
 * arrays re[], im[] holding the diagonals back to back in slot order, diagonal k starting at
 * start[k] = sum_{j<k} len[j], with len from diaq_len() below.  Element j of diagonal d sits at
 * matrix position (j, j+d) for d >= 0 and (j-d, j) for d < 0 (src/diaQMatrix.hpp:460-478).
 *
 * Arithmetic is plain IEEE double; the file is compiled with -ffp-contract=off so x86 and Arm
 * give identical bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Diagonal length, src/diaQMatrix.hpp:390-409 (getDiagonalLengthInternal) for in-range d.
 * Out-of-range diagonals (|d| beyond the matrix) have length 0 here. */
int64_t diaq_len(int64_t rows, int64_t cols, int32_t d) {
    int64_t len;
    if (d < 0) len = rows + d;
    else if (d > 0) len = cols - d;
    else len = rows < cols ? rows : cols;
    if (len > rows) len = rows;
    else if (len > cols) len = cols;
    return len < 0 ? 0 : len;
}

/* Packed start of every diagonal; returns the total stored length. */
int64_t diaq_starts(int64_t rows, int64_t cols, int32_t nd, const int32_t *off, int64_t *start) {
    int64_t s = 0;
    for (int32_t k = 0; k < nd; ++k) {
        start[k] = s;
        s += diaq_len(rows, cols, off[k]);
    }
    return s;
}

/* ------------------------------------------------------------------------------------------
 * SpMV  y = A x  (src/spMV.cpp:27-322 on the CPU; src/spMV_gpu.cu:74-136 on the GPU).
 * Row r sums the stored diagonals in slot order; y is overwritten.
 * ---------------------------------------------------------------------------------------- */
void diaq_spmv(int64_t rows, int64_t cols, int32_t nd, const int32_t *off, const double *re,
               const double *im, const double *xr, const double *xi, double *yr, double *yi) {
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (nd > 0 ? nd : 1));
    int64_t *len = (int64_t *)malloc(sizeof(int64_t) * (nd > 0 ? nd : 1));
    diaq_starts(rows, cols, nd, off, start);
    for (int32_t k = 0; k < nd; ++k) len[k] = diaq_len(rows, cols, off[k]);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < rows; ++r) {
        double sr = 0.0, si = 0.0;
        for (int32_t k = 0; k < nd; ++k) {
            const int64_t d = off[k];
            const int64_t pos = d >= 0 ? r : r + d;   /* position along the diagonal */
            if (pos < 0 || pos >= len[k]) continue;
            const int64_t c = r + d;
            const double ar = re[start[k] + pos], ai = im[start[k] + pos];
            sr += ar * xr[c] - ai * xi[c];
            si += ar * xi[c] + ai * xr[c];
        }
        yr[r] = sr;
        yi[r] = si;
    }
    free(start);
    free(len);
}

/* ------------------------------------------------------------------------------------------
 * SpGEMM structural dry-run (src/spGEMM.cpp:346-369, src/spGEMM_gpu.cu:92-101): every pair
 * (dA, dB) gives dC = dA + dB; keep dC in [-(rowsA-1), colsB-1]; the result offsets are the
 * ascending distinct values.  out must hold ndA*ndB entries.  Returns the count.
 * ---------------------------------------------------------------------------------------- */
static int cmp_i32(const void *a, const void *b) {
    const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

static int cmp_i64(const void *a, const void *b) {
    const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* Slot of offset d in keys sorted as (offset << 32 | slot); -1 when absent. */
static int32_t find_slot(const int64_t *keys, int32_t n, int64_t d) {
    int32_t lo = 0, hi = n;
    while (lo < hi) {
        const int32_t mid = lo + (hi - lo) / 2;
        if ((keys[mid] >> 32) < d) lo = mid + 1;
        else hi = mid;
    }
    if (lo < n && (keys[lo] >> 32) == d) return (int32_t)(keys[lo] & 0xffffffff);
    return -1;
}

int32_t diaq_spgemm_symbolic(int64_t rowsA, int32_t ndA, const int32_t *offA, int64_t colsB,
                             int32_t ndB, const int32_t *offB, int32_t *out) {
    const int64_t lo = -(rowsA - 1), hi = colsB - 1;
    int64_t n = 0;
    for (int32_t a = 0; a < ndA; ++a)
        for (int32_t b = 0; b < ndB; ++b) {
            const int64_t dc = (int64_t)offA[a] + offB[b];
            if (dc < lo || dc > hi) continue;
            out[n++] = (int32_t)dc;
        }
    qsort(out, (size_t)n, sizeof(int32_t), cmp_i32);
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i)
        if (m == 0 || out[m - 1] != out[i]) out[m++] = out[i];
    return (int32_t)m;
}

/* ------------------------------------------------------------------------------------------
 * SpGEMM numeric pass: C (structure from the dry-run, packed) = A B.  For result diagonal dC
 * and position t (row r = t + max(0,-dC)), sum over A's slots in order the products
 * A[r, r+dA] * B[r+dA, r+dC] that exist (src/spGEMM.cpp:53-301 aligns the same segments;
 * src/spGEMM_gpu.cu:55-77 sums the pairs of one result diagonal in A-slot order).
 * ---------------------------------------------------------------------------------------- */
void diaq_spgemm_numeric(int64_t rowsA, int64_t colsA, int32_t ndA, const int32_t *offA,
                         const double *Are, const double *Aim, int64_t colsB, int32_t ndB,
                         const int32_t *offB, const double *Bre, const double *Bim, int32_t ndC,
                         const int32_t *offC, double *Cre, double *Cim) {
    const int64_t rowsB = colsA, rowsC = rowsA, colsC = colsB;
    int64_t *sA = (int64_t *)malloc(sizeof(int64_t) * (ndA > 0 ? ndA : 1));
    int64_t *sB = (int64_t *)malloc(sizeof(int64_t) * (ndB > 0 ? ndB : 1));
    int64_t *sC = (int64_t *)malloc(sizeof(int64_t) * (ndC > 0 ? ndC : 1));
    diaq_starts(rowsA, colsA, ndA, offA, sA);
    diaq_starts(rowsB, colsB, ndB, offB, sB);
    diaq_starts(rowsC, colsC, ndC, offC, sC);
    /* B's offsets sorted with their slots, for the lookup dB = dC - dA (offsets are distinct). */
    int64_t *bkey = (int64_t *)malloc(sizeof(int64_t) * (ndB > 0 ? ndB : 1));
    for (int32_t j = 0; j < ndB; ++j) bkey[j] = (int64_t)offB[j] * 4294967296LL + j;
    qsort(bkey, (size_t)ndB, sizeof(int64_t), cmp_i64);
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t c = 0; c < ndC; ++c) {
        const int64_t dc = offC[c];
        const int64_t lenC = diaq_len(rowsC, colsC, (int32_t)dc);
        double *cr = Cre + sC[c], *ci = Cim + sC[c];
        for (int64_t t = 0; t < lenC; ++t) { cr[t] = 0.0; ci[t] = 0.0; }
        for (int32_t a = 0; a < ndA; ++a) {
            const int64_t da = offA[a], db = dc - da;
            const int32_t b = find_slot(bkey, ndB, db);
            if (b < 0) continue;
            const int64_t lenA = diaq_len(rowsA, colsA, (int32_t)da);
            const int64_t lenB = diaq_len(rowsB, colsB, (int32_t)db);
            const double *ar = Are + sA[a], *ai = Aim + sA[a];
            const double *br = Bre + sB[b], *bi = Bim + sB[b];
            /* row r = t + r0; A position pa = r + min(dA,0); B position pb = r + dA + min(dB,0) */
            const int64_t r0 = dc >= 0 ? 0 : -dc;
            const int64_t sa = r0 + (da < 0 ? da : 0);
            const int64_t sb = r0 + da + (db < 0 ? db : 0);
            int64_t t0 = 0, t1 = lenC;
            if (-sa > t0) t0 = -sa;
            if (-sb > t0) t0 = -sb;
            if (lenA - sa < t1) t1 = lenA - sa;
            if (lenB - sb < t1) t1 = lenB - sb;
            for (int64_t t = t0; t < t1; ++t) {
                const double xr = ar[t + sa], xi = ai[t + sa], yr = br[t + sb], yi = bi[t + sb];
                cr[t] += xr * yr - xi * yi;
                ci[t] += xr * yi + xi * yr;
            }
        }
    }
    free(bkey);
    free(sA);
    free(sB);
    free(sC);
}

/* Which diagonals hold a value other than exact zero (src/diaQMatrix.hpp:1555-1570). */
void diaq_nonzero_diags(int64_t rows, int64_t cols, int32_t nd, const int32_t *off,
                        const double *re, const double *im, int8_t *keep) {
    int64_t s = 0;
    for (int32_t k = 0; k < nd; ++k) {
        const int64_t len = diaq_len(rows, cols, off[k]);
        keep[k] = 0;
        for (int64_t j = 0; j < len; ++j)
            if (re[s + j] != 0.0 || im[s + j] != 0.0) { keep[k] = 1; break; }
        s += len;
    }
}

/* 1-norm estimate: max column sum of |re|+|im| (src/diaQMatrix.hpp:1287-1358). */
double diaq_norm1_est(int64_t rows, int64_t cols, int32_t nd, const int32_t *off,
                      const double *re, const double *im) {
    double *col = (double *)calloc((size_t)(cols > 0 ? cols : 1), sizeof(double));
    int64_t s = 0;
    for (int32_t k = 0; k < nd; ++k) {
        const int64_t d = off[k], len = diaq_len(rows, cols, off[k]);
        for (int64_t j = 0; j < len; ++j) {
            const int64_t c = d >= 0 ? d + j : j;
            col[c] += fabs(re[s + j]) + fabs(im[s + j]);
        }
        s += len;
    }
    double m = 0.0;
    for (int64_t c = 0; c < cols; ++c)
        if (col[c] > m) m = col[c];
    free(col);
    return m;
}

/* Frobenius norm over the stored values (src/diaQMatrix.hpp:1255-1284). */
double diaq_frobenius(int64_t total, const double *re, const double *im) {
    double s = 0.0;
    for (int64_t i = 0; i < total; ++i) s += re[i] * re[i] + im[i] * im[i];
    return sqrt(s);
}

/* ------------------------------------------------------------------------------------------
 * Taylor action of one time step, restating src/spHamSim_gpu_all_fused.cu:235-277:
 *   out = psi; term = psi; for k = 1..m: term = (-i dt/k) (H term); out += term.
 * ---------------------------------------------------------------------------------------- */
static void taylor_step(int64_t n, int32_t nd, const int32_t *off, const double *re,
                        const double *im, double dt, int32_t m, const double *pr, const double *pi,
                        double *outr, double *outi, double *tr, double *ti, double *wr,
                        double *wi) {
    memcpy(outr, pr, sizeof(double) * n);
    memcpy(outi, pi, sizeof(double) * n);
    memcpy(tr, pr, sizeof(double) * n);
    memcpy(ti, pi, sizeof(double) * n);
    for (int32_t k = 1; k <= m; ++k) {
        diaq_spmv(n, n, nd, off, re, im, tr, ti, wr, wi);
        const double scale = dt / (double)k;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            tr[i] = wi[i] * scale;
            ti[i] = -wr[i] * scale;
            outr[i] += tr[i];
            outi[i] += ti[i];
        }
    }
}

/* hamiltonian_simulation_cuda (src/spHamSim_gpu_all_fused.cu:287-376): t is the TOTAL time,
 * dt = t / r, every step applies exactly m Taylor terms, r = 0 returns psi0.
 * substeps > 1 splits every step into that many equal sub-steps of m terms each (the
 * reference has no sub-steps; substeps = 1 reproduces it). */
void diaq_ham_sim(int64_t n, int32_t nd, const int32_t *off, const double *re, const double *im,
                  const double *psir, const double *psii, double t, int64_t r, int32_t m,
                  int32_t substeps, double *outr, double *outi) {
    memcpy(outr, psir, sizeof(double) * n);
    memcpy(outi, psii, sizeof(double) * n);
    if (r == 0 || n == 0) return;
    if (substeps < 1) substeps = 1;
    double *buf = (double *)malloc(sizeof(double) * (size_t)n * 8);
    double *ar = buf, *ai = buf + n, *tr = buf + 2 * n, *ti = buf + 3 * n, *wr = buf + 4 * n,
           *wi = buf + 5 * n, *br = buf + 6 * n, *bi = buf + 7 * n;
    memcpy(ar, psir, sizeof(double) * n);
    memcpy(ai, psii, sizeof(double) * n);
    const double dt = t / (double)r / (double)substeps;
    for (int64_t step = 0; step < r * substeps; ++step) {
        taylor_step(n, nd, off, re, im, dt, m, ar, ai, br, bi, tr, ti, wr, wi);
        double *s;
        s = ar; ar = br; br = s;
        s = ai; ai = bi; bi = s;
    }
    memcpy(outr, ar, sizeof(double) * n);
    memcpy(outi, ai, sizeof(double) * n);
    free(buf);
}

/* ------------------------------------------------------------------------------------------
 * DIA x dense, src/spMM_device_gpu.cu:44-127 (spmm_dia_device): C = A B with A in the row-aligned
 * DIA format, vals[k*M + r] = A[r, r + off[k]] (columns outside [0, K) ignored), B K x R and C
 * M x R row-major, float64 (is_complex = 0) or interleaved complex128.  Every element of C sums
 * the diagonals in the order given (src/spMM_device_gpu.cu:60-74); C is overwritten.
 * ---------------------------------------------------------------------------------------- */
void diaq_spmm_dia(const int64_t *off, int32_t nd, int64_t M, int64_t K, const double *vals,
                   const double *B, int64_t R, double *C, int32_t is_complex) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < M; ++r) {
        for (int64_t j = 0; j < R; ++j) {
            double ar = 0.0, ai = 0.0;
            for (int32_t k = 0; k < nd; ++k) {
                const int64_t c = r + off[k];
                if (c < 0 || c >= K) continue;
                if (is_complex) {
                    const double vr = vals[2 * (k * M + r)], vi = vals[2 * (k * M + r) + 1];
                    const double br = B[2 * (c * R + j)], bi = B[2 * (c * R + j) + 1];
                    ar = ar + vr * br - vi * bi;
                    ai = ai + vr * bi + vi * br;
                } else {
                    ar = ar + vals[k * M + r] * B[c * R + j];
                }
            }
            if (is_complex) {
                C[2 * (r * R + j)] = ar;
                C[2 * (r * R + j) + 1] = ai;
            } else {
                C[r * R + j] = ar;
            }
        }
    }
}

int diaq_oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
