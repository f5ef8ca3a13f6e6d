/*
 * diaq_timing.c -- the reference's CPU SpMV scheme, restated for timing the CPU baseline.
 *
 * TEST INFRASTRUCTURE ONLY: bench.py's CPU legs (the reference arm and the cpu_baseline sample)
 * time it on hosts where the reference's own CPU library cannot be built (the GPU hosts do not
 * have the reference sources).  It is never the parity oracle (diaq_oracle.c is; this file is
 * compiled with -O3 and floating-point contraction, so its last bits differ) and never part of
 * the product.
 *
 * The scheme of src/spMV.cpp:62-307 (spMV, CPU build): the work is a list of tasks, one per
 * (diagonal, tile of `tile` consecutive elements along it), handed out to the OpenMP threads with a
 * static schedule; every thread accumulates into a zeroed thread-local y of its own (allocated and
 * zeroed per call by the calling thread, as the reference does), and a final parallel pass sums
 * the thread-local vectors into y.
 * The tile length follows src/config.hpp:114-116: 0.95 of the L1 data cache over six float64
 * arrays, rounded down to the SIMD width.  The inner loops are plain C that the compiler
 * vectorises (the reference hand-writes them with AVX-512 / NEON intrinsics,
 * src/simd_avx512_kernels.cpp:241-441).
 *
 * The time evolution on top is the rule of src/spHamSim_gpu_all_fused.cu:235-277 (exactly m Taylor
 * terms per sub-step; term_k = (-i dt / k) H term_{k-1}, sum += term_k), as in diaq_oracle.c.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int64_t len_of(int64_t n, int32_t d) {
    const int64_t a = d < 0 ? -(int64_t)d : (int64_t)d;
    return a < n ? n - a : 0;
}

static int64_t g_tile = 0;

/* Tile length from the L1 data cache size in bytes (0: 32 KB, the reference's fallback). */
void diaq_timing_set_l1(int64_t l1_bytes, int32_t vec_width) {
    if (l1_bytes <= 0) l1_bytes = 32768;
    if (vec_width <= 0) vec_width = 1;
    int64_t raw = (int64_t)((double)l1_bytes * 0.95 / (6.0 * sizeof(double)));
    int64_t t = raw / vec_width * vec_width;
    g_tile = t > 0 ? t : vec_width;
}

int64_t diaq_timing_tile(void) { return g_tile; }

/* y = A x for a square n x n DiaQ matrix (packed values, slot order). */
void diaq_timing_spmv(int64_t n, int32_t nd, const int32_t *off, const double *re, const double *im,
                      const double *xr, const double *xi, double *yr, double *yi) {
    if (g_tile <= 0) diaq_timing_set_l1(0, 8);
    const int64_t tile = g_tile;
    int64_t ntask = 0;
    for (int32_t k = 0; k < nd; ++k) ntask += (len_of(n, off[k]) + tile - 1) / tile;
    int32_t *tk = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ntask > 0 ? ntask : 1));
    int64_t *ts = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ntask > 0 ? ntask : 1));
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nd > 0 ? nd : 1));
    int64_t t = 0, pos = 0;
    for (int32_t k = 0; k < nd; ++k) {
        const int64_t L = len_of(n, off[k]);
        start[k] = pos;
        pos += L;
        for (int64_t s = 0; s < L; s += tile) {
            tk[t] = k;
            ts[t] = s;
            ++t;
        }
    }
#ifdef _OPENMP
    const int T = omp_get_max_threads();
#else
    const int T = 1;
#endif
    /* thread-local y, allocated and zeroed per call by the calling thread before the parallel
     * region, as src/spMV.cpp:146-153 does */
    double **lr = (double **)malloc(sizeof(double *) * (size_t)T);
    double **li = (double **)malloc(sizeof(double *) * (size_t)T);
    for (int q = 0; q < T; ++q) {
        lr[q] = (double *)malloc(sizeof(double) * (size_t)n);
        li[q] = (double *)malloc(sizeof(double) * (size_t)n);
        memset(lr[q], 0, sizeof(double) * (size_t)n);
        memset(li[q], 0, sizeof(double) * (size_t)n);
    }
#pragma omp parallel num_threads(T)
    {
#ifdef _OPENMP
        const int me = omp_get_thread_num();
#else
        const int me = 0;
#endif
        double *a = lr[me], *b = li[me];
#pragma omp for schedule(static)
        for (int64_t q = 0; q < ntask; ++q) {
            const int32_t k = tk[q];
            const int64_t d = off[k], L = len_of(n, off[k]);
            const int64_t s0 = ts[q], s1 = s0 + tile < L ? s0 + tile : L;
            const double *vr = re + start[k], *vi = im + start[k];
            /* element j of diagonal d: row j (d >= 0) or j - d (d < 0), column j + d or j */
            const int64_t ry = d >= 0 ? 0 : -d, cx = d >= 0 ? d : 0;
            double *__restrict__ ya = a + ry, *__restrict__ yb = b + ry;
            const double *__restrict__ pr = xr + cx, *__restrict__ pi = xi + cx;
            for (int64_t j = s0; j < s1; ++j) {
                ya[j] += vr[j] * pr[j] - vi[j] * pi[j];
                yb[j] += vr[j] * pi[j] + vi[j] * pr[j];
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double sr = 0.0, si = 0.0;
        for (int q = 0; q < T; ++q) {
            sr += lr[q][i];
            si += li[q][i];
        }
        yr[i] = sr;
        yi[i] = si;
    }
    for (int q = 0; q < T; ++q) {
        free(lr[q]);
        free(li[q]);
    }
    free(lr);
    free(li);
    free(tk);
    free(ts);
    free(start);
}

/* psi <- sum_{k=0..m} (-i dt H)^k / k! psi per sub-step, `steps` sub-steps of dt each (the
 * reference's rule with dt the sub-step), in place on psir / psii. */
void diaq_timing_ham_sim(int64_t n, int32_t nd, const int32_t *off, const double *re, const double *im,
                         double *psir, double *psii, double dt, int64_t steps, int32_t m) {
    double *buf = (double *)malloc(sizeof(double) * (size_t)n * 4);
    double *tr = buf, *ti = buf + n, *wr = buf + 2 * n, *wi = buf + 3 * n;
    for (int64_t st = 0; st < steps; ++st) {
        memcpy(tr, psir, sizeof(double) * (size_t)n);
        memcpy(ti, psii, sizeof(double) * (size_t)n);
        for (int32_t k = 1; k <= m; ++k) {
            diaq_timing_spmv(n, nd, off, re, im, tr, ti, wr, wi);
            const double scale = dt / (double)k;
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                tr[i] = wi[i] * scale;
                ti[i] = -wr[i] * scale;
                psir[i] += tr[i];
                psii[i] += ti[i];
            }
        }
    }
    free(buf);
}
