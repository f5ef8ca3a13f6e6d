// The diagonal-sparse SpMV kernel (y = A x for up to K right-hand sides at once), shared by the
// plain SpMV entry points and the fused time-evolution terms, which differ only in the epilogue.
//
// Work split: thread t of block b owns the V consecutive rows r0 = (b*256 + t)*V .. r0+V-1
// (V = 2 doubles or 4 floats = one 16-byte vector).  For every diagonal (metadata staged in
// shared memory in chunks), the thread loads the V matrix values of its rows as one aligned
// 16-byte vector per array (the row-phase aligned layout makes base + r0 a multiple of V), so a
// warp streams 512 contiguous bytes per array per diagonal: fully coalesced.  x is read at
// columns r0+d .. r0+d+V-1 -- as one vector when d is a multiple of V, else element by element --
// through L1/L2, where the reuse across diagonals and neighbouring blocks lives (the state
// vector of a 2^20-row problem is 16 MB, L2-resident on GB300).  Each row's sum runs over the
// diagonals in slot order with fused multiply-adds; the epilogue functor gets the V sums per
// right-hand side.
#pragma once

#include "diaq_internal.cuh"

namespace diaq_gb300 {

constexpr int kSpmvThreads = 256;
constexpr int kMetaChunk = 256;

template <typename T>
struct VecOf;
template <>
struct VecOf<double> {
    using type = double2;
    static constexpr int V = 2;
};
template <>
struct VecOf<float> {
    using type = float4;
    static constexpr int V = 4;
};

template <typename T>
__device__ __forceinline__ void load_vec(T (&dst)[VecOf<T>::V], const T *p) {
    using VT = typename VecOf<T>::type;
    const VT v = __ldg(reinterpret_cast<const VT *>(p));
    if constexpr (VecOf<T>::V == 2) {
        dst[0] = v.x;
        dst[1] = v.y;
    } else {
        dst[0] = v.x;
        dst[1] = v.y;
        dst[2] = v.z;
        dst[3] = v.w;
    }
}

// Matrix values stream once: evict them first from L2, keeping x resident.
template <typename T>
__device__ __forceinline__ void load_vec_stream(T (&dst)[VecOf<T>::V], const T *p) {
    using VT = typename VecOf<T>::type;
    const VT v = __ldcs(reinterpret_cast<const VT *>(p));
    if constexpr (VecOf<T>::V == 2) {
        dst[0] = v.x;
        dst[1] = v.y;
    } else {
        dst[0] = v.x;
        dst[1] = v.y;
        dst[2] = v.z;
        dst[3] = v.w;
    }
}

__device__ __forceinline__ bool aligned16(const void *p) {
    return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

template <typename T, int K, class Epi>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_spmv_kernel(const DiagMeta *__restrict__ meta, int nd, const T *__restrict__ are,
                    const T *__restrict__ aim, int64_t rows, const T *__restrict__ xr,
                    const T *__restrict__ xi, int64_t ldx, int kq, Epi epi) {
    constexpr int V = VecOf<T>::V;
    __shared__ DiagMeta sm[kMetaChunk];
    const int64_t r0 = ((int64_t)blockIdx.x * kSpmvThreads + threadIdx.x) * V;
    T accr[K][V], acci[K][V];
#pragma unroll
    for (int q = 0; q < K; ++q)
#pragma unroll
        for (int v = 0; v < V; ++v) accr[q][v] = acci[q][v] = (T)0;

    for (int c0 = 0; c0 < nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, nd - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < cn; i += kSpmvThreads) sm[i] = meta[c0 + i];
        __syncthreads();
        if (r0 >= rows) continue;
#pragma unroll 2
        for (int k = 0; k < cn; ++k) {
            const int64_t lo = sm[k].lo, hi = sm[k].hi;
            if (r0 + V <= lo || r0 >= hi) continue;
            const int64_t base = sm[k].base;
            const int64_t d = sm[k].off;
            T ar[V], ai[V];
            load_vec_stream<T>(ar, are + base + r0);
            load_vec_stream<T>(ai, aim + base + r0);
            const bool full = (r0 >= lo) && (r0 + V <= hi);
            if (!full) {
#pragma unroll
                for (int v = 0; v < V; ++v)
                    if (r0 + v < lo || r0 + v >= hi) ar[v] = ai[v] = (T)0;
            }
            const int64_t c = r0 + d;
#pragma unroll
            for (int q = 0; q < K; ++q) {
                if (q >= kq) break;
                const T *pxr = xr + q * ldx + c;
                const T *pxi = xi + q * ldx + c;
                T xrv[V], xiv[V];
                if (full && aligned16(pxr) && aligned16(pxi)) {
                    load_vec<T>(xrv, pxr);
                    load_vec<T>(xiv, pxi);
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const bool ok = (r0 + v >= lo) && (r0 + v < hi);
                        xrv[v] = ok ? __ldg(pxr + v) : (T)0;
                        xiv[v] = ok ? __ldg(pxi + v) : (T)0;
                    }
                }
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    accr[q][v] = fma(ar[v], xrv[v], accr[q][v]);
                    accr[q][v] = fma(-ai[v], xiv[v], accr[q][v]);
                    acci[q][v] = fma(ar[v], xiv[v], acci[q][v]);
                    acci[q][v] = fma(ai[v], xrv[v], acci[q][v]);
                }
            }
        }
    }
    if (r0 < rows) epi.template apply<T, K, V>(r0, rows, kq, accr, acci);
}

// Store y = A x.
template <typename T>
struct EpiStore {
    T *yr, *yi;
    int64_t ldy;
    template <typename U, int K, int V>
    __device__ __forceinline__ void apply(int64_t r0, int64_t rows, int kq, U (&ar)[K][V], U (&ai)[K][V]) const {
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (q >= kq) break;
            T *pr = yr + q * ldy + r0, *pi = yi + q * ldy + r0;
            if (r0 + V <= rows && aligned16(pr) && aligned16(pi)) {
                using VT = typename VecOf<T>::type;
                VT a, b;
                if constexpr (V == 2) {
                    a = VT{ar[q][0], ar[q][1]};
                    b = VT{ai[q][0], ai[q][1]};
                } else {
                    a = VT{ar[q][0], ar[q][1], ar[q][2], ar[q][3]};
                    b = VT{ai[q][0], ai[q][1], ai[q][2], ai[q][3]};
                }
                *reinterpret_cast<VT *>(pr) = a;
                *reinterpret_cast<VT *>(pi) = b;
            } else {
#pragma unroll
                for (int v = 0; v < V; ++v)
                    if (r0 + v < rows) {
                        pr[v] = ar[q][v];
                        pi[v] = ai[q][v];
                    }
            }
        }
    }
};

// One Taylor term of the reference's time evolution (src/spHamSim_gpu_all_fused.cu:206-229):
// term = (-i * scale) * (A term_in), i.e. (re, im) = (s_im * scale, -s_re * scale); acc += term.
// With init set, acc = init + term instead (the first term of a step starts the sum from the
// state itself, saving the copy).  Vectors and accumulator of type T.
template <typename T>
struct EpiTaylor {
    T *tr, *ti;      // term out
    T *accr, *acci;  // running sum
    const T *initr, *initi;
    int64_t ld;
    T scale;
    template <typename U, int K, int V>
    __device__ __forceinline__ void apply(int64_t r0, int64_t rows, int kq, U (&sr)[K][V], U (&si)[K][V]) const {
#pragma unroll
        for (int q = 0; q < K; ++q)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int64_t r = r0 + v;
                if (q < kq && r < rows) {
                    const int64_t i = q * ld + r;
                    const T a = sr[q][v], b = si[q][v];
                    const T nr = b * scale, ni = -a * scale;
                    tr[i] = nr;
                    ti[i] = ni;
                    if (initr) {
                        accr[i] = initr[i] + nr;
                        acci[i] = initi[i] + ni;
                    } else {
                        accr[i] += nr;
                        acci[i] += ni;
                    }
                }
            }
    }
};

inline unsigned spmv_blocks(int64_t rows, int V) {
    const int64_t per = (int64_t)kSpmvThreads * V;
    return (unsigned)((rows + per - 1) / per);
}

// Launch over the right-hand sides in chunks of up to 8 (one matrix read per chunk, the kernel
// instantiated for 1, 2, 4 or 8 with the unused slots masked); Epi must offer `shifted(q0)`, the
// same epilogue for right-hand sides q0.. .
template <typename T, class Epi>
int launch_dia_spmv_rhs(const Matrix &A, const T *xr, const T *xi, int64_t ldx, int nrhs, Epi epi,
                        cudaStream_t s) {
    constexpr int V = VecOf<T>::V;
    if (A.rows == 0 || nrhs <= 0) return DIAQ_OK;
    const unsigned grid = spmv_blocks(A.rows, V);
    int q0 = 0;
    while (q0 < nrhs) {
        const int left = nrhs - q0;
        const int kq = left < 8 ? left : 8;  // states in this launch; the matrix is read once for them
        const T *pxr = xr + q0 * ldx, *pxi = xi + q0 * ldx;
        const Epi e = epi.shifted(q0);
        if (kq > 4)
            dia_spmv_kernel<T, 8, Epi><<<grid, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, (const T *)A.re, (const T *)A.im,
                                                                     A.rows, pxr, pxi, ldx, kq, e);
        else if (kq > 2)
            dia_spmv_kernel<T, 4, Epi><<<grid, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, (const T *)A.re, (const T *)A.im,
                                                                     A.rows, pxr, pxi, ldx, kq, e);
        else if (kq == 2)
            dia_spmv_kernel<T, 2, Epi><<<grid, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, (const T *)A.re, (const T *)A.im,
                                                                     A.rows, pxr, pxi, ldx, kq, e);
        else
            dia_spmv_kernel<T, 1, Epi><<<grid, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, (const T *)A.re, (const T *)A.im,
                                                                     A.rows, pxr, pxi, ldx, kq, e);
        q0 += kq;
    }
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

template <typename T>
struct EpiStoreRhs : EpiStore<T> {
    EpiStoreRhs shifted(int q0) const {
        EpiStoreRhs e = *this;
        e.yr += q0 * this->ldy;
        e.yi += q0 * this->ldy;
        return e;
    }
};

template <typename T>
struct EpiTaylorRhs : EpiTaylor<T> {
    EpiTaylorRhs shifted(int q0) const {
        EpiTaylorRhs e = *this;
        const int64_t o = q0 * this->ld;
        e.tr += o;
        e.ti += o;
        e.accr += o;
        e.acci += o;
        if (e.initr) {
            e.initr += o;
            e.initi += o;
        }
        return e;
    }
};

}  // namespace diaq_gb300
