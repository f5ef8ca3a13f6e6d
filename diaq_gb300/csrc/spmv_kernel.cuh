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

// VR consecutive values of T as one aligned vector load (VR * sizeof(T) bytes).
template <typename T, int VR>
struct Vec;
template <>
struct Vec<double, 2> {
    using type = double2;
};
template <>
struct Vec<double, 1> {
    using type = double;
};
template <>
struct Vec<float, 4> {
    using type = float4;
};
template <>
struct Vec<float, 2> {
    using type = float2;
};
template <>
struct Vec<float, 1> {
    using type = float;
};

// The widest vector: 16 bytes.
template <typename T>
struct VecOf {
    static constexpr int V = 16 / sizeof(T);
    using type = typename Vec<T, V>::type;
};

template <typename VT, typename T, int VR>
__device__ __forceinline__ void unpack(T (&dst)[VR], const VT &v) {
    if constexpr (VR == 1) {
        dst[0] = v;
    } else if constexpr (VR == 2) {
        dst[0] = v.x;
        dst[1] = v.y;
    } else {
        dst[0] = v.x;
        dst[1] = v.y;
        dst[2] = v.z;
        dst[3] = v.w;
    }
}

template <typename T, int VR = VecOf<T>::V>
__device__ __forceinline__ void load_vec(T (&dst)[VR], const T *p) {
    using VT = typename Vec<T, VR>::type;
    unpack<VT, T, VR>(dst, __ldg(reinterpret_cast<const VT *>(p)));
}

// Matrix values stream once: evict them first from L2, keeping x resident.
template <typename T, int VR = VecOf<T>::V>
__device__ __forceinline__ void load_vec_stream(T (&dst)[VR], const T *p) {
    using VT = typename Vec<T, VR>::type;
    unpack<VT, T, VR>(dst, __ldcs(reinterpret_cast<const VT *>(p)));
}

template <int BYTES>
__device__ __forceinline__ bool aligned_to(const void *p) {
    return (reinterpret_cast<uintptr_t>(p) & (uintptr_t)(BYTES - 1)) == 0;
}
__device__ __forceinline__ bool aligned16(const void *p) { return aligned_to<16>(p); }

// K states (kq of them live), VR rows per thread.
template <typename T, int K, int VR, class Epi>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_spmv_kernel(const DiagMeta *__restrict__ meta, int nd, const T *__restrict__ are,
                    const T *__restrict__ aim, int64_t rows, const T *__restrict__ xr,
                    const T *__restrict__ xi, int64_t ldx, int kq, Epi epi) {
    constexpr int V = VR;
    constexpr int VB = VR * (int)sizeof(T);
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
            load_vec_stream<T, V>(ar, are + base + r0);
            load_vec_stream<T, V>(ai, aim + base + r0);
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
                if (full && aligned_to<VB>(pxr) && aligned_to<VB>(pxi)) {
                    load_vec<T, V>(xrv, pxr);
                    load_vec<T, V>(xiv, pxi);
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
            if (V > 1 && r0 + V <= rows && aligned_to<V * sizeof(T)>(pr) && aligned_to<V * sizeof(T)>(pi)) {
                using VT = typename Vec<T, V>::type;
                VT a, b;
                if constexpr (V == 2) {
                    a = VT{ar[q][0], ar[q][1]};
                    b = VT{ai[q][0], ai[q][1]};
                } else if constexpr (V == 4) {
                    a = VT{ar[q][0], ar[q][1], ar[q][2], ar[q][3]};
                    b = VT{ai[q][0], ai[q][1], ai[q][2], ai[q][3]};
                }
                if constexpr (V > 1) {
                    *reinterpret_cast<VT *>(pr) = a;
                    *reinterpret_cast<VT *>(pi) = b;
                }
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

// Launch shape of the SpMV family: at most kmax states per launch (the matrix is read once per
// launch), vr rows per thread (the tile of a block is 256 * vr rows).  vr = 0 picks the widest
// 16-byte vector.
struct SpmvCfg {
    int kmax = 8;
    int vr = 0;
    int pipe = 0;  // 1: the cp.async-pipelined float kernel (4 rows per thread)
};

template <typename T, int K, class Epi, int VR, int... More>
void launch_vr(int vr, const Matrix &A, const T *xr, const T *xi, int64_t ldx, int kq, const Epi &e,
               cudaStream_t s) {
    if constexpr (sizeof...(More) > 0) {
        if (vr != VR) {
            launch_vr<T, K, Epi, More...>(vr, A, xr, xi, ldx, kq, e, s);
            return;
        }
    }
    dia_spmv_kernel<T, K, VR, Epi><<<spmv_blocks(A.rows, VR), kSpmvThreads, 0, s>>>(
        A.d_meta, A.nd, (const T *)A.re, (const T *)A.im, A.rows, xr, xi, ldx, kq, e);
}

// Launch over the right-hand sides in chunks of up to cfg.kmax (<= 8; one matrix read per chunk,
// the kernel instantiated for 1, 2, 4 or 8 states with the unused slots masked).  VRs lists the
// rows-per-thread variants compiled for this epilogue (the first is the default).  Epi must
// offer `shifted(q0)`, the same epilogue for right-hand sides q0.. .
template <typename T, class Epi, int... VRs>
int launch_dia_spmv_rhs_cfg(const Matrix &A, const T *xr, const T *xi, int64_t ldx, int nrhs, Epi epi,
                            cudaStream_t s, SpmvCfg cfg) {
    if (A.rows == 0 || nrhs <= 0) return DIAQ_OK;
    const int kmax = cfg.kmax >= 8 ? 8 : cfg.kmax >= 4 ? 4 : cfg.kmax >= 2 ? 2 : 1;
    const int vr = cfg.vr > 0 ? cfg.vr : VecOf<T>::V;
    int q0 = 0;
    while (q0 < nrhs) {
        const int left = nrhs - q0;
        const int kq = left < kmax ? left : kmax;
        const T *pxr = xr + q0 * ldx, *pxi = xi + q0 * ldx;
        const Epi e = epi.shifted(q0);
        if (kq > 4)
            launch_vr<T, 8, Epi, VRs...>(vr, A, pxr, pxi, ldx, kq, e, s);
        else if (kq > 2)
            launch_vr<T, 4, Epi, VRs...>(vr, A, pxr, pxi, ldx, kq, e, s);
        else if (kq == 2)
            launch_vr<T, 2, Epi, VRs...>(vr, A, pxr, pxi, ldx, kq, e, s);
        else
            launch_vr<T, 1, Epi, VRs...>(vr, A, pxr, pxi, ldx, kq, e, s);
        q0 += kq;
    }
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// The default shape: 8 states per launch, 16-byte rows per thread.
template <typename T, class Epi>
int launch_dia_spmv_rhs(const Matrix &A, const T *xr, const T *xi, int64_t ldx, int nrhs, Epi epi,
                        cudaStream_t s) {
    return launch_dia_spmv_rhs_cfg<T, Epi, VecOf<T>::V>(A, xr, xi, ldx, nrhs, epi, s, SpmvCfg{});
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
