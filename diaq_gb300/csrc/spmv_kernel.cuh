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

// ---- zero-tile mask --------------------------------------------------------------------------------
// One bit per diagonal and 32-row tile: bit t of word w of diagonal j is set when rows
// 32 (32 w + t) .. 32 (32 w + t) + 31 of diagonal j hold a nonzero value (real or imaginary part),
// word (j, w) at mask[j * tile_mask_words(rows) + w].  Kernels whose warps cover aligned 32-row
// tiles skip a clear tile whole -- no matrix load, no state window, no multiply-adds.  In
// Pauli-sum Hamiltonians most off-diagonal tiles are zero: the hopping term of qubits k, k+1
// fills a quarter of the rows of its diagonal, in runs of 2^k rows.  Leaving out terms a * x
// with a == 0 changes no finite sum (up to the sign of a zero result).
inline int64_t tile_mask_words(int64_t rows) { return (rows + 1023) / 1024; }
// Fill the mask of A (tile_mask_words(A.rows) * A.nd words) on stream s.
int build_tile_mask(const Matrix &A, uint32_t *mask, cudaStream_t s);
// A's own mask, built (and waited for) on first use after its values were last written; NULL when
// it cannot be had now (s is being captured into a graph, or allocation failed): visit every tile.
const uint32_t *cached_tile_mask(const Matrix &A, cudaStream_t s);
// A's mask if it is built and current (never builds, never allocates), else NULL.
const uint32_t *existing_tile_mask(const Matrix &A, cudaStream_t s);

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

// Asks L2 for the values one diagonal holds in a block's rows: one bulk prefetch per plane and
// run of live 32-row tiles among the block's tiles from row row0 (mask bits `bits`, bit j = tile
// j), clipped to the stored rows [lo, hi) widened to whole tiles.  Tile starts are 128-byte
// aligned in every plane (base is a multiple of 32 values), and the widened ends stay inside the
// allocation (a guard of 32 values before the first diagonal and after the last).  The
// interleaved kernels (256 rows per block) use it; in the planar kernel below and the float-pair
// SpMV (1,024 rows per block, up to 8 KB per diagonal and plane ahead) it measured slower on the
// 20-qubit chain -- one-state Horner evolution 2,106 -> 1,693 states x steps/s, float-pair SpMV
// 99 -> 132 us -- and is not called there.  for_live_runs calls f(a, b) for each such run of rows.
template <class F>
__device__ __forceinline__ void for_live_runs(uint32_t bits, int64_t row0, int64_t lo, int64_t hi, F &&f) {
    while (bits) {
        const int j = __ffs(bits) - 1;
        const uint32_t run = bits >> j;
        const int len = run == 0xffffffffu ? 32 : __ffs(~run) - 1;   // live tiles j .. j + len - 1
        bits = len + j >= 32 ? 0u : bits & ~(((1u << len) - 1u) << j);
        const int64_t a = max(row0 + 32 * j, lo & ~(int64_t)31);
        const int64_t b = min(row0 + 32 * (int64_t)(j + len), (hi + 31) & ~(int64_t)31);
        if (a < b) f(a, b);
    }
}
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
template <typename T>
__device__ __forceinline__ void prefetch_tiles_l2(const T *are, const T *aim, int64_t base, int64_t lo, int64_t hi,
                                                  uint32_t bits, int64_t row0) {
    for_live_runs(bits, row0, lo, hi, [&](int64_t a, int64_t b) {
        const uint32_t bytes = (uint32_t)(b - a) * (uint32_t)sizeof(T);
        prefetch_l2(are + base + a, bytes);
        prefetch_l2(aim + base + a, bytes);
    });
}

// Mask bits of the `tiles` (1 .. 32) tiles from row row0 in the 1024-row mask word w.
__device__ __forceinline__ uint32_t block_tile_bits(uint32_t w, int64_t row0, int tiles) {
    return tiles >= 32 ? w : (w >> ((row0 >> 5) & 31)) & ((1u << tiles) - 1u);
}

// nrhs states in nchunk chunks of up to K, VR rows per thread.  Block b works on chunk
// b % nchunk of row tile b / nchunk: the blocks of one row tile are neighbours in launch order and
// run at the same time, so the matrix tile they all read comes from HBM once and from L2 for the
// other chunks -- the matrix traffic of one launch over all states, with the registers of K.
template <typename T, int K, int VR, class Epi>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_spmv_kernel(const DiagMeta *__restrict__ meta, int nd, const T *__restrict__ are,
                    const T *__restrict__ aim, int64_t rows, const T *__restrict__ xr,
                    const T *__restrict__ xi, int64_t ldx, int nrhs, int nchunk, const uint32_t *__restrict__ tmask,
                    int64_t mw, Epi epi0) {
    constexpr int V = VR;
    constexpr int VB = VR * (int)sizeof(T);
    // per diagonal: offset, row range and the zero-tile mask word of the block's rows in one
    // 16-byte record (rows < 2^31), the value base beside it
    __shared__ int4 sq[kMetaChunk];
    __shared__ int64_t sb[kMetaChunk];
    const int chunk = (int)(blockIdx.x % (unsigned)nchunk);
    const int64_t tile = blockIdx.x / (unsigned)nchunk;
    const int q0 = chunk * K;
    const int kq = min(K, nrhs - q0);
    xr += q0 * ldx;
    xi += q0 * ldx;
    const Epi epi = epi0.shifted(q0);
    const int64_t r0 = (tile * kSpmvThreads + threadIdx.x) * V;
    // a block's 256 V rows (V | 4) lie in one 1024-row mask word; a thread's V rows in one tile
    const int64_t mword = (tile * kSpmvThreads * V) >> 10;
    const int tbit = (int)((r0 >> 5) & 31);
    T accr[K][V], acci[K][V];
#pragma unroll
    for (int q = 0; q < K; ++q)
#pragma unroll
        for (int v = 0; v < V; ++v) accr[q][v] = acci[q][v] = (T)0;

    for (int c0 = 0; c0 < nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, nd - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < cn; i += kSpmvThreads) {
            const DiagMeta m = meta[c0 + i];
            const uint32_t w = tmask ? tmask[(int64_t)(c0 + i) * mw + mword] : 0xffffffffu;
            sq[i] = make_int4(m.off, (int)m.lo, (int)m.hi, (int)w);
            sb[i] = m.base;
        }
        __syncthreads();
        if (r0 >= rows) continue;
#pragma unroll 2
        for (int k = 0; k < cn; ++k) {
            const int4 q = sq[k];
            const int64_t lo = q.y, hi = q.z;
            if (r0 + V <= lo || r0 >= hi || !(((uint32_t)q.w >> tbit) & 1u)) continue;
            const int64_t base = sb[k];
            const int64_t d = q.x;
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

// ---- float variant with L2 prefetch of the matrix and shuffled state windows ----------------------
//
// The register kernel above waits, on every diagonal, for the HBM latency of its matrix vector:
// a warp has one diagonal's loads in flight, and a few dozen warps per SM do not cover the
// latency (profiles: ~30 % of HBM bandwidth, long-scoreboard stalls).  Here lane 0 of each warp
// asks L2 for the warp's 128-row strip of the matrix PF diagonals ahead with one bulk prefetch
// per array (cp.async.bulk.prefetch.L2: no registers, no shared memory), so the loads the warp
// then issues hit L2.
//
// The state windows of a diagonal whose offset is not a multiple of 4 start between 16-byte
// vectors.  The offset is the same for the whole warp, so each lane loads its aligned vector
// and takes the next one from the neighbouring lane (lane 31 loads it): one 16-byte load per
// lane instead of four 4-byte loads.  Strips that a diagonal covers only in part (at the
// matrix's edges) take the element-wise path of the register kernel.
//
// Needs cols % 4 == 0, ldx % 4 == 0 and 16-byte aligned x arrays (checked by the launcher);
// then every x read stays below column cols.

// Ask L2 for [p, p + bytes): p 16-byte aligned, bytes a multiple of 16.  The lines come in with
// evict-first priority, like the streaming loads that will read them, so that they do not push
// the re-read state windows out of L2.
__device__ __forceinline__ void prefetch_l2_bulk(const void *p, unsigned bytes) {
    uint64_t policy;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(policy));
    asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;\n" ::"l"(p), "r"(bytes), "l"(policy)
                 : "memory");
}

// Rows [w0, w0 + 128) of diagonal m, clipped to the diagonal's rows rounded out to 32 values
// (inside the allocation: the first diagonal starts 32 values in and 32 values follow the last;
// base is a multiple of 32, so the clipped range starts on a 128-byte boundary).
__device__ __forceinline__ void prefetch_strip(const DiagMeta &m, int64_t w0, const float *are,
                                               const float *aim) {
    const int64_t a = w0 > (m.lo & ~int64_t(31)) ? w0 : (m.lo & ~int64_t(31));
    const int64_t hi32 = (m.hi + 31) & ~int64_t(31);
    const int64_t b = (w0 + 128) < hi32 ? (w0 + 128) : hi32;
    if (a >= b) return;
    prefetch_l2_bulk(are + m.base + a, (unsigned)(b - a) * 4u);
    prefetch_l2_bulk(aim + m.base + a, (unsigned)(b - a) * 4u);
}

// The four values x[c .. c+3] for a warp whose lanes own consecutive 4-row groups, c - s the
// lane's aligned vector (s = c & 3, the same in every lane).
__device__ __forceinline__ void shifted_window(float (&out)[4], const float *aligned_p, int s, int lane) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(aligned_p));
    if (s == 0) {
        out[0] = a.x;
        out[1] = a.y;
        out[2] = a.z;
        out[3] = a.w;
        return;
    }
    float n0 = __shfl_down_sync(0xffffffffu, a.x, 1);
    float n1 = __shfl_down_sync(0xffffffffu, a.y, 1);
    float n2 = __shfl_down_sync(0xffffffffu, a.z, 1);
    if (lane == 31) {
        const float4 b = __ldg(reinterpret_cast<const float4 *>(aligned_p + 4));
        n0 = b.x;
        n1 = b.y;
        n2 = b.z;
    }
    if (s == 1) {
        out[0] = a.y;
        out[1] = a.z;
        out[2] = a.w;
        out[3] = n0;
    } else if (s == 2) {
        out[0] = a.z;
        out[1] = a.w;
        out[2] = n0;
        out[3] = n1;
    } else {
        out[0] = a.w;
        out[1] = n0;
        out[2] = n1;
        out[3] = n2;
    }
}

template <int K, int PF, class Epi>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_spmv_pf_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ are,
                       const float *__restrict__ aim, int64_t rows, const float *__restrict__ xr,
                       const float *__restrict__ xi, int64_t ldx, int kq, Epi epi) {
    constexpr int V = 4;
    __shared__ DiagMeta sm[kMetaChunk];
    const int lane = threadIdx.x & 31;
    const int64_t r0 = ((int64_t)blockIdx.x * kSpmvThreads + threadIdx.x) * V;
    const int64_t w0 = r0 - (int64_t)V * lane;  // first row of the warp's 128-row strip
    float accr[K][V], acci[K][V];
#pragma unroll
    for (int q = 0; q < K; ++q)
#pragma unroll
        for (int v = 0; v < V; ++v) accr[q][v] = acci[q][v] = 0.f;

    for (int c0 = 0; c0 < nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, nd - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < cn; i += kSpmvThreads) sm[i] = meta[c0 + i];
        __syncthreads();
        if (w0 >= rows) continue;  // the whole warp is past the last row
        if (PF > 0 && lane == 0)
            for (int k = 0; k < PF && k < cn; ++k) prefetch_strip(sm[k], w0, are, aim);
        for (int k = 0; k < cn; ++k) {
            if (PF > 0 && lane == 0 && k + PF < cn) prefetch_strip(sm[k + PF], w0, are, aim);
            const int64_t lo = sm[k].lo, hi = sm[k].hi;
            if (w0 >= hi || w0 + 32 * V <= lo) continue;  // the same for the whole warp
            const int64_t base = sm[k].base;
            const int64_t c = r0 + sm[k].off;
            if (w0 >= lo && w0 + 32 * V <= hi) {
                // the strip lies inside the diagonal: every lane has 4 valid rows
                float ar[V], ai[V];
                load_vec_stream<float, V>(ar, are + base + r0);
                load_vec_stream<float, V>(ai, aim + base + r0);
                const int s = (int)(c & 3);
                const int64_t ca = c - s;
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    if (q >= kq) break;
                    float xrv[V], xiv[V];
                    shifted_window(xrv, xr + q * ldx + ca, s, lane);
                    shifted_window(xiv, xi + q * ldx + ca, s, lane);
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        accr[q][v] = fmaf(ar[v], xrv[v], accr[q][v]);
                        accr[q][v] = fmaf(-ai[v], xiv[v], accr[q][v]);
                        acci[q][v] = fmaf(ar[v], xiv[v], acci[q][v]);
                        acci[q][v] = fmaf(ai[v], xrv[v], acci[q][v]);
                    }
                }
            } else {
                // edge strip: element-wise, rows outside [lo, hi) (and past the last row) masked
                if (r0 >= rows || r0 + V <= lo || r0 >= hi) continue;
                float ar[V], ai[V];
                load_vec_stream<float, V>(ar, are + base + r0);
                load_vec_stream<float, V>(ai, aim + base + r0);
#pragma unroll
                for (int v = 0; v < V; ++v)
                    if (r0 + v < lo || r0 + v >= hi) ar[v] = ai[v] = 0.f;
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    if (q >= kq) break;
                    const float *pxr = xr + q * ldx + c, *pxi = xi + q * ldx + c;
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const bool ok = (r0 + v >= lo) && (r0 + v < hi);
                        const float xv = ok ? __ldg(pxr + v) : 0.f, yv = ok ? __ldg(pxi + v) : 0.f;
                        accr[q][v] = fmaf(ar[v], xv, accr[q][v]);
                        accr[q][v] = fmaf(-ai[v], yv, accr[q][v]);
                        acci[q][v] = fmaf(ar[v], yv, acci[q][v]);
                        acci[q][v] = fmaf(ai[v], xv, acci[q][v]);
                    }
                }
            }
        }
    }
    if (r0 < rows) epi.template apply<float, K, V>(r0, rows, kq, accr, acci);
}

// Whether the prefetching kernel may run on these state arrays (see its notes).
inline bool pf_kernel_fits(const Matrix &A, const float *xr, const float *xi, int64_t ldx, int nrhs) {
    return A.cols % 4 == 0 && (nrhs == 1 || ldx % 4 == 0) && (reinterpret_cast<uintptr_t>(xr) & 15) == 0 &&
           (reinterpret_cast<uintptr_t>(xi) & 15) == 0;
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
    int pipe = 0;  // kernel variant: 0 registers; float kernels with 4 rows per thread: 1 cp.async pipeline,
                   // shuffled windows with L2 prefetch 4 (2) or 8 (3) diagonals ahead or none (4)
};

template <typename T, int K, class Epi, int VR, int... More>
void launch_vr(int vr, const Matrix &A, const T *xr, const T *xi, int64_t ldx, int nrhs, int nchunk,
               const Epi &e, cudaStream_t s, const uint32_t *tmask) {
    if constexpr (sizeof...(More) > 0) {
        if (vr != VR) {
            launch_vr<T, K, Epi, More...>(vr, A, xr, xi, ldx, nrhs, nchunk, e, s, tmask);
            return;
        }
    }
    dia_spmv_kernel<T, K, VR, Epi><<<spmv_blocks(A.rows, VR) * (unsigned)nchunk, kSpmvThreads, 0, s>>>(
        A.d_meta, A.nd, (const T *)A.re, (const T *)A.im, A.rows, xr, xi, ldx, nrhs, nchunk, tmask,
        tile_mask_words(A.rows), e);
}

// One launch over all right-hand sides, in chunks of up to cfg.kmax (<= 8) states per block
// (the kernel instantiated for 1, 2, 4 or 8 states, unused slots of the last chunk masked); the
// chunks of a row tile run side by side (see dia_spmv_kernel).  VRs lists the rows-per-thread
// variants compiled for this epilogue (the first is the default).  Epi must offer
// `shifted(q0)` on host and device, the same epilogue for right-hand sides q0.. .  tmask: A's
// zero-tile mask (build_tile_mask), or NULL to visit every tile.
template <typename T, class Epi, int... VRs>
int launch_dia_spmv_rhs_cfg(const Matrix &A, const T *xr, const T *xi, int64_t ldx, int nrhs, Epi epi,
                            cudaStream_t s, SpmvCfg cfg, const uint32_t *tmask = nullptr) {
    if (A.rows == 0 || nrhs <= 0) return DIAQ_OK;
    int k = cfg.kmax >= 8 ? 8 : cfg.kmax >= 4 ? 4 : cfg.kmax >= 2 ? 2 : 1;
    while (k > 1 && k / 2 >= nrhs) k /= 2;  // no wider than the states need
    const int vr = cfg.vr > 0 ? cfg.vr : VecOf<T>::V;
    const int nchunk = (nrhs + k - 1) / k;
    if ((uint64_t)spmv_blocks(A.rows, vr) * (uint64_t)nchunk > 0x7fffffffull)
        return set_error(DIAQ_ERR_UNSUPPORTED, "spmv: too many row tiles x state chunks for one launch");
    if (k == 8)
        launch_vr<T, 8, Epi, VRs...>(vr, A, xr, xi, ldx, nrhs, nchunk, epi, s, tmask);
    else if (k == 4)
        launch_vr<T, 4, Epi, VRs...>(vr, A, xr, xi, ldx, nrhs, nchunk, epi, s, tmask);
    else if (k == 2)
        launch_vr<T, 2, Epi, VRs...>(vr, A, xr, xi, ldx, nrhs, nchunk, epi, s, tmask);
    else
        launch_vr<T, 1, Epi, VRs...>(vr, A, xr, xi, ldx, nrhs, nchunk, epi, s, tmask);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// The shuffled-window float kernel over the states in chunks of up to kmax; variant 2 / 3
// prefetches the matrix 4 / 8 diagonals ahead, variant 4 does not prefetch.  Falls back to the
// register kernel (4 rows per thread) where pf_kernel_fits does not hold.
template <int K, class Epi>
void launch_pf_k(int variant, const Matrix &A, const float *xr, const float *xi, int64_t ldx, int kq, const Epi &e,
                 cudaStream_t s) {
    const unsigned g = spmv_blocks(A.rows, 4);
    const float *are = (const float *)A.re, *aim = (const float *)A.im;
    if (variant == 3)
        dia_spmv_pf_kernel<K, 8, Epi><<<g, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, are, aim, A.rows, xr, xi, ldx, kq, e);
    else if (variant == 4)
        dia_spmv_pf_kernel<K, 0, Epi><<<g, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, are, aim, A.rows, xr, xi, ldx, kq, e);
    else
        dia_spmv_pf_kernel<K, 4, Epi><<<g, kSpmvThreads, 0, s>>>(A.d_meta, A.nd, are, aim, A.rows, xr, xi, ldx, kq, e);
}

template <class Epi>
int launch_dia_spmv_pf(const Matrix &A, const float *xr, const float *xi, int64_t ldx, int nrhs, Epi epi,
                       cudaStream_t s, int kmax, int variant, int *launches) {
    if (A.rows == 0 || nrhs <= 0) return DIAQ_OK;
    if (!pf_kernel_fits(A, xr, xi, ldx, nrhs)) {
        ++*launches;
        return launch_dia_spmv_rhs_cfg<float, Epi, 4>(A, xr, xi, ldx, nrhs, epi, s, SpmvCfg{kmax, 4, 0});
    }
    kmax = kmax >= 8 ? 8 : kmax >= 4 ? 4 : kmax >= 2 ? 2 : 1;
    int q0 = 0;
    while (q0 < nrhs) {
        const int left = nrhs - q0;
        const int kq = left < kmax ? left : kmax;
        const float *pxr = xr + q0 * ldx, *pxi = xi + q0 * ldx;
        const Epi e = epi.shifted(q0);
        if (kq > 4)
            launch_pf_k<8, Epi>(variant, A, pxr, pxi, ldx, kq, e, s);
        else if (kq > 2)
            launch_pf_k<4, Epi>(variant, A, pxr, pxi, ldx, kq, e, s);
        else if (kq == 2)
            launch_pf_k<2, Epi>(variant, A, pxr, pxi, ldx, kq, e, s);
        else
            launch_pf_k<1, Epi>(variant, A, pxr, pxi, ldx, kq, e, s);
        q0 += kq;
        ++*launches;
    }
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// The default shape: 8 states per launch, 16-byte rows per thread.
template <typename T, class Epi>
int launch_dia_spmv_rhs(const Matrix &A, const T *xr, const T *xi, int64_t ldx, int nrhs, Epi epi,
                        cudaStream_t s) {
    return launch_dia_spmv_rhs_cfg<T, Epi, VecOf<T>::V>(A, xr, xi, ldx, nrhs, epi, s, SpmvCfg{},
                                                         cached_tile_mask(A, s));
}

template <typename T>
struct EpiStoreRhs : EpiStore<T> {
    __host__ __device__ EpiStoreRhs shifted(int q0) const {
        EpiStoreRhs e = *this;
        e.yr += q0 * this->ldy;
        e.yi += q0 * this->ldy;
        return e;
    }
};

template <typename T>
struct EpiTaylorRhs : EpiTaylor<T> {
    __host__ __device__ EpiTaylorRhs shifted(int q0) const {
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
