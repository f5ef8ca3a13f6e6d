// Complex128 SpMV on the FP32 pipes: DIAQ_C128F2 matrices.
//
// GB300 issues FP64 fused multiply-adds at 1/58 of its FP32 rate (0.59 vs 34.6 T/s measured),
// so the float64 SpMV (4 DFMA per stored value) tops out near 2.4 TB/s of matrix traffic -- FP64
// issue, not HBM, bounds it.  A DIAQ_C128F2 matrix keeps 16 bytes per complex value, but each
// float64 v as a pair of floats hi = fl32(v), lo = fl32(v - hi) (a 48-bit significand), and the
// kernel accumulates products of such pairs exactly enough on the FP32 pipes:
//   product   p = ah*xh (+ error fma(ah, xh, -p)) + ah*xl + al*xh          (Dekker/Knuth with FMA)
//   sum       (sh, sl) <- TwoSum(sh, p) with the error and the low parts added to sl
// About 12 FP32 operations per real product-accumulate, 48 per complex value, issued as packed
// two-lane instructions over pairs of rows (24 per complex value and row): ~0.7 T complex values/s
// or more, above the ~0.42 T/s at which HBM delivers the 16-byte values.  Relative error ~1e-14 (2^-48 per value plus accumulation): inside the 1e-12 of
// the float64 path's parity bar.  Range: magnitudes in roughly [1e-30, 1e38] keep the full
// precision (the low float must stay normal).
//
// x arrives as float64 and is split once per call (one pass over N values, without float64
// arithmetic: split64_fast); y is written as float64 (hi + lo in double, 2 conversions and 1 add
// per row).
//
// Storage: the layout of the other precisions, the re (im) array holding the hi plane of
// `capacity` floats followed by the lo plane.
#include <algorithm>

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

__device__ __forceinline__ void split64(double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

// split64 kept out of line, for the rare values split64_fast leaves to it.  Inlined, its
// conversions and float64 subtraction are if-converted into the fast path and issue on GB300's
// FP64 pipe for every value, taken or not: the split of x took 18.5 us instead of 8.2.
__device__ __noinline__ void split64_outlined(double v, float &h, float &l) { split64(v, h, l); }

// The split of x with bit operations and float32 arithmetic only.  hi is v truncated to 24
// significant bits (the high word and 3 bits of the low one); lo is the remaining 29 bits ml,
// rounded to 24 bits as 64 a + c (a = ml >> 6 and c = ml & 63 made exact floats by the 2^23
// magic number, one rounding in the fma) and scaled by v's exponent through its exponent field:
// |v - hi - lo| <= 2^-48 |v|, split64's bound.  Exponents where hi or lo would not be a normal
// float (|v| outside about [1e-22, 3e38]) take split64.
__device__ __forceinline__ void split64_fast(double v, float &h, float &l) {
    const uint32_t H = (uint32_t)__double2hiint(v), L = (uint32_t)__double2loint(v);
    const uint32_t e = (H >> 20) & 0x7ffu;
    if (e < 950u || e > 1150u) {
        split64_outlined(v, h, l);
        return;
    }
    const uint32_t sign = H & 0x80000000u;
    h = __uint_as_float(sign | ((e - 896u) << 23) | ((H & 0xfffffu) << 3) | (L >> 29));
    const uint32_t ml = L & 0x1fffffffu;  // lo = ml * 2^(e - 1075), ml < 2^29
    const float fa = __fsub_rn(__uint_as_float(0x4b000000u | (ml >> 6)), 8388608.0f);
    const float fc = __fsub_rn(__uint_as_float(0x4b000000u | (ml & 63u)), 8388608.0f);
    const float f = __fmaf_rn(fa, 64.0f, fc);
    l = ml ? __uint_as_float(sign | (__float_as_uint(f) - ((1075u - e) << 23))) : __uint_as_float(sign);
}

// packed float64 -> hi/lo planes
__global__ void f2_scatter_kernel(const DiagMeta *__restrict__ meta, int nd, const double *__restrict__ sre,
                                  const double *__restrict__ sim, float *__restrict__ re, float *__restrict__ im,
                                  int64_t cap) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        const int64_t len = m.hi - m.lo;
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < len; j += (int64_t)gridDim.x * blockDim.x) {
            const int64_t d = m.base + m.lo + j;
            split64(sre[m.pstart + j], re[d], re[cap + d]);
            split64(sim[m.pstart + j], im[d], im[cap + d]);
        }
    }
}

// hi/lo planes -> packed float64
__global__ void f2_gather_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ re,
                                 const float *__restrict__ im, int64_t cap, double *__restrict__ dre,
                                 double *__restrict__ dim) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        const int64_t len = m.hi - m.lo;
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < len; j += (int64_t)gridDim.x * blockDim.x) {
            const int64_t s = m.base + m.lo + j;
            dre[m.pstart + j] = (double)re[s] + (double)re[cap + s];
            dim[m.pstart + j] = (double)im[s] + (double)im[cap + s];
        }
    }
}

// both float64 vectors of x -> their four hi/lo planes in one launch; vec: x_re and x_im are
// 16-byte aligned, so pairs of values move as double2 -> float2
__global__ void f2_split_pair_kernel(const double *__restrict__ xr, const double *__restrict__ xi, int64_t n, int vec,
                                     float *__restrict__ rh, float *__restrict__ rl, float *__restrict__ ih,
                                     float *__restrict__ il) {
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    int64_t done = 0;
    if (vec) {
        const int64_t n2 = n / 2;
        for (int64_t i = t0; i < n2; i += stride) {
            const double2 a = reinterpret_cast<const double2 *>(xr)[i], b = reinterpret_cast<const double2 *>(xi)[i];
            float h0, l0, h1, l1;
            split64_fast(a.x, h0, l0);
            split64_fast(a.y, h1, l1);
            reinterpret_cast<float2 *>(rh)[i] = make_float2(h0, h1);
            reinterpret_cast<float2 *>(rl)[i] = make_float2(l0, l1);
            split64_fast(b.x, h0, l0);
            split64_fast(b.y, h1, l1);
            reinterpret_cast<float2 *>(ih)[i] = make_float2(h0, h1);
            reinterpret_cast<float2 *>(il)[i] = make_float2(l0, l1);
        }
        done = 2 * n2;
    }
    for (int64_t i = done + t0; i < n; i += stride) {
        split64_fast(xr[i], rh[i], rl[i]);
        split64_fast(xi[i], ih[i], il[i]);
    }
}

// s += a*x for float pairs (see the file comment), two rows at once: TwoProd (ph + the exact
// remainder by FMA) and TwoSum, on the packed two-lane FP32 instructions (__fmul2_rn, __ffma2_rn,
// __fadd2_rn: each lane the scalar operation with its rounding; a - b as a + (-b), which is exact).
// The _rn intrinsics keep the compiler from fusing the product into the sum, which would break
// both identities.  Negate ah and al to subtract.  Against one row per instruction: 101.1 -> 99.5
// us per SpMV on the 20-qubit chain, the same bits.
struct F2P {
    float2 h, l;
};
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ void f2_mac2(F2P &s, float2 ah, float2 al, float2 xh, float2 xl) {
    const float2 ph = __fmul2_rn(ah, xh);
    float2 pl = __ffma2_rn(ah, xh, neg2(ph));
    pl = __ffma2_rn(ah, xl, pl);
    pl = __ffma2_rn(al, xh, pl);
    const float2 t = __fadd2_rn(s.h, ph);
    const float2 bb = __fadd2_rn(t, neg2(s.h));
    const float2 e = __fadd2_rn(__fadd2_rn(s.h, neg2(__fadd2_rn(t, neg2(bb)))), __fadd2_rn(ph, neg2(bb)));
    s.h = t;
    s.l = __fadd2_rn(s.l, __fadd2_rn(e, pl));
}

// y = A x: each thread owns VR = 4 consecutive rows; hi and lo planes are separate SoA arrays, so
// every matrix load is a 16-byte vector of 4 rows.  Strips that lie inside a diagonal read the
// four x planes as aligned vectors shifted across lanes (the x planes are this file's scratch,
// padded to a multiple of 32 values, so the aligned vectors stay inside them; values past column
// cols are read but never used).  Each diagonal's offset, row range and the block's mask word are
// staged as one 16-byte shared-memory record.  (Prefetching the warp's strip of the four matrix
// planes into L2 a few diagonals ahead measured slower on the 20-qubit XXZ chain, 216 against
// 194 us, and was dropped.)

template <int MINB>
__global__ void __launch_bounds__(kSpmvThreads, MINB)
    f2_spmv_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ are,
                   const float *__restrict__ aim, int64_t cap, int64_t rows, const float *__restrict__ xrh,
                   const float *__restrict__ xrl, const float *__restrict__ xih, const float *__restrict__ xil,
                   double *__restrict__ yr, double *__restrict__ yi, const uint32_t *__restrict__ tmask, int64_t mw) {
    constexpr int V = 4;
    __shared__ int4 sq[kMetaChunk];     // offset, lo, hi, mask word (the block's 1024 rows are one word)
    __shared__ int64_t sb[kMetaChunk];  // value base
    const int lane = threadIdx.x & 31;
    const int64_t r0 = ((int64_t)blockIdx.x * kSpmvThreads + threadIdx.x) * V;
    const int64_t w0 = r0 - (int64_t)V * lane;
    F2P sr[V / 2], si[V / 2];   // rows (0, 1) and (2, 3)
#pragma unroll
    for (int v = 0; v < V / 2; ++v) sr[v] = si[v] = F2P{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    for (int c0 = 0; c0 < nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, nd - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < cn; i += kSpmvThreads) {
            const DiagMeta m = meta[c0 + i];
            const uint32_t w = tmask ? tmask[(int64_t)(c0 + i) * mw + blockIdx.x] : 0xffffffffu;
            sq[i] = make_int4(m.off, (int)m.lo, (int)m.hi, (int)w);
            sb[i] = m.base;
        }
        __syncthreads();
        if (w0 >= rows) continue;
        const int wbit = (int)((w0 >> 5) & 31);  // the warp's 128 rows: 4 tiles, bits wbit .. wbit + 3
        for (int k = 0; k < cn; ++k) {
            const int4 q = sq[k];
            const int64_t lo = q.y, hi = q.z;
            const uint32_t mword = (uint32_t)q.w;
            // the same for the whole warp (the windows below are shuffled across its lanes)
            if (w0 >= hi || w0 + 32 * V <= lo || !((mword >> wbit) & 0xfu)) continue;
            const int64_t b = sb[k] + r0, c = r0 + q.x;
            float arh[V], arl[V], aih[V], ail[V];
            float xrhv[V], xrlv[V], xihv[V], xilv[V];
            if (w0 >= lo && w0 + 32 * V <= hi) {
                // an aligned window needs no shuffle: a lane whose tile is zero drops out alone
                if ((q.x & 3) == 0 && !((mword >> ((r0 >> 5) & 31)) & 1u)) continue;
                load_vec_stream<float, V>(arh, are + b);
                load_vec_stream<float, V>(arl, are + cap + b);
                load_vec_stream<float, V>(aih, aim + b);
                load_vec_stream<float, V>(ail, aim + cap + b);
                const int s = (int)(c & 3);
                const int64_t ca = c - s;
                shifted_window(xrhv, xrh + ca, s, lane);
                shifted_window(xrlv, xrl + ca, s, lane);
                shifted_window(xihv, xih + ca, s, lane);
                shifted_window(xilv, xil + ca, s, lane);
            } else {
                if (r0 >= rows || r0 + V <= lo || r0 >= hi) continue;
                load_vec_stream<float, V>(arh, are + b);
                load_vec_stream<float, V>(arl, are + cap + b);
                load_vec_stream<float, V>(aih, aim + b);
                load_vec_stream<float, V>(ail, aim + cap + b);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const bool ok = (r0 + v >= lo) && (r0 + v < hi);
                    xrhv[v] = ok ? __ldg(xrh + c + v) : 0.f;
                    xrlv[v] = ok ? __ldg(xrl + c + v) : 0.f;
                    xihv[v] = ok ? __ldg(xih + c + v) : 0.f;
                    xilv[v] = ok ? __ldg(xil + c + v) : 0.f;
                    if (!ok) arh[v] = arl[v] = aih[v] = ail[v] = 0.f;
                }
            }
#pragma unroll
            for (int v = 0; v < V; v += 2) {
                const float2 rh = make_float2(arh[v], arh[v + 1]), rl = make_float2(arl[v], arl[v + 1]);
                const float2 ih = make_float2(aih[v], aih[v + 1]), il = make_float2(ail[v], ail[v + 1]);
                const float2 xrh2 = make_float2(xrhv[v], xrhv[v + 1]), xrl2 = make_float2(xrlv[v], xrlv[v + 1]);
                const float2 xih2 = make_float2(xihv[v], xihv[v + 1]), xil2 = make_float2(xilv[v], xilv[v + 1]);
                f2_mac2(sr[v / 2], rh, rl, xrh2, xrl2);
                f2_mac2(sr[v / 2], neg2(ih), neg2(il), xih2, xil2);
                f2_mac2(si[v / 2], rh, rl, xih2, xil2);
                f2_mac2(si[v / 2], ih, il, xrh2, xrl2);
            }
        }
    }
    if (r0 >= rows) return;
#pragma unroll
    for (int v = 0; v < V; ++v)
        if (r0 + v < rows) {
            const F2P &a = sr[v / 2], &b = si[v / 2];
            yr[r0 + v] = (double)((v & 1) ? a.h.y : a.h.x) + (double)((v & 1) ? a.l.y : a.l.x);
            yi[r0 + v] = (double)((v & 1) ? b.h.y : b.h.x) + (double)((v & 1) ? b.l.y : b.l.x);
        }
}

__global__ void f2_from_c128_kernel(const DiagMeta *__restrict__ meta, int nd, const double *__restrict__ sre,
                                    const double *__restrict__ sim, float *__restrict__ re, float *__restrict__ im,
                                    int64_t cap) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        for (int64_t r = m.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m.hi; r += (int64_t)gridDim.x * blockDim.x) {
            split64(sre[m.base + r], re[m.base + r], re[cap + m.base + r]);
            split64(sim[m.base + r], im[m.base + r], im[cap + m.base + r]);
        }
    }
}

__global__ void c128_from_f2_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ re,
                                    const float *__restrict__ im, int64_t cap, double *__restrict__ dre,
                                    double *__restrict__ dim) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        for (int64_t r = m.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m.hi; r += (int64_t)gridDim.x * blockDim.x) {
            dre[m.base + r] = (double)re[m.base + r] + (double)re[cap + m.base + r];
            dim[m.base + r] = (double)im[m.base + r] + (double)im[cap + m.base + r];
        }
    }
}

static dim3 f2_grid(const Matrix &M) {
    int64_t maxlen = 1;
    for (const auto &m : M.meta) maxlen = std::max(maxlen, m.hi - m.lo);
    return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>((maxlen + 1023) / 1024, 4 * num_sms())),
                (unsigned)std::min<int64_t>(std::max<int32_t>(M.nd, 1), 65535));
}

int f2_scatter(Matrix &M, const double *re, const double *im, cudaStream_t s) {
    M.tmask_ok = false;
    if (M.nd == 0) return DIAQ_OK;
    f2_scatter_kernel<<<f2_grid(M), 256, 0, s>>>(M.d_meta, M.nd, re, im, (float *)M.re, (float *)M.im, M.capacity);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

int f2_gather(const Matrix &M, double *re, double *im, cudaStream_t s) {
    if (M.nd == 0) return DIAQ_OK;
    f2_gather_kernel<<<f2_grid(M), 256, 0, s>>>(M.d_meta, M.nd, (const float *)M.re, (const float *)M.im, M.capacity, re,
                                                im);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// Same offsets and layout (src and dst planned alike); one precision is C128, the other C128F2.
int f2_convert(const Matrix &src, Matrix &dst, cudaStream_t s) {
    dst.tmask_ok = false;
    if (dst.nd == 0) return DIAQ_OK;
    if (src.prec == DIAQ_C128 && dst.prec == DIAQ_C128F2)
        f2_from_c128_kernel<<<f2_grid(dst), 256, 0, s>>>(src.d_meta, src.nd, (const double *)src.re, (const double *)src.im,
                                                        (float *)dst.re, (float *)dst.im, dst.capacity);
    else if (src.prec == DIAQ_C128F2 && dst.prec == DIAQ_C128)
        c128_from_f2_kernel<<<f2_grid(dst), 256, 0, s>>>(src.d_meta, src.nd, (const float *)src.re, (const float *)src.im,
                                                        src.capacity, (double *)dst.re, (double *)dst.im);
    else
        return set_error(DIAQ_ERR_UNSUPPORTED, "c128f2 matrices convert to and from c128 only");
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

int f2_spmv(const Matrix &A, const double *xr, const double *xi, double *yr, double *yi, cudaStream_t s) {
    if (A.rows == 0) return DIAQ_OK;
    const int64_t n = A.cols;
    const int64_t np = (n + 31) / 32 * 32;  // planes 128-byte aligned: equal alignment for hi and lo
    float *buf = nullptr;
    DQ_CUDA(dev_malloc_async(&buf, sizeof(float) * 4 * (size_t)std::max<int64_t>(np, 32), s));
    float *xrh = buf, *xrl = buf + np, *xih = buf + 2 * np, *xil = buf + 3 * np;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * num_sms()));
    const int vec = ((uintptr_t)xr % 16 == 0) && ((uintptr_t)xi % 16 == 0);
    f2_split_pair_kernel<<<g, 256, 0, s>>>(xr, xi, n, vec, xrh, xrl, xih, xil);
    // four blocks per SM (64 registers): 166.8 us on the 20-qubit chain; three (80 registers)
    // 189 us, five or six spill (252, 339 us)
    f2_spmv_kernel<4><<<spmv_blocks(A.rows, 4), kSpmvThreads, 0, s>>>(A.d_meta, A.nd, (const float *)A.re,
                                                                  (const float *)A.im, A.capacity, A.rows, xrh, xrl,
                                                                  xih, xil, yr, yi, cached_tile_mask(A, s),
                                                                  tile_mask_words(A.rows));
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return cuda_status(e, "f2 spmv", __FILE__, __LINE__);
    return DIAQ_OK;
}

}  // namespace diaq_gb300
