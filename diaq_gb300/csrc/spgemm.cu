// Diagonal-pair SpGEMM C = A B with its structural dry-run on the device.
// Replaces product / product_device / product_cuda (src/spGEMM.cpp:303-538,
// src/spGEMM_gpu.cu:25-161).
//
// Dry-run: every pair (dA, dB) marks dC = dA + dB in a flag array over the whole offset range
// [-(rowsA-1), colsB-1]; an exclusive prefix sum over the flags numbers the marked offsets, so
// compaction yields them ascending and distinct -- a counting sort, exact by construction, the
// set the reference collects in a std::map (src/spGEMM.cpp:346-369).
//
// Numeric pass: the grid is (row tiles of C, diagonals of C).  In row-indexed form
// C[r, dC] = sum_a A[r, dA_a] * B[r + dA_a, dC - dA_a]; the thread owning rows r0..r0+V-1 of
// one C diagonal walks A's slots in order (metadata staged in shared memory), finds B's slot
// for dC - dA through a dense offset->slot map, and accumulates the shifted products -- the
// SpMV access pattern with B's diagonal in place of x.  Pairs of one C diagonal are summed in
// A-slot order, as src/spGEMM_gpu.cu:55-77 and src/spGEMM.cpp:425-493 do.
#include <algorithm>

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

// ---- dry-run -----------------------------------------------------------------------------------
__global__ void mark_pairs_kernel(const int32_t *__restrict__ offA, int ndA, const int32_t *__restrict__ offB,
                                  int ndB, int64_t lo, int64_t hi, uint8_t *__restrict__ flags) {
    const int64_t n = (int64_t)ndA * ndB;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t dc = (int64_t)offA[p / ndB] + offB[p % ndB];
        if (dc >= lo && dc <= hi) flags[dc - lo] = 1;  // benign race: every writer stores 1
    }
}

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;  // flags per thread per block pass
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

// Per tile: number of set flags.
__global__ void count_tiles_kernel(const uint8_t *__restrict__ flags, int64_t n, int32_t *__restrict__ tile_count) {
    __shared__ int red[kScanThreads / 32];
    const int64_t t0 = blockIdx.x * kScanTile;
    int v = 0;
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t j = t0 + (int64_t)i * kScanThreads + threadIdx.x;
        if (j < n) v += flags[j];
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < kScanThreads / 32 ? red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) tile_count[blockIdx.x] = v;
    }
}

// Exclusive scan of the tile counts in one block (loops over chunks); total at [ntiles].
__global__ void scan_tiles_kernel(int32_t *__restrict__ tile_count, int64_t ntiles) {
    __shared__ int32_t buf[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t c0 = 0; c0 < ntiles; c0 += 1024) {
        const int64_t j = c0 + threadIdx.x;
        int32_t v = j < ntiles ? tile_count[j] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
            int32_t add = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += add;
            __syncthreads();
        }
        if (j < ntiles) tile_count[j] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_count[ntiles] = carry;
}

// Write the offsets of the set flags, ascending.
__global__ void compact_kernel(const uint8_t *__restrict__ flags, int64_t n, int64_t lo,
                               const int32_t *__restrict__ tile_base, int32_t *__restrict__ out) {
    __shared__ int32_t buf[kScanThreads];
    const int64_t t0 = blockIdx.x * kScanTile;
    int32_t base = tile_base[blockIdx.x];
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t j = t0 + (int64_t)i * kScanThreads + threadIdx.x;
        const int32_t f = (j < n) ? flags[j] : 0;
        buf[threadIdx.x] = f;
        __syncthreads();
        for (int o = 1; o < kScanThreads; o <<= 1) {
            int32_t add = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += add;
            __syncthreads();
        }
        if (f) out[base + buf[threadIdx.x] - 1] = (int32_t)(j + lo);
        const int32_t chunk_total = buf[kScanThreads - 1];
        __syncthreads();
        base += chunk_total;
    }
}

// Symbolic phase on the device: result offsets (ascending, distinct) to the host vector.
int spgemm_symbolic(const Matrix &A, const Matrix &B, std::vector<int32_t> &offC, cudaStream_t s) {
    if (A.prec == DIAQ_C128F2) return set_error(DIAQ_ERR_UNSUPPORTED, "product: convert a c128f2 matrix to c128 first");
    offC.clear();
    if (A.cols != B.rows) return set_error(DIAQ_ERR_INVALID, "diaQMatrix product_cuda: dimension mismatch.");
    if (A.nd == 0 || B.nd == 0 || A.rows == 0 || B.cols == 0) return DIAQ_OK;
    const int64_t lo = -(A.rows - 1), hi = B.cols - 1;
    const int64_t range = hi - lo + 1;
    const int64_t ntiles = (range + kScanTile - 1) / kScanTile;
    // one scratch allocation: flags | tile counts | offsets A | offsets B | output
    const size_t fbytes = (size_t)((range + 15) / 16 * 16);
    const size_t tbytes = sizeof(int32_t) * (size_t)(ntiles + 1);
    const size_t abytes = sizeof(int32_t) * A.nd, bbytes = sizeof(int32_t) * B.nd;
    const int64_t maxout = std::min<int64_t>((int64_t)A.nd * B.nd, range);
    const size_t obytes = sizeof(int32_t) * (size_t)maxout;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t total = up(fbytes) + up(tbytes) + up(abytes) + up(bbytes) + up(obytes);
    uint8_t *scratch = nullptr;
    DQ_CUDA(dev_malloc_async(&scratch, total, s));
    uint8_t *flags = scratch;
    int32_t *tiles = (int32_t *)(scratch + up(fbytes));
    int32_t *dA = (int32_t *)((uint8_t *)tiles + up(tbytes));
    int32_t *dB = (int32_t *)((uint8_t *)dA + up(abytes));
    int32_t *dout = (int32_t *)((uint8_t *)dB + up(bbytes));
    int st = DIAQ_OK;
    cudaError_t e = cudaMemsetAsync(flags, 0, fbytes, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dA, A.off.data(), abytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dB, B.off.data(), bbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const int64_t pairs = (int64_t)A.nd * B.nd;
        const int grid = (int)std::min<int64_t>((pairs + 255) / 256, 8 * num_sms());
        mark_pairs_kernel<<<grid, 256, 0, s>>>(dA, A.nd, dB, B.nd, lo, hi, flags);
        count_tiles_kernel<<<(unsigned)ntiles, kScanThreads, 0, s>>>(flags, range, tiles);
        scan_tiles_kernel<<<1, 1024, 0, s>>>(tiles, ntiles);
        compact_kernel<<<(unsigned)ntiles, kScanThreads, 0, s>>>(flags, range, lo, tiles, dout);
        e = cudaGetLastError();
    }
    int32_t count = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&count, tiles + ntiles, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && count > 0) {
        offC.resize(count);
        e = cudaMemcpyAsync(offC.data(), dout, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess) st = cuda_status(e, "spgemm dry-run", __FILE__, __LINE__);
    cudaFreeAsync(scratch, s);
    return st;
}

// ---- numeric pass -------------------------------------------------------------------------------
// Pair lists first: for every C diagonal c, the (A slot, B slot) pairs with dA + dB = dC whose
// rows can overlap C's, in A-slot order (the reference's summation order, src/spGEMM.cpp:346-378).
// One thread per C diagonal counts them, the host scans the counts, the same thread writes them.
// The numeric kernel then walks only the pairs of its C diagonal -- an earlier version scanned
// every A diagonal for every C diagonal and row tile (41 candidates for ~2.3 pairs on the
// 20-qubit XXZ H H) and spent half its instructions on that.

__device__ __forceinline__ bool pair_rows(const DiagMeta &ma, const DiagMeta &mb, const DiagMeta &mc, int64_t &lo,
                                          int64_t &hi) {
    // rows r with A valid (ma.lo <= r < ma.hi), B valid (mb.lo <= r + dA < mb.hi), C valid
    lo = max(max(ma.lo, mb.lo - (int64_t)ma.off), mc.lo);
    hi = min(min(ma.hi, mb.hi - (int64_t)ma.off), mc.hi);
    return lo < hi;
}

// fill == nullptr: count the pairs of each C diagonal into cnt; else write them at start[c].
__global__ void spgemm_pairs_kernel(const DiagMeta *__restrict__ mA, int ndA, const DiagMeta *__restrict__ mB,
                                    const int32_t *__restrict__ bslot, int64_t bmin, int64_t bmax,
                                    const DiagMeta *__restrict__ mC, int ndC, int32_t *__restrict__ cnt,
                                    const int64_t *__restrict__ start, int2 *__restrict__ fill) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ndC; c += gridDim.x * blockDim.x) {
        const DiagMeta mc = mC[c];
        int64_t w = fill ? start[c] : 0;
        int32_t n = 0;
        for (int a = 0; a < ndA; ++a) {
            const DiagMeta ma = mA[a];
            const int64_t db = (int64_t)mc.off - ma.off;
            if (db < bmin || db > bmax) continue;
            const int32_t b = bslot[db - bmin];
            if (b < 0) continue;
            int64_t lo, hi;
            if (!pair_rows(ma, mB[b], mc, lo, hi)) continue;
            if (fill) fill[w++] = make_int2(a, b);
            ++n;
        }
        if (!fill) cnt[c] = n;
    }
}

// bit of row r's 32-row tile in diagonal slot j of a zero-tile mask (mw words per diagonal)
__device__ __forceinline__ bool tile_live(const uint32_t *__restrict__ mask, int64_t mw, int j, int64_t r) {
    return (__ldg(mask + (int64_t)j * mw + (r >> 10)) >> ((r >> 5) & 31)) & 1u;
}

// Block (x, y): row tile x of the C diagonals y, y + gridDim.y, ...; thread t owns V rows.  With
// the operands' zero-tile masks (maskA, maskB) a pair is skipped where A's tile or both B tiles
// that its rows read are zero: a product with a zero factor adds nothing.
template <typename T>
__global__ void __launch_bounds__(kSpmvThreads)
    spgemm_numeric_kernel(const DiagMeta *__restrict__ mA, const T *__restrict__ Are, const T *__restrict__ Aim,
                          const DiagMeta *__restrict__ mB, const T *__restrict__ Bre, const T *__restrict__ Bim,
                          const DiagMeta *__restrict__ mC, int ndC, const int64_t *__restrict__ pstart,
                          const int2 *__restrict__ pairs, T *__restrict__ Cre, T *__restrict__ Cim,
                          const uint32_t *__restrict__ maskA, int64_t mwA, const uint32_t *__restrict__ maskB,
                          int64_t mwB) {
    constexpr int V = VecOf<T>::V;
    const int64_t r0 = ((int64_t)blockIdx.x * kSpmvThreads + threadIdx.x) * V;
    for (int c = blockIdx.y; c < ndC; c += gridDim.y) {
        const DiagMeta mc = mC[c];
        if (r0 >= mc.hi || r0 + V <= mc.lo) continue;
        T accr[V], acci[V];
#pragma unroll
        for (int v = 0; v < V; ++v) accr[v] = acci[v] = (T)0;
        const int64_t p1 = pstart[c + 1];
        for (int64_t p = pstart[c]; p < p1; ++p) {
            const int2 ab = pairs[p];
            const DiagMeta ma = mA[ab.x], mb = mB[ab.y];
            int64_t lo, hi;
            pair_rows(ma, mb, mc, lo, hi);
            if (r0 + V <= lo || r0 >= hi) continue;
            if (maskA) {  // r0 .. r0 + V - 1 share one tile (V | 32); their B rows span at most two
                if (!tile_live(maskA, mwA, ab.x, r0)) continue;
                const int64_t b0 = max(r0, lo) + ma.off, b1 = min(r0 + V, hi) - 1 + ma.off;
                if (!tile_live(maskB, mwB, ab.y, b0) && !tile_live(maskB, mwB, ab.y, b1)) continue;
            }
            T ar[V], ai[V], br[V], bi[V];
            load_vec<T, V>(ar, Are + ma.base + r0);
            load_vec<T, V>(ai, Aim + ma.base + r0);
            const bool full = (r0 >= lo) && (r0 + V <= hi);
            const T *pbr = Bre + mb.base + r0 + ma.off;
            const T *pbi = Bim + mb.base + r0 + ma.off;
            if (full && aligned16(pbr)) {
                load_vec<T, V>(br, pbr);
                load_vec<T, V>(bi, pbi);
            } else {
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const bool ok = (r0 + v >= lo) && (r0 + v < hi);
                    br[v] = ok ? __ldg(pbr + v) : (T)0;
                    bi[v] = ok ? __ldg(pbi + v) : (T)0;
                    if (!ok) ar[v] = ai[v] = (T)0;
                }
            }
#pragma unroll
            for (int v = 0; v < V; ++v) {
                accr[v] = fma(ar[v], br[v], accr[v]);
                accr[v] = fma(-ai[v], bi[v], accr[v]);
                acci[v] = fma(ar[v], bi[v], acci[v]);
                acci[v] = fma(ai[v], br[v], acci[v]);
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int64_t r = r0 + v;
            if (r >= mc.lo && r < mc.hi) {
                Cre[mc.base + r] = accr[v];
                Cim[mc.base + r] = acci[v];
            }
        }
    }
}

int spgemm_numeric(const Matrix &A, const Matrix &B, Matrix &C, cudaStream_t s) {
    if (A.prec == DIAQ_C128F2) return set_error(DIAQ_ERR_UNSUPPORTED, "product: convert a c128f2 matrix to c128 first");
    if (A.cols != B.rows || C.rows != A.rows || C.cols != B.cols)
        return set_error(DIAQ_ERR_INVALID, "diaQMatrix product_cuda: dimension mismatch.");
    if (A.prec != B.prec || A.prec != C.prec)
        return set_error(DIAQ_ERR_INVALID, "product: operands must have the same precision");
    C.tmask_ok = false;  // new values
    if (C.nd == 0 || C.rows == 0) return DIAQ_OK;
    // dense offset -> slot map of B
    const int64_t bmin = -(B.rows - 1), bmax = B.cols - 1;
    const int64_t span = bmax - bmin + 1;
    std::vector<int32_t> map((size_t)span, -1);
    for (int32_t k = 0; k < B.nd; ++k) map[(size_t)(B.off[k] - bmin)] = k;
    // scratch: B map, per-C counts, per-C starts
    const size_t mbytes = sizeof(int32_t) * (size_t)span, cbytes = sizeof(int32_t) * (size_t)C.nd,
                 sbytes = sizeof(int64_t) * ((size_t)C.nd + 1);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    uint8_t *scratch = nullptr;
    DQ_CUDA(dev_malloc_async(&scratch, up(mbytes) + up(cbytes) + sbytes, s));
    int32_t *dmap = (int32_t *)scratch;
    int32_t *dcnt = (int32_t *)(scratch + up(mbytes));
    int64_t *dstart = (int64_t *)(scratch + up(mbytes) + up(cbytes));
    int2 *dpairs = nullptr;
    std::vector<int32_t> cnt((size_t)C.nd);
    std::vector<int64_t> start((size_t)C.nd + 1, 0);
    const int pg = (int)std::max<int64_t>(1, std::min<int64_t>((C.nd + 127) / 128, 4 * num_sms()));
    cudaError_t e = cudaMemcpyAsync(dmap, map.data(), mbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        spgemm_pairs_kernel<<<pg, 128, 0, s>>>(A.d_meta, A.nd, B.d_meta, dmap, bmin, bmax, C.d_meta, C.nd, dcnt,
                                               nullptr, nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), dcnt, cbytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) {
        for (int32_t c = 0; c < C.nd; ++c) start[(size_t)c + 1] = start[(size_t)c] + cnt[(size_t)c];
        const int64_t npairs = start[(size_t)C.nd];
        e = cudaMemcpyAsync(dstart, start.data(), sbytes, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = dev_malloc_async((void **)&dpairs, sizeof(int2) * (size_t)std::max<int64_t>(npairs, 1), s);
    }
    if (e == cudaSuccess) {
        spgemm_pairs_kernel<<<pg, 128, 0, s>>>(A.d_meta, A.nd, B.d_meta, dmap, bmin, bmax, C.d_meta, C.nd, nullptr,
                                               dstart, dpairs);
        int64_t maxrows = 1;
        for (const auto &m : C.meta) maxrows = std::max(maxrows, m.hi);
        const int V = A.prec == DIAQ_C128 ? 2 : 4;
        // up to 64 C diagonals per block row: each block walks several diagonals' pairs
        const dim3 grid(spmv_blocks(maxrows, V), (unsigned)std::min<int64_t>(C.nd, 64));
        // the operands' masks (both or neither); taken here, outside any graph capture
        const uint32_t *ka = cached_tile_mask(A, s), *kb = ka ? cached_tile_mask(B, s) : nullptr;
        if (!kb) ka = nullptr;
        const int64_t wa = tile_mask_words(A.rows), wb = tile_mask_words(B.rows);
        if (A.prec == DIAQ_C128)
            spgemm_numeric_kernel<double><<<grid, kSpmvThreads, 0, s>>>(
                A.d_meta, (const double *)A.re, (const double *)A.im, B.d_meta, (const double *)B.re,
                (const double *)B.im, C.d_meta, C.nd, dstart, dpairs, (double *)C.re, (double *)C.im, ka, wa, kb, wb);
        else
            spgemm_numeric_kernel<float><<<grid, kSpmvThreads, 0, s>>>(
                A.d_meta, (const float *)A.re, (const float *)A.im, B.d_meta, (const float *)B.re,
                (const float *)B.im, C.d_meta, C.nd, dstart, dpairs, (float *)C.re, (float *)C.im, ka, wa, kb, wb);
        e = cudaGetLastError();
    }
    // the host vectors must outlive the async copies
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (dpairs) cudaFreeAsync(dpairs, s);
    cudaFreeAsync(scratch, s);
    if (e != cudaSuccess) return cuda_status(e, "spgemm numeric", __FILE__, __LINE__);
    return DIAQ_OK;
}

int spgemm(const Matrix &A, const Matrix &B, bool prune, cudaStream_t s, Matrix **out) {
    if (A.prec == DIAQ_C128F2) return set_error(DIAQ_ERR_UNSUPPORTED, "product: convert a c128f2 matrix to c128 first");
    if (A.cols != B.rows) return set_error(DIAQ_ERR_INVALID, "diaQMatrix product_cuda: dimension mismatch.");
    if (A.prec != B.prec) return set_error(DIAQ_ERR_INVALID, "product: operands must have the same precision");
    std::vector<int32_t> offC;
    DQ_TRY(spgemm_symbolic(A, B, offC, s));
    Matrix *C = nullptr;
    // the numeric pass writes every stored value of C: only the gaps around them need zeroing
    DQ_TRY(make_zero(A.rows, B.cols, (int32_t)offC.size(), offC.data(), A.prec, s, &C, false));
    int st = spgemm_numeric(A, B, *C, s);
    if (st == DIAQ_OK) st = zero_gaps(*C, s);
    if (st == DIAQ_OK && prune) {
        Matrix *P = nullptr;
        st = prune_matrix(*C, s, &P);
        if (st == DIAQ_OK) {
            destroy(C);
            C = P;
        }
    }
    if (st != DIAQ_OK) {
        destroy(C);
        return st;
    }
    *out = C;
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_spgemm_symbolic(diaq_matrix_t A, diaq_matrix_t B, int32_t *offsets_out, int32_t *count,
                         void *stream) {
    if (!A || !B || !count) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    std::vector<int32_t> offC;
    DQ_TRY(spgemm_symbolic(*A, *B, offC, (cudaStream_t)stream));
    if (!offC.empty() && !offsets_out) return set_error(DIAQ_ERR_INVALID, "offsets_out is NULL");
    std::copy(offC.begin(), offC.end(), offsets_out);
    *count = (int32_t)offC.size();
    return DIAQ_OK;
}

int diaq_spgemm_numeric(diaq_matrix_t A, diaq_matrix_t B, diaq_matrix_t C, void *stream) {
    if (!A || !B || !C) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    return spgemm_numeric(*A, *B, *C, (cudaStream_t)stream);
}

int diaq_spgemm(diaq_matrix_t A, diaq_matrix_t B, int prune, void *stream, diaq_matrix_t *C) {
    if (!A || !B || !C) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    Matrix *M = nullptr;
    DQ_TRY(spgemm(*A, *B, prune != 0, (cudaStream_t)stream, &M));
    *C = handle(M);
    return DIAQ_OK;
}

}  // extern "C"
