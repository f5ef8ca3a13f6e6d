// Zero-tile masks of device matrices (the layout is described with tile_mask_words in
// spmv_kernel.cuh).  One block per (1024-row word, diagonal): each warp tests four 32-row tiles
// with a ballot, the block ORs the bits into one word.  Reads every stored value once.
#include <algorithm>
#include <vector>

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

template <typename T>
__global__ void tile_mask_kernel(const DiagMeta *__restrict__ meta, int nd, const T *__restrict__ re,
                                 const T *__restrict__ im, int64_t W, uint32_t *__restrict__ mask) {
    __shared__ uint32_t word;
    const int lane = (int)threadIdx.x & 31, warp = (int)threadIdx.x >> 5;
    const int64_t w = blockIdx.x;
    for (int j = blockIdx.y; j < nd; j += gridDim.y) {
        __syncthreads();  // the previous diagonal's word is stored
        if (threadIdx.x == 0) word = 0u;
        __syncthreads();
        const DiagMeta m = meta[j];
        for (int t = warp; t < 32; t += (int)(blockDim.x >> 5)) {
            const int64_t r = (w * 32 + t) * 32 + lane;
            bool nz = false;
            if (r >= m.lo && r < m.hi) nz = re[m.base + r] != (T)0 || im[m.base + r] != (T)0;
            const unsigned any = __ballot_sync(0xffffffffu, nz);
            if (any && lane == 0) atomicOr(&word, 1u << t);
        }
        __syncthreads();
        if (threadIdx.x == 0) mask[(int64_t)j * W + w] = word;
    }
}

int build_tile_mask(const Matrix &A, uint32_t *mask, cudaStream_t s) {
    if (A.nd == 0 || A.rows == 0) return DIAQ_OK;
    const int64_t W = tile_mask_words(A.rows);
    if (W > 0x7fffffffll) return set_error(DIAQ_ERR_UNSUPPORTED, "tile mask: too many rows");
    const dim3 grid((unsigned)W, (unsigned)std::min(A.nd, 65535));
    // float pairs: the hi planes (the first `capacity` floats); a zero hi part has a zero lo part
    if (A.prec == DIAQ_C64 || A.prec == DIAQ_C128F2)
        tile_mask_kernel<float><<<grid, 256, 0, s>>>(A.d_meta, A.nd, (const float *)A.re, (const float *)A.im, W, mask);
    else
        tile_mask_kernel<double><<<grid, 256, 0, s>>>(A.d_meta, A.nd, (const double *)A.re, (const double *)A.im, W,
                                                      mask);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

const uint32_t *existing_tile_mask(const Matrix &A, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;
    }
    return A.tmask_ok ? A.tmask : nullptr;
}

const uint32_t *cached_tile_mask(const Matrix &A, cudaStream_t s) {
    if (A.nd == 0 || A.rows == 0) return nullptr;
    // no mask in a recorded graph: a replay could outlive the values the mask was taken from
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;
    }
    if (A.tmask_ok) return A.tmask;
    if (!A.tmask && dev_malloc(&A.tmask, sizeof(uint32_t) * (size_t)A.nd * (size_t)tile_mask_words(A.rows)) != cudaSuccess) {
        cudaGetLastError();
        A.tmask = nullptr;
        return nullptr;
    }
    if (build_tile_mask(A, A.tmask, s) != DIAQ_OK || cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    A.tmask_ok = true;
    return A.tmask;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" int diaq_matrix_live_values(diaq_matrix_t A, int64_t *out, void *stream) {
    if (!A || !out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    *out = 0;
    if (A->nd == 0 || A->rows == 0) return DIAQ_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t W = tile_mask_words(A->rows);
    uint32_t *mask = nullptr;
    DQ_CUDA(dev_malloc(&mask, sizeof(uint32_t) * (size_t)A->nd * (size_t)W));
    std::vector<uint32_t> h((size_t)A->nd * (size_t)W);
    int st = build_tile_mask(*A, mask, s);
    cudaError_t e = cudaSuccess;
    if (st == DIAQ_OK) e = cudaMemcpyAsync(h.data(), mask, sizeof(uint32_t) * h.size(), cudaMemcpyDeviceToHost, s);
    if (st == DIAQ_OK && e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(mask);
    if (st != DIAQ_OK) return st;
    if (e != cudaSuccess) return cuda_status(e, "live values", __FILE__, __LINE__);
    // every set bit is a 32-row tile with a nonzero: count its stored rows (a tile at either end
    // of a diagonal holds fewer)
    int64_t live = 0;
    for (int j = 0; j < A->nd; ++j) {
        const DiagMeta &m = A->meta[j];
        for (int64_t w = 0; w < W; ++w) {
            uint32_t bits = h[(size_t)j * W + w];
            while (bits) {
                const int b = __builtin_ctz(bits);
                bits &= bits - 1;
                const int64_t r0 = (w * 32 + b) * 32, r1 = r0 + 32;
                live += std::max<int64_t>(0, std::min(r1, m.hi) - std::max(r0, m.lo));
            }
        }
    }
    *out = live;
    return DIAQ_OK;
}

