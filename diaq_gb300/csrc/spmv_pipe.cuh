// Pipelined variant of the diagonal SpMV for several states: asynchronous copies (cp.async)
// bring the matrix values and the shifted state windows of the next STAGES-1 diagonals into
// shared memory while the current diagonal is multiplied.
//
// Why: with K states the register version keeps K*VR*2 accumulators live, so few warps fit on
// an SM, and each warp issues one diagonal's loads and then waits for them (in-order issue):
// the kernel is latency-bound far below HBM bandwidth.  Copies in flight through cp.async hold
// no registers, so STAGES-1 diagonals of loads stay in flight per thread.
//
// Each thread copies exactly the values it later reads (its VR rows, for the matrix and for
// every state), so no block barrier is needed: cp.async.wait_group orders a thread's own copies.
// Rows outside a diagonal get zero-filled copies (source size 0: nothing is read).  Matrix
// vectors are 16-byte copies at row-phase aligned addresses (always inside the allocation, see
// the layout notes); state windows use one VR-wide copy when aligned and fully inside, else
// one 4-byte copy per row.
#pragma once

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void *dst, const void *src) {
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(smem_addr(dst)), "l"(src), "n"(BYTES));
}

// 4-byte copy that writes zero instead when `valid` is false (nothing is read then).
__device__ __forceinline__ void cp_async4_or_zero(void *dst, const void *src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_addr(dst)), "l"(src),
                 "r"(valid ? 4 : 0));
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Shared memory per thread and stage: (2 + 2K) * VR floats.
template <int K, int VR>
constexpr int pipe_floats_per_thread() {
    return (2 + 2 * K) * VR;
}

template <int K, int VR, int STAGES, class Epi>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_spmv_pipe_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ are,
                         const float *__restrict__ aim, int64_t rows, const float *__restrict__ xr,
                         const float *__restrict__ xi, int64_t ldx, int kq, Epi epi) {
    static_assert(VR == 4, "the pipelined kernel moves 16-byte matrix vectors");
    constexpr int F = pipe_floats_per_thread<K, VR>();
    extern __shared__ __align__(16) float pipe_smem[];
    // stage s, thread t: floats [((s * kSpmvThreads) + t) * F, + F): a_re[VR] a_im[VR] x_re[K][VR] x_im[K][VR]
    float *mine = pipe_smem + (size_t)threadIdx.x * F;
    const int64_t r0 = ((int64_t)blockIdx.x * kSpmvThreads + threadIdx.x) * VR;
    const bool active = r0 < rows;

    auto issue = [&](int k, int stage) {
        float *slot = mine + (size_t)stage * kSpmvThreads * F;
        const DiagMeta m = meta[k];
        const bool touch = active && (r0 + VR > m.lo) && (r0 < m.hi);
        if (touch) {
            cp_async<16>(slot, are + m.base + r0);
            cp_async<16>(slot + VR, aim + m.base + r0);
            const int64_t c = r0 + m.off;
            const bool full = (r0 >= m.lo) && (r0 + VR <= m.hi);
#pragma unroll
            for (int q = 0; q < K; ++q) {
                if (q >= kq) break;
                const float *pr = xr + q * ldx + c, *pi = xi + q * ldx + c;
                float *dr = slot + 2 * VR + q * VR, *di = slot + 2 * VR + (K + q) * VR;
                if (full && aligned_to<16>(pr) && aligned_to<16>(pi)) {
                    cp_async<16>(dr, pr);
                    cp_async<16>(di, pi);
                } else {
#pragma unroll
                    for (int v = 0; v < VR; ++v) {
                        const bool ok = (r0 + v >= m.lo) && (r0 + v < m.hi);
                        // a rejected copy reads nothing; point it at a value that exists
                        cp_async4_or_zero(dr + v, ok ? pr + v : xr, ok);
                        cp_async4_or_zero(di + v, ok ? pi + v : xi, ok);
                    }
                }
            }
        }
        cp_async_commit();  // one group per diagonal, empty when the thread has nothing to copy
    };

    float accr[K][VR], acci[K][VR];
#pragma unroll
    for (int q = 0; q < K; ++q)
#pragma unroll
        for (int v = 0; v < VR; ++v) accr[q][v] = acci[q][v] = 0.f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nd) issue(s, s);
        else cp_async_commit();
    }
    for (int k = 0; k < nd; ++k) {
        const int nk = k + STAGES - 1;
        if (nk < nd) issue(nk, nk % STAGES);
        else cp_async_commit();
        cp_async_wait<STAGES - 1>();  // diagonal k's copies (this thread's) have landed
        const DiagMeta m = meta[k];
        if (!active || r0 + VR <= m.lo || r0 >= m.hi) continue;
        const float *slot = mine + (size_t)(k % STAGES) * kSpmvThreads * F;
        float ar[VR], ai[VR];
#pragma unroll
        for (int v = 0; v < VR; ++v) {
            const bool ok = (r0 + v >= m.lo) && (r0 + v < m.hi);
            ar[v] = ok ? slot[v] : 0.f;
            ai[v] = ok ? slot[VR + v] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (q >= kq) break;
            const float *dr = slot + 2 * VR + q * VR, *di = slot + 2 * VR + (K + q) * VR;
#pragma unroll
            for (int v = 0; v < VR; ++v) {
                const float xv = dr[v], yv = di[v];
                accr[q][v] = fmaf(ar[v], xv, accr[q][v]);
                accr[q][v] = fmaf(-ai[v], yv, accr[q][v]);
                acci[q][v] = fmaf(ar[v], yv, acci[q][v]);
                acci[q][v] = fmaf(ai[v], xv, acci[q][v]);
            }
        }
    }
    cp_async_wait<0>();
    if (active) epi.template apply<float, K, VR>(r0, rows, kq, accr, acci);
}

template <int K, int STAGES>
constexpr size_t pipe_smem_bytes() {
    return (size_t)STAGES * kSpmvThreads * pipe_floats_per_thread<K, 4>() * sizeof(float);
}

// Stages per state count: the deepest pipeline that fits the 227 KB of shared memory a block may use.
template <int K>
constexpr int pipe_stages() {
    return K == 8 ? 3 : 4;
}

template <int K, int STAGES, class Epi>
void launch_pipe_k(const Matrix &A, const float *xr, const float *xi, int64_t ldx, int kq, const Epi &e,
                   cudaStream_t s) {
    constexpr size_t bytes = pipe_smem_bytes<K, STAGES>();
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(dia_spmv_pipe_kernel<K, 4, STAGES, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes);
        configured = true;
    }
    dia_spmv_pipe_kernel<K, 4, STAGES, Epi><<<spmv_blocks(A.rows, 4), kSpmvThreads, bytes, s>>>(
        A.d_meta, A.nd, (const float *)A.re, (const float *)A.im, A.rows, xr, xi, ldx, kq, e);
}

// Pipelined launch over the states in chunks of up to kmax (1, 2, 4 or 8), 4 rows per thread.
// The state windows must be float arrays with N values per state at leading dimension ldx.
template <class Epi>
int launch_dia_spmv_pipe(const Matrix &A, const float *xr, const float *xi, int64_t ldx, int nrhs, Epi epi,
                         cudaStream_t s, int kmax, int *launches) {
    if (A.rows == 0 || nrhs <= 0) return DIAQ_OK;
    kmax = kmax >= 8 ? 8 : kmax >= 4 ? 4 : kmax >= 2 ? 2 : 1;
    int q0 = 0;
    while (q0 < nrhs) {
        const int left = nrhs - q0;
        const int kq = left < kmax ? left : kmax;
        const float *pxr = xr + q0 * ldx, *pxi = xi + q0 * ldx;
        const Epi e = epi.shifted(q0);
        if (kq > 4)
            launch_pipe_k<8, pipe_stages<8>(), Epi>(A, pxr, pxi, ldx, kq, e, s);
        else if (kq > 2)
            launch_pipe_k<4, pipe_stages<4>(), Epi>(A, pxr, pxi, ldx, kq, e, s);
        else if (kq == 2)
            launch_pipe_k<2, pipe_stages<2>(), Epi>(A, pxr, pxi, ldx, kq, e, s);
        else
            launch_pipe_k<1, pipe_stages<1>(), Epi>(A, pxr, pxi, ldx, kq, e, s);
        q0 += kq;
        ++*launches;
    }
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

}  // namespace diaq_gb300
