// The chosen form's Taylor term fed by bulk asynchronous copies (plan variant 10).
//
// A block owns R rows (R = 32 * 8 / (sp / G)) of the tiled interleaved states and runs nine
// warps: eight consumers (warp w: rows 32 (w / groups) .. + 31 of the block, states G g .. of
// quad group g = w mod groups) and one producer.  The producer walks the diagonals that are live
// for the block (a nonzero in any of its tiles, from the zero-tile mask) and, for each, copies
// into a ring of S shared-memory stages with `cp.async.bulk` (the TMA engine, no registers held):
// the block's rows of the diagonal's matrix values (re, im) and the tiles of state rows its
// window reaches (R / 32 + 1 tiles of every state, re and im), completing on the stage's `full`
// mbarrier.  Consumers wait on `full`, multiply-add from shared memory, and release the stage on
// its `empty` mbarrier (one arrival per warp); the producer refills a stage once all eight have
// released it.  Up to S diagonals of every block are in flight with no consumer waiting on
// global memory.
//
// Every wait is bounded in time (%globaltimer, nanoseconds): a consumer warp that waits longer
// than `wait_ns` for a stage records an error in *err and leaves; the producer gives up a wait for
// a free stage after `wait_ns` as well.  On every exit path the producer first waits -- bounded by
// `drain_ns`, which the launcher sets well above the microseconds a copy takes -- for the last
// fill of every stage it used, so no copy lands in the shared memory of a finished block.  The
// plan reports the error to the caller (diaq_evolve_check, or the next run).
#pragma once

#include "spmv_il.cuh"

namespace diaq_gb300 {

constexpr int kTmaStagesMax = 8;
constexpr int kTmaConsumerWarps = 8;
constexpr int kTmaThreads = 32 * (kTmaConsumerWarps + 1);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One poll that never suspends the thread.
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// One poll: the thread may be suspended for up to about hint_ns while the phase is incomplete.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase of `parity` to complete; false (and *err set to code) once limit_ns
// nanoseconds have passed by %globaltimer, or 4 * limit_ns SM cycles by clock64, whichever comes
// first (the global timer ticks about once a microsecond; the cycle bound makes bounds below its
// resolution effective and lasts limit_ns or longer at any SM clock up to 4 GHz).  Each round
// polls once without suspending, checks the bound, then polls with a suspension hinted to at most
// min(limit_ns, 20 us).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *err, int code,
                                                  uint64_t limit_ns) {
    const uint32_t hint = (uint32_t)(limit_ns < 20000ull ? limit_ns : 20000ull);
    const uint64_t t0 = globaltimer_ns();
    const long long c0 = clock64();
    for (;;) {
        if (mbar_test_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit_ns || (uint64_t)(clock64() - c0) > 4ull * limit_ns) break;
        if (mbar_try_wait(bar, parity, hint)) return true;
    }
    atomicExch(err, code);
    return false;
}

// bytes (a multiple of 16) from global src to shared dst (both 16-byte aligned), completing on bar
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Floats of one stage: matrix re, matrix im (R each) and, when the windows are staged (WIN),
// window re, window im ((R / 32 + 1) tiles of 32 sp floats each).
__host__ __device__ inline int64_t tma_stage_floats(int R, int sp, bool win) {
    return 2 * (int64_t)R + (win ? 2 * (int64_t)(R / 32 + 1) * 32 * sp : 0);
}
__host__ __device__ inline size_t tma_smem_bytes(int R, int sp, bool win, int stages) {
    return 2 * 8 * kTmaStagesMax + sizeof(float) * (size_t)stages * (size_t)tma_stage_floats(R, sp, win);
}

// nd <= kMetaChunk (the launcher falls back to the register kernel otherwise).  WIN: stage the
// state windows as well (else only the matrix values, the windows read through L1); S stages.
template <class Epi, int G, bool WIN, int S>
__global__ void __launch_bounds__(kTmaThreads)
    dia_spmv_tma_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ are,
                        const float *__restrict__ aim, int64_t rows, int64_t n_pad, const float *__restrict__ xr,
                        const float *__restrict__ xi, const uint32_t *__restrict__ tmask, int64_t mw, Epi epi,
                        int *err, uint64_t wait_ns, uint64_t drain_ns) {
    static_assert(G == 4 || G == 8, "4 or 8 states per thread");
    __shared__ DiagMeta sm[kMetaChunk];
    __shared__ uint32_t smk[kMetaChunk];
    extern __shared__ __align__(128) unsigned char dyn[];
    static_assert(S <= kTmaStagesMax, "stages");
    uint64_t *full = reinterpret_cast<uint64_t *>(dyn), *empty = full + S;
    float *stages = reinterpret_cast<float *>(dyn + 2 * 8 * kTmaStagesMax);

    const int sp = epi.sp, quads = sp >> 2, groups = sp / G;
    const int R = 32 * (8 / groups), tiles = R / 32;
    const int64_t a0 = (int64_t)blockIdx.x * R;  // R | 1024: the block's tiles share one mask word
    const int tbit0 = (int)((a0 >> 5) & 31);
    const uint32_t bmask = (tiles >= 32 ? 0xffffffffu : ((1u << tiles) - 1u)) << tbit0;
    const int64_t SF = tma_stage_floats(R, sp, WIN), WF = (int64_t)(tiles + 1) * 32 * sp;

    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
        sm[i] = meta[i];
        smk[i] = tmask[(int64_t)i * mw + (a0 >> 10)];
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kTmaConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int wid = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    if (wid == kTmaConsumerWarps) {  // producer
        if (lane != 0) return;
        int i = 0;
        // fills i - S .. i - 1 are the last of every stage used: wait until their copies have
        // landed (a copy in flight always completes; the bound only guards the wait itself)
        auto drain = [&]() {
            for (int f = max(i - S, 0); f < i; ++f) mbar_wait_bounded(&full[f % S], (uint32_t)((f / S) & 1), err, 3, drain_ns);
        };
        for (int j = 0; j < nd; ++j) {
            if (!(smk[j] & bmask)) continue;
            const int s = i % S;
            if (i >= S && !mbar_wait_bounded(&empty[s], (uint32_t)((i / S - 1) & 1), err, 1, wait_ns)) {
                drain();
                return;
            }
            const DiagMeta m = sm[j];
            float *st = stages + s * SF;
            // matrix rows [a0, a0 + R) clipped to the diagonal's stored rows widened to 16-byte
            // vectors (inside the 32-value guards)
            const int64_t rl = max(a0, m.lo & ~(int64_t)3), rh = min(a0 + R, (m.hi + 3) & ~(int64_t)3);
            const uint32_t bm = (uint32_t)(rh - rl) * 4u;
            // state tiles t0 .. t0 + tiles, clipped to the vector
            const int64_t t0 = (a0 + m.off) >> 5;
            const int64_t ta = max(t0, (int64_t)0), tb = min(t0 + tiles + 1, n_pad >> 5);
            const uint32_t bw = WIN ? (uint32_t)(tb - ta) * 128u * (uint32_t)sp : 0u;
            mbar_expect_tx(&full[s], 2 * bm + 2 * bw);
            bulk_g2s(st + (rl - a0), are + m.base + rl, bm, &full[s]);
            bulk_g2s(st + R + (rl - a0), aim + m.base + rl, bm, &full[s]);
            if (WIN) {
                bulk_g2s(st + 2 * R + (ta - t0) * 32 * sp, xr + ta * 32 * sp, bw, &full[s]);
                bulk_g2s(st + 2 * R + WF + (ta - t0) * 32 * sp, xi + ta * 32 * sp, bw, &full[s]);
            }
            ++i;
        }
        drain();
        return;
    }

    // consumers
    const int g = wid % groups;
    const int64_t r = a0 + (int64_t)(wid / groups) * 32 + lane;
    const int tbit = (int)((r >> 5) & 31);
    float accr[G], acci[G];
#pragma unroll
    for (int q = 0; q < G; ++q) accr[q] = acci[q] = 0.f;
    int i = 0;
    for (int j = 0; j < nd; ++j) {
        if (!(smk[j] & bmask)) continue;
        const int s = i % S;
        // every lane waits (each must observe the copy's completion); the warp leaves together when
        // any lane gave up, so no lane is left behind at the __syncwarp below
        const bool ok = mbar_wait_bounded(&full[s], (uint32_t)((i / S) & 1), err, 2, wait_ns);
        if (!__all_sync(0xffffffffu, ok)) return;
        const DiagMeta &m = sm[j];
        if (((smk[j] >> tbit) & 1u) && r >= m.lo && r < m.hi) {
            const float *st = stages + s * SF;
            const float a = st[r - a0], b = st[R + (r - a0)];
            const int64_t c = r + m.off, t0f = ((a0 + m.off) >> 5) * 32 * sp;
            if (!WIN) {
                il_term<G>(c, g * (G / 4), quads, a, b, xr, xi, accr, acci);
            } else {
            const float4 *wre = reinterpret_cast<const float4 *>(st + 2 * R);
            const float4 *wim = reinterpret_cast<const float4 *>(st + 2 * R + WF);
            IlWindow<G> w;
#pragma unroll
            for (int h = 0; h < G / 4; ++h) {
                const int64_t at = (il_at(c, g * (G / 4) + h, quads) - t0f) >> 2;
                w.x[h] = wre[at];
                w.y[h] = wim[at];
            }
            il_fma<G>(a, b, w, accr, acci);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
        ++i;
    }
    if (r >= rows) return;
#pragma unroll
    for (int h = 0; h < G / 4; ++h) {
        const float ar4[4] = {accr[4 * h], accr[4 * h + 1], accr[4 * h + 2], accr[4 * h + 3]};
        const float ai4[4] = {acci[4 * h], acci[4 * h + 1], acci[4 * h + 2], acci[4 * h + 3]};
        epi.apply(r, g * (G / 4) + h, ar4, ai4);
    }
}

}  // namespace diaq_gb300
