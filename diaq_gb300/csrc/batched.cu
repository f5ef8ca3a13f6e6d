// Batched time evolution: many Hamiltonians of uneven size, each with several states, advanced
// together.  No counterpart in the reference, which evolves one state of one Hamiltonian per
// call (src/spHamSim_gpu_all_fused.cu:287-376).
//
// Work queue.  Every instance i is cut into items (i, row tile, chunk of up to K states); the
// item list, largest instances first, lives on the device.  One time step is a sequence of
// phases; in phase p instance i runs Taylor term k = p mod m_i + 1 of sub-step p / m_i while
// p < 2^s_i m_i (instances with fewer phases sit out the later ones).  Each phase is one launch
// of a persistent kernel (grid = resident blocks of the whole GPU) whose blocks take items from
// the list in a fixed stride; each item reads its instance's diagonals once for its K states.
// The phases of one step are recorded as a CUDA graph and replayed for every step.
//
// Arithmetic per instance (T = float for complex64 matrices, double for complex128):
//   t = (-i tau/k) (H v) in T;  (hi, lo) <- TwoSum-accumulated sum of the terms in T;
//   last term of a sub-step:    psi += hi + lo in float64, and v <- T(psi) for the next one.
// The term vectors ping-pong between two buffers; when an instance's step has an odd number of
// launches, one extra phase copies its first input back into place.
//
// Horner form (diaq_batch_set_horner, instances with m >= 2): w_m = psi, w_k = T(psi) +
// (-i tau/(k+1)) H w_{k+1}, psi += (-i tau) H w_1 in float64 -- no running sum.  T(psi) stays in
// v_a for the whole sub-step (the last term refreshes it), w alternates between v_b and the
// otherwise unused hi vectors, and no copy phase is needed.
//
// Interleaved instances.  A complex64 instance with 4 to 32 states keeps its float32 work vectors
// in the tiled interleaved layout (spmv_il.cuh: 32 rows x 4 states per 512-byte tile, the states
// padded to sp, a power of two) and runs in a second kernel of the same phase: one block per
// block of rows and all sp states, G = 8 states per thread when sp is a multiple of 8, else 4.
// Every window load of a warp is then one contiguous 512-byte run and every matrix value is read
// once per row block for all the states.  The other instances (1-3 or more than 32 states,
// complex128) keep the planar layout and the persistent kernel above.
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "spmv_il.cuh"

namespace diaq_gb300 {

struct BatchInst {
    const DiagMeta *meta;
    const void *are, *aim;
    int64_t rows;
    int nd, nrhs;
    int m, phases;   // Taylor terms per sub-step; launches per step (2^s m, +1 when odd)
    int sub;         // 2^s
    int horner;      // Horner evaluation (m >= 2 and the batch's form)
    int il_ok, il;   // may use / uses the interleaved layout
    int sp;          // interleaved: states padded to a power of two >= 4
    int64_t n_pad;   // interleaved: rows padded to a multiple of 32
    const uint32_t *tmask;  // zero-tile mask of the matrix (rebuilt at every run), mw words per diagonal
    int64_t mw;
    double tau;      // dt / 2^s
    double *pr, *pi; // states, leading dimension rows
    void *var, *vai, *vbr, *vbi, *hr, *hi, *lr, *li;  // T work vectors, leading dimension rows
};

struct BatchItem {
    int inst, tile, chunk, pad;
};

// TwoSum with unfused adds (as spmv_il.cuh's two_sum), and an unfused add, per precision.
__device__ __forceinline__ void two_sum_t(float a, float b, float &s, float &e) { two_sum(a, b, s, e); }
__device__ __forceinline__ void two_sum_t(double a, double b, double &s, double &e) {
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// phase < 0: initialise v_a = T(psi) for every item.
template <typename T, int K, int VR>
__global__ void __launch_bounds__(kSpmvThreads)
    batched_phase_kernel(const BatchInst *__restrict__ insts, const BatchItem *__restrict__ items, int n_items,
                         int phase) {
    __shared__ int4 sq[kMetaChunk];     // offset, lo, hi, mask word of the item's rows
    __shared__ int64_t sb[kMetaChunk];  // value base
    __shared__ BatchInst si;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BatchItem item = items[it];
        __syncthreads();  // previous item done with the shared copies
        if (threadIdx.x == 0) si = insts[item.inst];
        __syncthreads();
        const BatchInst &I = si;
        const int64_t r0 = ((int64_t)item.tile * kSpmvThreads + threadIdx.x) * VR;
        const int q0 = item.chunk * K;
        const int kq = min(K, I.nrhs - q0);
        const int64_t ld = I.rows;
        if (phase < 0 || phase >= I.sub * I.m) {
            // initialisation, or the copy phase of an odd step (v_b -> v_a), or idle
            const bool init = phase < 0;
            const bool copy = !init && phase == I.sub * I.m && (I.phases > I.sub * I.m);
            if (!init && !copy) continue;
            for (int q = 0; q < kq; ++q)
                for (int v = 0; v < VR; ++v) {
                    const int64_t r = r0 + v;
                    if (r >= I.rows) continue;
                    const int64_t i = (int64_t)(q0 + q) * ld + r;
                    if (init) {
                        ((T *)I.var)[i] = (T)I.pr[i];
                        ((T *)I.vai)[i] = (T)I.pi[i];
                    } else {
                        ((T *)I.var)[i] = ((const T *)I.vbr)[i];
                        ((T *)I.vai)[i] = ((const T *)I.vbi)[i];
                    }
                }
            continue;
        }
        const int k = phase % I.m + 1;
        const bool first = (k == 1), last = (k == I.m);
        const T *xr, *xi;
        T *outr, *outi;
        if (I.horner) {  // x: T(psi) for the first term, else the previous term's w
            xr = (const T *)(first ? I.var : ((k - 1) & 1) ? I.vbr : I.hr);
            xi = (const T *)(first ? I.vai : ((k - 1) & 1) ? I.vbi : I.hi);
            outr = (T *)((k & 1) ? I.vbr : I.hr);
            outi = (T *)((k & 1) ? I.vbi : I.hi);
        } else {
            xr = (const T *)((phase & 1) ? I.vbr : I.var);
            xi = (const T *)((phase & 1) ? I.vbi : I.vai);
            outr = (T *)((phase & 1) ? I.var : I.vbr);
            outi = (T *)((phase & 1) ? I.vai : I.vbi);
        }
        xr += (int64_t)q0 * ld;
        xi += (int64_t)q0 * ld;

        T accr[K][VR], acci[K][VR];
#pragma unroll
        for (int q = 0; q < K; ++q)
#pragma unroll
            for (int v = 0; v < VR; ++v) accr[q][v] = acci[q][v] = (T)0;
        const T *are = (const T *)I.are, *aim = (const T *)I.aim;
        for (int c0 = 0; c0 < I.nd; c0 += kMetaChunk) {
            const int cn = min(kMetaChunk, I.nd - c0);
            __syncthreads();
            // the item's 256 VR rows (VR | 4) lie in one 1024-row mask word, a thread's VR in one tile
            const int64_t mword = ((int64_t)item.tile * kSpmvThreads * VR) >> 10;
            for (int j = threadIdx.x; j < cn; j += kSpmvThreads) {
                const DiagMeta m = I.meta[c0 + j];
                sq[j] = make_int4(m.off, (int)m.lo, (int)m.hi, (int)I.tmask[(int64_t)(c0 + j) * I.mw + mword]);
                sb[j] = m.base;
            }
            __syncthreads();
            if (r0 >= I.rows) continue;
            const int tbit = (int)((r0 >> 5) & 31);
            for (int j = 0; j < cn; ++j) {
                const int4 q = sq[j];
                const int64_t lo = q.y, hi = q.z;
                if (r0 + VR <= lo || r0 >= hi || !(((uint32_t)q.w >> tbit) & 1u)) continue;
                const int64_t base = sb[j], c = r0 + q.x;
                T ar[VR], ai[VR];
                load_vec_stream<T, VR>(ar, are + base + r0);
                load_vec_stream<T, VR>(ai, aim + base + r0);
                const bool full = (r0 >= lo) && (r0 + VR <= hi);
                if (!full) {
#pragma unroll
                    for (int v = 0; v < VR; ++v)
                        if (r0 + v < lo || r0 + v >= hi) ar[v] = ai[v] = (T)0;
                }
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    if (q >= kq) break;
                    const T *pxr = xr + q * ld + c, *pxi = xi + q * ld + c;
                    T xv[VR], yv[VR];
                    if (full && aligned_to<VR * sizeof(T)>(pxr) && aligned_to<VR * sizeof(T)>(pxi)) {
                        load_vec<T, VR>(xv, pxr);
                        load_vec<T, VR>(yv, pxi);
                    } else {
#pragma unroll
                        for (int v = 0; v < VR; ++v) {
                            const bool ok = (r0 + v >= lo) && (r0 + v < hi);
                            xv[v] = ok ? __ldg(pxr + v) : (T)0;
                            yv[v] = ok ? __ldg(pxi + v) : (T)0;
                        }
                    }
#pragma unroll
                    for (int v = 0; v < VR; ++v) {
                        accr[q][v] = fma(ar[v], xv[v], accr[q][v]);
                        accr[q][v] = fma(-ai[v], yv[v], accr[q][v]);
                        acci[q][v] = fma(ar[v], yv[v], acci[q][v]);
                        acci[q][v] = fma(ai[v], xv[v], acci[q][v]);
                    }
                }
            }
        }
        if (r0 >= I.rows) continue;
        if (I.horner) {
            const T scale = (T)(I.tau / (double)(I.m - k + 1));
            T *fr = (T *)I.var, *fi = (T *)I.vai;
#pragma unroll
            for (int q = 0; q < K; ++q) {
                if (q >= kq) break;
#pragma unroll
                for (int v = 0; v < VR; ++v) {
                    const int64_t r = r0 + v;
                    if (r >= I.rows) continue;
                    const int64_t i = (int64_t)(q0 + q) * ld + r;
                    const T tr = acci[q][v] * scale, ti = -accr[q][v] * scale;
                    if (!last) {
                        outr[i] = add_rn(fr[i], tr);
                        outi[i] = add_rn(fi[i], ti);
                    } else {  // this launch reads w_1, not T(psi): refreshing it here is safe
                        const double nr = I.pr[i] + (double)tr, ni = I.pi[i] + (double)ti;
                        I.pr[i] = nr;
                        I.pi[i] = ni;
                        fr[i] = (T)nr;
                        fi[i] = (T)ni;
                    }
                }
            }
            continue;
        }
        const T scale = (T)(I.tau / (double)k);
        T *hr = (T *)I.hr, *hi_ = (T *)I.hi, *lr = (T *)I.lr, *li = (T *)I.li;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (q >= kq) break;
#pragma unroll
            for (int v = 0; v < VR; ++v) {
                const int64_t r = r0 + v;
                if (r >= I.rows) continue;
                const int64_t i = (int64_t)(q0 + q) * ld + r;
                const T tr = acci[q][v] * scale, ti = -accr[q][v] * scale;
                T h_r, h_i, l_r, l_i;
                if (first) {
                    h_r = tr;
                    h_i = ti;
                    l_r = (T)0;
                    l_i = (T)0;
                } else {
                    T e_r, e_i;
                    two_sum_t(hr[i], tr, h_r, e_r);
                    two_sum_t(hi_[i], ti, h_i, e_i);
                    l_r = lr[i] + e_r;
                    l_i = li[i] + e_i;
                }
                if (!last) {
                    hr[i] = h_r;
                    hi_[i] = h_i;
                    lr[i] = l_r;
                    li[i] = l_i;
                    outr[i] = tr;
                    outi[i] = ti;
                } else {
                    const double nr = I.pr[i] + ((double)h_r + (double)l_r);
                    const double ni = I.pi[i] + ((double)h_i + (double)l_i);
                    I.pr[i] = nr;
                    I.pi[i] = ni;
                    outr[i] = (T)nr;
                    outi[i] = (T)ni;
                }
            }
        }
    }
}

// One item of an interleaved instance: row block `tile` (32 * 8 / (sp / G) rows) and all sp
// states.  Phases as in batched_phase_kernel; the initialisation and copy phases move the item's
// rows of every state, which are one contiguous range of the tiled vectors.
template <int G, bool HORNER>
__device__ __forceinline__ void batched_il_item(const BatchInst &I, int4 *sq, int64_t *sb, int64_t tile,
                                                int phase) {
    const int quads = I.sp >> 2, groups = I.sp / G;
    const int64_t rpb = 32 * (8 / groups);
    const int64_t r0 = tile * rpb, ld = I.rows;
    float *var = (float *)I.var, *vai = (float *)I.vai, *vbr = (float *)I.vbr, *vbi = (float *)I.vbi;
    if (phase < 0 || phase >= I.sub * I.m) {
        const bool init = phase < 0;
        const bool copy = !init && phase == I.sub * I.m && (I.phases > I.sub * I.m);
        if (!init && !copy) return;
        const int64_t e1 = min(r0 + rpb, I.n_pad) * I.sp;
        for (int64_t e = r0 * I.sp + threadIdx.x; e < e1; e += blockDim.x) {
            if (init) {  // element e of the tiled vector is state q of row r
                const int64_t blk = e / (quads * 128);
                const int rem = (int)(e - blk * quads * 128);
                const int64_t r = blk * 32 + ((rem & 127) >> 2);
                const int q = (rem >> 7) * 4 + (rem & 3);
                const bool live = r < I.rows && q < I.nrhs;
                var[e] = live ? (float)I.pr[q * ld + r] : 0.f;
                vai[e] = live ? (float)I.pi[q * ld + r] : 0.f;
            } else {
                var[e] = vbr[e];
                vai[e] = vbi[e];
            }
        }
        return;
    }
    const int k = phase % I.m + 1;
    const bool first = (k == 1), last = (k == I.m);
    const float *xr, *xi;
    float *outr, *outi;
    if (HORNER) {
        xr = first ? var : ((k - 1) & 1) ? vbr : (float *)I.hr;
        xi = first ? vai : ((k - 1) & 1) ? vbi : (float *)I.hi;
        outr = (k & 1) ? vbr : (float *)I.hr;
        outi = (k & 1) ? vbi : (float *)I.hi;
    } else {
        xr = (phase & 1) ? vbr : var;
        xi = (phase & 1) ? vbi : vai;
        outr = (phase & 1) ? var : vbr;
        outi = (phase & 1) ? vai : vbi;
    }
    const int wid = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int g = wid % groups;
    const int64_t r = r0 + (int64_t)(wid / groups) * 32 + lane;
    float accr[G], acci[G];
#pragma unroll
    for (int q = 0; q < G; ++q) accr[q] = acci[q] = 0.f;
    const float *are = (const float *)I.are, *aim = (const float *)I.aim;
    for (int c0 = 0; c0 < I.nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, I.nd - c0);
        __syncthreads();
        for (int j = threadIdx.x; j < cn; j += kSpmvThreads) {
            const DiagMeta m = I.meta[c0 + j];
            // the item's <= 256 rows: one mask word
            const uint32_t w = I.tmask[(int64_t)(c0 + j) * I.mw + (r0 >> 10)];
            sq[j] = make_int4(m.off, (int)m.lo, (int)m.hi, (int)w);
            sb[j] = m.base;
        }
        __syncthreads();
        {
            // the item's live tiles of diagonal j, asked of L2 after the barrier by lane j / 8 of
            // warp j % 8 (7,629 -> 7,733 states x steps/s on the 512-instance set, Horner)
            const int j = lane * 8 + wid;
            if (j < cn) {
                const int4 q = sq[j];
                prefetch_tiles_l2(are, aim, sb[j], (int64_t)q.y, (int64_t)q.z,
                                  block_tile_bits((uint32_t)q.w, r0, 8 / groups), r0);
            }
        }
        if (r >= I.rows) continue;
        il_accumulate32<G>(sq, sb, cn, (int)r, g * (G / 4), quads, are, aim, xr, xi, accr, acci);
    }
    if (r >= I.rows) return;
    if constexpr (HORNER) {  // the last step reads w_1, not fp32(psi): refreshing v_a there is safe
        const EpiHornerIL e{outr, outi, var, vai, var, vai, I.pr, I.pi, ld, I.sp, I.nrhs,
                            (float)(I.tau / (double)(I.m - k + 1)), last};
#pragma unroll
        for (int h = 0; h < G / 4; ++h) {
            const float ar4[4] = {accr[4 * h], accr[4 * h + 1], accr[4 * h + 2], accr[4 * h + 3]};
            const float ai4[4] = {acci[4 * h], acci[4 * h + 1], acci[4 * h + 2], acci[4 * h + 3]};
            e.apply(r, g * (G / 4) + h, ar4, ai4);
        }
    } else {
        const EpiMixedIL e{outr, outi, (float *)I.hr, (float *)I.hi, (float *)I.lr, (float *)I.li, I.pr, I.pi, ld, I.sp,
                           I.nrhs, (float)(I.tau / (double)k), first, last};
#pragma unroll
        for (int h = 0; h < G / 4; ++h) {
            const float ar4[4] = {accr[4 * h], accr[4 * h + 1], accr[4 * h + 2], accr[4 * h + 3]};
            const float ai4[4] = {acci[4 * h], acci[4 * h + 1], acci[4 * h + 2], acci[4 * h + 3]};
            e.apply(r, g * (G / 4) + h, ar4, ai4);
        }
    }
}

// Items of the instances with G states per thread in the Horner (HORNER) or the compensated form
// (separate lists and launches, so that each kernel keeps only its own registers).  Blocks per
// SM, measured on the 512-instance set: Horner at six (7,040 states x steps/s; 6,751 at five,
// 5,904 at four, 5,543 at eight, whose spills cost more than the occupancy gains), the
// compensated form at five (5,759; 5,637 at six); with the compact metadata loop
// (il_accumulate32) 7,571 and 6,091.
template <int G, bool HORNER>
__global__ void __launch_bounds__(kSpmvThreads, HORNER ? 6 : 5)
    batched_il_kernel(const BatchInst *__restrict__ insts, const BatchItem *__restrict__ items, int phase) {
    __shared__ int4 sq[kMetaChunk];
    __shared__ int64_t sb[kMetaChunk];
    __shared__ BatchInst si;
    const BatchItem item = items[blockIdx.x];
    if (threadIdx.x == 0) si = insts[item.inst];
    __syncthreads();
    batched_il_item<G, HORNER>(si, sq, sb, item.tile, phase);
}

struct Batch {
    int prec = DIAQ_C64;
    std::vector<BatchInst> inst;      // host copy
    std::vector<int64_t> rows;
    BatchInst *d_inst = nullptr;
    BatchItem *d_items = nullptr;     // planar instances
    int n_items = 0;
    BatchItem *d_il_items = nullptr;  // interleaved instances, one block each, in four segments:
    int n_il_items = 0;               // (G 8, Horner), (G 8, compensated), (G 4, Horner), (G 4, compensated)
    int il_seg[5] = {0, 0, 0, 0, 0};  // segment starts
    std::vector<char> items_horner;   // Horner flags the lists were built for
    bool il_on = true;                // interleave the instances that can be
    int items_il = -1;                // il_on of the current item lists
    void *work = nullptr;
    uint32_t *masks = nullptr;        // zero-tile masks of every instance's matrix
    std::vector<const Matrix *> mats;
    cudaStream_t s = nullptr;         // capture stream
    SpmvCfg cfg{8, 0};
    bool tuned = false;
    bool user_cfg = false;            // shape set by the caller
    int items_cfg_k = 0, items_cfg_vr = 0;
    cudaGraphExec_t graph = nullptr;
    std::vector<int> graph_key;       // (s_i, m_i) of the recorded graph, plus dt bits
    double graph_dt = 0.0;
    int max_phases = 0;
    bool horner = false;              // Horner evaluation for instances with m >= 2
    ~Batch() {
        if (graph) cudaGraphExecDestroy(graph);
        cudaFree(d_inst);
        cudaFree(d_items);
        cudaFree(d_il_items);
        cudaFree(work);
        cudaFree(masks);
        if (s) cudaStreamDestroy(s);
    }
};

}  // namespace diaq_gb300

struct diaq_batch_s : public diaq_gb300::Batch {};

namespace diaq_gb300 {

static int vr_of(const Batch &B) { return B.cfg.vr > 0 ? B.cfg.vr : (B.prec == DIAQ_C64 ? 4 : 2); }

// Item list for the current launch shape: largest instances first.
static int build_items(Batch &B) {
    const int K = B.cfg.kmax, VR = vr_of(B);
    std::vector<char> hf(B.inst.size());
    for (size_t i = 0; i < hf.size(); ++i) hf[i] = (char)B.inst[i].horner;
    if (B.d_items && B.items_cfg_k == K && B.items_cfg_vr == VR && B.items_il == (int)B.il_on && hf == B.items_horner)
        return DIAQ_OK;
    std::vector<int> order(B.inst.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return B.inst[a].rows * B.inst[a].nd * B.inst[a].nrhs > B.inst[b].rows * B.inst[b].nd * B.inst[b].nrhs;
    });
    std::vector<BatchItem> items, seg[4];
    for (int i : order) {
        const BatchInst &I = B.inst[i];
        if (I.il) {
            const bool eight = I.sp % 8 == 0;
            const int64_t rpb = 32 * (8 / (I.sp / (eight ? 8 : 4)));
            std::vector<BatchItem> &dst = seg[(eight ? 0 : 2) + (I.horner ? 0 : 1)];
            for (int64_t t = 0; t < (I.rows + rpb - 1) / rpb; ++t) dst.push_back(BatchItem{i, (int)t, 0, 0});
            continue;
        }
        const int64_t tiles = (B.inst[i].rows + (int64_t)kSpmvThreads * VR - 1) / ((int64_t)kSpmvThreads * VR);
        const int chunks = (B.inst[i].nrhs + K - 1) / K;
        for (int64_t t = 0; t < tiles; ++t)
            for (int c = 0; c < chunks; ++c) items.push_back(BatchItem{i, (int)t, c, 0});
    }
    std::vector<BatchItem> il_items;
    for (int q = 0; q < 4; ++q) {
        B.il_seg[q] = (int)il_items.size();
        il_items.insert(il_items.end(), seg[q].begin(), seg[q].end());
    }
    B.il_seg[4] = (int)il_items.size();
    if (B.d_items) cudaFree(B.d_items);
    if (B.d_il_items) cudaFree(B.d_il_items);
    B.d_items = B.d_il_items = nullptr;
    DQ_CUDA(dev_malloc(&B.d_items, sizeof(BatchItem) * std::max<size_t>(items.size(), 1)));
    DQ_CUDA(dev_malloc(&B.d_il_items, sizeof(BatchItem) * std::max<size_t>(il_items.size(), 1)));
    DQ_CUDA(cudaMemcpy(B.d_items, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice));
    DQ_CUDA(cudaMemcpy(B.d_il_items, il_items.data(), sizeof(BatchItem) * il_items.size(), cudaMemcpyHostToDevice));
    B.n_items = (int)items.size();
    B.n_il_items = (int)il_items.size();
    B.items_cfg_k = K;
    B.items_cfg_vr = VR;
    B.items_il = (int)B.il_on;
    B.items_horner = hf;
    return DIAQ_OK;
}

template <typename T, int K, int VR>
static int launch_phase_t(const Batch &B, int phase, cudaStream_t s) {
    if (B.n_items == 0) return DIAQ_OK;
    static int blocks_per_sm = 0;
    if (blocks_per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, batched_phase_kernel<T, K, VR>, kSpmvThreads, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    const int grid = std::max(1, std::min(B.n_items, blocks_per_sm * num_sms()));
    batched_phase_kernel<T, K, VR><<<grid, kSpmvThreads, 0, s>>>(B.d_inst, B.d_items, B.n_items, phase);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

template <typename T, int K>
static int launch_phase_k(const Batch &B, int phase, cudaStream_t s) {
    switch (vr_of(B)) {
        case 1: return launch_phase_t<T, K, 1>(B, phase, s);
        case 2: return launch_phase_t<T, K, 2>(B, phase, s);
        default:
            if constexpr (sizeof(T) == 4) return launch_phase_t<T, K, 4>(B, phase, s);
            return launch_phase_t<T, K, 2>(B, phase, s);
    }
}

template <typename T>
static int launch_phase(const Batch &B, int phase, cudaStream_t s) {
    switch (B.cfg.kmax) {
        case 1: return launch_phase_k<T, 1>(B, phase, s);
        case 2: return launch_phase_k<T, 2>(B, phase, s);
        case 4: return launch_phase_k<T, 4>(B, phase, s);
        default: return launch_phase_k<T, 8>(B, phase, s);
    }
}

static int phase(const Batch &B, int p, cudaStream_t s) {
    DQ_TRY(B.prec == DIAQ_C64 ? launch_phase<float>(B, p, s) : launch_phase<double>(B, p, s));
    const BatchItem *it = B.d_il_items;
    const int *q = B.il_seg;
    if (q[1] > q[0]) batched_il_kernel<8, true><<<q[1] - q[0], kSpmvThreads, 0, s>>>(B.d_inst, it + q[0], p);
    if (q[2] > q[1]) batched_il_kernel<8, false><<<q[2] - q[1], kSpmvThreads, 0, s>>>(B.d_inst, it + q[1], p);
    if (q[3] > q[2]) batched_il_kernel<4, true><<<q[3] - q[2], kSpmvThreads, 0, s>>>(B.d_inst, it + q[2], p);
    if (q[4] > q[3]) batched_il_kernel<4, false><<<q[4] - q[3], kSpmvThreads, 0, s>>>(B.d_inst, it + q[3], p);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// Per-instance schedules into the device table.
static int set_schedule(Batch &B, double dt, const int *sl, const int *m) {
    B.max_phases = 0;
    for (size_t i = 0; i < B.inst.size(); ++i) {
        if (sl[i] < 0 || sl[i] > 20 || m[i] < 1 || m[i] > 200)
            return set_error(DIAQ_ERR_INVALID, "batch: need 0 <= s <= 20 and 1 <= m <= 200 per instance");
        BatchInst &I = B.inst[i];
        I.sub = 1 << sl[i];
        I.m = m[i];
        I.tau = dt / (double)I.sub;
        I.horner = B.horner && I.m >= 2;
        I.il = I.il_ok && B.il_on;
        const int launches = I.sub * I.m;
        I.phases = I.horner ? launches : launches + (launches & 1);
        B.max_phases = std::max(B.max_phases, I.phases);
    }
    DQ_CUDA(cudaMemcpy(B.d_inst, B.inst.data(), sizeof(BatchInst) * B.inst.size(), cudaMemcpyHostToDevice));
    return DIAQ_OK;
}

static int enqueue_step(const Batch &B, cudaStream_t s) {
    for (int p = 0; p < B.max_phases; ++p) DQ_TRY(phase(B, p, s));
    return DIAQ_OK;
}

// ---- autotuner (same JSON cache as the evolution plans) ------------------------------------------
static std::string batch_cache_path() {
    if (const char *p = std::getenv("DIAQ_AUTOTUNE_CACHE")) return p;
    const char *home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/diaq_gb300/autotune.json";
}

static bool cache_lookup(const std::string &key, int &k, int &v) {
    std::ifstream f(batch_cache_path());
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    const size_t i = t.find("\"" + key + "\"");
    if (i == std::string::npos) return false;
    const size_t br = t.find('[', i);
    return br != std::string::npos && std::sscanf(t.c_str() + br, "[%d ,%d]", &k, &v) == 2;
}

static void cache_store(const std::string &key, int k, int v) {
    const std::string path = batch_cache_path();
    std::string body;
    {
        std::ifstream f(path);
        if (f) {
            std::stringstream ss;
            ss << f.rdbuf();
            body = ss.str();
        }
    }
    const size_t close = body.rfind('}');
    std::string entry = "  \"" + key + "\": [" + std::to_string(k) + ", " + std::to_string(v) + "]";
    std::string out;
    if (close == std::string::npos || body.find('"') == std::string::npos)
        out = "{\n" + entry + "\n}\n";
    else
        out = body.substr(0, close);
    if (close != std::string::npos && body.find('"') != std::string::npos) {
        while (!out.empty() && (out.back() == '\n' || out.back() == ' ')) out.pop_back();
        out += ",\n" + entry + "\n}\n";
    }
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        const std::string dir = path.substr(0, slash);
        for (size_t k2 = 1; k2 <= dir.size(); ++k2)
            if (k2 == dir.size() || dir[k2] == '/') mkdir(dir.substr(0, k2).c_str(), 0755);
    }
    // a temporary of this process's own, renamed into place: ranks sharing HOME never interleave
    const std::string tmp = path + "." + std::to_string((long)getpid()) + ".tmp";
    std::ofstream f(tmp);
    if (!f) return;
    f << out;
    f.close();
    std::rename(tmp.c_str(), path.c_str());
}

static std::string batch_key(const Batch &B) {
    int64_t rows = 0, states = 0;
    int il = 0;
    for (const auto &I : B.inst) {
        rows += I.rows;
        states += I.nrhs * I.rows;
        il += I.il;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, dev);
    std::string name(prop.name);
    for (auto &ch : name)
        if (ch == '"' || ch == ' ') ch = '_';
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s|batch|%s%s|inst=%zu|il=%d|rows=%lld|staterows=%lld|phases=%d",
                  name.c_str(), B.prec == DIAQ_C64 ? "c64" : "c128", B.horner ? "|horner" : "", B.inst.size(), il,
                  (long long)rows, (long long)states, B.max_phases);
    return buf;
}

// Time one step per candidate shape on scratch states (the caller's are saved and restored).
static int autotune(Batch &B) {
    if (std::all_of(B.inst.begin(), B.inst.end(), [](const BatchInst &I) { return I.il != 0; })) {
        B.tuned = true;  // no planar instance: the shape is unused
        return DIAQ_OK;
    }
    const std::string key = batch_key(B);
    int k = 0, v = 0;
    // a cached shape is used only if the compiled kernels include it
    if (cache_lookup(key, k, v) && (k == 1 || k == 2 || k == 4 || k == 8) &&
        (v == 1 || v == 2 || (B.prec == DIAQ_C64 && v == 4))) {
        B.cfg = SpmvCfg{k, v};
        B.tuned = true;
        return DIAQ_OK;
    }
    std::vector<SpmvCfg> cand;
    if (B.prec == DIAQ_C64)
        cand = {{8, 1}, {8, 2}, {4, 2}, {4, 4}, {2, 4}, {1, 4}};
    else
        cand = {{8, 1}, {4, 1}, {4, 2}, {2, 2}, {1, 2}};
    // save the states
    size_t total = 0;
    for (const auto &I : B.inst) total += 2 * (size_t)I.nrhs * (size_t)I.rows;
    double *save = nullptr;
    DQ_CUDA(dev_malloc(&save, sizeof(double) * std::max<size_t>(total, 1)));
    size_t o = 0;
    for (const auto &I : B.inst) {
        const size_t c = (size_t)I.nrhs * (size_t)I.rows;
        cudaMemcpyAsync(save + o, I.pr, c * sizeof(double), cudaMemcpyDeviceToDevice, B.s);
        cudaMemcpyAsync(save + o + c, I.pi, c * sizeof(double), cudaMemcpyDeviceToDevice, B.s);
        o += 2 * c;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = -1.f;
    SpmvCfg best_cfg = cand[0];
    int st = DIAQ_OK;
    for (const auto &c : cand) {
        B.cfg = c;
        st = build_items(B);
        if (st == DIAQ_OK) st = phase(B, -1, B.s);
        if (st == DIAQ_OK) st = enqueue_step(B, B.s);
        if (st != DIAQ_OK) break;
        cudaEventRecord(e0, B.s);
        st = enqueue_step(B, B.s);
        if (st != DIAQ_OK) break;
        cudaEventRecord(e1, B.s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            st = cuda_status(e, "batch autotune", __FILE__, __LINE__);
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (best < 0.f || ms < best) {
            best = ms;
            best_cfg = c;
        }
    }
    o = 0;
    for (const auto &I : B.inst) {
        const size_t c = (size_t)I.nrhs * (size_t)I.rows;
        cudaMemcpyAsync(I.pr, save + o, c * sizeof(double), cudaMemcpyDeviceToDevice, B.s);
        cudaMemcpyAsync(I.pi, save + o + c, c * sizeof(double), cudaMemcpyDeviceToDevice, B.s);
        o += 2 * c;
    }
    cudaStreamSynchronize(B.s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(save);
    if (st != DIAQ_OK) return st;
    B.cfg = best_cfg;
    B.tuned = true;
    cache_store(key, best_cfg.kmax, vr_of(B));
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_batch_create(int n_inst, const diaq_matrix_t *H, const int *nrhs, double *const *psi_re,
                      double *const *psi_im, diaq_batch_t *out) {
    if (!out || n_inst < 1 || !H || !nrhs || !psi_re || !psi_im) return set_error(DIAQ_ERR_INVALID, "batch: bad argument");
    const int prec = H[0] ? H[0]->prec : DIAQ_C64;
    const size_t esz = prec == DIAQ_C64 ? sizeof(float) : sizeof(double);
    // one work vector of instance i: planar nrhs x rows, or tiled sp x n_pad (complex64, 4-32 states),
    // rounded up to 256 bytes so that every vector starts aligned for 16-byte loads
    auto il_shape = [&](int i, int &sp, int64_t &n_pad) {
        sp = 4;
        while (sp < nrhs[i]) sp *= 2;
        n_pad = (H[i]->rows + 31) / 32 * 32;
        // (the interleaved kernels index rows and tiled vectors in 32 bits)
        return prec == DIAQ_C64 && nrhs[i] >= 4 && nrhs[i] <= 32 && (int64_t)sp * n_pad < ((int64_t)1 << 31);
    };
    auto vec_bytes = [&](int i) {
        int sp;
        int64_t n_pad;
        size_t e = (size_t)nrhs[i] * (size_t)H[i]->rows;
        if (il_shape(i, sp, n_pad)) e = std::max(e, (size_t)sp * (size_t)n_pad);
        return (e * esz + 255) / 256 * 256;
    };
    size_t work_bytes = 0;
    for (int i = 0; i < n_inst; ++i) {
        if (!H[i] || !psi_re[i] || !psi_im[i]) return set_error(DIAQ_ERR_INVALID, "batch: NULL matrix or state pointer");
        if (H[i]->rows != H[i]->cols) return set_error(DIAQ_ERR_INVALID, "batch: every H must be square");
        if (H[i]->prec != prec) return set_error(DIAQ_ERR_INVALID, "batch: all matrices must have the same precision");
        if (prec == DIAQ_C128F2) return set_error(DIAQ_ERR_UNSUPPORTED, "batch: c128 or c64 matrices only");
        if (nrhs[i] < 1) return set_error(DIAQ_ERR_INVALID, "batch: every instance needs at least one state");
        work_bytes += 8 * vec_bytes(i);
    }
    diaq_batch_s *B = new diaq_batch_s();
    B->prec = prec;
    cudaError_t e = cudaStreamCreateWithFlags(&B->s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dev_malloc(&B->work, work_bytes + 256);
    size_t mask_words = 0;
    for (int i = 0; i < n_inst; ++i) mask_words += (size_t)H[i]->nd * (size_t)tile_mask_words(H[i]->rows);
    if (e == cudaSuccess) e = dev_malloc(&B->masks, sizeof(uint32_t) * std::max<size_t>(mask_words, 1));
    if (e == cudaSuccess) e = dev_malloc(&B->d_inst, sizeof(BatchInst) * n_inst);
    if (e != cudaSuccess) {
        delete B;
        return cuda_status(e, "batch create", __FILE__, __LINE__);
    }
    uint8_t *w = (uint8_t *)B->work;
    size_t mask_off = 0;
    for (int i = 0; i < n_inst; ++i) {
        BatchInst I{};
        I.meta = H[i]->d_meta;
        I.are = H[i]->re;
        I.aim = H[i]->im;
        I.rows = H[i]->rows;
        I.nd = H[i]->nd;
        I.nrhs = nrhs[i];
        I.pr = psi_re[i];
        I.pi = psi_im[i];
        I.il_ok = il_shape(i, I.sp, I.n_pad) ? 1 : 0;
        I.tmask = B->masks + mask_off;
        I.mw = tile_mask_words(H[i]->rows);
        mask_off += (size_t)H[i]->nd * (size_t)I.mw;
        B->mats.push_back(H[i]);
        const size_t vb = vec_bytes(i);
        void **slots[8] = {&I.var, &I.vai, &I.vbr, &I.vbi, &I.hr, &I.hi, &I.lr, &I.li};
        for (int j = 0; j < 8; ++j) {
            *slots[j] = w;
            w += vb;
        }
        B->inst.push_back(I);
    }
    *out = B;
    return DIAQ_OK;
}

int diaq_batch_destroy(diaq_batch_t B) {
    delete B;
    return DIAQ_OK;
}

int diaq_batch_set_config(diaq_batch_t B, int states_per_launch, int rows_per_thread) {
    if (!B) return set_error(DIAQ_ERR_INVALID, "batch is NULL");
    if (states_per_launch == 0) {
        B->tuned = B->user_cfg = false;
    } else {
        const bool vr_ok = rows_per_thread == 1 || rows_per_thread == 2 || (B->prec == DIAQ_C64 && rows_per_thread == 4);
        if (!(states_per_launch == 1 || states_per_launch == 2 || states_per_launch == 4 || states_per_launch == 8) ||
            !vr_ok)
            return set_error(DIAQ_ERR_INVALID, "batch: states_per_launch 1, 2, 4 or 8; rows_per_thread 1, 2 (4 for c64)");
        B->cfg = SpmvCfg{states_per_launch, rows_per_thread};
        B->tuned = B->user_cfg = true;
    }
    if (B->graph) cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
    return DIAQ_OK;
}

int diaq_batch_set_horner(diaq_batch_t B, int on) {
    if (!B) return set_error(DIAQ_ERR_INVALID, "batch is NULL");
    if (B->horner != (on != 0)) {
        B->horner = on != 0;
        if (B->graph) cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;  // the schedule (phases per instance) is rebuilt on the next run
    }
    return DIAQ_OK;
}

int diaq_batch_set_interleaved(diaq_batch_t B, int on) {
    if (!B) return set_error(DIAQ_ERR_INVALID, "batch is NULL");
    if (B->il_on != (on != 0)) {
        B->il_on = on != 0;
        if (!B->user_cfg) B->tuned = false;  // other planar instances: tune again (or use the cache)
        if (B->graph) cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;
    }
    return DIAQ_OK;
}

int diaq_batch_config(diaq_batch_t B, int *states_per_launch, int *rows_per_thread, int *phases_per_step) {
    if (!B) return set_error(DIAQ_ERR_INVALID, "batch is NULL");
    if (states_per_launch) *states_per_launch = B->cfg.kmax;
    if (rows_per_thread) *rows_per_thread = vr_of(*B);
    if (phases_per_step) *phases_per_step = B->max_phases;
    return DIAQ_OK;
}

int diaq_batch_run(diaq_batch_t B, double dt, const int *substeps_log2, const int *m, int64_t steps, void *stream) {
    if (!B || !substeps_log2 || !m || steps < 0) return set_error(DIAQ_ERR_INVALID, "batch run: bad argument");
    if (steps == 0) return DIAQ_OK;
    cudaStream_t user = (cudaStream_t)stream;
    // the matrices are the caller's: their zero-tile masks are taken afresh at every run
    for (size_t i = 0; i < B->inst.size(); ++i) DQ_TRY(build_tile_mask(*B->mats[i], (uint32_t *)B->inst[i].tmask, user));
    DQ_CUDA(cudaStreamSynchronize(user));
    std::vector<int> key(substeps_log2, substeps_log2 + B->inst.size());
    key.insert(key.end(), m, m + B->inst.size());
    if (!B->graph || key != B->graph_key || dt != B->graph_dt) {
        if (B->graph) cudaGraphExecDestroy(B->graph);
        B->graph = nullptr;
        DQ_TRY(set_schedule(*B, dt, substeps_log2, m));
        if (!B->tuned) DQ_TRY(autotune(*B));
        DQ_TRY(build_items(*B));
        cudaGraph_t g = nullptr;
        DQ_CUDA(cudaStreamBeginCapture(B->s, cudaStreamCaptureModeThreadLocal));
        const int st = enqueue_step(*B, B->s);
        cudaError_t e = cudaStreamEndCapture(B->s, &g);
        if (st != DIAQ_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_status(e, "batch capture", __FILE__, __LINE__);
        e = cudaGraphInstantiate(&B->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_status(e, "batch instantiate", __FILE__, __LINE__);
        B->graph_key = key;
        B->graph_dt = dt;
    }
    DQ_TRY(phase(*B, -1, user));  // v_a = T(psi)
    for (int64_t i = 0; i < steps; ++i) DQ_CUDA(cudaGraphLaunch(B->graph, user));
    return DIAQ_OK;
}

}  // extern "C"
