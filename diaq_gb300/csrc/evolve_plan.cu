// Evolution plans: many states under one Hamiltonian, one CUDA graph per time step.
//
// A plan owns the work vectors for nrhs states.  run() records (once per (dt, s, m, psi), on a
// private capture stream) a graph of one time step -- 2^s sub-steps of m Taylor-term launches,
// each launch reading every matrix value once for all the states of a block of up to 8 -- and
// replays it `steps` times on the caller's stream.
//
// Modes
//  DIAQ_EVOLVE_C128   plain: complex128 matrix, vectors and sums (the reference's arithmetic).
//  DIAQ_EVOLVE_HORNER complex64 matrix; p(A) psi = psi + A (psi + A/2 (psi + ... A/m psi)),
//                     A = -i tau H, evaluated from the inside out in float32: each term reads
//                     the previous w and fp32(psi) and writes the next w; the outermost step
//                     adds A w_1 to psi in float64 and refreshes fp32(psi).
//  DIAQ_EVOLVE_MIXED  complex64 matrix and Taylor terms, the running sum of one sub-step kept as a
//                     compensated (hi, lo) pair of floats (TwoSum per term), and the state itself
//                     in float64: psi <- psi + (hi + lo) in double at the end of every sub-step.
//
// Buffers, with the terms of one step ping-ponging between two vectors (the last term of a
// sub-step writes the next sub-step's first input, fp32(psi), into the buffer the term would
// have used):
//   C128:  psi (caller's), sum, term_a, term_b                 (float64)
//   MIXED: psi (caller's, float64); v_a, v_b, hi, lo           (float32)
//
// Term kernels (the launch shape's `pipe` variant; the autotuner times the candidates once per
// plan shape and caches its choice): 0 the planar register kernel of spmv_kernel.cuh; 1-4 its
// float pipelines (cp.async, L2 prefetch, shuffled windows); 6-9 and 12 the states interleaved
// in 32-row tiles (spmv_il.cuh: 4 or 8 states per thread, an optional register ring of matrix
// values, 12 with compact 32-bit metadata -- the fastest on the 20-qubit chain); 10-11 the same
// fed through shared memory by bulk asynchronous copies (spmv_tma.cuh).  Every kernel skips the
// 32-row tiles of a diagonal that hold only zeros (the plan's zero-tile mask).
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
#include <tuple>

#include "spmv_il.cuh"
#include "spmv_pipe.cuh"
#include "spmv_tma.cuh"

namespace diaq_gb300 {

// ---- epilogues ---------------------------------------------------------------------------------------
// Plain term: term = (-i*scale) * (A x); out = base + term, base = init (first term) or `in`.
struct EpiPlain {
    double *tr, *ti;              // term out (NULL on a sub-step's last term: nobody reads it)
    const double *br, *bi;        // base of the sum
    double *outr, *outi;          // sum out
    int64_t ld;
    double scale;
    __host__ __device__ EpiPlain shifted(int q0) const {
        EpiPlain e = *this;
        const int64_t o = q0 * ld;
        if (e.tr) {
            e.tr += o;
            e.ti += o;
        }
        e.br += o;
        e.bi += o;
        e.outr += o;
        e.outi += o;
        return e;
    }
    template <typename U, int K, int V>
    __device__ __forceinline__ void apply(int64_t r0, int64_t rows, int kq, U (&sr)[K][V], U (&si)[K][V]) const {
#pragma unroll
        for (int q = 0; q < K; ++q)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int64_t r = r0 + v;
                if (q < kq && r < rows) {
                    const int64_t i = q * ld + r;
                    const double nr = si[q][v] * scale, ni = -sr[q][v] * scale;
                    if (tr) {
                        tr[i] = nr;
                        ti[i] = ni;
                    }
                    outr[i] = br[i] + nr;
                    outi[i] = bi[i] + ni;
                }
            }
    }
};

// Mixed term k of a sub-step: t = (-i*scale) * (A v) in float32;
//   k == 1:  hi = t, lo = 0;  else (hi, e) = TwoSum(hi, t), lo += e;
//   k <  m:  vout = t;
//   k == m:  psi += (double)hi + (double)lo;  vout = fp32(psi)  (next sub-step's input).
struct EpiMixed {
    float *vr, *vi;                     // vout
    float *hr, *hi_, *lr, *li;          // compensated sum (hi, lo), re and im
    double *pr, *pi;                    // state
    int64_t ld;
    float scale;
    int first, last;
    __host__ __device__ EpiMixed shifted(int q0) const {
        EpiMixed e = *this;
        const int64_t o = q0 * ld;
        e.vr += o;
        e.vi += o;
        e.hr += o;
        e.hi_ += o;
        e.lr += o;
        e.li += o;
        e.pr += o;
        e.pi += o;
        return e;
    }
    template <typename U, int K, int V>
    __device__ __forceinline__ void apply(int64_t r0, int64_t rows, int kq, U (&sr)[K][V], U (&si)[K][V]) const {
#pragma unroll
        for (int q = 0; q < K; ++q)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int64_t r = r0 + v;
                if (q >= kq || r >= rows) continue;
                const int64_t i = q * ld + r;
                const float tr = si[q][v] * scale, ti = -sr[q][v] * scale;
                float h_r, h_i, l_r, l_i;
                // plain loads and stores: part of the sums stays in L2 until the next launch reads
                // it (streaming them with evict-first hints measured 20 % slower)
                if (first) {
                    h_r = tr;
                    h_i = ti;
                    l_r = 0.f;
                    l_i = 0.f;
                } else {
                    float e_r, e_i;
                    two_sum(hr[i], tr, h_r, e_r);
                    two_sum(hi_[i], ti, h_i, e_i);
                    l_r = lr[i] + e_r;
                    l_i = li[i] + e_i;
                }
                if (!last) {
                    hr[i] = h_r;
                    hi_[i] = h_i;
                    lr[i] = l_r;
                    li[i] = l_i;
                    vr[i] = tr;
                    vi[i] = ti;
                } else {
                    const double nr = pr[i] + ((double)h_r + (double)l_r);
                    const double ni = pi[i] + ((double)h_i + (double)l_i);
                    pr[i] = nr;
                    pi[i] = ni;
                    vr[i] = (float)nr;
                    vi[i] = (float)ni;
                }
            }
    }
};

// One Horner step: w_out = fp32(psi) + (-i * scale) (A w_in); on the outermost step (last)
// psi += (-i * scale) (A w_1) in float64 and the fresh fp32(psi) goes to g (which is not the
// fp32(psi) this launch reads when the step's SpMV also reads it, m = 1).
// LAST = 0 / 1: a middle / the last step fixed at compile time (the kernels of middle steps then
// carry no float64 code); -1: the runtime field `last` decides.
template <int LAST = -1>
struct EpiHornerP {
    float *wr, *wi;                 // w out
    const float *fr, *fi;           // fp32(psi)
    double *pr, *pi;                // psi
    float *gr, *gi;                 // fp32(psi) written on the last step
    int64_t ld;
    float scale;
    int last;
    __host__ __device__ __forceinline__ bool is_last() const { return LAST < 0 ? last != 0 : LAST == 1; }
    __host__ __device__ EpiHornerP shifted(int q0) const {
        EpiHornerP e = *this;
        const int64_t o = q0 * ld;
        e.wr += o;
        e.wi += o;
        e.fr += o;
        e.fi += o;
        e.pr += o;
        e.pi += o;
        e.gr += o;
        e.gi += o;
        return e;
    }
    template <typename U, int K, int V>
    __device__ __forceinline__ void apply(int64_t r0, int64_t rows, int kq, U (&sr)[K][V], U (&si)[K][V]) const {
#pragma unroll
        for (int q = 0; q < K; ++q)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int64_t r = r0 + v;
                if (q >= kq || r >= rows) continue;
                const int64_t i = q * ld + r;
                const float tr = si[q][v] * scale, ti = -sr[q][v] * scale;
                if (!is_last()) {
                    wr[i] = __fadd_rn(fr[i], tr);  // unfused, as the interleaved epilogue
                    wi[i] = __fadd_rn(fi[i], ti);
                } else {
                    const double nr = pr[i] + (double)tr, ni = pi[i] + (double)ti;
                    pr[i] = nr;
                    pi[i] = ni;
                    gr[i] = (float)nr;
                    gi[i] = (float)ni;
                }
            }
    }
};

// Renormalisation in float64: per state, partial sums of |psi|^2 over row blocks (fixed order),
// then every block sums its state's partials and scales its rows; in the mixed mode it also
// refreshes the float32 copy the next step starts from.
constexpr int kNormBlocks = 256;

// Recorded time steps a plan keeps (one per (dt, s, m, state pointers, ld)).
constexpr size_t kMaxGraphs = 16;
// Bounds of the bulk-copy kernels' waits (variants 10, 11): one wait for a shared-memory stage, and
// the producer's wait for its copies in flight before its block may finish.
constexpr uint64_t kWaitNs = 20000000ull;   // 20 ms
constexpr uint64_t kDrainNs = 10000000ull;  // 10 ms

__global__ void norm_partial_kernel(const double *__restrict__ pr, const double *__restrict__ pi, int64_t n,
                                    double *__restrict__ part) {
    const int q = blockIdx.y;
    const double *a = pr + (int64_t)q * n, *b = pi + (int64_t)q * n;
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], a[i], fma(b[i], b[i], s));
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) part[q * kNormBlocks + blockIdx.x] = v;
    }
}

__global__ void renorm_kernel(double *__restrict__ pr, double *__restrict__ pi, float *__restrict__ fr,
                              float *__restrict__ fi, int64_t n, const double *__restrict__ part, int sp) {
    const int q = blockIdx.y;
    __shared__ double inv;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int j = 0; j < kNormBlocks; ++j) s += part[q * kNormBlocks + j];
        inv = s > 0.0 ? 1.0 / sqrt(s) : 1.0;
    }
    __syncthreads();
    const double c = inv;
    double *a = pr + (int64_t)q * n, *b = pi + (int64_t)q * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = a[i] * c, y = b[i] * c;
        a[i] = x;
        b[i] = y;
        if (fr) {  // the float32 copy: planar (sp = 0) or tiled interleaved
            const int64_t j = sp ? il_at(i, q >> 2, sp >> 2) + (q & 3) : (int64_t)q * n + i;
            fr[j] = (float)x;
            fi[j] = (float)y;
        }
    }
}

__global__ void to_f32_kernel(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// ---- interleaved states (kernel variants 6-9) -------------------------------------------------------
// The float32 work vectors of the float32 modes can hold the states interleaved in tiles: rows in
// blocks of 32, and within a block each quad of 4 states stored as 32 rows x 4 floats (512
// bytes).  Element (r, q) sits at ((r / 32) * (sp / 4) + q / 4) * 128 + (r mod 32) * 4 + q mod 4,
// sp = nrhs rounded up to a power of two >= 4 (at most 32; the padding states are zero) and the
// rows padded to a multiple of 32.  A warp works on 32 consecutive rows and one or two quads: its
// state window at any diagonal offset is one or two contiguous 512-byte runs (one 16-byte load
// per lane and quad), its matrix values 128 contiguous bytes, and its epilogue reads and writes
// contiguous quads too.  (The planar layout splits the windows of offsets that are not multiples
// of 4; a row-major interleave spreads a warp's window over sp * 128 bytes.)

// psi (state q at p[q * ld + r]) -> tiled float32, padding states and rows zero.
__global__ void to_f32_il_kernel(const double *__restrict__ pr, const double *__restrict__ pi, int64_t ld,
                                 int64_t n, int64_t n_pad, int nrhs, int sp, float *__restrict__ fr,
                                 float *__restrict__ fi) {
    const int64_t cnt = n_pad * sp;
    const int quads = sp >> 2;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t blk = e / (quads * 128);
        const int rem = (int)(e - blk * quads * 128);
        const int quad = rem >> 7, lr = (rem & 127) >> 2, c = rem & 3;
        const int64_t r = blk * 32 + lr;
        const int q = quad * 4 + c;
        const bool live = r < n && q < nrhs;
        fr[e] = live ? (float)pr[q * ld + r] : 0.f;
        fi[e] = live ? (float)pi[q * ld + r] : 0.f;
    }
}

// Thread mapping: warp w of a block takes quad group g = w mod (sp/G) of the 32 rows of row
// block (block * 8 / (sp/G) + w / (sp/G)); lane l takes row 32 * (that row block) + l.
//
// D > 0: the matrix values (one float per plane and row) of the next D diagonals are loaded
// into a register ring ahead of use, so a thread has D HBM reads of the matrix stream in flight
// and waits on each diagonal only for its state windows (L2 hits, mostly).
//
// G states per thread (4 or 8; sp a multiple of G): with 8, a warp covers 8 states of its rows --
// one matrix load per row and diagonal, two window vectors per plane.  (Several rows per thread,
// for a wider tile, measured slower: 2.86-3.89 ms per step against 2.53 on the 20-qubit chain.)
//
// (Two diagonals per iteration, every load of both issued before their FMAs, measured 2.34 against
// 2.29 ms per Horner step: 64 registers, 4 blocks per SM, no gain.)
template <class Epi, int D, int G = 4>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_spmv_il_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ are,
                       const float *__restrict__ aim, int64_t rows, const float *__restrict__ xr,
                       const float *__restrict__ xi, const uint32_t *__restrict__ tmask, int64_t mw, Epi epi) {
    static_assert(G == 4 || G == 8, "4 or 8 states per thread");
    __shared__ DiagMeta sm[kMetaChunk];
    __shared__ uint32_t smk[kMetaChunk];  // zero-tile mask word of the block rows, per diagonal
    const int quads = epi.sp >> 2, groups = epi.sp / G;
    const int wid = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int g = wid % groups;
    const int64_t row0 = (int64_t)blockIdx.x * (8 / groups) * 32;  // <= 256 rows: one mask word
    const int64_t r = row0 + (wid / groups) * 32 + lane;
    const int tbit = (int)((r >> 5) & 31);
    float accr[G], acci[G];
#pragma unroll
    for (int q = 0; q < G; ++q) accr[q] = acci[q] = 0.f;
    auto term = [&](const DiagMeta &m, float a, float b) {
        il_term<G>(r + m.off, g * (G / 4), quads, a, b, xr, xi, accr, acci);
    };
    for (int c0 = 0; c0 < nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, nd - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < cn; i += kSpmvThreads) {
            sm[i] = meta[c0 + i];
            smk[i] = tmask ? tmask[(int64_t)(c0 + i) * mw + (row0 >> 10)] : 0xffffffffu;
        }
        __syncthreads();
        if (r >= rows) continue;
        // a warp's 32 rows are one tile: the whole warp skips a zero tile
        auto live = [&](int k) { return r >= sm[k].lo && r < sm[k].hi && ((smk[k] >> tbit) & 1u); };
        if constexpr (D == 0) {
#pragma unroll 4
            for (int k = 0; k < cn; ++k) {
                if (!live(k)) continue;
                term(sm[k], __ldcs(are + sm[k].base + r), __ldcs(aim + sm[k].base + r));
            }
        } else {
            // ring slot d holds diagonal k0 + d; rows outside a diagonal load nothing (value 0)
            float ra[D], rb[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const bool in = d < cn && live(d);
                ra[d] = in ? __ldcs(are + sm[d].base + r) : 0.f;
                rb[d] = in ? __ldcs(aim + sm[d].base + r) : 0.f;
            }
            for (int k0 = 0; k0 < cn; k0 += D) {
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const int k = k0 + d;
                    if (k < cn) {
                        const float a = ra[d], b = rb[d];
                        const int kn = k + D;
                        const bool in = kn < cn && live(kn);
                        ra[d] = in ? __ldcs(are + sm[kn].base + r) : 0.f;
                        rb[d] = in ? __ldcs(aim + sm[kn].base + r) : 0.f;
                        if (live(k)) term(sm[k], a, b);
                    }
                }
            }
        }
    }
    if (r >= rows) return;
#pragma unroll
    for (int h = 0; h < G / 4; ++h) {  // the epilogue works on quads of states
        const float ar4[4] = {accr[4 * h], accr[4 * h + 1], accr[4 * h + 2], accr[4 * h + 3]};
        const float ai4[4] = {acci[4 * h], acci[4 * h + 1], acci[4 * h + 2], acci[4 * h + 3]};
        epi.apply(r, g * (G / 4) + h, ar4, ai4);
    }
}

// Variant 12: variant 9's loop with 32-bit row and window arithmetic (n_pad * sp < 2^31) and the
// per-diagonal metadata the loop reads -- offset, row range and the block's mask word -- packed
// in one 16-byte shared-memory record, the value base in a second array: fewer registers and one
// shared-memory load per diagonal.
//
// Further measures, all bit-neutral:
// - An epilogue that reads an fp32(psi) quad per plane and row (the Horner middle step,
//   Epi::kPsiTile) gets it from shared memory: each lane copies its quads with cp.async when the
//   warp starts and waits for them only after its diagonal loop, so the epilogue no longer stalls
//   on an HBM read at the end of every warp (106.5 -> 102.9 us per 8-state term on the 20-qubit
//   chain, in isolation).
// - When the block count is a multiple of 4, consecutive blocks take row blocks b, b + B/4,
//   b + B/2, b + 3B/4 (B blocks): the blocks resident together spread over four distant parts of
//   the rows (-2 %).
// - Right after the metadata barrier, lane i / 8 of warp i % 8 asks L2 for diagonal i's values in
//   the block's live tiles (bulk prefetches, one per run of live tiles and plane), and thread 0,
//   at block start, for the block's own rows of the input states: the warps' matrix loads of the
//   later diagonals then hit L2 (104.6 -> 93.5 us per 8-state term, 201 -> 171 us for 16 states;
//   issued by the staging threads before the barrier, where the other warps waited on them:
//   100.1 us).  Asking for the tiles of the block that launches one resident wave later instead
//   made it slower (117 us), and so did asking with each live run for the state windows it reads
//   (111 us); asking at block start for the float64 states of the last step's epilogue changed
//   nothing.
// - The multiply-adds run two states per instruction (il_fma's packed form, __ffma2_rn): 58.0 M
//   instead of 67.5 M instructions per launch, 93.1 -> 91.1 us per 8-state term.
// - The Horner epilogue's middle and last steps are separate instantiations (EpiHornerT<0> and
//   <1>): the middle steps' kernel holds no float64 code.
template <class Epi, int G, int MINB>
__global__ void __launch_bounds__(kSpmvThreads, MINB)
    dia_spmv_il32_kernel(const DiagMeta *__restrict__ meta, int nd, const float *__restrict__ are,
                         const float *__restrict__ aim, int rows, const float *__restrict__ xr,
                         const float *__restrict__ xi, const uint32_t *__restrict__ tmask, int64_t mw, Epi epi) {
    static_assert(G == 4 || G == 8, "4 or 8 states per thread");
    constexpr bool kTile = Epi::kPsiTile;
    __shared__ int4 sq[kMetaChunk];       // off, lo, hi, mask word
    __shared__ int64_t sb[kMetaChunk];    // base
    __shared__ __align__(16) float4 spsi[kTile ? kSpmvThreads / 32 : 1][G / 4][2][32];
    const int quads = epi.sp >> 2, groups = epi.sp / G;
    const int wid = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int g = wid % groups;
    const unsigned nb = gridDim.x;
    const int bi = (nb & 3u) ? (int)blockIdx.x : (int)((blockIdx.x & 3u) * (nb >> 2) + (blockIdx.x >> 2));
    const int row0 = bi * (8 / groups) * 32;
    const int r = row0 + (wid / groups) * 32 + lane;
    float accr[G], acci[G];
#pragma unroll
    for (int q = 0; q < G; ++q) accr[q] = acci[q] = 0.f;
    bool tile = false;
    if constexpr (kTile) {
        tile = epi.reads_psi() && r < rows;
        if (tile) {
#pragma unroll
            for (int h = 0; h < G / 4; ++h) {
                const int64_t i = il_at(r, g * (G / 4) + h, quads);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                 (uint32_t)__cvta_generic_to_shared(&spsi[wid][h][0][lane])),
                             "l"(epi.fr + i)
                             : "memory");
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                 (uint32_t)__cvta_generic_to_shared(&spsi[wid][h][1][lane])),
                             "l"(epi.fi + i)
                             : "memory");
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    if (threadIdx.x == 0 && row0 < rows) {
        // the block's own rows of the input states (all quads: one contiguous run per plane),
        // inside the rows padded to 32
        const int64_t at = (int64_t)(row0 >> 5) * quads * 128;
        const int tiles = min(8 / groups, (rows + 31 - row0) >> 5);
        const uint32_t bytes = (uint32_t)tiles * (uint32_t)quads * 512u;
        prefetch_l2(xr + at, bytes);
        prefetch_l2(xi + at, bytes);
    }
    for (int c0 = 0; c0 < nd; c0 += kMetaChunk) {
        const int cn = min(kMetaChunk, nd - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < cn; i += kSpmvThreads) {
            const DiagMeta m = meta[c0 + i];
            const uint32_t w = tmask ? tmask[(int64_t)(c0 + i) * mw + (row0 >> 10)] : 0xffffffffu;
            sq[i] = make_int4(m.off, (int)m.lo, (int)m.hi, (int)w);
            sb[i] = m.base;
        }
        __syncthreads();
        {
            // the block's tiles of diagonal i (inside one mask word), asked for after the barrier
            // by lane i / 8 of warp i % 8, so that no warp waits on them
            const int i = lane * 8 + wid;
            if (i < cn) {
                const int4 q = sq[i];
                prefetch_tiles_l2(are, aim, sb[i], (int64_t)q.y, (int64_t)q.z,
                                  block_tile_bits((uint32_t)q.w, row0, 8 / groups), row0);
            }
        }
        if (r >= rows) continue;
        il_accumulate32<G, true>(sq, sb, cn, r, g * (G / 4), quads, are, aim, xr, xi, accr, acci);
    }
    if constexpr (kTile) asm volatile("cp.async.wait_all;" ::: "memory");
    if (r >= rows) return;
#pragma unroll
    for (int h = 0; h < G / 4; ++h) {
        const float ar4[4] = {accr[4 * h], accr[4 * h + 1], accr[4 * h + 2], accr[4 * h + 3]};
        const float ai4[4] = {acci[4 * h], acci[4 * h + 1], acci[4 * h + 2], acci[4 * h + 3]};
        if constexpr (kTile) {
            if (tile) {
                epi.apply_psi(r, g * (G / 4) + h, ar4, ai4, spsi[wid][h][0][lane], spsi[wid][h][1][lane]);
                continue;
            }
        }
        epi.apply(r, g * (G / 4) + h, ar4, ai4);
    }
}

// ---- the plan ------------------------------------------------------------------------------------------
struct EvolvePlan {
    const Matrix *H = nullptr;   // the caller's matrix (c128)
    Matrix *Hc = nullptr;        // c64 copy (float32-term modes)
    bool owns_hc = true;         // Hc and tmask are this plan's own (else borrowed from the plan that owns this one)
    int mode = 0, nrhs = 1;
    int64_t n = 0;
    void *buf = nullptr;         // work vectors
    cudaStream_t s = nullptr;    // capture stream
    // diaq_evolve_run_host: the real and the imaginary planes are copied on two streams at once
    // (two copy engines), the run itself on the first
    cudaStream_t hs[2] = {nullptr, nullptr};
    cudaEvent_t hev[2] = {nullptr, nullptr};
    struct Key {
        double dt;
        int sl, m;
        double *pr, *pi;
        int64_t ld;
        bool operator<(const Key &o) const {
            return std::tie(dt, sl, m, pr, pi, ld) < std::tie(o.dt, o.sl, o.m, o.pr, o.pi, o.ld);
        }
    };
    std::map<Key, cudaGraphExec_t> graphs;   // one recorded step per key, at most kMaxGraphs
    int launches_per_step = 0;
    SpmvCfg cfg;          // launch shape of the term kernel
    bool tuned = false;   // cfg chosen (by the autotuner or the caller)
    bool renorm = false;  // rescale every state to norm 1 (float64) after each step
    double *part = nullptr;  // renormalisation partial sums, nrhs * kNormBlocks
    uint32_t *tmask = nullptr;  // zero-tile mask of the matrix the term kernels read (Hc, or H for C128)
    int *err = nullptr;           // bounded waits of the bulk-copy kernels (variants 10, 11) record here
    int *err_host = nullptr;      // pinned copy of *err taken after each run
    cudaEvent_t err_ev = nullptr; // ... and the event that says it has landed
    uint64_t wait_ns = kWaitNs;   // bound of one wait of the bulk-copy kernels
    int sp = 4;           // interleaved layout: nrhs rounded up to a power of two >= 4 (<= 32 used)
    int64_t n_pad = 0;    // rows rounded up to a multiple of 32
    double *stage = nullptr;  // device copy of the states for diaq_evolve_run_host, 2 * nrhs * n
    // diaq_evolve_run_host, one step of an even number (>= 8) of float32-term states: two plans
    // for the two halves of the states, run one after the other on stream hcomp while the second
    // half is copied up and the first copied down (events hsev)
    EvolvePlan *half[2] = {nullptr, nullptr};
    cudaStream_t hcomp = nullptr;
    cudaEvent_t hsev[4] = {nullptr, nullptr, nullptr, nullptr};

    bool f32() const { return mode == DIAQ_EVOLVE_MIXED || mode == DIAQ_EVOLVE_HORNER; }
    bool interleaved() const { return f32() && cfg.pipe >= 6; }
    // floats per float32 work vector (all states)
    int64_t vlen() const { return interleaved() ? (int64_t)sp * n_pad : (int64_t)nrhs * n; }

    ~EvolvePlan() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        if (buf) cudaFree(buf);
        if (part) cudaFree(part);
        if (tmask && owns_hc) cudaFree(tmask);
        if (err) cudaFree(err);
        if (err_host) cudaFreeHost(err_host);
        if (err_ev) cudaEventDestroy(err_ev);
        if (stage) cudaFree(stage);
        if (Hc && owns_hc) destroy(Hc);
        if (s) cudaStreamDestroy(s);
        for (int j = 0; j < 2; ++j) {
            if (hs[j]) cudaStreamDestroy(hs[j]);
            if (hev[j]) cudaEventDestroy(hev[j]);
            delete half[j];
        }
        if (hcomp) cudaStreamDestroy(hcomp);
        for (auto ev : hsev)
            if (ev) cudaEventDestroy(ev);
    }
};

}  // namespace diaq_gb300

// The public handle is the plan itself; every plan is allocated as one.
struct diaq_evolve_s : public diaq_gb300::EvolvePlan {};

namespace diaq_gb300 {

// The interleaved kernel for plan variant 6 (no ring), 7 (ring of 4), 8 (ring of 8), 9 (8
// states per thread; 4 when the padded state count is 4) or 10 (bulk copies through shared
// memory, spmv_tma.cuh; 8 or 4 states per thread as 9; the register kernel of 9 when the matrix
// has more diagonals than one metadata chunk).
template <class Epi>
int launch_il(const EvolvePlan &P, const float *xr, const float *xi, const Epi &e) {
    const int v = P.cfg.pipe;
    const bool eight = v >= 9 && P.sp % 8 == 0;
    if (v == 12 && (int64_t)P.n_pad * P.sp < ((int64_t)1 << 31)) {
        const int groups = P.sp / (eight ? 8 : 4);
        const int64_t rows_per_block = 32 * (8 / groups);
        const unsigned g = (unsigned)((P.n_pad + rows_per_block - 1) / rows_per_block);
        const float *are = (const float *)P.Hc->re, *aim = (const float *)P.Hc->im;
        const int64_t mw = tile_mask_words(P.n);
        // blocks per SM: 5 (48 registers) for 8 states per thread -- 107.7 us per 8-state term on
        // the 20-qubit chain, against 112.9 at 6 (40 registers and spills)
        if (eight)
            dia_spmv_il32_kernel<Epi, 8, 5><<<g, kSpmvThreads, 0, P.s>>>(P.Hc->d_meta, P.Hc->nd, are, aim, (int)P.n, xr,
                                                                         xi, P.tmask, mw, e);
        else
            dia_spmv_il32_kernel<Epi, 4, 6><<<g, kSpmvThreads, 0, P.s>>>(P.Hc->d_meta, P.Hc->nd, are, aim, (int)P.n, xr,
                                                                         xi, P.tmask, mw, e);
        DQ_CUDA(cudaGetLastError());
        return DIAQ_OK;
    }
    if ((v == 10 || v == 11) && P.Hc->nd <= kMetaChunk) {
        const int G = P.sp % 8 == 0 ? 8 : 4;
        const int R = 32 * (8 / (P.sp / G));
        const unsigned gt = (unsigned)((P.n_pad + R - 1) / R);
        const bool win = v == 10;
        const size_t smem = tma_smem_bytes(R, P.sp, win, win ? 4 : 8);
        const float *are = (const float *)P.Hc->re, *aim = (const float *)P.Hc->im;
        const int64_t mw = tile_mask_words(P.n);
        const DiagMeta *md = P.Hc->d_meta;
        const int nd = P.Hc->nd;
        // a copy lands within microseconds: the drain bound is generous whatever the wait bound
        const uint64_t wn = P.wait_ns, dn = std::max<uint64_t>(P.wait_ns, kDrainNs);
        if (G == 8 && win)
            dia_spmv_tma_kernel<Epi, 8, true, 4><<<gt, kTmaThreads, smem, P.s>>>(md, nd, are, aim, P.n, P.n_pad, xr, xi,
                                                                                 P.tmask, mw, e, P.err, wn, dn);
        else if (G == 8)
            dia_spmv_tma_kernel<Epi, 8, false, 8><<<gt, kTmaThreads, smem, P.s>>>(md, nd, are, aim, P.n, P.n_pad, xr, xi,
                                                                                  P.tmask, mw, e, P.err, wn, dn);
        else if (win)
            dia_spmv_tma_kernel<Epi, 4, true, 4><<<gt, kTmaThreads, smem, P.s>>>(md, nd, are, aim, P.n, P.n_pad, xr, xi,
                                                                                 P.tmask, mw, e, P.err, wn, dn);
        else
            dia_spmv_tma_kernel<Epi, 4, false, 8><<<gt, kTmaThreads, smem, P.s>>>(md, nd, are, aim, P.n, P.n_pad, xr, xi,
                                                                                  P.tmask, mw, e, P.err, wn, dn);
        DQ_CUDA(cudaGetLastError());
        return DIAQ_OK;
    }
    const int groups = P.sp / (eight ? 8 : 4);          // warps per row block of 32: 1, 2, 4 or 8
    const int64_t rows_per_block = 32 * (8 / groups);
    const unsigned g = (unsigned)((P.n_pad + rows_per_block - 1) / rows_per_block);
    const float *are = (const float *)P.Hc->re, *aim = (const float *)P.Hc->im;
    const DiagMeta *md = P.Hc->d_meta;
    const int nd = P.Hc->nd;
    const uint32_t *tm = P.tmask;
    const int64_t mw = tile_mask_words(P.n);
    if (eight)
        dia_spmv_il_kernel<Epi, 0, 8><<<g, kSpmvThreads, 0, P.s>>>(md, nd, are, aim, P.n, xr, xi, tm, mw, e);
    else if (v == 7)
        dia_spmv_il_kernel<Epi, 4><<<g, kSpmvThreads, 0, P.s>>>(md, nd, are, aim, P.n, xr, xi, tm, mw, e);
    else if (v == 8)
        dia_spmv_il_kernel<Epi, 8><<<g, kSpmvThreads, 0, P.s>>>(md, nd, are, aim, P.n, xr, xi, tm, mw, e);
    else
        dia_spmv_il_kernel<Epi, 0><<<g, kSpmvThreads, 0, P.s>>>(md, nd, are, aim, P.n, xr, xi, tm, mw, e);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// The bulk-copy kernels hold up to kTmaStages stages of 25 KB of dynamic shared memory: raise
// their limit once, before any launch is recorded.
template <class Epi>
static int allow_tma_smem() {
    const int b = 128 * 1024;
    DQ_CUDA(cudaFuncSetAttribute(dia_spmv_tma_kernel<Epi, 8, true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    DQ_CUDA(cudaFuncSetAttribute(dia_spmv_tma_kernel<Epi, 4, true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    return DIAQ_OK;
}

// share: a float32-term plan of the same matrix whose c64 copy and zero-tile mask the new plan
// borrows instead of making its own (the half plans of diaq_evolve_run_host); NULL: its own.
static int plan_create(const Matrix &H, int nrhs, int mode, EvolvePlan **out, const EvolvePlan *share = nullptr) {
    if (H.rows != H.cols) return set_error(DIAQ_ERR_INVALID, "evolve: H must be square");
    if (H.prec != DIAQ_C128) return set_error(DIAQ_ERR_INVALID, "evolve: pass the c128 matrix (the plan makes its own c64 copy)");
    if (nrhs < 1) return set_error(DIAQ_ERR_INVALID, "evolve: nrhs must be >= 1");
    if (mode != DIAQ_EVOLVE_C128 && mode != DIAQ_EVOLVE_MIXED && mode != DIAQ_EVOLVE_HORNER)
        return set_error(DIAQ_ERR_INVALID, "evolve: unknown mode");
    EvolvePlan *P = new diaq_evolve_s();
    P->H = &H;
    P->mode = mode;
    P->nrhs = nrhs;
    P->n = H.rows;
    P->sp = 4;
    while (P->sp < nrhs) P->sp *= 2;
    P->n_pad = (P->n + 31) / 32 * 32;
    int st = DIAQ_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&P->s, cudaStreamNonBlocking);
    const size_t vec = (size_t)nrhs * (size_t)P->n;
    // the mixed mode sizes its 8 float vectors for the interleaved layout (>= nrhs states)
    const size_t bytes = mode == DIAQ_EVOLVE_C128 ? 6 * vec * sizeof(double)
                                                  : 8 * std::max<size_t>((size_t)P->sp * (size_t)P->n_pad,
                                                                         vec) * sizeof(float);
    if (e == cudaSuccess && bytes) e = dev_malloc(&P->buf, bytes);
    if (e != cudaSuccess) st = cuda_status(e, "evolve plan", __FILE__, __LINE__);
    const bool borrow = share && share->Hc && mode != DIAQ_EVOLVE_C128;
    if (borrow) {
        P->Hc = share->Hc;
        P->tmask = share->tmask;
        P->owns_hc = false;
    }
    if (st == DIAQ_OK && mode != DIAQ_EVOLVE_C128 && !borrow) st = copy_as(H, DIAQ_C64, P->s, &P->Hc);
    if (st == DIAQ_OK && mode == DIAQ_EVOLVE_MIXED) st = allow_tma_smem<EpiMixedIL>();
    if (st == DIAQ_OK && mode == DIAQ_EVOLVE_HORNER) st = allow_tma_smem<EpiHornerT<0>>();
    if (st == DIAQ_OK && mode == DIAQ_EVOLVE_HORNER) st = allow_tma_smem<EpiHornerT<1>>();
    if (st == DIAQ_OK) {
        e = dev_malloc(&P->err, sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(P->err, 0, sizeof(int), P->s);
        if (e == cudaSuccess) e = cudaMallocHost(&P->err_host, sizeof(int));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->err_ev, cudaEventDisableTiming);
        if (e == cudaSuccess) *P->err_host = 0;
        if (e != cudaSuccess) st = cuda_status(e, "evolve plan", __FILE__, __LINE__);
    }
    if (st == DIAQ_OK && H.nd > 0 && !borrow) {
        // the mask of the plan's own c64 copy is built once; that of the caller's c128 matrix
        // again at every run (its values may have changed)
        e = dev_malloc(&P->tmask, sizeof(uint32_t) * (size_t)H.nd * (size_t)tile_mask_words(H.rows));
        if (e != cudaSuccess) st = cuda_status(e, "evolve plan mask", __FILE__, __LINE__);
        if (st == DIAQ_OK) st = build_tile_mask(P->Hc ? *P->Hc : H, P->tmask, P->s);
        if (st == DIAQ_OK && (e = cudaStreamSynchronize(P->s)) != cudaSuccess)
            st = cuda_status(e, "evolve plan mask", __FILE__, __LINE__);
    }
    if (st != DIAQ_OK) {
        delete static_cast<diaq_evolve_s *>(P);
        return st;
    }
    *out = P;
    return DIAQ_OK;
}

// The partial sums of the renormalisation; allocated before any step is recorded (no
// allocation is allowed while a stream is being captured).
static int ensure_renorm_buffer(EvolvePlan &P) {
    if (P.renorm && !P.part) DQ_CUDA(dev_malloc(&P.part, sizeof(double) * kNormBlocks * P.nrhs));
    return DIAQ_OK;
}

static int enqueue_renorm(EvolvePlan &P, double *pr, double *pi, float *fr, float *fi) {
    if (!P.renorm) return DIAQ_OK;
    if (!P.part) return set_error(DIAQ_ERR_INVALID, "evolve: renormalisation buffer missing");
    const dim3 g(kNormBlocks, (unsigned)P.nrhs);
    norm_partial_kernel<<<g, 256, 0, P.s>>>(pr, pi, P.n, P.part);
    renorm_kernel<<<g, 256, 0, P.s>>>(pr, pi, fr, fi, P.n, P.part, P.interleaved() ? P.sp : 0);
    DQ_CUDA(cudaGetLastError());
    P.launches_per_step += 2;
    return DIAQ_OK;
}

// Enqueue one time step on P->s (used under stream capture).
static int enqueue_step(EvolvePlan &P, double dt, int sl, int m, double *pr, double *pi, int64_t ld) {
    const int64_t n = P.n, k = P.nrhs;
    const int sub = 1 << sl;
    const double tau = dt / (double)sub;
    P.launches_per_step = 0;
    if (P.mode == DIAQ_EVOLVE_C128) {
        double *w = (double *)P.buf;
        const int64_t L = n;  // work vectors use ld = n
        double *sr = w, *si = w + k * L, *ar = w + 2 * k * L, *ai = w + 3 * k * L, *br = w + 4 * k * L,
               *bi = w + 5 * k * L;
        // work vectors have leading dimension n; the caller's psi uses ld.  The first term of a
        // sub-step reads psi; keep the caller's layout by requiring ld == n here.
        if (ld != n) return set_error(DIAQ_ERR_UNSUPPORTED, "evolve c128: psi leading dimension must equal N");
        double *cur_r = pr, *cur_i = pi, *oth_r = sr, *oth_i = si;
        for (int j = 0; j < sub; ++j) {
            const double *tin_r = cur_r, *tin_i = cur_i;
            double *tout_r = ar, *tout_i = ai;
            for (int t = 1; t <= m; ++t) {
                EpiPlain e;
                const bool last = (t == m);
                e.tr = last ? nullptr : tout_r;
                e.ti = last ? nullptr : tout_i;
                e.br = (t == 1) ? cur_r : oth_r;
                e.bi = (t == 1) ? cur_i : oth_i;
                e.outr = oth_r;
                e.outi = oth_i;
                e.ld = L;
                e.scale = tau / (double)t;
                DQ_TRY((launch_dia_spmv_rhs_cfg<double, EpiPlain, 2, 1>(*P.H, tin_r, tin_i, L, (int)k, e, P.s, P.cfg, P.tmask)));
                ++P.launches_per_step;
                tin_r = tout_r;
                tin_i = tout_i;
                tout_r = (tout_r == ar) ? br : ar;
                tout_i = (tout_i == ai) ? bi : ai;
            }
            if (m == 0) continue;
            std::swap(cur_r, oth_r);
            std::swap(cur_i, oth_i);
        }
        if (cur_r != pr) {
            DQ_CUDA(cudaMemcpyAsync(pr, cur_r, sizeof(double) * k * L, cudaMemcpyDeviceToDevice, P.s));
            DQ_CUDA(cudaMemcpyAsync(pi, cur_i, sizeof(double) * k * L, cudaMemcpyDeviceToDevice, P.s));
        }
        return enqueue_renorm(P, pr, pi, nullptr, nullptr);
    }
    if (P.mode == DIAQ_EVOLVE_HORNER) {
        float *w = (float *)P.buf;
        const int64_t L = n, VL = P.vlen();
        if (ld != n) return set_error(DIAQ_ERR_UNSUPPORTED, "evolve horner: psi leading dimension must equal N");
        float *fr = w, *fi = w + VL, *war = w + 2 * VL, *wai = w + 3 * VL, *wbr = w + 4 * VL, *wbi = w + 5 * VL;
        for (int j = 0; j < sub; ++j) {
            const float *in_r = fr, *in_i = fi;  // w_m = psi
            float *out_r = war, *out_i = wai;
            for (int t = 1; t <= m; ++t) {
                const float scale = (float)(tau / (double)(m - t + 1));
                const bool last = (t == m);
                // the last step refreshes fp32(psi); when it also reads fp32(psi) (m = 1) it writes
                // the fresh copy to the free w vector, copied back after the launch
                float *gr = (last && in_r == fr) ? out_r : fr, *gi = (last && in_r == fr) ? out_i : fi;
                // middle and last steps are separate kernel instantiations (EpiHorner*<0> / <1>)
                if (P.interleaved()) {
                    if (last) {
                        EpiHornerT<1> e{out_r, out_i, fr, fi, gr, gi, pr, pi, ld, P.sp, (int)k, scale, 1};
                        DQ_TRY(launch_il(P, in_r, in_i, e));
                    } else {
                        EpiHornerT<0> e{out_r, out_i, fr, fi, gr, gi, pr, pi, ld, P.sp, (int)k, scale, 0};
                        DQ_TRY(launch_il(P, in_r, in_i, e));
                    }
                } else if (last) {
                    EpiHornerP<1> e{out_r, out_i, fr, fi, pr, pi, gr, gi, L, scale, 1};
                    DQ_TRY((launch_dia_spmv_rhs_cfg<float, EpiHornerP<1>, 4, 2, 1>(*P.Hc, in_r, in_i, L, (int)k, e,
                                                                                P.s, P.cfg, P.tmask)));
                } else {
                    EpiHornerP<0> e{out_r, out_i, fr, fi, pr, pi, gr, gi, L, scale, 0};
                    DQ_TRY((launch_dia_spmv_rhs_cfg<float, EpiHornerP<0>, 4, 2, 1>(*P.Hc, in_r, in_i, L, (int)k, e,
                                                                                P.s, P.cfg, P.tmask)));
                }
                ++P.launches_per_step;
                if (gr != fr) {
                    DQ_CUDA(cudaMemcpyAsync(fr, gr, sizeof(float) * VL, cudaMemcpyDeviceToDevice, P.s));
                    DQ_CUDA(cudaMemcpyAsync(fi, gi, sizeof(float) * VL, cudaMemcpyDeviceToDevice, P.s));
                }
                in_r = out_r;
                in_i = out_i;
                out_r = (out_r == war) ? wbr : war;
                out_i = (out_i == wai) ? wbi : wai;
            }
        }
        return enqueue_renorm(P, pr, pi, fr, fi);
    }
    // MIXED
    float *w = (float *)P.buf;
    const int64_t L = n, VL = P.vlen();
    if (ld != n) return set_error(DIAQ_ERR_UNSUPPORTED, "evolve mixed: psi leading dimension must equal N");
    float *var = w, *vai = w + VL, *vbr = w + 2 * VL, *vbi = w + 3 * VL;
    float *hr = w + 4 * VL, *hi = w + 5 * VL, *lr = w + 6 * VL, *li = w + 7 * VL;
    float *in_r = var, *in_i = vai, *out_r = vbr, *out_i = vbi;  // v_a holds fp32(psi) on entry
    for (int j = 0; j < sub; ++j) {
        for (int t = 1; t <= m; ++t) {
            if (P.interleaved()) {
                EpiMixedIL e{out_r, out_i, hr, hi, lr, li, pr, pi, ld, P.sp, (int)k, (float)(tau / (double)t),
                             t == 1, t == m};
                DQ_TRY(launch_il(P, in_r, in_i, e));
                ++P.launches_per_step;
                std::swap(in_r, out_r);
                std::swap(in_i, out_i);
                continue;
            }
            EpiMixed e;
            e.vr = out_r;
            e.vi = out_i;
            e.hr = hr;
            e.hi_ = hi;
            e.lr = lr;
            e.li = li;
            e.pr = pr;
            e.pi = pi;
            e.ld = L;
            e.scale = (float)(tau / (double)t);
            e.first = (t == 1);
            e.last = (t == m);
            if (P.cfg.pipe >= 2) {
                DQ_TRY(launch_dia_spmv_pf<EpiMixed>(*P.Hc, in_r, in_i, L, (int)k, e, P.s, P.cfg.kmax, P.cfg.pipe,
                                                    &P.launches_per_step));
            } else if (P.cfg.pipe == 1) {
                DQ_TRY(launch_dia_spmv_pipe<EpiMixed>(*P.Hc, in_r, in_i, L, (int)k, e, P.s, P.cfg.kmax,
                                                      &P.launches_per_step));
            } else {
                DQ_TRY((launch_dia_spmv_rhs_cfg<float, EpiMixed, 4, 2, 1>(*P.Hc, in_r, in_i, L, (int)k, e, P.s, P.cfg, P.tmask)));
                ++P.launches_per_step;  // one launch over all states
            }
            std::swap(in_r, out_r);
            std::swap(in_i, out_i);
        }
    }
    if (in_r != var) {  // an odd number of launches: put fp32(psi) back where the next step reads it
        DQ_CUDA(cudaMemcpyAsync(var, in_r, sizeof(float) * VL, cudaMemcpyDeviceToDevice, P.s));
        DQ_CUDA(cudaMemcpyAsync(vai, in_i, sizeof(float) * VL, cudaMemcpyDeviceToDevice, P.s));
    }
    return enqueue_renorm(P, pr, pi, var, vai);
}

// fp32(psi) into v_a, in the layout of the plan's current kernel (psi with leading dimension n).
static int fp32_state(EvolvePlan &P, const double *pr, const double *pi, cudaStream_t s) {
    float *var = (float *)P.buf, *vai = var + P.vlen();
    if (P.interleaved()) {
        const int64_t cnt = P.n_pad * P.sp;
        const int grid = (int)std::min<int64_t>((cnt + 255) / 256, 8 * num_sms());
        to_f32_il_kernel<<<grid, 256, 0, s>>>(pr, pi, P.n, P.n, P.n_pad, P.nrhs, P.sp, var, vai);
    } else {
        const int64_t cnt = P.nrhs * P.n;
        const int grid = (int)std::min<int64_t>((cnt + 255) / 256, 8 * num_sms());
        to_f32_kernel<<<grid, 256, 0, s>>>(pr, var, cnt);
        to_f32_kernel<<<grid, 256, 0, s>>>(pi, vai, cnt);
    }
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

// Clear the bulk-copy kernels' error flag (device and pinned copy).
static int clear_wait_error(EvolvePlan &P) {
    *P.err_host = 0;
    DQ_CUDA(cudaMemsetAsync(P.err, 0, sizeof(int), P.s));
    DQ_CUDA(cudaStreamSynchronize(P.s));
    return DIAQ_OK;
}

// DIAQ_ERR_TIMEOUT, and the flag cleared, when a wait of a bulk-copy kernel (variants 10, 11) of
// an earlier run gave up; that run's states are then not advanced correctly.  sync: wait for the
// last run's copy of the flag; else look only if it has landed.
static int take_wait_error(EvolvePlan &P, bool sync) {
    if (sync) {
        const cudaError_t e = cudaEventSynchronize(P.err_ev);
        if (e != cudaSuccess) return cuda_status(e, "evolve: wait for the run", __FILE__, __LINE__);
    } else if (cudaEventQuery(P.err_ev) != cudaSuccess) {
        return DIAQ_OK;
    }
    const int code = *P.err_host;
    if (code == 0) return DIAQ_OK;
    DQ_TRY(clear_wait_error(P));
    const char *what = code == 2 ? "a consumer warp's wait for a filled stage"
                       : code == 1 ? "the producer's wait for a free stage"
                                   : "the producer's wait for its copies in flight";
    return set_error(DIAQ_ERR_TIMEOUT, std::string("evolve: the bulk-copy term kernel gave up ") + what +
                                           " after its time bound; the states of that run are not valid");
}

// ---- autotuner ----------------------------------------------------------------------------------------
// Candidate launch shapes (states per launch, rows per thread) are timed on two steps of the
// caller's problem, run on scratch copies of the states (the caller's are not advanced), and the
// fastest is kept.  Choices are cached in a JSON file (DIAQ_AUTOTUNE_CACHE, else
// $HOME/.cache/diaq_gb300/autotune.json) keyed by GPU, mode, rows, diagonals, states and (s, m).

static std::string cache_path() {
    if (const char *p = std::getenv("DIAQ_AUTOTUNE_CACHE")) return p;
    const char *home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/diaq_gb300/autotune.json";
}

// The cache is a flat JSON object {"key": [states_per_block, rows_per_thread, pipelined], ...}.
static std::map<std::string, SpmvCfg> read_cache() {
    std::map<std::string, SpmvCfg> out;
    std::ifstream f(cache_path());
    if (!f) return out;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    size_t i = 0;
    while ((i = t.find('"', i)) != std::string::npos) {
        const size_t j = t.find('"', i + 1);
        if (j == std::string::npos) break;
        const std::string key = t.substr(i + 1, j - i - 1);
        int a = 0, b = 0, c = 0;
        const size_t br = t.find('[', j);
        if (br == std::string::npos || std::sscanf(t.c_str() + br, "[%d ,%d ,%d]", &a, &b, &c) < 2) break;
        out[key] = SpmvCfg{a, b, c};
        i = t.find(']', br);
        if (i == std::string::npos) break;
    }
    return out;
}

static void write_cache(const std::map<std::string, SpmvCfg> &c) {
    const std::string path = cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        // create the directory (one level below an existing parent is all we need)
        std::string dir = path.substr(0, slash);
        for (size_t k = 1; k <= dir.size(); ++k)
            if (k == dir.size() || dir[k] == '/') mkdir(dir.substr(0, k).c_str(), 0755);
    }
    // a temporary of this process's own, renamed into place: ranks sharing HOME never interleave
    const std::string tmp = path + "." + std::to_string((long)getpid()) + ".tmp";
    std::ofstream f(tmp);
    if (!f) return;
    f << "{\n";
    size_t n = 0;
    for (const auto &kv : c)
        f << "  \"" << kv.first << "\": [" << kv.second.kmax << ", " << kv.second.vr << ", " << kv.second.pipe << "]"
          << (++n < c.size() ? ",\n" : "\n");
    f << "}\n";
    f.close();
    std::rename(tmp.c_str(), path.c_str());
}

static std::string tune_key(const EvolvePlan &P, int sl, int m) {
    cudaDeviceProp prop{};
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    std::string name(prop.name);
    for (auto &ch : name)
        if (ch == '"' || ch == ' ') ch = '_';
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s|%s|n=%lld|nd=%d|k=%d|s=%d|m=%d", name.c_str(),
                  P.mode == DIAQ_EVOLVE_MIXED ? "mixed" : P.mode == DIAQ_EVOLVE_HORNER ? "horner" : "c128",
                  (long long)P.n, P.H->nd, P.nrhs, sl, m);
    return buf;
}

static int autotune(EvolvePlan &P, double dt, int sl, int m, double *pr, double *pi, int64_t ld, cudaStream_t user) {
    std::vector<SpmvCfg> cand;
    if (P.f32())
        cand = {{8, 1, 0}, {8, 2, 0}, {8, 4, 0}, {4, 2, 0}, {4, 4, 0}, {2, 4, 0}, {1, 4, 0},
                {8, 4, 1}, {4, 4, 1}, {2, 4, 1}, {1, 4, 1},
                {8, 4, 2}, {4, 4, 2}, {2, 4, 2}, {1, 4, 2}, {8, 4, 3}, {4, 4, 3}, {2, 4, 3},
                {8, 4, 4}, {4, 4, 4}, {2, 4, 4}, {4, 1, 6}, {4, 1, 7}, {4, 1, 8}, {4, 1, 9}, {4, 1, 12}};
    // (the bulk-copy variants 10 and 11 measured slower than 9 and 12 on every workload and stay
    // selectable through diaq_evolve_set_config only)
    else
        cand = {{8, 1, 0}, {8, 2, 0}, {4, 2, 0}, {2, 2, 0}, {1, 2, 0}};
    // drop shapes with more states per launch than the plan has (same launches as a smaller one)
    int kcap = 1;
    while (kcap < P.nrhs && kcap < 8) kcap *= 2;
    std::vector<SpmvCfg> c2;
    for (auto c : cand)
        if (c.kmax <= kcap && (c.pipe < 6 || P.nrhs <= 32)) c2.push_back(c);
    cand.swap(c2);
    const std::string key = tune_key(P, sl, m);
    auto cache = read_cache();
    auto hit = cache.find(key);
    // a cached shape is used only if it is still one of the library's candidates
    const bool known = hit != cache.end() && std::any_of(cand.begin(), cand.end(), [&](const SpmvCfg &c) {
                           return c.kmax == hit->second.kmax && c.vr == hit->second.vr && c.pipe == hit->second.pipe;
                       });
    if (known) {
        P.cfg = hit->second;
        P.tuned = true;
        return DIAQ_OK;
    }
    if (cand.size() == 1) {
        P.cfg = cand[0];
        P.tuned = true;
        return DIAQ_OK;
    }
    // scratch copies of the states
    const size_t cnt = (size_t)P.nrhs * (size_t)P.n;
    double *tmp = nullptr;
    DQ_CUDA(dev_malloc(&tmp, 2 * cnt * sizeof(double)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int st = DIAQ_OK;
    float best = -1.f;
    SpmvCfg best_cfg = cand[0];
    cudaError_t e = cudaStreamSynchronize(user);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp, pr, cnt * sizeof(double), cudaMemcpyDeviceToDevice, P.s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + cnt, pi, cnt * sizeof(double), cudaMemcpyDeviceToDevice, P.s);
    if (e != cudaSuccess) st = cuda_status(e, "autotune", __FILE__, __LINE__);
    for (size_t c = 0; c < cand.size() && st == DIAQ_OK; ++c) {
        P.cfg = cand[c];
        if (P.f32()) {
            st = fp32_state(P, tmp, tmp + cnt, P.s);
            if (st != DIAQ_OK) break;
        }
        st = enqueue_step(P, dt, sl, m, tmp, tmp + cnt, P.n);  // warm-up
        if (st != DIAQ_OK) break;
        cudaEventRecord(e0, P.s);
        st = enqueue_step(P, dt, sl, m, tmp, tmp + cnt, P.n);
        if (st != DIAQ_OK) break;
        cudaEventRecord(e1, P.s);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            st = cuda_status(e, "autotune", __FILE__, __LINE__);
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        // a candidate whose bounded waits gave up is not eligible (its time means nothing)
        int flag = 0;
        e = cudaMemcpy(&flag, P.err, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            st = cuda_status(e, "autotune", __FILE__, __LINE__);
            break;
        }
        if (flag != 0) {
            st = clear_wait_error(P);
            continue;
        }
        if (best < 0.f || ms < best) {
            best = ms;
            best_cfg = cand[c];
        }
    }
    cudaStreamSynchronize(P.s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(tmp);
    if (st != DIAQ_OK) return st;
    P.cfg = best_cfg;
    P.tuned = true;
    cache[key] = best_cfg;
    write_cache(cache);
    return DIAQ_OK;
}

static int plan_run(EvolvePlan &P, double *pr, double *pi, int64_t ld, double dt, int64_t steps, int sl, int m,
                    cudaStream_t user) {
    if (steps < 0 || m < 0 || sl < 0 || sl > 20) return set_error(DIAQ_ERR_INVALID, "evolve: bad steps / s / m");
    // dt keys the recorded steps: a NaN would compare equal to every key and replay another dt
    if (!std::isfinite(dt)) return set_error(DIAQ_ERR_INVALID, "evolve: dt must be finite");
    if (!pr || !pi) return set_error(DIAQ_ERR_INVALID, "evolve: psi pointer is NULL");
    if (steps == 0 || m == 0 || P.n == 0) return DIAQ_OK;
    // an earlier run's bulk-copy kernel gave up a wait (the copy of its flag has landed)
    DQ_TRY(take_wait_error(P, false));
    if (!P.Hc && P.tmask) DQ_TRY(build_tile_mask(*P.H, P.tmask, user));
    DQ_TRY(ensure_renorm_buffer(P));
    if (!P.tuned) DQ_TRY(autotune(P, dt, sl, m, pr, pi, ld, user));
    const EvolvePlan::Key key{dt, sl, m, pr, pi, ld};
    auto it = P.graphs.find(key);
    if (it == P.graphs.end()) {
        // a caller that passes ever new state pointers or time steps would otherwise grow the
        // cache without end: past kMaxGraphs the recorded steps are dropped (an executable graph
        // still in flight is released when it completes)
        if (P.graphs.size() >= kMaxGraphs) {
            for (auto &kv : P.graphs) cudaGraphExecDestroy(kv.second);
            P.graphs.clear();
        }
        // record one step on the plan's own stream (capture needs a stream other than the
        // legacy default); nothing runs during capture
        cudaGraph_t g = nullptr;
        DQ_CUDA(cudaStreamBeginCapture(P.s, cudaStreamCaptureModeThreadLocal));
        const int st = enqueue_step(P, dt, sl, m, pr, pi, ld);
        cudaError_t e = cudaStreamEndCapture(P.s, &g);
        if (st != DIAQ_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        cudaGraphExec_t ge = nullptr;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate", __FILE__, __LINE__);
        it = P.graphs.emplace(key, ge).first;
    }
    // everything below runs on the caller's stream
    if (P.f32()) DQ_TRY(fp32_state(P, pr, pi, user));  // fp32(psi) for the first sub-step
    for (int64_t i = 0; i < steps; ++i) DQ_CUDA(cudaGraphLaunch(it->second, user));
    DQ_CUDA(cudaMemcpyAsync(P.err_host, P.err, sizeof(int), cudaMemcpyDeviceToHost, user));
    DQ_CUDA(cudaEventRecord(P.err_ev, user));
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_evolve_create(diaq_matrix_t H, int nrhs, int mode, diaq_evolve_t *out) {
    if (!H || !out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    EvolvePlan *P = nullptr;
    DQ_TRY(plan_create(*H, nrhs, mode, &P));
    *out = static_cast<diaq_evolve_t>(P);
    return DIAQ_OK;
}

int diaq_evolve_destroy(diaq_evolve_t E) {
    delete E;
    return DIAQ_OK;
}

int diaq_evolve_run(diaq_evolve_t E, double *psi_re, double *psi_im, int64_t ld, double dt, int64_t steps,
                    int substeps_log2, int m, void *stream) {
    if (!E) return set_error(DIAQ_ERR_INVALID, "evolve plan is NULL");
    return plan_run(*E, psi_re, psi_im, ld, dt, steps, substeps_log2, m, (cudaStream_t)stream);
}

int diaq_evolve_launches_per_step(diaq_evolve_t E) { return E ? E->launches_per_step : 0; }

int diaq_evolve_set_config(diaq_evolve_t E, int states_per_block, int rows_per_thread, int pipelined) {
    if (!E) return set_error(DIAQ_ERR_INVALID, "evolve plan is NULL");
    if (states_per_block == 0) {  // back to automatic choice
        E->tuned = false;
        E->cfg = SpmvCfg{};
    } else {
        const bool f32 = E->f32();
        const bool vr_ok = rows_per_thread == 1 || rows_per_thread == 2 || (f32 && rows_per_thread == 4);
        if (states_per_block < 1 || states_per_block > 8 || !vr_ok)
            return set_error(DIAQ_ERR_INVALID, "evolve: states_per_block in 1..8, rows_per_thread 1, 2 (or 4 for mixed)");
        if (pipelined < 0 || pipelined > 12 || pipelined == 5)
            return set_error(DIAQ_ERR_INVALID, "evolve: pipelined is 0 (registers), 1 (cp.async), 2 or 3 (L2 prefetch), "
                                               "4 (shuffled windows), 6-12 (interleaved states)");
        if (pipelined >= 6) {
            if (!(f32 && states_per_block == 4 && rows_per_thread == 1))
                return set_error(DIAQ_ERR_INVALID, "evolve: the interleaved kernel is the mixed mode's, 4 states and "
                                                   "1 row per thread");
            if (E->nrhs > 32) return set_error(DIAQ_ERR_INVALID, "evolve: the interleaved kernels take at most 32 states");
        } else if (pipelined && !(f32 && rows_per_thread == 4)) {
            return set_error(DIAQ_ERR_INVALID, "evolve: the pipelined kernels are the mixed mode's, with 4 rows per thread");
        }
        E->cfg = SpmvCfg{states_per_block, rows_per_thread, pipelined};
        E->tuned = true;
    }
    for (auto &kv : E->graphs) cudaGraphExecDestroy(kv.second);
    E->graphs.clear();
    // an error of the previous kernel is not carried over to the new one
    DQ_CUDA(cudaEventSynchronize(E->err_ev));
    return clear_wait_error(*E);
}

int diaq_evolve_set_wait_limit(diaq_evolve_t E, int64_t wait_ns) {
    if (!E) return set_error(DIAQ_ERR_INVALID, "evolve plan is NULL");
    if (wait_ns < 0) return set_error(DIAQ_ERR_INVALID, "evolve: the wait limit must be >= 0 nanoseconds");
    const uint64_t w = wait_ns == 0 ? kWaitNs : (uint64_t)wait_ns;
    if (w != E->wait_ns) {  // the bound is a kernel argument of the recorded steps
        E->wait_ns = w;
        for (auto &kv : E->graphs) cudaGraphExecDestroy(kv.second);
        E->graphs.clear();
    }
    return DIAQ_OK;
}

int diaq_evolve_check(diaq_evolve_t E) {
    if (!E) return set_error(DIAQ_ERR_INVALID, "evolve plan is NULL");
    return take_wait_error(*E, true);
}

int diaq_evolve_set_renormalize(diaq_evolve_t E, int on) {
    if (!E) return set_error(DIAQ_ERR_INVALID, "evolve plan is NULL");
    if (E->renorm != (on != 0)) {
        E->renorm = on != 0;
        for (auto &kv : E->graphs) cudaGraphExecDestroy(kv.second);
        E->graphs.clear();
    }
    return DIAQ_OK;
}

int diaq_evolve_config(diaq_evolve_t E, int *states_per_block, int *rows_per_thread, int *pipelined) {
    if (!E || !states_per_block || !rows_per_thread) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    *states_per_block = E->cfg.kmax;
    *rows_per_thread = E->cfg.vr > 0 ? E->cfg.vr : (E->f32() ? 4 : 2);
    if (pipelined) *pipelined = E->cfg.pipe;
    return DIAQ_OK;
}

}  // extern "C"

namespace diaq_gb300 {

// One step of the states in host memory as two half plans, so that the link and the GPU work at
// once: half 0 up; half 0 runs while half 1 goes up; half 1 runs while half 0 comes down; half 1
// down.  The states of a half are contiguous in each plane (state q at psi[q n + r]).  Each half
// plan runs the launch shape of the whole plan (the same sums per state, so the same bits as
// an unsplit run) with the whole plan's settings.
static int run_host_split(EvolvePlan &E, double *psi_re, double *psi_im, double dt, int sl, int m) {
    const int h = E.nrhs / 2;
    const size_t cnt = (size_t)E.nrhs * (size_t)E.n, hc = (size_t)h * (size_t)E.n;
    for (int j = 0; j < 2; ++j) {
        if (!E.half[j]) {
            DQ_TRY(plan_create(*E.H, h, E.mode, &E.half[j], &E));
            E.half[j]->cfg = E.cfg;
            E.half[j]->tuned = true;
        }
        EvolvePlan &Hp = *E.half[j];
        if (Hp.wait_ns != E.wait_ns || Hp.renorm != E.renorm || Hp.cfg.kmax != E.cfg.kmax || Hp.cfg.vr != E.cfg.vr ||
            Hp.cfg.pipe != E.cfg.pipe) {
            Hp.wait_ns = E.wait_ns;
            Hp.renorm = E.renorm;
            Hp.cfg = E.cfg;
            for (auto &kv : Hp.graphs) cudaGraphExecDestroy(kv.second);
            Hp.graphs.clear();
        }
    }
    if (!E.hcomp) DQ_CUDA(cudaStreamCreateWithFlags(&E.hcomp, cudaStreamNonBlocking));
    for (auto &ev : E.hsev)
        if (!ev) DQ_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    double *d = E.stage;
    cudaStream_t up = E.hs[0], down = E.hs[1], comp = E.hcomp;
    const size_t hb = hc * sizeof(double);
    cudaError_t e = cudaSuccess;
    int st = DIAQ_OK;
    // up: both halves on one stream, an event after each
    for (int j = 0; j < 2 && e == cudaSuccess; ++j) {
        e = cudaMemcpyAsync(d + j * hc, psi_re + j * hc, hb, cudaMemcpyHostToDevice, up);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + cnt + j * hc, psi_im + j * hc, hb, cudaMemcpyHostToDevice, up);
        if (e == cudaSuccess) e = cudaEventRecord(E.hsev[j], up);
    }
    if (e != cudaSuccess) st = cuda_status(e, "evolve upload", __FILE__, __LINE__);
    // run: each half once its states have landed, one after the other on comp
    for (int j = 0; j < 2 && st == DIAQ_OK; ++j) {
        e = cudaStreamWaitEvent(comp, E.hsev[j], 0);
        if (e != cudaSuccess) {
            st = cuda_status(e, "evolve run_host", __FILE__, __LINE__);
            break;
        }
        st = plan_run(*E.half[j], d + j * hc, d + cnt + j * hc, E.n, dt, 1, sl, m, comp);
        if (st == DIAQ_OK) {
            e = cudaEventRecord(E.hsev[2 + j], comp);
            if (e != cudaSuccess) st = cuda_status(e, "evolve run_host", __FILE__, __LINE__);
        }
    }
    // down: each half once it has run
    for (int j = 0; j < 2 && st == DIAQ_OK; ++j) {
        e = cudaStreamWaitEvent(down, E.hsev[2 + j], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(psi_re + j * hc, d + j * hc, hb, cudaMemcpyDeviceToHost, down);
        if (e == cudaSuccess) e = cudaMemcpyAsync(psi_im + j * hc, d + cnt + j * hc, hb, cudaMemcpyDeviceToHost, down);
        if (e != cudaSuccess) st = cuda_status(e, "evolve download", __FILE__, __LINE__);
    }
    const cudaError_t eu = cudaStreamSynchronize(up), ec = cudaStreamSynchronize(comp),
                      ed = cudaStreamSynchronize(down);
    if (st == DIAQ_OK && eu != cudaSuccess) st = cuda_status(eu, "evolve run_host", __FILE__, __LINE__);
    if (st == DIAQ_OK && ec != cudaSuccess) st = cuda_status(ec, "evolve run_host", __FILE__, __LINE__);
    if (st == DIAQ_OK && ed != cudaSuccess) st = cuda_status(ed, "evolve run_host", __FILE__, __LINE__);
    for (int j = 0; j < 2 && st == DIAQ_OK; ++j) st = take_wait_error(*E.half[j], true);
    return st;
}

}  // namespace diaq_gb300

extern "C" {

int diaq_evolve_run_host(diaq_evolve_t E, double *psi_re, double *psi_im, double dt, int64_t steps,
                         int substeps_log2, int m) {
    if (!E) return set_error(DIAQ_ERR_INVALID, "evolve plan is NULL");
    if (!psi_re || !psi_im) return set_error(DIAQ_ERR_INVALID, "evolve: psi pointer is NULL");
    const size_t cnt = (size_t)E->nrhs * (size_t)E->n;
    if (cnt == 0) return DIAQ_OK;
    // the device copy of the states is the plan's own, allocated on the first call and kept, so
    // that later calls allocate nothing and find the step recorded for it
    if (!E->stage) DQ_CUDA(dev_malloc(&E->stage, 2 * cnt * sizeof(double)));
    for (int j = 0; j < 2; ++j) {
        if (!E->hs[j]) DQ_CUDA(cudaStreamCreateWithFlags(&E->hs[j], cudaStreamNonBlocking));
        if (!E->hev[j]) DQ_CUDA(cudaEventCreateWithFlags(&E->hev[j], cudaEventDisableTiming));
    }
    // a single step of 8 or more float32-term states, once the plan has its launch shape: the
    // halves overlap the copies with the run (on the 20-qubit chain, 8 states: the copies take
    // ~1.4 ms per step against 1.1 ms of run)
    if (steps == 1 && m > 0 && E->f32() && E->tuned && E->nrhs >= 8 && E->nrhs % 2 == 0 && std::isfinite(dt) &&
        substeps_log2 >= 0 && substeps_log2 <= 20)
        return run_host_split(*E, psi_re, psi_im, dt, substeps_log2, m);
    double *d = E->stage;
    cudaStream_t a = E->hs[0], b = E->hs[1];
    const size_t bytes = cnt * sizeof(double);
    // up: re on a, im on b at the same time; the run on a once both have landed
    cudaError_t e = cudaMemcpyAsync(d, psi_re, bytes, cudaMemcpyHostToDevice, a);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + cnt, psi_im, bytes, cudaMemcpyHostToDevice, b);
    if (e == cudaSuccess) e = cudaEventRecord(E->hev[1], b);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(a, E->hev[1], 0);
    int st = e == cudaSuccess ? DIAQ_OK : cuda_status(e, "evolve upload", __FILE__, __LINE__);
    if (st == DIAQ_OK) st = plan_run(*E, d, d + cnt, E->n, dt, steps, substeps_log2, m, a);
    if (st == DIAQ_OK) {
        // down: both planes once the run has finished, again on the two streams
        e = cudaEventRecord(E->hev[0], a);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b, E->hev[0], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(psi_re, d, bytes, cudaMemcpyDeviceToHost, a);
        if (e == cudaSuccess) e = cudaMemcpyAsync(psi_im, d + cnt, bytes, cudaMemcpyDeviceToHost, b);
        if (e != cudaSuccess) st = cuda_status(e, "evolve download", __FILE__, __LINE__);
    }
    // synchronous: both streams drained whatever happened above
    const cudaError_t ea = cudaStreamSynchronize(a), eb = cudaStreamSynchronize(b);
    if (st == DIAQ_OK && ea != cudaSuccess) st = cuda_status(ea, "evolve run_host", __FILE__, __LINE__);
    if (st == DIAQ_OK && eb != cudaSuccess) st = cuda_status(eb, "evolve run_host", __FILE__, __LINE__);
    // the run has finished: a wait that gave up in it is reported now, not at the next call
    if (st == DIAQ_OK) st = take_wait_error(*E, true);
    return st;
}

}  // extern "C"
