// Tiled interleaved float32 states and the epilogues that work on them, shared by the evolution
// plans and the batched form.
//
// Layout: rows in blocks of 32, and within a block each quad of 4 states stored as 32 rows x 4
// floats (512 bytes).  Element (r, q) sits at ((r / 32) * (sp / 4) + q / 4) * 128 + (r mod 32) * 4
// + q mod 4, sp = the state count rounded up to a power of two >= 4 (padding states zero), rows
// padded to a multiple of 32.  A warp over 32 consecutive rows and one quad reads its state
// window at any diagonal offset as one contiguous 512-byte run (one 16-byte load per lane).
#pragma once

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

// TwoSum (Knuth): s + e = a + b exactly, s = fl(a + b).  The _rn intrinsics keep the compiler
// from fusing an add with the multiply that produced b, which would break the identity.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Float index of state 4 quad of row r in the tiled interleaved layout (quads = sp / 4); states
// 4 quad .. 4 quad + 3 of the row follow it as one 16-byte-aligned float4.
__device__ __forceinline__ int64_t il_at(int64_t r, int quad, int quads) {
    return ((r >> 5) * quads + quad) * 128 + ((r & 31) << 2);
}

// One Taylor term's epilogue for four interleaved states of one row: the compensated forward sum
// (the arithmetic of the planar EpiMixed of the evolution plans).
struct EpiMixedIL {
    static constexpr bool kPsiTile = false;
    float *vr, *vi;                 // term out (interleaved)
    float *hr, *hi_, *lr, *li;      // compensated sum (interleaved)
    double *pr, *pi;                // state, q at p[q * ld + r]
    int64_t ld;
    int sp, nrhs;
    float scale;
    int first, last;
    __device__ __forceinline__ void apply(int64_t r, int g, const float (&sr)[4], const float (&si)[4]) const {
        const int64_t i = il_at(r, g, sp >> 2);
        float tr[4], ti[4], h_r[4], h_i[4], l_r[4], l_i[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tr[c] = si[c] * scale;
            ti[c] = -sr[c] * scale;
        }
        if (first) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                h_r[c] = tr[c];
                h_i[c] = ti[c];
                l_r[c] = l_i[c] = 0.f;
            }
        } else {
            const float4 a = *reinterpret_cast<const float4 *>(hr + i), b = *reinterpret_cast<const float4 *>(hi_ + i);
            const float4 c4 = *reinterpret_cast<const float4 *>(lr + i), d = *reinterpret_cast<const float4 *>(li + i);
            const float ha[4] = {a.x, a.y, a.z, a.w}, hb[4] = {b.x, b.y, b.z, b.w};
            const float la[4] = {c4.x, c4.y, c4.z, c4.w}, lb[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float e_r, e_i;
                two_sum(ha[c], tr[c], h_r[c], e_r);
                two_sum(hb[c], ti[c], h_i[c], e_i);
                l_r[c] = la[c] + e_r;
                l_i[c] = lb[c] + e_i;
            }
        }
        if (!last) {
            *reinterpret_cast<float4 *>(hr + i) = make_float4(h_r[0], h_r[1], h_r[2], h_r[3]);
            *reinterpret_cast<float4 *>(hi_ + i) = make_float4(h_i[0], h_i[1], h_i[2], h_i[3]);
            *reinterpret_cast<float4 *>(lr + i) = make_float4(l_r[0], l_r[1], l_r[2], l_r[3]);
            *reinterpret_cast<float4 *>(li + i) = make_float4(l_i[0], l_i[1], l_i[2], l_i[3]);
            *reinterpret_cast<float4 *>(vr + i) = make_float4(tr[0], tr[1], tr[2], tr[3]);
            *reinterpret_cast<float4 *>(vi + i) = make_float4(ti[0], ti[1], ti[2], ti[3]);
        } else {
            float nr_[4], ni_[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int q = 4 * g + c;
                nr_[c] = ni_[c] = 0.f;
                if (q < nrhs) {
                    const double nr = pr[q * ld + r] + ((double)h_r[c] + (double)l_r[c]);
                    const double ni = pi[q * ld + r] + ((double)h_i[c] + (double)l_i[c]);
                    pr[q * ld + r] = nr;
                    pi[q * ld + r] = ni;
                    nr_[c] = (float)nr;
                    ni_[c] = (float)ni;
                }
            }
            *reinterpret_cast<float4 *>(vr + i) = make_float4(nr_[0], nr_[1], nr_[2], nr_[3]);
            *reinterpret_cast<float4 *>(vi + i) = make_float4(ni_[0], ni_[1], ni_[2], ni_[3]);
        }
    }
};

// The Horner step (EpiHorner) for four interleaved states of one row.  LAST = 0 / 1 fixes at compile
// time whether this is a middle or the last step (-1: the runtime field `last` says), so that a
// middle step's kernel carries none of the last step's float64 code.
template <int LAST = -1>
struct EpiHornerT {
    float *wr, *wi;                 // interleaved: w out
    const float *fr, *fi;           // fp32(psi)
    float *gr, *gi;                 // fp32(psi) written on the last step
    double *pr, *pi;                // psi, q at p[q * ld + r]
    int64_t ld;
    int sp, nrhs;
    float scale;
    int last;
    // A middle step reads one fp32(psi) quad per plane and row: kernels may fetch it ahead into
    // shared memory and hand it to apply_psi.
    static constexpr bool kPsiTile = true;
    __host__ __device__ __forceinline__ bool is_last() const { return LAST < 0 ? last != 0 : LAST == 1; }
    __device__ __forceinline__ bool reads_psi() const { return !is_last(); }
    __device__ __forceinline__ void apply_psi(int64_t r, int g, const float (&sr)[4], const float (&si)[4],
                                              const float4 &a, const float4 &b) const {
        const int64_t i = il_at(r, g, sp >> 2);
        float tr[4], ti[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tr[c] = si[c] * scale;
            ti[c] = -sr[c] * scale;
        }
        // unfused (rounded product, then rounded sum): the planar kernels give the same bits
        *reinterpret_cast<float4 *>(wr + i) = make_float4(__fadd_rn(a.x, tr[0]), __fadd_rn(a.y, tr[1]),
                                                          __fadd_rn(a.z, tr[2]), __fadd_rn(a.w, tr[3]));
        *reinterpret_cast<float4 *>(wi + i) = make_float4(__fadd_rn(b.x, ti[0]), __fadd_rn(b.y, ti[1]),
                                                          __fadd_rn(b.z, ti[2]), __fadd_rn(b.w, ti[3]));
    }
    __device__ __forceinline__ void apply(int64_t r, int g, const float (&sr)[4], const float (&si)[4]) const {
        const int64_t i = il_at(r, g, sp >> 2);
        float tr[4], ti[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tr[c] = si[c] * scale;
            ti[c] = -sr[c] * scale;
        }
        if (!is_last()) {
            const float4 a = *reinterpret_cast<const float4 *>(fr + i), b = *reinterpret_cast<const float4 *>(fi + i);
            apply_psi(r, g, sr, si, a, b);
        } else {
            float nr_[4], ni_[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int q = 4 * g + c;
                nr_[c] = ni_[c] = 0.f;
                if (q < nrhs) {
                    const double nr = pr[q * ld + r] + (double)tr[c], ni = pi[q * ld + r] + (double)ti[c];
                    pr[q * ld + r] = nr;
                    pi[q * ld + r] = ni;
                    nr_[c] = (float)nr;
                    ni_[c] = (float)ni;
                }
            }
            *reinterpret_cast<float4 *>(gr + i) = make_float4(nr_[0], nr_[1], nr_[2], nr_[3]);
            *reinterpret_cast<float4 *>(gi + i) = make_float4(ni_[0], ni_[1], ni_[2], ni_[3]);
        }
    }
};
using EpiHornerIL = EpiHornerT<-1>;

// The state window of G states (G / 4 quads from quad g0) at column c: two 16-byte loads per quad.
template <int G>
struct IlWindow {
    float4 x[G / 4], y[G / 4];
};
template <int G>
__device__ __forceinline__ void il_load(int64_t c, int g0, int quads, const float *__restrict__ xr,
                                        const float *__restrict__ xi, IlWindow<G> &w) {
#pragma unroll
    for (int h = 0; h < G / 4; ++h) {
        const int64_t at = il_at(c, g0 + h, quads);
        w.x[h] = __ldg(reinterpret_cast<const float4 *>(xr + at));
        w.y[h] = __ldg(reinterpret_cast<const float4 *>(xi + at));
    }
}
// acc += (a + i b) * window, per state.  PACKED: two states per instruction (__ffma2_rn: each
// lane one fmaf, the same rounding, so the same bits) -- 93.1 -> 91.1 us per 8-state Horner term
// of the evolution plans; in the register-bounded batched kernels (six blocks per SM) it cost
// 10 % (7,955 -> 7,122 states x steps/s), so they keep one FMA per state.
template <int G, bool PACKED = false>
__device__ __forceinline__ void il_fma(float a, float b, const IlWindow<G> &w, float (&accr)[G], float (&acci)[G]) {
    if constexpr (PACKED) {
        const float2 aa = make_float2(a, a), bb = make_float2(b, b), nb = make_float2(-b, -b);
#pragma unroll
        for (int h = 0; h < G / 4; ++h) {
            const float2 x01 = make_float2(w.x[h].x, w.x[h].y), x23 = make_float2(w.x[h].z, w.x[h].w);
            const float2 y01 = make_float2(w.y[h].x, w.y[h].y), y23 = make_float2(w.y[h].z, w.y[h].w);
            float2 r01 = make_float2(accr[4 * h], accr[4 * h + 1]), r23 = make_float2(accr[4 * h + 2], accr[4 * h + 3]);
            float2 i01 = make_float2(acci[4 * h], acci[4 * h + 1]), i23 = make_float2(acci[4 * h + 2], acci[4 * h + 3]);
            r01 = __ffma2_rn(aa, x01, r01);
            r23 = __ffma2_rn(aa, x23, r23);
            r01 = __ffma2_rn(nb, y01, r01);
            r23 = __ffma2_rn(nb, y23, r23);
            i01 = __ffma2_rn(aa, y01, i01);
            i23 = __ffma2_rn(aa, y23, i23);
            i01 = __ffma2_rn(bb, x01, i01);
            i23 = __ffma2_rn(bb, x23, i23);
            accr[4 * h] = r01.x;
            accr[4 * h + 1] = r01.y;
            accr[4 * h + 2] = r23.x;
            accr[4 * h + 3] = r23.y;
            acci[4 * h] = i01.x;
            acci[4 * h + 1] = i01.y;
            acci[4 * h + 2] = i23.x;
            acci[4 * h + 3] = i23.y;
        }
    } else {
#pragma unroll
        for (int h = 0; h < G / 4; ++h) {
            const float xv[4] = {w.x[h].x, w.x[h].y, w.x[h].z, w.x[h].w};
            const float yv[4] = {w.y[h].x, w.y[h].y, w.y[h].z, w.y[h].w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                accr[4 * h + q] = fmaf(a, xv[q], accr[4 * h + q]);
                accr[4 * h + q] = fmaf(-b, yv[q], accr[4 * h + q]);
                acci[4 * h + q] = fmaf(a, yv[q], acci[4 * h + q]);
                acci[4 * h + q] = fmaf(b, xv[q], acci[4 * h + q]);
            }
        }
    }
}

// One diagonal's contribution to G states of row r, window at column c = r + off.
template <int G>
__device__ __forceinline__ void il_term(int64_t c, int g0, int quads, float a, float b, const float *__restrict__ xr,
                                        const float *__restrict__ xi, float (&accr)[G], float (&acci)[G]) {
    IlWindow<G> w;
    il_load<G>(c, g0, quads, xr, xi, w);
    il_fma<G>(a, b, w, accr, acci);
}

// The diagonals k < cn of one metadata chunk for row r (32-bit row and window arithmetic: rows
// and n_pad * sp below 2^31).  sq[k] = (offset, lo, hi, mask word of the block's rows), sb[k] =
// value base: one 16-byte and one 8-byte shared-memory load per diagonal; a warp skips a dead
// tile or a diagonal outside its rows together.
template <int G, bool PACKED = false>
__device__ __forceinline__ void il_accumulate32(const int4 *sq, const int64_t *sb, int cn, int r, int g0, int quads,
                                                const float *__restrict__ are, const float *__restrict__ aim,
                                                const float *__restrict__ xr, const float *__restrict__ xi,
                                                float (&accr)[G], float (&acci)[G]) {
    const int tbit = (r >> 5) & 31;
    // unrolled by 2: 93.1 us per 8-state Horner term on the 20-qubit chain (1 and 4: 95.0 and 93.9)
#pragma unroll 2
    for (int k = 0; k < cn; ++k) {
        const int4 q = sq[k];
        if (r < q.y || r >= q.z || !(((uint32_t)q.w >> tbit) & 1u)) continue;
        const int64_t vb = sb[k] + r;
        const float a = __ldcs(are + vb), b = __ldcs(aim + vb);
        const int c = r + q.x;
        IlWindow<G> w;
#pragma unroll
        for (int h = 0; h < G / 4; ++h) {
            const int at = ((((c >> 5) * quads) + g0 + h) << 7) + ((c & 31) << 2);
            w.x[h] = __ldg(reinterpret_cast<const float4 *>(xr + at));
            w.y[h] = __ldg(reinterpret_cast<const float4 *>(xi + at));
        }
        il_fma<G, PACKED>(a, b, w, accr, acci);
    }
}

}  // namespace diaq_gb300
