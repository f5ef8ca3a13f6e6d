// The learned (s, m) proposer: a small FP32 MLP, 16 features -> 64 -> 64 -> 21 + 30 logits
// (s in 0..20, m in 1..30), with hand-written forward, softmax cross-entropy, backward and Adam
// kernels.  No counterpart in the reference, whose expm picks s by the norm bound alone
// (src/spME.cpp:256-262) and m by a Frobenius stop test.
//
// Parameters live in one flat float buffer: W1[16][64] b1[64] W2[64][64] b2[64] W3[64][51] b3[51]
// (W[i][j] maps input i to output j).  Every reduction over the batch runs in a fixed order in one
// thread, so gradients are deterministic.
#include <cmath>
#include <random>
#include <vector>

#include "diaq_internal.cuh"

namespace diaq_gb300 {

constexpr int kIn = 16, kH1 = 64, kH2 = 64, kOutS = 21, kOutM = 30, kOut = kOutS + kOutM;
constexpr int oW1 = 0, oB1 = oW1 + kIn * kH1, oW2 = oB1 + kH1, oB2 = oW2 + kH1 * kH2, oW3 = oB2 + kH2,
              oB3 = oW3 + kH2 * kOut, kParams = oB3 + kOut;

struct Mlp {
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // params, grads, Adam moments
    float *work = nullptr;                                          // activations for `cap` rows
    int cap = 0;
    int64_t t = 0;  // Adam step
    ~Mlp() {
        cudaFree(p);
        cudaFree(work);
    }
};

// out[b][j] = act(sum_i in[b][i] W[i][j] + bias[j]); also keeps the pre-activation z.
__global__ void dense_fwd(const float *__restrict__ in, int B, int din, const float *__restrict__ W,
                          const float *__restrict__ bias, int dout, int relu, float *__restrict__ z,
                          float *__restrict__ out) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * dout) return;
    const int b = (int)(idx / dout), j = (int)(idx % dout);
    float s = bias[j];
    for (int i = 0; i < din; ++i) s = fmaf(in[(int64_t)b * din + i], W[i * dout + j], s);
    if (z) z[idx] = s;
    out[idx] = relu ? fmaxf(s, 0.f) : s;
}

// Per row: loss = CE(softmax(logits[0:21]), s) + CE(softmax(logits[21:51]), m-1); dlogits =
// (softmax - onehot) / B.  Labels outside range give loss 0 and no gradient for that head.
__global__ void softmax_ce(const float *__restrict__ logits, const int32_t *__restrict__ ys,
                           const int32_t *__restrict__ ym, int B, float *__restrict__ dlog,
                           float *__restrict__ loss) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *l = logits + (int64_t)b * kOut;
    float *d = dlog + (int64_t)b * kOut;
    float total = 0.f;
    for (int head = 0; head < 2; ++head) {
        const int o0 = head == 0 ? 0 : kOutS, n = head == 0 ? kOutS : kOutM;
        const int lab = head == 0 ? ys[b] : ym[b] - 1;
        float mx = l[o0];
        for (int j = 1; j < n; ++j) mx = fmaxf(mx, l[o0 + j]);
        float se = 0.f;
        for (int j = 0; j < n; ++j) se += expf(l[o0 + j] - mx);
        const bool ok = lab >= 0 && lab < n;
        for (int j = 0; j < n; ++j) {
            const float pj = expf(l[o0 + j] - mx) / se;
            d[o0 + j] = ok ? (pj - (j == lab ? 1.f : 0.f)) / (float)B : 0.f;
        }
        if (ok) total += -(l[o0 + lab] - mx - logf(se));
    }
    loss[b] = total;
}

// dW[i][j] = sum_b in[b][i] dout[b][j]; db[j] = sum_b dout[b][j] (thread per weight, batch in order).
__global__ void dense_bwd_w(const float *__restrict__ in, const float *__restrict__ dout, int B, int din, int dn,
                            float *__restrict__ dW, float *__restrict__ db) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < din * dn) {
        const int i = idx / dn, j = idx % dn;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s = fmaf(in[(int64_t)b * din + i], dout[(int64_t)b * dn + j], s);
        dW[idx] = s;
    } else if (idx < din * dn + dn) {
        const int j = idx - din * dn;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += dout[(int64_t)b * dn + j];
        db[j] = s;
    }
}

// dIn[b][i] = (sum_j dout[b][j] W[i][j]) * (z[b][i] > 0)
__global__ void dense_bwd_x(const float *__restrict__ dout, const float *__restrict__ W, const float *__restrict__ z,
                            int B, int din, int dn, float *__restrict__ dIn) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * din) return;
    const int b = (int)(idx / din), i = (int)(idx % din);
    float s = 0.f;
    for (int j = 0; j < dn; ++j) s = fmaf(dout[(int64_t)b * dn + j], W[i * dn + j], s);
    dIn[idx] = z[idx] > 0.f ? s : 0.f;
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float bc1,
                            float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void argmax_heads(const float *__restrict__ logits, int B, int32_t *__restrict__ s_out,
                             int32_t *__restrict__ m_out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *l = logits + (int64_t)b * kOut;
    int bs = 0, bm = 0;
    for (int j = 1; j < kOutS; ++j)
        if (l[j] > l[bs]) bs = j;
    for (int j = 1; j < kOutM; ++j)
        if (l[kOutS + j] > l[kOutS + bm]) bm = j;
    s_out[b] = bs;
    m_out[b] = bm + 1;
}

// Activations for B rows: z1 a1 (B x 64) z2 a2 (B x 64) logits dlog (B x 51) d2 d1 (B x 64) loss (B)
static int ensure_work(Mlp &M, int B) {
    if (B <= M.cap) return DIAQ_OK;
    if (M.work) cudaFree(M.work);
    M.work = nullptr;
    M.cap = 0;
    const size_t per = 6 * kH1 + 2 * kOut + 1;
    DQ_CUDA(dev_malloc(&M.work, sizeof(float) * per * (size_t)B));
    M.cap = B;
    return DIAQ_OK;
}

struct Acts {
    float *z1, *a1, *z2, *a2, *lg, *dl, *d2, *d1, *loss;
};
static Acts acts(const Mlp &M) {
    const int64_t B = M.cap;
    float *w = M.work;
    Acts a;
    a.z1 = w;
    a.a1 = w + B * kH1;
    a.z2 = w + 2 * B * kH1;
    a.a2 = w + 3 * B * kH1;
    a.lg = w + 4 * B * kH1;
    a.dl = a.lg + B * kOut;
    a.d2 = a.dl + B * kOut;
    a.d1 = a.d2 + B * kH2;
    a.loss = a.d1 + B * kH1;
    return a;
}

static inline unsigned nb(int64_t n) { return (unsigned)((n + 255) / 256); }

static int forward(Mlp &M, const float *X, int B, cudaStream_t s) {
    const Acts a = acts(M);
    dense_fwd<<<nb((int64_t)B * kH1), 256, 0, s>>>(X, B, kIn, M.p + oW1, M.p + oB1, kH1, 1, a.z1, a.a1);
    dense_fwd<<<nb((int64_t)B * kH2), 256, 0, s>>>(a.a1, B, kH1, M.p + oW2, M.p + oB2, kH2, 1, a.z2, a.a2);
    dense_fwd<<<nb((int64_t)B * kOut), 256, 0, s>>>(a.a2, B, kH2, M.p + oW3, M.p + oB3, kOut, 0, nullptr, a.lg);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

static int gradient(Mlp &M, const float *X, const int32_t *ys, const int32_t *ym, int B, cudaStream_t s) {
    DQ_TRY(forward(M, X, B, s));
    const Acts a = acts(M);
    softmax_ce<<<nb(B), 256, 0, s>>>(a.lg, ys, ym, B, a.dl, a.loss);
    dense_bwd_w<<<nb(kH2 * kOut + kOut), 256, 0, s>>>(a.a2, a.dl, B, kH2, kOut, M.g + oW3, M.g + oB3);
    dense_bwd_x<<<nb((int64_t)B * kH2), 256, 0, s>>>(a.dl, M.p + oW3, a.z2, B, kH2, kOut, a.d2);
    dense_bwd_w<<<nb(kH1 * kH2 + kH2), 256, 0, s>>>(a.a1, a.d2, B, kH1, kH2, M.g + oW2, M.g + oB2);
    dense_bwd_x<<<nb((int64_t)B * kH1), 256, 0, s>>>(a.d2, M.p + oW2, a.z1, B, kH1, kH2, a.d1);
    dense_bwd_w<<<nb(kIn * kH1 + kH1), 256, 0, s>>>(X, a.d1, B, kIn, kH1, M.g + oW1, M.g + oB1);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

struct diaq_mlp_s : public Mlp {};

extern "C" {

int diaq_mlp_num_params(void) { return kParams; }

int diaq_mlp_create(uint64_t seed, diaq_mlp_t *out) {
    if (!out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    std::vector<float> h(kParams, 0.f);
    std::mt19937_64 rng(seed);
    auto init = [&](int off, int fan_in, int n) {  // He initialisation, biases stay 0
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / fan_in));
        for (int i = 0; i < n; ++i) h[off + i] = (float)nd(rng);
    };
    init(oW1, kIn, kIn * kH1);
    init(oW2, kH1, kH1 * kH2);
    init(oW3, kH2, kH2 * kOut);
    diaq_mlp_s *M = new diaq_mlp_s();
    cudaError_t e = dev_malloc(&M->p, sizeof(float) * 4 * kParams);
    if (e == cudaSuccess) {
        M->g = M->p + kParams;
        M->m = M->p + 2 * kParams;
        M->v = M->p + 3 * kParams;
        e = cudaMemset(M->p, 0, sizeof(float) * 4 * kParams);
    }
    if (e == cudaSuccess) e = cudaMemcpy(M->p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete M;
        return cuda_status(e, "mlp create", __FILE__, __LINE__);
    }
    *out = M;
    return DIAQ_OK;
}

int diaq_mlp_destroy(diaq_mlp_t M) {
    delete M;
    return DIAQ_OK;
}

int diaq_mlp_get_params(diaq_mlp_t M, float *host_out) {
    if (!M || !host_out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    DQ_CUDA(cudaMemcpy(host_out, M->p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    return DIAQ_OK;
}

int diaq_mlp_set_params(diaq_mlp_t M, const float *host_in) {
    if (!M || !host_in) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    DQ_CUDA(cudaMemcpy(M->p, host_in, sizeof(float) * kParams, cudaMemcpyHostToDevice));
    DQ_CUDA(cudaMemset(M->m, 0, sizeof(float) * 2 * kParams));
    M->t = 0;
    return DIAQ_OK;
}

int diaq_mlp_forward(diaq_mlp_t M, const float *X, int B, float *logits, void *stream) {
    if (!M || !X || !logits || B < 0) return set_error(DIAQ_ERR_INVALID, "mlp forward: bad argument");
    if (B == 0) return DIAQ_OK;
    cudaStream_t s = (cudaStream_t)stream;
    DQ_TRY(ensure_work(*M, B));
    DQ_TRY(forward(*M, X, B, s));
    DQ_CUDA(cudaMemcpyAsync(logits, acts(*M).lg, sizeof(float) * kOut * (size_t)B, cudaMemcpyDeviceToDevice, s));
    return DIAQ_OK;
}

int diaq_mlp_gradient(diaq_mlp_t M, const float *X, const int32_t *s_label, const int32_t *m_label, int B,
                      float *grad_out, float *loss_out, void *stream) {
    if (!M || !X || !s_label || !m_label || B <= 0) return set_error(DIAQ_ERR_INVALID, "mlp gradient: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    DQ_TRY(ensure_work(*M, B));
    DQ_TRY(gradient(*M, X, s_label, m_label, B, s));
    if (grad_out) DQ_CUDA(cudaMemcpyAsync(grad_out, M->g, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, s));
    if (loss_out) DQ_CUDA(cudaMemcpyAsync(loss_out, acts(*M).loss, sizeof(float) * B, cudaMemcpyDeviceToDevice, s));
    return DIAQ_OK;
}

int diaq_mlp_train_step(diaq_mlp_t M, const float *X, const int32_t *s_label, const int32_t *m_label, int B,
                        float lr, float *loss_out, void *stream) {
    DQ_TRY(diaq_mlp_gradient(M, X, s_label, m_label, B, nullptr, loss_out, stream));
    cudaStream_t s = (cudaStream_t)stream;
    M->t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - (float)std::pow((double)b1, (double)M->t);
    const float bc2 = 1.f - (float)std::pow((double)b2, (double)M->t);
    adam_kernel<<<nb(kParams), 256, 0, s>>>(M->p, M->g, M->m, M->v, kParams, lr, b1, b2, 1e-8f, bc1, bc2);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

int diaq_mlp_propose(diaq_mlp_t M, const float *X, int B, int32_t *s_out, int32_t *m_out, void *stream) {
    if (!M || !X || !s_out || !m_out || B < 0) return set_error(DIAQ_ERR_INVALID, "mlp propose: bad argument");
    if (B == 0) return DIAQ_OK;
    cudaStream_t s = (cudaStream_t)stream;
    DQ_TRY(ensure_work(*M, B));
    DQ_TRY(forward(*M, X, B, s));
    argmax_heads<<<nb(B), 256, 0, s>>>(acts(*M).lg, B, s_out, m_out);
    DQ_CUDA(cudaGetLastError());
    return DIAQ_OK;
}

}  // extern "C"
