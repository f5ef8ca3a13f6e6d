// Time evolution psi(t) = exp(-i H t) psi0 with the reference's semantics.
// Replaces hamiltonian_simulation_cuda / expm_action_taylor_device
// (src/spHamSim_gpu_all_fused.cu:235-376): one fused launch per Taylor term (SpMV + term
// scaling + accumulation) instead of three, and no device-wide synchronisation per step.
#include <cmath>

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

// r steps of dt = t / r, each exactly m terms: acc = psi + sum_k term_k with
// term_k = (-i dt/k) H term_{k-1}, term_0 = psi.  work holds 6 vectors of n doubles.
// tmask: H's zero-tile mask or NULL.
int ham_sim_run(const Matrix &H, const double *p0r, const double *p0i, double t, int64_t r, int m,
                double *outr, double *outi, double *work, cudaStream_t s, const uint32_t *tmask) {
    const int64_t n = H.rows;
    const size_t bytes = sizeof(double) * (size_t)n;
    if (r == 0 || m <= 0) {
        // r = 0: psi0 unchanged (src/spHamSim_gpu_all_fused.cu:333-346); m = 0: the sum is psi
        if (outr != p0r) DQ_CUDA(cudaMemcpyAsync(outr, p0r, bytes, cudaMemcpyDeviceToDevice, s));
        if (outi != p0i) DQ_CUDA(cudaMemcpyAsync(outi, p0i, bytes, cudaMemcpyDeviceToDevice, s));
        return DIAQ_OK;
    }
    double *ar = work, *ai = work + n;            // state
    double *br = work + 2 * n, *bi = work + 3 * n;  // next state (the sum)
    double *t0r = work + 4 * n, *t0i = work + 5 * n;  // term ping-pong partner
    DQ_CUDA(cudaMemcpyAsync(ar, p0r, bytes, cudaMemcpyDeviceToDevice, s));
    DQ_CUDA(cudaMemcpyAsync(ai, p0i, bytes, cudaMemcpyDeviceToDevice, s));
    const double dt = t / (double)r;
    for (int64_t step = 0; step < r; ++step) {
        // Term 1 reads the state and starts the sum at state + term_1; from then on the sum
        // holds the state, so the state buffer and t0 ping-pong as term in/out.
        double *tin_r = ar, *tin_i = ai, *tout_r = t0r, *tout_i = t0i;
        for (int k = 1; k <= m; ++k) {
            DQ_TRY(taylor_term_launch(H, tin_r, tin_i, tout_r, tout_i, br, bi, k == 1 ? ar : nullptr,
                                      k == 1 ? ai : nullptr, dt / (double)k, 1, n, s, tmask));
            std::swap(tin_r, tout_r);
            std::swap(tin_i, tout_i);
        }
        std::swap(ar, br);
        std::swap(ai, bi);
    }
    DQ_CUDA(cudaMemcpyAsync(outr, ar, bytes, cudaMemcpyDeviceToDevice, s));
    DQ_CUDA(cudaMemcpyAsync(outi, ai, bytes, cudaMemcpyDeviceToDevice, s));
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_ham_sim(diaq_matrix_t H, const double *psi0_re, const double *psi0_im, double t,
                 int64_t r, int max_iterations, double *psi_re, double *psi_im, void *stream) {
    if (!H) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H is null");
    if (H->rows != H->cols) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H must be square");
    if (H->prec != DIAQ_C128) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H must be c128");
    if (r < 0) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: r must be non-negative");
    if (H->rows == 0) return DIAQ_OK;
    if (!psi0_re || !psi0_im || !psi_re || !psi_im)
        return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: vector pointer is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    double *work = nullptr;
    DQ_CUDA(dev_malloc_async(&work, sizeof(double) * 6 * (size_t)H->rows, s));
    const int st = ham_sim_run(*H, psi0_re, psi0_im, t, r, max_iterations, psi_re, psi_im, work, s,
                               cached_tile_mask(*H, s));
    cudaError_t e = cudaFreeAsync(work, s);
    if (st != DIAQ_OK) return st;
    if (e != cudaSuccess) return cuda_status(e, "cudaFreeAsync", __FILE__, __LINE__);
    return DIAQ_OK;
}

}  // extern "C"

extern "C" {

int diaq_ham_sim_host(diaq_matrix_t H, const double *psi0_re, const double *psi0_im, double t,
                      int64_t r, int max_iterations, double *psi_re, double *psi_im) {
    if (!H) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H is null");
    if (H->rows != H->cols) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H must be square");
    if (H->rows == 0) return DIAQ_OK;
    if (!psi0_re || !psi0_im || !psi_re || !psi_im)
        return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: vector pointer is NULL");
    const int64_t n = H->rows;
    double *buf = nullptr;
    DQ_CUDA(dev_malloc(&buf, sizeof(double) * 2 * (size_t)n));
    cudaError_t e = cudaMemcpy(buf, psi0_re, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(buf + n, psi0_im, sizeof(double) * n, cudaMemcpyHostToDevice);
    int st = e == cudaSuccess ? DIAQ_OK : cuda_status(e, "upload psi0", __FILE__, __LINE__);
    if (st == DIAQ_OK) st = diaq_ham_sim(H, buf, buf + n, t, r, max_iterations, buf, buf + n, nullptr);
    if (st == DIAQ_OK) {
        e = cudaMemcpy(psi_re, buf, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(psi_im, buf + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_status(e, "download psi", __FILE__, __LINE__);
    }
    cudaFree(buf);
    return st;
}

}  // extern "C"

extern "C" {

// Smallest Taylor degree k <= max_m with theta^(k+1)/(k+1)! e^theta <= budget (max_m + 1 if none).
static int taylor_degree(double theta, double budget, int max_m) {
    double term = theta * std::exp(theta);  // k = 0
    for (int k = 1; k <= max_m; ++k) {
        term *= theta / (double)(k + 1);
        if (term <= budget) return k;
    }
    return max_m + 1;
}

int diaq_select_sm_min_cost(double norm1, double tau, double tol, int max_s, int max_m,
                            int *substeps_log2, int *m) {
    if (!substeps_log2 || !m) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    if (!(norm1 >= 0) || !(tol > 0) || max_m < 1 || max_s < 0 || max_s > 30)
        return set_error(DIAQ_ERR_INVALID, "select_sm_min_cost: need norm1 >= 0, tol > 0, max_m >= 1, 0 <= max_s <= 30");
    const double theta0 = std::fabs(tau) * norm1;
    int best_s = -1, best_m = 0;
    double best = 0.0;
    for (int s = 0; s <= max_s; ++s) {
        const int k = taylor_degree(std::ldexp(theta0, -s), std::ldexp(tol, -s), max_m);
        if (k > max_m) continue;
        const double cost = std::ldexp((double)k, s);
        if (best_s < 0 || cost < best) {
            best = cost;
            best_s = s;
            best_m = k;
        }
    }
    if (best_s < 0) return set_error(DIAQ_ERR_UNSUPPORTED, "select_sm_min_cost: no (s, m) in range meets the tolerance");
    *substeps_log2 = best_s;
    *m = best_m;
    return DIAQ_OK;
}

int diaq_select_sm(double norm1, double tau, double tol, double scale_cutoff, int max_m,
                   int *substeps_log2, int *m) {
    if (!substeps_log2 || !m) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    if (!(norm1 >= 0) || !(tol > 0) || !(scale_cutoff > 0) || max_m < 1)
        return set_error(DIAQ_ERR_INVALID, "select_sm: need norm1 >= 0, tol > 0, cutoff > 0, max_m >= 1");
    const double theta0 = std::fabs(tau) * norm1;
    const double scaled = theta0 + 1e-12;
    int s = scaled > scale_cutoff ? (int)std::ceil(std::log2(scaled / scale_cutoff)) : 0;
    if (s > 30) return set_error(DIAQ_ERR_UNSUPPORTED, "select_sm: more than 2^30 sub-steps");
    const double theta = std::ldexp(theta0, -s);
    const double budget = std::ldexp(tol, -s);
    // remainder bound theta^(k+1)/(k+1)! e^theta, built up term by term
    double term = theta * std::exp(theta);  // k = 0
    int k = 0;
    while (k < max_m) {
        ++k;
        term *= theta / (double)(k + 1);
        if (term <= budget) break;
    }
    *substeps_log2 = s;
    *m = k;
    return DIAQ_OK;
}

}  // extern "C"
