// diaq_ham_sim_noalloc: the reference-semantics time evolution (diaq_ham_sim) for callers that
// cannot allocate device memory.
//
// Who needs it: code that runs as a plugin inside a host framework which owns the GPU's memory
// through its own pool allocator (such frameworks reserve most of the device up front, so a
// cudaMalloc from inside the plugin fails or splits the pool), and latency-critical loops where
// the implicit synchronisation and unbounded latency of cudaMalloc/cudaFree are not acceptable.
// diaq_ham_sim obtains its six work vectors from cudaMallocAsync on every call; this entry point
// uses a fixed scratch area compiled into the library instead and allocates nothing.
//
// The scratch is the file-scope array below: 6 vectors of kNoAllocMaxRows doubles = 3 MiB.  Every
// GPU that loads the library holds it until the process exits.  Matrices with more rows are
// rejected with DIAQ_ERR_INVALID.  All calls share the one array and it keeps the last call's
// contents; nothing in it has to start at zero (each work vector is written before it is read),
// but two calls whose work overlaps on the GPU -- on different streams, or from different host
// threads -- race on it and corrupt each other's results.
//
// Host code must not pass the array's name to a kernel: in host code the name is only a
// host-side stand-in.  The device address is looked up with cudaGetSymbolAddress once per
// device, with that device current, on the first call made on it; that first call should come
// before any stream capture.
#include <mutex>

#include "diaq_internal.cuh"

namespace diaq_gb300 {

int ham_sim_run(const Matrix &H, const double *p0r, const double *p0i, double t, int64_t r, int m,
                double *outr, double *outi, double *work, cudaStream_t s, const uint32_t *tmask);
const uint32_t *existing_tile_mask(const Matrix &A, cudaStream_t s);

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 16;
constexpr int kNoAllocVectors = 6;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_ham_sim_scratch[kNoAllocVectors * kNoAllocMaxRows];

static std::mutex g_scratch_mu;
static double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
static int scratch_on_current_device(double **out) {
    int dev = 0;
    DQ_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(DIAQ_ERR_UNSUPPORTED, "ham_sim_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        DQ_CUDA(cudaGetSymbolAddress((void **)&p, g_ham_sim_scratch));
        if (!p) return set_error(DIAQ_ERR_CUDA, "ham_sim_noalloc: no device address for the scratch array");
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_ham_sim_noalloc(diaq_matrix_t H, const double *psi0_re, const double *psi0_im, double t,
                         int64_t r, int max_iterations, double *psi_re, double *psi_im, void *stream) {
    if (!H) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H is null");
    if (H->rows != H->cols) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H must be square");
    if (H->prec != DIAQ_C128) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: H must be c128");
    if (r < 0) return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: r must be non-negative");
    if (H->rows > kNoAllocMaxRows)
        return set_error(DIAQ_ERR_INVALID, "ham_sim_noalloc: H has " + std::to_string(H->rows) +
                                               " rows; the built-in scratch holds at most " +
                                               std::to_string(kNoAllocMaxRows) + " (use diaq_ham_sim)");
    if (H->rows == 0) return DIAQ_OK;
    if (!psi0_re || !psi0_im || !psi_re || !psi_im)
        return set_error(DIAQ_ERR_INVALID, "hamiltonian_simulation_cuda: vector pointer is NULL");
    double *work = nullptr;
    DQ_TRY(scratch_on_current_device(&work));
    // H's zero-tile mask only if an earlier call already built it: building one allocates
    return ham_sim_run(*H, psi0_re, psi0_im, t, r, max_iterations, psi_re, psi_im, work, (cudaStream_t)stream,
                       existing_tile_mask(*H, (cudaStream_t)stream));
}

}  // extern "C"
