/*
 * diaq_gb300.h -- C ABI of libdiaq_gb300.so, the GB300 (sm_103a) implementation of DiaQ's
 * diagonal-sparse hot path: complex SpMV, diagonal-pair SpGEMM with its structural dry-run,
 * Taylor + scaling-and-squaring matrix exponential, and Hamiltonian time evolution.
 *
 * Conventions
 *  - Every function returns a diaq_status (0 = DIAQ_OK).  On failure diaq_last_error() gives a
 *    message for the calling thread.  CUDA failures read "CUDA error: <text> (file:line)", the
 *    text the reference raises (src/cuda_check.hpp:11-18).
 *  - A matrix is the DiaQ format: rows x cols, ndiag distinct diagonal offsets in slot order
 *    (column = row + offset), and the values of each diagonal back to back in two float64
 *    arrays re[] / im[] ("packed": diagonal k starts at sum of the lengths of diagonals < k;
 *    the length of diagonal d is min(rows, cols) minus the part outside the matrix), the device
 *    layout of the reference (src/deviceMatrix_gpu.cu:30-55).
 *  - Vectors are SoA: separate real and imaginary arrays.  Several right-hand sides are stored
 *    one after another with leading dimension ld (element (q, i) at x[q * ld + i]).
 *  - `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).  Functions
 *    documented as asynchronous only enqueue work; the others return after the work is done.
 *  - Sizes are 64-bit; diagonal offsets are int32.
 */
#ifndef DIAQ_GB300_H
#define DIAQ_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DIAQ_OK = 0,
    DIAQ_ERR_INVALID = 1,     /* bad argument: shapes, offsets, null pointers */
    DIAQ_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    DIAQ_ERR_OOM = 3,         /* device allocation failed */
    DIAQ_ERR_UNSUPPORTED = 4, /* valid request the library does not handle */
    DIAQ_ERR_TIMEOUT = 5      /* a bounded device-side wait gave up */
} diaq_status;

typedef enum {
    DIAQ_C128 = 0,  /* complex double, SoA float64 */
    DIAQ_C64 = 1,   /* complex float, SoA float32 */
    DIAQ_C128F2 = 2 /* complex double held as float pairs (hi + lo, ~48-bit significand, 16 bytes
                       per value) so that SpMV runs on the FP32 pipes: on GB300 FP64 issues at
                       1/58 of the FP32 rate.  Relative error ~1e-14; magnitudes in about
                       [1e-30, 1e38].  Supports create / download / copy / convert (to and from
                       c128) and SpMV with float64 vectors (diaq_spmv_z, diaq_spmm,
                       diaq_spmv_host); other operations return DIAQ_ERR_UNSUPPORTED. */
} diaq_precision;

typedef enum {
    DIAQ_EVOLVE_C128 = 0, /* complex128 throughout (the reference's arithmetic) */
    DIAQ_EVOLVE_MIXED = 1, /* complex64 matrix and Taylor terms, compensated float sums,
                              float64 state */
    DIAQ_EVOLVE_HORNER = 2 /* complex64 matrix, the Taylor polynomial evaluated in Horner form
                              in float32 (w_k = psi + A w_{k+1} / (k+1), w_m = psi), the last
                              step psi + A w_1 in float64: no running sum, half the state
                              traffic of DIAQ_EVOLVE_MIXED */
} diaq_evolve_mode;

typedef struct diaq_matrix_s *diaq_matrix_t;
typedef struct diaq_evolve_s *diaq_evolve_t;
typedef struct diaq_mlp_s *diaq_mlp_t;
typedef struct diaq_batch_s *diaq_batch_t;

/* Message of the last failing call on this thread ("" if none). */
const char *diaq_last_error(void);

/* Library version string. */
const char *diaq_version(void);

/* ------------------------------------------------------------------------------------------
 * Device matrices.  Replace deviceDiaQMatrix (src/deviceMatrix_gpu.hpp:37-68,
 * src/deviceMatrix_gpu.cu:30-113).
 * ---------------------------------------------------------------------------------------- */

/* Create a device matrix from packed float64 values (re/im on the host, or on the device when
 * values_on_device != 0).  precision DIAQ_C64 rounds the values to float32 on the device.
 * re/im may both be NULL for a matrix of zeros.  Offsets must be distinct and inside the
 * matrix.  Replaces deviceDiaQMatrix(const shared_ptr<diaQMatrix>&) (src/deviceMatrix_gpu.cu:58-76). */
int diaq_matrix_create(int64_t rows, int64_t cols, int32_t ndiag, const int32_t *offsets,
                       const double *re, const double *im, int values_on_device, int precision,
                       void *stream, diaq_matrix_t *out);

/* Free a device matrix (NULL is ignored).  Replaces ~deviceDiaQMatrix (src/deviceMatrix_gpu.cu:78-85). */
int diaq_matrix_destroy(diaq_matrix_t A);

/* Shape, diagonal count, stored (packed) value count and precision. */
int diaq_matrix_info(diaq_matrix_t A, int64_t *rows, int64_t *cols, int32_t *ndiag,
                     int64_t *total, int *precision);

/* Copy the offsets (slot order) to a host array of ndiag entries. */
int diaq_matrix_offsets(diaq_matrix_t A, int32_t *offsets);

/* Stored values that lie in 32-row tiles holding a nonzero (real or imaginary part): the values
 * the SpMV and time-evolution kernels read, since they skip all-zero tiles -- the figure their
 * algorithmic bytes are counted from.  Synchronous on stream.  No counterpart in the reference. */
int diaq_matrix_live_values(diaq_matrix_t A, int64_t *live, void *stream);

/* Packed float64 values to re/im (host arrays, or device arrays when dst_on_device != 0).
 * Replaces deviceDiaQMatrix::to_host (src/deviceMatrix_gpu.cu:97-113). */
int diaq_matrix_download(diaq_matrix_t A, double *re, double *im, int dst_on_device, void *stream);

/* A second device matrix with the same values.  Replaces deviceDiaQMatrix::copy
 * (src/deviceMatrix_gpu.cu:87-95). */
int diaq_matrix_copy(diaq_matrix_t A, void *stream, diaq_matrix_t *out);

/* The same matrix in another precision (c128 -> c64 rounds to nearest). */
int diaq_matrix_convert(diaq_matrix_t A, int precision, void *stream, diaq_matrix_t *out);

/* Drop the diagonals whose values are all exactly zero (real and imaginary == 0.0).  Replaces
 * diaQMatrix::pruneMatrix (src/diaQMatrix.hpp:1543-1604). */
int diaq_matrix_prune(diaq_matrix_t A, void *stream, diaq_matrix_t *out);

/* H = sum_k c_k P_k built on the device from n_strings Pauli strings over n_qubits (<= 30).
 * String k: complex coefficient (coeff_re[k], coeff_im[k]; coeff_im may be NULL), flip mask
 * x_mask[k] (X or Y) and phase mask z_mask[k] (Z or Y) over the basis index, bit p belonging to
 * qubit n_qubits-1-p (qubit 0 most significant, the Kronecker order).  The result holds the
 * diagonals that are not exactly zero, ascending.  Replaces building Hamiltonians with the
 * Kronecker helpers (src/spKron.cpp:189-1271), which overflow 32-bit indices at 2^16 rows. */
int diaq_matrix_from_pauli(int n_qubits, int32_t n_strings, const double *coeff_re,
                           const double *coeff_im, const uint64_t *x_mask, const uint64_t *z_mask,
                           int precision, void *stream, diaq_matrix_t *out);

/* A device matrix from a dense rows x cols array of interleaved complex128 values, row-major
 * (numpy / torch complex128), on the device (on_device != 0) or the host: the diagonals holding
 * a value other than exact zero, in ascending order, as from_numpy builds them
 * (src/dense_to_diagonals.hpp:20-58, include/pythonWrappers.cpp:146-193), but on the GPU.
 * Synchronous. */
int diaq_matrix_from_dense(int64_t rows, int64_t cols, const double *dense, int on_device,
                           int precision, void *stream, diaq_matrix_t *out);

/* The dense rows x cols array (interleaved complex128, row-major) of A, written on the device
 * (on_device != 0; asynchronous on stream) or the host (synchronous).  Replaces to_numpy(A)
 * after DeviceMatrix.to_host() (include/pythonWrappers.cpp:195-218, src/deviceMatrix_gpu.cu:62-113). */
int diaq_matrix_to_dense(diaq_matrix_t A, double *dense, int on_device, void *stream);

/* ------------------------------------------------------------------------------------------
 * SpMV.  Replaces spmv_device (src/spMV_gpu.cu:142-168): y = A x on device arrays, y
 * overwritten, asynchronous on stream.  The kernels skip the 32-row tiles of a diagonal that hold
 * only zeros, from a mask of A taken on the first call after A's values were last written (that
 * call waits for the stream once); outside graph capture only.
 * ---------------------------------------------------------------------------------------- */

/* c128 matrix, float64 vectors. */
int diaq_spmv_z(diaq_matrix_t A, const double *x_re, const double *x_im, double *y_re,
                double *y_im, void *stream);

/* c64 matrix, float32 vectors. */
int diaq_spmv_c(diaq_matrix_t A, const float *x_re, const float *x_im, float *y_re, float *y_im,
                void *stream);

/* nrhs right-hand sides at once (each diagonal value is read once per launch); vectors of the
 * matrix's precision, element (q, i) at x[q*ldx + i], y[q*ldy + i]. */
int diaq_spmm(diaq_matrix_t A, int nrhs, const void *x_re, const void *x_im, int64_t ldx,
              void *y_re, void *y_im, int64_t ldy, void *stream);

/* Host vectors in and out (x, y copied; A stays on the device).  Replaces
 * spmv_cuda(shared_ptr<deviceDiaQMatrix>, x) (src/spMV_gpu.cu:170-204).  c128 or c128f2 matrix.
 * Synchronous. */
int diaq_spmv_host(diaq_matrix_t A, const double *x_re, const double *x_im, double *y_re,
                   double *y_im);

/* y = A^n x by n repeated products on the device, host vectors.  n = 0 copies x (square A
 * only); n > 1 needs a square A.  Replaces spMV_ntimes_cuda (src/spMV_ntimes_gpu.cu:61-263).
 * c128 only.  Synchronous. */
int diaq_spmv_ntimes_host(diaq_matrix_t A, const double *x_re, const double *x_im, int n,
                          double *y_re, double *y_im);

/* C = A B with A in the row-aligned DIA format and B, C dense, every array on the device:
 * offsets int64[n_diags]; vals[k*n_rows + r] = A[r, r + offsets[k]] (entries whose column lies
 * outside [0, n_cols) are ignored); B n_cols x n_right and C n_rows x n_right, row-major;
 * float64 (is_complex = 0) or interleaved complex128 (is_complex != 0).  C is overwritten;
 * diagonals are summed in the order given.  Asynchronous on stream.  Replaces spmm_dia_device
 * (src/spMM_device_gpu.cu:113-127, bound at include/pythonWrappers.cpp:622-633). */
int diaq_spmm_dia_device(const int64_t *offsets, const void *vals, int n_diags, int64_t n_rows,
                         int64_t n_cols, const void *B, int64_t n_right, void *C, int is_complex,
                         void *stream);

/* ------------------------------------------------------------------------------------------
 * SpGEMM.  Replaces product_device / product_cuda (src/spGEMM_gpu.cu:84-161) and the host
 * dry-run of product (src/spGEMM.cpp:346-378).
 * ---------------------------------------------------------------------------------------- */

/* Structural dry-run on the device: the ascending distinct offsets dA+dB inside
 * [-(rowsA-1), colsB-1].  offsets_out (host) needs room for ndiagA*ndiagB entries; *count
 * receives the number written.  Synchronous. */
int diaq_spgemm_symbolic(diaq_matrix_t A, diaq_matrix_t B, int32_t *offsets_out, int32_t *count,
                         void *stream);

/* Numeric pass into C, whose offsets must come from diaq_spgemm_symbolic(A, B) (every product
 * diagonal present); per result diagonal the pairs are summed in A-slot order.  Asynchronous. */
int diaq_spgemm_numeric(diaq_matrix_t A, diaq_matrix_t B, diaq_matrix_t C, void *stream);

/* C = A B (dry-run + numeric); prune != 0 also drops exact-zero diagonals, as the host entry
 * point `product` does (src/spGEMM.cpp:516-534); product(DeviceMatrix, DeviceMatrix) does not.
 * A and B must have the same precision.  Synchronous. */
int diaq_spgemm(diaq_matrix_t A, diaq_matrix_t B, int prune, void *stream, diaq_matrix_t *C);

/* ------------------------------------------------------------------------------------------
 * Norms and the matrix exponential.
 * ---------------------------------------------------------------------------------------- */

/* Max column sum of |re|+|im| (src/diaQMatrix.hpp:1287-1358).  Synchronous. */
int diaq_norm1_est(diaq_matrix_t A, double *out, void *stream);

/* Frobenius norm of the stored values (src/diaQMatrix.hpp:1255-1284).  Synchronous. */
int diaq_frobenius(diaq_matrix_t A, double *out, void *stream);

/* A^n: s squarings for n = 2^s, else binary exponentiation (src/spPow.cpp:19-56,
 * src/spPow_gpu.cu:21-56).  prune as in diaq_spgemm. */
int diaq_pow(diaq_matrix_t A, int n, int prune, void *stream, diaq_matrix_t *out);

/* exp(-i t A) by Taylor + scaling and squaring: s = ceil(log2((|t| ||A||_1 + 1e-12)/cutoff)),
 * Taylor terms of t/2^s until the Frobenius norm of a term < max(1e-15, tol 2^-s) or
 * max_iterations, then s squarings (src/spME.cpp:230-295 with :158-223; its GPU twin
 * src/spME_gpu.cu:156-294).  prune != 0 prunes every product as the CPU path does.
 * s_out / terms_out may be NULL.  Synchronous. */
int diaq_expm_negative(diaq_matrix_t A, double t, int max_iterations, double scale_cutoff,
                       double tolerance, int prune, void *stream, diaq_matrix_t *U, int *s_out,
                       int *terms_out);

/* exp(-i t A) as the reference's Pade routine computes it (diaq::expm_negative_pade,
 * src/spME.cpp:298-445, declared in src/matrixKernels.hpp:86).  A matrix with one diagonal gets
 * the single-diagonal exponential (exp(t b)(cos(t a) - i sin(t a)) of its values on the main
 * diagonal of the identity, :309-336); every other input fails as the reference's fails:
 * rectangular -> DIAQ_ERR_INVALID "addMatrixScaled: matrix shapes do not match"; square with two
 * or more diagonals -> DIAQ_ERR_UNSUPPORTED "set: diagonal index not present in dIndices." (its
 * inverse, :521-589, stores the solution into a matrix holding about half the diagonals); square
 * with none -> DIAQ_ERR_UNSUPPORTED "Matrix is singular, cannot compute inverse." (the reference's
 * process ends there).  Synchronous. */
int diaq_expm_negative_pade(diaq_matrix_t A, double t, int max_iterations, double scale_cutoff,
                            double tolerance, void *stream, diaq_matrix_t *U);

/* exp(A), same method (src/spME.cpp:13-150, src/spME_gpu.cu:10-150). */
int diaq_expm(diaq_matrix_t A, int max_iterations, double scale_cutoff, double tolerance,
              int prune, void *stream, diaq_matrix_t *U);

/* ------------------------------------------------------------------------------------------
 * Time evolution psi(t) = exp(-i H t) psi0.
 * ---------------------------------------------------------------------------------------- */

/* The reference's fused Hamiltonian simulation (hamiltonian_simulation_cuda,
 * src/spHamSim_gpu_all_fused.cu:287-376): t is the TOTAL time, r steps of dt = t/r, each step
 * exactly max_iterations Taylor terms (no scaling, no truncation test, no renormalisation);
 * r = 0 copies psi0.  H must be square and c128; psi0 and psi_out are float64 device arrays of
 * length N (psi_out may equal psi0).  Asynchronous. */
int diaq_ham_sim(diaq_matrix_t H, const double *psi0_re, const double *psi0_im, double t,
                 int64_t r, int max_iterations, double *psi_re, double *psi_im, void *stream);

/* An evolution plan for nrhs states under H (a c128 matrix; mode DIAQ_EVOLVE_MIXED keeps its own
 * c64 copy) with the work vectors it needs.  No counterpart in the reference, whose
 * hamiltonian_simulation_cuda (src/spHamSim_gpu_all_fused.cu:287-376) evolves one state with a
 * fixed number of terms and no sub-steps; with nrhs = 1, mode C128, 2^s = 1 and m =
 * max_iterations a plan computes the same thing. */
int diaq_evolve_create(diaq_matrix_t H, int nrhs, int mode, diaq_evolve_t *out);

int diaq_evolve_destroy(diaq_evolve_t E);

/* Advance the nrhs states in place by `steps` time steps of dt, each 2^substeps_log2 sub-steps
 * of m Taylor terms.  psi_re/psi_im: float64 device arrays, state q at psi[q*ld ..]; ld must be
 * N.  The first call for a given (dt, s, m, psi) records one step as a CUDA graph; every step is
 * a replay.  A plan keeps up to 16 recorded steps and drops them all when a 17th is needed.
 * dt must be finite.  Asynchronous on stream: a bounded wait of the bulk-copy kernels (variants
 * 10 and 11, chosen only through diaq_evolve_set_config) that gave up during this run is reported
 * by diaq_evolve_check, or else by the next diaq_evolve_run once the run has finished, as
 * DIAQ_ERR_TIMEOUT; the states of that run are then not valid. */
int diaq_evolve_run(diaq_evolve_t E, double *psi_re, double *psi_im, int64_t ld, double dt,
                    int64_t steps, int substeps_log2, int m, void *stream);

/* diaq_evolve_run with host arrays: the nrhs states (state q at psi[q*N ..]) are copied to the
 * device, advanced, and copied back.  Synchronous.  The device copy of the states belongs to the
 * plan: allocated by the first call, reused by the later ones, freed with the plan.
 * A wait that gave up during the run is reported by this call (DIAQ_ERR_TIMEOUT).
 * One step (steps == 1) of an even nrhs >= 8 in the float32-term modes, once the plan has its
 * launch shape, runs as two plans of nrhs / 2 states (made on first use, sharing the plan's
 * float32 matrix): the second half is copied up and the first copied down while the GPU works;
 * the results are the same bits. */
int diaq_evolve_run_host(diaq_evolve_t E, double *psi_re, double *psi_im, double dt, int64_t steps,
                         int substeps_log2, int m);

/* Wait for the plan's last run on its stream and report whether a bounded wait of a bulk-copy
 * kernel gave up in it: DIAQ_ERR_TIMEOUT (the error is then cleared), else DIAQ_OK.  No
 * counterpart in the reference, whose kernels do not wait inside a block. */
int diaq_evolve_check(diaq_evolve_t E);

/* Time bound, in nanoseconds, of one device-side wait of the bulk-copy kernels (variants 10 and
 * 11): a consumer warp's wait for a filled shared-memory stage and the producer's wait for a free
 * one (default 20 ms; 0 restores it).  A wait that runs out records DIAQ_ERR_TIMEOUT for
 * diaq_evolve_check and its warp leaves; the producer always waits for its copies in flight
 * (bounded by max(wait, 10 ms)) before its block finishes.  Drops the recorded graphs.  No
 * counterpart in the reference. */
int diaq_evolve_set_wait_limit(diaq_evolve_t E, int64_t wait_ns);

/* Launch shape of the plan's term kernel: states per block (1..8: one launch covers every state,
 * in chunks of this many per block, the chunks of a row tile side by side so that the matrix
 * tile comes from HBM about once), rows per thread (1, 2, or 4 for the float32 modes) and the
 * kernel variant `pipelined`: 0 registers only; for the float32 modes with 4 rows, 1 streams the
 * next diagonals through shared memory with asynchronous copies, 2 / 3 / 4 read unaligned state
 * windows as aligned vectors shifted across lanes and prefetch the matrix into L2 4 / 8 / 0
 * diagonals ahead; for the float32 modes with (4 states, 1 row), 6 / 7 / 8 keep the work vectors
 * interleaved in tiles of 32 rows x 4 states (any window one aligned vector per lane) and load the
 * matrix 0 / 4 / 8 diagonals ahead into registers; 9 with 8 states per thread; 10 / 11 feed the
 * block's live diagonals through a ring of shared-memory stages filled by bulk asynchronous copies
 * (matrix values and state windows / matrix values only; never picked by the autotuner, which
 * measured them slower); 12 is 9 with 32-bit row arithmetic and
 * each diagonal's metadata in one 16-byte shared-memory record (n_pad * states < 2^31).  Every kernel of a
 * plan skips the 32-row tiles of a diagonal that hold only zeros (a mask built from the matrix the
 * plan reads).
 * 0 states = choose automatically: on the first run the autotuner times the candidate shapes on
 * two steps of scratch copies of the states and keeps the fastest, caching the choice in a JSON
 * file (DIAQ_AUTOTUNE_CACHE, else $HOME/.cache/diaq_gb300/autotune.json).  Setting a shape drops
 * the recorded graphs.  pipelined may be NULL in diaq_evolve_config. */
int diaq_evolve_set_config(diaq_evolve_t E, int states_per_block, int rows_per_thread, int pipelined);
int diaq_evolve_config(diaq_evolve_t E, int *states_per_block, int *rows_per_thread, int *pipelined);

/* on != 0: after every step rescale each state to norm 1, the norm computed in float64 (the
 * exact evolution is unitary; this removes the drift of the truncated series).  Off by default:
 * the reference's rule does not renormalise. */
int diaq_evolve_set_renormalize(diaq_evolve_t E, int on);

/* Kernel launches in one recorded time step of the last graph built (0 before any run). */
int diaq_evolve_launches_per_step(diaq_evolve_t E);

/* Norm-bound choice of the sub-step count and Taylor degree for one time step tau: the
 * reference's scaling rule s = ceil(log2(tau*norm1/cutoff)) (src/spME.cpp:256-262) gives 2^s
 * sub-steps of theta = tau*norm1/2^s each, and m is the smallest degree whose Taylor remainder
 * bound theta^(m+1)/(m+1)! * exp(theta) is <= tol / 2^s (capped at max_m).  Host-only. */
int diaq_select_sm(double norm1, double tau, double tol, double scale_cutoff, int max_m,
                   int *substeps_log2, int *m);

/* The cheapest (2^s * m) pair whose remainder bound meets tol (per step, split over the 2^s
 * sub-steps as in diaq_select_sm), searching s = 0..max_s.  Host-only. */
int diaq_select_sm_min_cost(double norm1, double tau, double tol, int max_s, int max_m,
                            int *substeps_log2, int *m);

/* diaq_ham_sim with host vectors (psi0 uploaded once, the result downloaded once), as
 * hamiltonian_simulation_cuda does.  Synchronous. */
int diaq_ham_sim_host(diaq_matrix_t H, const double *psi0_re, const double *psi0_im, double t,
                      int64_t r, int max_iterations, double *psi_re, double *psi_im);

/* ------------------------------------------------------------------------------------------
 * Batched evolution: n_inst Hamiltonians of any sizes (all c64 -> float32 terms, or all c128 ->
 * float64 terms; compensated sums and float64 states either way), instance i with nrhs[i]
 * states stored at psi_re[i] / psi_im[i] (device, state q at [q*N_i ..]).  One step is one
 * persistent, work-queued launch per Taylor phase over every instance, recorded as a CUDA graph.
 * No counterpart in the reference, which evolves one state of one Hamiltonian per call
 * (src/spHamSim_gpu_all_fused.cu:287-376).  The matrices and state arrays must outlive the batch.
 * ---------------------------------------------------------------------------------------- */
int diaq_batch_create(int n_inst, const diaq_matrix_t *H, const int *nrhs, double *const *psi_re,
                      double *const *psi_im, diaq_batch_t *out);
int diaq_batch_destroy(diaq_batch_t B);

/* Advance every state by `steps` steps of dt; instance i uses 2^substeps_log2[i] sub-steps of
 * m[i] terms.  The first run (and any change of dt or schedule) records the step's graph; the
 * first run also autotunes the launch shape unless one was set.  Asynchronous on stream after
 * the stream's earlier work has finished. */
int diaq_batch_run(diaq_batch_t B, double dt, const int *substeps_log2, const int *m, int64_t steps,
                   void *stream);

/* Force a launch shape (states per launch 1, 2, 4 or 8; rows per thread 1, 2, or 4 for c64), or
 * 0 states for automatic; and read back the shape and the phases per step. */
int diaq_batch_set_config(diaq_batch_t B, int states_per_launch, int rows_per_thread);
int diaq_batch_config(diaq_batch_t B, int *states_per_launch, int *rows_per_thread, int *phases_per_step);

/* on != 0: evaluate the Taylor polynomial of instances with m >= 2 in Horner form (as
 * DIAQ_EVOLVE_HORNER: w_k = psi + A w_{k+1} / (k+1) in the batch's precision, the last step in
 * float64), no running sum and no copy phase; off (the compensated forward sum) by default.
 * Drops the recorded step. */
int diaq_batch_set_horner(diaq_batch_t B, int on);

/* on != 0 (the default): complex64 instances with 4 to 32 states keep their float32 work vectors
 * interleaved in tiles of 32 rows x 4 states and run in a second kernel per phase, one block per
 * block of rows and all the states; off: every instance planar.  Same arithmetic either way.
 * Drops the recorded step. */
int diaq_batch_set_interleaved(diaq_batch_t B, int on);

/* ------------------------------------------------------------------------------------------
 * The learned (s, m) proposer: an FP32 MLP 16 -> 64 -> 64 -> 21 + 30 logits (ReLU), trained
 * with softmax cross-entropy on both heads (s in 0..20, m in 1..30) and Adam.  No counterpart in
 * the reference, whose exponential picks s by the norm bound alone (src/spME.cpp:256-262).
 * All arrays are device arrays, row-major (row b = one instance): X[B][16] float32, labels
 * int32.  Asynchronous on stream except create/destroy/get/set.
 * ---------------------------------------------------------------------------------------- */

/* Number of float parameters (W1[16][64] b1[64] W2[64][64] b2[64] W3[64][51] b3[51]). */
int diaq_mlp_num_params(void);

/* He-initialised network (deterministic for a seed), Adam state zeroed. */
int diaq_mlp_create(uint64_t seed, diaq_mlp_t *out);
int diaq_mlp_destroy(diaq_mlp_t M);

/* Copy the flat parameter vector to / from the host (set also resets the Adam state). */
int diaq_mlp_get_params(diaq_mlp_t M, float *host_out);
int diaq_mlp_set_params(diaq_mlp_t M, const float *host_in);

/* logits[B][51]: the 21 s-logits then the 30 m-logits. */
int diaq_mlp_forward(diaq_mlp_t M, const float *X, int B, float *logits, void *stream);

/* Gradient of the mean (over the batch) of CE_s + CE_m into grad_out[num_params] and the
 * per-row loss into loss_out[B] (either may be NULL); parameters unchanged. */
int diaq_mlp_gradient(diaq_mlp_t M, const float *X, const int32_t *s_label, const int32_t *m_label,
                      int B, float *grad_out, float *loss_out, void *stream);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the batch's gradient; loss_out[B] may be NULL. */
int diaq_mlp_train_step(diaq_mlp_t M, const float *X, const int32_t *s_label,
                        const int32_t *m_label, int B, float lr, float *loss_out, void *stream);

/* argmax of each head: s_out[B] in 0..20, m_out[B] in 1..30. */
int diaq_mlp_propose(diaq_mlp_t M, const float *X, int B, int32_t *s_out, int32_t *m_out,
                     void *stream);

/* diaq_ham_sim for callers that cannot allocate device memory.  No counterpart in the
 * reference.  Same arguments, results and stream semantics as diaq_ham_sim, but its work
 * vectors live in a scratch array built into the library (3 MiB per GPU, held until the process
 * exits) instead of cudaMallocAsync, so the call allocates nothing.  Limit: H may have at most
 * 65536 rows (16 qubits); larger matrices are rejected with DIAQ_ERR_INVALID.  All calls share
 * the scratch: calls whose work overlaps on the GPU (other streams, other host threads) race on
 * it.  The first call on a device looks up the scratch's device address; make that first call
 * before any stream capture. */
int diaq_ham_sim_noalloc(diaq_matrix_t H, const double *psi0_re, const double *psi0_im, double t,
                         int64_t r, int max_iterations, double *psi_re, double *psi_im, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* DIAQ_GB300_H */
