// On-device Hamiltonian builder: H = sum_k c_k P_k from Pauli strings, straight into the DiaQ
// layout.  Replaces building test Hamiltonians with the reference's Kronecker helpers
// (src/spKron.cpp:189-1271), whose 32-bit flat indices overflow at 2^16 rows
// (src/diaQMatrix.hpp:455-509).
//
// String k is given by two bit masks over the basis index (bit p belongs to qubit n-1-p, qubit 0
// being the most significant): x = flip mask (X or Y), z = phase mask (Z or Y).  On a basis state
// |b>:  P|b> = i^(#Y) (-1)^popcount(b & z) |b ^ x>.  So H[b ^ x, b] += c i^(#Y) (-1)^popcount(b & z),
// on the diagonal d = b - (b ^ x): each string touches the 2^popcount(x) offsets
// sum_{p in x} +-2^p.  The host enumerates those offsets (the structure); one thread per
// (diagonal, row) then sums the contributing strings in input order.  Diagonals that come out
// exactly zero are dropped, so the structure equals that of the dense matrix's nonzero diagonals,
// ascending.
#include <algorithm>
#include <map>
#include <vector>

#include "spmv_kernel.cuh"

namespace diaq_gb300 {

struct PauliTerm {
    double cr, ci;     // coefficient times i^(#Y)
    uint64_t x, z;
};

// For diagonal k: the strings (indices into terms) that may land on it, in input order.
template <typename T>
__global__ void pauli_fill_kernel(const DiagMeta *__restrict__ meta, int nd, const PauliTerm *__restrict__ terms,
                                  const int32_t *__restrict__ list_start, const int32_t *__restrict__ list,
                                  T *__restrict__ re, T *__restrict__ im) {
    for (int k = blockIdx.y; k < nd; k += gridDim.y) {
        const DiagMeta m = meta[k];
        const int32_t a = list_start[k], b = list_start[k + 1];
        for (int64_t r = m.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m.hi;
             r += (int64_t)gridDim.x * blockDim.x) {
            const uint64_t col = (uint64_t)(r + m.off);
            const uint64_t row = (uint64_t)r;
            double sr = 0.0, si = 0.0;
            for (int32_t j = a; j < b; ++j) {
                const PauliTerm t = terms[list[j]];
                if ((row ^ col) != t.x) continue;
                const double sg = (__popcll(col & t.z) & 1) ? -1.0 : 1.0;
                sr += sg * t.cr;
                si += sg * t.ci;
            }
            re[m.base + r] = (T)sr;
            im[m.base + r] = (T)si;
        }
    }
}

int pauli_build(int nq, int32_t ns, const double *cre, const double *cim, const uint64_t *xm, const uint64_t *zm,
                int prec, cudaStream_t s, Matrix **out) {
    if (nq < 1 || nq > 30) return set_error(DIAQ_ERR_INVALID, "pauli: 1 <= n_qubits <= 30");
    if (prec == DIAQ_C128F2) {  // built in float64, then split into float pairs
        Matrix *D = nullptr;
        DQ_TRY(pauli_build(nq, ns, cre, cim, xm, zm, DIAQ_C128, s, &D));
        const int st = copy_as(*D, DIAQ_C128F2, s, out);
        cudaStreamSynchronize(s);
        destroy(D);
        return st;
    }
    if (ns < 0 || (ns > 0 && (!cre || !xm || !zm))) return set_error(DIAQ_ERR_INVALID, "pauli: NULL string arrays");
    const int64_t N = int64_t(1) << nq;
    const uint64_t full = (uint64_t)N - 1;
    std::vector<PauliTerm> terms(ns);
    std::map<int64_t, std::vector<int32_t>> by_off;  // offset -> strings, ascending offsets
    for (int32_t k = 0; k < ns; ++k) {
        if ((xm[k] | zm[k]) & ~full) return set_error(DIAQ_ERR_INVALID, "pauli: mask has bits beyond n_qubits");
        const int ny = __builtin_popcountll(xm[k] & zm[k]);
        double r = cre[k], i = cim ? cim[k] : 0.0;
        for (int t = 0; t < (ny & 3); ++t) {  // times i^(#Y)
            const double nr = -i, ni = r;
            r = nr;
            i = ni;
        }
        terms[k] = PauliTerm{r, i, xm[k], zm[k]};
        // offsets: sum over the flipped bits of +-2^p
        std::vector<int> bits;
        for (int p = 0; p < nq; ++p)
            if (xm[k] >> p & 1) bits.push_back(p);
        const int nb = (int)bits.size();
        for (int mask = 0; mask < (1 << nb); ++mask) {
            int64_t d = 0;
            for (int j = 0; j < nb; ++j) d += ((mask >> j) & 1) ? (int64_t(1) << bits[j]) : -(int64_t(1) << bits[j]);
            by_off[d].push_back(k);
        }
    }
    std::vector<int32_t> off, starts{0}, list;
    for (auto &kv : by_off) {
        off.push_back((int32_t)kv.first);
        list.insert(list.end(), kv.second.begin(), kv.second.end());
        starts.push_back((int32_t)list.size());
    }
    Matrix *M = nullptr;
    DQ_TRY(make_zero(N, N, (int32_t)off.size(), off.data(), prec, s, &M));
    if (M->nd == 0) {
        *out = M;
        return DIAQ_OK;
    }
    // one staging allocation: terms | starts | list
    const size_t tb = sizeof(PauliTerm) * terms.size(), sb = sizeof(int32_t) * starts.size(),
                 lb = sizeof(int32_t) * list.size();
    uint8_t *d = nullptr;
    cudaError_t e = dev_malloc(&d, tb + sb + lb + 64);
    PauliTerm *dt = (PauliTerm *)d;
    int32_t *ds = (int32_t *)(d + tb), *dl = (int32_t *)(d + tb + sb);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, terms.data(), tb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ds, starts.data(), sb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dl, list.data(), lb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const dim3 g((unsigned)std::min<int64_t>((N + 255) / 256, 2 * num_sms()), (unsigned)std::min<int64_t>(M->nd, 65535));
        if (prec == DIAQ_C128)
            pauli_fill_kernel<double><<<g, 256, 0, s>>>(M->d_meta, M->nd, dt, ds, dl, (double *)M->re, (double *)M->im);
        else
            pauli_fill_kernel<float><<<g, 256, 0, s>>>(M->d_meta, M->nd, dt, ds, dl, (float *)M->re, (float *)M->im);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (d) cudaFree(d);
    if (e != cudaSuccess) {
        destroy(M);
        return cuda_status(e, "pauli build", __FILE__, __LINE__);
    }
    // drop the diagonals whose strings cancelled exactly
    Matrix *P = nullptr;
    const int st = prune_matrix(*M, s, &P);
    destroy(M);
    if (st != DIAQ_OK) return st;
    *out = P;
    return DIAQ_OK;
}

}  // namespace diaq_gb300

using namespace diaq_gb300;

extern "C" {

int diaq_matrix_from_pauli(int n_qubits, int32_t n_strings, const double *coeff_re, const double *coeff_im,
                           const uint64_t *x_mask, const uint64_t *z_mask, int precision, void *stream,
                           diaq_matrix_t *out) {
    if (!out) return set_error(DIAQ_ERR_INVALID, "NULL argument");
    Matrix *M = nullptr;
    DQ_TRY(pauli_build(n_qubits, n_strings, coeff_re, coeff_im, x_mask, z_mask, precision, (cudaStream_t)stream, &M));
    *out = handle(M);
    return DIAQ_OK;
}

}  // extern "C"
