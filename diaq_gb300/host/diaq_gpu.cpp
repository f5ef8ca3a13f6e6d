// diaq_gpu -- the Python module of the GB300 build, a drop-in for the reference's `diaq_gpu`
// pybind11 module (include/pythonWrappers.cpp:31-35, hot-path bindings :146-653).
//
// Host types (diaQMatrix, vector) live here in C++; everything that computes goes through the C
// ABI of libdiaq_gb300.so (include/diaq_gb300.h).  Names, argument names, defaults and return
// types follow the reference; C ABI failures raise RuntimeError with the library's message
// (the reference raises std::runtime_error, i.e. RuntimeError, for the same conditions).
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <array>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "diaq_gb300.h"

namespace py = pybind11;
using cplx = std::complex<double>;

namespace {

void check(int st) {
    if (st != DIAQ_OK) throw std::runtime_error(diaq_last_error());
}

int64_t diag_len(int64_t rows, int64_t cols, int64_t d) {
    int64_t len;
    if (d < 0) len = rows + d;
    else if (d > 0) len = cols - d;
    else len = rows < cols ? rows : cols;
    if (len > rows) len = rows;
    else if (len > cols) len = cols;
    return len < 0 ? 0 : len;
}

// 0, -1, +1, -2, +2, ... (src/diaQMatrix.hpp:24-39)
std::vector<int> symmetric_order(unsigned n) {
    std::vector<int> o;
    for (unsigned i = 0; i < n; ++i) o.push_back(i == 0 ? 0 : (i % 2 == 1 ? -(int)((i + 1) / 2) : (int)(i / 2)));
    return o;
}

// ---- host matrix (the reference's diaQMatrix, packed: no SIMD padding) --------------------------
struct HostMatrix {
    std::array<int64_t, 2> matrix_shape{0, 0};
    std::vector<int> dIndices;
    std::vector<int64_t> diagOffsets;  // packed start of each diagonal
    int64_t totalLength = 0;
    std::vector<double> re, im;

    HostMatrix() = default;
    HostMatrix(int64_t rows, int64_t cols, std::vector<int> d) : matrix_shape{rows, cols}, dIndices(std::move(d)) {
        layout();
    }
    void layout() {
        diagOffsets.assign(dIndices.size(), 0);
        int64_t s = 0;
        for (size_t k = 0; k < dIndices.size(); ++k) {
            const int64_t d = dIndices[k];
            if (d <= -matrix_shape[0] || d >= matrix_shape[1])
                throw std::runtime_error("diagonal index " + std::to_string(d) + " outside the matrix");
            diagOffsets[k] = s;
            s += diag_len(matrix_shape[0], matrix_shape[1], d);
        }
        totalLength = s;
        re.assign(s, 0.0);
        im.assign(s, 0.0);
    }
    int64_t len(size_t k) const { return diag_len(matrix_shape[0], matrix_shape[1], dIndices[k]); }
    int find(int d) const {
        for (size_t k = 0; k < dIndices.size(); ++k)
            if (dIndices[k] == d) return (int)k;
        return -1;
    }
    std::shared_ptr<HostMatrix> copy() const { return std::make_shared<HostMatrix>(*this); }
    void set_at_diag(int d, int64_t pos, double r, double i) {
        const int k = find(d);
        if (k < 0) throw std::runtime_error("set_diag: diagonal index not present in dIndices.");
        if (pos < 0 || pos >= len(k)) throw std::runtime_error("set_diag: position outside the diagonal");
        re[diagOffsets[k] + pos] = r;
        im[diagOffsets[k] + pos] = i;
    }
    double sparsity() const {
        int64_t nnz = 0;
        for (int64_t i = 0; i < totalLength; ++i) nnz += (re[i] != 0.0 || im[i] != 0.0);
        const double all = (double)matrix_shape[0] * (double)matrix_shape[1];
        return all > 0 ? 1.0 - (double)nnz / all : 0.0;
    }
    // drop exact-zero diagonals (src/diaQMatrix.hpp:1543-1604)
    void prune() {
        std::vector<int> keep;
        for (size_t k = 0; k < dIndices.size(); ++k) {
            const int64_t o = diagOffsets[k], n = len(k);
            bool nz = false;
            for (int64_t j = 0; j < n && !nz; ++j) nz = re[o + j] != 0.0 || im[o + j] != 0.0;
            if (nz) keep.push_back((int)k);
        }
        if (keep.size() == dIndices.size()) return;
        HostMatrix P;
        P.matrix_shape = matrix_shape;
        for (int k : keep) P.dIndices.push_back(dIndices[k]);
        P.layout();
        for (size_t j = 0; j < keep.size(); ++j) {
            const int k = keep[j];
            std::copy(re.begin() + diagOffsets[k], re.begin() + diagOffsets[k] + len(k), P.re.begin() + P.diagOffsets[j]);
            std::copy(im.begin() + diagOffsets[k], im.begin() + diagOffsets[k] + len(k), P.im.begin() + P.diagOffsets[j]);
        }
        *this = std::move(P);
    }
    void print_meta() const {
        std::printf("matrix_shape (%lld,%lld)\n#Diagonals = %zu\ndIndices: [", (long long)matrix_shape[0],
                    (long long)matrix_shape[1], dIndices.size());
        for (size_t k = 0; k < dIndices.size(); ++k) std::printf(k ? ", %d" : "%d", dIndices[k]);
        std::printf("]\nTotal stored elements = %lld\nSparsity = %g\n", (long long)totalLength, sparsity());
        std::fflush(stdout);
    }
};
using HostPtr = std::shared_ptr<HostMatrix>;

// ---- state vector ---------------------------------------------------------------------------------
struct HostVector {
    std::vector<double> re, im;
    explicit HostVector(int64_t n = 0) : re(n, 0.0), im(n, 0.0) {}
    int64_t numRows() const { return (int64_t)re.size(); }
};
using VecPtr = std::shared_ptr<HostVector>;

// ---- device matrix --------------------------------------------------------------------------------
struct DeviceMatrix {
    diaq_matrix_t h = nullptr;
    explicit DeviceMatrix(diaq_matrix_t m) : h(m) {}
    DeviceMatrix(const HostPtr &A, int precision) {
        check(diaq_matrix_create(A->matrix_shape[0], A->matrix_shape[1], (int32_t)A->dIndices.size(),
                                 A->dIndices.data(), A->totalLength ? A->re.data() : nullptr,
                                 A->totalLength ? A->im.data() : nullptr, 0, precision, nullptr, &h));
    }
    ~DeviceMatrix() { diaq_matrix_destroy(h); }
    DeviceMatrix(const DeviceMatrix &) = delete;
    DeviceMatrix &operator=(const DeviceMatrix &) = delete;

    void info(int64_t &rows, int64_t &cols, int32_t &nd, int64_t &total, int &prec) const {
        check(diaq_matrix_info(h, &rows, &cols, &nd, &total, &prec));
    }
    std::vector<int> diagonals() const {
        int64_t r, c, t;
        int32_t nd;
        int p;
        info(r, c, nd, t, p);
        std::vector<int> off(nd);
        check(diaq_matrix_offsets(h, off.data()));
        return off;
    }
    HostPtr to_host() const {
        int64_t r, c, t;
        int32_t nd;
        int p;
        info(r, c, nd, t, p);
        auto H = std::make_shared<HostMatrix>(r, c, diagonals());
        if (t > 0) check(diaq_matrix_download(h, H->re.data(), H->im.data(), 0, nullptr));
        return H;
    }
};
using DevPtr = std::shared_ptr<DeviceMatrix>;

DevPtr upload(const HostPtr &A, int prec = DIAQ_C128) { return std::make_shared<DeviceMatrix>(A, prec); }

int parse_precision(const std::string &p) {
    if (p == "c128" || p == "complex128" || p == "fp64") return DIAQ_C128;
    if (p == "c64" || p == "complex64" || p == "fp32") return DIAQ_C64;
    if (p == "c128f2") return DIAQ_C128F2;
    throw std::invalid_argument("precision must be 'c128', 'c64' or 'c128f2'");
}

// ---- conversions (src/conversions.cpp, src/dense_to_diagonals.hpp:20-58) --------------------------
HostPtr from_dense(const cplx *v, int64_t rows, int64_t cols) {
    std::vector<int> diags;
    for (int64_t d = -(rows - 1); d <= cols - 1; ++d) {
        const int64_t r0 = d >= 0 ? 0 : -d, c0 = d >= 0 ? d : 0;
        const int64_t n = std::min(rows - r0, cols - c0);
        for (int64_t j = 0; j < n; ++j) {
            const cplx x = v[(r0 + j) * cols + c0 + j];
            if (x.real() != 0.0 || x.imag() != 0.0) {
                diags.push_back((int)d);
                break;
            }
        }
    }
    auto A = std::make_shared<HostMatrix>(rows, cols, diags);
    for (size_t k = 0; k < diags.size(); ++k) {
        const int64_t d = diags[k];
        const int64_t r0 = d >= 0 ? 0 : -d, c0 = d >= 0 ? d : 0;
        const int64_t n = A->len(k);
        for (int64_t j = 0; j < n; ++j) {
            const cplx x = v[(r0 + j) * cols + c0 + j];
            A->re[A->diagOffsets[k] + j] = x.real();
            A->im[A->diagOffsets[k] + j] = x.imag();
        }
    }
    return A;
}

py::array_t<cplx> to_dense(const HostPtr &A) {
    const int64_t rows = A->matrix_shape[0], cols = A->matrix_shape[1];
    py::array_t<cplx> out({rows, cols});
    cplx *p = out.mutable_data();
    std::fill(p, p + rows * cols, cplx(0.0, 0.0));
    for (size_t k = 0; k < A->dIndices.size(); ++k) {
        const int64_t d = A->dIndices[k];
        const int64_t r0 = d >= 0 ? 0 : -d, c0 = d >= 0 ? d : 0;
        for (int64_t j = 0; j < A->len(k); ++j)
            p[(r0 + j) * cols + c0 + j] = cplx(A->re[A->diagOffsets[k] + j], A->im[A->diagOffsets[k] + j]);
    }
    return out;
}

VecPtr vec_from_numpy(py::array_t<cplx, py::array::c_style | py::array::forcecast> a) {
    auto v = std::make_shared<HostVector>(a.size());
    const cplx *p = a.data();
    for (py::ssize_t i = 0; i < a.size(); ++i) {
        v->re[i] = p[i].real();
        v->im[i] = p[i].imag();
    }
    return v;
}

py::array_t<cplx> vec_to_numpy(const VecPtr &v) {
    py::array_t<cplx> out(v->numRows());
    cplx *p = out.mutable_data();
    for (int64_t i = 0; i < v->numRows(); ++i) p[i] = cplx(v->re[i], v->im[i]);
    return out;
}

// ---- operations --------------------------------------------------------------------------------------
VecPtr spmv_dev(const DevPtr &A, const VecPtr &x) {
    int64_t r, c, t;
    int32_t nd;
    int p;
    A->info(r, c, nd, t, p);
    if (x->numRows() != c) throw std::runtime_error("spmv_cuda: dimension mismatch (x length vs A.cols)");
    auto y = std::make_shared<HostVector>(r);
    check(diaq_spmv_host(A->h, x->re.data(), x->im.data(), y->re.data(), y->im.data()));
    return y;
}

HostPtr product_host(const HostPtr &A, const HostPtr &B) {
    if (A->matrix_shape[1] != B->matrix_shape[0]) throw std::runtime_error("diaQMatrix product_cuda: dimension mismatch.");
    auto dA = upload(A), dB = upload(B);
    diaq_matrix_t C = nullptr;
    check(diaq_spgemm(dA->h, dB->h, 1, nullptr, &C));
    return DeviceMatrix(C).to_host();
}

}  // namespace

PYBIND11_MODULE(diaq_gpu, m) {
    m.doc() = "DiaQ diagonal-sparse hot path on GB300 (sm_103a): drop-in for the reference's diaq_gpu module";
    m.def("version", []() { return std::string(diaq_version()); });

    py::class_<HostMatrix, HostPtr>(m, "diaQMatrix")
        .def(py::init([](unsigned s) { return std::make_shared<HostMatrix>(s, s, std::vector<int>{}); }))
        .def(py::init([](unsigned s, unsigned nd) { return std::make_shared<HostMatrix>(s, s, symmetric_order(nd)); }))
        .def(py::init([](std::array<unsigned, 2> sh) { return std::make_shared<HostMatrix>(sh[0], sh[1], std::vector<int>{}); }))
        .def(py::init([](std::array<unsigned, 2> sh, const std::vector<int> &d) { return std::make_shared<HostMatrix>(sh[0], sh[1], d); }))
        .def(py::init([](std::array<unsigned, 2> sh, const std::vector<int> &d, std::vector<unsigned>) {
            return std::make_shared<HostMatrix>(sh[0], sh[1], d);
        }))
        .def_property_readonly("matrix_shape", [](const HostMatrix &a) { return a.matrix_shape; })
        .def_property_readonly("shape", [](const HostMatrix &a) { return std::vector<int64_t>{a.matrix_shape[0], a.matrix_shape[1]}; })
        .def_readonly("dIndices", &HostMatrix::dIndices)
        .def_readonly("diagOffsets", &HostMatrix::diagOffsets)
        .def_readonly("totalLength", &HostMatrix::totalLength)
        .def("num_diags", [](const HostMatrix &a) { return a.dIndices.size(); })
        .def("get_diagonals", [](const HostMatrix &a) { return a.dIndices; })
        .def("set_at_diag", &HostMatrix::set_at_diag)
        .def("copy", &HostMatrix::copy)
        .def("pruneMatrix", &HostMatrix::prune)
        .def("sparsity", &HostMatrix::sparsity)
        .def("print_meta", &HostMatrix::print_meta)
        .def("getItem", [](const HostMatrix &a, std::array<unsigned, 2> pos) {
            const int d = (int)pos[1] - (int)pos[0];
            const int k = a.find(d);
            if (k < 0) return cplx(0.0, 0.0);
            const int64_t j = d >= 0 ? pos[0] : pos[1];
            return cplx(a.re[a.diagOffsets[k] + j], a.im[a.diagOffsets[k] + j]);
        })
        // packed values as numpy arrays (copies): (offsets, re, im)
        .def("diagonal_data", [](const HostMatrix &a) {
            py::array_t<int32_t> off(a.dIndices.size());
            std::copy(a.dIndices.begin(), a.dIndices.end(), off.mutable_data());
            py::array_t<double> re(a.totalLength), im(a.totalLength);
            std::copy(a.re.begin(), a.re.end(), re.mutable_data());
            std::copy(a.im.begin(), a.im.end(), im.mutable_data());
            return py::make_tuple(off, re, im);
        });

    py::class_<HostVector, VecPtr>(m, "vector")
        .def(py::init<int64_t>())
        .def_property_readonly("numRows", &HostVector::numRows)
        .def("copy", [](const HostVector &v) { return std::make_shared<HostVector>(v); });

    py::class_<DeviceMatrix, DevPtr>(m, "DeviceMatrix",
                                     "A diaQMatrix in GPU memory (uploaded once).  spMV(DeviceMatrix, vector) copies only "
                                     "the vectors; product(DeviceMatrix, DeviceMatrix) stays on the GPU; to_host() downloads.")
        .def(py::init([](const HostPtr &A, const std::string &precision) { return upload(A, parse_precision(precision)); }),
             py::arg("A"), py::arg("precision") = "c128")
        .def("to_host", &DeviceMatrix::to_host)
        .def("copy", [](const DeviceMatrix &d) {
            diaq_matrix_t c = nullptr;
            check(diaq_matrix_copy(d.h, nullptr, &c));
            return std::make_shared<DeviceMatrix>(c);
        })
        .def("to_precision", [](const DeviceMatrix &d, const std::string &p) {
            diaq_matrix_t c = nullptr;
            check(diaq_matrix_convert(d.h, parse_precision(p), nullptr, &c));
            return std::make_shared<DeviceMatrix>(c);
        })
        .def_property_readonly("shape", [](const DeviceMatrix &d) {
            int64_t r, c, t;
            int32_t nd;
            int p;
            d.info(r, c, nd, t, p);
            return std::array<int64_t, 2>{r, c};
        })
        .def_property_readonly("num_diags", [](const DeviceMatrix &d) {
            int64_t r, c, t;
            int32_t nd;
            int p;
            d.info(r, c, nd, t, p);
            return nd;
        })
        .def_property_readonly("precision", [](const DeviceMatrix &d) {
            int64_t r, c, t;
            int32_t nd;
            int p;
            d.info(r, c, nd, t, p);
            return std::string(p == DIAQ_C128 ? "c128" : p == DIAQ_C64 ? "c64" : "c128f2");
        })
        .def_property_readonly("diagonals", &DeviceMatrix::diagonals)
        .def_property_readonly("handle", [](const DeviceMatrix &d) { return reinterpret_cast<uintptr_t>(d.h); });

    // ---- conversions ----
    m.def("from_numpy", [](py::array_t<cplx, py::array::c_style | py::array::forcecast> a) {
        if (a.ndim() != 2) throw std::runtime_error("from_numpy: expected a 2-D array");
        return from_dense(a.data(), a.shape(0), a.shape(1));
    });
    m.def("from_numpy", [](py::array_t<cplx, py::array::c_style | py::array::forcecast> a, std::vector<unsigned> shape) {
        if (a.ndim() != 1) throw std::runtime_error("Input arrays must be 1-dimensional.");
        if (shape.size() != 2 || (int64_t)shape[0] * shape[1] != a.size())
            throw std::runtime_error("from_numpy: shape does not match the number of values");
        return from_dense(a.data(), shape[0], shape[1]);
    });
    m.def("to_numpy", &to_dense);
    m.def("to_numpy", [](const DevPtr &A) {  // dense array written on the GPU, then copied once
        int64_t r, c, t;
        int32_t nd;
        int p;
        A->info(r, c, nd, t, p);
        py::array_t<cplx> out({r, c});
        check(diaq_matrix_to_dense(A->h, reinterpret_cast<double *>(out.mutable_data()), 0, nullptr));
        return out;
    });
    m.def(
        "from_numpy_device",
        [](py::array_t<cplx, py::array::c_style | py::array::forcecast> a, const std::string &precision) {
            if (a.ndim() != 2) throw std::runtime_error("from_numpy: expected a 2-D array");
            diaq_matrix_t h = nullptr;
            check(diaq_matrix_from_dense(a.shape(0), a.shape(1), reinterpret_cast<const double *>(a.data()), 0,
                                         parse_precision(precision), nullptr, &h));
            return std::make_shared<DeviceMatrix>(h);
        },
        py::arg("arr"), py::arg("precision") = "c128",
        "from_numpy straight to a DeviceMatrix: the nonzero diagonals are found and gathered on the GPU.");
    m.def("from_numpy_vector", &vec_from_numpy);
    m.def("to_numpy_vector", &vec_to_numpy);
    m.def(
        "from_diagonals",
        [](int64_t rows, int64_t cols, std::vector<int> offsets, py::array_t<double, py::array::c_style | py::array::forcecast> re,
           py::array_t<double, py::array::c_style | py::array::forcecast> im) {
            auto A = std::make_shared<HostMatrix>(rows, cols, offsets);
            if (re.size() != A->totalLength || im.size() != A->totalLength)
                throw std::runtime_error("from_diagonals: value arrays must hold " + std::to_string(A->totalLength) + " values");
            std::copy(re.data(), re.data() + re.size(), A->re.begin());
            std::copy(im.data(), im.data() + im.size(), A->im.begin());
            return A;
        },
        py::arg("rows"), py::arg("cols"), py::arg("offsets"), py::arg("re"), py::arg("im"),
        "A diaQMatrix from its offsets (slot order) and packed float64 values.");

    // ---- device matrices ----
    m.def("to_device", [](const HostPtr &A, const std::string &precision) { return upload(A, parse_precision(precision)); },
          py::arg("A"), py::arg("precision") = "c128", "Upload a diaQMatrix to the GPU (a DeviceMatrix).");

    // ---- SpMV ----
    m.def("spMV", [](const HostPtr &A, const VecPtr &x) { return spmv_dev(upload(A), x); });
    m.def("spMV", [](const HostPtr &A, const VecPtr &x, const VecPtr &y) {
        if (y->numRows() != A->matrix_shape[0]) throw std::runtime_error("spmv_cuda: dimension mismatch (y length vs A.rows)");
        auto r = spmv_dev(upload(A), x);
        y->re = r->re;
        y->im = r->im;
        return y;
    });
    m.def("spMV", [](const DevPtr &A, const VecPtr &x) { return spmv_dev(A, x); });
    m.def("spMV_ntimes", [](const HostPtr &A, const VecPtr &x, int n) {
        if (x->numRows() != A->matrix_shape[1]) throw std::runtime_error("spmv_ntimes_cuda: dimension mismatch (x length vs A.cols)");
        auto y = std::make_shared<HostVector>(A->matrix_shape[0]);
        auto dA = upload(A);
        check(diaq_spmv_ntimes_host(dA->h, x->re.data(), x->im.data(), n, y->re.data(), y->im.data()));
        return y;
    });
    m.def("spMV_ntimes", [](const HostPtr &A, const VecPtr &x, const VecPtr &y, int n) {
        if (x->numRows() != A->matrix_shape[1]) throw std::runtime_error("spmv_ntimes_cuda: dimension mismatch (x length vs A.cols)");
        if (y->numRows() != A->matrix_shape[0]) throw std::runtime_error("spmv_ntimes_cuda: dimension mismatch (y length vs A.rows)");
        auto dA = upload(A);
        check(diaq_spmv_ntimes_host(dA->h, x->re.data(), x->im.data(), n, y->re.data(), y->im.data()));
        return y;
    });
    m.def(
        "spmv_device",
        [](const DevPtr &A, uintptr_t x_real, uintptr_t x_imag, uintptr_t y_real, uintptr_t y_imag, uintptr_t stream) {
            int64_t r, c, t;
            int32_t nd;
            int p;
            A->info(r, c, nd, t, p);
            if (p != DIAQ_C64)
                check(diaq_spmv_z(A->h, reinterpret_cast<const double *>(x_real), reinterpret_cast<const double *>(x_imag),
                                  reinterpret_cast<double *>(y_real), reinterpret_cast<double *>(y_imag),
                                  reinterpret_cast<void *>(stream)));
            else
                check(diaq_spmv_c(A->h, reinterpret_cast<const float *>(x_real), reinterpret_cast<const float *>(x_imag),
                                  reinterpret_cast<float *>(y_real), reinterpret_cast<float *>(y_imag),
                                  reinterpret_cast<void *>(stream)));
        },
        py::arg("A"), py::arg("x_real"), py::arg("x_imag"), py::arg("y_real"), py::arg("y_imag"), py::arg("stream") = 0,
        "y = A x with x, y as GPU arrays (float64 for a c128 or c128f2 matrix, float32 for c64; real and imaginary parts, e.g. "
        "torch data pointers); y is overwritten; asynchronous on `stream`.");
    m.def(
        "spmm_device",
        [](const DevPtr &A, int nrhs, uintptr_t x_real, uintptr_t x_imag, int64_t ldx, uintptr_t y_real, uintptr_t y_imag,
           int64_t ldy, uintptr_t stream) {
            check(diaq_spmm(A->h, nrhs, reinterpret_cast<const void *>(x_real), reinterpret_cast<const void *>(x_imag), ldx,
                            reinterpret_cast<void *>(y_real), reinterpret_cast<void *>(y_imag), ldy,
                            reinterpret_cast<void *>(stream)));
        },
        py::arg("A"), py::arg("nrhs"), py::arg("x_real"), py::arg("x_imag"), py::arg("ldx"), py::arg("y_real"),
        py::arg("y_imag"), py::arg("ldy"), py::arg("stream") = 0,
        "Y = A X for nrhs right-hand sides stored one after another (leading dimensions ldx, ldy); asynchronous.");
    // include/pythonWrappers.cpp:622-633
    m.def(
        "spmm_dia_device",
        [](uintptr_t offsets, uintptr_t vals, int n_diags, int64_t n_rows, int64_t n_cols, uintptr_t B, int64_t n_right,
           uintptr_t C, bool is_complex, uintptr_t stream) {
            check(diaq_spmm_dia_device(reinterpret_cast<const int64_t *>(offsets), reinterpret_cast<const void *>(vals),
                                       n_diags, n_rows, n_cols, reinterpret_cast<const void *>(B), n_right,
                                       reinterpret_cast<void *>(C), is_complex ? 1 : 0, reinterpret_cast<void *>(stream)));
        },
        py::arg("offsets"), py::arg("vals"), py::arg("n_diags"), py::arg("n_rows"), py::arg("n_cols"), py::arg("B"),
        py::arg("n_right"), py::arg("C"), py::arg("is_complex"), py::arg("stream") = 0,
        "C = A * B, A in row-aligned DIA format (offsets int64[n_diags], vals[n_diags * n_rows]); B (n_cols x "
        "n_right) and C (n_rows x n_right) row-major; double or complex double; all pointers on the GPU.");

    // ---- SpGEMM ----
    m.def("product", &product_host, "C = A B for host matrices; exact-zero result diagonals are pruned.");
    m.def("product", [](const DevPtr &A, const DevPtr &B) {
        diaq_matrix_t C = nullptr;
        check(diaq_spgemm(A->h, B->h, 0, nullptr, &C));
        return std::make_shared<DeviceMatrix>(C);
    });
    m.def("spgemm_symbolic", [](const DevPtr &A, const DevPtr &B) {
        const size_t cap = std::max<size_t>(1, (size_t)A->diagonals().size() * B->diagonals().size());
        std::vector<int32_t> out(cap);
        int32_t n = 0;
        check(diaq_spgemm_symbolic(A->h, B->h, out.data(), &n, nullptr));
        out.resize(n);
        return out;
    }, "Offsets of A B (ascending, distinct), computed on the device.");

    // ---- norms, pow, exponential ----
    m.def("norm1_est", [](const DevPtr &A) {
        double v = 0.0;
        check(diaq_norm1_est(A->h, &v, nullptr));
        return v;
    });
    m.def("frobenius", [](const DevPtr &A) {
        double v = 0.0;
        check(diaq_frobenius(A->h, &v, nullptr));
        return v;
    });
    m.def(
        "pow",
        [](const HostPtr &A, int power, bool prune) {
            if (power < 0) throw std::runtime_error("pow_cuda: negative exponent not supported");
            auto dA = upload(A);
            diaq_matrix_t P = nullptr;
            check(diaq_pow(dA->h, power, prune ? 1 : 0, nullptr, &P));
            return DeviceMatrix(P).to_host();
        },
        py::arg("A"), py::arg("power"), py::arg("prune") = true);
    m.def(
        "expm",
        [](const HostPtr &A, int max_iterations, double scale_cutoff, double tolerance, bool prune) {
            auto dA = upload(A);
            diaq_matrix_t U = nullptr;
            check(diaq_expm(dA->h, max_iterations, scale_cutoff, tolerance, prune ? 1 : 0, nullptr, &U));
            return DeviceMatrix(U).to_host();
        },
        py::arg("A"), py::arg("max_iterations") = 100, py::arg("scale_cutoff") = 1.0, py::arg("tolerance") = 1e-12,
        py::arg("prune") = true);
    m.def(
        "expm_negative",
        [](const HostPtr &A, double t, int max_iterations, double scale_cutoff, double tolerance, bool prune) {
            auto dA = upload(A);
            diaq_matrix_t U = nullptr;
            check(diaq_expm_negative(dA->h, t, max_iterations, scale_cutoff, tolerance, prune ? 1 : 0, nullptr, &U,
                                     nullptr, nullptr));
            return DeviceMatrix(U).to_host();
        },
        py::arg("A"), py::arg("t"), py::arg("max_iterations") = 100, py::arg("scale_cutoff") = 1.0,
        py::arg("tolerance") = 1e-12, py::arg("prune") = true);
    m.def(
        "expm_negative_device",
        [](const DevPtr &A, double t, int max_iterations, double scale_cutoff, double tolerance, bool prune) {
            diaq_matrix_t U = nullptr;
            int s = 0, terms = 0;
            check(diaq_expm_negative(A->h, t, max_iterations, scale_cutoff, tolerance, prune ? 1 : 0, nullptr, &U, &s,
                                     &terms));
            return py::make_tuple(std::make_shared<DeviceMatrix>(U), s, terms);
        },
        py::arg("A"), py::arg("t"), py::arg("max_iterations") = 100, py::arg("scale_cutoff") = 1.0,
        py::arg("tolerance") = 1e-12, py::arg("prune") = true,
        "exp(-i t A) of a DeviceMatrix, kept on the device: (U, s, taylor_terms).");

    // ---- time evolution ----
    m.def(
        "hamiltonian_simulation_cuda",
        [](const HostPtr &H, const VecPtr &psi0, double dt, unsigned long r, int max_iterations, double, double) {
            if (H->matrix_shape[0] != H->matrix_shape[1])
                throw std::runtime_error("hamiltonian_simulation_cuda: H must be square");
            if (psi0->numRows() != H->matrix_shape[1])
                throw std::runtime_error("hamiltonian_simulation_cuda: psi0 dimension mismatch");
            auto out = std::make_shared<HostVector>(psi0->numRows());
            if (psi0->numRows() == 0) return out;
            auto dH = upload(H);
            check(diaq_ham_sim_host(dH->h, psi0->re.data(), psi0->im.data(), dt, (int64_t)r, max_iterations,
                                    out->re.data(), out->im.data()));
            return out;
        },
        py::arg("H"), py::arg("psi0"), py::arg("dt"), py::arg("r"), py::arg("max_iterations") = 100,
        py::arg("scale_cutoff") = 1.0, py::arg("tolerance") = 1e-12,
        "psi after r Taylor steps of exp(-i H dt/r); `dt` is the TOTAL time (the reference's convention, "
        "src/spHamSim_gpu_all_fused.cu:347); every step applies exactly max_iterations terms.");

    m.def("install_info", []() {
        py::dict info;
        info["CUDA_ENABLED"] = true;
        info["GPU_ARCH"] = "sm_103a";
        info["valType"] = "double";
        info["precisions"] = std::vector<std::string>{"c128", "c64", "c128f2"};
        info["version"] = std::string(diaq_version());
        return info;
    });
}
