// The reference's compiled `marslib` module (marslib.cc:152-179), rebuilt over
// the GB300 C ABI (include/mars_gpu.h): the same class, methods, argument
// names and conversions, the same RuntimeError messages. mars.fit from the
// reference (its mars.py, unchanged) runs on the GPU when this module is the
// `marslib` it imports; so does mars_gb300.mars.fit.
//
// Behaviour kept from the reference binding:
//   * MarsAlgo(X, y, w, max_terms): no implicit conversion of X, y, w; X is
//     column-major float32 and borrowed (kept alive with the MarsAlgo,
//     py::keep_alive<1, 2>), y and w copied (marslib.cc:12-37, 160-167).
//   * eval(mask, min_span, endspan, linear_only, threads, cuda=False) ->
//     (dsse, linear, hinge, cut), mask row-major bool with nbasis columns;
//     the interpreter lock is released while the GPU evaluates
//     (marslib.cc:41-148). threads and cuda are accepted: every candidate is
//     evaluated on the GPU.
//   * append(type, xcol, bcol, h) -> mse (or -1 when degenerate), nbasis(),
//     yvar(), __version__.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

#include "mars_gpu.h"

namespace py = pybind11;

namespace {

void check(int rc)
{
    if (rc != MARS_GPU_OK) {
        throw std::runtime_error(mars_gpu_last_error());
    }
}

void verify(bool ok, const char *msg)
{
    if (!ok) {
        throw std::runtime_error(msg);
    }
}

// One fit's device state (mars_gpu_algo), owned by the Python object.
struct GpuAlgo {
    mars_gpu_algo *h = nullptr;
    GpuAlgo() = default;
    GpuAlgo(const GpuAlgo &) = delete;
    GpuAlgo &operator=(const GpuAlgo &) = delete;
    ~GpuAlgo()
    {
        if (h) {
            mars_gpu_destroy(h);
        }
    }
    int nbasis() const
    {
        int v = 0;
        check(mars_gpu_nbasis(h, &v));
        return v;
    }
    double yvar() const
    {
        double v = 0;
        check(mars_gpu_yvar(h, &v));
        return v;
    }
};

GpuAlgo *new_algo(py::array_t<float> X_array, py::array_t<float> y_array,
                  py::array_t<float> w_array, int max_terms)
{
    py::buffer_info X = X_array.request();
    py::buffer_info y = y_array.request();
    py::buffer_info w = w_array.request();
    verify(X.ndim == 2, "expected 2D array for X");
    verify(y.ndim == 1, "expected 1D array for y");
    verify(w.ndim == 1, "expected 1D array for w");
    verify(X.strides[0] == sizeof(float), "X must be column-major");
    verify(y.strides[0] == sizeof(float), "y must be column-major");
    verify(w.strides[0] == sizeof(float), "w must be column-major");
    verify(X.shape[0] == y.shape[0], "invalid dimension for y");
    verify(X.shape[0] == w.shape[0], "invalid dimension for w");
    const size_t n = (size_t)X.shape[0], p = (size_t)X.shape[1];
    const size_t ldx = p > 1 ? (size_t)(X.strides[1] / (ssize_t)sizeof(float)) : n;
    auto *a = new GpuAlgo;
    const int rc = mars_gpu_create(static_cast<const float *>(X.ptr),
                                   static_cast<const float *>(y.ptr),
                                   static_cast<const float *>(w.ptr), n, p, ldx,
                                   (size_t)std::max(max_terms, 0), &a->h);
    if (rc != MARS_GPU_OK) {
        delete a;
        check(rc);
    }
    // MARS_GPU_PRECISION=mixed selects the mixed-precision fast pass
    const char *mode = std::getenv("MARS_GPU_PRECISION");
    if (mode && std::strcmp(mode, "mixed") == 0) {
        check(mars_gpu_set_precision(a->h, MARS_GPU_PREC_MIXED));
    }
    return a;
}

py::tuple eval(GpuAlgo &algo, py::array_t<bool> mask_array, int min_span, int endspan,
               bool linear, int threads, bool cuda)
{
    (void)threads;
    (void)cuda;
    py::buffer_info mask = mask_array.request();
    verify(mask.ndim == 2, "expected 2D array for mask");
    verify(mask.strides[1] == sizeof(bool), "mask must be row-major");
    verify(mask.shape[1] == algo.nbasis(), "invalid dimension for mask");
    verify(min_span >= 1, "min_span must be >= 1");
    const ssize_t rows = mask.shape[0], cols = mask.shape[1];
    py::array_t<double> lin({rows, cols}), hin({rows, cols}), cut({rows, cols});
    double dsse = 0.0;
    int rc;
    {
        py::gil_scoped_release release;
        rc = mars_gpu_eval(algo.h, static_cast<const bool *>(mask.ptr), (int)rows,
                           rows > 0 ? (int)(mask.strides[0] / (ssize_t)sizeof(bool)) : (int)cols,
                           min_span, endspan, linear ? 1 : 0, &dsse, lin.mutable_data(),
                           hin.mutable_data(), cut.mutable_data());
    }
    check(rc);
    return py::make_tuple(dsse, lin, hin, cut);
}

double append(GpuAlgo &algo, char type, int xcol, int bcol, float h)
{
    double mse = 0.0;
    check(mars_gpu_append(algo.h, type, xcol, bcol, h, &mse));
    return mse;
}

}  // namespace

PYBIND11_MODULE(marslib, m)
{
    py::options options;
    options.disable_function_signatures();
    m.doc() = "Multivariate Adaptive Regression Splines (GB300 forward pass)";
    m.attr("__version__") = "0.12";
    py::class_<GpuAlgo>(m, "MarsAlgo")
        .def(py::init(&new_algo), py::arg("X").noconvert(), py::arg("y").noconvert(),
             py::arg("w").noconvert(), py::arg("max_terms"), py::keep_alive<1, 2>())
        .def("eval", &eval, py::arg("mask").noconvert(), py::arg("min_span"),
             py::arg("endspan"), py::arg("linear_only"), py::arg("threads"),
             py::arg("cuda") = false)
        .def("nbasis", &GpuAlgo::nbasis)
        .def("yvar", &GpuAlgo::yvar)
        .def("append", &append);
}
