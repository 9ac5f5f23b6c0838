// The pybind11 module `libffrs`: a drop-in for the reference's extension of
// the same name (libffrs/pyffrs.cpp:101-138).  Classes, constructor
// signatures, properties, defaults, exceptions and return types follow the
// reference binding; the arithmetic runs on the GPU through the C ABI in
// include/ffgpu.h.  There is no CPU fallback: a missing or failing GPU raises.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstring>
#include <optional>
#include <string>
#include <vector>

#include "ffgpu.h"
#include "pyffrs_common.h"

namespace py = pybind11;
using namespace pybind11::literals;

void register_gf(py::module &m);
void register_rs256(py::module &m);
void register_rsi16(py::module &m);
void register_circ16(py::module &m);

// create_buffer (libffrs/pyffrs.cpp:41-98): the reference returns zeroed,
// locked, hugepage-advised anonymous memory as a writable memoryview.  Here
// the memory is page-locked CUDA host memory, so host<->device copies of it
// run at full link speed.
static py::memoryview py_create_buffer(size_t requested_size) {
    void *ptr = nullptr;
    ffgpu_check(ffgpu_host_alloc(requested_size, &ptr));
    py::capsule owner(ptr, "ffgpu_host_buffer", [](void *p) { ffgpu_host_free(p); });
    Py_buffer view;
    if (PyBuffer_FillInfo(&view, owner.ptr(), ptr, (Py_ssize_t)requested_size, 0, PyBUF_CONTIG) < 0)
        throw py::error_already_set();
    return py::reinterpret_steal<py::memoryview>(PyMemoryView_FromBuffer(&view));
}

PYBIND11_MODULE(libffrs, m) {
    m.attr("__version__") = "0.1.0+gb300";
    m.attr("compiler_info") = std::string("gcc") + __VERSION__ + " / " + ffgpu_version();

    m.def("create_buffer", &py_create_buffer, "size"_a,
          R"(Create a zeroed, page-locked host buffer of the given size as a writable memoryview.)");
    // set_logger (libffrs/pyffrs.cpp:123-126): the GPU build emits no per-row
    // log records; the logger is kept so callers can pass and clear it.
    m.attr("_logger") = py::none();
    m.def(
        "set_logger",
        [m](py::object logger) mutable { m.attr("_logger") = logger; },
        "logger"_a, R"(Logger object to be used by the library or ``None`` to disable logging.)");
    m.def("_kernel_launches", []() { return ffgpu_kernel_launches(); });
    m.doc() = R"(FFRS - Fairly Fast & Flexible Reed-Solomon coding, GB300 build)";

    register_gf(m);
    register_rs256(m);
    register_rsi16(m);
    register_circ16(m);
}
