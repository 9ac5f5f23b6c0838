// Helpers shared by the binding translation units: status -> Python
// exception mapping and buffer adaptors mirroring libffrs/util.hpp:30-55.
#pragma once

#include <pybind11/pybind11.h>

#include <stdexcept>
#include <string>

#include "ffgpu.h"

namespace py = pybind11;

inline void ffgpu_check(int rc) {
    if (rc == FFGPU_OK) return;
    std::string msg = ffgpu_last_error();
    if (rc == FFGPU_EINVAL) throw py::value_error(msg);
    if (rc == FFGPU_ENOMEM) throw std::bad_alloc();
    throw std::runtime_error(msg);
}

// The reference asserts with RuntimeError "<file>:<line>: Assertion failed"
// (libffrs/util.hpp:98-102); the GPU build raises RuntimeError the same way.
inline void py_assert_like(bool cond, const std::string &what) {
    if (!cond) throw std::runtime_error("Assertion failed: " + what);
}

// buffer_ro / buffer_rw (libffrs/util.hpp:30-55): a buffer-protocol object
// viewed as an array of T; ValueError when its byte size is not a multiple of
// sizeof(T).
template <typename T, bool Writable>
struct Buf {
    py::buffer obj;
    py::buffer_info info;
    size_t size = 0;
    T *data = nullptr;
    explicit Buf(const py::buffer &o) : obj(o), info(obj.request(Writable)) {
        if (info.size * info.itemsize % (py::ssize_t)sizeof(T) != 0)
            throw py::value_error("Invalid buffer size: " + std::to_string(info.size * info.itemsize));
        size = (size_t)(info.size * info.itemsize) / sizeof(T);
        data = reinterpret_cast<T *>(info.ptr);
    }
};
template <typename T>
using BufRO = Buf<const T, false>;
template <typename T>
using BufRW = Buf<T, true>;

// A result bytearray of n bytes, left uninitialised: every caller fills all
// n bytes before returning it (parity, statuses, syndromes, copies).  Zeroing
// it first would fault in and clear every page on the calling thread before
// the GPU work starts (about 1.9 ms for the 33 MB parity of 262,144 RSi16
// blocks); the host pipelines map the pages in parallel while the GPU runs.
inline py::bytearray make_bytearray(size_t n) {
    PyObject *o = PyByteArray_FromStringAndSize(nullptr, (Py_ssize_t)n);
    if (!o) throw py::error_already_set();
    return py::reinterpret_steal<py::bytearray>(o);
}
inline char *bytearray_data(py::bytearray &b) { return PyByteArray_AsString(b.ptr()); }
