// RSi16 binding (placeholder until the RSi16 kernels land).
#include <pybind11/pybind11.h>
namespace py = pybind11;
void register_rsi16(py::module &) {}
