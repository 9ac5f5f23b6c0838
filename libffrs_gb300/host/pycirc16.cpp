// CIRC16 binding (placeholder until the CIRC16 kernels land).
#include <pybind11/pybind11.h>
namespace py = pybind11;
void register_circ16(py::module &) {}
