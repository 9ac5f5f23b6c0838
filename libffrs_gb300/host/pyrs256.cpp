// RS256 binding: the reference's PyRS256 surface (libffrs/pyrs256.hpp:58-210)
// backed by the GPU kernels, plus batched entry points over contiguous
// multi-block buffers.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <memory>
#include <optional>
#include <string>

#include "pyffrs_common.h"

namespace py = pybind11;
using namespace pybind11::literals;

py::object make_gf256(uint8_t primitive, uint16_t polynomial);

class PyRS256 {
public:
    ffgpu_rs256 *code = nullptr;
    size_t ecc_len = 0;
    size_t block_len = 0;
    uint8_t primitive;
    uint16_t polynomial;

    // PyRS256 ctor and _get_ecc_len (pyrs256.hpp:63-97, 195-209)
    PyRS256(std::optional<uint8_t> block_len_, std::optional<uint8_t> message_len_, std::optional<uint8_t> ecc_len_,
            uint8_t primitive_, uint16_t polynomial_)
        : primitive(primitive_), polynomial(polynomial_) {
        size_t ecc;
        if (ecc_len_) {
            ecc = *ecc_len_;
        } else if (message_len_ && block_len_) {
            if (*message_len_ >= *block_len_) throw py::value_error("block_len must be greater than message_len");
            ecc = (size_t)*block_len_ - *message_len_;
        } else {
            throw py::value_error("Must specify either (block_len, message_len) or ecc_len");
        }
        if (ecc < 1 || ecc > 254) throw py::value_error("ecc_len must be in [1, 254]");
        ecc_len = ecc;
        set_block_len(block_len_ ? *block_len_ : 255);
        if (ecc_len_ && message_len_) {
            if (block_len_ && (size_t)*message_len_ + *ecc_len_ != *block_len_)
                throw py::value_error("block_len must be equal to message_len + ecc_len");
            else if (!block_len_)
                set_block_len((size_t)*message_len_ + (size_t)*ecc_len_);
        }
        // device tables last: every argument error above is raised first
        ffgpu_check(ffgpu_rs256_create((int)ecc, primitive_, polynomial_, &code));
    }
    ~PyRS256() {
        if (code) ffgpu_rs256_destroy(code);
    }

    void set_block_len(size_t bl) {
        if (bl <= ecc_len) throw py::value_error("block_len must be greater than ecc_len");
        if (bl > 255) throw py::value_error("block_len must be <= 255");
        block_len = bl;
    }
    size_t message_len() const { return block_len - ecc_len; }

    // PyRS256::py_encode (pyrs256.hpp:99-127)
    py::bytearray encode(py::buffer b) {
        BufRO<uint8_t> buf(b);
        if (buf.size == 0) return make_bytearray(0);
        const size_t ml = message_len();
        const size_t full = buf.size / ml, rem = buf.size - full * ml;
        const size_t out_size = (full + (rem ? 1 : 0)) * ecc_len;
        py::bytearray out = make_bytearray(out_size);
        ffgpu_check(ffgpu_rs256_encode_host(code, buf.data, buf.size, ml, (uint8_t *)bytearray_data(out)));
        return out;
    }

    // PyRS256::py_repair (pyrs256.hpp:129-131): one block, in place
    bool repair(py::buffer b, py::buffer e) {
        BufRW<uint8_t> buf(b), ecc(e);
        const size_t ml = message_len();
        if (buf.size < ml) throw py::value_error("buffer shorter than message_len");
        if (ecc.size < ecc_len) throw py::value_error("ecc shorter than ecc_len");
        uint8_t st = 0;
        ffgpu_check(ffgpu_rs256_decode_host(code, buf.data, ecc.data, 1, ml, &st));
        return st != 0;
    }

    // Batched repair over contiguous nblocks x message_len data and
    // nblocks x ecc_len parity; returns one status byte (1/0) per block.
    py::bytearray repair_blocks(py::buffer b, py::buffer e) {
        BufRW<uint8_t> buf(b), ecc(e);
        const size_t ml = message_len();
        if (buf.size % ml) throw py::value_error("buffer size must be a multiple of message_len");
        const size_t nb = buf.size / ml;
        if (ecc.size != nb * ecc_len) throw py::value_error("ecc size must be nblocks * ecc_len");
        py::bytearray st = make_bytearray(nb);
        if (nb) ffgpu_check(ffgpu_rs256_decode_host(code, buf.data, ecc.data, nb, ml, (uint8_t *)bytearray_data(st)));
        return st;
    }

    // PyRS256::py_synds (pyrs256.hpp:133-140)
    py::bytearray synds(py::buffer b) {
        BufRO<uint8_t> buf(b);
        if (buf.size < ecc_len) return make_bytearray(0);
        if (buf.size < block_len) throw py::value_error("buffer shorter than block_len");
        return synds_blocks_impl(buf.data, buf.data + message_len(), 1);
    }

    py::bytearray synds_blocks_impl(const uint8_t *data, const uint8_t *parity, size_t nb);

    py::bytes generator() const {
        std::string g(ecc_len + 1, '\0'), r(ecc_len, '\0');
        ffgpu_check(ffgpu_rs256_generator(code, (uint8_t *)&g[0], (uint8_t *)&r[0]));
        return py::bytes(g);
    }
    py::bytes generator_roots() const {
        std::string g(ecc_len + 1, '\0'), r(ecc_len, '\0');
        ffgpu_check(ffgpu_rs256_generator(code, (uint8_t *)&g[0], (uint8_t *)&r[0]));
        return py::bytes(r);
    }
};

py::bytearray PyRS256::synds_blocks_impl(const uint8_t *data, const uint8_t *parity, size_t nb) {
    py::bytearray out = make_bytearray(nb * ecc_len);
    ffgpu_check(ffgpu_rs256_synds_host(code, data, parity, nb, message_len(), (uint8_t *)bytearray_data(out)));
    return out;
}

void register_rs256(py::module &m) {
    py::class_<PyRS256>(m, "RS256")
        .def(py::init<std::optional<uint8_t>, std::optional<uint8_t>, std::optional<uint8_t>, uint8_t, uint16_t>(),
             R"(Instantiate a Reed-Solomon encoder with the given configuration)", "block_len"_a = py::none(),
             "message_len"_a = py::none(), "ecc_len"_a = py::none(), "primitive"_a = 2, "polynomial"_a = 0x11d)
        .def_property_readonly("ecc_len", [](PyRS256 &s) { return s.ecc_len; })
        .def_property_readonly("ecc_size", [](PyRS256 &s) { return s.ecc_len; })
        .def_property(
            "block_len", [](PyRS256 &s) { return s.block_len; }, &PyRS256::set_block_len)
        .def_property(
            "block_size", [](PyRS256 &s) { return s.block_len; }, &PyRS256::set_block_len)
        .def_property_readonly("message_len", [](PyRS256 &s) { return s.message_len(); })
        .def_property_readonly("message_size", [](PyRS256 &s) { return s.message_len(); })
        .def_property_readonly("gf", [](PyRS256 &s) { return make_gf256(s.primitive, s.polynomial); })
        .def_property_readonly("generator", &PyRS256::generator)
        .def_property_readonly("generator_roots", &PyRS256::generator_roots)
        .def("__sizeof_cpp__", [](PyRS256 &) { return sizeof(PyRS256); })
        .def("encode", &PyRS256::encode, R"(Encode message, return ecc)", "buffer"_a)
        .def("repair", &PyRS256::repair, R"(Repair message + ecc)", "buffer"_a, "ecc"_a)
        .def("repair_blocks", &PyRS256::repair_blocks,
             R"(Repair nblocks contiguous messages and their contiguous ecc; returns one status byte per block)",
             "buffer"_a, "ecc"_a)
        .def("_synds", &PyRS256::synds, R"(Compute syndromes)", "buffer"_a)
        .doc() = R"(Reed-Solomon coding over :math:`GF(2^8)`)";
}
