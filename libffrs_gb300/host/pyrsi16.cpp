// RSi16 binding: the reference's PyRSi16 surface (libffrs/pyrsi16.hpp:34-320)
// on the GPU kernels, with W = 1 semantics for every repair (the SIMD width
// flags are accepted and reported but select no code path).
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <optional>
#include <string>
#include <vector>

#include "pyffrs_common.h"

namespace py = pybind11;
using namespace pybind11::literals;

enum class RepairStatus : uint32_t { NoErrors, NoErrorsZero, RepairOk, RepairFail, ErrorLocationFail };

py::object make_gfi16(uint32_t primitive);

static uint32_t rbo_bits(uint32_t i, size_t ntt_len) {
    uint16_t b = (uint16_t)i;
    b = (uint16_t)(((b >> 1) & 0x5555) | ((b & 0x5555) << 1));
    b = (uint16_t)(((b >> 2) & 0x3333) | ((b & 0x3333) << 2));
    b = (uint16_t)(((b >> 4) & 0x0f0f) | ((b & 0x0f0f) << 4));
    b = (uint16_t)((b >> 8) | (b << 8));
    return (uint32_t)(b >> (16 - __builtin_ctzl(ntt_len)));
}

// The NTT helper object the reference exposes as RSi16.ntt (libffrs/pyntt.hpp);
// only its geometry and rbo() are provided.
struct PyNTT {
    size_t ntt_len, block_len, ecc_len;
    uint32_t rbo(uint32_t i) const { return rbo_bits(i, ntt_len); }
};

class PyRSi16 {
public:
    ffgpu_rsi16 *code = nullptr;
    size_t block_len, message_len, ecc_len, interleave;
    uint32_t primitive;
    uint32_t root = 0;
    size_t ntt_len = 0;
    bool simd_x4, simd_x8, simd_x16;

    PyRSi16(size_t block_len_, uint16_t ecc_len_, size_t interleave_, uint32_t primitive_,
            std::optional<bool> x4, std::optional<bool> x8, std::optional<bool> x16)
        : block_len(block_len_), message_len(block_len_ - ecc_len_), ecc_len(ecc_len_), interleave(interleave_),
          primitive(primitive_), simd_x4(x4.value_or(false)), simd_x8(x8.value_or(false)),
          simd_x16(x16.value_or(false)) {
        if (interleave == 0) throw std::runtime_error("Assertion failed: interleave > 0");
        ffgpu_check(ffgpu_rsi16_create(block_len_, ecc_len_, primitive_, &code));
        ffgpu_check(ffgpu_rsi16_info(code, &root, &ntt_len));
    }
    ~PyRSi16() {
        if (code) ffgpu_rsi16_destroy(code);
    }
    size_t ilen(size_t n) const { return n * interleave; }

    // PyRSi16::py_encode (pyrsi16.hpp:568-586)
    py::bytearray encode(py::buffer b) {
        BufRO<uint16_t> buf(b);
        if (buf.size == 0) return make_bytearray(0);
        py_assert_like(buf.size % ilen(message_len) == 0, "buf.size % interleaved_message_len == 0: " +
                                                             std::to_string(buf.size));
        const size_t nb = buf.size / ilen(message_len);
        py::bytearray out = make_bytearray(nb * ilen(ecc_len) * 2);
        ffgpu_check(ffgpu_rsi16_encode_host(code, buf.data, nb, interleave, (uint16_t *)bytearray_data(out)));
        return out;
    }

    // PyRSi16::py_repair (pyrsi16.hpp:588-631)
    RepairStatus repair(py::buffer m, py::buffer e, std::optional<std::vector<size_t>> error_pos) {
        if (error_pos && error_pos->empty()) return RepairStatus::NoErrors;
        BufRW<uint16_t> msg(m), ecc(e);
        py_assert_like(msg.size == ilen(message_len), "message.size == message_len: " + std::to_string(msg.size));
        py_assert_like(ecc.size == ilen(ecc_len), "ecc.size == ecc_len: " + std::to_string(ecc.size));
        std::vector<uint32_t> pos;
        if (error_pos) {
            py_assert_like(error_pos->size() <= ecc_len, "error_pos->size() <= ecc_len");
            for (size_t p : *error_pos) {
                if (p >= block_len) throw py::value_error("error position out of range: " + std::to_string(p));
                pos.push_back((uint32_t)p);
            }
        }
        uint8_t st = 0;
        ffgpu_check(ffgpu_rsi16_repair_host(code, msg.data, ecc.data, 1, interleave, pos.data(),
                                            error_pos ? (long)pos.size() : -1L, &st));
        if (st == FFGPU_STATUS_ASSERT) throw std::runtime_error("Assertion failed: g_len > 0 (NTT-domain Sugiyama)");
        return (RepairStatus)st;
    }

    // Batched unknown-location repair of nblocks contiguous blocks
    // (interleave == 1): returns one RepairStatus byte per block, 255 where
    // the reference raises RuntimeError (that block is left untouched).
    py::bytearray repair_blocks(py::buffer m, py::buffer e) {
        BufRW<uint16_t> msg(m), ecc(e);
        if (interleave != 1) throw py::value_error("repair_blocks requires interleave == 1");
        if (msg.size % message_len) throw py::value_error("message size must be a multiple of message_len");
        const size_t nb = msg.size / message_len;
        if (ecc.size != nb * ecc_len) throw py::value_error("ecc size must be nblocks * ecc_len");
        py::bytearray st = make_bytearray(nb);
        if (nb)
            ffgpu_check(ffgpu_rsi16_repair_host(code, msg.data, ecc.data, nb, 1, nullptr, -1L,
                                                (uint8_t *)bytearray_data(st)));
        return st;
    }

    // PyRSi16::py_synd (pyrsi16.hpp:633-651)
    std::vector<uint32_t> synd(py::buffer m, py::buffer e);
    py::tuple sugiyama(std::vector<uint32_t> s, size_t W);
    std::vector<size_t> roots(std::vector<uint32_t> poly);

    size_t message_offset(size_t row, size_t col) const {
        py_assert_like(row < message_len, "row < message_len");
        py_assert_like(col < interleave, "col < interleave");
        return row * interleave + col;
    }
    size_t ecc_offset(size_t row, size_t col) const {
        py_assert_like(row < ecc_len, "row < ecc_len");
        py_assert_like(col < interleave, "col < interleave");
        return row * interleave + col;
    }
};

std::vector<uint32_t> PyRSi16::synd(py::buffer m, py::buffer e) {
    BufRO<uint16_t> msg(m), ecc(e);
    py_assert_like(msg.size % message_len == 0, std::to_string(msg.size));
    py_assert_like(ecc.size % ecc_len == 0, std::to_string(ecc.size));
    const size_t count = msg.size / message_len;
    py_assert_like(ecc.size / ecc_len == count, "ecc.size / ecc_len == count");
    std::vector<uint32_t> out(count * ecc_len);
    if (count) ffgpu_check(ffgpu_rsi16_synd_host(code, msg.data, ecc.data, count, out.data()));
    return out;
}

py::tuple PyRSi16::sugiyama(std::vector<uint32_t> s, size_t W) {
    if (s.size() < W * ecc_len) s.resize(W * ecc_len, 0);
    std::vector<uint32_t> loc(W * ecc_len), ev(W * ecc_len);
    std::vector<uint8_t> st(W);
    ffgpu_check(ffgpu_rsi16_sugiyama_host(code, s.data(), W, loc.data(), ev.data(), st.data()));
    for (auto x : st)
        if (x == FFGPU_STATUS_ASSERT) throw std::runtime_error("Assertion failed: g_len > 0 (NTT-domain Sugiyama)");
    return py::make_tuple(loc, ev);
}

std::vector<size_t> PyRSi16::roots(std::vector<uint32_t> poly) {
    py_assert_like(poly.size() == ecc_len, "poly.size() == ecc_len");
    std::vector<uint8_t> z(block_len);
    ffgpu_check(ffgpu_rsi16_roots_host(code, poly.data(), z.data()));
    std::vector<size_t> out;
    for (size_t i = 0; i < block_len; ++i)
        if (z[i]) out.push_back(i);
    return out;
}

void register_rsi16(py::module &m) {
    py::enum_<RepairStatus>(m, "RepairStatus", R"(Repair operation status)")
        .value("NoErrors", RepairStatus::NoErrors)
        .value("NoErrorsZero", RepairStatus::NoErrorsZero)
        .value("RepairOk", RepairStatus::RepairOk)
        .value("RepairFail", RepairStatus::RepairFail)
        .value("ErrorLocationFail", RepairStatus::ErrorLocationFail);

    py::class_<PyNTT>(m, "NTT")
        .def_property_readonly("ntt_len", [](PyNTT &s) { return s.ntt_len; })
        .def_property_readonly("ntt_size", [](PyNTT &s) { return s.ntt_len * 2; })
        .def_property_readonly("block_len", [](PyNTT &s) { return s.block_len; })
        .def_property_readonly("ecc_len", [](PyNTT &s) { return s.ecc_len; })
        .def_property_readonly("ecc_size", [](PyNTT &s) { return s.ecc_len * 2; })
        .def("rbo", &PyNTT::rbo, "i"_a);

    py::class_<PyRSi16>(m, "RSi16")
        .def(py::init<size_t, uint16_t, size_t, uint32_t, std::optional<bool>, std::optional<bool>,
                      std::optional<bool>>(),
             R"(Instantiate a Reed-Solomon encoder with the given configuration)", "block_len"_a, "ecc_len"_a,
             "interleave"_a = 1, py::kw_only(), "primitive"_a = 3, "simd_x4"_a = py::none(), "simd_x8"_a = py::none(),
             "simd_x16"_a = py::none())
        .def_property_readonly("block_len", [](PyRSi16 &s) { return s.ilen(s.block_len); })
        .def_property_readonly("block_size", [](PyRSi16 &s) { return s.ilen(s.block_len) * 2; })
        .def_property_readonly("message_len", [](PyRSi16 &s) { return s.ilen(s.message_len); })
        .def_property_readonly("message_size", [](PyRSi16 &s) { return s.ilen(s.message_len) * 2; })
        .def_property_readonly("ecc_len", [](PyRSi16 &s) { return s.ilen(s.ecc_len); })
        .def_property_readonly("ecc_size", [](PyRSi16 &s) { return s.ilen(s.ecc_len) * 2; })
        .def_property_readonly("rs_block_len", [](PyRSi16 &s) { return s.block_len; })
        .def_property_readonly("rs_block_size", [](PyRSi16 &s) { return s.block_len * 2; })
        .def_property_readonly("rs_message_len", [](PyRSi16 &s) { return s.message_len; })
        .def_property_readonly("rs_message_size", [](PyRSi16 &s) { return s.message_len * 2; })
        .def_property_readonly("rs_ecc_len", [](PyRSi16 &s) { return s.ecc_len; })
        .def_property_readonly("rs_ecc_size", [](PyRSi16 &s) { return s.ecc_len * 2; })
        .def_property_readonly("ntt_len", [](PyRSi16 &s) { return s.ntt_len; })
        .def_property_readonly("ntt_size", [](PyRSi16 &s) { return s.ntt_len * 2; })
        .def_property_readonly("root", [](PyRSi16 &s) { return s.root; })
        .def_property_readonly("gf", [](PyRSi16 &s) { return make_gfi16(s.primitive); })
        .def_property_readonly("ntt", [](PyRSi16 &s) { return PyNTT{s.ntt_len, s.block_len, s.ecc_len}; })
        .def_property_readonly("interleave", [](PyRSi16 &s) { return s.interleave; })
        .def_property_readonly("simd_x4", [](PyRSi16 &s) { return s.simd_x4; })
        .def_property_readonly("simd_x8", [](PyRSi16 &s) { return s.simd_x8; })
        .def_property_readonly("simd_x16", [](PyRSi16 &s) { return s.simd_x16; })
        .def("__sizeof_cpp__", [](PyRSi16 &) { return sizeof(PyRSi16); })
        .def("encode", &PyRSi16::encode, R"(Systematic encode)", "buffer"_a)
        .def("repair", &PyRSi16::repair, R"(Repair a block with the given error locations)", "message"_a, "ecc"_a,
             "error_pos"_a = py::none())
        .def("repair_blocks", &PyRSi16::repair_blocks,
             R"(Repair nblocks contiguous blocks with unknown error locations; one status byte per block)",
             "message"_a, "ecc"_a)
        .def("_synd", &PyRSi16::synd, "message"_a, "ecc"_a)
        .def("_sugiyama", [](PyRSi16 &s, std::vector<uint32_t> v) { return s.sugiyama(v, 1); }, "synd"_a)
        .def("_sugiyama4", [](PyRSi16 &s, std::vector<uint32_t> v) { return s.sugiyama(v, 4); }, "synd"_a)
        .def("_sugiyama8", [](PyRSi16 &s, std::vector<uint32_t> v) { return s.sugiyama(v, 8); }, "synd"_a)
        .def("_sugiyama16", [](PyRSi16 &s, std::vector<uint32_t> v) { return s.sugiyama(v, 16); }, "synd"_a)
        .def("message_offset", &PyRSi16::message_offset, "row"_a, "col"_a)
        .def("ecc_offset", &PyRSi16::ecc_offset, "row"_a, "col"_a)
        .def("_roots", &PyRSi16::roots, "synd"_a)
        .doc() = R"(Reed-Solomon coding over :math:`GF(65537)`)";
}
