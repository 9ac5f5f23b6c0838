// CIRC16 binding: the reference's PyCIRC16 surface (libffrs/pycirc16.hpp:33-431)
// on the GPU pipeline.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <optional>
#include <string>
#include <vector>

#include "pyffrs_common.h"

namespace py = pybind11;
using namespace pybind11::literals;

class PyCIRC16 {
public:
    ffgpu_circ16 *code = nullptr;
    py::object rsi, rso;
    size_t ib, ie, ob, oe, interleave;
    uint32_t primitive;
    bool x4, x8, x16;
    size_t message_len = 0, ecc_len = 0;
    size_t ri_ml, ro_ml, rso_interleave, rso_ieccl;

    PyCIRC16(size_t ib_, size_t ie_, size_t ob_, size_t oe_, size_t interleave_, uint32_t primitive_,
             std::optional<bool> sx4, std::optional<bool> sx8, std::optional<bool> sx16, py::object rsi_cls)
        : ib(ib_), ie(ie_), ob(ob_), oe(oe_), interleave(interleave_), primitive(primitive_),
          x4(sx4.value_or(false)), x8(sx8.value_or(false)), x16(sx16.value_or(false)) {
        // PyCIRC16 ctor (pycirc16.hpp:46-65): rsi = RSi16(ib, ie),
        // rso = RSi16(ob, oe, interleave = rsi.message_len * interleave)
        rsi = rsi_cls(ib, ie, 1, "primitive"_a = primitive, "simd_x4"_a = sx4, "simd_x8"_a = sx8, "simd_x16"_a = sx16);
        ri_ml = ib - ie;
        rso_interleave = ri_ml * interleave;
        rso = rsi_cls(ob, oe, rso_interleave, "primitive"_a = primitive, "simd_x4"_a = sx4, "simd_x8"_a = sx8,
                      "simd_x16"_a = sx16);
        ro_ml = ob - oe;
        ffgpu_check(ffgpu_circ16_create(ib, ie, ob, oe, interleave, primitive, &code));
        ffgpu_check(ffgpu_circ16_info(code, &message_len, &ecc_len));
        rso_ieccl = oe * rso_interleave;
    }
    ~PyCIRC16() {
        if (code) ffgpu_circ16_destroy(code);
    }

    // PyCIRC16::py_encode (pycirc16.hpp:337-350)
    py::bytearray encode(py::buffer b) {
        BufRO<uint16_t> buf(b);
        py_assert_like(buf.size % message_len == 0, std::to_string(buf.size));
        const size_t nb = buf.size / message_len;
        py::bytearray out = make_bytearray(nb * ecc_len * 2);
        if (nb) ffgpu_check(ffgpu_circ16_encode_host(code, buf.data, nb, (uint16_t *)bytearray_data(out)));
        return out;
    }

    // PyCIRC16::py_repair (pycirc16.hpp:365-384): always returns False
    bool repair(py::buffer m, py::buffer e) {
        BufRW<uint16_t> msg(m), ecc(e);
        py_assert_like(msg.size == message_len, std::to_string(msg.size) + " != " + std::to_string(message_len));
        py_assert_like(ecc.size == ecc_len, std::to_string(ecc.size));
        uint8_t st = 0;
        ffgpu_check(ffgpu_circ16_repair_host(code, msg.data, ecc.data, 1, &st));
        if (st == FFGPU_STATUS_ASSERT) throw std::runtime_error("Assertion failed: g_len > 0 (NTT-domain Sugiyama)");
        return false;
    }

    // Batched repair of nblocks contiguous CIRC16 blocks; one status byte per
    // block (0, or 255 where the reference raises RuntimeError).
    py::bytearray repair_blocks(py::buffer m, py::buffer e) {
        BufRW<uint16_t> msg(m), ecc(e);
        if (msg.size % message_len) throw py::value_error("message size must be a multiple of message_len");
        const size_t nb = msg.size / message_len;
        if (ecc.size != nb * ecc_len) throw py::value_error("ecc size must be nblocks * ecc_len");
        py::bytearray st = make_bytearray(nb);
        if (nb) ffgpu_check(ffgpu_circ16_repair_host(code, msg.data, ecc.data, nb, (uint8_t *)bytearray_data(st)));
        return st;
    }

    // PyCIRC16::py_find_outer_error_locations (pycirc16.hpp:386-405)
    std::vector<size_t> find_outer(py::buffer m, py::buffer e, size_t k) {
        BufRO<uint16_t> msg(m), ecc(e);
        py_assert_like(msg.size == message_len, std::to_string(msg.size) + " != " + std::to_string(message_len));
        py_assert_like(ecc.size == ecc_len, std::to_string(ecc.size));
        std::vector<uint32_t> rows(ob);
        size_t n = 0;
        ffgpu_check(ffgpu_circ16_find_outer_error_locations_host(code, msg.data, ecc.data, k, rows.data(), &n));
        return std::vector<size_t>(rows.begin(), rows.begin() + n);
    }

    // offsets (pycirc16.hpp:407-430)
    size_t message_offset(size_t k, size_t row, size_t col) const {
        py_assert_like(k < interleave, "interleave < this->interleave");
        py_assert_like(row < ro_ml, "row < rso.message_len");
        py_assert_like(col < ri_ml, "col < rsi.message_len");
        return rso_interleave * row + k * ri_ml + col;
    }
    size_t rso_ecc_offset(size_t k, size_t row, size_t col) const {
        py_assert_like(k < interleave, "interleave < this->interleave");
        py_assert_like(row < oe, "row < rso.ecc_len");
        py_assert_like(col < ri_ml, "col < rsi.message_len");
        return rso_interleave * row + k * ri_ml + col;
    }
    size_t rsi_ecc_offset(size_t k, size_t row, size_t col) const {
        py_assert_like(k < interleave, "interleave < this->interleave");
        py_assert_like(row < ob, "row < rso.block_len");
        py_assert_like(col < ie, "col < rsi.ecc_len");
        return rso_ieccl + (row * interleave + k) * ie + col;
    }
};

void register_circ16(py::module &m) {
    py::object rsi_cls = m.attr("RSi16");
    py::class_<PyCIRC16>(m, "CIRC16")
        .def(py::init([rsi_cls](size_t ib, size_t ie, size_t ob, size_t oe, size_t interleave, uint32_t primitive,
                                std::optional<bool> x4, std::optional<bool> x8, std::optional<bool> x16) {
                 return new PyCIRC16(ib, ie, ob, oe, interleave, primitive, x4, x8, x16, rsi_cls);
             }),
             R"(Cross-interleaved Reed-Solomon coder)", "inner_block_len"_a, "inner_ecc_len"_a, "outer_block_len"_a,
             "outer_ecc_len"_a, "interleave"_a = 1, py::kw_only(), "primitive"_a = 3, "simd_x4"_a = py::none(),
             "simd_x8"_a = py::none(), "simd_x16"_a = py::none())
        .def_property_readonly("rsi", [](PyCIRC16 &s) { return s.rsi; })
        .def_property_readonly("rso", [](PyCIRC16 &s) { return s.rso; })
        .def_property_readonly("block_len", [](PyCIRC16 &s) { return s.ib * s.ob * s.interleave; })
        .def_property_readonly("block_size", [](PyCIRC16 &s) { return s.ib * s.ob * s.interleave * 2; })
        .def_property_readonly("message_len", [](PyCIRC16 &s) { return s.message_len; })
        .def_property_readonly("message_size", [](PyCIRC16 &s) { return s.message_len * 2; })
        .def_property_readonly("ecc_len", [](PyCIRC16 &s) { return s.ecc_len; })
        .def_property_readonly("ecc_size", [](PyCIRC16 &s) { return s.ecc_len * 2; })
        .def_property_readonly("inner_block_len", [](PyCIRC16 &s) { return s.ib; })
        .def_property_readonly("inner_block_size", [](PyCIRC16 &s) { return s.ib * 2; })
        .def_property_readonly("inner_message_len", [](PyCIRC16 &s) { return s.ri_ml; })
        .def_property_readonly("inner_message_size", [](PyCIRC16 &s) { return s.ri_ml * 2; })
        .def_property_readonly("inner_ecc_len", [](PyCIRC16 &s) { return s.ie; })
        .def_property_readonly("inner_ecc_size", [](PyCIRC16 &s) { return s.ie * 2; })
        .def_property_readonly("outer_block_len", [](PyCIRC16 &s) { return s.ob; })
        .def_property_readonly("outer_message_len", [](PyCIRC16 &s) { return s.ro_ml; })
        .def_property_readonly("outer_ecc_len", [](PyCIRC16 &s) { return s.oe; })
        .def_property_readonly("outer_interleave", [](PyCIRC16 &s) { return s.rso_interleave; })
        .def_property_readonly("interleave", [](PyCIRC16 &s) { return s.interleave; })
        .def_property_readonly("primitive", [](PyCIRC16 &s) { return s.primitive; })
        .def_property_readonly("simd_x4", [](PyCIRC16 &s) { return s.x4; })
        .def_property_readonly("simd_x8", [](PyCIRC16 &s) { return s.x8; })
        .def_property_readonly("simd_x16", [](PyCIRC16 &s) { return s.x16; })
        .def("__sizeof_cpp__", [](PyCIRC16 &) { return sizeof(PyCIRC16); })
        .def("encode", &PyCIRC16::encode, R"(Encode data)", "buffer"_a)
        .def("repair", &PyCIRC16::repair, R"(Repair data)", "message"_a, "ecc"_a)
        .def("repair_blocks", &PyCIRC16::repair_blocks, "message"_a, "ecc"_a)
        .def("_find_outer_error_locations", &PyCIRC16::find_outer, "message"_a, "ecc"_a, "interleave"_a)
        .def("message_offset", &PyCIRC16::message_offset, "interleave"_a, "row"_a, "col"_a)
        .def("rso_ecc_offset", &PyCIRC16::rso_ecc_offset, "interleave"_a, "row"_a, "col"_a)
        .def("rsi_ecc_offset", &PyCIRC16::rsi_ecc_offset, "interleave"_a, "row"_a, "col"_a)
        .doc() = R"(Cross-interleaved Reed-Solomon coding over :math:`GF(65537)`)";
}
