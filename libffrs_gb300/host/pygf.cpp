// GF256 and GFi16 scalar/polynomial helpers (libffrs/pygf256.hpp,
// libffrs/pygfi16.hpp).  These are host-side conveniences used by callers and
// tests (e.g. RS256.gf.poly_mod_x_n); they have no throughput role, so they
// are plain C++ with the reference's conventions (galois.hpp).
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "pyffrs_common.h"

namespace py = pybind11;
using namespace pybind11::literals;

class PyGF256 {
public:
    uint8_t primitive, poly1;
    uint8_t exp_[256], log_[256];

    static uint8_t mul_serial(uint8_t p1, uint8_t a, uint8_t b) {
        uint8_t r = 0;
        for (int i = 7; i >= 0; --i) {
            r = (r & 0x80) ? (uint8_t)((r << 1) ^ p1) : (uint8_t)(r << 1);
            if (a & (1u << i)) r ^= b;
        }
        return r;
    }
    PyGF256(uint8_t primitive_, uint16_t poly) : primitive(primitive_), poly1((uint8_t)(poly & 0xff)) {
        std::memset(exp_, 0, 256);
        std::memset(log_, 0, 256);
        uint8_t x = 1;
        for (int i = 0; i < 256; ++i) {
            exp_[i] = x;
            log_[x] = (uint8_t)i;
            x = mul_serial(poly1, x, primitive);
        }
    }
    uint8_t mul(uint8_t a, uint8_t b) const {
        if (!a || !b) return 0;
        unsigned r = (unsigned)log_[a] + log_[b];
        if (r >= 255) r -= 255;
        return exp_[r];
    }
    uint8_t add(uint8_t a, uint8_t b) const { return a ^ b; }
    uint8_t inv(uint8_t a) const { return exp_[255 - log_[a]]; }
    uint8_t div(uint8_t a, uint8_t b) const {
        if (!a) return 0;
        unsigned r = (unsigned)log_[a] + 255 - log_[b];
        if (r >= 255) r -= 255;
        return exp_[r];
    }
    uint8_t pow(uint8_t a, uint8_t b) const { return exp_[((unsigned)log_[a] * b) % 255]; }

    static std::vector<uint8_t> vec(py::buffer b) {
        BufRO<uint8_t> v(b);
        return std::vector<uint8_t>(v.data, v.data + v.size);
    }
    static py::bytearray ba(const std::vector<uint8_t> &v, size_t n) {
        py::bytearray o = make_bytearray(n);
        if (n) std::memcpy(bytearray_data(o), v.data(), n);
        return o;
    }
    // galois.hpp:533-550, 560-577
    py::bytearray poly_addsub(py::buffer a_, py::buffer b_) {
        auto a = vec(a_), b = vec(b_);
        size_t n = std::max(a.size(), b.size());
        std::vector<uint8_t> o(n, 0);
        if (a.size() > b.size()) {
            size_t s = a.size() - b.size();
            for (size_t i = 0; i < n; ++i) o[i] = a[i] ^ (i >= s ? b[i - s] : 0);
        } else {
            size_t s = b.size() - a.size();
            for (size_t i = 0; i < n; ++i) o[i] = b[i] ^ (i >= s ? a[i - s] : 0);
        }
        return ba(o, n);
    }
    // galois.hpp:579-595
    py::bytearray poly_mul(py::buffer a_, py::buffer b_) {
        auto a = vec(a_), b = vec(b_);
        size_t n = a.size() + b.size() - 1;
        std::vector<uint8_t> o(n, 0);
        for (size_t i = 0; i < a.size(); ++i)
            for (size_t j = 0; j < b.size(); ++j) o[i + j] ^= mul(a[i], b[j]);
        return ba(o, n);
    }
    // galois.hpp:427-459
    py::bytearray poly_mod(py::buffer a_, py::buffer b_) {
        auto a = vec(a_), b = vec(b_);
        if (b.size() < 2) return make_bytearray(0);
        size_t sr = b.size() - 1;
        std::vector<uint8_t> rem(sr, 0);
        std::copy_n(a.begin(), std::min(a.size(), sr), rem.begin());
        if (a.size() < b.size()) return ba(rem, a.size());
        uint8_t nf = inv(b[0]);
        for (size_t i = 0; i < a.size() - sr; ++i) {
            uint8_t c = mul(rem[0], nf);
            std::rotate(rem.begin(), rem.begin() + 1, rem.end());
            rem[sr - 1] = a[sr + i];
            if (!c) continue;
            for (size_t j = 0; j < sr; ++j) rem[j] ^= mul(b[j + 1], c);
        }
        return ba(rem, sr);
    }
    // galois.hpp:406-425
    py::tuple poly_divmod(py::buffer a_, py::buffer b_) {
        auto a = vec(a_), b = vec(b_);
        size_t sep = 0;
        if (b.size() <= a.size()) {
            uint8_t nf = inv(b[0]);
            for (size_t i = 0; i < a.size() - b.size() + 1; ++i) {
                uint8_t c = a[i] = mul(a[i], nf);
                if (!c) continue;
                for (size_t j = 1; j < b.size(); ++j) a[i + j] ^= mul(b[j], c);
            }
            sep = a.size() - b.size() + 1;
        }
        std::vector<uint8_t> q(a.begin(), a.begin() + sep), r(a.begin() + sep, a.end());
        return py::make_tuple(ba(q, q.size()), ba(r, r.size()));
    }
    // galois.hpp:462-499
    py::bytearray poly_mod_x_n(py::buffer a_, py::buffer b_) {
        auto a = vec(a_), b = vec(b_);
        const size_t sb = b.size();
        std::vector<uint8_t> rem(sb, 0);
        if (a.size() >= sb) {
            std::copy_n(a.begin(), sb, rem.begin());
            for (size_t i = 0; i < a.size() - sb; ++i) {
                uint8_t c = rem[0];
                rem[0] = a[sb + i];
                std::rotate(rem.begin(), rem.begin() + 1, rem.end());
                if (!c) continue;
                for (size_t j = 0; j < sb; ++j) rem[j] ^= mul(b[j], c);
            }
        } else {
            std::copy_n(a.begin(), a.size(), rem.begin() + (sb - a.size()));
        }
        for (size_t i = 0; i < sb; ++i) {
            uint8_t c = rem[0];
            rem[0] = 0;
            std::rotate(rem.begin(), rem.begin() + 1, rem.end());
            if (!c) continue;
            for (size_t j = 0; j < sb; ++j) rem[j] ^= mul(b[j], c);
        }
        return ba(rem, sb);
    }
    uint8_t poly_eval(py::buffer p_, uint8_t x) {
        auto p = vec(p_);
        uint8_t r = 0;
        for (auto c : p) r = mul(r, x) ^ c;
        return r;
    }
    // gf_wide_mul (galois.hpp:670-723): eight independent lanes
    uint64_t mul_wide(uint64_t a, uint64_t b) const {
        uint64_t r = 0;
        for (int lane = 0; lane < 8; ++lane) {
            uint8_t x = (uint8_t)(a >> (8 * lane)), y = (uint8_t)(b >> (8 * lane));
            r |= (uint64_t)mul_serial(poly1, x, y) << (8 * lane);
        }
        return r;
    }
    py::bytearray poly_eval8(py::buffer p_, py::buffer xs_) {
        auto p = vec(p_), xs = vec(xs_);
        if (xs.size() > 8) throw py::value_error("Invalid buffer size");
        uint64_t x = 0;
        std::memcpy(&x, xs.data(), xs.size());
        uint64_t r = 0;
        for (auto c : p) r = mul_wide(r, x) ^ (0x0101010101010101ull * c);
        std::vector<uint8_t> o(8);
        std::memcpy(o.data(), &r, 8);
        return ba(o, 8);
    }
    py::bytearray mul8(py::buffer a_, py::buffer b_) {
        auto a = vec(a_), b = vec(b_);
        if (a.size() != 8 || b.size() != 8) throw py::value_error("Can only multiply 8-byte wide arrays");
        uint64_t x, y;
        std::memcpy(&x, a.data(), 8);
        std::memcpy(&y, b.data(), 8);
        uint64_t r = mul_wide(x, y);
        std::vector<uint8_t> o(8);
        std::memcpy(o.data(), &r, 8);
        return ba(o, 8);
    }
};

py::object make_gf256(uint8_t primitive, uint16_t polynomial) { return py::cast(PyGF256(primitive, polynomial)); }

// GF(65537) (galois.hpp:168-216, 258-395; pygfi16.hpp)
class PyGFi16 {
public:
    uint32_t primitive;
    std::vector<uint32_t> exp_, log_;
    explicit PyGFi16(uint32_t primitive_) : primitive(primitive_), exp_(65537), log_(65537, 0) {
        uint32_t x = 1;
        for (uint32_t i = 0; i < 65537; ++i) {
            exp_[i] = x;
            log_[x] = i;
            uint64_t prod = (uint64_t)x * primitive;
            x = (prod > 0xffffffffull ? 1u : (uint32_t)prod) % 0x10001u;
        }
        if (!(pow(primitive, 32768) == 65536 && pow(primitive, 65536) == 1))
            throw std::runtime_error(std::to_string(primitive) + " is not a primitive element of GF(65537)");
    }
    static uint32_t mul(uint32_t a, uint32_t b) {
        uint32_t r = a * b;
        if (r == 0 && a && b) return 1;
        r = (r & 0xffff) - (r >> 16);
        if (r >= 0x80000000u) r += 0x10001u;
        return r;
    }
    static uint32_t add(uint32_t a, uint32_t b) {
        uint32_t r = a + b;
        if (r >= 0x10001u) r -= 0x10001u;
        return r;
    }
    static uint32_t sub(uint32_t a, uint32_t b) {
        uint32_t r = a - b;
        if (r >= 0x80000000u) r += 0x10001u;
        return r;
    }
    uint32_t inv(uint32_t a) const { return exp_.at(65536u - log_.at(a)); }
    uint32_t div(uint32_t a, uint32_t b) const {
        if (!a) return 0;
        uint32_t r = log_.at(a) + 65536u - log_.at(b);
        if (r >= 65536u) r -= 65536u;
        return exp_[r];
    }
    uint32_t pow(uint32_t a, uint32_t e) const { return exp_[(uint32_t)(log_.at(a) * e) % 65536u]; }
    uint32_t exp(uint32_t a) const { return exp_.at(a); }
    uint32_t log(uint32_t a) const { return log_.at(a); }
};

py::object make_gfi16(uint32_t primitive) { return py::cast(PyGFi16(primitive)); }

void register_gf(py::module &m) {
    py::class_<PyGF256>(m, "GF256")
        .def(py::init<uint8_t, uint16_t>(), "primitive"_a = 2, "poly1"_a = 0x11d)
        .def_property_readonly("prime", [](PyGF256 &) { return 2; }, "Always 2")
        .def_property_readonly("power", [](PyGF256 &) { return 8; }, "Always 8")
        .def_property_readonly("primitive", [](PyGF256 &s) { return s.primitive; })
        .def_property_readonly("poly1", [](PyGF256 &s) { return s.poly1; })
        .def_property_readonly("field_elements", [](PyGF256 &) { return 256; })
        .def("__sizeof_cpp__", [](PyGF256 &) { return sizeof(PyGF256); })
        .def("mul", &PyGF256::mul, "lhs"_a, "rhs"_a)
        .def("add", &PyGF256::add, "lhs"_a, "rhs"_a)
        .def("sub", &PyGF256::add, "lhs"_a, "rhs"_a)
        .def("inv", &PyGF256::inv, "value"_a)
        .def("div", &PyGF256::div, "num"_a, "den"_a)
        .def("exp", [](PyGF256 &s, uint8_t v) { return s.exp_[v]; }, "value"_a)
        .def("log", [](PyGF256 &s, uint8_t v) { return s.log_[v]; }, "value"_a)
        .def("pow", &PyGF256::pow, "base"_a, "exponent"_a)
        .def("poly_add", &PyGF256::poly_addsub, "p1"_a, "p2"_a)
        .def("poly_sub", &PyGF256::poly_addsub, "p1"_a, "p2"_a)
        .def("poly_mul", &PyGF256::poly_mul, "p1"_a, "p2"_a)
        .def("poly_mod", &PyGF256::poly_mod, "p1"_a, "p2"_a)
        .def("poly_eval", &PyGF256::poly_eval, "poly"_a, "x"_a)
        .def("poly_eval8", &PyGF256::poly_eval8, "poly"_a, "xs"_a)
        .def("mul8", &PyGF256::mul8, "a"_a, "b"_a)
        .def("poly_divmod", &PyGF256::poly_divmod, "p1"_a, "p2"_a)
        .def("poly_mod_x_n", &PyGF256::poly_mod_x_n, "p1"_a, "p2"_a)
        .doc() = R"(Finite-field operations optimized for :math:`GF(2^8)`)";

    py::class_<PyGFi16>(m, "GFi16")
        .def(py::init<uint32_t>(), "primitive"_a = 3)
        .def_property_readonly("prime", [](PyGFi16 &) { return 0x10001u; })
        .def_property_readonly("power", [](PyGFi16 &) { return 1; })
        .def_property_readonly("primitive", [](PyGFi16 &s) { return s.primitive; })
        .def_property_readonly("field_elements", [](PyGFi16 &) { return 0x10001u; })
        .def("__sizeof_cpp__", [](PyGFi16 &) { return sizeof(PyGFi16); })
        .def("mul", [](PyGFi16 &, uint32_t a, uint32_t b) { return PyGFi16::mul(a, b); }, "lhs"_a, "rhs"_a)
        .def("add", [](PyGFi16 &, uint32_t a, uint32_t b) { return PyGFi16::add(a, b); }, "lhs"_a, "rhs"_a)
        .def("sub", [](PyGFi16 &, uint32_t a, uint32_t b) { return PyGFi16::sub(a, b); }, "lhs"_a, "rhs"_a)
        .def("inv", &PyGFi16::inv, "value"_a)
        .def("div", &PyGFi16::div, "num"_a, "den"_a)
        .def("exp", &PyGFi16::exp, "value"_a)
        .def("log", &PyGFi16::log, "value"_a)
        .def("pow", &PyGFi16::pow, "base"_a, "exponent"_a)
        .doc() = R"(Finite-field operations over :math:`GF(65537)`)";
}
