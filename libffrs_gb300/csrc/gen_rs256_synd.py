"""Generates rs256_synd_gen.cuh: the straight-line GF(2) networks of the
bitsliced RS256 syndrome kernel for ecc_len 32 (field polynomial 0x11d,
primitive 2).

    python libffrs_gb300/csrc/gen_rs256_synd.py      # rewrites the header

The syndromes S_j = r(a^j), j < 32, of a codeword r(x) = sum_d r_d x^d are
split by bit plane: with r_d = sum_b r_{d,b} a^b (bit b of byte r_d),
S_j = sum_b a^b s_{b,j} and s_{b,j} = sum_d r_{d,b} a^{j d}, a polynomial
with coefficients in GF(2) evaluated at a^j.  For such a polynomial
s_{b,2j} = s_{b,j}^2, so per plane only the odd j < 32 and j = 0 are
evaluated: 1 + 16 * 8 = 129 bits (the "rows").  The evaluation is Horner in
steps of 32 degrees, s_o <- s_o a^{32 o} + sum_k in_k a^{(31-k) o}, the input
bits taken four at a time with all 15 XOR combinations formed once and
shared by every row ("four Russians").  synd_combine_* then forms
S_j = sum_b a^b s_{b,o}^{2^k} (j = 2^k o) from the rows of all 8 planes.
Every constant is resolved here, so the code reaches the device as plain
LOP3 networks over registers.
"""

import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "rs256_synd_gen.cuh")


def gmul(a, b):
    r = 0
    while b:
        if b & 1:
            r ^= a
        a <<= 1
        if a & 0x100:
            a ^= 0x11D
        b >>= 1
    return r


EXP = [1] * 512
for _i in range(1, 512):
    EXP[_i] = gmul(EXP[_i - 1], 2)

ODD = list(range(1, 32, 2))
NROWS = 1 + 8 * len(ODD)  # 129


def row(o, p):
    return 0 if o == 0 else 1 + 8 * ODD.index(o) + p


def apow(e):
    return EXP[e % 255]


def xor_expr(terms):
    """XOR of the operand strings, grouped three at a time (ptxas turns each
    three-input XOR into one LOP3)"""
    terms = list(terms)
    if not terms:
        return "0u"
    while len(terms) > 1:
        nxt = []
        i = 0
        while i < len(terms):
            if i + 2 < len(terms):
                nxt.append("(%s ^ %s ^ %s)" % (terms[i], terms[i + 1], terms[i + 2]))
                i += 3
            elif i + 1 < len(terms):
                nxt.append("(%s ^ %s)" % (terms[i], terms[i + 1]))
                i += 2
            else:
                nxt.append(terms[i])
                i += 1
        terms = nxt
    return terms[0]


def gen_step():
    L = []
    L.append("// One Horner step of 32 degrees for one bit plane: in(k) is the plane word")
    L.append("// of the degree (top - k), k = 0..31; s holds the %d rows (row 0: o = 0," % NROWS)
    L.append("// row 1 + 8m + p: bit p of s_o, o = 2m + 1).")
    L.append("template <typename In>")
    L.append("__device__ __forceinline__ void synd_step32(In in, uint32_t (&s)[%d]) {" % NROWS)
    # multiplication part: s_o <- s_o * a^{32 o}
    for o in ODD:
        c = apow(32 * o)
        L.append("    {")
        L.append("        const uint32_t %s;" % ", ".join("q%d = s[%d]" % (q, row(o, q)) for q in range(8)))
        for p in range(8):
            ins = ["q%d" % q for q in range(8) if (gmul(c, 1 << q) >> p) & 1]
            L.append("        s[%d] = %s;" % (row(o, p), xor_expr(ins)))
        L.append("    }")
    # input groups of four, two groups per pass
    for g0 in range(0, 8, 2):
        L.append("    {")
        for gi, g in enumerate((g0, g0 + 1)):
            nm = "ab"[gi]
            for m in range(4):
                L.append("        const uint32_t %s%d = in(%d);" % (nm, 1 << m, 4 * g + m))
            # combinations (pairs, triples, the quadruple)
            L.append("        const uint32_t %s3 = %s1 ^ %s2, %s5 = %s1 ^ %s4, %s6 = %s2 ^ %s4, %s9 = %s1 ^ %s8, "
                     "%s10 = %s2 ^ %s8, %s12 = %s4 ^ %s8;" % ((nm,) * 18))
            L.append("        const uint32_t %s7 = %s3 ^ %s4, %s11 = %s3 ^ %s8, %s13 = %s5 ^ %s8, %s14 = %s6 ^ %s8, "
                     "%s15 = %s3 ^ %s12;" % ((nm,) * 15))
        for o in [0] + ODD:
            for p in range(8 if o else 1):
                sel = []
                for g in (g0, g0 + 1):
                    msk = 0
                    for m in range(4):
                        k = 4 * g + m
                        if (apow((31 - k) * o) >> p) & 1:
                            msk |= 1 << m
                    sel.append(msk)
                terms = ["s[%d]" % row(o, p)]
                if sel[0]:
                    terms.append("a%d" % sel[0])
                if sel[1]:
                    terms.append("b%d" % sel[1])
                if len(terms) > 1:
                    L.append("        s[%d] = %s;" % (row(o, p), xor_expr(terms)))
        L.append("    }")
    L.append("}")
    return L


def synd_parts(j):
    if j == 0:
        return 0, 0
    o, k = j, 0
    while o % 2 == 0:
        o //= 2
        k += 1
    return o, k


HALF_A = [0, 1, 3, 5, 7, 9, 11, 13]
HALF_B = [15, 17, 19, 21, 23, 25, 27, 29, 31]


def half_rows(half):
    rows = []
    for o in half:
        rows += [row(o, 0)] if o == 0 else [row(o, p) for p in range(8)]
    return rows


def syndromes_of(half):
    return [j for j in range(32) if synd_parts(j)[0] in half]


def split(js, nw=8):
    per = -(-len(js) // nw)
    return [js[w * per:(w + 1) * per] for w in range(nw)]


def gen_combine(name, half):
    """synd_combine_<name><W>(X, out): warp W's syndromes of this half; X
    holds the half's rows of all planes at X[(i * 8 + b) * 32] (i: row index
    within the half), out[(8 j + p) * 32] receives plane p of S_j"""
    rows = half_rows(half)
    ridx = {r: i for i, r in enumerate(rows)}
    L = []
    for w, js in enumerate(split(syndromes_of(half))):
        L.append("__device__ __forceinline__ void synd_combine_%s%d(const uint32_t *X, uint32_t *out) {" % (name, w))
        for j in js:
            o, k = synd_parts(j)
            L.append("    {  // S_%d" % j)
            if o == 0:
                for p in range(8):
                    L.append("        out[%d * 32] = X[(%d * 8 + %d) * 32];" % (8 * j + p, ridx[row(0, 0)], p))
            else:
                L.append("        uint32_t y[64];")
                L.append("#pragma unroll")
                L.append("        for (int q = 0; q < 8; ++q)")
                L.append("#pragma unroll")
                L.append("            for (int b = 0; b < 8; ++b) y[8 * b + q] = X[((%d + q) * 8 + b) * 32];" % ridx[row(o, 0)])
                for p in range(8):
                    ins = ["y[%d]" % (8 * b + q) for b in range(8) for q in range(8)
                           if (apow(b + q * (1 << k)) >> p) & 1]
                    L.append("        out[%d * 32] = %s;" % (8 * j + p, xor_expr(ins)))
            L.append("    }")
        L.append("}")
        L.append("")
    return L


def generate():
    L = ["// Generated by gen_rs256_synd.py -- do not edit; run the script instead.",
         "// GF(2) networks of the bitsliced RS256 syndromes for ecc_len 32 (field",
         "// polynomial 0x11d, primitive 2); see the script for the derivation.",
         "#pragma once", "", "#include <cstdint>", "",
         "namespace ffgpu {", "namespace bs {", "",
         "constexpr int kSyndRows = %d;" % NROWS,
         "constexpr int kSyndRowsA = %d;  // rows of o in {%s}" % (len(half_rows(HALF_A)), ", ".join(map(str, HALF_A))),
         "constexpr int kSyndRowsB = %d;  // rows of o in {%s}" % (len(half_rows(HALF_B)), ", ".join(map(str, HALF_B))),
         ""]
    L += gen_step()
    L.append("")
    L += gen_combine("A", HALF_A)
    L += gen_combine("B", HALF_B)
    L += ["}  // namespace bs", "}  // namespace ffgpu", ""]
    return "\n".join(L)


if __name__ == "__main__":
    with open(OUT, "w") as f:
        f.write(generate())
    print(OUT)
