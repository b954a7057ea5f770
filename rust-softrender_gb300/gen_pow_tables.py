"""Writes include/sr_pow_tables.h: the tables of the table-driven log2 / exp2
used by sr_powf (include/sr_shaders.h).

    python rust-softrender_gb300/gen_pow_tables.py

log2 table, 64 entries: for c_i = 1 + (i + 1/2)/64, INV[i] = c_i^-1 rounded to
float and -log2(INV[i]) as a float pair (hi, lo), so that for m in
[1 + i/64, 1 + (i+1)/64) log2(m) = -log2(INV[i]) + log2(1 + r) with
r = m * INV[i] - 1, |r| < 2^-7.
exp2 table, 65 entries: 2^(j/64) for j = -32..32 as a float pair (hi, lo).
Values come from 50-digit decimal arithmetic (the decimal module's ln / exp),
rounded to nearest float32."""
import os
import struct
from decimal import Decimal, getcontext

getcontext().prec = 50
LN2 = Decimal(2).ln()


def f32(d):
    """Decimal -> nearest float32 (via the double nearest to d; the double
    carries 53 bits, so the pair hi + lo below keeps ~48 bits)."""
    return struct.unpack("f", struct.pack("f", float(d)))[0]


def pair(d):
    hi = f32(d)
    lo = f32(d - Decimal(repr(hi)))
    return hi, lo


def fmt(v):
    return "%.9ef" % v if v != 0.0 else "0.0f"


def main():
    inv, lh, ll = [], [], []
    for i in range(64):
        c = Decimal(1) + (Decimal(i) + Decimal("0.5")) / 64
        iv = f32(Decimal(1) / c)
        inv.append(iv)
        L = -(Decimal(repr(iv)).ln() / LN2)
        h, lo = pair(L)
        lh.append(h)
        ll.append(lo)
    eh, el = [], []
    for j in range(-32, 33):
        v = (Decimal(j) / 64 * LN2).exp()
        h, lo = pair(v)
        eh.append(h)
        el.append(lo)
    out = ["/* sr_pow_tables.h -- generated by rust-softrender_gb300/gen_pow_tables.py; do not edit.",
           " * Tables of the table-driven log2 / exp2 behind sr_powf (sr_shaders.h). */",
           "#ifndef SR_POW_TABLES_H", "#define SR_POW_TABLES_H", "",
           "#if defined(__CUDA_ARCH__)", "#define SR_TAB(name, i) __ldg(&name##_D[(i)])", "#else",
           "#define SR_TAB(name, i) name[(i)]", "#endif", ""]

    def arr(name, vals):
        body = []
        for k in range(0, len(vals), 4):
            body.append("    " + ", ".join(fmt(v) for v in vals[k:k + 4]) + ",")
        # a host copy, and a device copy for CUDA device code (SR_TAB picks)
        out.append("static const float %s[%d] = {" % (name, len(vals)))
        out.extend(body)
        out.append("};")
        out.append("#if defined(__CUDACC__)")
        out.append("static __device__ const float %s_D[%d] = {" % (name, len(vals)))
        out.extend(body)
        out.append("};")
        out.append("#endif")

    arr("SR_LOG2_INV", inv)
    arr("SR_LOG2_HI", lh)
    arr("SR_LOG2_LO", ll)
    arr("SR_EXP2_HI", eh)
    arr("SR_EXP2_LO", el)
    out += ["", "#endif /* SR_POW_TABLES_H */", ""]
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(os.path.dirname(here), "include", "sr_pow_tables.h")
    with open(path, "w") as f:
        f.write("\n".join(out))
    print(path)


if __name__ == "__main__":
    main()
