"""
Generate lean_tables.inc: the constant tables of the FP64 elementary
functions in lean_math.cuh, correctly rounded with mpmath.

* log table (Tang's table-driven logarithm, ACM TOMS 16(4), 1990): grid
  g_k = 0.75 + k / 256, k = 0..192, covering the reduced mantissa range
  [0.75, 1.5]; C[k] = float32 nearest 1/g_k (exact in double) and
  L[k] = -ln(C[k]) rounded to double.  g_64 = 1 gives C = 1, L = 0 exactly,
  so logarithms of arguments near 1 have no table error.
* argument table: TH[j] = double(j * pi / 128), j = -32..32 (one quadrant
  split in 64 steps), with COS[j], SIN[j] the correctly rounded cosine and
  sine of the double TH[j]; COSF/SINF hold the same cosine and sine as
  float pairs (hi = nearest float, lo = nearest float to the remainder),
  interleaved hi, lo.
* kThirdHi/kThirdLo: 1/3 as a float pair; LOGLF = -ln C[k] and THF = TH[j]
  as float pairs; ln 2 and pi/2 as three floats (12-bit head).

Run:  python harmonica_gb300/csrc/gen_tables.py   (writes next to this file)
"""

import os

import mpmath as mp
import numpy as np

mp.mp.dps = 50
HERE = os.path.dirname(os.path.abspath(__file__))


def d(x):
    return float(x).hex()


def fl(x):
    return float(x).hex() + "f"


def f32pair(x):
    hi = np.float32(float(x))
    lo = np.float32(float(x - mp.mpf(float(hi))))
    return float(hi), float(lo)


def main():
    lines = [
        "// Generated by gen_tables.py -- do not edit.",
        "// Tables of lean_math.cuh (see gen_tables.py for their definition).",
        "#pragma once",
        "",
        "namespace hg {",
        "namespace lean {",
        "",
        "constexpr int kLogTableSize = 193;",
        "constexpr int kArgTableHalf = 32;",
        "constexpr int kArgTableSize = 65;",
        "",
    ]
    c, L = [], []
    for k in range(193):
        g = mp.mpf(3) / 4 + mp.mpf(k) / 256
        ck = float(np.float32(float(1 / g)))
        c.append(ck)
        L.append(float(-mp.log(mp.mpf(ck))))
    assert c[64] == 1.0 and L[64] == 0.0
    lines.append("HG_TABLE_QUAL double kLogC[kLogTableSize] = {")
    lines += [f"    {d(v)}," for v in c]
    lines.append("};")
    lines.append("HG_TABLE_QUAL double kLogL[kLogTableSize] = {")
    lines += [f"    {d(v)}," for v in L]
    lines.append("};")
    th, co, si = [], [], []
    for j in range(-32, 33):
        t = float(mp.mpf(j) * mp.pi / 128)
        th.append(t)
        co.append(float(mp.cos(mp.mpf(t))))
        si.append(float(mp.sin(mp.mpf(t))))
    for name, vals in (("kArgTh", th), ("kArgCos", co), ("kArgSin", si)):
        lines.append(f"HG_TABLE_QUAL double {name}[kArgTableSize] = {{")
        lines += [f"    {d(v)}," for v in vals]
        lines.append("};")
    for name, vals in (("kArgCosF", co), ("kArgSinF", si)):
        lines.append(f"HG_TABLE_QUAL float {name}[2 * kArgTableSize] = {{")
        for t, v in zip(th, vals):
            exact = mp.cos(mp.mpf(t)) if name == "kArgCosF" else mp.sin(mp.mpf(t))
            hi, lo = f32pair(exact)
            lines.append(f"    {fl(hi)}, {fl(lo)},")
        lines.append("};")
    hi, lo = f32pair(mp.mpf(1) / 3)
    lines.append(f"constexpr float kThirdHi = {fl(hi)};")
    lines.append(f"constexpr float kThirdLo = {fl(lo)};")
    # -ln(C[k]) and TH[j] as float pairs, interleaved hi, lo
    lines.append("HG_TABLE_QUAL float kLogLF[2 * kLogTableSize] = {")
    for ck in c:
        hi, lo = f32pair(-mp.log(mp.mpf(ck)))
        lines.append(f"    {fl(hi)}, {fl(lo)},")
    lines.append("};")
    lines.append("HG_TABLE_QUAL float kArgThF[2 * kArgTableSize] = {")
    for j in range(-32, 33):
        hi, lo = f32pair(mp.mpf(j) * mp.pi / 128)
        lines.append(f"    {fl(hi)}, {fl(lo)},")
    lines.append("};")
    # ln 2 and pi/2 as three floats: the first with 12 significant bits (an
    # integer of up to 12 bits times it is exact in a float), the second the
    # nearest float to the remainder, the third the nearest to what is left
    for name, val in (("Ln2", mp.log(2)), ("Pio2", mp.pi / 2)):
        m, e = mp.frexp(val)
        f1 = float(mp.ldexp(mp.floor(mp.ldexp(m, 12)), e - 12))
        f2 = float(np.float32(float(val - mp.mpf(f1))))
        f3 = float(np.float32(float(val - mp.mpf(f1) - mp.mpf(f2))))
        lines.append(f"constexpr float k{name}F1 = {fl(f1)};")
        lines.append(f"constexpr float k{name}F2 = {fl(f2)};")
        lines.append(f"constexpr float k{name}F3 = {fl(f3)};")
    # constants split in a high part with 40 significant bits (so that an
    # integer of up to 13 bits times the high part is exact) and a low part
    for name, val in (("Ln2", mp.log(2)), ("Pio2", mp.pi / 2)):
        m, e = mp.frexp(val)
        hi = float(mp.ldexp(mp.floor(mp.ldexp(m, 40)), e - 40))
        lo = float(val - mp.mpf(hi))
        lines.append(f"constexpr double k{name}Hi = {d(hi)};")
        lines.append(f"constexpr double k{name}Lo = {d(lo)};")
    lines += ["", "}  // namespace lean", "}  // namespace hg", ""]
    with open(os.path.join(HERE, "lean_tables.inc"), "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
