"""Writes sod_dd_tables.h: the constants of the double-float (float pair) exp and sincos in
sod_dd.cuh, computed with mpmath at 60 digits and split into float pairs (hi = nearest float,
lo = nearest float of the remainder).  Run: python gen_dd_tables.py > sod_dd_tables.h"""
import mpmath as mp
import numpy as np

mp.mp.dps = 60


def f32(x):
    return np.float32(float(x))


def split(x):
    hi = f32(x)
    lo = f32(x - mp.mpf(float(hi)))
    return hi, lo


def hexf(v):
    v = float(v)
    if v == 0.0:
        return "0.0f"
    return v.hex().replace("0x", "0x") + "f"


def cody_waite(x, bits_first):
    """x = c1 + c2 + c3 with c1 carrying `bits_first` significant bits (so m*c1 is exact for small m)."""
    e = mp.floor(mp.log(abs(x), 2))
    scale = mp.mpf(2) ** (e - bits_first + 1)
    c1 = mp.nint(x / scale) * scale
    r = x - c1
    c2 = f32(r)
    c3 = f32(r - mp.mpf(float(c2)))
    return f32(c1), c2, c3


out = ["// Generated by gen_dd_tables.py (mpmath, 60 digits).  Do not edit.", "#pragma once", "namespace sod {", ""]
out.append("// 2^(j/64), j = 0..63, as float pairs")
out.append("SOD_DD_TABLE float c_dd_exp2_tab[64][2] = {")
for j in range(64):
    hi, lo = split(mp.power(2, mp.mpf(j) / 64))
    out.append(f"    {{{hexf(hi)}, {hexf(lo)}}},")
out.append("};")
out.append("// sin(j pi/32), cos(j pi/32), j = 0..63, as float pairs {sin_hi, sin_lo, cos_hi, cos_lo}")
out.append("SOD_DD_TABLE float c_dd_sincos_tab[64][4] = {")
for j in range(64):
    a = mp.pi * j / 32
    sh, sl = split(mp.sin(a))
    ch, cl = split(mp.cos(a))
    out.append(f"    {{{hexf(sh)}, {hexf(sl)}, {hexf(ch)}, {hexf(cl)}}},")
out.append("};")
l1, l2, l3 = cody_waite(mp.log(2) / 64, 11)
p1, p2, p3 = cody_waite(mp.pi / 32, 11)
out.append(f"constexpr float kDdLn2o64_1 = {hexf(l1)}, kDdLn2o64_2 = {hexf(l2)}, kDdLn2o64_3 = {hexf(l3)};")
out.append(f"constexpr float kDdPio32_1 = {hexf(p1)}, kDdPio32_2 = {hexf(p2)}, kDdPio32_3 = {hexf(p3)};")
out.append(f"constexpr float kDd64oLn2 = {hexf(f32(64 / mp.log(2)))}, kDd32oPi = {hexf(f32(32 / mp.pi))};")
for name, val in (("Third", mp.mpf(1) / 3), ("Sixth", mp.mpf(1) / 6), ("Thirtieth", mp.mpf(1) / 30),
                  ("TwentyFourth", mp.mpf(1) / 24), ("M144th", mp.mpf(-1) / 144)):
    hi, lo = split(val)
    out.append(f"constexpr float kDd{name}_hi = {hexf(hi)}, kDd{name}_lo = {hexf(lo)};")
out.append("")
out.append("}  // namespace sod")
print("\n".join(out))
