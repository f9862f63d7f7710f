"""Generate st_crmath_tables.h: the constants of the correctly rounded log,
sin/cos and acos used by the trajectory (st_crmath.cuh), as double-double
pairs (hi = the double nearest the value, lo = the double nearest the rest),
computed with mpmath at 300 bits.  Run: python gen_crmath_tables.py > st_crmath_tables.h
(needs mpmath; the generated header is committed, so builds do not)."""
from __future__ import annotations

import mpmath as mp

mp.mp.prec = 300


def dd(v):
    hi = float(v)
    lo = float(v - mp.mpf(hi))
    return hi, lo


def h(x: float) -> str:
    return float.hex(x)


def split(v, bits):
    """v rounded to `bits` significant bits (as a double), and the rest."""
    e = mp.floor(mp.log(abs(v), 2))
    scale = mp.mpf(2) ** (bits - 1 - e)
    head = mp.nint(v * scale) / scale
    return float(head), v - head


out = []
out.append("// Generated by gen_crmath_tables.py (mpmath, 300 bits): double-double constants of st_crmath.cuh.")
out.append("#pragma once")
out.append("namespace st {")
out.append("namespace crm {")
# log: bins of width 1/128 over m in [0.75, 1.5); R_j ~ 1/c_j (c_j the bin centre), L_j = -log(R_j)
out.append("// log: m in [0.75, 1.5) in 96 bins of 1/128; kLogR[j] ~ 1 / bin centre (1 for the two bins")
out.append("// around 1), kLogL[j] = -log(kLogR[j]) as hi, lo.  Global memory: lanes index them differently.")
rs, ls = [], []
for j in range(96):
    lo_edge = mp.mpf("0.75") + mp.mpf(j) / 128
    if j in (31, 32):
        r = 1.0
    else:
        c = lo_edge + mp.mpf(1) / 256
        r = float(1 / c)
    rs.append(r)
    ls.append(dd(-mp.log(mp.mpf(r))))
out.append("static __device__ const double kLogR[96] = {" + ", ".join(h(r) for r in rs) + "};")
out.append("static __device__ const double kLogL[96][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in ls) + "};")
ln2 = dd(mp.log(2))
out.append("constexpr double kLn2Hi = %s, kLn2Lo = %s;" % (h(ln2[0]), h(ln2[1])))
third = dd(mp.mpf(1) / 3)
out.append("constexpr double kThirdHi = %s, kThirdLo = %s;" % (h(third[0]), h(third[1])))
sixth = dd(mp.mpf(1) / 6)
out.append("constexpr double kSixthHi = %s, kSixthLo = %s;" % (h(sixth[0]), h(sixth[1])))
# pi/2 and pi/64 in three parts: 33 + 33 + 53 bits
for name, v in (("kPio2", mp.pi / 2), ("kPio256", mp.pi / 256)):
    p1, rest = split(v, 33)
    p2, rest = split(rest, 33)
    p3 = float(rest)
    out.append("constexpr double %s1 = %s, %s2 = %s, %s3 = %s;" % (name, h(p1), name, h(p2), name, h(p3)))
out.append("constexpr double kTwoOverPi = %s, k256OverPi = %s;" % (h(float(2 / mp.pi)), h(float(256 / mp.pi))))
# the accurate paths: pi/2 and pi/256 in four parts (33 + 33 + 33 + 53 bits), and the
# Taylor coefficients 1/n (log1p) and 1/n! (sin, cos) as double-double
out.append("// Accurate paths: pi/2 and pi/256 in four parts (33 + 33 + 33 + 53 bits).")
for name, v in (("kPio2q", mp.pi / 2), ("kPio256q", mp.pi / 256)):
    p1, rest = split(v, 33)
    p2, rest = split(rest, 33)
    p3, rest = split(rest, 33)
    p4 = float(rest)
    out.append("constexpr double %s1 = %s, %s2 = %s, %s3 = %s, %s4 = %s;" % (name, h(p1), name, h(p2), name, h(p3),
                                                                         name, h(p4)))
inv = [(0.0, 0.0)] + [dd(mp.mpf(1) / n) for n in range(1, 24)]
out.append("// 1/n, n = 0..23 (entry 0 unused), as hi, lo.")
out.append("static __device__ const double kInvN[24][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in inv) + "};")
fac = [dd(mp.mpf(1) / mp.factorial(n)) for n in range(0, 20)]
out.append("// 1/n!, n = 0..19, as hi, lo.")
out.append("static __device__ const double kInvFact[20][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in fac) + "};")
# sin, cos of j pi / 256, j = 0..64
out.append("// sin(j pi / 256), cos(j pi / 256), j = 0..64, as hi, lo.")
sv = [dd(mp.sin(j * mp.pi / 256)) for j in range(65)]
cv = [dd(mp.cos(j * mp.pi / 256)) for j in range(65)]
out.append("static __device__ const double kSinA[65][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in sv) + "};")
out.append("static __device__ const double kCosA[65][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in cv) + "};")
# the fast sin/cos path: pi/1024 in three parts (33 + 33 + 53 bits) and sin, cos of
# j pi / 1024, j = 0..256
p1, rest = split(mp.pi / 1024, 33)
p2, rest = split(rest, 33)
out.append("// Fast sin/cos path: pi/1024 in three parts (33 + 33 + 53 bits), 1024/pi, and")
out.append("// sin(j pi / 1024), cos(j pi / 1024), j = 0..256, as hi, lo.")
out.append("constexpr double kPio10241 = %s, kPio10242 = %s, kPio10243 = %s;" % (h(p1), h(p2), h(float(rest))))
out.append("constexpr double k1024OverPi = %s;" % h(float(1024 / mp.pi)))
sv = [dd(mp.sin(j * mp.pi / 1024)) for j in range(257)]
cv = [dd(mp.cos(j * mp.pi / 1024)) for j in range(257)]
out.append("static __device__ const double kSinB[257][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in sv) + "};")
out.append("static __device__ const double kCosB[257][2] = {" + ", ".join("{%s, %s}" % (h(a), h(b)) for a, b in cv) + "};")
out.append("}  // namespace crm")
out.append("}  // namespace st")
print("\n".join(out))
