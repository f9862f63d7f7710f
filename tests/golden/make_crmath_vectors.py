"""Generate crmath_vectors.txt: arguments and correctly rounded results (mpmath
at 300 bits, rounded to the nearest double) of log, sin, cos and acos over the
argument ranges the trajectory uses: log of 1 - u and of Marsaglia's s in
(0, 1), sin and cos of 2 pi u and of acos(sqrt u), acos of sqrt u; plus edge
arguments (near 1 for log, near the quadrant boundaries for sin and cos, near
0 and 1 for acos).  One line per case: "fn x y" with C99 hex floats.
Run: python tests/golden/make_crmath_vectors.py (needs mpmath)."""
from __future__ import annotations

from pathlib import Path

import mpmath as mp
import numpy as np

mp.mp.prec = 300
rng = np.random.default_rng(7)
n = 400
u = rng.random(n)
v = rng.random(n) * 2 - 1
w = rng.random(n) * 2 - 1
s = u * 0 + (v * v + w * w)
s = s[(s < 1) & (s > 0)]
lines = []


def add(fn, xs, f):
    for x in xs:
        x = float(x)
        y = float(f(mp.mpf(x)))
        lines.append(f"{fn} {x.hex()} {y.hex()}")


ulp1 = np.nextafter(1.0, 0.0)
log_x = np.concatenate([1.0 - u, s, [1.0, ulp1, 1.0 - 2**-40, 1.0 + 2**-40, 0.5, 0.75, 1.5 - 2**-52, 2**-53, 2**-104]])
add("log", log_x, mp.log)
phi = np.arccos(np.sqrt(u))
edges = []
for k in range(5):
    c = k * np.pi / 2
    edges += [c, np.nextafter(c, 0.0), np.nextafter(c, 10.0), c + 1e-9, c - 1e-9]
for j in range(-16, 17):
    edges.append(j * np.pi / 64 + np.pi / 2)
trig_x = np.concatenate([2.0 * np.pi * u, phi, [e for e in edges if e >= 0.0]])
add("sin", trig_x, mp.sin)
add("cos", trig_x, mp.cos)
acos_x = np.concatenate([np.sqrt(u), [0.0, 1.0, ulp1, 2**-53, 1 - 2**-30, 0.5, np.sqrt(0.5)]])
add("acos", acos_x, mp.acos)
(Path(__file__).resolve().parent / "crmath_vectors.txt").write_text("\n".join(lines) + "\n")
print(len(lines), "cases")
