"""The committed double-double tables of the correctly rounded functions
(st_crmath_tables.h) are exactly what their generator produces (mpmath at 300
bits), and the log table's reduction factors keep |m R - 1| <= 2^-7 over
their bins, the bound the series in st_crmath.cuh is sized for."""
from __future__ import annotations

import re
import subprocess
import sys
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "spin-tracking_gb300" / "csrc"


def test_tables_match_their_generator():
    pytest.importorskip("mpmath")
    out = subprocess.run([sys.executable, str(CSRC / "gen_crmath_tables.py")], capture_output=True, text=True,
                         check=True).stdout
    assert out.strip() == (CSRC / "st_crmath_tables.h").read_text().strip()


def test_log_reduction_bound():
    text = (CSRC / "st_crmath_tables.h").read_text()
    body = re.search(r"kLogR\[96\] = \{([^}]*)\}", text).group(1)
    rs = [float.fromhex(t.strip()) for t in body.split(",")]
    assert len(rs) == 96
    for j, r in enumerate(rs):
        lo, hi = 0.75 + j / 128, 0.75 + (j + 1) / 128
        assert max(abs(lo * r - 1), abs(hi * r - 1)) <= 2.0 ** -7, j
