"""The device's correctly rounded trajectory functions (st_crmath.cuh),
compiled for the host (tests/crmath_host.cpp gives CUDA's intrinsics their
IEEE meaning) and checked against binary128 without a GPU: on seeded
trajectory arguments every result is the correctly rounded one, and each fast
path's largest error stays at least 2 bits below the bound its rounding test
assumes (the bound is what makes a kept fast result certain)."""
from __future__ import annotations

import platform
import shutil
import subprocess

import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def crmath_host(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path_factory.mktemp("crmath") / "crmath_host"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-frounding-math",
           f"-I{REPO / 'spin-tracking_gb300' / 'csrc'}", str(REPO / "tests" / "crmath_host.cpp"), "-o", str(exe)]
    if platform.machine() in ("x86_64", "i686", "i386"):
        cmd.append("-lquadmath")  # binary128 from libquadmath; aarch64's long double is binary128
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def run(exe, n, seed):
    out = subprocess.run([str(exe), str(n), str(seed)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        key, *rest = line.split()
        if key == "n":
            continue
        res.setdefault(rest[0], {})[key] = float(rest[1])
    return res


@pytest.mark.parametrize("seed", [1, 2])
def test_correctly_rounded_and_within_bounds(crmath_host, seed):
    res = run(crmath_host, 200_000, seed)
    assert set(res) == {"sin", "cos", "acos", "sin_acos", "cos_acos", "log"}
    for name, r in res.items():
        assert r["wrong"] == 0, (name, r)
        assert r["maxerr"] <= r["bound"] - 2.0, (name, r)
    # the accurate paths are rare: ~2^-12 of the trig and acos calls, ~2^-17 of the logs
    assert res["sin"]["slow"] < 200_000 * 2 ** -9
    assert res["acos"]["slow"] < 200_000 * 2 ** -9
    assert res["log"]["slow"] < 400_000 * 2 ** -12
