"""The C++ binding of the repository's integration guide (the reference's
`particle` class re-implemented over the C ABI) compiles and links against the
library, with stand-ins for the reference's `coords`, `options` and `Logger`
types."""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent

HARNESS = """#include <cstdint>
#include <cstddef>
#include "spintrack.h"
struct coords { double x, y, z; };
typedef st_options options;
struct Logger {
  void writeSnapshot(double*, coords*, coords*, coords*, int*, size_t*, size_t*, size_t*) {}
};
"""


def test_particle_binding_compiles_and_links(stlib, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    doc = (REPO / "INTEGRATION.md").read_text()
    code = re.search(r"```cpp\n(// particle.h replacement.*?)```", doc, re.S).group(1)
    src = tmp_path / "binding.cpp"
    src.write_text(HARNESS + code.replace('#include "spintrack.h"\n', "") +
                   "int main() { return sizeof(particle) > 0 ? 0 : 1; }\n")
    lib = REPO / "spin-tracking_gb300" / "_build"
    r = subprocess.run([gxx, "-std=c++17", f"-I{REPO / 'include'}", str(src), f"-L{lib}", "-lspintrack",
                        "-o", str(tmp_path / "binding")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
