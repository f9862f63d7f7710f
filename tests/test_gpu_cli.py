"""The `spintrack` executable (the reference's `main PARAMS OUT`): its format
'A' file is byte-identical to the library's mainAnalysis on the same params
file, for both kernels; without arguments it fails with a usage message."""
from __future__ import annotations

import subprocess

import pytest

from conftest import GOLDEN
import spintrack as st
from spintrack.build import CLI

@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["persistent", "plain"])
def test_cli_writes_the_same_file_as_main_analysis(gpu, tmp_path, kernel):
    params = GOLDEN / "c1_precess.params"
    out_cli, out_lib = tmp_path / "cli.bin", tmp_path / "lib.bin"
    r = subprocess.run([str(CLI), str(params), str(out_cli), "--kernel", kernel], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    st.main_analysis(st.derive(st.parse_params(params)), out_lib,
                     st.KERNEL_PLAIN if kernel == "plain" else st.KERNEL_PERSISTENT)
    assert out_cli.read_bytes() == out_lib.read_bytes()


def test_cli_usage_error_without_arguments(stlib):
    r = subprocess.run([str(CLI)], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "Expects" in (r.stdout + r.stderr)
