"""The reference GPU-kernel comparator (oracle/ref_gpu.py) lays out the
reference's structs by size; those sizes must be the reference build's
(checked on CPU against ref_probe, which is compiled from the reference
sources), and on a GPU the reference's own kernels, run through the cubin,
reproduce the reference CPU build's golden output within the golden bars
(they are the reference's GPU path of the same algorithm)."""
from __future__ import annotations

import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, REPO

sys.path.insert(0, str(REPO / "oracle"))
import ref_gpu  # noqa: E402

PROBE = REPO / "oracle" / "_ref" / "ref_probe"


def test_struct_sizes_match_the_reference_build():
    if not PROBE.exists():
        pytest.skip("reference build absent")
    out = subprocess.run([str(PROBE), "sizes", str(GOLDEN / "c1_precess.params")], capture_output=True, text=True,
                         check=True).stdout.split()
    sizes = {out[k]: int(out[k + 1]) for k in range(0, len(out), 2)}
    assert sizes == ref_gpu.SIZES
    assert [s for _, s in ref_gpu.ARRAYS] == [24] * 5 + [8] * 6 + [48, 8, 8, 8, 4, 4, 1, 1, 1, 2600]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c1_precess", "m42_diffuse"])
def test_reference_gpu_kernel_reproduces_the_golden_run(gpu, case):
    if not ref_gpu.available():
        pytest.skip("reference GPU cubin absent")
    import spintrack as st
    from spintrack.formats import read_format_a
    opt = st.derive(st.parse_params(GOLDEN / f"{case}.params"))
    secs, got = ref_gpu.RefGPU().run(opt, ref_gpu.windows_of(opt))
    _, snaps = read_format_a(GOLDEN / f"{case}.bin")
    ref = snaps[-1]
    same = np.all([got[f] == ref[f] for f in ("fail", "n_coll", "n_bounce", "n_steps")], axis=0)
    print(f"{case}: {same.sum()} of {len(same)} particles with the golden counts; {secs * 1e3:.1f} ms")
    assert same.mean() >= 0.9
    m = same & ~np.isnan(ref["S"][:, 0])
    assert np.max(np.abs(got["S"][m] - ref["S"][m])) <= 1e-8
