"""Generate the golden fixtures in tests/golden/ by running the REFERENCE build.

Requires the reference sources (the oracle recipe's REF, or $SPINTRACK_REF)
and builds them with `make -C oracle ref` (the reference's own .cpp files
compiled unchanged against oracle/ref_stubs).  Writes, per case:
  <case>.params          the params.txt the reference read
  <case>.bin             its output format 'A' file
and probe vectors (C99 hex floats) from oracle/_ref/ref_probe:
  probe_init_<dist>.txt, probe_draws.txt, probe_events.txt, probe_dop.txt,
  probe_rk45.txt, probe_magnus.txt, probe_rk45q.txt, probe_rkf45.txt,
  probe_rkf45q.txt (single segments of every stepper),
  probe_spectrum.txt, probe_spectrum_m.txt (integratorType 6: Floquet
  frequencies and each particle's noise-spectrum aggregator after a window)
Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
ORACLE = REPO / "oracle"
# where the reference sources are: $SPINTRACK_REF, else the oracle recipe's default
REF_ARGS = [f"REF={os.environ['SPINTRACK_REF']}"] if os.environ.get("SPINTRACK_REF") else []

BASE = {
    "L": "0.07, 0.1, 0.4", "B0": "3e-6, 0, 0", "E": "0, 0, 75e5", "gamma": "-2.038e8", "m": "1.20239e-26",
    "rtol": "1e-12", "atol": "1e-12", "h": "1e-3", "hmax": "1", "hmin": "1e-8", "t0": "0", "seed": "0",
    "integratorType": "0",
}
G_FULL = {"Gx": "1.3e-9, -0.4e-9, 1e-9", "Gy": "0.2e-9, 0.7e-9, -1.1e-9", "Gz": "-0.5e-9, 0.9e-9, 0.3e-9"}

# Every case sets every key it depends on: the reference's code defaults differ
# from its README (E, yi, diffuse, tf).
CASES = {
    # config 1 as written (CPU-runnable plain method), fewer particles / windows
    "c1_literal": dict(numParticles="24", dist="C", V="5", gravity="true", diffuse="0", gas_coll="false",
                       Gx="0, 0, 1e-9", yi="1, 0, 0", tf="0.5", ioutInt="0.05"),
    "c1_precess": dict(numParticles="24", dist="C", V="5", gravity="true", diffuse="0", gas_coll="false",
                       Gx="0, 0, 1e-9", yi="0, 0, 1", tf="0.5", ioutInt="0.05", seed="3"),
    # config-2 physics (MB at 4.2 K, diffuse 0.1, full gradient tensor), gas off
    "m42_diffuse": dict(numParticles="24", dist="M", T="4.2", gas_coll="false", diffuse="0.1", gravity="true",
                        yi="0, 0, 1", tf="0.2", ioutInt="0.05", seed="11", **G_FULL),
    # gas collisions at 0.4 K (tc = 0.21 ms), MB redraw
    "m04_gas": dict(numParticles="24", dist="M", T="0.4", gas_coll="true", diffuse="0.3", gravity="true",
                    yi="0, 0, 1", tf="0.3", ioutInt="0.05", seed="7", **G_FULL),
    # gas collisions with the 'C' (fixed speed, isotropic) redraw
    "c_gas": dict(numParticles="16", dist="C", V="5", T="0.4", gas_coll="true", diffuse="0.5", gravity="true",
                  yi="0, 1, 0", tf="0.3", ioutInt="0.1", seed="5", **G_FULL),
    # spin dressing pulse along z, w = 2 pi 1 kHz, hmax 1e-4
    "pulse": dict(numParticles="8", dist="C", V="5", gas_coll="false", diffuse="0.5", gravity="true",
                  yi="0, 0, 1", a="5e-6", w="6283.185307179586", hmax="1e-4", tf="0.02", ioutInt="0.01",
                  **G_FULL),
    # RK45 with its first-stage quirk
    "rk45": dict(numParticles="4", dist="C", V="5", gas_coll="false", diffuse="0", gravity="true",
                 yi="0, 0, 1", integratorType="1", tf="0.004", ioutInt="0.001", **G_FULL),
    # integratorType 2-5 (src/integrator.cpp:339-722)
    "magnus": dict(numParticles="6", dist="M", T="4.2", gas_coll="false", diffuse="0.2", gravity="true",
                   yi="0, 0, 1", integratorType="2", a="5e-6", w="6283.185307179586", hmax="1e-4", tf="0.02",
                   ioutInt="0.005", seed="12", **G_FULL),
    "rk45q": dict(numParticles="6", dist="M", T="4.2", gas_coll="false", diffuse="0.2", gravity="true",
                  yi="0, 0, 1", integratorType="3", rtol="1e-10", tf="0.02", ioutInt="0.005", seed="13", **G_FULL),
    "rkf45": dict(numParticles="6", dist="C", V="5", gas_coll="false", diffuse="0.2", gravity="true",
                  yi="0, 1, 0", integratorType="4", rtol="1e-3", tf="0.02", ioutInt="0.005", seed="14", **G_FULL),
    "rkf45q": dict(numParticles="6", dist="C", V="5", T="0.4", gas_coll="true", diffuse="0.2", gravity="true",
                   yi="0, 0, 1", integratorType="5", rtol="1e-6", tf="0.02", ioutInt="0.005", seed="15", **G_FULL),
    # Magnus carrying its step size across windows, gas collisions, no gravity
    "magnus_keep": dict(numParticles="6", dist="C", V="5", T="0.4", gas_coll="true", diffuse="0.3", gravity="false",
                        yi="1, 0, 0", integratorType="2", keepStepSize="true", tf="0.03", ioutInt="0.01", seed="21",
                        **G_FULL),
    # RKF45's error estimate is its whole fourth-order increment: at rtol 1e-12
    # the step shrinks below hmin at once (-1)
    "rkf45_hmin": dict(numParticles="4", dist="C", V="5", gas_coll="false", diffuse="0", gravity="true",
                       yi="0, 0, 1", integratorType="4", tf="0.01", ioutInt="0.005", **G_FULL),
    # a fixed step of types 2-5 never tests the segment end: nmax attempts, then -2
    "magnus_fixed": dict(numParticles="4", dist="C", V="5", gas_coll="false", diffuse="0", gravity="true",
                         yi="0, 0, 1", integratorType="2", fixedStepSize="true", h="1e-4", nmax="40", tf="0.01",
                         ioutInt="0.005", **G_FULL),
    "nograv": dict(numParticles="16", dist="C", V="5", gas_coll="false", diffuse="0", gravity="false",
                   yi="0, 0, 1", tf="0.3", ioutInt="0.05", **G_FULL),
    "keep": dict(numParticles="8", dist="M", T="4.2", gas_coll="false", diffuse="0", gravity="true", yi="0, 0, 1",
                 keepStepSize="true", tf="0.2", ioutInt="0.05", **G_FULL),
    "fixed": dict(numParticles="6", dist="C", V="5", gas_coll="false", diffuse="0", gravity="true", yi="0, 0, 1",
                  fixedStepSize="true", h="2e-4", tf="0.1", ioutInt="0.05", **G_FULL),
    # failure path: more than nmax attempts in a segment stops the particle (-1)
    "nmax": dict(numParticles="8", dist="M", T="4.2", gas_coll="false", diffuse="0", gravity="true", yi="0, 0, 1",
                 nmax="3", tf="0.1", ioutInt="0.05", **G_FULL),
    # integratorType outside 0-6: trajectory only
    "traj": dict(numParticles="12", dist="C", V="5", gas_coll="false", diffuse="0.2", gravity="true",
                 yi="0, 0, 1", integratorType="-1", tf="1.0", ioutInt="0.1"),
    # the reference's end-to-end output test (tests/output_tests.cpp:20-82)
    "output_test": dict(numParticles="3", B0="3e-6, 0, 0", E="0, 0, 0", T="0.4", tf="0.2", t0="0", rtol="1e-12",
                        atol="1e-12", h="1e-5", yi="0, 0, 1", gravity="false", ioutInt="0.05",
                        integratorType="0", dist="C", V="5", gas_coll="true", diffuse="1.0"),
    # edge cases: no particles; a block-ragged particle count
    "empty": dict(numParticles="0", dist="C", V="5", gas_coll="false", diffuse="0", gravity="true",
                  yi="0, 0, 1", tf="0.1", ioutInt="0.05"),
    "ragged": dict(numParticles="130", numPerGPUBlock="128", dist="M", T="4.2", gas_coll="false", diffuse="0.1",
                   gravity="true", yi="0, 0, 1", tf="0.1", ioutInt="0.05", seed="99", **G_FULL),
}


def params_text(case: dict) -> str:
    d = dict(BASE)
    d.update(case)
    return "".join(f"{k}, {v}\n" for k, v in d.items())


def run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    return r


def main() -> int:
    r = run(["make", "-C", str(ORACLE), "ref", *REF_ARGS])
    if r.returncode:
        print(r.stdout, r.stderr, file=sys.stderr)
        return 1
    exe = ORACLE / "_ref" / "spintrack_ref"
    probe = ORACLE / "_ref" / "ref_probe"
    for name, case in CASES.items():
        p = HERE / f"{name}.params"
        p.write_text(params_text(case))
        out = HERE / f"{name}.bin"
        r = run([str(exe), str(p), str(out)])
        # the reference aborts in ~BinaryLogger (double free, src/logger.cpp:40-43)
        # after the file is complete; accept that when the size is exact
        n = int(case.get("numParticles", "1000"))
        print(f"{name}: rc={r.returncode} size={out.stat().st_size} (n={n})")
    # ---- probe vectors
    pp = HERE / "probe.params"
    pp.write_text(params_text(dict(numParticles="6", dist="C", V="5", gas_coll="true", T="0.4", diffuse="0.5",
                                   gravity="true", yi="0, 0, 1", tf="0.2", ioutInt="0.05", seed="17", **G_FULL)))
    pm = HERE / "probe_m.params"
    pm.write_text(params_text(dict(numParticles="6", dist="M", T="4.2", gas_coll="true", diffuse="0.1",
                                   gravity="true", yi="0, 0, 1", tf="0.2", ioutInt="0.05",
                                   seed="-3", **G_FULL)))
    (HERE / "probe_init_C.txt").write_text(run([str(probe), "init", str(pp)]).stdout)
    (HERE / "probe_init_M.txt").write_text(run([str(probe), "init", str(pm)]).stdout)
    (HERE / "probe_draws.txt").write_text(run([str(probe), "draws", str(pp), "24"]).stdout)
    (HERE / "probe_events.txt").write_text(run([str(probe), "events", str(pp), "40"]).stdout +
                                           run([str(probe), "events", str(pm), "40"]).stdout)
    # single-segment steppers: free precession (tests/integrator_validation.cpp:12-46)
    # and a moving particle in the full field
    pf = HERE / "probe_free.params"
    pf.write_text(params_text(dict(numParticles="1", B0="3e-6, 0, 0", E="0, 0, 0", gravity="false", h="1e-4",
                                   tf="1.2", t0="0.1")))
    seg_cases = [
        (pf, ["0.1", "1.2", "0", "0", "1", "0", "0", "0", "0", "0", "0", "1e-4", "0"]),
        (pp, ["0.0", "0.013", "0", "0", "1", "0.01", "-0.02", "0.05", "3", "-2", "1", "1e-3", "0"]),
        (pp, ["0.25", "0.3", "0.6", "0.0", "0.8", "-0.03", "0.04", "-0.15", "-1.5", "4", "0.5", "2e-5", "0"]),
    ]
    lines_dop, lines_rk = [], []
    for pf_, args in seg_cases:
        lines_dop.append(f"{pf_.name} {' '.join(args)} | " + run([str(probe), "dop", str(pf_), *args]).stdout.strip())
    rk_cases = [
        (pf, ["0.1", "0.1005", "0", "0", "1", "0", "0", "0", "0", "0", "0", "1e-5", "0"]),
        (pp, ["0.0", "0.0004", "0", "0", "1", "0.01", "-0.02", "0.05", "3", "-2", "1", "1e-5", "0"]),
    ]
    for pf_, args in rk_cases:
        lines_rk.append(f"{pf_.name} {' '.join(args)} | " + run([str(probe), "rk45", str(pf_), *args]).stdout.strip())
    (HERE / "probe_dop.txt").write_text("\n".join(lines_dop) + "\n")
    (HERE / "probe_rk45.txt").write_text("\n".join(lines_rk) + "\n")
    # integratorType 2-5 over single segments: free precession, a moving
    # particle in the full field, and the same with the dressing pulse
    pd = HERE / "probe_pulse.params"
    pd.write_text(params_text(dict(numParticles="6", dist="C", V="5", gas_coll="false", gravity="true",
                                   yi="0, 0, 1", a="5e-6", w="6283.185307179586", hmax="1e-4", tf="0.2",
                                   ioutInt="0.05", seed="17", **G_FULL)))
    ext_segs = [
        (pf, ["0.1", "0.1005", "0", "0", "1", "0", "0", "0", "0", "0", "0", "1e-5", "0"]),
        (pp, ["0.0", "0.0004", "0", "0", "1", "0.01", "-0.02", "0.05", "3", "-2", "1", "1e-5", "0"]),
        (pd, ["0.25", "0.2504", "0.6", "0.0", "0.8", "-0.03", "0.04", "-0.15", "-1.5", "4", "0.5", "2e-5", "0"]),
    ]
    for cmd in ("magnus", "rk45q", "rkf45", "rkf45q"):
        lines = []
        for pf_, args in ext_segs:
            # RKF45 (and its quaternion form at rtol 1e-12) fails with -1; with a
            # loose tolerance (params differing only in rtol) it takes steps
            variants = [pf_]
            if cmd in ("rkf45", "rkf45q"):
                pz = HERE / f"{pf_.stem}_rtol3.params"
                pz.write_text(pf_.read_text().replace("rtol, 1e-12", "rtol, 1e-3"))
                variants.append(pz)
            for pz in variants:
                lines.append(f"{pz.name} {' '.join(args)} | " + run([str(probe), cmd, str(pz), *args]).stdout.strip())
        (HERE / f"probe_{cmd}.txt").write_text("\n".join(lines) + "\n")
    spectrum_probes(probe)
    print("probes written")
    return 0


# integratorType 6 (the noise spectrum): a dressed run with gas, diffuse walls,
# the full gradient tensor and a test noise field, and a Maxwell-Boltzmann run
# with specular walls and no pulse amplitude (the Floquet period still comes
# from w).  The noise amplitudes and frequencies follow the params file on the
# probe's command line (the reference's parser has no keys for them).
SPECTRUM_CASES = {
    "probe_spectrum": (dict(numParticles="8", dist="C", V="5", gas_coll="true", T="0.4", diffuse="0.3",
                            gravity="true", yi="0, 0, 1", a="5e-6", w="6283.185307179586", h="1e-5", tf="0.02",
                            ioutInt="0.01", integratorType="6", seed="5", **G_FULL),
                       ["1e-9", "2e-9", "0", "300", "700", "0"]),
    "probe_spectrum_m": (dict(numParticles="8", dist="M", T="4.2", gas_coll="false", diffuse="0", gravity="true",
                              yi="0, 0, 1", a="0", w="3141.592653589793", h="2e-5", tf="0.01", ioutInt="0.01",
                              integratorType="6", seed="11", **G_FULL),
                         ["0", "0", "0", "0", "0", "0"]),
}


def spectrum_probes(probe) -> None:
    for name, (case, noise) in SPECTRUM_CASES.items():
        p = HERE / f"{name}.params"
        p.write_text(params_text(case))
        out = run([str(probe), "spectrum", str(p), *noise]).stdout
        (HERE / f"{name}.txt").write_text("noise " + " ".join(noise) + "\n" + out)


if __name__ == "__main__":
    if sys.argv[1:] == ["spectrum"]:  # only the integratorType 6 probes
        spectrum_probes(ORACLE / "_ref" / "ref_probe")
        sys.exit(0)
    sys.exit(main())
