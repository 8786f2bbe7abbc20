"""PhysUnits3D of the C++ shim (plb/physunits_gpu.h) against the reference's
src/physunits.h:32-93: every conversion, bit for bit (tests/physunits_eval.cpp
compiled against either header).  The reference's flow parameters come from
Palabos' IncomprFlowParam, restated in the harness stand-ins
(oracle/ref_harness/include/palabos3D.h) and in the shim alike."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "physunits_eval.cpp"
SHIM = ROOT / "lbdemcoupling-public_gb300" / "plb"


def _run(tmp_path, name, includes):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / name
    cmd = [cxx, "-O2", "-std=c++11", "-ffp-contract=off", "-w", *[f"-I{p}" for p in includes], str(SRC), "-o",
           str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()


def _shim_lines(tmp_path):
    # physunits_gpu.h stands in under the reference's header name
    inc = tmp_path / "shim_inc"
    inc.mkdir()
    (inc / "physunits.h").write_text(f'#include "{SHIM / "physunits_gpu.h"}"\n')
    return _run(tmp_path, "units_shim", [inc])


def test_shim_conversions_are_consistent(tmp_path):
    vals = {}
    for ln in _shim_lines(tmp_path)[:200]:
        k, v = ln.split()
        vals.setdefault(k, []).append(float.fromhex(v) if k != "getLbSteps" else int(v))
    # lattice units (first system): deltaX = 1, deltaT = 1, positions offset by 1/2
    assert vals["deltaX"][0] == 1.0 and vals["deltaT"][0] == 1.0
    assert vals["getLbPosition"][1] == 0.5 and vals["getPhysPosition"][1] == 1.5
    assert vals["getLbLength"][3] == 12.5 and vals["getPhysForce"][3] == 12.5


def test_shim_matches_reference_physunits(tmp_path):
    from oracle import ref_build
    if not ref_build.reference_present():
        pytest.skip("reference tree not present")
    ref = _run(tmp_path, "units_ref", [ROOT / "oracle" / "ref_harness" / "include", ref_build.REFERENCE / "src"])
    shim = _shim_lines(tmp_path)
    assert len(ref) == len(shim) > 500
    for a, b in zip(ref, shim):
        assert a == b
