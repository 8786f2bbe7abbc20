"""The reference's own case-driver lines compile, unchanged, against the C++ shim
(lbdemcoupling-public_gb300/plb/lbdem_plb.h).

From examples/sedimentingSphere/sedimentingSphere.cpp of the reference tree
(read at test time; the test is skipped where the tree is absent) the test
takes, as text: the DYNAMICS macro (:39), the lattice set-up lines
defineDynamics / periodicity().toggleAll / initialize (:181, :183, :196) and
the whole coupling loop (:212-238: setSpheresOnLattice, collideAndStream,
getForcesFromLattice(lattice, wrapper, units), wrapper.run, the MLUPS log),
and compiles them into a program whose lattice is a plb::GpuLattice3D, whose
wrapper is the LIGGGHTS stand-in of the example programs, and whose remaining
Palabos names come from tests/driver_standin.h.  The same is done for the
coupling calls of examples/benchmark/benchmark.cpp and
examples/showcaseRectChannel/showcaseRectChannel.cpp (setSpheresOnLattice with
initWithVel, getForcesFromLattice).
"""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "lbdemcoupling-public_gb300"


def _reference():
    from oracle import ref_build
    if not ref_build.reference_present():
        pytest.skip("reference tree not present")
    return ref_build.REFERENCE


def _loop(text, head):
    """The statement starting at `head` through its matching closing brace."""
    i = text.index(head)
    depth, j = 0, text.index("{", i)
    while True:
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[i:j + 1]
        j += 1


def _line(text, start):
    return next(l for l in text.splitlines() if l.strip().startswith(start)).strip()


PROGRAM = """#include <ctime>
#include <vector>
#include "driver_standin.h"
#include "dem_standin.h"
#include "lbdem_plb.h"
#include "physunits_gpu.h"
using namespace plb;
using namespace std;
typedef double T;
#define DESCRIPTOR descriptors::D3Q19Descriptor
{dynamics}
template <class Lattice>
void writeVTK(Lattice&, IncomprFlowParam<T> const&, PhysUnits3D<T> const&, plint) {{}}
int run_driver() {{
    IncomprFlowParam<T> parameters(0.6);
    PhysUnits3D<T> units(1.0, 1.0, 0.1 / 3.0, 20, 20, 40, 1, 1.0, 1.0);
    LiggghtsCouplingWrapper wrapper;
    const plint maxSteps = 3, vtkSteps = 1000, logSteps = 1000, demSubsteps = 10;
    bool initWithVel = true;
    (void)initWithVel;
    GpuLattice3D lattice(20, 20, 40, new DYNAMICS);
    {setup}
    clock_t start = clock();
    {loop}
    return 0;
}}
"""


def _compile(tmp_path, src_text):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "driver.cpp"
    src.write_text(src_text)
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wno-unused-variable",
                        f"-I{ROOT / 'include'}", f"-I{PKG / 'plb'}", f"-I{PKG / 'examples'}", f"-I{ROOT / 'tests'}",
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_sedimenting_sphere_driver_lines_compile(tmp_path):
    ref = _reference()
    text = (ref / "examples" / "sedimentingSphere" / "sedimentingSphere.cpp").read_text()
    dynamics = _line(text, "#define DYNAMICS")
    setup = "\n    ".join([_line(text, "defineDynamics(lattice"), _line(text, "lattice.periodicity()"),
                           _line(text, "lattice.initialize()")])
    loop = _loop(text, "for (plint iT=0; iT<maxSteps; ++iT)")
    assert "getForcesFromLattice(lattice,wrapper,units);" in loop
    assert "setSpheresOnLattice(lattice,wrapper,units,false);" in loop
    _compile(tmp_path, PROGRAM.format(dynamics=dynamics, setup=setup, loop=loop))


@pytest.mark.parametrize("case", ["benchmark/benchmark.cpp", "showcaseRectChannel/showcaseRectChannel.cpp"])
def test_other_drivers_coupling_calls_compile(tmp_path, case):
    ref = _reference()
    text = (ref / "examples" / case).read_text()
    calls = [l.strip() for l in text.splitlines()
             if re.match(r"\s*(setSpheresOnLattice|getForcesFromLattice)\(lattice", l)]
    assert len(calls) == 2
    loop = "for (plint iT=0; iT<maxSteps; ++iT) {\n      " + "\n      ".join(calls[:1] + ["lattice.collideAndStream();"] +
                                                             calls[1:]) + "\n    }"
    dyn = _line(text, "#define DYNAMICS")
    base = [l.strip() for l in text.splitlines() if l.strip().startswith("#define BASEDYNAMICS")]
    _compile(tmp_path, PROGRAM.format(dynamics="\n".join(base + [dyn]), setup=_line(text, "defineDynamics(lattice"),
                                      loop=loop))
