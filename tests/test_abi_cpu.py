"""The C ABI library builds, loads and exports every symbol include/lbdem_gpu.h
declares; argument checks run before any device work, so they are testable
without a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "lbdem_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbdem_[a-z_]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ("lbdem_create", "lbdem_destroy", "lbdem_set_particles", "lbdem_collide_and_stream",
                 "lbdem_get_forces", "lbdem_get_field", "lbdem_cycle", "lbdem_mass"):
        assert must in names


def test_library_exports_every_declared_symbol(lbdem_lib):
    lib = lbdem_lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) == set(lbdem_lib.SIGNATURES), "ctypes signatures out of date"


def test_config_struct_matches_header(lbdem_lib):
    lib = lbdem_lib.load()
    cfg = lbdem_lib.Config()
    lib.lbdem_config_default(C.byref(cfg))
    assert (cfg.nx, cfg.ny, cfg.nz) == (32, 32, 32)
    assert list(cfg.periodic) == [1, 1, 1]
    assert cfg.omega == 1.0 and cfg.max_particles == 1024 and cfg.max_tag == 1 << 20
    assert cfg.max_radius == 16.0


@pytest.mark.parametrize("cname,pyname", [("lbdem_config", "Config"), ("lbdem_pressure_drop", "PressureDrop"),
                                           ("lbdem_domain", "Domain"), ("lbdem_batch_config", "BatchConfig")])
def test_struct_layout_matches_c_compiler(lbdem_lib, tmp_path, cname, pyname):
    """ctypes field offsets and sizes equal the C compiler's offsetof/sizeof."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    st = getattr(lbdem_lib, pyname)
    fields = [f[0] for f in st._fields_]
    src = tmp_path / "probe.c"
    body = "".join(f'printf("%zu\\n", offsetof({cname}, {f}));' for f in fields)
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "lbdem_gpu.h"\n'
                   f'int main(void){{{body} printf("%zu\\n", sizeof({cname})); return 0;}}\n')
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [getattr(st, f).offset for f in fields] + [C.sizeof(st)]
    assert got == want


@pytest.mark.parametrize("field,value", [("nx", 0), ("omega", 2.0), ("omega", 0.0), ("precision", 7),
                                         ("max_tag", 1 << 25), ("max_radius", -1.0), ("max_particles", -1)])
def test_create_rejects_bad_config(lbdem_lib, field, value):
    lib = lbdem_lib.load()
    cfg = lbdem_lib.Config()
    lib.lbdem_config_default(C.byref(cfg))
    setattr(cfg, field, value)
    h = C.c_void_p()
    assert lib.lbdem_create(C.byref(cfg), C.byref(h)) == 1
    assert not h.value


def test_null_handle_calls_fail_cleanly(lbdem_lib):
    lib = lbdem_lib.load()
    assert lib.lbdem_collide_and_stream(None) == 1
    assert lib.lbdem_destroy(None) == 1
    assert lib.lbdem_synchronize(None) == 1
    assert lib.lbdem_status_string(5) == b"device error word set"
    assert lib.lbdem_last_error(None) == b"null handle"


def test_no_device_is_an_error_not_a_fallback(lbdem_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(lbdem_lib.LbdemError) as ei:
        lbdem_lib.Lattice(8, 8, 8, 1.0)
    assert ei.value.status == 6


def test_division_by_invariant_divisor():
    """The multiply-high division the collide kernel uses to split a segment index
    (DivMagic in csrc/lbdem_internal.h): for d >= 2, s = ceil(log2 d) - 1,
    m = ceil(2^(32+s) / d) fits in 32 bits and (n * m) >> (32 + s) == n // d for
    every n < 2^31; checked here at the multiples of d and their neighbours."""
    import numpy as np
    rng = np.random.default_rng(3)
    divisors = list(range(2, 600)) + [1023, 1024, 1025, 4095, 4096, 65535, 65536, 65537, 2**20 + 7, 2**30, 2**31 - 1]
    for d in divisors:
        l = 0
        while (1 << l) < d:
            l += 1
        s = l - 1
        m = ((1 << (32 + s)) + d - 1) // d
        assert m < 2**32
        ks = np.unique(np.concatenate([np.arange(0, 50), rng.integers(0, (2**31 - 1) // d + 1, 200),
                                       [(2**31 - 1) // d]]))
        for k in ks:
            for n in (int(k) * d - 1, int(k) * d, int(k) * d + 1, int(k) * d + d - 1):
                if 0 <= n < 2**31:
                    assert ((n * m) >> 32) >> s == n // d, (d, n)


def test_integration_binding_snippet_compiles():
    """The C++ binding a maintainer adds on the reference side (tests/integration_binding.cpp,
    quoted in INTEGRATION.md) compiles against the C ABI header, the PhysUnits3D shim and
    the LIGGGHTS stand-in of the example programs (its templates instantiated with double)."""
    import shutil
    import subprocess
    from pathlib import Path
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    root = Path(__file__).resolve().parents[1]
    pkg = root / "lbdemcoupling-public_gb300"
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", f"-I{root / 'include'}", f"-I{pkg / 'plb'}",
                        f"-I{pkg / 'examples'}", str(root / "tests" / "integration_binding.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
