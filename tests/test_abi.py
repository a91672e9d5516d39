"""The C ABI library and the pbig.h archive load and export what the headers
declare (no GPU needed); clients of the legacy API compile and link."""
import ctypes
import os
import re
import subprocess

import pytest

from pbig_gb300 import build, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference project's source tree (awatch/pbig), when a copy is at hand
REF = os.environ.get("PBIG_REFERENCE_DIR", "")


def _declared(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        txt = f.read()
    return sorted(set(re.findall(r"PBIG2_API\s+[\w\s\*]+?\b(pbig2_\w+)\s*\(", txt)))


def test_engine_library_exports_every_declared_symbol():
    names = _declared("pbig2.h")
    assert len(names) >= 15
    lib = ctypes.CDLL(build.build(with_oracle=False)["engine"])
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(engine.EXPORTS) == names


def test_grid_cells_saturates():
    """Cell counts of fine grids over wide ranges do not wrap: in 3-D at range
    2^24, shifts 0, 1 and 2 give 2^72, 2^69 and 2^66 cells."""
    f = engine.lib().pbig2_grid_cells
    big = (1 << 64) - 1
    for shift in (0, 1, 2):
        assert f(1 << 24, shift, 3) == big
    assert f(1 << 24, 0, 3) > 1 << 32
    assert f(1 << 24, 3, 3) == 1 << 63
    assert f(1 << 24, 16, 3) == 256 ** 3
    assert f(0xFFFFFFFF, 0, 2) == 0xFFFFFFFF ** 2
    assert f(0xFFFFFFFF, 0, 3) == big
    assert f(1000, 3, 2) == 125 * 125
    assert f(1000, 31, 3) == 1
    assert f(1 << 24, 22, 3) == 64


def test_legacy_archive_exports_mangled_api():
    a = build.build(with_oracle=False)["legacy"]
    out = subprocess.run(["nm", a], capture_output=True, text=True, check=True).stdout
    for sym in ["_Z9pbig_initjjjjj", "_Z10pbig_checkP8RectInfoP6report", "_Z13pbig_finalizev",
                "_Z11device_initj", "_Z13cuda_finalizev"]:
        assert re.search(r"\bT " + sym + r"\b", out), sym


def test_legacy_client_builds(tmp_path):
    for kind in ("counting", "recording"):
        d = os.path.join(ROOT, "tests", "clients", kind)
        exe = build.compile_client([os.path.join(ROOT, "tests", "clients", "legacy_client.cc"),
                                    os.path.join(d, "report.cc")], str(tmp_path / kind), include_first=[d])
        assert os.path.exists(exe)


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="PBIG_REFERENCE_DIR not set")
def test_reference_example_client_links_unchanged(tmp_path):
    """package/main.cc + package/report.cc of the reference, unmodified,
    against this library (the shim is compiled with the package's report.h)."""
    pkg = os.path.join(REF, "package")
    exe = build.compile_client([os.path.join(pkg, "main.cc"), os.path.join(pkg, "report.cc")],
                               str(tmp_path / "pbig_example"), include_first=[pkg])
    assert os.path.exists(exe)


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="PBIG_REFERENCE_DIR not set")
def test_reference_harness_links_unchanged(tmp_path):
    """src/pbig/main.cc + hybrid.cc + report.cc (check.PBIG) link against the
    library, using its device_init/pbig_* symbols."""
    src = os.path.join(REF, "src", "pbig")
    exe = build.compile_client([os.path.join(src, f) for f in ("main.cc", "hybrid.cc", "report.cc")],
                               str(tmp_path / "check.PBIG"), include_first=[src], std="-std=gnu++98",
                               extra=["-DUSE_PBIG=1"])
    assert os.path.exists(exe)
