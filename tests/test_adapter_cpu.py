"""The LMT++-side adapter (include/lmtpp/gpu_formulation.h), a FormulationAncestor<double> that
routes elasticity_iso through liblmtg, builds as the reference builds its own code: gnu++98,
-fpermissive, -DDONT_WANT_XML -DDINT, against the reference's headers and include/lmtg.h, linked
with liblmtg.so (tests/adapter_main.cpp holds it through the reference's virtual API, which
fails to compile if any pure virtual is left out).  INTEGRATION.md shows this exact file.

The reference's sources are needed: the test runs where oracle/build_ref.sh found them (it
records their location in oracle/_ref/lmtpp_src) and is skipped elsewhere.  Running the program
needs a GPU and the same build machine, so it is compiled and linked here, not run.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lmtpp", "gpu_formulation.h")


def lmtpp_src():
    p = os.path.join(ROOT, "oracle", "_ref", "lmtpp_src")
    if not os.path.exists(p):
        return None
    src = open(p).read().strip()
    return src if os.path.isdir(os.path.join(src, "include", "formulation")) else None


def test_integration_doc_shows_the_compiled_adapter():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", doc, flags=re.S)
    assert open(HEADER).read() in blocks


def test_adapter_builds_with_reference_flags(tmp_path):
    src = lmtpp_src()
    if src is None:
        pytest.skip("LMTpp sources not present (oracle/build_ref.sh did not run here)")
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    from lmtpp_gb300 import _build
    lib = _build.build()
    exe = str(tmp_path / "adapter")
    cmd = ["g++", "-O1", "-std=gnu++98", "-fpermissive", "-DDONT_WANT_XML", "-DDINT",
           "-I" + os.path.join(src, "include"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "adapter_main.cpp"), "-o", exe,
           "-L" + os.path.dirname(lib), "-llmtg", "-Wl,--allow-shlib-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert os.path.exists(exe)
