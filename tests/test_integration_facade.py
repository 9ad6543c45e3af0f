"""The C++ facade a maintainer adds (the first ```cpp block of INTEGRATION.md)
compiles against include/phelm_gb300.h, so the document and the C ABI cannot
drift apart.  Syntax/type check only (no GPU, no link)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_facade_compiles(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", doc, re.S)
    assert blocks, "no C++ block in INTEGRATION.md"
    src = tmp_path / "facade.cpp"
    src.write_text(blocks[0] + "\nint main() { return 0; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
