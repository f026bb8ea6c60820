"""The reference-side binding of INTEGRATION.md section 2 compiles: its C++
snippets, against the reference's own headers and include/ldo.h (syntax and
types only; no link, no GPU).  Skipped where no reference checkout is present."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

DOC = os.path.join(ROOT, "INTEGRATION.md")


def snippets():
    text = open(DOC).read()
    sec = text[text.index("## 2. "):text.index("## 3. ")]
    return re.findall(r"```cpp\n(.*?)```", sec, re.S)


def test_integration_binding_compiles(tmp_path):
    import sys
    sys.path.insert(0, ROOT)
    import __graft_entry__
    ref = __graft_entry__.reference_dir()
    if ref is None:
        pytest.skip("no reference checkout")
    blocks = snippets()
    assert len(blocks) >= 4
    # the first block is a translation unit; the others are statements of a
    # driver function with the reference's parameter object in scope
    body = "\n".join(blocks[1:])
    src = blocks[0] + '''
#include <vector>
#include "LatticeDNAOrigami/parser.hpp"
void driver(parser::InputParameters& params, int n_ladders, int n_temps, uint32_t seed, long long swaps,
            int exchange_interval) {
''' + body + "\n}\n"
    path = tmp_path / "gpu_simulation.cpp"
    path.write_text(src)
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle", "ref", "stubs"), "-I" + os.path.join(ref, "include"),
           "-I" + os.path.join(ref, "include", "LatticeDNAOrigami"), str(path)]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
