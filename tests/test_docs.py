"""The Python examples in INTEGRATION.md and README.md name functions that
exist: every `module.attr` / `h.method` they use resolves (CPU, no calls)."""
import os
import re

import pytest

from gisbdw_gb300 import _lib, gnn, graphs, treedepth
import gisbdw_gb300

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODULES = {"gnn": gnn, "graphs": graphs, "h": _lib.Handle, "d": treedepth.DynamicGPU,
           "gisbdw_gb300": gisbdw_gb300}


def python_blocks(name):
    text = open(os.path.join(ROOT, name)).read()
    return re.findall(r"```python\n(.*?)```", text, flags=re.S)


@pytest.mark.parametrize("name", ["INTEGRATION.md", "README.md"])
def test_examples_compile_and_name_existing_functions(name):
    blocks = python_blocks(name)
    assert blocks, name
    for code in blocks:
        compile(code, name, "exec")
        for mod, attr in re.findall(r"\b(gnn|graphs|h|d)\.([A-Za-z_]\w*)\s*\(", code):
            assert hasattr(MODULES[mod], attr), f"{name}: {mod}.{attr}"
        for imported in re.findall(r"from gisbdw_gb300 import ([\w, ]+)", code):
            for item in (x.strip() for x in imported.split(",")):
                assert hasattr(gisbdw_gb300, item) or item in ("gnn", "graphs"), f"{name}: {item}"
