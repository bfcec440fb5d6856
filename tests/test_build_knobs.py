"""The build's tuning knob MTJG_BUILD_DEFINES takes -D flags only (anything
else could change the code generation the kernels are measured with)."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "matrix-toolkits-java_gb300"))


def test_build_defines_reject_other_flags(monkeypatch):
    build = importlib.import_module("build")
    monkeypatch.setenv("MTJG_BUILD_DEFINES", "-DMTJG_TILE_NNZ=1152 -O0")
    with pytest.raises(RuntimeError, match="-D flags only"):
        build.build()
