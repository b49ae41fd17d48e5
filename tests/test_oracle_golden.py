"""The CPU oracle against golden vectors of the reference itself.

tests/golden/golden.npz holds colour and depth of every case in
tests/golden/cases.py as rendered by the reference compiled from its own
sources (exact-reciprocal flavour; tests/golden/make_golden.py).  The oracle
must reproduce depth bit for bit and colour bit for bit, except on hosts
whose libm powf may round differently from the x86-64 glibc the goldens were
made with: there the Gouraud-specular cases may differ by one LSB.
"""
import platform
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(HERE))
from cases import cases, uses_host_powf  # noqa: E402

GOLDEN = np.load(HERE / "golden.npz")
CASES = cases()
X86 = platform.machine() in ("x86_64", "AMD64")


def check(name, fr, tol):
    gc, gd = GOLDEN[f"{name}.color"], GOLDEN[f"{name}.depth"]
    assert fr.color.shape == gc.shape
    if gd.size:
        nd = int((fr.depth.view(np.uint32) != gd.view(np.uint32)).sum())
        assert nd == 0, f"{name}: {nd} depth values differ from the reference"
    diff = np.abs(fr.color.astype(np.int32) - gc.astype(np.int32))
    assert int(diff.max()) <= tol, f"{name}: colour differs by {int(diff.max())} on {int((diff > 0).any(-1).sum())} pixels"


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(oracle, name):
    tol = 1 if (uses_host_powf(name) and not X86) else 0
    check(name, CASES[name](oracle), tol)


def test_golden_cases_render_something():
    drawn = [n for n in CASES if n.startswith("kat_") and
             len(np.unique(GOLDEN[f"{n}.color"].reshape(-1, 4), axis=0)) > 1]
    assert len(drawn) == len([n for n in CASES if n.startswith("kat_")])
