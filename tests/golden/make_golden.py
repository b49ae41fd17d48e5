"""Generate tests/golden/golden.npz from the reference itself.

Runs every case of tests/golden/cases.py on the reference compiled from its
own sources with exact rcp/rsqrt (oracle/_ref/libpf_shim.so, built by
``make -C oracle ref``; x86-64 with the reference sources present) and
stores colour and depth of each.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(HERE))

from pixelforge_gb300.abi import PixelForgeLib  # noqa: E402
from cases import cases  # noqa: E402


def main():
    shim = ROOT / "oracle" / "_ref" / "libpf_shim.so"
    if not shim.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    lib = PixelForgeLib(str(shim))
    out = {}
    for name, run in cases().items():
        fr = run(lib)
        out[f"{name}.color"] = fr.color
        out[f"{name}.depth"] = fr.depth if fr.depth is not None else np.zeros((0,), np.float32)
    np.savez_compressed(HERE / "golden.npz", **out)
    print(f"{len(out) // 2} cases -> {HERE / 'golden.npz'}")


if __name__ == "__main__":
    main()
