"""In-tree build of libpixelforge_gb300.so (sm_103a).

    python -m pixelforge_gb300.build

compiles the CUDA units of csrc/ with nvcc for sm_103a only and csrc/pf_host.cpp
with the host C++ compiler, in parallel, and links them with the static CUDA
runtime into pixelforge_gb300/libpixelforge_gb300.so.  Flags that matter for
parity: -fmad=false (device) and -ffp-contract=off (host) keep every
multiply and add separately rounded, as in the reference's AVX2 build.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libpixelforge_gb300.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and (Path(c) / "bin" / "nvcc").exists():
            return Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


CUDA_UNITS = ("pf_kernels.cu", "pf_noalloc.cu", "pf_grad.cu")


def _sources():
    return [*(CSRC / u for u in CUDA_UNITS), CSRC / "pf_host.cpp", CSRC / "pf_layout.h", CSRC / "pf_device.h",
            CSRC / "pf_common.cuh", CSRC / "pf_pixfmt.h", INCLUDE / "pixelforge.h", INCLUDE / "pixelforge_grad.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    cobjs = [BUILD / (u.rsplit(".", 1)[0] + ".o") for u in CUDA_UNITS]
    hobj = BUILD / "pf_host.o"
    ccmds = [[nvcc, *ARCH, "-lineinfo", "-O3", "-fmad=false", "-std=c++17", "-Xptxas", "-v",
              "-Xcompiler", "-fPIC,-fvisibility=hidden", *inc, "-c", str(CSRC / u), "-o", str(o)]
             for u, o in zip(CUDA_UNITS, cobjs)]
    cxx = os.environ.get("CXX", "g++")
    hcmd = [cxx, "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fvisibility=hidden",
            "-Wall", "-Wno-unused-function", *inc, f"-I{cuda / 'include'}", "-c", str(CSRC / "pf_host.cpp"),
            "-o", str(hobj)]
    procs = [(cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for cmd in (*ccmds, hcmd)]
    logs = []
    for cmd, p in procs:
        out, _ = p.communicate()
        logs.append(out)
        if p.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{out}")
    (BUILD / "ptxas.log").write_text("\n".join(logs[:len(CUDA_UNITS)]))
    libdir = cuda / "lib64"
    if not (libdir / "libcudart_static.a").exists():
        alt = cuda / "targets" / ("sbsa-linux" if os.uname().machine == "aarch64" else "x86_64-linux") / "lib"
        libdir = alt if (alt / "libcudart_static.a").exists() else libdir
    tmp = LIB.with_suffix(".so.tmp")
    lcmd = [cxx, "-shared", "-o", str(tmp), str(hobj), *map(str, cobjs), f"-L{libdir}", "-lcudart_static",
            "-lrt", "-ldl", "-lpthread", "-Wl,-Bsymbolic"]
    r = subprocess.run(lcmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(lcmd)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(logs[0])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
