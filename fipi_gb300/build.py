"""Build of libfipi_gb300.so (the C-ABI library) for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
`fipi_gb300/_build/libfipi_gb300.so` (in-tree, git-ignored).  The particle
unit is compiled with -fmad=false so its FP64 arithmetic rounds exactly as
the reference's (no fused multiply-add).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libfipi_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "capi.cu": [],
    "fields.cu": [],
    "adjoint.cu": [],
    "particles.cu": ["-fmad=false"],
    "vtk.cu": ["-Xcompiler", "-ffp-contract=off"],
    "initial.cu": ["-Xcompiler", "-ffp-contract=off"],
    "probe.cu": [],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise FileNotFoundError("nvcc not found")
    return cand


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(SRC.glob("*")) + [REPO / "include" / "fipi.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    if not force and not _stale(LIB):
        return LIB
    OUT.mkdir(exist_ok=True)
    cc = nvcc()
    common = [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(REPO / "include"), *(extra or [])]
    if verbose:
        common += ["-Xptxas", "-v"]
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = OUT / (Path(unit).stem + ".o")
        cmd = [cc, *common, *flags, "-c", str(SRC / unit), "-o", str(obj)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out)
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    tmp = OUT / (LIB.name + f".tmp{os.getpid()}")
    subprocess.run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
