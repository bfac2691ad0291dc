"""TEST INFRASTRUCTURE ONLY (oracle recipe).

Compiles the reference FIPI sources, unmodified and where they lie
(`$FIPI_REFERENCE_SRC`, else the reference checkout mounted beside this
repository: `../reference/src/{field,cluster,element,linked_list,primitive}.cpp`),
into one shared library per configuration under `oracle/_ref/`:

  g++ -include oracle/_ref/cfg_<name>.hpp -I oracle/ref -I <ref>/src ...

The pre-included header defines the reference's HEAD include guard and
every constant of head.hpp:27-74 for that configuration (the reference
only has compile-time constants), then includes the reference's own
parameter.hpp, then makes `private` `public` so the harness can reach the
objects' state.  FFTW3 (external to the reference, not installed) is
replaced by the FFTW-API shim in this folder.  main.cpp is not compiled;
ref_harness.cpp restates its loop body.

Nothing here runs where the reference sources are absent.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
REPO = ORACLE.parent
OUT = ORACLE / "_ref"
# the reference's sources: $FIPI_REFERENCE_SRC, else the checkout mounted beside
# this repository; where neither exists nothing here runs
REF_SRC = Path(os.environ.get("FIPI_REFERENCE_SRC", str(REPO.parent / "reference" / "src")))
REF_UNITS = ["field.cpp", "cluster.cpp", "element.cpp", "linked_list.cpp", "primitive.cpp"]

sys.path.insert(0, str(REPO))


def reference_available() -> bool:
    return all((REF_SRC / u).is_file() for u in REF_UNITS)


def _g(x: float) -> str:
    return repr(float(x))


def config_header(w) -> str:
    p = w.params()
    assert p.k_n == 0.5 * p.sigma and p.margin == 0.0, "parameter.hpp fixes k_n and margin"
    assert p.r_eq == 5 * p.r_p and p.r_c == 5 * p.r_p, "head.hpp:64-65 fix r_eq, r_c"
    lines = [
        f"/* generated by oracle/ref/build_ref.py for workload {w.name} */",
        "#ifndef HEAD",
        "#define HEAD",
        "#include <fftw3.h>",
        "#include <cmath>", "#include <ctime>", "#include <iostream>", "#include <cstdlib>",
        "#include <fstream>", "#include <sstream>", "#include <cstring>", "#include <string>",
        f"const double pi = {_g(p.pi)};",
        f"const int Nx = {p.nx};", f"const int Ny = {p.ny};", f"const int Nz = {p.nz};",
        f"const double Lx = {_g(p.lx)};", f"const double Ly = {_g(p.ly)};",
        f"const double Lz = {_g(p.lz)};",
        "const double dx = Lx/Nx;", "const double dy = Ly/Ny;", "const double dz = Lz/Nz;",
        f"const double dt = {_g(p.dt)};",
        f"const int t_end = {p.t_end};",
        "const double Bo = 0.0;",
        f"const double sigma = {_g(p.sigma)};",
        f"const double epsilon = {_g(p.epsilon)};",
        f"const double lambda = {_g(p.lambda_)};",
        "const double r_drop = 0.4*Lx;",
        f"const double gravity = {_g(p.gravity)};",
        f"const double rho1 = {_g(p.rho1)};",
        f"const double rho2 = {_g(p.rho2)};",
        f"const double mu = {_g(p.mu)};",
        f"const double A = {_g(p.A)};",
        f"const double mobility = {_g(p.mobility)};",
        f"const double r_p = {_g(p.r_p)};",
        "const double rho_p = rho1;",
        f"const int N_p = {p.n_p};",
        "const double r_eq = 5*r_p;",
        "const double r_c = 5*r_p;",
        "const double r_t = r_p;",
        "const double kt = 0.0;",
        '#include "parameter.hpp"',
        f"const bool switch_particle = {'true' if p.switch_particle else 'false'};",
        f"const bool switch_ch = {'true' if p.switch_ch else 'false'};",
        f"const bool switch_ns = {'true' if p.switch_ns else 'false'};",
        "#define private public",
        "#endif",
        "",
    ]
    return "\n".join(lines)


def lib_path(name: str) -> Path:
    return OUT / f"libfipi_ref_{name}.so"


def build(name: str, force: bool = False) -> Path:
    from fipi_gb300.params import workload

    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REF_SRC}")
    OUT.mkdir(parents=True, exist_ok=True)
    w = workload(name)
    hdr = OUT / f"cfg_{name}.hpp"
    text = config_header(w)
    lib = lib_path(name)
    deps = [HERE / "ref_harness.cpp", HERE / "fftw_shim.c", HERE / "fftw3.h", ORACLE / "fft_c2c.c", Path(__file__)]
    fresh = lib.exists() and all(d.stat().st_mtime <= lib.stat().st_mtime for d in deps)
    if fresh and hdr.exists() and hdr.read_text() == text and not force:
        return lib
    hdr.write_text(text)
    objdir = OUT / f"obj_{name}"
    objdir.mkdir(exist_ok=True)
    common = ["-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-w"]
    objs = []
    cmds = []
    for u in REF_UNITS + ["HARNESS"]:
        src = HERE / "ref_harness.cpp" if u == "HARNESS" else REF_SRC / u
        obj = objdir / (Path(src).stem + ".o")
        cmds.append(["g++", "-std=c++17", *common, "-include", str(hdr), "-I", str(HERE),
                     "-I", str(REF_SRC), "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    for src in [HERE / "fftw_shim.c", ORACLE / "fft_c2c.c"]:
        obj = objdir / (src.stem + ".o")
        cmds.append(["gcc", *common, "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    procs = [subprocess.Popen(c, stderr=subprocess.PIPE, text=True) for c in cmds]
    for c, pr in zip(cmds, procs):
        _, err = pr.communicate()
        if pr.returncode != 0:
            raise RuntimeError("reference build failed: " + " ".join(c) + "\n" + err)
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", str(lib), *map(str, objs), "-lm"],
                   check=True)
    return lib


if __name__ == "__main__":
    names = sys.argv[1:] or ["t16", "t32", "t32_aniso", "t32_2pi", "cfg1_64"]
    for n in names:
        print(build(n))
