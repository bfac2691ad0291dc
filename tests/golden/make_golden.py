"""Generates the golden vectors in this folder from the reference itself.

The reference FIPI sources are compiled in place for each workload by
oracle/ref/build_ref.py; this script drives them (through the harness that
restates main.cpp's loop body) on seeded inputs and stores inputs and
outputs as .npz files.  The initial phase field is drawn on the
reference's own 1e-3 lattice (rand()%1000/1e3*0.2-0.1, field.cpp:96) from a
seeded generator, so it is stored compactly as integers.

Run where the reference sources exist:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "oracle"))

import oracle as O  # noqa: E402
from fipi_gb300.params import workload  # noqa: E402

CASES = {"t16": 4, "t32": 3, "t32_aniso": 3, "t32_2pi": 3}


def inputs(name, seed):
    w = workload(name)
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 1000, w.V).astype(np.uint16)
    c0 = k.astype(np.float64) / 1e3 * 0.2 - 0.1
    L = np.array([w.lx, w.ly, w.lz])
    u = rng.integers(0, 1000, (w.n_p, 3)).astype(np.float64) / 1e3  # cluster.cpp:63-72 lattice
    p0 = (u * L).ravel()
    return w, k, c0, p0


def main():
    for name, steps in CASES.items():
        w, k, c0, p0 = inputs(name, 100 + len(name))
        ref = O.Ref(name)
        assert ref.init(c0, p0) == 0
        assert ref.step(steps) == 0
        p, fpp, fpi = ref.particles()
        # fine-grained reference calls on the initial positions
        st, keys, srt, off, mark = ref.sorting(p0)
        assert st == 0
        rng = np.random.default_rng(7)
        f_pi = rng.standard_normal(3 * w.n_p)
        st, fpp0, tau0 = ref.f_pp(p0, 3, f_pi)
        sp = ref.spread(p0, fpp0)
        nz = np.nonzero(sp)[0]
        np.savez_compressed(
            HERE / f"{name}.npz",
            c0_lattice=k, p0=p0, steps=steps,
            phase=ref.phase(), velocity=ref.velocity() if w.V <= 4096 else np.zeros(0),
            velocity_l2=np.linalg.norm(ref.velocity()),
            p=p, f_pp=fpp, f_pi=fpi, tau=ref.tau(), free_energy=ref.free_energy(),
            keys=keys, sorted=srt, offsets=off, it_mark=mark,
            f_pi_in=f_pi, f_pp0=fpp0, tau0=tau0, spread_idx=nz.astype(np.int32), spread_val=sp[nz],
        )
        print(name, (HERE / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
