"""Particle-model extensions on the oracle side (no device needed).

The reference carries a fluid-to-particle coupling (get_local_u,
element.cpp:38-52) and a Brownian force (get_f_rand, element.cpp:109-144)
that its step never uses.  The oracle restates both; the Brownian draw uses
Philox-4x32-10 in place of rand(), checked here against the published
known-answer vectors of Salmon et al. (SC 2011, Random123).
"""
import numpy as np
import pytest

from conftest import seeded_state

REF_PI = 3.1415926


def test_philox_known_answers(oracle_mod):
    ph = oracle_mod.philox4x32
    assert ph([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert ph([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert ph([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_brownian_normals(oracle_mod):
    bn = oracle_mod.brownian_normals
    a = bn(7, 3, 11, REF_PI)
    assert np.array_equal(a, bn(7, 3, 11, REF_PI))  # deterministic
    assert not np.array_equal(a, bn(7, 4, 11, REF_PI))  # another particle
    assert not np.array_equal(a, bn(7, 3, 12, REF_PI))  # another step
    assert not np.array_equal(a, bn(8, 3, 11, REF_PI))  # another seed
    g = np.concatenate([bn(1, i, 0, REF_PI) for i in range(4000)])
    assert np.all(np.abs(g) <= 5.0)
    # uniforms on the 1/1000 lattice: every value is sqrt(-2 ln(a/1000)) cos(2 pi b/1000)
    assert abs(g.mean()) < 0.05
    assert 0.93 < g.var() < 1.07


def test_extensions_change_the_step_and_default_is_unchanged(fipi, oracle_mod):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 41)
    runs = {}
    for key, (couple, kt) in {"plain": (False, 0.0), "off": (False, 0.0), "brown": (False, 1.0),
                              "couple": (True, 0.0)}.items():
        port = oracle_mod.Port(P)
        port.set_state(c, p, r, ct)
        if key != "plain":
            port.set_extensions(couple, kt, 5)
        assert port.step(2) == 0
        runs[key] = port.particles()[0]
    assert np.array_equal(runs["plain"], runs["off"])
    d_brown = np.abs(runs["brown"] - runs["plain"]).max()
    assert 1e-4 < d_brown < 0.2  # ~sqrt(kt dt / (3 pi mu r)) per step
    assert not np.array_equal(runs["couple"], runs["plain"])
