"""The reference's own initial state for a seed (main.cpp:24, 34, 58-66).

srand(seed) followed by the phase field's draws (field.cpp:85-99) and
cluster::distribute's random sequential addition (cluster.cpp:53-113): the
oracle's restatement (glibc's rand() restated, O(N^2) overlap scan as the
reference) must equal the reference compiled in place bit for bit, and the
library's host implementation (hash-grid overlap test) must equal the oracle.
No device is needed.
"""
import numpy as np
import pytest

SEEDS = [1, 7, 12345, 2**31 - 1, 3_000_000_000]


@pytest.fixture(scope="module")
def ref_mod(oracle_mod):
    if not oracle_mod.reference_available():
        pytest.skip("reference sources absent")
    return oracle_mod


@pytest.mark.parametrize("seed", SEEDS)
def test_oracle_matches_reference(fipi, ref_mod, seed):
    w = fipi.workload("cfg1_64")
    ref = ref_mod.Ref("cfg1_64")
    c_ref, p_ref = ref.initial_state(seed)
    st, c, p = ref_mod.reference_initial_state(w.params(), seed)
    assert st == 0
    assert np.array_equal(c, c_ref)
    assert np.array_equal(p, p_ref)
    # the draws are the quantised values of field.cpp:96 and cluster.cpp:63-71
    assert c.min() >= -0.1 and c.max() <= 0.0999 + 1e-15
    assert np.all(np.isclose(p / w.lx * 1000, np.round(p / w.lx * 1000), rtol=0, atol=1e-9))


@pytest.mark.parametrize("name,seed", [("cfg1_64", 1), ("cfg1_64", 3_000_000_000), ("t32", 5)])
def test_library_matches_oracle(fipi, oracle_mod, name, seed):
    w = fipi.workload(name)
    P = w.params()
    st, c_o, p_o = oracle_mod.reference_initial_state(P, seed)
    assert st == 0
    c, p = fipi.reference_initial_state(P, seed)
    assert np.array_equal(c, c_o)
    assert np.array_equal(p, p_o)
    # without the phase field the same stream is consumed
    c2, p2 = fipi.reference_initial_state(P, seed, phase=False)
    assert c2 is None and np.array_equal(p2, p_o)


def test_library_matches_oracle_dense(fipi, oracle_mod):
    """2000 spheres r = 4 in 128^3 (26 % volume fraction): many rejected
    candidates, every one of which must be rejected by both."""
    w = fipi.workload("cfg4_128")
    P = w.params()
    st, _, p_o = oracle_mod.reference_initial_state(P, 99)
    assert st == 0
    _, p = fipi.reference_initial_state(P, 99, phase=False)
    assert np.array_equal(p, p_o)
    d = p.reshape(-1, 3)
    # no pair closer than 2 r_p without periodic images (check_overlap)
    diff = d[:, None, :] - d[None, :, :]
    dist = np.sqrt((diff ** 2).sum(-1)) + np.eye(len(d)) * 1e9
    assert dist.min() >= 2 * P.r_p


def test_infeasible_placement_is_an_error(fipi, oracle_mod):
    w = fipi.workload("cfg1_64")
    P = w.params()
    P.n_p = 2
    P.r_p = 60.0  # 2 r_p exceeds the box diagonal: the second sphere has no place
    st, _, _ = oracle_mod.reference_initial_state(P, 3, max_candidates=20000)
    assert st != 0
    with pytest.raises(fipi.FipiError):
        fipi.reference_initial_state(P, 3, phase=False)
