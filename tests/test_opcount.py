"""The frozen algorithmic operation counts (bench/flops.h) are what the oracle's own
arithmetic does: a recount with the operation-counting build (oracle/opcount.cpp) on
the benchmark's CPU sample gives the committed constants, and the unit counts are
those of sp2 graphite (3 bonds, 6 triplets per atom; vdW on half the directed pairs,
three intralayer neighbours per pair)."""
import pytest

import opcount


@pytest.fixture(scope="module")
def recount():
    s = opcount.sample()
    return opcount.constants(opcount.count(s), s.n)


def test_header_matches_a_fresh_count(recount):
    frozen = opcount.read_header()
    for k, v in recount.items():
        assert k in frozen, k
        assert abs(frozen[k] - v) <= 1e-3, (k, frozen[k], v)


def test_unit_counts_are_those_of_sp2_graphite(recount):
    assert recount["TERS_BONDS_PER_ATOM"] == 3.0
    assert recount["TERS_TRIPLETS_PER_ATOM"] == 6.0
    assert recount["VDW_PER_PAIR"] == 0.5
    assert recount["KTERMS_PER_PAIR"] == 3.0
    # a candidate is a displacement and r^2: 3 subtractions, 3 multiplications, 2 additions
    assert recount["FLOPS_ILP_CAND"] == 8.0
    # two exponentials per repulsion term, exp and pow per vdW term
    assert recount["CALLS_ILP_PAIR"] == 2.0 and recount["CALLS_ILP_VDW"] == 2.0
