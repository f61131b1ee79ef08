"""CPU: the closure study's metric -- the KE-error measure, the pairing of
every closure run with the cheapest plain run at least as accurate, and the
headline pick -- on synthetic run records (no GPU)."""
import math

import numpy as np
import pytest

from conftest import load_package


@pytest.fixture(scope="module")
def C():
    return load_package().closure


def test_ke_error_normalises_and_flags_blow_up(C):
    ref = np.array([2.0, 1.8, 1.5, 1.0])
    assert C.ke_error(ref * 3.0, ref) == 0.0  # both normalised by their first sample
    coarse = np.array([1.0, 0.9, 0.7, 0.5])
    want = math.sqrt(np.mean((coarse - ref / 2.0) ** 2))
    assert C.ke_error(coarse, ref) == pytest.approx(want, rel=1e-12)
    assert C.ke_error([1.0, 0.9, np.nan, np.nan], ref) == float("inf")
    assert C.ke_error([1.0, 0.9, np.inf, 0.5], ref) == float("inf")


def _runs():
    # shaped like the 512^3 -> 256^3 ... 32^3 study: plain BGK blows up below 128^3
    return [
        {"n": 256, "kind": "plain", "ke_error": 0.00085, "seconds": 2.98},
        {"n": 128, "kind": "plain", "ke_error": 0.0036, "seconds": 0.193},
        {"n": 64, "kind": "plain", "ke_error": float("inf"), "seconds": 0.016},
        {"n": 32, "kind": "plain", "ke_error": float("inf"), "seconds": 0.005},
        {"n": 128, "kind": "closure", "ke_error": 0.0013, "seconds": 0.401},
        {"n": 64, "kind": "closure", "ke_error": 0.009, "seconds": 0.052},
        {"n": 32, "kind": "closure", "ke_error": 0.069, "seconds": 0.014},
    ]


def test_each_closure_run_is_paired_with_the_cheapest_plain_run_as_accurate(C):
    pairs = {p["closure_n"]: p for p in C.speedup_at_equal_error(_runs())}
    assert set(pairs) == {128, 64, 32}
    # 0.0013 is beaten only by plain 256^3
    assert pairs[128]["plain_n"] == 256
    assert pairs[128]["speedup"] == pytest.approx(2.98 / 0.401)
    # both finite plain runs are at least as accurate as 0.009: the cheaper one
    assert pairs[64]["plain_n"] == 128
    assert pairs[64]["speedup"] == pytest.approx(0.193 / 0.052)
    assert pairs[32]["plain_n"] == 128
    # a blown-up plain run is never a match
    assert all(p["plain_ke_error"] is None or math.isfinite(p["plain_ke_error"])
               for p in pairs.values())


def test_a_closure_run_more_accurate_than_every_plain_run_has_no_pair(C):
    runs = _runs() + [{"n": 96, "kind": "closure", "ke_error": 0.0001, "seconds": 0.2}]
    p = next(q for q in C.speedup_at_equal_error(runs) if q["closure_n"] == 96)
    assert p["plain_n"] is None and p["speedup"] is None


def test_diverged_closure_runs_are_left_out(C):
    runs = _runs() + [{"n": 16, "kind": "closure", "ke_error": float("inf"), "seconds": 0.01}]
    assert 16 not in {p["closure_n"] for p in C.speedup_at_equal_error(runs)}


def test_headline_is_the_largest_speedup_within_the_error_bound(C):
    pairs = C.speedup_at_equal_error(_runs())
    best = C.headline(pairs, max_error=0.01)
    # 32^3 is faster still but its error (0.069) is above the bound
    assert best["closure_n"] == 128
    assert C.headline(pairs, max_error=0.1)["closure_n"] == 32
    assert C.headline(pairs, max_error=0.001) is None
