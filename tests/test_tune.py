"""Host logic of the window-width autotuner (bend-groth16_gb300/tune_msm.py): the search that
widens its range while the fastest width sits on an edge, and the header it writes, which the
library compiles in.  No GPU: the measurements are a fake cost curve."""
import re

import pytest

import tune_msm


def test_search_widens_past_the_lower_edge():
    calls = []

    def cost(c):
        calls.append(c)
        return abs(c - 7) + 1.0
    times = tune_msm.search(cost, 10, 14, 3, 20)
    assert min(times, key=times.get) == 7
    assert sorted(times) == list(range(6, 15))      # one width past the optimum, then stop
    assert len(calls) == len(set(calls))            # nothing measured twice


def test_search_widens_past_the_upper_edge_and_clamps():
    times = tune_msm.search(lambda c: -c, 16, 19, 3, 20)
    assert sorted(times) == [16, 17, 18, 19, 20]    # stops at c_max
    times = tune_msm.search(lambda c: c, 1, 5, 3, 20)
    assert sorted(times) == [3, 4, 5]               # clamped below, optimum on c_min


def test_search_interior_optimum_measures_only_the_range():
    times = tune_msm.search(lambda c: (c - 12) ** 2, 10, 14, 3, 20)
    assert sorted(times) == [10, 11, 12, 13, 14]


def test_a_width_that_changes_the_result_stops_the_tuning():
    """every width must give the same MSM result or proof; the tuner keeps the first and stops
    at the first width that differs, so no such width can reach the committed header"""
    seen = {}
    tune_msm.same_result(seen, ("table", 18), "A 0x1")
    tune_msm.same_result(seen, ("table", 18), "A 0x1")
    tune_msm.same_result(seen, ("table", 20), "A 0x2")
    with pytest.raises(RuntimeError):
        tune_msm.same_result(seen, ("table", 18), "A 0x3")


def test_header_text_rows():
    sets = {0: {10: 8, 11: 9, 22: 17}, 1: {10: 8}}
    tables = {0: {18: 17}, 1: {}}
    h = tune_msm.header_text(sets, tables, "test gpu")
    rows = re.findall(r"\{([0-9, ]+)\}", h)
    assert len(rows) == 6
    vals = [[int(x) for x in r.split(",")] for r in rows]
    assert all(len(v) == tune_msm.MAX_LOG2 - tune_msm.MIN_LOG2 + 1 for v in vals)
    assert vals[0][0] == 8 and vals[0][1] == 9 and vals[0][-1] == 17 and vals[0][5] == 0
    assert vals[1][0] == 8 and sum(vals[1]) == 8
    assert vals[2][18 - tune_msm.MIN_LOG2] == 17 and sum(vals[3]) == 0
    assert "kTuneMinLog2 = %d" % tune_msm.MIN_LOG2 in h


def test_committed_header_is_in_range():
    """the committed table holds 0 (size rule) or a width the MSM supports, per curve and size"""
    import os
    src = open(os.path.join(os.path.dirname(tune_msm.__file__), "csrc", "msm_tune.h")).read()
    rows = re.findall(r"\{([0-9, ]+)\}", src)
    assert len(rows) == 6
    for r in rows:
        v = [int(x) for x in r.split(",")]
        assert len(v) == tune_msm.MAX_LOG2 - tune_msm.MIN_LOG2 + 1
        assert all(x == 0 or 3 <= x <= 20 for x in v)


def test_committed_tables_round_trip(tmp_path):
    """--keep reads a header back into the tables the writer takes"""
    sets = {0: {10: 8, 14: 9, 22: 17}, 1: {12: 9}}
    tables = {0: {18: 17}, 1: {10: 10, 20: 17}}
    proof = {0: {}, 1: {18: 13}}
    p = tmp_path / "t.h"
    p.write_text(tune_msm.header_text(sets, tables, "test gpu", proof))
    assert tune_msm.committed_tables(str(p)) == (sets, tables, proof)


def test_pair_round_model(built_lib):
    """the batch-affine rounds are taken only where they measured faster on GB300: G1 MSMs of at
    least 2^23 entries with 32 or more per bucket (bg_msm_pair_rounds is host logic, no GPU)"""
    import bendg
    L = bendg.lib()
    G1, G2 = bendg.CURVE_G1, bendg.CURVE_G2
    assert L.bg_msm_pair_rounds(1 << 20, G1) == 2     # c = 15, W = 17: 17.8 M entries, 64 per bucket
    assert L.bg_msm_pair_rounds(1 << 22, G1) == 2
    assert L.bg_msm_pair_rounds(1 << 18, G1) == 0     # 4.5 M entries
    assert L.bg_msm_pair_rounds(1 << 20, G2) == 0
    assert L.bg_msm_pair_rounds(1 << 18, G2) == 0
    assert L.bg_msm_pair_rounds(0, G1) == 0
