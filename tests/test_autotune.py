"""Autotuner search logic and its table round trip through the library's
tuning store (host-only calls; no GPU needed)."""
import os

from ddla_gb300 import autotune


def test_search_finds_coordinate_minimum():
    grid = {"a": [1, 2, 3], "b": [10, 20]}
    cost = {(1, 10): 5.0, (2, 10): 3.0, (3, 10): 4.0, (2, 20): 1.0, (1, 20): 9.0, (3, 20): 8.0}
    calls = []

    def t(table):
        calls.append(dict(table))
        return cost[(table["a"], table["b"])]

    best, bt, log = autotune.search(grid, t)
    assert best == {"a": 2, "b": 20} and bt == 1.0
    assert len(log) == len(calls) == 1 + 2 + 1


def test_table_round_trip(tmp_path):
    table = {"batched.nb.32": 8, "batched.ctas_per_sm": 2, "lu.nb": 32}
    p = os.path.join(tmp_path, "t.json")
    autotune.save(table, p)
    try:
        assert autotune.load(p) == table
        for k, v in table.items():
            assert autotune.tune_get(k, -1) == v
    finally:
        for k in table:
            autotune.tune_set(k, 0)
    assert autotune.tune_get("lu.nb", -1) == 0
