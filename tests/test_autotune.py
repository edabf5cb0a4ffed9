"""The autotuner's table (csrc/autotune.cpp) on CPU: the selection rule (lowest finite cost, ties to the earlier
candidate, no finite cost -> error), lookups with a fallback, and the table's file round trip.  The measured
choices themselves need a GPU (tests/test_gpu_autotune.py)."""
import ctypes
import json

import numpy as np
import pytest

import libkriging_gb300 as lk
from libkriging_gb300._lib import last_error


def _record(lib, key, cands, costs):
    c = (ctypes.c_int * len(cands))(*cands)
    d = (ctypes.c_double * len(costs))(*costs)
    return lib.lkg_autotune_record(key.encode(), c, d, len(cands))


def test_selection_rule_and_lookup():
    lib = lk.load()
    lib.lkg_autotune_clear()
    inf = float("inf")
    assert _record(lib, "t:a", [0, 5, 6, 7], [9.0, inf, 3.0, 3.0]) == 6  # ties -> the earlier candidate
    assert _record(lib, "t:b", [0, 5], [2.0, 1.0]) == 5
    assert _record(lib, "t:c", [0, 5], [inf, inf]) == -1 and "finite" in last_error()
    assert lib.lkg_autotune_lookup(b"t:a", -3) == 6
    assert lib.lkg_autotune_lookup(b"t:missing", -3) == -3
    need = lib.lkg_autotune_report(None, 0)
    buf = ctypes.create_string_buffer(need)
    lib.lkg_autotune_report(buf, need)
    lines = sorted(buf.value.decode().splitlines())
    assert lines[0].split("\t")[:2] == ["t:a", "6"] and lines[1].split("\t")[:2] == ["t:b", "5"]
    lib.lkg_autotune_clear()


def test_table_file_round_trip(tmp_path):
    lib = lk.load()
    lib.lkg_autotune_clear()
    _record(lib, "precision:k=3:nm=1:n=16384:d=8:tol=1e-08,1e-06", [0, 5, 6, 7], [3900.0, float("inf"), 230.0, 240.0])
    _record(lib, "t:x", [1, 2], [0.5, 0.25])
    f = tmp_path / "tune.json"
    assert lib.lkg_autotune_save(str(f).encode()) == 0
    table = json.loads(f.read_text())
    assert table["t:x"] == [2, 0.25]
    lib.lkg_autotune_clear()
    assert lib.lkg_autotune_lookup(b"t:x", -1) == -1
    assert lib.lkg_autotune_load(str(f).encode()) == 0
    assert lib.lkg_autotune_lookup(b"t:x", -1) == 2
    assert lib.lkg_autotune_lookup(b"precision:k=3:nm=1:n=16384:d=8:tol=1e-08,1e-06", -1) == 6
    bad = tmp_path / "bad.json"
    bad.write_text('{"k": [1 2]}')
    assert lib.lkg_autotune_load(str(bad).encode()) == -1
    lib.lkg_autotune_clear()
