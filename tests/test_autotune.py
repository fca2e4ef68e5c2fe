"""The autotuner's table through the C ABI (CPU: no kernel runs) and its save/load round trip."""
import os

import pytest


def test_table_round_trip(tmp_path):
    from stwo_gb300 import _lib, autotune

    autotune.clear()
    autotune.set_mode(autotune.OFF)
    _lib.call("stwo_autotune_set_entry", 1, (17 << 32) | 80, 2)
    _lib.call("stwo_autotune_set_entry", 2, (17 << 40) | (1 << 32) | 1296, 4)
    _lib.call("stwo_autotune_set_entry", 1, (17 << 32) | 80, 3)  # replaces
    got = sorted((e["site"], e["key"], e["choice"]) for e in autotune.entries())
    assert got == [(1, (17 << 32) | 80, 3), (2, (17 << 40) | (1 << 32) | 1296, 4)]
    path = os.path.join(tmp_path, "table.json")
    assert autotune.save(path) == 2
    autotune.clear()
    assert autotune.entries() == []
    assert autotune.load(path) == 2
    assert sorted((e["site"], e["key"], e["choice"]) for e in autotune.entries()) == got
    assert autotune.summary() == {"merkle_layer": {"3": 1}, "quotient_rows": {"4": 1}}
    autotune.clear()


def test_mode_is_checked():
    from stwo_gb300 import _lib, autotune

    with pytest.raises(_lib.StwoError):
        autotune.set_mode(3)
    autotune.set_mode(autotune.OFF)
