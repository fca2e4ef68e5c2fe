"""The library's autotuner from Python: mode switch, and the choice table saved to / loaded from a
JSON file of {"site", "key", "choice"} entries (stwo_autotune_* in include/stwo_cuda.h)."""
from __future__ import annotations

import ctypes as C
import json

from . import _lib

OFF, USE, TUNE = 0, 1, 2
SITES = {1: "merkle_layer", 2: "quotient_rows"}


def set_mode(mode: int) -> None:
    _lib.call("stwo_autotune_mode", mode)


def entries() -> list[dict]:
    lib = _lib.load()
    n = lib.stwo_autotune_entries(None, None, None, 0)
    sites = (C.c_uint32 * max(n, 1))()
    keys = (C.c_uint64 * max(n, 1))()
    choices = (C.c_uint32 * max(n, 1))()
    n = min(n, lib.stwo_autotune_entries(sites, keys, choices, n))
    return [{"site": int(sites[i]), "key": int(keys[i]), "choice": int(choices[i])} for i in range(n)]


def clear() -> None:
    _lib.call("stwo_autotune_clear")


def load(path: str) -> int:
    """Adds the entries of a saved table; returns how many."""
    with open(path) as f:
        table = json.load(f)
    for e in table:
        _lib.call("stwo_autotune_set_entry", int(e["site"]), int(e["key"]), int(e["choice"]))
    return len(table)


def save(path: str) -> int:
    table = entries()
    with open(path, "w") as f:
        json.dump(table, f, indent=1)
    return len(table)


def summary() -> dict:
    """Entries per site and how often each choice was taken."""
    out: dict = {}
    for e in entries():
        site = SITES.get(e["site"], str(e["site"]))
        d = out.setdefault(site, {})
        d[str(e["choice"])] = d.get(str(e["choice"]), 0) + 1
    return out
