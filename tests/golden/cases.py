"""Seeded inputs of the golden proof cases (shared by the fixture generator and the tests).

Word i of stream k: splitmix64(k + (i + 1) * 0x9E3779B97F4A7C15) mod (2^31 - 1).
"""
import numpy as np

P = (1 << 31) - 1


def words(k: int, n: int) -> np.ndarray:
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(k) + (i + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z % np.uint64(P)).astype(np.uint32)


# name -> parameters. Wide-Fibonacci rows start from (a[r], b[r]); Poseidon2 uses the reference's
# deterministic inputs (init None) or seeded states; GKR layers use seeded QM31 columns.
WIDE_FIB = {
    "wide_fib_log5_cols100": dict(log=5, cols=100, seed=11, cfg=(5, 1, 0, 3)),
    "wide_fib_log9_cols16_blowup2": dict(log=9, cols=16, seed=12, cfg=(3, 2, 1, 5)),
}
POSEIDON = {
    "poseidon_log4_reference_inputs": dict(log=4, seed=None, cfg=(5, 1, 0, 3)),
    "poseidon_log6_seeded_pow10": dict(log=6, seed=13, cfg=(10, 1, 0, 3)),
}
GKR = {
    "gkr_generic_log10": dict(layers=[(1, 10)], seed=14),
    "gkr_mixed_batch": dict(layers=[(0, 6), (1, 8), (2, 5), (3, 7)], seed=15),
}


def wide_fib_inputs(case):
    n = 1 << case["log"]
    return words(case["seed"], n), words(case["seed"] + 1000, n)


def poseidon_inputs(case):
    if case["seed"] is None:
        return None
    return words(case["seed"], (1 << case["log"]) * 8 * 16)


def gkr_layers(case):
    """[(kind, [columns...])] with secure columns as (4, n) arrays and multiplicities (n,)."""
    out = []
    for j, (kind, log) in enumerate(case["layers"]):
        n = 1 << log
        w = words(case["seed"] * 100 + j, 9 * n)
        sec_a, sec_b = w[:4 * n].reshape(4, n), w[4 * n:8 * n].reshape(4, n)
        if kind == 0:
            cols = [sec_a]
        elif kind == 1:
            cols = [sec_a, sec_b]
        elif kind == 2:
            cols = [w[8 * n:], sec_b]
        else:
            cols = [sec_b]
        out.append((kind, [np.ascontiguousarray(c) for c in cols]))
    return out
