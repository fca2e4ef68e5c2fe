"""Circle-group index arithmetic (crates/prover/src/core/circle.rs:221-430,
poly/circle/canonic.rs:27-60). Indices are integers modulo 2^31; i stands for i * M31_CIRCLE_GEN."""
from __future__ import annotations

from ._lib import Coset

LOG_ORDER = 31
MASK = (1 << LOG_ORDER) - 1


def subgroup_gen(log_size: int) -> int:
    return 1 << (LOG_ORDER - log_size)


def coset(initial_index: int, log_size: int) -> Coset:
    return Coset(initial_index & MASK, subgroup_gen(log_size), log_size)


def coset_raw(initial_index: int, step_size: int, log_size: int) -> Coset:
    return Coset(initial_index & MASK, step_size & MASK, log_size)


def odds(log_size: int) -> Coset:
    return coset(subgroup_gen(log_size + 1), log_size)


def half_odds(log_size: int) -> Coset:
    return coset(subgroup_gen(log_size + 2), log_size)


def canonic_half_coset(log_size: int) -> Coset:
    """CanonicCoset(log_size).half_coset() = Coset::half_odds(log_size - 1)."""
    return half_odds(log_size - 1)


def double(c: Coset) -> Coset:
    return Coset((c.initial_index * 2) & MASK, (c.step_size * 2) & MASK, max(c.log_size - 1, 0))


def repeated_double(c: Coset, n: int) -> Coset:
    for _ in range(n):
        c = double(c)
    return c


def as_tuple(c: Coset):
    return (c.initial_index, c.step_size, c.log_size)
