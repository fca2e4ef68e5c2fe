"""Pins the oracle's Poseidon252 hasher and channel (oracle/poseidon252.h).

- The reference's own vectors: crates/prover/src/core/vcs/poseidon252_merkle.rs:72-91 (test_vector).
- An independent big-integer restatement (tests/p252.py) on seeded inputs: hash, hash_many of every
  padding case, hash_node with and without children over 0..20 values, the channel's draws and
  mixes, trailing zeros and the minimum-nonce grind.
- The reference's channel behaviour tests (crates/prover/src/core/channel/poseidon252.rs:120-190).
"""
import numpy as np

from tests import p252


def test_reference_test_vector(oracle):
    assert oracle.p252_hash_node(None, [0, 1]) == \
        2552053700073128806553921687214114320458351061521275103654266875084493044716
    assert oracle.p252_hash_node((1, 2), [3]) == \
        159358216886023795422515519110998391754567506678525778721401012606792642769


def test_hash_and_hash_many_match_restatement(oracle):
    rng = np.random.default_rng(252)
    felts = [int.from_bytes(rng.bytes(32), "little") % p252.P252 for _ in range(8)]
    assert oracle.p252_hash(felts[0], felts[1]) == p252.hash2(felts[0], felts[1])
    for n in range(6):
        assert oracle.p252_hash_many(felts[:n]) == p252.hash_many(felts[:n])


def test_hash_node_matches_restatement(oracle):
    rng = np.random.default_rng(253)
    for n in [0, 1, 7, 8, 9, 16, 20]:
        vals = [int(x) for x in rng.integers(0, p252.P31, n)]
        ch = tuple(int.from_bytes(rng.bytes(32), "little") % p252.P252 for _ in range(2))
        assert oracle.p252_hash_node(None, vals) == p252.hash_node(None, vals)
        assert oracle.p252_hash_node(ch, vals) == p252.hash_node(ch, vals)


def test_commit_on_layer_matches_hash_node(oracle):
    rng = np.random.default_rng(254)
    log, ncols = 3, 11
    cols = [rng.integers(0, p252.P31, 1 << log, dtype=np.int64).astype(np.uint32) for _ in range(ncols)]
    prev = rng.integers(0, 1 << 32, size=(2 << log, 8), dtype=np.uint64).astype(np.uint32)
    prev[:, 7] &= 0x03FFFFFF  # canonical felts below p
    got = oracle.p252_commit_on_layer(log, prev, cols)
    as_int = lambda w: sum(int(v) << (32 * i) for i, v in enumerate(w))
    for i in range(1 << log):
        want = p252.hash_node((as_int(prev[2 * i]), as_int(prev[2 * i + 1])), [int(c[i]) for c in cols])
        assert as_int(got[i]) == want


def test_channel_matches_restatement(oracle):
    rng = np.random.default_rng(255)
    felts = [tuple(int(x) for x in rng.integers(0, p252.P31, 4)) for _ in range(5)]
    for start in [0, 123456789]:
        ch = p252.Channel(start)
        ch.mix_felts(felts)
        want = ch.draw_felts(9)
        got, digest = oracle.p252_channel(start, felts, 9)
        assert got == want and digest == ch.digest
    # No mix: draws from the initial digest (a default channel starts at 0).
    got, _ = oracle.p252_channel(0, [], 5)
    assert got == p252.Channel(0).draw_felts(5)


def test_draws_are_distinct_and_mixing_changes_digest(oracle):
    """test_draw_felts / test_mix_felts (channel/poseidon252.rs:163-190)."""
    draws, d0 = oracle.p252_channel(0, [], 9)
    assert len(set(draws)) == 9
    _, d1 = oracle.p252_channel(0, [(1923782, 0, 0, 0), (1923783, 0, 0, 0)], 0)
    assert d1 != d0


def test_trailing_zeros_and_grind(oracle):
    rng = np.random.default_rng(256)
    for _ in range(20):
        d = int.from_bytes(rng.bytes(32), "little") % p252.P252
        assert oracle.p252_trailing_zeros(d) == p252.trailing_zeros(d)
    for pow_bits in [0, 1, 3, 5]:
        d = int.from_bytes(rng.bytes(32), "little") % p252.P252
        nonce = oracle.p252_grind(d, pow_bits)
        assert p252.trailing_zeros(p252.hash2(d, nonce)) >= pow_bits
        assert all(p252.trailing_zeros(p252.hash2(d, k)) < pow_bits for k in range(nonce))


def test_device_constant_table_is_current():
    """The committed round-constant table of the device kernels is what its generator writes from
    the published constant derivation, and its first constant is the restatement's, in Montgomery
    form (times 2^256 mod p)."""
    import importlib.util
    import os
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = os.path.join(root, "stwo_gb300", "csrc", "gen_poseidon252_constants.py")
    spec = importlib.util.spec_from_file_location("gen_p252", path)
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    text = gen.render()
    assert open(gen.OUT).read() == text
    first = re.search(r"c_p252_ark\[273\]\[8\] = \{\s*\{([^}]*)\}", text).group(1)
    limbs = [int(x.strip().rstrip("u"), 16) for x in first.split(",")]
    assert sum(v << (32 * i) for i, v in enumerate(limbs)) == p252._ARK[0] * 2 ** 256 % p252.P252
