"""The oracle's multi-component prove() and verify() on the reference's Plonk and state-machine
examples (CPU): proofs verify, and a flipped byte or a wrong claimed sum is rejected."""
import pytest


@pytest.mark.parametrize("log_n,cfg", [(4, (5, 1, 0, 3)), (7, (8, 2, 1, 5))])
def test_plonk_prove_verify(oracle, log_n, cfg):
    proof, cs = oracle.prove_plonk(log_n, cfg)
    assert oracle.verify_plonk(log_n, cs, proof) == (True, "")
    bad = bytearray(proof)
    bad[len(bad) // 2] ^= 1
    assert not oracle.verify_plonk(log_n, cs, bytes(bad))[0]
    assert not oracle.verify_plonk(log_n, (cs[0] ^ 1,) + cs[1:], proof)[0]


@pytest.mark.parametrize("log_n,initial", [(5, (0, 0)), (8, (17, 12))])
def test_state_machine_prove_verify(oracle, log_n, initial):
    proof, sums = oracle.prove_state_machine(log_n, initial)
    assert oracle.verify_state_machine(log_n, sums, proof) == (True, "")
    bad = bytearray(proof)
    bad[-40] ^= 1
    assert not oracle.verify_state_machine(log_n, sums, bytes(bad))[0]
    assert not oracle.verify_state_machine(log_n, (sums[1], sums[0]), proof)[0]


def test_blake_prove_verify(oracle):
    """The full Blake example (scheduler, two round components, five XOR tables): the eight claimed
    sums add to zero, so every round and XOR lookup is balanced by the scheduler and the tables;
    the proof verifies; a flipped byte or a changed sum is rejected."""
    P = (1 << 31) - 1
    proof, sums = oracle.prove_blake(4)
    total = [sum(q[k] for q in sums) % P for k in range(4)]
    assert total == [0, 0, 0, 0]
    assert all(q != (0, 0, 0, 0) for q in sums)
    assert oracle.verify_blake(4, sums, proof) == (True, "")
    bad = bytearray(proof)
    bad[len(bad) // 3] ^= 1
    assert not oracle.verify_blake(4, sums, bytes(bad))[0]
    moved = [list(q) for q in sums]
    moved[0][0] = (moved[0][0] + 1) % P
    moved[3][0] = (moved[3][0] - 1) % P  # still sums to zero, but not the traces' sums
    ok, why = oracle.verify_blake(4, [tuple(q) for q in moved], proof)
    assert not ok
    assert oracle.verify_blake(4, [sums[1], sums[0]] + sums[2:], proof)[0] is False


def test_blake_scheduler_rounds_are_blake2s(oracle):
    """Pins the scheduler's round function to BLAKE2s itself: ten rounds on the compression's
    working vector (h, IV ^ (t, f)), finalised as h ^ v[0..8] ^ v[8..16], give hashlib's BLAKE2s-256
    of a one-block 64-byte message (RFC 7693: parameter block 0x01010020, t = 64, last block)."""
    import hashlib
    import struct

    iv = [0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A, 0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19]
    for seed in range(3):
        msg = bytes((seed * 97 + 13 * i) & 0xFF for i in range(64))
        m = list(struct.unpack("<16I", msg))
        h = [iv[0] ^ 0x01010020] + iv[1:]
        v = h + iv[:4] + [iv[4] ^ 64, iv[5], iv[6] ^ 0xFFFFFFFF, iv[7]]
        out = oracle.blake2s_rounds(v, m)
        digest = struct.pack("<8I", *[h[i] ^ out[i] ^ out[i + 8] for i in range(8)])
        assert digest == hashlib.blake2s(msg).digest()
