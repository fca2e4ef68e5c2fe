"""Writes poseidon252_constants.cuh: the Hades round constants of the Starknet Poseidon hash and
the Montgomery constants of the STARK field, for the device Poseidon252 kernels.

The published constant generation of the hash (starknet-crypto 0.6.2, which the reference's
Poseidon252 hasher and channel call): round constant k, k = 3 * round + word for 91 rounds of a
width-3 state, is SHA-256("Hades" || decimal k) read as a big-endian integer, mod
p = 2^251 + 17 * 2^192 + 1. They are stored in Montgomery form (times 2^256 mod p) as 8
little-endian 32-bit limbs. Run by the build; the output is committed so that the sources build
as they are.
"""
import os
import sys
from hashlib import sha256

P = 2 ** 251 + 17 * 2 ** 192 + 1
R = 2 ** 256
ROUNDS = 8 + 83
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "poseidon252_constants.cuh")


def limbs(x):
    return ", ".join(f"0x{(x >> (32 * i)) & 0xFFFFFFFF:08x}u" for i in range(8))


def render() -> str:
    ark = [int(sha256(f"Hades{k}".encode()).hexdigest(), 16) % P for k in range(3 * ROUNDS)]
    lines = [
        "// Generated by gen_poseidon252_constants.py from the published constant generation of the",
        "// Starknet Poseidon hash; do not edit. Field p = 2^251 + 17 * 2^192 + 1, Montgomery radix 2^256,",
        "// values as 8 little-endian 32-bit limbs.",
        "#pragma once",
        "#include <cstdint>",
        "",
        "namespace stwo {",
        "",
        f"constexpr int P252_ROUNDS = {ROUNDS};",
        "// Round constant 3 * round + word, in Montgomery form.",
        f"__constant__ uint32_t c_p252_ark[{3 * ROUNDS}][8] = {{",
    ]
    lines += [f"    {{{limbs(c * R % P)}}}," for c in ark]
    lines += [
        "};",
        f"__constant__ uint32_t c_p252_r2[8] = {{{limbs(R * R % P)}}};    // 2^512 mod p: into Montgomery form",
        f"__constant__ uint32_t c_p252_one[8] = {{{limbs(R % P)}}};   // 1 in Montgomery form",
        f"__constant__ uint32_t c_p252_two[8] = {{{limbs(2 * R % P)}}};   // 2 in Montgomery form",
        "",
        "}  // namespace stwo",
        "",
    ]
    return "\n".join(lines)


def main(check: bool = False) -> bool:
    text = render()
    if os.path.exists(OUT) and open(OUT).read() == text:
        return True
    if check:
        return False
    with open(OUT, "w") as f:
        f.write(text)
    return True


if __name__ == "__main__":
    ok = main(check="--check" in sys.argv)
    sys.exit(0 if ok else 1)
