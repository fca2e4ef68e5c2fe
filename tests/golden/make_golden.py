"""Writes tests/golden/proofs.json: SHA-256 and length of the oracle's canonical proof bytes for
each case in cases.py. Run from the repository root: python -m tests.golden.make_golden"""
import hashlib
import json
import os

from tests.golden import cases

HERE = os.path.dirname(os.path.abspath(__file__))


def oracle_digests():
    import oracle.pyoracle as O

    out = {}
    for name, c in cases.WIDE_FIB.items():
        a, b = cases.wide_fib_inputs(c)
        p = O.prove_wide_fib(c["log"], c["cols"], a, b, c["cfg"])
        out[name] = {"sha256": hashlib.sha256(p).hexdigest(), "len": len(p)}
    for name, c in cases.POSEIDON.items():
        p, cs = O.prove_poseidon(c["log"], cases.poseidon_inputs(c), c["cfg"])
        out[name] = {"sha256": hashlib.sha256(p).hexdigest(), "len": len(p), "claimed_sum": list(cs)}
    for name, c in cases.GKR.items():
        p, d = O.gkr_prove(cases.gkr_layers(c))
        out[name] = {"sha256": hashlib.sha256(p).hexdigest(), "len": len(p), "final_digest": d.hex()}
    return out


if __name__ == "__main__":
    from stwo_gb300.build import build_oracle

    build_oracle()
    with open(os.path.join(HERE, "proofs.json"), "w") as f:
        json.dump(oracle_digests(), f, indent=1, sort_keys=True)
        f.write("\n")
