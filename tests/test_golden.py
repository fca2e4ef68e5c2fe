"""Golden proof digests (tests/golden/proofs.json, written by tests/golden/make_golden.py from the
oracle): the oracle must keep reproducing them, and the GPU must produce the same bytes without
any oracle at run time."""
import hashlib
import json
import os

import numpy as np
import pytest

from tests.golden import cases

GOLDEN = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "proofs.json")))


def test_oracle_reproduces_golden(oracle):
    from tests.golden.make_golden import oracle_digests

    assert oracle_digests() == GOLDEN


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.WIDE_FIB))
def test_gpu_wide_fib_matches_golden(cuda, name):
    from stwo_gb300.prover import prove_wide_fib, wide_fib_trace

    c = cases.WIDE_FIB[name]
    a, b = cases.wide_fib_inputs(c)
    trace = wide_fib_trace(c["log"], c["cols"], _dev(a), _dev(b))
    p = prove_wide_fib(c["log"], trace, c["cfg"])
    assert (hashlib.sha256(p).hexdigest(), len(p)) == (GOLDEN[name]["sha256"], GOLDEN[name]["len"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.POSEIDON))
def test_gpu_poseidon_matches_golden(cuda, name):
    from stwo_gb300.prover import prove_poseidon

    c = cases.POSEIDON[name]
    init = cases.poseidon_inputs(c)
    p, cs = prove_poseidon(c["log"], _dev(init) if init is not None else None, c["cfg"])
    assert hashlib.sha256(p).hexdigest() == GOLDEN[name]["sha256"]
    assert list(cs) == GOLDEN[name]["claimed_sum"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.GKR))
def test_gpu_gkr_matches_golden(cuda, name):
    from stwo_gb300.backend import GkrLayer, GkrOps, SecureColumn

    def sec(a):
        return SecureColumn([_dev(a[i]) for i in range(4)])

    layers = []
    for kind, cols in cases.gkr_layers(cases.GKR[name]):
        if kind == 0:
            layers.append(GkrLayer(0, sec(cols[0])))
        elif kind == 1:
            layers.append(GkrLayer(1, sec(cols[0]), sec(cols[1])))
        elif kind == 2:
            layers.append(GkrLayer(2, _dev(cols[0]), sec(cols[1])))
        else:
            layers.append(GkrLayer(3, None, sec(cols[0])))
    p, d = GkrOps.prove_batch(layers)
    assert hashlib.sha256(p).hexdigest() == GOLDEN[name]["sha256"]
    assert d.hex() == GOLDEN[name]["final_digest"]
