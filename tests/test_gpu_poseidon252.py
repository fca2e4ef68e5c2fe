"""MerkleOps<Poseidon252MerkleHasher>::commit_on_layer and GrindOps<Poseidon252Channel>::grind on the
device (stwo_merkle_commit_layer_poseidon252, stwo_grind_poseidon252) against the oracle, bit for
bit. Layers cover no columns, fewer than one packed block (8 values), exact blocks, ragged blocks
and many columns, with and without a previous layer; grinding covers pow_bits 0..12."""
import ctypes as C

import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def _dev(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.uint32)).view(np.int32)).cuda()


def _felts(rng, n):
    """n canonical felts as n x 8 words (top limb masked below 2^250 < p)."""
    w = rng.integers(0, 1 << 32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
    w[:, 7] &= 0x03FFFFFF
    return w


@pytest.mark.parametrize("log,ncols,prev", [(0, 0, False), (0, 0, True), (3, 1, False), (4, 7, True), (5, 8, False),
                                            (5, 9, True), (6, 16, False), (4, 100, True), (10, 3, False),
                                            (12, 0, True), (14, 2, False)])
def test_commit_on_layer_poseidon252(cuda, oracle, log, ncols, prev):
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.backend import _ptrs, _stream

    rng = np.random.default_rng(2520 + 31 * log + ncols)
    n = 1 << log
    cols = [F.rand_m31(rng, n) for _ in range(ncols)]
    if ncols:
        cols[0][:2] = [0, F.P - 1][: min(2, n)]
    prev_np = _felts(rng, 2 * n) if prev else None
    out = torch.empty(n * 8, dtype=torch.int32, device="cuda")
    dcols = [_dev(c) for c in cols]
    dprev = _dev(prev_np) if prev else None
    st = _lib.load().stwo_merkle_commit_layer_poseidon252(log, dprev.data_ptr() if prev else None, _ptrs(dcols),
                                                          ncols, out.data_ptr(), _stream())
    assert st == 0, _lib.load().stwo_last_error()
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32).reshape(-1, 8)
    assert np.array_equal(got, oracle.p252_commit_on_layer(log, prev_np, cols))


@pytest.mark.parametrize("pow_bits", [0, 1, 4, 8, 12])
def test_grind_poseidon252(cuda, oracle, pow_bits):
    from stwo_gb300 import _lib

    rng = np.random.default_rng(2600 + pow_bits)
    d = _felts(rng, 1)[0]
    nonce = C.c_uint64()
    st = _lib.load().stwo_grind_poseidon252((C.c_uint32 * 8)(*[int(x) for x in d]), pow_bits, C.byref(nonce), None)
    assert st == 0, _lib.load().stwo_last_error()
    assert nonce.value == oracle.p252_grind(sum(int(v) << (32 * i) for i, v in enumerate(d)), pow_bits)
