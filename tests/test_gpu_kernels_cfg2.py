"""The kernel microbench at its own size, bit for bit against the oracle, through the C ABI.

Inputs are the benchmark's seeded words: 256 columns of 2^20 M31 values on the canonic coset of
log 20, interpolated, evaluated at blowup 4 (2^22 points each) and committed in one Blake2s
Merkle tree (16 compressions per leaf); and one QM31 circle evaluation of 2^22 points folded
into a 2^21 line and then line-folded down to 2^4 points with seeded alphas. The Merkle root
pins every evaluation word; every FRI layer is compared in full. The oracle runs the same pass
(its multi-threaded C++ restatement of the reference CPU backend).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_COLS, LOG, BLOWUP, FRI_LOG, FRI_LAST = 256, 20, 2, 22, 4


def test_kernel_microbench_full_size_matches_oracle(cuda, oracle):
    import torch

    from stwo_gb300.backend import CudaBackend as B, SecureColumn, TwiddleTree
    from stwo_gb300.circle import canonic_half_coset, double

    L = LOG + BLOWUP
    n = 1 << LOG
    inp = torch.empty((N_COLS, n), dtype=torch.int32, device="cuda")
    for c in range(N_COLS):
        inp[c].copy_(torch.from_numpy(oracle.gen_words(1, c, n).view(np.int32)))
    evals = torch.empty((N_COLS, 1 << L), dtype=torch.int32, device="cuda")
    tw = TwiddleTree(canonic_half_coset(L))
    small, big = canonic_half_coset(LOG), canonic_half_coset(L)
    cols = [inp[c] for c in range(N_COLS)]
    B.interpolate_columns(cols, small, tw)
    B.evaluate_polynomials(cols, big, tw, out=[evals[c] for c in range(N_COLS)])
    layer = B.commit_on_layer(L, None, [evals[c] for c in range(N_COLS)])
    for lg in range(L - 1, -1, -1):
        layer = B.commit_on_layer(lg, layer, [])
    root = layer.cpu().numpy().view(np.uint32).reshape(-1)
    del evals, inp

    fri_half = canonic_half_coset(FRI_LOG)
    fsrc = SecureColumn([torch.from_numpy(oracle.gen_words(1, 1000 + k, 1 << FRI_LOG).view(np.int32)).cuda()
                         for k in range(4)])
    aw = oracle.gen_words(1, 2000, 4 * FRI_LOG)
    alphas = [tuple(int(x) for x in aw[4 * j:4 * j + 4]) for j in range(FRI_LOG)]
    line = SecureColumn([torch.zeros(1 << (FRI_LOG - 1), dtype=torch.int32, device="cuda") for _ in range(4)])
    B.fold_circle_into_line(line, fsrc, fri_half, alphas[0], tw)
    got_layers = [np.stack([c.cpu().numpy().view(np.uint32) for c in line.cols])]
    cur, dom, j = line, fri_half, 1
    while len(cur) > (1 << FRI_LAST):
        cur = B.fold_line(cur, dom, alphas[j], tw)
        dom = double(dom)
        j += 1
        got_layers.append(np.stack([c.cpu().numpy().view(np.uint32) for c in cur.cols]))
    torch.cuda.synchronize()

    want_root, want_layers = oracle.cfg2_outputs(N_COLS, LOG, BLOWUP, FRI_LOG)
    assert np.array_equal(root, want_root), "Merkle root of the 256 x 2^22 evaluations differs"
    assert len(got_layers) == len(want_layers) == FRI_LOG - FRI_LAST
    for i, (g, w) in enumerate(zip(got_layers, want_layers)):
        assert np.array_equal(g, w), f"FRI layer {i} ({w.shape[1]} points) differs"
