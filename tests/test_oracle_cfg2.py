"""The oracle's kernel-microbench pass (the checker of the full-size GPU test) agrees with the
oracle's per-operation entry points on a small case: interpolate -> evaluate -> Merkle layers,
and the FRI fold chain layer by layer."""
import numpy as np

from tests import m31 as F


def test_cfg2_pass_equals_composed_ops(oracle):
    n_cols, log, blowup, fri_log = 3, 6, 2, 8
    L = log + blowup
    small, big = F.canonic_half(log), F.canonic_half(L)
    evals = []
    for c in range(n_cols):
        coeffs = oracle.interpolate(small, big, oracle.gen_words(1, c, 1 << log))
        evals.append(oracle.evaluate(big, big, coeffs))
    layer = oracle.commit_on_layer(L, None, evals)
    for lg in range(L - 1, -1, -1):
        layer = oracle.commit_on_layer(lg, layer, [])
    src = [oracle.gen_words(1, 1000 + k, 1 << fri_log) for k in range(4)]
    aw = oracle.gen_words(1, 2000, 4 * fri_log)
    alphas = [tuple(int(x) for x in aw[4 * j:4 * j + 4]) for j in range(fri_log)]
    fhalf = F.canonic_half(fri_log)
    line = oracle.fold_circle_into_line(fhalf, [np.zeros(1 << (fri_log - 1), np.uint32)] * 4, src, alphas[0])
    want = [np.stack(line)]
    dom, j = fhalf, 1
    while len(line[0]) > 16:
        line = oracle.fold_line(dom, line, alphas[j])
        dom = (2 * dom[0] % (1 << 31), 2 * dom[1] % (1 << 31), dom[2] - 1)
        j += 1
        want.append(np.stack(line))
    root, layers = oracle.cfg2_outputs(n_cols, log, blowup, fri_log)
    assert np.array_equal(root, np.asarray(layer).reshape(-1))
    assert len(layers) == len(want)
    for g, w in zip(layers, want):
        assert np.array_equal(g, w)
