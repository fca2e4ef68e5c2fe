"""The reference's prove() driven through the per-operation C ABI (stwo_gb300/host_prover.py):
interpolate / evaluate / commit_on_layer / eval_at_points / accumulate_quotients / FRI folds / grind /
generate_secure_powers plus the per-component stwo_eval_constraints, with device memory from the
column model only. Its proof bytes equal the oracle's and those of the fused device prover
(stwo_prove_wide_fib) on the same trace, for blowup factors 1 (the composition evaluated on the
committed domain) and 2 (the component extends its trace first)."""
import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("log_n,n_cols,cfg", [(3, 3, (5, 1, 0, 3)), (5, 10, (5, 1, 0, 3)), (8, 100, (5, 1, 0, 3)),
                                              (6, 20, (8, 2, 1, 5)), (10, 16, (5, 1, 0, 3))])
def test_host_prover_matches_oracle_and_fused_prover(cuda, oracle, log_n, n_cols, cfg):
    import torch

    from stwo_gb300 import host_prover
    from stwo_gb300.prover import prove_wide_fib, wide_fib_trace

    rng = np.random.default_rng(4000 + 13 * log_n + n_cols)
    a = F.rand_m31(rng, 1 << log_n)
    b = F.rand_m31(rng, 1 << log_n)
    da = torch.from_numpy(a.view(np.int32)).cuda()
    db = torch.from_numpy(b.view(np.int32)).cuda()
    got = host_prover.prove_wide_fib(log_n, n_cols, da.data_ptr(), db.data_ptr(), cfg)
    want = oracle.prove_wide_fib(log_n, n_cols, a, b, cfg)
    assert got == want
    fused = prove_wide_fib(log_n, wide_fib_trace(log_n, n_cols, da, db), cfg)
    assert fused == want
    ok, why = oracle.verify_wide_fib(log_n, n_cols, got)
    assert ok, why


@pytest.mark.parametrize("log_n,n_cols,cfg", [(5, 10, (5, 1, 0, 3)), (8, 100, (5, 1, 0, 3)), (6, 20, (8, 2, 1, 5))])
def test_host_prover_with_generated_constraints_matches_oracle(cuda, oracle, log_n, n_cols, cfg):
    """The same prove() with the component's constraints generated from its recorded expressions
    (generated domain kernel, expression evaluation at the out-of-domain point): the proof bytes
    equal the oracle's."""
    import torch

    from stwo_gb300 import host_prover

    rng = np.random.default_rng(4100 + 13 * log_n + n_cols)
    a = F.rand_m31(rng, 1 << log_n)
    b = F.rand_m31(rng, 1 << log_n)
    da = torch.from_numpy(a.view(np.int32)).cuda()
    db = torch.from_numpy(b.view(np.int32)).cuda()
    got = host_prover.prove_wide_fib(log_n, n_cols, da.data_ptr(), db.data_ptr(), cfg, generated=True)
    assert got == oracle.prove_wide_fib(log_n, n_cols, a, b, cfg)
