"""Whole proofs of the reference's examples that have no hand-written device prover, from their
constraint-framework definitions alone: the Plonk example (preprocessed columns, LogUp in pairs)
and the state machine (two components of different sizes in one proof). Constraint evaluation
and the LogUp interaction trace run in generated kernels; the proof bytes equal the oracle's
restatement of prove_fibonacci_plonk / prove_state_machine (oracle/components.h)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("log_n,cfg", [(4, (5, 1, 0, 3)), (6, (5, 1, 0, 3)), (8, (8, 2, 1, 5)), (10, (5, 1, 0, 3))])
def test_plonk_proof_matches_oracle(cuda, oracle, log_n, cfg):
    from stwo_gb300 import framework_prover

    got, cs = framework_prover.prove_plonk(log_n, cfg)
    want, want_cs = oracle.prove_plonk(log_n, cfg)
    assert cs == want_cs
    assert got == want
    ok, why = oracle.verify_plonk(log_n, cs, got)
    assert ok, why


@pytest.mark.parametrize("log_n,initial,cfg", [(5, (0, 0), (5, 1, 0, 3)), (7, (17, 12), (5, 1, 0, 3)),
                                               (9, (123456, 7), (8, 2, 1, 5))])
def test_state_machine_proof_matches_oracle(cuda, oracle, log_n, initial, cfg):
    from stwo_gb300 import framework_prover

    got, sums = framework_prover.prove_state_machine(log_n, initial, cfg)
    want, want_sums = oracle.prove_state_machine(log_n, initial, cfg)
    assert sums == want_sums
    assert got == want
    ok, why = oracle.verify_state_machine(log_n, sums, got)
    assert ok, why
