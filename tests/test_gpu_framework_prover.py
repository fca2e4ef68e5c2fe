"""Whole proofs of the reference's examples that have no hand-written device prover, from their
constraint-framework definitions alone: the Plonk example (preprocessed columns, LogUp in pairs),
the state machine (two components of different sizes in one proof) and the full Blake example
(eight components of five sizes, preprocessed XOR tables). Constraint evaluation and the LogUp
interaction trace run in generated kernels; the proof bytes equal the oracle's restatement of
prove_fibonacci_plonk / prove_state_machine / prove_blake (oracle/components.h,
oracle/air_blake_full.h)."""
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


@pytest.mark.parametrize("log_n,cfg", [(4, (5, 1, 0, 3)), (5, (6, 2, 1, 4)), (7, (10, 2, 2, 8))])
def test_blake_proof_matches_oracle(cuda, oracle, log_n, cfg):
    """The full Blake example (scheduler, two round components, five XOR tables, preprocessed XOR
    tables) from its framework definitions: the claimed sums and the proof bytes equal the
    oracle's restatement of prove_blake, and the oracle's verify_blake accepts the proof."""
    from stwo_gb300 import framework_prover

    got, sums = framework_prover.prove_blake(log_n, cfg)
    want, want_sums = oracle.prove_blake(log_n, cfg)
    assert sums == want_sums
    assert got == want
    ok, why = oracle.verify_blake(log_n, sums, got)
    assert ok, why


@pytest.mark.parametrize("log_n", [4, 6, 10])
def test_blake_device_trace_matches_oracle(cuda, oracle, log_n):
    """stwo_gen_blake_example_trace (scheduler, round components, XOR multiplicities counted with
    atomics) equals the oracle's trace of prove_blake column for column."""
    import numpy as np

    from stwo_gb300 import framework_prover

    cols = framework_prover.blake_device_trace(log_n)
    got = np.concatenate([_download(c) for c in cols])
    pre = framework_prover.blake_preprocessed(log_n)
    want, k = oracle.blake_traces(log_n)
    assert k == len(pre) + len(cols)
    n_pre = sum(len(p) for p in pre)
    assert np.array_equal(np.concatenate(pre), want[:n_pre])
    assert np.array_equal(got, want[n_pre:])


def _download(buf):
    import ctypes as C

    import numpy as np

    from stwo_gb300.host_prover import call

    out = np.zeros(buf.n, np.uint32)
    call("stwo_buf_download", out.ctypes.data_as(C.c_void_p), buf.ptr, buf.n * 4, None)
    return out
