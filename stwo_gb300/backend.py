"""`CudaBackend`: the reference's backend trait family over the C ABI, for Python callers.

Method names and argument meaning follow the reference traits (crates/prover/src/core/backend/
mod.rs:19-65 and the trait homes cited per method). Columns are 1-D torch int32 tensors on the
GPU holding canonical M31 words; torch only provides device memory and the stream. Every
operation runs in libstwo_gb300.so; nothing here computes on the CPU beyond O(1) index
arithmetic, and a missing library raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import torch

from . import _lib
from ._lib import Coset, QM31, QM31Point, SampleBatch, call
from .circle import canonic_half_coset

QM31T = Tuple[int, int, int, int]


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptrs(tensors: Sequence[torch.Tensor]):
    arr = (C.c_void_p * max(1, len(tensors)))()
    for i, t in enumerate(tensors):
        assert t.is_cuda and t.dtype == torch.int32 and t.is_contiguous()
        arr[i] = t.data_ptr()
    return arr


def _q(x: QM31T) -> QM31:
    q = QM31()
    for i in range(4):
        q.v[i] = int(x[i])
    return q


def _point(p) -> QM31Point:
    (x, y) = p
    return QM31Point(_q(x), _q(y))


def zeros(n: int) -> torch.Tensor:
    return torch.zeros(n, dtype=torch.int32, device="cuda")


def empty(n: int) -> torch.Tensor:
    return torch.empty(n, dtype=torch.int32, device="cuda")


@dataclass
class SecureColumn:
    """SecureColumnByCoords (crates/prover/src/core/fields/secure_column.rs:15): 4 M31 columns."""

    cols: List[torch.Tensor]

    @staticmethod
    def zeros(n: int) -> "SecureColumn":
        return SecureColumn([zeros(n) for _ in range(4)])

    def __len__(self) -> int:
        return self.cols[0].numel()


class TwiddleTree:
    """PolyOps::Twiddles resident in HBM (crates/prover/src/core/poly/twiddles.rs:9-14)."""

    def __init__(self, root: Coset):
        h = C.c_void_p()
        call("stwo_twiddles_precompute", root, C.byref(h), _stream())
        self.handle = h
        self.root = root

    def arrays(self):
        tw, itw, n = C.c_void_p(), C.c_void_p(), C.c_size_t()
        call("stwo_twiddles_info", self.handle, None, C.byref(tw), C.byref(itw), C.byref(n))
        return tw.value, itw.value, n.value

    def __del__(self):
        try:
            if self.handle:
                _lib.load().stwo_twiddles_free(self.handle)
        except Exception:
            pass


class CudaBackend:
    """Static backend methods, as the reference's zero-sized backend types."""

    # ------------------------------------------------------------ PolyOps (poly/circle/ops.rs:13-69)
    @staticmethod
    def precompute_twiddles(coset: Coset) -> TwiddleTree:
        return TwiddleTree(coset)

    @staticmethod
    def interpolate_columns(columns: Sequence[torch.Tensor], domain_half: Coset, twiddles: TwiddleTree) -> None:
        """In place: bit-reversed evaluations -> coefficients."""
        call("stwo_interpolate_columns", twiddles.handle, domain_half, _ptrs(columns), len(columns), _stream())

    @staticmethod
    def evaluate_polynomials(coeffs: Sequence[torch.Tensor], domain_half: Coset, twiddles: TwiddleTree,
                             out: Optional[Sequence[torch.Tensor]] = None) -> List[torch.Tensor]:
        n = 1 << (domain_half.log_size + 1)
        if out is None:
            out = [empty(n) for _ in coeffs]
        logc = coeffs[0].numel().bit_length() - 1 if coeffs else 0
        call("stwo_evaluate_columns", twiddles.handle, domain_half, _ptrs(coeffs), logc, _ptrs(out), len(coeffs),
             _stream())
        return list(out)

    @staticmethod
    def extend(coeffs: torch.Tensor, log_size: int) -> torch.Tensor:
        out = empty(1 << log_size)
        call("stwo_extend", coeffs.data_ptr(), coeffs.numel().bit_length() - 1, out.data_ptr(), log_size, _stream())
        return out

    @staticmethod
    def eval_at_points(polys: Sequence[torch.Tensor], queries: Sequence[Tuple[int, tuple]]) -> List[QM31T]:
        """queries: (poly index, ((x0..x3), (y0..y3))) pairs -> values."""
        n = len(queries)
        logs = (C.c_uint32 * max(1, len(polys)))(*[p.numel().bit_length() - 1 for p in polys])
        poly_of = (C.c_uint32 * max(1, n))(*[q[0] for q in queries])
        pts = (QM31Point * max(1, n))(*[_point(q[1]) for q in queries])
        out = (QM31 * max(1, n))()
        call("stwo_eval_at_points", _ptrs(polys), logs, len(polys), poly_of, pts, n, out, _stream())
        return [tuple(out[i].v) for i in range(n)]

    # ------------------------------------------------------------ ColumnOps (backend/mod.rs:38-44)
    @staticmethod
    def bit_reverse_column(col: torch.Tensor) -> None:
        call("stwo_bit_reverse_column", col.data_ptr(), col.numel().bit_length() - 1, _stream())

    # ------------------------------------------------------------ MerkleOps (vcs/ops.rs:25-46)
    @staticmethod
    def commit_on_layer(log_size: int, prev_layer: Optional[torch.Tensor], columns: Sequence[torch.Tensor],
                        out: Optional[torch.Tensor] = None) -> torch.Tensor:
        if out is None:
            out = torch.empty((1 << log_size, 8), dtype=torch.int32, device="cuda")
        call("stwo_merkle_commit_layer", log_size, prev_layer.data_ptr() if prev_layer is not None else None,
             _ptrs(columns), len(columns), out.data_ptr(), _stream())
        return out

    # ------------------------------------------------------------ FriOps (fri.rs:92-139)
    @staticmethod
    def fold_line(eval_: SecureColumn, line_domain: Coset, alpha: QM31T, twiddles: TwiddleTree) -> SecureColumn:
        out = SecureColumn([empty(len(eval_) // 2) for _ in range(4)])
        call("stwo_fri_fold_line", twiddles.handle, line_domain, _ptrs(eval_.cols), _q(alpha), _ptrs(out.cols),
             _stream())
        return out

    @staticmethod
    def fold_circle_into_line(dst: SecureColumn, src: SecureColumn, src_half: Coset, alpha: QM31T,
                              twiddles: TwiddleTree) -> None:
        call("stwo_fri_fold_circle_into_line", twiddles.handle, src_half, _ptrs(dst.cols), _ptrs(src.cols),
             _q(alpha), _stream())

    @staticmethod
    def decompose(eval_: SecureColumn) -> Tuple[SecureColumn, QM31T]:
        g = SecureColumn([empty(len(eval_)) for _ in range(4)])
        lam = QM31()
        call("stwo_fri_decompose", _ptrs(eval_.cols), len(eval_).bit_length() - 1, _ptrs(g.cols), C.byref(lam),
             _stream())
        return g, tuple(lam.v)

    # ------------------------------------------------------------ QuotientOps (pcs/quotients.rs:21-35)
    @staticmethod
    def accumulate_quotients(domain_log_size: int, columns: Sequence[torch.Tensor], random_coeff: QM31T,
                             sample_batches, log_blowup_factor: int) -> SecureColumn:
        """sample_batches: [(point, [(column_index, value), ...]), ...] in BTreeMap order."""
        n = 1 << domain_log_size
        out = SecureColumn([empty(n) for _ in range(4)])
        keep = []
        arr = (SampleBatch * max(1, len(sample_batches)))()
        for i, (pt, cv) in enumerate(sample_batches):
            idx = (C.c_uint32 * max(1, len(cv)))(*[c for c, _ in cv])
            vals = (QM31 * max(1, len(cv)))(*[_q(v) for _, v in cv])
            keep += [idx, vals]
            arr[i] = SampleBatch(_point(pt), len(cv), idx, vals)
        call("stwo_accumulate_quotients", domain_log_size, _ptrs(columns), len(columns), _q(random_coeff), arr,
             len(sample_batches), log_blowup_factor, _ptrs(out.cols), _stream())
        return out

    # ------------------------------------------------------------ AccumulationOps (air/accumulation.rs:151-158)
    @staticmethod
    def accumulate(acc: SecureColumn, other: SecureColumn) -> None:
        call("stwo_secure_accumulate", _ptrs(acc.cols), _ptrs(other.cols), len(acc), _stream())

    @staticmethod
    def generate_secure_powers(felt: QM31T, n_powers: int) -> List[QM31T]:
        out = (QM31 * max(1, n_powers))()
        call("stwo_generate_secure_powers", _q(felt), n_powers, out, _stream())
        return [tuple(out[i].v) for i in range(n_powers)]

    # ------------------------------------------------------------ GrindOps (proof_of_work.rs:3-7)
    @staticmethod
    def grind(digest_words: Sequence[int], pow_bits: int) -> int:
        d = (C.c_uint32 * 8)(*digest_words)
        nonce = C.c_uint64()
        call("stwo_grind_blake2s", d, pow_bits, C.byref(nonce), _stream())
        return nonce.value


GRAND_PRODUCT, LOGUP_GENERIC, LOGUP_MULTIPLICITIES, LOGUP_SINGLES = 0, 1, 2, 3


@dataclass
class GkrLayer:
    """Layer (crates/prover/src/core/lookups/gkr_prover.rs:94-108): `num` is the grand product's
    column, the secure numerators, or (multiplicities) a base column; `den` the denominators."""

    kind: int
    num: Optional[object] = None
    den: Optional[SecureColumn] = None

    def __len__(self) -> int:
        col = self.num if self.kind == GRAND_PRODUCT else self.den
        return col.numel() if isinstance(col, torch.Tensor) else len(col)

    def n_variables(self) -> int:
        return len(self).bit_length() - 1

    def _num_ptrs(self):
        if self.kind == LOGUP_SINGLES:
            return None
        if self.kind == LOGUP_MULTIPLICITIES:
            return _ptrs([self.num] * 4)
        return _ptrs(self.num.cols)

    def _den_ptrs(self):
        return None if self.kind == GRAND_PRODUCT else _ptrs(self.den.cols)


class GkrOps:
    """GkrOps (gkr_prover.rs:22-42) and MleOps (lookups/mle.rs:9-14) on the GPU."""

    @staticmethod
    def gen_eq_evals(y: Sequence[QM31T], v: QM31T) -> SecureColumn:
        out = SecureColumn([empty(1 << len(y)) for _ in range(4)])
        arr = (QM31 * max(1, len(y)))(*[_q(x) for x in y])
        call("stwo_gkr_gen_eq_evals", arr, len(y), _q(v), _ptrs(out.cols), _stream())
        return out

    @staticmethod
    def next_layer(layer: GkrLayer) -> GkrLayer:
        h = len(layer) // 2
        num = SecureColumn([empty(h) for _ in range(4)])
        if layer.kind == GRAND_PRODUCT:
            call("stwo_gkr_next_layer", layer.kind, layer.n_variables(), layer._num_ptrs(), None, _ptrs(num.cols),
                 None, _stream())
            return GkrLayer(GRAND_PRODUCT, num)
        den = SecureColumn([empty(h) for _ in range(4)])
        call("stwo_gkr_next_layer", layer.kind, layer.n_variables(), layer._num_ptrs(), layer._den_ptrs(),
             _ptrs(num.cols), _ptrs(den.cols), _stream())
        return GkrLayer(LOGUP_GENERIC, num, den)

    @staticmethod
    def sum_as_poly_in_first_variable(layer: GkrLayer, eq_evals: SecureColumn, y: Sequence[QM31T], lam: QM31T,
                                      eq_fixed_var_correction: QM31T, claim: QM31T) -> List[QM31T]:
        ys = (QM31 * max(1, len(y)))(*[_q(x) for x in y])
        coeffs = (QM31 * 4)()
        n = C.c_uint32()
        call("stwo_gkr_sum_as_poly_in_first_variable", layer.kind, layer.n_variables(), layer._num_ptrs(),
             layer._den_ptrs(), _ptrs(eq_evals.cols), ys, len(y), _q(lam), _q(eq_fixed_var_correction), _q(claim),
             coeffs, C.byref(n), _stream())
        return [tuple(coeffs[i].v) for i in range(n.value)]

    @staticmethod
    def fix_first_variable(mle, assignment: QM31T) -> SecureColumn:
        if isinstance(mle, torch.Tensor):
            n = mle.numel()
            out = SecureColumn([empty(n // 2) for _ in range(4)])
            call("stwo_mle_fix_first_variable_base", n.bit_length() - 1, C.c_void_p(mle.data_ptr()), _q(assignment),
                 _ptrs(out.cols), _stream())
            return out
        n = len(mle)
        out = SecureColumn([empty(n // 2) for _ in range(4)])
        call("stwo_mle_fix_first_variable_secure", n.bit_length() - 1, _ptrs(mle.cols), _q(assignment),
             _ptrs(out.cols), _stream())
        return out

    @staticmethod
    def prove_batch(layers: Sequence[GkrLayer], digest: Optional[bytes] = None,
                    capacity: int = 16 << 20) -> Tuple[bytes, bytes]:
        """gkr_prover::prove_batch: (canonical proof + artifact bytes, final channel digest)."""
        k = len(layers)
        kinds = (C.c_uint32 * k)(*[l.kind for l in layers])
        logs = (C.c_uint32 * k)(*[l.n_variables() for l in layers])
        nums = (C.c_void_p * (4 * k))()
        dens = (C.c_void_p * (4 * k))()
        for i, l in enumerate(layers):
            if isinstance(l.num, torch.Tensor):
                nums[4 * i] = l.num.data_ptr()
            elif l.num is not None:
                for c in range(4):
                    nums[4 * i + c] = l.num.cols[c].data_ptr()
            if l.den is not None:
                for c in range(4):
                    dens[4 * i + c] = l.den.cols[c].data_ptr()
        out = (C.c_uint8 * capacity)()
        n = C.c_size_t()
        din = (C.c_uint8 * 32).from_buffer_copy(digest) if digest is not None else None
        dout = (C.c_uint8 * 32)()
        call("stwo_gkr_prove_batch", k, kinds, logs, nums, dens, din, out, capacity, C.byref(n), dout, _stream())
        return bytes(out[:n.value]), bytes(dout)


def canonic_twiddles(log_size: int) -> TwiddleTree:
    """Twiddles for CanonicCoset(log_size).circle_domain() and every domain it doubles into."""
    return TwiddleTree(canonic_half_coset(log_size))
