//! PolyOps (crates/prover/src/core/poly/circle/ops.rs:13-69): twiddle trees resident in HBM, circle
//! FFT / IFFT, point evaluation and extension, each one call into the library.

use std::collections::BTreeMap;
use std::ptr::null_mut;
use std::sync::Arc;

use stwo_prover::core::backend::Column;
use stwo_prover::core::circle::{CirclePoint, Coset};
use stwo_prover::core::fields::m31::BaseField;
use stwo_prover::core::fields::qm31::SecureField;
use stwo_prover::core::poly::circle::{CircleDomain, CircleEvaluation, CirclePoly, PolyOps};
use stwo_prover::core::poly::twiddles::TwiddleTree;
use stwo_prover::core::poly::BitReversedOrder;
use stwo_prover::core::ColumnVec;

use crate::column::CudaColumn;
use crate::ffi::*;
use crate::{from_qm31, qm31, CudaBackend};

/// A twiddle tree in HBM (the library caches trees per root coset and device).
pub struct TreeHandle(pub(crate) Tree);
unsafe impl Send for TreeHandle {}
unsafe impl Sync for TreeHandle {}
impl Drop for TreeHandle {
    fn drop(&mut self) {
        unsafe { stwo_twiddles_free(self.0) };
    }
}

/// B::Twiddles: one handle serves both directions (the tree holds the inverses too).
#[derive(Clone)]
pub struct CudaTwiddles(pub Arc<TreeHandle>);

pub(crate) fn coset(c: &Coset) -> StwoCoset {
    StwoCoset { initial_index: c.initial_index.0 as u32, step_size: c.step_size.0 as u32, log_size: c.log_size }
}

pub(crate) fn handle(t: &TwiddleTree<CudaBackend>) -> Tree {
    t.twiddles.0 .0
}

impl PolyOps for CudaBackend {
    type Twiddles = CudaTwiddles;

    fn interpolate(
        eval: CircleEvaluation<Self, BaseField, BitReversedOrder>,
        itwiddles: &TwiddleTree<Self>,
    ) -> CirclePoly<Self> {
        let mut values = eval.values;
        let cols = [values.ptr_mut()];
        check(unsafe {
            stwo_interpolate_columns(handle(itwiddles), coset(&eval.domain.half_coset), cols.as_ptr(), 1, null_mut())
        });
        CirclePoly::new(values)
    }

    fn interpolate_columns(
        columns: impl IntoIterator<Item = CircleEvaluation<Self, BaseField, BitReversedOrder>>,
        twiddles: &TwiddleTree<Self>,
    ) -> Vec<CirclePoly<Self>> {
        // One call per domain, in place: the columns of a tree share their domain.
        let evals: Vec<_> = columns.into_iter().collect();
        let mut by_domain: BTreeMap<(usize, usize, u32), Vec<usize>> = BTreeMap::new();
        for (i, e) in evals.iter().enumerate() {
            let h = &e.domain.half_coset;
            by_domain.entry((h.initial_index.0, h.step_size.0, h.log_size)).or_default().push(i);
        }
        let mut values: Vec<CudaColumn<BaseField>> = Vec::with_capacity(evals.len());
        let mut domains = Vec::with_capacity(evals.len());
        for e in evals {
            domains.push(e.domain);
            values.push(e.values);
        }
        for idx in by_domain.values() {
            let ptrs: Vec<*mut u32> = idx.iter().map(|&i| values[i].ptr_mut()).collect();
            check(unsafe {
                stwo_interpolate_columns(handle(twiddles), coset(&domains[idx[0]].half_coset), ptrs.as_ptr(),
                                         ptrs.len() as u32, null_mut())
            });
        }
        values.into_iter().map(CirclePoly::new).collect()
    }

    fn eval_at_point(poly: &CirclePoly<Self>, point: CirclePoint<SecureField>) -> SecureField {
        let ptrs = [poly.coeffs.ptr()];
        let logs = [poly.log_size()];
        let poly_of = [0u32];
        let pts = [StwoQm31Point { x: qm31(point.x), y: qm31(point.y) }];
        let mut out = StwoQm31::default();
        check(unsafe {
            stwo_eval_at_points(ptrs.as_ptr(), logs.as_ptr(), 1, poly_of.as_ptr(), pts.as_ptr(), 1, &mut out,
                                null_mut())
        });
        from_qm31(out)
    }

    fn extend(poly: &CirclePoly<Self>, log_size: u32) -> CirclePoly<Self> {
        assert!(log_size >= poly.log_size());
        let mut out = unsafe { CudaColumn::<BaseField>::uninitialized(1 << log_size) };
        check(unsafe { stwo_extend(poly.coeffs.ptr(), poly.log_size(), out.ptr_mut(), log_size, null_mut()) });
        CirclePoly::new(out)
    }

    fn evaluate(
        poly: &CirclePoly<Self>,
        domain: CircleDomain,
        twiddles: &TwiddleTree<Self>,
    ) -> CircleEvaluation<Self, BaseField, BitReversedOrder> {
        let mut out = unsafe { CudaColumn::<BaseField>::uninitialized(domain.size()) };
        let src = [poly.coeffs.ptr()];
        let dst = [out.ptr_mut()];
        check(unsafe {
            stwo_evaluate_columns(handle(twiddles), coset(&domain.half_coset), src.as_ptr(), poly.log_size(),
                                  dst.as_ptr(), 1, null_mut())
        });
        CircleEvaluation::new(domain, out)
    }

    fn evaluate_polynomials(
        polynomials: &ColumnVec<CirclePoly<Self>>,
        log_blowup_factor: u32,
        twiddles: &TwiddleTree<Self>,
    ) -> Vec<CircleEvaluation<Self, BaseField, BitReversedOrder>> {
        // One call per coefficient log size (one FFT launch sequence over all those columns).
        let mut outs: Vec<Option<CudaColumn<BaseField>>> = polynomials.iter().map(|_| None).collect();
        let mut by_log: BTreeMap<u32, Vec<usize>> = BTreeMap::new();
        for (i, p) in polynomials.iter().enumerate() {
            by_log.entry(p.log_size()).or_default().push(i);
        }
        for (&log, idx) in &by_log {
            let domain = stwo_prover::core::poly::circle::CanonicCoset::new(log + log_blowup_factor).circle_domain();
            let mut cols: Vec<CudaColumn<BaseField>> =
                idx.iter().map(|_| unsafe { CudaColumn::uninitialized(domain.size()) }).collect();
            let src: Vec<*const u32> = idx.iter().map(|&i| polynomials[i].coeffs.ptr()).collect();
            let dst: Vec<*mut u32> = cols.iter_mut().map(|c| c.ptr_mut()).collect();
            check(unsafe {
                stwo_evaluate_columns(handle(twiddles), coset(&domain.half_coset), src.as_ptr(), log, dst.as_ptr(),
                                      dst.len() as u32, null_mut())
            });
            for (&i, c) in idx.iter().zip(cols) {
                outs[i] = Some(c);
            }
        }
        outs.into_iter()
            .zip(polynomials.iter())
            .map(|(c, p)| {
                let domain =
                    stwo_prover::core::poly::circle::CanonicCoset::new(p.log_size() + log_blowup_factor).circle_domain();
                CircleEvaluation::new(domain, c.unwrap())
            })
            .collect()
    }

    fn precompute_twiddles(coset_: Coset) -> TwiddleTree<Self> {
        let mut t = null_mut();
        check(unsafe { stwo_twiddles_precompute(coset(&coset_), &mut t, null_mut()) });
        let h = CudaTwiddles(Arc::new(TreeHandle(t)));
        TwiddleTree { root_coset: coset_, twiddles: h.clone(), itwiddles: h }
    }
}
