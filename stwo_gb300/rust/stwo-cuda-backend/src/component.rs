//! ComponentProver<CudaBackend>: the per-component constraint evaluation on the domain
//! (crates/prover/src/core/air/mod.rs:59-62; the SIMD implementation is
//! crates/prover/src/constraint_framework/component.rs:278-416). Its steps are kept — extend the
//! component's columns to the evaluation domain, take the accumulator's slice of random-coefficient
//! powers — and the row evaluation is one library call:
//!   * `CudaAir` components (wide-Fibonacci, Poseidon2, Blake2s round) use the hand-written kernels
//!     through `stwo_eval_constraints`;
//!   * `Generated<E>` wraps any FrameworkEval whose kernel was generated from its recorded
//!     expressions (stwo_gb300/codegen.py emits the source; this side compiles or loads it) and runs
//!     it through `stwo_eval_constraints_codegen`.

use std::ffi::CString;
use std::ptr::null_mut;

use itertools::Itertools;
use stwo_prover::constraint_framework::{FrameworkComponent, FrameworkEval, PREPROCESSED_TRACE_IDX};
use stwo_prover::core::air::accumulation::{DomainEvaluationAccumulator, PointEvaluationAccumulator};
use stwo_prover::core::air::{Component, ComponentProver, Trace};
use stwo_prover::core::backend::Column;
use stwo_prover::core::circle::CirclePoint;
use stwo_prover::core::fields::m31::BaseField;
use stwo_prover::core::fields::qm31::SecureField;
use stwo_prover::core::pcs::TreeVec;
use stwo_prover::core::poly::circle::{CanonicCoset, CircleDomain, PolyOps};
use stwo_prover::core::ColumnVec;

use crate::column::CudaColumn;
use crate::ffi::*;
use crate::ops::coords_mut;
use crate::{qm31, CudaBackend};

/// The component's columns (preprocessed by index, then its trace subtrees) on `eval_domain`,
/// extended where the committed domain differs (component.rs:305-322). Tree by tree, each tree's
/// columns land in one contiguous block, which the hand-written Poseidon2 and Blake2s-round kernels
/// require.
fn extended_columns<E: FrameworkEval>(
    component: &FrameworkComponent<E>,
    trace: &Trace<'_, CudaBackend>,
    eval_domain: CircleDomain,
) -> (Vec<CudaColumn<BaseField>>, Vec<*const u32>) {
    let mut polys = trace.polys.sub_tree(component.trace_locations());
    polys[PREPROCESSED_TRACE_IDX] = component
        .preproccessed_column_indices()
        .iter()
        .map(|&i| trace.polys[PREPROCESSED_TRACE_IDX][i])
        .collect();
    let twiddles = CudaBackend::precompute_twiddles(eval_domain.half_coset);
    let mut blocks = Vec::new();
    let mut ptrs = Vec::new();
    for tree in polys.iter() {
        if tree.is_empty() {
            continue;
        }
        let block = unsafe { CudaColumn::<BaseField>::uninitialized(tree.len() * eval_domain.size()) };
        let by_log = tree.iter().enumerate().into_group_map_by(|(_, p)| p.log_size());
        for (log, group) in by_log {
            let src: Vec<*const u32> = group.iter().map(|(_, p)| p.coeffs.ptr()).collect();
            let dst: Vec<*mut u32> =
                group.iter().map(|(i, _)| unsafe { block.ptr.add(i * eval_domain.size()) }).collect();
            check(unsafe {
                stwo_evaluate_columns(crate::poly::handle(&twiddles), crate::poly::coset(&eval_domain.half_coset),
                                      src.as_ptr(), log, dst.as_ptr(), dst.len() as u32, null_mut())
            });
        }
        for i in 0..tree.len() {
            ptrs.push(unsafe { block.ptr.add(i * eval_domain.size()) as *const u32 });
        }
        blocks.push(block);
    }
    (blocks, ptrs)
}

/// An AIR whose constraints the library evaluates with a hand-written kernel.
pub trait CudaAir: FrameworkEval {
    /// STWO_AIR_WIDE_FIB (n_cols = N), STWO_AIR_POSEIDON (elements z, alpha) or STWO_AIR_BLAKE_ROUND
    /// (z, alpha of RoundElements, then of BlakeXorElements 12, 9, 8, 7, 4).
    fn descriptor(&self) -> (u32, u32, Vec<StwoQm31>);
}

impl<E: CudaAir + Sync> ComponentProver<CudaBackend> for FrameworkComponent<E> {
    fn evaluate_constraint_quotients_on_domain(
        &self,
        trace: &Trace<'_, CudaBackend>,
        evaluation_accumulator: &mut DomainEvaluationAccumulator<CudaBackend>,
    ) {
        if self.n_constraints() == 0 {
            return;
        }
        let eval_domain = CanonicCoset::new(self.max_constraint_log_degree_bound()).circle_domain();
        let (_blocks, cols) = extended_columns(self, trace, eval_domain);
        let (air, n_cols, elements) = self.descriptor();
        let comp = StwoComponent {
            air,
            log_n_rows: self.log_size(),
            n_cols,
            claimed_sum: qm31(self.claimed_sum()),
            h_elements: elements.as_ptr(),
            n_elements: elements.len() as u32,
        };
        let [mut accum] = evaluation_accumulator.columns([(eval_domain.log_size(), self.n_constraints())]);
        // The accumulator's slice as it comes: the entry point reverses it (component.rs:331).
        let powers: Vec<StwoQm31> = accum.random_coeff_powers.iter().map(|&p| qm31(p)).collect();
        check(unsafe {
            stwo_eval_constraints(&comp, cols.as_ptr(), cols.len() as u32, powers.as_ptr(), powers.len() as u32,
                                  coords_mut(accum.col).as_ptr(), null_mut())
        });
    }
}

/// A framework component with a generated constraint kernel: the emitted source (or a cached cubin)
/// and the values of the formal parameters its constraints name, in the emitter's order.
pub struct Generated<E: FrameworkEval> {
    pub inner: FrameworkComponent<E>,
    handle: Codegen,
    params: Vec<StwoQm31>,
}

unsafe impl<E: FrameworkEval + Sync> Sync for Generated<E> {}

impl<E: FrameworkEval> Generated<E> {
    /// Compiles `source` (NVRTC, sm_103a). `params` are the values of the emitter's parameter list:
    /// relation elements as `<relation>_z`, `<relation>_alpha{i}`, then `claimed_sum` and
    /// `column_size` = 2^log_size where the component has a LogUp relation.
    pub fn new(inner: FrameworkComponent<E>, source: &str, n_cols: u32, params: Vec<SecureField>) -> Self {
        let src = CString::new(source).unwrap();
        let mut handle = null_mut();
        check(unsafe {
            stwo_codegen_compile(src.as_ptr(), n_cols, params.len() as u32, inner.n_constraints() as u32, 1,
                                 &mut handle)
        });
        Self { inner, handle, params: params.into_iter().map(qm31).collect() }
    }
}

impl<E: FrameworkEval> Drop for Generated<E> {
    fn drop(&mut self) {
        unsafe { stwo_codegen_destroy(self.handle) };
    }
}

impl<E: FrameworkEval> Component for Generated<E> {
    fn n_constraints(&self) -> usize {
        self.inner.n_constraints()
    }
    fn max_constraint_log_degree_bound(&self) -> u32 {
        self.inner.max_constraint_log_degree_bound()
    }
    fn trace_log_degree_bounds(&self) -> TreeVec<ColumnVec<u32>> {
        self.inner.trace_log_degree_bounds()
    }
    fn mask_points(&self, point: CirclePoint<SecureField>) -> TreeVec<ColumnVec<Vec<CirclePoint<SecureField>>>> {
        self.inner.mask_points(point)
    }
    fn preproccessed_column_indices(&self) -> ColumnVec<usize> {
        self.inner.preproccessed_column_indices()
    }
    fn evaluate_constraint_quotients_at_point(
        &self,
        point: CirclePoint<SecureField>,
        mask: &TreeVec<ColumnVec<Vec<SecureField>>>,
        evaluation_accumulator: &mut PointEvaluationAccumulator,
    ) {
        // The out-of-domain point stays on the host, as in the reference.
        self.inner.evaluate_constraint_quotients_at_point(point, mask, evaluation_accumulator)
    }
}

impl<E: FrameworkEval + Sync> ComponentProver<CudaBackend> for Generated<E> {
    fn evaluate_constraint_quotients_on_domain(
        &self,
        trace: &Trace<'_, CudaBackend>,
        evaluation_accumulator: &mut DomainEvaluationAccumulator<CudaBackend>,
    ) {
        if self.n_constraints() == 0 {
            return;
        }
        let eval_domain = CanonicCoset::new(self.max_constraint_log_degree_bound()).circle_domain();
        let (_blocks, cols) = extended_columns(&self.inner, trace, eval_domain);
        let [mut accum] = evaluation_accumulator.columns([(eval_domain.log_size(), self.n_constraints())]);
        let powers: Vec<StwoQm31> = accum.random_coeff_powers.iter().map(|&p| qm31(p)).collect();
        check(unsafe {
            stwo_eval_constraints_codegen(self.handle, self.inner.log_size(), eval_domain.log_size(), cols.as_ptr(),
                                          cols.len() as u32, self.params.as_ptr(), self.params.len() as u32,
                                          powers.as_ptr(), powers.len() as u32, coords_mut(accum.col).as_ptr(),
                                          null_mut())
        });
    }
}
