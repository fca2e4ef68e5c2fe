//! GkrOps and MleOps (crates/prover/src/core/lookups/{gkr_prover,mle}.rs) over the GKR kernels.
//! Secure MLE columns are four coordinate planes, which is what the ABI's `d[4]` arguments take.

use std::ptr::null_mut;

use stwo_prover::core::backend::Column;
use stwo_prover::core::fields::m31::BaseField;
use stwo_prover::core::fields::qm31::SecureField;
use stwo_prover::core::lookups::gkr_prover::{GkrMultivariatePolyOracle, GkrOps, Layer};
use stwo_prover::core::lookups::mle::{Mle, MleOps};
use stwo_prover::core::lookups::utils::UnivariatePoly;

use crate::column::CudaColumn;
use crate::ffi::*;
use crate::{from_qm31, qm31, CudaBackend};

type SecureCol = CudaColumn<SecureField>;

fn planes(c: &SecureCol) -> [*const u32; 4] {
    let p = c.planes4();
    [p[0], p[1], p[2], p[3]]
}

/// (kind, numerator planes, denominator planes) of a layer: kind 0 GrandProduct, 1 LogUpGeneric,
/// 2 LogUpMultiplicities (numerator plane 0 = the base column), 3 LogUpSingles.
fn layer_args(layer: &Layer<CudaBackend>) -> (u32, [*const u32; 4], [*const u32; 4]) {
    let none = [std::ptr::null(); 4];
    match layer {
        Layer::GrandProduct(m) => (0, planes(m), none),
        Layer::LogUpGeneric { numerators, denominators } => (1, planes(numerators), planes(denominators)),
        Layer::LogUpMultiplicities { numerators, denominators } => {
            (2, [numerators.ptr(), std::ptr::null(), std::ptr::null(), std::ptr::null()], planes(denominators))
        }
        Layer::LogUpSingles { denominators } => (3, none, planes(denominators)),
    }
}

impl GkrOps for CudaBackend {
    fn gen_eq_evals(y: &[SecureField], v: SecureField) -> Mle<Self, SecureField> {
        let out = unsafe { SecureCol::uninitialized(1 << y.len()) };
        let ys: Vec<StwoQm31> = y.iter().map(|&e| qm31(e)).collect();
        check(unsafe { stwo_gkr_gen_eq_evals(ys.as_ptr(), ys.len() as u32, qm31(v), out.planes4().as_ptr(), null_mut()) });
        Mle::new(out)
    }

    fn next_layer(layer: &Layer<Self>) -> Layer<Self> {
        let n = layer.n_variables() as u32;
        let (kind, num, den) = layer_args(layer);
        let half = 1usize << (n - 1);
        let next_num = unsafe { SecureCol::uninitialized(half) };
        let next_den = unsafe { SecureCol::uninitialized(half) };
        check(unsafe {
            stwo_gkr_next_layer(kind, n, num.as_ptr(), den.as_ptr(), next_num.planes4().as_ptr(),
                                next_den.planes4().as_ptr(), null_mut())
        });
        // A product layer folds into a product layer; every LogUp layer into a generic one.
        if kind == 0 {
            Layer::GrandProduct(Mle::new(next_num))
        } else {
            Layer::LogUpGeneric { numerators: Mle::new(next_num), denominators: Mle::new(next_den) }
        }
    }

    fn sum_as_poly_in_first_variable(
        h: &GkrMultivariatePolyOracle<'_, Self>,
        claim: SecureField,
    ) -> UnivariatePoly<SecureField> {
        let n = h.input_layer.n_variables() as u32;
        let (kind, num, den) = layer_args(&h.input_layer);
        let eq: &SecureCol = &h.eq_evals;
        let ys: Vec<StwoQm31> = h.eq_evals.y().iter().map(|&e| qm31(e)).collect();
        let mut coeffs = [StwoQm31::default(); 8];
        let mut n_coeffs = 0u32;
        check(unsafe {
            stwo_gkr_sum_as_poly_in_first_variable(kind, n, num.as_ptr(), den.as_ptr(), planes(eq).as_ptr(),
                                                   ys.as_ptr(), ys.len() as u32, qm31(h.lambda),
                                                   qm31(h.eq_fixed_var_correction), qm31(claim),
                                                   coeffs.as_mut_ptr(), &mut n_coeffs, null_mut())
        });
        UnivariatePoly::new(coeffs[..n_coeffs as usize].iter().map(|&c| from_qm31(c)).collect())
    }
}

impl MleOps<BaseField> for CudaBackend {
    fn fix_first_variable(mle: Mle<Self, BaseField>, assignment: SecureField) -> Mle<Self, SecureField> {
        let n = mle.n_variables() as u32;
        let out = unsafe { SecureCol::uninitialized(1 << (n - 1)) };
        check(unsafe {
            stwo_mle_fix_first_variable_base(n, mle.ptr(), qm31(assignment), out.planes4().as_ptr(), null_mut())
        });
        Mle::new(out)
    }
}

impl MleOps<SecureField> for CudaBackend {
    fn fix_first_variable(mle: Mle<Self, SecureField>, assignment: SecureField) -> Mle<Self, SecureField> {
        let n = mle.n_variables() as u32;
        let out = unsafe { SecureCol::uninitialized(1 << (n - 1)) };
        check(unsafe {
            stwo_mle_fix_first_variable_secure(n, planes(&mle).as_ptr(), qm31(assignment), out.planes4().as_ptr(),
                                               null_mut())
        });
        Mle::new(out)
    }
}
