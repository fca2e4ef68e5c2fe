//! ColumnOps, MerkleOps (Blake2s and Poseidon252), FriOps, QuotientOps, AccumulationOps and
//! GrindOps, each a call into the library (include/stwo_cuda.h cites the reference for each).

use std::ptr::{null, null_mut};

use starknet_ff::FieldElement as FieldElement252;
use stwo_prover::core::backend::{Col, Column, ColumnOps};
use stwo_prover::core::channel::{Blake2sChannel, Poseidon252Channel};
use stwo_prover::core::fields::m31::BaseField;
use stwo_prover::core::fields::qm31::SecureField;
use stwo_prover::core::fields::secure_column::SecureColumnByCoords;
use stwo_prover::core::fri::FriOps;
use stwo_prover::core::pcs::quotients::{ColumnSampleBatch, QuotientOps};
use stwo_prover::core::poly::circle::{CircleDomain, CircleEvaluation, SecureEvaluation};
use stwo_prover::core::poly::line::LineEvaluation;
use stwo_prover::core::poly::twiddles::TwiddleTree;
use stwo_prover::core::poly::BitReversedOrder;
use stwo_prover::core::air::accumulation::AccumulationOps;
use stwo_prover::core::proof_of_work::GrindOps;
use stwo_prover::core::vcs::blake2_hash::Blake2sHash;
use stwo_prover::core::vcs::blake2_merkle::Blake2sMerkleHasher;
use stwo_prover::core::vcs::ops::MerkleOps;
use stwo_prover::core::vcs::poseidon252_merkle::Poseidon252MerkleHasher;

use crate::column::{CudaColumn, DeviceWords};
use crate::ffi::*;
use crate::poly::{coset, handle};
use crate::{from_qm31, qm31, CudaBackend};

/// The four coordinate columns of a secure column, as the ABI's `d[4]` arguments.
pub(crate) fn coords(c: &SecureColumnByCoords<CudaBackend>) -> [*const u32; 4] {
    [c.columns[0].ptr(), c.columns[1].ptr(), c.columns[2].ptr(), c.columns[3].ptr()]
}
pub(crate) fn coords_mut(c: &mut SecureColumnByCoords<CudaBackend>) -> [*mut u32; 4] {
    let [a, b, c2, d] = &mut c.columns;
    [a.ptr_mut(), b.ptr_mut(), c2.ptr_mut(), d.ptr_mut()]
}
pub(crate) fn secure_uninit(len: usize) -> SecureColumnByCoords<CudaBackend> {
    SecureColumnByCoords { columns: std::array::from_fn(|_| unsafe { CudaColumn::uninitialized(len) }) }
}

impl ColumnOps<BaseField> for CudaBackend {
    type Column = CudaColumn<BaseField>;
    fn bit_reverse_column(column: &mut Self::Column) {
        check(unsafe { stwo_bit_reverse_column(column.ptr_mut(), column.len().ilog2(), null_mut()) });
    }
}

impl ColumnOps<SecureField> for CudaBackend {
    type Column = CudaColumn<SecureField>;
    fn bit_reverse_column(column: &mut Self::Column) {
        for k in 0..4 {
            check(unsafe { stwo_bit_reverse_column(column.plane(k), column.len().ilog2(), null_mut()) });
        }
    }
}

impl ColumnOps<Blake2sHash> for CudaBackend {
    type Column = CudaColumn<Blake2sHash>;
    fn bit_reverse_column(_column: &mut Self::Column) {
        unimplemented!("Merkle layers are never bit-reversed");
    }
}

impl DeviceWords for FieldElement252 {
    const WORDS: usize = 8;
    const PLANAR: bool = false;
    fn to_words(&self, out: &mut [u32]) {
        let be = self.to_bytes_be();
        for k in 0..8 {
            let o = 32 - 4 * (k + 1);
            out[k] = u32::from_be_bytes(be[o..o + 4].try_into().unwrap());
        }
    }
    fn from_words(w: &[u32]) -> Self {
        let mut be = [0u8; 32];
        for k in 0..8 {
            let o = 32 - 4 * (k + 1);
            be[o..o + 4].copy_from_slice(&w[k].to_be_bytes());
        }
        FieldElement252::from_bytes_be(&be).expect("canonical field element")
    }
}

impl ColumnOps<FieldElement252> for CudaBackend {
    type Column = CudaColumn<FieldElement252>;
    fn bit_reverse_column(_column: &mut Self::Column) {
        unimplemented!("Merkle layers are never bit-reversed");
    }
}

impl MerkleOps<Blake2sMerkleHasher> for CudaBackend {
    fn commit_on_layer(
        log_size: u32,
        prev_layer: Option<&Col<Self, Blake2sHash>>,
        columns: &[&Col<Self, BaseField>],
    ) -> Col<Self, Blake2sHash> {
        let mut out = unsafe { CudaColumn::<Blake2sHash>::uninitialized(1 << log_size) };
        let cols: Vec<*const u32> = columns.iter().map(|c| c.ptr()).collect();
        check(unsafe {
            stwo_merkle_commit_layer(log_size, prev_layer.map_or(null(), |p| p.ptr()), cols.as_ptr(),
                                     cols.len() as u32, out.ptr_mut(), null_mut())
        });
        out
    }
}

impl MerkleOps<Poseidon252MerkleHasher> for CudaBackend {
    fn commit_on_layer(
        log_size: u32,
        prev_layer: Option<&Col<Self, FieldElement252>>,
        columns: &[&Col<Self, BaseField>],
    ) -> Col<Self, FieldElement252> {
        let mut out = unsafe { CudaColumn::<FieldElement252>::uninitialized(1 << log_size) };
        let cols: Vec<*const u32> = columns.iter().map(|c| c.ptr()).collect();
        check(unsafe {
            stwo_merkle_commit_layer_poseidon252(log_size, prev_layer.map_or(null(), |p| p.ptr()), cols.as_ptr(),
                                                 cols.len() as u32, out.ptr_mut(), null_mut())
        });
        out
    }
}

impl FriOps for CudaBackend {
    fn fold_line(
        eval: &LineEvaluation<Self>,
        alpha: SecureField,
        twiddles: &TwiddleTree<Self>,
    ) -> LineEvaluation<Self> {
        let domain = eval.domain();
        let mut out = secure_uninit(eval.len() / 2);
        check(unsafe {
            stwo_fri_fold_line(handle(twiddles), coset(&domain.coset()), coords(&eval.values).as_ptr(), qm31(alpha),
                               coords_mut(&mut out).as_ptr(), null_mut())
        });
        LineEvaluation::new(domain.double(), out)
    }

    fn fold_circle_into_line(
        dst: &mut LineEvaluation<Self>,
        src: &SecureEvaluation<Self, BitReversedOrder>,
        alpha: SecureField,
        twiddles: &TwiddleTree<Self>,
    ) {
        check(unsafe {
            stwo_fri_fold_circle_into_line(handle(twiddles), coset(&src.domain.half_coset),
                                           coords_mut(&mut dst.values).as_ptr(), coords(&src.values).as_ptr(),
                                           qm31(alpha), null_mut())
        });
    }

    fn decompose(eval: &SecureEvaluation<Self, BitReversedOrder>) -> (SecureEvaluation<Self, BitReversedOrder>, SecureField) {
        let mut g = secure_uninit(eval.values.len());
        let mut lambda = StwoQm31::default();
        check(unsafe {
            stwo_fri_decompose(coords(&eval.values).as_ptr(), eval.domain.log_size(), coords_mut(&mut g).as_ptr(),
                               &mut lambda, null_mut())
        });
        (SecureEvaluation::new(eval.domain, g), from_qm31(lambda))
    }
}

impl QuotientOps for CudaBackend {
    fn accumulate_quotients(
        domain: CircleDomain,
        columns: &[&CircleEvaluation<Self, BaseField, BitReversedOrder>],
        random_coeff: SecureField,
        sample_batches: &[ColumnSampleBatch],
        log_blowup_factor: u32,
    ) -> SecureEvaluation<Self, BitReversedOrder> {
        // One StwoSampleBatch per ColumnSampleBatch, in the order given (the reference's BTreeMap
        // order by point).
        let idx: Vec<Vec<u32>> = sample_batches
            .iter()
            .map(|b| b.columns_and_values.iter().map(|(c, _)| *c as u32).collect())
            .collect();
        let vals: Vec<Vec<StwoQm31>> =
            sample_batches.iter().map(|b| b.columns_and_values.iter().map(|(_, v)| qm31(*v)).collect()).collect();
        let batches: Vec<StwoSampleBatch> = sample_batches
            .iter()
            .zip(idx.iter().zip(&vals))
            .map(|(b, (i, v))| StwoSampleBatch {
                point: StwoQm31Point { x: qm31(b.point.x), y: qm31(b.point.y) },
                n_columns: i.len() as u32,
                h_column_indices: i.as_ptr(),
                h_values: v.as_ptr(),
            })
            .collect();
        let cols: Vec<*const u32> = columns.iter().map(|c| c.values.ptr()).collect();
        let mut out = secure_uninit(domain.size());
        check(unsafe {
            stwo_accumulate_quotients(domain.log_size(), cols.as_ptr(), cols.len() as u32, qm31(random_coeff),
                                      batches.as_ptr(), batches.len() as u32, log_blowup_factor,
                                      coords_mut(&mut out).as_ptr(), null_mut())
        });
        SecureEvaluation::new(domain, out)
    }
}

impl AccumulationOps for CudaBackend {
    fn accumulate(column: &mut SecureColumnByCoords<Self>, other: &SecureColumnByCoords<Self>) {
        let n = column.len();
        check(unsafe { stwo_secure_accumulate(coords_mut(column).as_ptr(), coords(other).as_ptr(), n, null_mut()) });
    }

    fn generate_secure_powers(felt: SecureField, n_powers: usize) -> Vec<SecureField> {
        let mut out = vec![StwoQm31::default(); n_powers];
        check(unsafe { stwo_generate_secure_powers(qm31(felt), n_powers as u32, out.as_mut_ptr(), null_mut()) });
        out.into_iter().map(from_qm31).collect()
    }
}

impl GrindOps<Blake2sChannel> for CudaBackend {
    fn grind(channel: &Blake2sChannel, pow_bits: u32) -> u64 {
        let mut w = [0u32; 8];
        channel.digest().to_words(&mut w);
        let mut nonce = 0u64;
        check(unsafe { stwo_grind_blake2s(w.as_ptr(), pow_bits, &mut nonce, null_mut()) });
        nonce
    }
}

impl GrindOps<Poseidon252Channel> for CudaBackend {
    fn grind(channel: &Poseidon252Channel, pow_bits: u32) -> u64 {
        let mut w = [0u32; 8];
        channel.digest().to_words(&mut w);
        let mut nonce = 0u64;
        check(unsafe { stwo_grind_poseidon252(w.as_ptr(), pow_bits, &mut nonce, null_mut()) });
        nonce
    }
}
