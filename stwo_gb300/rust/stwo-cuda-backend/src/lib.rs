//! `CudaBackend`: stwo-prover's backend trait family on a GB300, through the C ABI of
//! libstwo_gb300.so (include/stwo_cuda.h). `prove::<CudaBackend, Blake2sMerkleChannel>` and the
//! reference's `verify()` run unchanged; every O(trace) backend call is one library call, and the
//! channel, decommitment walk and out-of-domain point evaluation stay on the host, as in the
//! reference.
//!
//! Trait map (reference file:line of each trait):
//!   ColumnOps / Column        core/backend/mod.rs:38-65         column.rs, ops.rs
//!   PolyOps                   core/poly/circle/ops.rs:13-69      poly.rs
//!   MerkleOps (Blake2s, Poseidon252) core/vcs/ops.rs:25-46     ops.rs
//!   FriOps                    core/fri.rs:92-139                ops.rs
//!   QuotientOps               core/pcs/quotients.rs:21-35        ops.rs
//!   AccumulationOps           core/air/accumulation.rs:151-158   ops.rs
//!   GkrOps / MleOps           core/lookups/gkr_prover.rs:22-42, mle.rs:9-14   gkr.rs
//!   GrindOps (Blake2s, Poseidon252) core/proof_of_work.rs:3-7   ops.rs
//!   ComponentProver           core/air/mod.rs:59-62             component.rs

pub mod column;
pub mod component;
pub mod ffi;
pub mod gkr;
pub mod ops;
pub mod poly;

use serde::{Deserialize, Serialize};
use stwo_prover::core::backend::{Backend, BackendForChannel};
use stwo_prover::core::fields::qm31::SecureField;
use stwo_prover::core::vcs::blake2_merkle::Blake2sMerkleChannel;
use stwo_prover::core::vcs::poseidon252_merkle::Poseidon252MerkleChannel;

pub use component::{CudaAir, Generated};
use ffi::StwoQm31;

#[derive(Copy, Clone, Debug, Serialize, Deserialize)]
pub struct CudaBackend;

impl Backend for CudaBackend {}
impl BackendForChannel<Blake2sMerkleChannel> for CudaBackend {}
impl BackendForChannel<Poseidon252MerkleChannel> for CudaBackend {}

/// Selects the GPU for the calling thread (before the first backend call).
pub fn init(device: i32) {
    ffi::check(unsafe { ffi::stwo_device_init(device) });
}

pub(crate) fn qm31(f: SecureField) -> StwoQm31 {
    let [a, b, c, d] = f.to_m31_array();
    StwoQm31 { v: [a.0, b.0, c.0, d.0] }
}

pub(crate) fn from_qm31(q: StwoQm31) -> SecureField {
    SecureField::from_u32_unchecked(q.v[0], q.v[1], q.v[2], q.v[3])
}
