//! The C ABI of libstwo_gb300.so, declared exactly as in include/stwo_cuda.h.
#![allow(non_camel_case_types)]

use std::ffi::{c_char, c_int, c_void, CStr};

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct StwoCoset {
    pub initial_index: u32,
    pub step_size: u32,
    pub log_size: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub struct StwoQm31 {
    pub v: [u32; 4],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct StwoQm31Point {
    pub x: StwoQm31,
    pub y: StwoQm31,
}

#[repr(C)]
pub struct StwoSampleBatch {
    pub point: StwoQm31Point,
    pub n_columns: u32,
    pub h_column_indices: *const u32,
    pub h_values: *const StwoQm31,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct StwoPcsConfig {
    pub pow_bits: u32,
    pub log_blowup_factor: u32,
    pub log_last_layer_degree_bound: u32,
    pub n_queries: u32,
}

#[repr(C)]
pub struct StwoComponent {
    pub air: u32,
    pub log_n_rows: u32,
    pub n_cols: u32,
    pub claimed_sum: StwoQm31,
    pub h_elements: *const StwoQm31,
    pub n_elements: u32,
}

pub type Status = i32;
pub type Tree = *mut c_void;
pub type Codegen = *mut c_void;
pub type Stream = *mut c_void;

pub const STWO_AIR_WIDE_FIB: u32 = 0;
pub const STWO_AIR_POSEIDON: u32 = 1;
pub const STWO_AIR_BLAKE_ROUND: u32 = 2;

extern "C" {
    pub fn stwo_status_string(status: Status) -> *const c_char;
    pub fn stwo_last_error() -> *const c_char;
    pub fn stwo_device_init(device: c_int) -> Status;
    pub fn stwo_sync(stream: Stream) -> Status;
    pub fn stwo_kernel_launches() -> u64;

    pub fn stwo_buf_alloc(d_ptr: *mut *mut c_void, bytes: usize, stream: Stream) -> Status;
    pub fn stwo_buf_free(d_ptr: *mut c_void, stream: Stream) -> Status;
    pub fn stwo_buf_upload(d_dst: *mut c_void, h_src: *const c_void, bytes: usize, stream: Stream) -> Status;
    pub fn stwo_buf_download(h_dst: *mut c_void, d_src: *const c_void, bytes: usize, stream: Stream) -> Status;
    pub fn stwo_buf_zero(d_dst: *mut c_void, bytes: usize, stream: Stream) -> Status;
    pub fn stwo_read_words(d_col: *const u32, h_idx: *const u64, n: usize, h_out: *mut u32, stream: Stream)
        -> Status;

    pub fn stwo_twiddles_precompute(root: StwoCoset, out: *mut Tree, stream: Stream) -> Status;
    pub fn stwo_twiddles_free(tree: Tree) -> Status;
    pub fn stwo_interpolate_columns(tree: Tree, half: StwoCoset, d_cols: *const *mut u32, n_cols: u32,
                                    stream: Stream) -> Status;
    pub fn stwo_evaluate_columns(tree: Tree, half: StwoCoset, d_coeffs: *const *const u32, coeff_log_size: u32,
                                 d_out: *const *mut u32, n_cols: u32, stream: Stream) -> Status;
    pub fn stwo_extend(d_coeffs: *const u32, coeff_log_size: u32, d_out: *mut u32, log_size: u32, stream: Stream)
        -> Status;
    pub fn stwo_eval_at_points(d_coeffs: *const *const u32, h_log_sizes: *const u32, n_polys: u32,
                               h_poly_of: *const u32, h_points: *const StwoQm31Point, n_evals: u32,
                               h_out: *mut StwoQm31, stream: Stream) -> Status;
    pub fn stwo_bit_reverse_column(d_col: *mut u32, log_size: u32, stream: Stream) -> Status;

    pub fn stwo_merkle_commit_layer(log_size: u32, d_prev: *const u32, d_cols: *const *const u32, n_cols: u32,
                                    d_out: *mut u32, stream: Stream) -> Status;
    pub fn stwo_merkle_commit_layer_poseidon252(log_size: u32, d_prev: *const u32, d_cols: *const *const u32,
                                                n_cols: u32, d_out: *mut u32, stream: Stream) -> Status;

    pub fn stwo_fri_fold_line(tree: Tree, line_domain: StwoCoset, d_eval: *const *const u32, alpha: StwoQm31,
                              d_out: *const *mut u32, stream: Stream) -> Status;
    pub fn stwo_fri_fold_circle_into_line(tree: Tree, src_half: StwoCoset, d_dst: *const *mut u32,
                                          d_src: *const *const u32, alpha: StwoQm31, stream: Stream) -> Status;
    pub fn stwo_fri_decompose(d_eval: *const *const u32, log_size: u32, d_g: *const *mut u32,
                              h_lambda: *mut StwoQm31, stream: Stream) -> Status;

    pub fn stwo_accumulate_quotients(domain_log_size: u32, d_cols: *const *const u32, n_cols: u32,
                                     random_coeff: StwoQm31, h_batches: *const StwoSampleBatch, n_batches: u32,
                                     log_blowup_factor: u32, d_out: *const *mut u32, stream: Stream) -> Status;
    pub fn stwo_secure_accumulate(d_acc: *const *mut u32, d_other: *const *const u32, n: usize, stream: Stream)
        -> Status;
    pub fn stwo_generate_secure_powers(felt: StwoQm31, n_powers: u32, h_out: *mut StwoQm31, stream: Stream)
        -> Status;

    pub fn stwo_gkr_gen_eq_evals(h_y: *const StwoQm31, n_y: u32, v: StwoQm31, d_out: *const *mut u32,
                                 stream: Stream) -> Status;
    pub fn stwo_gkr_next_layer(kind: u32, log_n: u32, d_num: *const *const u32, d_den: *const *const u32,
                               d_next_num: *const *mut u32, d_next_den: *const *mut u32, stream: Stream) -> Status;
    pub fn stwo_gkr_sum_as_poly_in_first_variable(kind: u32, log_n: u32, d_num: *const *const u32,
                                                  d_den: *const *const u32, d_eq: *const *const u32,
                                                  h_y: *const StwoQm31, n_y: u32, lambda: StwoQm31,
                                                  correction: StwoQm31, claim: StwoQm31, h_coeffs: *mut StwoQm31,
                                                  h_n_coeffs: *mut u32, stream: Stream) -> Status;
    pub fn stwo_mle_fix_first_variable_base(log_n: u32, d_mle: *const u32, assignment: StwoQm31,
                                            d_out: *const *mut u32, stream: Stream) -> Status;
    pub fn stwo_mle_fix_first_variable_secure(log_n: u32, d_mle: *const *const u32, assignment: StwoQm31,
                                              d_out: *const *mut u32, stream: Stream) -> Status;

    pub fn stwo_grind_blake2s(h_digest: *const u32, pow_bits: u32, h_nonce: *mut u64, stream: Stream) -> Status;
    pub fn stwo_grind_poseidon252(h_digest: *const u32, pow_bits: u32, h_nonce: *mut u64, stream: Stream)
        -> Status;

    pub fn stwo_component_info(component: *const StwoComponent, h_n_constraints: *mut u32,
                               h_eval_log_size: *mut u32, h_n_trees: *mut u32, h_tree_n_cols: *mut u32) -> Status;
    pub fn stwo_eval_constraints(component: *const StwoComponent, d_cols: *const *const u32, n_cols: u32,
                                 h_coeff_powers: *const StwoQm31, n_coeff_powers: u32, d_accum: *const *mut u32,
                                 stream: Stream) -> Status;

    pub fn stwo_codegen_compile(kernel_source: *const c_char, n_cols: u32, n_params: u32, n_constraints: u32,
                                load_now: c_int, out: *mut Codegen) -> Status;
    pub fn stwo_codegen_cubin(component: Codegen, h_dst: *mut c_void, capacity: usize, h_size: *mut usize)
        -> Status;
    pub fn stwo_codegen_from_cubin(h_cubin: *const c_void, size: usize, n_cols: u32, n_params: u32,
                                   n_constraints: u32, load_now: c_int, out: *mut Codegen) -> Status;
    pub fn stwo_codegen_destroy(component: Codegen) -> Status;
    pub fn stwo_eval_constraints_codegen(component: Codegen, trace_log_size: u32, eval_log_size: u32,
                                         d_cols: *const *const u32, n_cols: u32, h_params: *const StwoQm31,
                                         n_params: u32, h_coeff_powers: *const StwoQm31, n_coeff_powers: u32,
                                         d_accum: *const *mut u32, stream: Stream) -> Status;
    pub fn stwo_logup_interaction_codegen(component: Codegen, log_size: u32, d_cols: *const *const u32,
                                          n_cols: u32, h_params: *const StwoQm31, n_params: u32, d_out: *mut u32,
                                          h_claimed_sum: *mut StwoQm31, stream: Stream) -> Status;
    // The full Blake example's trace in HBM (examples/blake/air.rs:363-400).
    pub fn stwo_gen_blake_example_trace(log_n: u32, d_trace: *mut u32, d_scratch: *mut u32, stream: Stream)
                                        -> Status;
}

/// The reference panics on contract violations (`assert!`); the binding does the same with the
/// library's message.
pub fn check(status: Status) {
    if status != 0 {
        let msg = unsafe { CStr::from_ptr(stwo_last_error()) }.to_string_lossy().into_owned();
        let name = unsafe { CStr::from_ptr(stwo_status_string(status)) }.to_string_lossy().into_owned();
        panic!("stwo_gb300: {name}: {msg}");
    }
}
