//! Device columns: owned buffers of canonical 32-bit words in HBM (`stwo_buf_*`).
//!
//! Layouts are the ones the C ABI expects: a base-field column is one word per value; a secure
//! column is four coordinate planes of `len` words each (SecureColumnByCoords order, so a plane is a
//! plain base column); a hash column is eight words per node, node after node, as the Merkle layer
//! kernels write them.

use std::fmt::{self, Debug};
use std::marker::PhantomData;
use std::ptr::null_mut;

use stwo_prover::core::fields::m31::BaseField;
use stwo_prover::core::fields::qm31::SecureField;
use stwo_prover::core::vcs::blake2_hash::Blake2sHash;

use crate::ffi::*;

/// A value type a device column can hold, with its word layout.
pub trait DeviceWords: Copy + Debug + Default {
    /// 32-bit words per value.
    const WORDS: usize;
    /// Words stored plane by plane (word k of value i at k * len + i) rather than value by value.
    const PLANAR: bool;
    fn to_words(&self, out: &mut [u32]);
    fn from_words(w: &[u32]) -> Self;
}

impl DeviceWords for BaseField {
    const WORDS: usize = 1;
    const PLANAR: bool = true;
    fn to_words(&self, out: &mut [u32]) {
        out[0] = self.0;
    }
    fn from_words(w: &[u32]) -> Self {
        BaseField::from_u32_unchecked(w[0])
    }
}

impl DeviceWords for SecureField {
    const WORDS: usize = 4;
    const PLANAR: bool = true;
    fn to_words(&self, out: &mut [u32]) {
        for (o, c) in out.iter_mut().zip(self.to_m31_array()) {
            *o = c.0;
        }
    }
    fn from_words(w: &[u32]) -> Self {
        SecureField::from_u32_unchecked(w[0], w[1], w[2], w[3])
    }
}

impl DeviceWords for Blake2sHash {
    const WORDS: usize = 8;
    const PLANAR: bool = false;
    fn to_words(&self, out: &mut [u32]) {
        for (k, o) in out.iter_mut().enumerate() {
            *o = u32::from_le_bytes(self.0[4 * k..4 * k + 4].try_into().unwrap());
        }
    }
    fn from_words(w: &[u32]) -> Self {
        let mut b = [0u8; 32];
        for k in 0..8 {
            b[4 * k..4 * k + 4].copy_from_slice(&w[k].to_le_bytes());
        }
        Blake2sHash(b)
    }
}

/// An owned device column of `len` values of type T.
pub struct CudaColumn<T: DeviceWords> {
    pub(crate) ptr: *mut u32,
    pub(crate) len: usize,
    _t: PhantomData<T>,
}

// The buffer is plain device memory; the library's calls are thread-safe on distinct streams.
unsafe impl<T: DeviceWords> Send for CudaColumn<T> {}
unsafe impl<T: DeviceWords> Sync for CudaColumn<T> {}

impl<T: DeviceWords> CudaColumn<T> {
    fn alloc(len: usize) -> Self {
        let mut p = null_mut();
        check(unsafe { stwo_buf_alloc(&mut p, (len * T::WORDS).max(1) * 4, null_mut()) });
        Self { ptr: p.cast(), len, _t: PhantomData }
    }
    pub fn ptr(&self) -> *const u32 {
        self.ptr
    }
    pub fn ptr_mut(&mut self) -> *mut u32 {
        self.ptr
    }
    /// Plane k of a planar column (a base column of `len` words).
    pub fn plane(&self, k: usize) -> *mut u32 {
        debug_assert!(T::PLANAR && k < T::WORDS);
        unsafe { self.ptr.add(k * self.len) }
    }
    /// The four coordinate planes of a secure column, as the ABI's `d[4]` arguments.
    pub fn planes4(&self) -> [*mut u32; 4] {
        [self.plane(0), self.plane(1), self.plane(2), self.plane(3)]
    }
    fn word_index(&self, i: usize, k: usize) -> u64 {
        (if T::PLANAR { k * self.len + i } else { i * T::WORDS + k }) as u64
    }
    fn upload_values(&mut self, values: &[T]) {
        let n = values.len();
        let mut words = vec![0u32; n * T::WORDS];
        let mut w = vec![0u32; T::WORDS];
        for (i, v) in values.iter().enumerate() {
            v.to_words(&mut w);
            for k in 0..T::WORDS {
                words[self.word_index(i, k) as usize] = w[k];
            }
        }
        check(unsafe { stwo_buf_upload(self.ptr.cast(), words.as_ptr().cast(), words.len() * 4, null_mut()) });
    }
}

impl<T: DeviceWords> Drop for CudaColumn<T> {
    fn drop(&mut self) {
        unsafe { stwo_buf_free(self.ptr.cast(), null_mut()) };
    }
}

impl<T: DeviceWords> Debug for CudaColumn<T> {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "CudaColumn {{ len: {}, words: {} }}", self.len, T::WORDS)
    }
}

impl<T: DeviceWords> Clone for CudaColumn<T> {
    fn clone(&self) -> Self {
        // The ABI has no device-to-device copy: the words pass through the host (Clone is not on
        // the prove path).
        let mut out = Self::alloc(self.len);
        let mut words = vec![0u32; self.len * T::WORDS];
        check(unsafe { stwo_buf_download(words.as_mut_ptr().cast(), self.ptr.cast(), words.len() * 4, null_mut()) });
        check(unsafe { stwo_buf_upload(out.ptr.cast(), words.as_ptr().cast(), words.len() * 4, null_mut()) });
        out
    }
}

impl<T: DeviceWords> FromIterator<T> for CudaColumn<T> {
    fn from_iter<I: IntoIterator<Item = T>>(iter: I) -> Self {
        let values: Vec<T> = iter.into_iter().collect();
        let mut out = Self::alloc(values.len());
        out.upload_values(&values);
        out
    }
}

impl<T: DeviceWords> stwo_prover::core::backend::Column<T> for CudaColumn<T> {
    fn zeros(len: usize) -> Self {
        let out = Self::alloc(len);
        check(unsafe { stwo_buf_zero(out.ptr.cast(), len * T::WORDS * 4, null_mut()) });
        out
    }
    unsafe fn uninitialized(len: usize) -> Self {
        Self::alloc(len)
    }
    fn to_cpu(&self) -> Vec<T> {
        let mut words = vec![0u32; self.len * T::WORDS];
        check(unsafe { stwo_buf_download(words.as_mut_ptr().cast(), self.ptr.cast(), words.len() * 4, null_mut()) });
        let mut w = vec![0u32; T::WORDS];
        (0..self.len)
            .map(|i| {
                for k in 0..T::WORDS {
                    w[k] = words[self.word_index(i, k) as usize];
                }
                T::from_words(&w)
            })
            .collect()
    }
    fn len(&self) -> usize {
        self.len
    }
    /// Column::at backs decommitment reads: one stwo_read_words of the value's words.
    fn at(&self, index: usize) -> T {
        let idx: Vec<u64> = (0..T::WORDS).map(|k| self.word_index(index, k)).collect();
        let mut w = vec![0u32; T::WORDS];
        check(unsafe { stwo_read_words(self.ptr, idx.as_ptr(), idx.len(), w.as_mut_ptr(), null_mut()) });
        T::from_words(&w)
    }
    fn set(&mut self, index: usize, value: T) {
        let mut w = vec![0u32; T::WORDS];
        value.to_words(&mut w);
        for k in 0..T::WORDS {
            let off = self.word_index(index, k) as usize;
            check(unsafe { stwo_buf_upload(self.ptr.add(off).cast(), (&w[k] as *const u32).cast(), 4, null_mut()) });
        }
    }
}
