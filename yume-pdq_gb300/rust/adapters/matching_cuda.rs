//! src/matching/cuda.rs of yume-pdq (behind a `cuda` feature that depends on
//! yume-pdq-gb300-sys): a `PDQMatcher` whose haystack lives on a GB300 and whose needles are
//! the query, like the Vulkan matcher (src/matching/vulkan.rs:334-473). It differs in what
//! it reports: every (row, needle) pair within the threshold, in the scalar CpuMatcher's
//! order (rows ascending, then needles), so `FindsAllMatches = B1`; the Vulkan matcher
//! returns only the lowest match.
//!
//! Written against the reference's trait definitions (src/matching/mod.rs:50-105,
//! src/kernel/type_traits.rs:60-188); not compiled here (no Rust toolchain on this image).

use alloc::vec::Vec;
use core::ptr::null_mut;

use generic_array::{
    GenericArray,
    sequence::Flatten,
    typenum::{B1, U8, U32},
};
use yume_pdq_gb300_sys as sys;

use super::PDQMatcher;
use crate::kernel::type_traits::{EvaluateHardwareFeature, kernel_sealing::KernelSealed};

/// A CUDA device of compute capability 10.3 (GB300) with libyumepdq_gb300 loaded.
pub struct CudaAccelerator;

impl KernelSealed for CudaAccelerator {}

impl EvaluateHardwareFeature for CudaAccelerator {
    type Name = &'static str;
    type EnabledStatic = B1;
    type MustCheck = B1;

    fn name() -> Self::Name {
        "CUDA sm_103a"
    }

    fn met_runtime() -> bool {
        let mut ctx = null_mut();
        let ok = unsafe { sys::ypdq_ctx_create(0, &mut ctx) } == sys::YPDQ_OK;
        if ok {
            unsafe { sys::ypdq_ctx_destroy(ctx) };
        }
        ok
    }
}

fn check(status: sys::ypdq_status) {
    assert_eq!(status, sys::YPDQ_OK, "libyumepdq_gb300 call failed (status {status})");
}

/// The haystack uploaded once to device memory (ypdq_db_create), with the per-query device
/// buffers the scan writes into.
pub struct CudaMatcher {
    ctx: *mut sys::ypdq_ctx,
    db: *mut sys::ypdq_db,
    threshold: u32,
    d_needles: *mut core::ffi::c_void,
    d_hits: *mut sys::ypdq_hit,
    d_count: *mut u64,
    capacity: u64,
    hits: Vec<sys::ypdq_hit>,
}

impl CudaMatcher {
    /// Upload `haystack` (rows of 32 bytes) to device 0 and match at `threshold` bits.
    pub fn new(haystack: &[GenericArray<u8, U32>], threshold: u32) -> Self {
        let mut ctx = null_mut();
        check(unsafe { sys::ypdq_ctx_create(0, &mut ctx) });
        let mut db = null_mut();
        check(unsafe {
            sys::ypdq_db_create(ctx, haystack.as_ptr().cast(), haystack.len() as u64, &mut db)
        });
        let capacity = 1u64 << 16;
        let mut needles = null_mut();
        let mut hits = null_mut();
        let mut count = null_mut();
        check(unsafe { sys::ypdq_malloc_device(ctx, 8 * 32, &mut needles) });
        check(unsafe { sys::ypdq_malloc_device(ctx, capacity as usize * 16, &mut hits) });
        check(unsafe { sys::ypdq_malloc_device(ctx, 8, &mut count) });
        Self {
            ctx,
            db,
            threshold,
            d_needles: needles,
            d_hits: hits.cast(),
            d_count: count.cast(),
            capacity,
            hits: Vec::new(),
        }
    }

    /// Scan the 8 needles; returns the true hit count and leaves up to `capacity` hits,
    /// sorted into the scalar matcher's order, in `self.hits`.
    fn run(&mut self, needles: &[u8], capacity: u64) -> u64 {
        let mut rows = core::ptr::null();
        let mut n_rows = 0u64;
        check(unsafe { sys::ypdq_db_info(self.db, &mut rows, &mut n_rows) });
        check(unsafe {
            sys::ypdq_memcpy(self.ctx, self.d_needles, needles.as_ptr().cast(), needles.len(),
                             sys::YPDQ_H2D, null_mut())
        });
        check(unsafe {
            sys::ypdq_scan(self.ctx, rows, n_rows, self.d_needles.cast(), 8, self.threshold,
                           self.d_hits, capacity, self.d_count, sys::YPDQ_SCAN_AUTO, null_mut())
        });
        let mut total = 0u64;
        check(unsafe {
            sys::ypdq_memcpy(self.ctx, (&mut total as *mut u64).cast(), self.d_count.cast(), 8,
                             sys::YPDQ_D2H, null_mut())
        });
        check(unsafe { sys::ypdq_stream_sync(self.ctx, null_mut()) });
        let kept = total.min(capacity);
        self.hits.clear();
        if kept > 0 {
            check(unsafe { sys::ypdq_sort_hits(self.ctx, self.d_hits, kept, null_mut()) });
            self.hits.resize(kept as usize, sys::ypdq_hit::default());
            check(unsafe {
                sys::ypdq_memcpy(self.ctx, self.hits.as_mut_ptr().cast(), self.d_hits.cast(),
                                 kept as usize * 16, sys::YPDQ_D2H, null_mut())
            });
            check(unsafe { sys::ypdq_stream_sync(self.ctx, null_mut()) });
        }
        total
    }
}

impl Drop for CudaMatcher {
    fn drop(&mut self) {
        unsafe {
            sys::ypdq_free_device(self.ctx, self.d_needles);
            sys::ypdq_free_device(self.ctx, self.d_hits.cast());
            sys::ypdq_free_device(self.ctx, self.d_count.cast());
            sys::ypdq_db_destroy(self.db);
            sys::ypdq_ctx_destroy(self.ctx);
        }
    }
}

impl PDQMatcher for CudaMatcher {
    type BatchSize = U8;
    type RequiredHardwareFeature = CudaAccelerator;
    type InputDimension = U32;
    type Aligner<T> = T;
    type NoFalseNegative = B1;
    type NoFalsePositive = B1;
    type FindsAllMatches = B1;
    type Ident = &'static str;

    fn ident() -> Self::Ident {
        "CUDA sm_103a exact matcher (tcgen05 FP8 / SIMT popcount)"
    }

    /// A scan with capacity 0: the count alone says whether any row matched.
    fn scan(&mut self, query: &GenericArray<GenericArray<u8, U32>, U8>) -> bool {
        self.run(query.flatten().as_slice(), 0) > 0
    }

    /// Every match in (row, needle) order; `f(row, needle)` as the Vulkan matcher calls it.
    fn find<R, F: FnMut(usize, usize) -> Option<R>>(
        &mut self,
        query: &GenericArray<GenericArray<u8, U32>, U8>,
        mut f: F,
    ) -> Option<R> {
        let needles = query.flatten();
        let mut capacity = self.capacity;
        loop {
            let total = self.run(needles.as_slice(), capacity);
            if total <= capacity {
                break;
            }
            // more hits than the device buffer: grow it to the true count and scan again
            unsafe { sys::ypdq_free_device(self.ctx, self.d_hits.cast()) };
            let mut hits = null_mut();
            check(unsafe { sys::ypdq_malloc_device(self.ctx, total as usize * 16, &mut hits) });
            self.d_hits = hits.cast();
            self.capacity = total;
            capacity = total;
        }
        self.hits
            .iter()
            .find_map(|h| f(h.index as usize, h.query as usize))
    }
}
