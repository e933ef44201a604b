//! FFI declarations of libyumepdq_gb300 (include/ypdq.h), the batched, device-resident C ABI
//! of the GB300 backend. Every call returns a `ypdq_status` (`YPDQ_OK` = 0). Pointers named
//! `d_*` are device memory, `h_*` host memory; streams are CUDA streams (null = default).
//! The drop-in symbols of include/yume_pdq.h are yume-pdq's own C ABI and are not repeated.
#![allow(non_camel_case_types)]
#![no_std]

use core::ffi::{c_char, c_int, c_void};

pub type ypdq_status = c_int;
pub const YPDQ_OK: ypdq_status = 0;
pub const YPDQ_ERR_INVALID: ypdq_status = 1;
pub const YPDQ_ERR_ALIGN: ypdq_status = 2;
pub const YPDQ_ERR_CUDA: ypdq_status = 3;
pub const YPDQ_ERR_NOMEM: ypdq_status = 4;
pub const YPDQ_ERR_OVERFLOW: ypdq_status = 5;
pub const YPDQ_ERR_TIMEOUT: ypdq_status = 6;
pub const YPDQ_ERR_UNSUPPORTED: ypdq_status = 7;
pub const YPDQ_ERR_BUSY: ypdq_status = 8;

pub const YPDQ_INPUT_F32: c_int = 0;
pub const YPDQ_INPUT_U8: c_int = 1;
pub const YPDQ_INPUT_RGB8: c_int = 2;
pub const YPDQ_INPUT_RGBA8: c_int = 3;
pub const YPDQ_DCT_FP32: c_int = 0;
pub const YPDQ_DIHEDRAL_EXACT: c_int = 0;
pub const YPDQ_DIHEDRAL_AVX2: c_int = 1;
pub const YPDQ_DIHEDRAL_SCALAR: c_int = 2;
pub const YPDQ_SCAN_AUTO: c_int = 0;
pub const YPDQ_SCAN_SIMT: c_int = 1;
pub const YPDQ_SCAN_B1MMA: c_int = 2;
pub const YPDQ_SCAN_TC: c_int = 3;
pub const YPDQ_SCAN_TC_FP4: c_int = 4;
pub const YPDQ_SCAN_TC_FP8: c_int = 5;
pub const YPDQ_PDQF_T: c_int = 0;
pub const YPDQ_PDQF_NEGATE_ALT_COLS: c_int = 1;
pub const YPDQ_PDQF_NEGATE_ALT_ROWS: c_int = 2;
pub const YPDQ_PDQF_NEGATE_OFF_DIAGONALS: c_int = 3;
pub const YPDQ_H2D: c_int = 0;
pub const YPDQ_D2H: c_int = 1;

#[repr(C)]
pub struct ypdq_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct ypdq_db {
    _private: [u8; 0],
}
pub type ypdq_stream_t = *mut c_void;

/// One match: database row, query number and Hamming distance (16 bytes).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq, Eq)]
pub struct ypdq_hit {
    pub index: u64,
    pub query: u32,
    pub distance: u32,
}

unsafe extern "C" {
    pub fn ypdq_ctx_create(device: c_int, out: *mut *mut ypdq_ctx) -> ypdq_status;
    pub fn ypdq_ctx_destroy(ctx: *mut ypdq_ctx) -> ypdq_status;
    pub fn ypdq_last_error() -> *const c_char;
    pub fn ypdq_check_device_errors(ctx: *mut ypdq_ctx) -> ypdq_status;
    pub fn ypdq_dropin_semantics(semantics: *mut c_int) -> ypdq_status;

    pub fn ypdq_hash_batch(ctx: *mut ypdq_ctx, d_images: *const c_void, n: i64, input_kind: c_int,
                           dct_precision: c_int, semantics: c_int, d_hashes: *mut u8,
                           d_quality: *mut f32, d_thresholds: *mut f32, d_pdqf: *mut f32,
                           pdqf_slots: c_int, d_buf1: *mut f32, stream: ypdq_stream_t)
                           -> ypdq_status;
    pub fn ypdq_dihedrals_batch(ctx: *mut ypdq_ctx, d_pdqf: *const f32, d_thresholds: *const f32,
                                n: i64, semantics: c_int, d_hashes: *mut u8, d_quality: *mut f32,
                                d_thresholds_out: *mut f32, d_pdqf_out: *mut f32,
                                stream: ypdq_stream_t) -> ypdq_status;
    pub fn ypdq_dct2d_batch(ctx: *mut ypdq_ctx, d_buf1: *const f32, n: i64, stride: c_int,
                            d_pdqf: *mut f32, stream: ypdq_stream_t) -> ypdq_status;
    pub fn ypdq_sum_of_gradients_batch(ctx: *mut ypdq_ctx, d_pdqf: *const f32, n: i64,
                                       d_out: *mut f32, stream: ypdq_stream_t) -> ypdq_status;
    pub fn ypdq_pdqf_transform_batch(ctx: *mut ypdq_ctx, d_pdqf: *mut f32, n: i64, op: c_int,
                                     negate: c_int, semantics: c_int, stream: ypdq_stream_t)
                                     -> ypdq_status;
    pub fn ypdq_cvt_luma8f(ctx: *mut ypdq_ctx, d_pixels: *const u8, n_pixels: i64, channels: c_int,
                           r_coeff: f32, g_coeff: f32, b_coeff: f32, d_out: *mut f32,
                           stream: ypdq_stream_t) -> ypdq_status;

    pub fn ypdq_scan(ctx: *mut ypdq_ctx, d_rows: *const u8, n_rows: u64, d_queries: *const u8,
                     n_queries: u32, threshold: u32, d_hits: *mut ypdq_hit, capacity: u64,
                     d_count: *mut u64, algo: c_int, stream: ypdq_stream_t) -> ypdq_status;
    pub fn ypdq_sort_hits(ctx: *mut ypdq_ctx, d_hits: *mut ypdq_hit, n: u64,
                          stream: ypdq_stream_t) -> ypdq_status;

    pub fn ypdq_db_create(ctx: *mut ypdq_ctx, h_rows: *const u8, n_rows: u64, out: *mut *mut ypdq_db)
                          -> ypdq_status;
    pub fn ypdq_db_destroy(db: *mut ypdq_db) -> ypdq_status;
    pub fn ypdq_db_info(db: *mut ypdq_db, d_rows: *mut *const u8, n_rows: *mut u64) -> ypdq_status;
    pub fn ypdq_screen_host(ctx: *mut ypdq_ctx, db: *mut ypdq_db, h_images: *const c_void, n: i64,
                            input_kind: c_int, dct_precision: c_int, semantics: c_int,
                            threshold: u32, h_hits: *mut ypdq_hit, capacity: u64,
                            n_hits: *mut u64, h_hashes: *mut u8, h_quality: *mut f32)
                            -> ypdq_status;

    pub fn ypdq_malloc_device(ctx: *mut ypdq_ctx, bytes: usize, d_ptr: *mut *mut c_void)
                              -> ypdq_status;
    pub fn ypdq_free_device(ctx: *mut ypdq_ctx, d_ptr: *mut c_void) -> ypdq_status;
    pub fn ypdq_memcpy(ctx: *mut ypdq_ctx, dst: *mut c_void, src: *const c_void, bytes: usize,
                       kind: c_int, stream: ypdq_stream_t) -> ypdq_status;
    pub fn ypdq_memset(ctx: *mut ypdq_ctx, d_ptr: *mut c_void, value: c_int, bytes: usize,
                       stream: ypdq_stream_t) -> ypdq_status;
    pub fn ypdq_stream_sync(ctx: *mut ypdq_ctx, stream: ypdq_stream_t) -> ypdq_status;
}
