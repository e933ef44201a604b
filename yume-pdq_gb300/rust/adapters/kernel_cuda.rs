//! src/kernel/cuda.rs of yume-pdq (behind a `cuda` feature that depends on
//! yume-pdq-gb300-sys): a `Kernel` (src/kernel/mod.rs:268-497) whose every method runs on a
//! GB300 through libyumepdq_gb300's batched calls with a batch of one. Its results equal
//! DefaultKernelPadXYTo128's bit for bit (f32, the reference's operation order); the sign
//! convention of the PDQF negations is chosen at construction (`scalar` reproduces the
//! trait defaults, `avx2` / `exact` the AVX2 / AVX-512 kernels' overrides). For many images
//! at once, call `ypdq_hash_batch` directly: thousands of images per launch.
//!
//! Each clone owns its device scratch (the trait's methods take `&mut self` and callers
//! clone one kernel per thread, src/lib.rs:266) and shares one `ypdq_ctx`.
//! Written against the reference's trait definitions; not compiled here (no Rust toolchain
//! on this image).

use alloc::sync::Arc;
use core::ffi::{c_int, c_void};
use core::ptr::null_mut;

use generic_array::{
    GenericArray,
    typenum::{U2, U3, U4, U16, U128, U512},
};
use yume_pdq_gb300_sys as sys;

use super::{Kernel, QUALITY_ADJUST_DIVISOR};
use crate::matching::cuda::CudaAccelerator;

struct Ctx(*mut sys::ypdq_ctx);
unsafe impl Send for Ctx {}
unsafe impl Sync for Ctx {}
impl Drop for Ctx {
    fn drop(&mut self) {
        unsafe { sys::ypdq_ctx_destroy(self.0) };
    }
}

fn check(status: sys::ypdq_status) {
    assert_eq!(status, sys::YPDQ_OK, "libyumepdq_gb300 call failed (status {status})");
}

const IMAGE_BYTES: usize = 512 * 512 * 4;
const BUF1_BYTES: usize = 127 * 128 * 4;
const PDQF_BYTES: usize = 256 * 4;
const OUT_BYTES: usize = 256 + 8 * 4;  // 8 hashes, then 8 thresholds
const ROW_BYTES: usize = 512 * 4;

/// GPU implementation of the `Kernel` trait.
pub struct CudaKernel {
    ctx: Arc<Ctx>,
    semantics: c_int,
    d_image: *mut c_void,  // the 512x512 input, or a row of RGB(A) pixels
    d_buf1: *mut c_void,   // 127 rows x 128 f32
    d_pdqf: *mut c_void,   // 16 x 16 f32
    d_out: *mut c_void,    // hashes and thresholds, or a luma row
}
unsafe impl Send for CudaKernel {}

impl CudaKernel {
    /// A kernel on device 0 with the given sign convention (sys::YPDQ_DIHEDRAL_*).
    pub fn new(semantics: c_int) -> Self {
        let mut ctx = null_mut();
        check(unsafe { sys::ypdq_ctx_create(0, &mut ctx) });
        Self::with_ctx(Arc::new(Ctx(ctx)), semantics)
    }

    fn with_ctx(ctx: Arc<Ctx>, semantics: c_int) -> Self {
        let mut p = [null_mut(); 4];
        for (ptr, bytes) in p.iter_mut().zip([IMAGE_BYTES, BUF1_BYTES, PDQF_BYTES, OUT_BYTES.max(ROW_BYTES)]) {
            check(unsafe { sys::ypdq_malloc_device(ctx.0, bytes, ptr) });
        }
        Self { ctx, semantics, d_image: p[0], d_buf1: p[1], d_pdqf: p[2], d_out: p[3] }
    }

    fn h2d(&self, dst: *mut c_void, src: *const c_void, bytes: usize) {
        check(unsafe { sys::ypdq_memcpy(self.ctx.0, dst, src, bytes, sys::YPDQ_H2D, null_mut()) });
    }

    fn d2h(&self, dst: *mut c_void, src: *const c_void, bytes: usize) {
        check(unsafe { sys::ypdq_memcpy(self.ctx.0, dst, src, bytes, sys::YPDQ_D2H, null_mut()) });
        check(unsafe { sys::ypdq_stream_sync(self.ctx.0, null_mut()) });
    }

    fn pdqf_op(&mut self, pdqf: &mut GenericArray<GenericArray<f32, U16>, U16>, op: c_int, negate: bool) {
        self.h2d(self.d_pdqf, pdqf.as_ptr().cast(), PDQF_BYTES);
        check(unsafe {
            sys::ypdq_pdqf_transform_batch(self.ctx.0, self.d_pdqf.cast(), 1, op, negate as c_int,
                                           self.semantics, null_mut())
        });
        self.d2h(pdqf.as_mut_ptr().cast(), self.d_pdqf, PDQF_BYTES);
    }

    fn luma(&mut self, px: *const u8, channels: c_int, coeffs: [f32; 3],
            output: &mut GenericArray<f32, U512>) {
        self.h2d(self.d_image, px.cast(), 512 * channels as usize);
        check(unsafe {
            sys::ypdq_cvt_luma8f(self.ctx.0, self.d_image.cast(), 512, channels, coeffs[0],
                                 coeffs[1], coeffs[2], self.d_out.cast(), null_mut())
        });
        self.d2h(output.as_mut_ptr().cast(), self.d_out, ROW_BYTES);
    }
}

impl Clone for CudaKernel {
    fn clone(&self) -> Self {
        Self::with_ctx(self.ctx.clone(), self.semantics)
    }
}

impl Drop for CudaKernel {
    fn drop(&mut self) {
        for p in [self.d_image, self.d_buf1, self.d_pdqf, self.d_out] {
            unsafe { sys::ypdq_free_device(self.ctx.0, p) };
        }
    }
}

impl Kernel for CudaKernel {
    type Buffer1WidthX = U128;
    type Buffer1LengthY = U128;
    type InputDimension = U512;
    type OutputDimension = U16;
    type RequiredHardwareFeature = CudaAccelerator;
    type Ident = &'static str;
    type InternalFloat = f32;

    fn ident(&self) -> &'static str {
        "cuda_sm103a_f32"
    }

    fn cvt_rgb8_to_luma8f<const R_COEFF: u32, const G_COEFF: u32, const B_COEFF: u32>(
        &mut self,
        input: &GenericArray<GenericArray<u8, U3>, U512>,
        output: &mut GenericArray<f32, U512>,
    ) {
        let c = [f32::from_bits(R_COEFF), f32::from_bits(G_COEFF), f32::from_bits(B_COEFF)];
        self.luma(input.as_ptr().cast(), 3, c, output);
    }

    fn cvt_rgba8_to_luma8f<const R_COEFF: u32, const G_COEFF: u32, const B_COEFF: u32>(
        &mut self,
        input: &GenericArray<GenericArray<u8, U4>, U512>,
        output: &mut GenericArray<f32, U512>,
    ) {
        let c = [f32::from_bits(R_COEFF), f32::from_bits(G_COEFF), f32::from_bits(B_COEFF)];
        self.luma(input.as_ptr().cast(), 4, c, output);
    }

    fn pdqf_t(&mut self, input: &mut GenericArray<GenericArray<f32, U16>, U16>) {
        self.pdqf_op(input, sys::YPDQ_PDQF_T, false);
    }

    fn pdqf_negate_alt_cols<const NEGATE: bool>(
        &mut self,
        input: &mut GenericArray<GenericArray<f32, U16>, U16>,
    ) {
        self.pdqf_op(input, sys::YPDQ_PDQF_NEGATE_ALT_COLS, NEGATE);
    }

    fn pdqf_negate_alt_rows<const NEGATE: bool>(
        &mut self,
        input: &mut GenericArray<GenericArray<f32, U16>, U16>,
    ) {
        self.pdqf_op(input, sys::YPDQ_PDQF_NEGATE_ALT_ROWS, NEGATE);
    }

    fn pdqf_negate_off_diagonals(&mut self, input: &mut GenericArray<GenericArray<f32, U16>, U16>) {
        self.pdqf_op(input, sys::YPDQ_PDQF_NEGATE_OFF_DIAGONALS, false);
    }

    /// The library's fused hash kernel with only its compressed-image output (rows of 128
    /// floats, the first 127 written); the padding row and column are left as they are.
    fn jarosz_compress(
        &mut self,
        buffer: &GenericArray<GenericArray<f32, U512>, U512>,
        output: &mut GenericArray<GenericArray<f32, U128>, U128>,
    ) {
        self.h2d(self.d_image, buffer.as_ptr().cast(), IMAGE_BYTES);
        check(unsafe {
            sys::ypdq_hash_batch(self.ctx.0, self.d_image, 1, sys::YPDQ_INPUT_F32,
                                 sys::YPDQ_DCT_FP32, self.semantics, null_mut(), null_mut(),
                                 null_mut(), null_mut(), 1, self.d_buf1.cast(), null_mut())
        });
        let mut rows = [[0.0f32; 128]; 127];
        self.d2h(rows.as_mut_ptr().cast(), self.d_buf1, BUF1_BYTES);
        for (dst, src) in output.iter_mut().zip(rows.iter()) {
            dst[..127].copy_from_slice(&src[..127]);
        }
    }

    fn quantize(
        &mut self,
        input: &GenericArray<GenericArray<f32, U16>, U16>,
        threshold: &mut f32,
        output: &mut GenericArray<GenericArray<u8, U2>, U16>,
    ) {
        self.h2d(self.d_pdqf, input.as_ptr().cast(), PDQF_BYTES);
        let d_hashes = self.d_out.cast::<u8>();
        let d_thr = unsafe { d_hashes.add(256) }.cast::<f32>();
        check(unsafe {
            sys::ypdq_dihedrals_batch(self.ctx.0, self.d_pdqf.cast(), core::ptr::null(), 1,
                                      self.semantics, d_hashes, null_mut(), d_thr, null_mut(),
                                      null_mut())
        });
        let mut out = [0u8; OUT_BYTES];
        self.d2h(out.as_mut_ptr().cast(), self.d_out, OUT_BYTES);
        // slot 0: the matrix quantized at its own median (byte 31 - k / 8, bit k % 8)
        output.as_mut_slice().iter_mut().flat_map(|r| r.iter_mut()).zip(&out[..32])
            .for_each(|(d, s)| *d = *s);
        *threshold = f32::from_ne_bytes(out[256..260].try_into().unwrap());
    }

    fn sum_of_gradients(&mut self, input: &GenericArray<GenericArray<f32, U16>, U16>) -> f32 {
        self.h2d(self.d_pdqf, input.as_ptr().cast(), PDQF_BYTES);
        check(unsafe {
            sys::ypdq_sum_of_gradients_batch(self.ctx.0, self.d_pdqf.cast(), 1,
                                             self.d_out.cast(), null_mut())
        });
        let mut g = 0.0f32;
        self.d2h((&mut g as *mut f32).cast(), self.d_out, 4);
        g
    }

    fn adjust_quality(input: f32) -> f32 {
        (input / QUALITY_ADJUST_DIVISOR as f32).min(1.0)
    }

    /// Buffer rows are 128 floats apart: the first 127 rows go to the device as they are
    /// and the DCT reads their first 127 columns. `tmp_row_buffer` is not used.
    fn dct2d(
        &mut self,
        buffer: &GenericArray<GenericArray<f32, U128>, U128>,
        _tmp_row_buffer: &mut GenericArray<f32, U128>,
        output: &mut GenericArray<GenericArray<f32, U16>, U16>,
    ) {
        self.h2d(self.d_buf1, buffer.as_ptr().cast(), BUF1_BYTES);
        check(unsafe {
            sys::ypdq_dct2d_batch(self.ctx.0, self.d_buf1.cast(), 1, 128, self.d_pdqf.cast(),
                                  null_mut())
        });
        self.d2h(output.as_mut_ptr().cast(), self.d_pdqf, PDQF_BYTES);
    }
}
