// Host-side interfaces shared by the translation units of the backend.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lp_device.cuh"

namespace lp {

// Work folded into a row (x-direction) pass.
struct RowOps {
  // x-domain multiplier: lens phase and/or mask, applied to the loaded line
  // before the transform, or (x_at_store) to the transformed line before it
  // is stored -- the adjoint of "multiply, then transform" is "transform,
  // then multiply by the conjugate".
  int lens;                  // 1: multiply by exp(+-2*pi*i * kappa*(jx^2+jy^2))
  float kap_hi, kap_lo;      // kappa = dL^2 * k0 / (4*pi*f) in cycles, float-float
  const void* xmask;         // optional x-domain multiplier
  int xmask_type;
  int conj;                  // conjugate the multiplier
  int x_at_store;            // apply after the transform instead of before
  // Epilogue.
  float scale;               // real factor on the output (1 = none)
  float* iprofile;           // optional |out|^2 (float32)
  // optional: += sum I, sum jx I, sum jy I, sum jx^2 I, sum jy^2 I over the
  // tile (I = |out|^2, jx / jy = offsets from the grid centre), FP64
  double* moments;
};

// Work folded into a column (y-direction) pass at the spectral point.
struct ColOps {
  KParams kp;
  int apply_h;               // multiply by the transfer function
  int phase_fp32;            // plain-FP32 phase variant
  int evan_mask;             // H = 0 on evanescent points (reference: H = 1)
  int conj;                  // adjoint: conjugate multipliers
  int dz;                    // also multiply by -2*pi*i*k0*sqrt(v)  (d/dz)
  const void* kmask;         // optional k-domain multiplier
  int kmask_type;
  float2* spectrum_out;      // optional write of the multiplied spectrum (pre-scale)
  float scale;               // real factor applied after the spectral multipliers
};

enum ColMode { COL_FWD = 0, COL_INV = 1, COL_FUSED = 2 };

// Launchers for one transform size.
struct SizeOps {
  int n;
  cudaError_t (*init)();  // per-device set-up (twiddle table, smem attributes)
  cudaError_t (*row)(int inverse, const float2* in, float2* out, const RowOps& ops,
                     cudaStream_t st);
  cudaError_t (*col)(int mode, const float2* in, float2* out, const ColOps& ops,
                     cudaStream_t st);
  // Resident CTAs per SM for the persistent row (kind 0) / column (kind 1)
  // kernels; 0 restores the built-in choice.  Returns the value in effect.
  int (*set_ctas_per_sm)(int kind, int value);
  // Device address of this size's stage-twiddle table (valid after init).
  const float2* (*twiddles)();
  // 1 if a bounded device-side wait of this size's kernels gave up since the
  // last call (the flag is cleared), 0 if not, -1 on a CUDA error.
  int (*take_async_error)();
};

// Per-device set-up of the batched persistent kernel (lp_batch.cu).
cudaError_t batch_init();

// Transfer-function constants for grid n, side `area`, wavelength wl and
// distance z (all in the caller's length unit).
KParams make_kparams(int n, double area, double wl, double z);
// Column-pass ops of a propagate: H(z) (if apply_h) and the lp_flags bits.
ColOps make_colops(int n, double area, double wl, double z, bool apply_h, uint32_t flags);
// Thin-lens phase of focal length f folded into a row pass.
void set_lens(RowOps& o, int n, double area, double wl, double f);

const SizeOps* size_ops(int n);

// Grid sizes outside the power-of-two pass kernels (lp_bluestein.cu): n in
// 2..4096 that is not a power of two in 16..8192.
bool bluestein_n(int n);
// The power-of-two size M >= 2n-1 of the Bluestein convolution grid.
int bluestein_m(int n);
// n x n 2-D DFT (forward, or unscaled inverse) times `scale`, through an
// M x M work grid `ws` (M = bluestein_m(n)); in may equal out.  The first
// call for a size on a device builds its tables (cudaMalloc + copy) and is
// refused inside stream capture (cudaErrorStreamCaptureUnsupported).
cudaError_t bluestein_dft2(const float2* in, float2* out, int n, int inverse, float scale,
                           float2* ws, cudaStream_t st);
// Pointwise x-domain multipliers (RowOps: lens, mask, conj) and spectral
// multipliers (ColOps: H, d/dz, kmask, spectrum write, scale) for any n.
cudaError_t generic_xmul(const float2* in, float2* out, int n, const RowOps& ops,
                         cudaStream_t st);
cudaError_t generic_spectral(const float2* in, float2* out, int n, const ColOps& ops,
                             cudaStream_t st);
// Frees the Bluestein tables of every device.
void bluestein_release();

// Tensor map of an n x n complex64 grid at `base` for 2-D TMA boxes of
// bx x by elements (cached per argument set).  false if the driver entry
// point is unavailable or the encoding is refused (callers then use their
// plain-load kernels).
bool grid_tensor_map(CUtensorMap* out, const void* base, int n, int bx, int by);

// Sets the thread-local text returned by lp_last_error() and returns `s`.
int set_last_error(int s, const char* msg);

inline RowOps row_ops_none() {
  RowOps o{};
  o.scale = 1.0f;
  return o;
}
inline ColOps col_ops_none() {
  ColOps o{};
  o.scale = 1.0f;
  return o;
}

}  // namespace lp
