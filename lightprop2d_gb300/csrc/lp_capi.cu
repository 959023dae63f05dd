// C ABI of the backend (include/lightprop2d_gb300.h): argument checks,
// per-device set-up, the per-(device, stream) scratch grid, the pass
// sequences behind every entry point, and the small elementwise kernels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "lightprop2d_gb300.h"
#include "lp_internal.h"

namespace lp {
extern const SizeOps size_ops_16, size_ops_32, size_ops_64, size_ops_128, size_ops_256,
    size_ops_512, size_ops_1024, size_ops_2048, size_ops_4096, size_ops_8192;

const SizeOps* size_ops(int n) {
  switch (n) {
    case 16: return &size_ops_16;
    case 32: return &size_ops_32;
    case 64: return &size_ops_64;
    case 128: return &size_ops_128;
    case 256: return &size_ops_256;
    case 512: return &size_ops_512;
    case 1024: return &size_ops_1024;
    case 2048: return &size_ops_2048;
    case 4096: return &size_ops_4096;
    case 8192: return &size_ops_8192;
    default: return nullptr;
  }
}
}  // namespace lp

using namespace lp;

namespace {

thread_local std::string t_last_error;
thread_local cudaEvent_t t_events[8];
thread_local int t_nevents = 0;

// Records profiling event i (see lp_profile_events) when the hook is armed.
inline void mark(int i, cudaStream_t st) {
  if (i < t_nevents) cudaEventRecord(t_events[i], st);
}

lp_status fail(lp_status s, const char* fmt, ...) {
  char msg[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  t_last_error = msg;
  return s;
}

lp_status cuda_fail(cudaError_t e, const char* where) {
  return fail(LP_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define LP_CUDA(call, where)                          \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

constexpr int kMaxDevices = 64;
std::mutex g_mu;
bool g_ready[kMaxDevices] = {};

lp_status init_device(int dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= kMaxDevices) return fail(LP_ERR_INVALID_ARGUMENT, "device %d out of range", dev);
  if (g_ready[dev]) return LP_OK;
  int prev = -1;
  LP_CUDA(cudaGetDevice(&prev), "cudaGetDevice");
  if (prev != dev) LP_CUDA(cudaSetDevice(dev), "cudaSetDevice");
  static const int sizes[] = {16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192};
  for (int n : sizes) {
    cudaError_t e = size_ops(n)->init();
    if (e != cudaSuccess) {
      if (prev != dev) cudaSetDevice(prev);
      return cuda_fail(e, "per-size set-up");
    }
  }
  {
    cudaError_t e = batch_init();
    if (e != cudaSuccess) {
      if (prev != dev) cudaSetDevice(prev);
      return cuda_fail(e, "batch kernel set-up");
    }
  }
  if (prev != dev) LP_CUDA(cudaSetDevice(prev), "cudaSetDevice");
  g_ready[dev] = true;
  return LP_OK;
}

// Makes sure the current device is set up; refuses first use inside capture.
lp_status ensure_ready(cudaStream_t st, int* dev_out) {
  int dev = 0;
  LP_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  *dev_out = dev;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (dev >= 0 && dev < kMaxDevices && g_ready[dev]) return LP_OK;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  LP_CUDA(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing");
  if (cs != cudaStreamCaptureStatusNone)
    return fail(LP_ERR_NOT_INITIALIZED,
                "first use of device %d inside stream capture: call lp_init() first", dev);
  return init_device(dev);
}

// Scratch grids of the unfused comparison path, cached per (device, stream).
// The fused paths need none: each pass reads whole lines into registers
// before writing them back, so intermediates live in the output grid.
struct Scratch {
  void* hbuf = nullptr;
  size_t hbuf_bytes = 0;
  void* blue = nullptr;  // M x M work grid of the transforms for other sizes
  size_t blue_bytes = 0;
  void* kz = nullptr;
  size_t kz_bytes = 0;
  int kz_n = 0;
  double kz_area = 0, kz_wl = 0;
};
std::map<std::pair<int, uintptr_t>, Scratch> g_scratch;

lp_status grow(void** p, size_t* have, size_t need, const char* what) {
  if (*have >= need) return LP_OK;
  if (*p) {
    cudaError_t e = cudaFree(*p);
    *p = nullptr;
    *have = 0;
    if (e != cudaSuccess) return cuda_fail(e, "cudaFree(scratch)");
  }
  cudaError_t e = cudaMalloc(p, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(LP_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu bytes) for %s: %s", need, what,
                cudaGetErrorString(e));
  }
  *have = need;
  return LP_OK;
}

Scratch& scratch_for(int dev, cudaStream_t st) {
  return g_scratch[std::make_pair(dev, (uintptr_t)st)];
}

#define LP_TRY(x)                  \
  do {                             \
    lp_status s_ = (x);            \
    if (s_ != LP_OK) return s_;    \
  } while (0)

// ---------------------------------------------------------------- checks --
bool aligned8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

lp_status check_grid(int n) {
  if (!size_ops(n) && !bluestein_n(n))
    return fail(LP_ERR_UNSUPPORTED_SIZE,
                "npoints=%d is not supported (2..4096, or a power of two up to 8192)", n);
  return LP_OK;
}

// Work grid of the transforms for sizes other than the power-of-two kernels'
// (per device and stream; grown with cudaMalloc, which is refused inside a
// stream capture: make one call of that size first).
lp_status blue_workspace(int dev, cudaStream_t st, int n, float2** ws) {
  const int m = bluestein_m(n);
  const size_t need = sizeof(float2) * (size_t)m * m;
  std::lock_guard<std::mutex> lk(g_mu);
  Scratch& s = g_scratch[std::make_pair(dev, (uintptr_t)st)];
  if (s.blue_bytes < need) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    LP_CUDA(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone)
      return fail(LP_ERR_NOT_INITIALIZED,
                  "npoints=%d needs a %dx%d work grid: make one call of this size before "
                  "stream capture", n, m, m);
    LP_TRY(grow(&s.blue, &s.blue_bytes, need, "transform work grid"));
  }
  *ws = reinterpret_cast<float2*>(s.blue);
  return LP_OK;
}

lp_status blue_call(cudaError_t e, const char* what) {
  if (e == cudaErrorStreamCaptureUnsupported)
    return fail(LP_ERR_NOT_INITIALIZED,
                "%s: the first transform of this grid size builds tables; make it before "
                "stream capture", what);
  if (e != cudaSuccess) return cuda_fail(e, what);
  return LP_OK;
}

lp_status check_ptr(const void* p, const char* name, bool required) {
  if (!p) return required ? fail(LP_ERR_INVALID_ARGUMENT, "%s is NULL", name) : LP_OK;
  if (!aligned8(p)) return fail(LP_ERR_MISALIGNED, "%s is not 8-byte aligned", name);
  return LP_OK;
}

lp_status check_mask(const void* m, int type, const char* name, bool k_domain = false) {
  if (type < LP_MASK_NONE || type > LP_MASK_SEP_C64)
    return fail(LP_ERR_INVALID_ARGUMENT, "%s: unknown mask type %d", name, type);
  if (k_domain && type == LP_MASK_SPAN_I32)
    return fail(LP_ERR_INVALID_ARGUMENT, "%s: LP_MASK_SPAN_I32 is an x-domain mask type", name);
  if (type == LP_MASK_NONE) return LP_OK;
  if (!m) return fail(LP_ERR_INVALID_ARGUMENT, "%s: NULL with mask type %d", name, type);
  const uintptr_t a = reinterpret_cast<uintptr_t>(m);
  const uintptr_t need = (type == LP_MASK_U8) ? 1 : (type == LP_MASK_C128) ? 16
                         : (type == LP_MASK_C64 || type == LP_MASK_F64 || type == LP_MASK_SEP_C64)
                             ? 8 : 4;
  if (a % need) return fail(LP_ERR_MISALIGNED, "%s is not %zu-byte aligned", name, (size_t)need);
  return LP_OK;
}

lp_status check_geometry(double area, double wl) {
  if (!(std::isfinite(area) && area > 0))
    return fail(LP_ERR_INVALID_ARGUMENT, "area_size must be finite and > 0");
  if (!(std::isfinite(wl) && wl > 0)) return fail(LP_ERR_INVALID_ARGUMENT, "wl must be finite and > 0");
  return LP_OK;
}


}  // namespace

// Transfer-function constants (see lp_device.cuh: kz_phase_ff).
KParams lp::make_kparams(int n, double area, double wl, double z) {
  const double dL = area / n;               // beam2d.py:299
  const double val = 1.0 / (n * dL);        // numpy fftfreq spacing (beam2d.py:205)
  const double k0 = 1.0 / wl;               // beam2d.py:304
  const double bw = val * wl;
  KParams kp;
  const FF beta = ff_from_double(bw * bw);
  const FF R = ff_from_double(z * k0);
  kp.beta_hi = beta.hi;
  kp.beta_lo = beta.lo;
  kp.R_hi = R.hi;
  kp.R_lo = R.lo;
  kp.two_pi_k0 = (float)(2.0 * kPi * k0);
  return kp;
}

ColOps lp::make_colops(int n, double area, double wl, double z, bool apply_h, uint32_t flags) {
  ColOps o = col_ops_none();
  o.kp = make_kparams(n, area, wl, z);
  o.apply_h = apply_h ? 1 : 0;
  o.phase_fp32 = (flags & LP_FLAG_PHASE_FP32) ? 1 : 0;
  o.evan_mask = (flags & LP_FLAG_EVANESCENT_MASK) ? 1 : 0;
  o.conj = (flags & LP_FLAG_ADJOINT) ? 1 : 0;
  o.dz = (flags & LP_FLAG_DZ) ? 1 : 0;
  return o;
}

void lp::set_lens(RowOps& o, int n, double area, double wl, double f) {
  // (X^2+Y^2)*k0/(2f) radians with X = jx*dL  ->  kappa*(jx^2+jy^2) cycles.
  const double dL = area / n;
  const double kap = dL * dL * (1.0 / wl) / (4.0 * kPi * f);
  const FF k = ff_from_double(kap);
  o.lens = 1;
  o.kap_hi = k.hi;
  o.kap_lo = k.lo;
}

namespace {

// ------------------------------------------------------ elementwise kernels --
__global__ void iprofile_kernel(const float2* __restrict__ f, float* __restrict__ out, size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const float2 v = f[i];
    out[i] = fmaf(v.x, v.x, v.y * v.y);
  }
}

// field *= lens(f) * mask  (x domain), without a transform.
__global__ void xmul_kernel(float2* __restrict__ f, int n, RowOps ops) {
  const size_t n2 = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / n), x = (int)(i % n);
    float2 m = make_float2(1.0f, 0.0f);
    if (ops.lens) {
      // X = arange(-n//2, n//2) * dL (beam2d.py:299-300): centre (n+1)/2
      const int jx = x - (n + 1) / 2, jy = y - (n + 1) / 2;
      m = cis_cycles(lens_cycles(ops.kap_hi, ops.kap_lo, jx * jx + jy * jy), 1.0f);
    }
    if (ops.xmask) m = cmul(m, mask_value_xy(ops.xmask, ops.xmask_type, y, x, n));
    if (ops.conj) m = cconj(m);
    f[i] = cmul(f[i], m);
  }
}

// Transfer function at point i of an N x N spectrum (float-float phase).
__device__ __forceinline__ float2 transfer_at(size_t i, int n, const ColOps& ops) {
  const int ky = (int)(i / n), kx = (int)(i % n);
  // fftfreq order (beam2d.py:205): k for k < (n+1)/2, k - n above
  const int sx = kx < (n + 1) / 2 ? kx : kx - n, sy = ky < (n + 1) / 2 ? ky : ky - n;
  const float qx = (float)(sx * sx), qy = (float)(sy * sy);
  bool evan;
  float sv, f;
  if (ops.phase_fp32) {
    f = kz_phase_f32(ops.kp, qx, qy, evan, sv);
  } else {
    float a_hi, a_lo;
    column_constant(ops.kp, qx, a_hi, a_lo);
    f = kz_phase_ff(ops.kp, a_hi, a_lo, qy, evan, sv);
  }
  float2 h = cis_cycles(f, ops.conj ? 1.0f : -1.0f);
  if (evan) h = ops.evan_mask ? make_float2(0.0f, 0.0f) : make_float2(1.0f, 0.0f);
  return h;
}

__global__ void apply_transfer_kernel(float2* __restrict__ s, int n, ColOps ops) {
  const size_t n2 = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x)
    s[i] = cmul(s[i], transfer_at(i, n, ops));
}

// Plain path: H materialised in HBM (float-float phase).
__global__ void build_h_kernel(float2* __restrict__ h, int n, ColOps ops) {
  const size_t n2 = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x)
    h[i] = transfer_at(i, n, ops);
}

// Plain path, reference-literal: Kz grid in FP64 (beam2d.py:305-308) ...
__global__ void build_kz_fp64_kernel(double* __restrict__ kz, int n, double val, double k0) {
  const size_t n2 = (size_t)n * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ky = (int)(i / n), kx = (int)(i % n);
    const double fx = (double)(kx < (n + 1) / 2 ? kx : kx - n) * val;
    const double fy = (double)(ky < (n + 1) / 2 ? ky : ky - n) * val;
    const double v = (k0 * k0 - fx * fx) - fy * fy;
    kz[i] = v >= 0.0 ? sqrt(v) : 0.0;  // nan_to_num(sqrt(negative)) = 0
  }
}

// ... and H from it in FP64: phase = 2*pi*(trunc(Kz z) - Kz z) (beam2d.py:485-489).
__global__ void build_h_fp64_kernel(float2* __restrict__ h, const double* __restrict__ kz,
                                    size_t n2, double z) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const double dk = kz[i] * z;
    const double ph = 2.0 * kPi * (trunc(dk) - dk);
    double s, c;
    sincos(ph, &s, &c);
    h[i] = make_float2((float)c, (float)s);
  }
}

__global__ void cmul_inplace_kernel(float2* __restrict__ a, const float2* __restrict__ b,
                                    size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] = cmul(a[i], b[i]);
}

int ew_grid(size_t n2) {
  size_t g = (n2 + 255) / 256;
  return (int)(g > 152 * 16 ? 152 * 16 : (g ? g : 1));
}

// Forward 2-D transform: rows (with x-domain prologue ops) then columns, the
// intermediate kept in `out`.
lp_status run_fft2_fwd(const SizeOps* so, const float2* in, float2* out, const RowOps& rops,
                       cudaStream_t st) {
  LP_CUDA(so->row(0, in, out, rops, st), "row pass (forward)");
  LP_CUDA(so->col(COL_FWD, out, out, col_ops_none(), st), "column pass (forward)");
  return LP_OK;
}

}  // namespace

int lp::set_last_error(int s, const char* msg) {
  t_last_error = msg;
  return s;
}

// =================================================================== ABI ==
extern "C" {

int lp_abi_version(void) { return LP_ABI_VERSION; }

const char* lp_last_error(void) { return t_last_error.c_str(); }

const char* lp_status_string(int s) {
  switch (s) {
    case LP_OK: return "ok";
    case LP_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LP_ERR_UNSUPPORTED_SIZE: return "unsupported grid size";
    case LP_ERR_MISALIGNED: return "misaligned pointer";
    case LP_ERR_CUDA: return "CUDA error";
    case LP_ERR_OUT_OF_MEMORY: return "out of device memory";
    case LP_ERR_NOT_INITIALIZED: return "device not initialised";
    case LP_ERR_TIMEOUT: return "device-side wait timed out";
    default: return "internal error";
  }
}

int lp_is_supported_n(int n) { return (size_ops(n) || bluestein_n(n)) ? 1 : 0; }

int lp_tune_ctas_per_sm(int n, int kind, int value) {
  const SizeOps* so = size_ops(n);
  if (!so || (kind != 0 && kind != 1)) return -1;
  return so->set_ctas_per_sm(kind, value);
}

lp_status lp_init(int device) {
  int count = 0;
  LP_CUDA(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
  if (device < 0 || device >= count)
    return fail(LP_ERR_INVALID_ARGUMENT, "device %d out of range (count %d)", device, count);
  return init_device(device);
}

lp_status lp_workspace_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  int prev = 0;
  cudaGetDevice(&prev);
  lp_status r = LP_OK;
  for (auto& kv : g_scratch) {
    cudaSetDevice(kv.first.first);
    Scratch& s = kv.second;
    for (void* p : {s.hbuf, s.kz, s.blue})
      if (p && cudaFree(p) != cudaSuccess) r = fail(LP_ERR_CUDA, "cudaFree failed");
  }
  g_scratch.clear();
  bluestein_release();
  cudaSetDevice(prev);
  return r;
}

lp_status lp_async_status(void* stream) {
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "lp_async_status: synchronize");
  int bad = 0;
  for (int n = 16; n <= 8192; n *= 2) {
    const int r = size_ops(n)->take_async_error();
    if (r < 0) return fail(LP_ERR_CUDA, "lp_async_status: reading the error record failed");
    bad |= r;
  }
  if (bad) return fail(LP_ERR_TIMEOUT, "a bounded device-side wait gave up (TMA copy never landed)");
  return LP_OK;
}

lp_status lp_profile_events(void** events, int count) {
  if (count < 0 || count > 8 || (count > 0 && !events))
    return fail(LP_ERR_INVALID_ARGUMENT, "lp_profile_events: 0 <= count <= 8 events");
  for (int i = 0; i < count; ++i) t_events[i] = reinterpret_cast<cudaEvent_t>(events[i]);
  t_nevents = count;
  return LP_OK;
}

lp_status lp_fft2(const lp_cfloat* in, lp_cfloat* out, int n, int inverse, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(in, "in", true));
  LP_TRY(check_ptr(out, "out", true));
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  const SizeOps* so = size_ops(n);
  const float2* src = reinterpret_cast<const float2*>(in);
  float2* dst = reinterpret_cast<float2*>(out);
  if (!so) {  // other sizes: Bluestein through a power-of-two work grid
    float2* ws;
    LP_TRY(blue_workspace(dev, st, n, &ws));
    return blue_call(bluestein_dft2(src, dst, n, inverse ? 1 : 0,
                                    inverse ? 1.0f / ((float)n * (float)n) : 1.0f, ws, st),
                     "fft2");
  }
  if (!inverse) return run_fft2_fwd(so, src, dst, row_ops_none(), st);
  ColOps c = col_ops_none();
  c.scale = 1.0f / ((float)n * (float)n);
  LP_CUDA(so->col(COL_INV, src, dst, c, st), "column pass (inverse)");
  LP_CUDA(so->row(1, dst, dst, row_ops_none(), st), "row pass (inverse)");
  return LP_OK;
}

lp_status lp_propagate(lp_cfloat* spectrum, lp_cfloat* field, int n, double area_size,
                       double wl, double z, const void* kmask, int kmask_type,
                       uint32_t flags, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(spectrum, "spectrum", true));
  LP_TRY(check_ptr(field, "field", true));
  LP_TRY(check_mask(kmask, kmask_type, "kmask", true));
  LP_TRY(check_geometry(area_size, wl));
  if (!std::isfinite(z)) return fail(LP_ERR_INVALID_ARGUMENT, "z must be finite");
  if ((const void*)spectrum == (const void*)field)
    return fail(LP_ERR_INVALID_ARGUMENT, "spectrum and field must be different grids");
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  const SizeOps* so = size_ops(n);
  float2* f = reinterpret_cast<float2*>(field);
  ColOps c = make_colops(n, area_size, wl, z, z != 0.0 || (flags & LP_FLAG_DZ), flags);
  c.kmask = kmask_type ? kmask : nullptr;
  c.kmask_type = kmask_type;
  if (!(flags & LP_FLAG_SPECTRUM_READONLY)) c.spectrum_out = reinterpret_cast<float2*>(spectrum);
  c.scale = 1.0f / ((float)n * (float)n);
  if (!so) {  // other sizes: pointwise multipliers, then a Bluestein inverse transform
    float2* ws;
    LP_TRY(blue_workspace(dev, st, n, &ws));
    LP_CUDA(generic_spectral(reinterpret_cast<const float2*>(spectrum), f, n, c, st),
            "spectral multipliers");
    return blue_call(bluestein_dft2(f, f, n, 1, 1.0f, ws, st), "inverse transform");
  }
  mark(0, st);
  LP_CUDA(so->col(COL_INV, reinterpret_cast<const float2*>(spectrum), f, c, st),
          "column pass (transfer + inverse)");
  mark(1, st);
  LP_CUDA(so->row(1, f, f, row_ops_none(), st), "row pass (inverse)");
  mark(2, st);
  return LP_OK;
}

lp_status lp_propagate_field(const lp_cfloat* field_in, lp_cfloat* field_out,
                             lp_cfloat* spectrum_out, float* iprofile_out, int n,
                             double area_size, double wl, double z, double lens_f,
                             const void* xmask, int xmask_type, const void* kmask,
                             int kmask_type, uint32_t flags, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(field_in, "field_in", true));
  LP_TRY(check_ptr(field_out, "field_out", true));
  LP_TRY(check_ptr(spectrum_out, "spectrum_out", false));
  if (iprofile_out && (reinterpret_cast<uintptr_t>(iprofile_out) & 3u))
    return fail(LP_ERR_MISALIGNED, "iprofile_out is not 4-byte aligned");
  LP_TRY(check_mask(xmask, xmask_type, "xmask"));
  LP_TRY(check_mask(kmask, kmask_type, "kmask", true));
  LP_TRY(check_geometry(area_size, wl));
  if (!std::isfinite(z) || !std::isfinite(lens_f))
    return fail(LP_ERR_INVALID_ARGUMENT, "z and lens_f must be finite");
  if (spectrum_out && (const void*)spectrum_out == (const void*)field_out)
    return fail(LP_ERR_INVALID_ARGUMENT, "spectrum_out and field_out must be different grids");
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  const SizeOps* so = size_ops(n);
  float2* out = reinterpret_cast<float2*>(field_out);

  // x-domain multiplier m: before the forward transform (P(m u)) or, with
  // XMASK_AFTER, after the inverse (m P(u)).  The adjoint conjugates every
  // multiplier and moves m to the other side: (P diag(m))^H = diag(conj(m)) P^H.
  const bool adjoint = (flags & LP_FLAG_ADJOINT) != 0;
  const bool after = ((flags & LP_FLAG_XMASK_AFTER) != 0) != adjoint;
  RowOps x = row_ops_none();
  if (lens_f != 0.0) set_lens(x, n, area_size, wl, lens_f);
  x.xmask = xmask_type ? xmask : nullptr;
  x.xmask_type = xmask_type;
  x.conj = adjoint ? 1 : 0;
  RowOps r = row_ops_none(), e = row_ops_none();
  if (after) {
    e = x;
    e.x_at_store = 1;
  } else {
    r = x;
  }
  e.iprofile = iprofile_out;
  ColOps c = make_colops(n, area_size, wl, z, z != 0.0 || (flags & LP_FLAG_DZ), flags);
  c.kmask = kmask_type ? kmask : nullptr;
  c.kmask_type = kmask_type;
  c.spectrum_out = reinterpret_cast<float2*>(spectrum_out);
  c.scale = 1.0f / ((float)n * (float)n);

  if (!so) {
    // Other sizes: the same operator as the fused passes, composed of
    // pointwise passes and Bluestein transforms.
    float2* ws;
    LP_TRY(blue_workspace(dev, st, n, &ws));
    const float2* src = reinterpret_cast<const float2*>(field_in);
    if (r.lens || r.xmask) {
      LP_CUDA(generic_xmul(src, out, n, r, st), "x-domain multipliers");
      src = out;
    }
    LP_TRY(blue_call(bluestein_dft2(src, out, n, 0, 1.0f, ws, st), "forward transform"));
    LP_CUDA(generic_spectral(out, out, n, c, st), "spectral multipliers");
    LP_TRY(blue_call(bluestein_dft2(out, out, n, 1, 1.0f, ws, st), "inverse transform"));
    if (e.lens || e.xmask) LP_CUDA(generic_xmul(out, out, n, e, st), "x-domain multipliers");
    if (iprofile_out) {
      const size_t n2 = (size_t)n * n;
      iprofile_kernel<<<ew_grid(n2), 256, 0, st>>>(out, iprofile_out, n2);
      LP_CUDA(cudaGetLastError(), "iprofile");
    }
    return LP_OK;
  }

  mark(0, st);
  LP_CUDA(so->row(0, reinterpret_cast<const float2*>(field_in), out, r, st),
          "row pass (forward)");
  mark(1, st);
  LP_CUDA(so->col(COL_FUSED, out, out, c, st), "column pass (forward, transfer, inverse)");
  mark(2, st);
  LP_CUDA(so->row(1, out, out, e, st), "row pass (inverse)");
  mark(3, st);
  return LP_OK;
}

static lp_status xdomain_op(lp_cfloat* field, lp_cfloat* spectrum_out, int n, RowOps r,
                            void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  float2* f = reinterpret_cast<float2*>(field);
  const size_t n2 = (size_t)n * n;
  xmul_kernel<<<ew_grid(n2), 256, 0, st>>>(f, n, r);
  LP_CUDA(cudaGetLastError(), "x-domain multiply");
  if (!spectrum_out) return LP_OK;
  if (!size_ops(n)) {
    float2* ws;
    LP_TRY(blue_workspace(dev, st, n, &ws));
    return blue_call(bluestein_dft2(f, reinterpret_cast<float2*>(spectrum_out), n, 0, 1.0f, ws,
                                    st),
                     "fft2");
  }
  return run_fft2_fwd(size_ops(n), f, reinterpret_cast<float2*>(spectrum_out), row_ops_none(),
                      st);
}

lp_status lp_lens(lp_cfloat* field, lp_cfloat* spectrum_out, int n, double area_size,
                  double wl, double f, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(field, "field", true));
  LP_TRY(check_ptr(spectrum_out, "spectrum_out", false));
  LP_TRY(check_geometry(area_size, wl));
  if (!std::isfinite(f) || f == 0.0)
    return fail(LP_ERR_INVALID_ARGUMENT, "focal length must be finite and non-zero");
  RowOps r = row_ops_none();
  set_lens(r, n, area_size, wl, f);
  return xdomain_op(field, spectrum_out, n, r, stream);
}

lp_status lp_coordinate_filter(lp_cfloat* field, lp_cfloat* spectrum_out, int n,
                               const void* mask, int mask_type, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(field, "field", true));
  LP_TRY(check_ptr(spectrum_out, "spectrum_out", false));
  LP_TRY(check_mask(mask, mask_type, "mask"));
  if (mask_type == LP_MASK_NONE) return fail(LP_ERR_INVALID_ARGUMENT, "mask is required");
  RowOps r = row_ops_none();
  r.xmask = mask;
  r.xmask_type = mask_type;
  return xdomain_op(field, spectrum_out, n, r, stream);
}

lp_status lp_spectral_filter(lp_cfloat* spectrum, lp_cfloat* field_out, int n,
                             const void* mask, int mask_type, void* stream) {
  if (mask_type == LP_MASK_NONE) return fail(LP_ERR_INVALID_ARGUMENT, "mask is required");
  // spectrum *= mask; field = ifft2(spectrum): lp_propagate with z = 0.
  return lp_propagate(spectrum, field_out, n, 1.0, 1.0, 0.0, mask, mask_type, 0u, stream);
}

lp_status lp_iprofile(const lp_cfloat* field, float* out, int n, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(field, "field", true));
  if (!out || (reinterpret_cast<uintptr_t>(out) & 3u))
    return fail(LP_ERR_INVALID_ARGUMENT, "out must be a 4-byte aligned device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  const size_t n2 = (size_t)n * n;
  iprofile_kernel<<<ew_grid(n2), 256, 0, st>>>(reinterpret_cast<const float2*>(field), out, n2);
  LP_CUDA(cudaGetLastError(), "iprofile");
  return LP_OK;
}

lp_status lp_apply_transfer(lp_cfloat* spectrum, int n, double area_size, double wl,
                            double z, uint32_t flags, void* stream) {
  LP_TRY(check_grid(n));
  LP_TRY(check_ptr(spectrum, "spectrum", true));
  LP_TRY(check_geometry(area_size, wl));
  if (!std::isfinite(z)) return fail(LP_ERR_INVALID_ARGUMENT, "z must be finite");
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  if (z == 0.0) return LP_OK;
  const size_t n2 = (size_t)n * n;
  apply_transfer_kernel<<<ew_grid(n2), 256, 0, st>>>(reinterpret_cast<float2*>(spectrum), n,
                                                      make_colops(n, area_size, wl, z, true, flags));
  LP_CUDA(cudaGetLastError(), "apply transfer");
  return LP_OK;
}

lp_status lp_plain_propagate_field(const lp_cfloat* field_in, lp_cfloat* field_out, int n,
                                   double area_size, double wl, double z, uint32_t flags,
                                   void* stream) {
  if (!size_ops(n))
    return fail(LP_ERR_UNSUPPORTED_SIZE,
                "lp_plain_propagate_field: npoints=%d (powers of two from 16 to 8192)", n);
  LP_TRY(check_ptr(field_in, "field_in", true));
  LP_TRY(check_ptr(field_out, "field_out", true));
  LP_TRY(check_geometry(area_size, wl));
  if (!std::isfinite(z)) return fail(LP_ERR_INVALID_ARGUMENT, "z must be finite");
  cudaStream_t st = (cudaStream_t)stream;
  int dev;
  LP_TRY(ensure_ready(st, &dev));
  const SizeOps* so = size_ops(n);
  const size_t n2 = (size_t)n * n;
  float2* out = reinterpret_cast<float2*>(field_out);
  float2* h;
  double* kz = nullptr;
  bool build_kz = false;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    Scratch& s = scratch_for(dev, st);
    LP_TRY(grow(&s.hbuf, &s.hbuf_bytes, sizeof(float2) * n2, "H grid"));
    h = reinterpret_cast<float2*>(s.hbuf);
    if (flags & LP_FLAG_PLAIN_FP64_H) {
      // The reference keeps Kz as beam state built once at construction.
      if (s.kz_n != n || s.kz_area != area_size || s.kz_wl != wl || !s.kz) {
        LP_TRY(grow(&s.kz, &s.kz_bytes, sizeof(double) * n2, "Kz grid"));
        s.kz_n = n;
        s.kz_area = area_size;
        s.kz_wl = wl;
        build_kz = true;
      }
      kz = reinterpret_cast<double*>(s.kz);
    }
  }
  const int g = ew_grid(n2);
  if (build_kz) {
    const double dL = area_size / n;
    build_kz_fp64_kernel<<<g, 256, 0, st>>>(kz, n, 1.0 / (n * dL), 1.0 / wl);
    LP_CUDA(cudaGetLastError(), "Kz build");
  }
  LP_TRY(run_fft2_fwd(so, reinterpret_cast<const float2*>(field_in), out, row_ops_none(), st));
  if (kz)
    build_h_fp64_kernel<<<g, 256, 0, st>>>(h, kz, n2, z);
  else
    build_h_kernel<<<g, 256, 0, st>>>(h, n, make_colops(n, area_size, wl, z, true, flags));
  LP_CUDA(cudaGetLastError(), "H build");
  cmul_inplace_kernel<<<g, 256, 0, st>>>(out, h, n2);
  LP_CUDA(cudaGetLastError(), "spectrum *= H");
  ColOps c = col_ops_none();
  c.scale = 1.0f / ((float)n * (float)n);
  LP_CUDA(so->col(COL_INV, out, out, c, st), "column pass (inverse)");
  LP_CUDA(so->row(1, out, out, row_ops_none(), st), "row pass (inverse)");
  return LP_OK;
}

}  // extern "C"
