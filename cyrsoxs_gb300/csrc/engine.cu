// GB300 scattering engine: host orchestration and the C ABI (include/cyrsoxs.h).
//
// One request = one morphology with its energies, k vectors and E angles.
// The path per energy (src/cudaMain.cu:586-971 restated for one GPU):
//
//   LAB frame (default): the polarization is linear in E (p = Nt E / 4pi,
//   include/uniaxial.h:75, :106-151), and the window, the FFT, the DC
//   replacement and the shift are linear too, so the spectrum of every E
//   angle is  P(angle) = sum_b E_b(angle) FFT(Nt e_b).  The engine transforms
//   the 5 (k along z) or 6 distinct entries of the symmetric tensor Nt once
//   per energy and forms each angle's intensity from them in the Ewald
//   kernel, instead of 3 FFTs per angle.
//   MATERIAL frame: p = R^T Nt R x depends on the angle non-linearly; the
//   engine runs the reference's per-angle schedule (3 volumes per angle).
//
//   k_build -> k_fft_pass<x,y,z> -> k_dc -> per k: k_ewald_angles ->
//   k_rotate_average -> k_fill + k_warp (detector) -> projection[e][k]
//
// FIELDS strategy (fields.cuh): the spectra of the 7 M + 1 energy independent
// morphology fields are formed once per request; every energy and angle is
// combined from them inside the Ewald kernel, batched over energies:
//
//   k_moments -> k_build_fields -> 3D FFT -> per k and
//   energy batch: k_ewald_fields -> k_rotate_average -> k_fill + k_warp
//
// All per-request constants (optical constants of every energy, angle
// coefficients, warp coefficients, q-grid and window tables) are computed on
// the host in double and uploaded once, before any kernel of the request.

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/cyrsoxs.h"
#include "geometry.h"
#include "kernels.cuh"
#include "fields.cuh"
#include "fp64.cuh"

namespace cyr {
namespace {

thread_local std::string g_error;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

#define CYR_CUDA(call)                                                                               \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      return fail(e_ == cudaErrorMemoryAllocation ? CYR_ERR_MEMORY : CYR_ERR_CUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                                \
  } while (0)

#define CYR_TRY(expr)         \
  do {                        \
    int rc_ = (expr);         \
    if (rc_ != CYR_OK) return rc_; \
  } while (0)

// ---------------------------------------------------------------------------
// FFT plans
// ---------------------------------------------------------------------------
bool factorize(uint32_t n, std::vector<uint32_t> &radix) {
  radix.clear();
  uint32_t r = n;
  while (r % 8 == 0) radix.push_back(8), r /= 8;
  while (r % 4 == 0) radix.push_back(4), r /= 4;
  while (r % 2 == 0) radix.push_back(2), r /= 2;
  for (uint32_t p : {3u, 5u, 7u})
    while (r % p == 0) radix.push_back(p), r /= p;
  return r == 1 && radix.size() <= 16;
}

constexpr size_t kFftSmemBudget = 200 * 1024;

// The FFT kernels address elements inside one volume with 32-bit offsets.
constexpr size_t kMaxVolumeVoxels = 0xffffffffull;

// Lines per block: about 4096 elements per tile, at most 16 lines.
uint32_t fft_lines_per_block(uint32_t n) {
  uint32_t tx = 16;
  while (tx > 1 && size_t(n) * tx > 4096) tx /= 2;
  while (tx > 1 && size_t(2) * n * (tx + 1) * sizeof(float2) > kFftSmemBudget) tx /= 2;
  return tx;
}

bool smooth7(uint32_t n) {
  std::vector<uint32_t> r;
  return factorize(n, r);
}

// Lengths with a prime factor above 7 run as Bluestein transforms over a
// padded length M >= 2N - 1, itself limited to one block's FFT: the next power
// of two while that is at most 1024 (the warp FFT's lengths), else the
// smallest 7-smooth M.
constexpr uint32_t kMaxBluesteinPad = 4096;
uint32_t bluestein_length(uint32_t n) {
  uint32_t p2 = 128;
  while (p2 < 2 * n - 1) p2 *= 2;
  if (p2 <= 1024) return p2;
  uint32_t m = 2 * n - 1;
  while (!smooth7(m)) ++m;
  return m;
}

// An axis length the FFT handles: 7-smooth within one block's shared memory,
// or any other length whose Bluestein length is at most kMaxBluesteinPad.
bool fft_length_ok(uint32_t n, const char **why) {
  if (n <= 1) return true;
  if (smooth7(n)) {
    if (size_t(2) * n * 2 * sizeof(float2) > kFftSmemBudget) {
      *why = "exceeds the single-block FFT limit";
      return false;
    }
    return true;
  }
  if (n > (kMaxBluesteinPad + 1) / 2 || bluestein_length(n) > kMaxBluesteinPad) {
    *why = "has a prime factor above 7 and exceeds the Bluestein limit of 2048";
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Per-device context: cached twiddle tables and grow-only scratch.
// ---------------------------------------------------------------------------
// Grow-only device buffer.  With `stream` set (serving slots) it allocates
// and frees stream-ordered, so growing one slot's buffer does not stall the
// others; `generation` counts reallocations (captured graphs hold pointers).
struct DeviceBuffer {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  uint64_t *generation = nullptr;
  int ensure(size_t need) {
    if (need <= bytes) return CYR_OK;
    release();
    if (need == 0) return CYR_OK;
    if (stream)
      CYR_CUDA(cudaMallocAsync(&ptr, need, stream));
    else
      CYR_CUDA(cudaMalloc(&ptr, need));
    bytes = need;
    if (generation) ++*generation;
    return CYR_OK;
  }
  void release() {
    if (ptr) {
      if (stream)
        cudaFreeAsync(ptr, stream);
      else
        cudaFree(ptr);
      if (generation) ++*generation;
    }
    ptr = nullptr;
    bytes = 0;
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

// Optional per-launch timing: an event pair around every kernel launch,
// read back after the caller has synchronised (cyr_profile_end).
enum Stage {
  kBuild = 0, kFftX, kFftY, kFftZ, kDc, kEwald, kRotate, kFill, kWarp, kMom, kMeans, kBuildZ,
  kFieldMeans, kBuildFields, kEwaldFields, kRotateGram, kFftRows, kFftColsY, kFftColsZ, kBluestein, kBuildFieldsRows,
  kZMask, kNumStages
};
const char *const kStageNames[kNumStages] = {"k_build", "k_fft_pass<x>", "k_fft_pass<y>", "k_fft_pass<z>", "k_dc",
                                             "k_ewald_angles", "k_rotate_average", "k_fill", "k_warp",
                                             "k_moments", "k_entry_means", "k_build_fft_z",
                                             "k_field_means", "k_build_fields", "k_ewald_fields", "k_rotate_gram",
                                             "k_fft_rows", "k_fft_cols<y>", "k_fft_cols<z>", "k_bluestein",
                                             "k_build_fields_rows", "k_zmask"};

// Launches made while a stream is being captured into a CUDA graph (the
// serving slots' graphs) are not timed: an event recorded during capture
// becomes a graph node and cannot be waited on.  They count as dropped.  The
// serving worker and the caller's thread both reach the profiler, so its
// state is guarded by its own mutex.
struct Profiler {
  std::atomic<bool> active{false};
  std::mutex mu;
  std::vector<cudaEvent_t> events;  // pairs
  std::vector<int> stage;           // stage of pair i
  std::vector<int> count;           // kernel launches inside pair i
  size_t used = 0;                  // pairs recorded
  size_t dropped = 0;
  int begin(int st, cudaStream_t s, int launches = 1) {
    if (!active.load(std::memory_order_relaxed)) return -1;
    std::lock_guard<std::mutex> lk(mu);
    if (!active.load(std::memory_order_relaxed)) return -1;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (used >= stage.size() || cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
      dropped += launches;
      return -1;
    }
    stage[used] = st;
    count[used] = launches;
    cudaEventRecord(events[2 * used], s);
    return int(used++);
  }
  void end(int slot, cudaStream_t s) {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(mu);
    if (size_t(slot) < used) cudaEventRecord(events[2 * size_t(slot) + 1], s);
  }
};

// Autotuned launch configuration of the fused build + z FFT per shape.
struct ZTune {
  bool stage = false;
  uint32_t tx = 4;
  float ms = 0.f;
};

// Device scratch of one request in flight (grow-only).  The plain entry points
// share the device context's; every serving slot owns one.
struct Scratch {
  DeviceBuffer spec, images, avg, params, dc, moments, means, errors, conv, flags, fmean;
  DeviceBuffer blue;               // padded lines of the Bluestein transforms
  DeviceBuffer zmask;              // store mask of the FIELDS z pass (k_zmask)
  cudaEvent_t last_use = nullptr;  // completion of the last request that used it
  uint64_t generation = 0;         // bumped by every (re)allocation of a buffer above
  int init() {
    if (!last_use) CYR_CUDA(cudaEventCreateWithFlags(&last_use, cudaEventDisableTiming));
    return CYR_OK;
  }
  // serving slots: stream-ordered allocations on `st`
  void bind(cudaStream_t st) {
    for (DeviceBuffer *b : {&spec, &images, &avg, &params, &dc, &moments, &means, &errors, &conv, &flags, &fmean, &blue, &zmask})
      b->stream = st, b->generation = &generation;
  }
  void release() {
    for (DeviceBuffer *b : {&spec, &images, &avg, &params, &dc, &moments, &means, &errors, &conv, &flags, &fmean, &blue, &zmask})
      b->release();
  }
};

// Launch forms of a y or z column pass (autotuned per shape on the FIELDS path):
// TMA tiles with a producer warp (32-column tiles in three stages for 128-
// and 256-point lines when nx allows, 16 columns in two stages for 512, 8 for
// 1024), the same 256-point tiles in two stages, the block-synchronous TMA
// form (256-point lines), or cp.async tiles.  All forms run the same warp FFT,
// so their results are identical; kFormAuto is the fixed choice below.
enum ColForm : uint32_t { kFormAuto = 0, kFormTmaWs = 1, kFormTmaSync = 2, kFormCp = 3, kFormTmaWs2 = 4 };
const char *form_name(uint32_t f) {
  return f == kFormTmaWs     ? "tma_ws"
         : f == kFormTmaWs2  ? "tma_ws2"
         : f == kFormTmaSync ? "tma_sync"
         : f == kFormCp      ? "cp_async"
                             : "auto";
}

struct DeviceContext {
  int device = -1;
  Profiler prof;
  std::mutex mu;         // the plain entry points (they share `main`)
  std::mutex tables_mu;  // twiddles, autotuning results, kernel attributes
  std::map<std::string, ZTune> ztune;  // key: nx,ny,nz,nmat,nvol,morphology
  struct FieldTune {
    uint32_t form[3] = {kFormAuto, kFormAuto, kFormAuto};  // per axis (y and z tuned)
    bool fused = true;                                     // field build fused with the x pass
    std::string report;
  };
  std::map<std::string, FieldTune> ftune;  // key: nx,ny,nz,npk (FIELDS path)
  bool autotune = true;                    // CYRSOXS_GB300_AUTOTUNE=0 keeps the fixed choices
  bool sparse_ewald = true;                // CYRSOXS_GB300_SPARSE_EWALD=0 forms every combination term
  bool zmask = true;                       // CYRSOXS_GB300_ZMASK=0: the FIELDS z pass stores every plane
  bool attrs_done = false;
  bool attrs64 = false;                    // the FP64 FFT kernels' shared-memory attribute is set
  std::map<uint32_t, float2 *> twiddles;
  struct BlueTables {
    uint32_t m = 0;
    float2 *chirp = nullptr, *bhat = nullptr;
  };
  std::map<uint32_t, BlueTables> blue;  // per Bluestein line length
  std::map<uint32_t, double2 *> tw64;   // FP64 twiddles W_n^m per length
  struct BlueTables64 {
    uint32_t m = 0;
    double2 *chirp = nullptr, *bhat = nullptr;
  };
  std::map<uint32_t, BlueTables64> blue64;  // the FP64 pipeline's Bluestein tables per line length
  struct Fp64Scratch {
    DeviceBuffer spec, images, avg, params, params64, vox, out, blue;
  } f64;                                // the FP64 pipeline's buffers (plain entry points)
  Scratch main;
  DeviceBuffer vox_in, out_in;  // host-buffer entry points: morphology and projections
  // cyr_cuda_main's compute and copy streams and its slab-upload events, made once per device and reused
  // by every call (the calls hold `mu`)
  cudaStream_t main_stream = nullptr, copy_stream = nullptr;
  std::vector<cudaEvent_t> slab_events;
  // TMA column passes: the driver's tensor-map encoder, and a word set when a
  // tile copy did not complete within the kernel's wait limit
  void *encode_tiled = nullptr;
  unsigned *tma_error = nullptr;
};

std::mutex g_ctx_mu;
std::map<int, std::unique_ptr<DeviceContext>> g_ctx;

int get_context(DeviceContext **out) {
  int dev = 0;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
    cudaGetLastError();
    return fail(CYR_ERR_NO_DEVICE, "no CUDA device visible");
  }
  CYR_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto &slot = g_ctx[dev];
  if (!slot) {
    slot.reset(new DeviceContext);
    slot->device = dev;
    const char *env = std::getenv("CYRSOXS_GB300_AUTOTUNE");
    slot->autotune = !(env && std::strcmp(env, "0") == 0);
    env = std::getenv("CYRSOXS_GB300_ZMASK");
    slot->zmask = !(env && std::strcmp(env, "0") == 0);
    env = std::getenv("CYRSOXS_GB300_SPARSE_EWALD");
    slot->sparse_ewald = !(env && std::strcmp(env, "0") == 0);
  }
  *out = slot.get();
  return CYR_OK;
}

// Columns per block of the strided warp-FFT passes (one warp per column):
// 8 along y (row stride), 16 along z (plane stride), the faster of the two on
// GB300 for each.
constexpr uint32_t kColsTxY = 8, kColsTxZ = 16;

int setup_attrs(DeviceContext &ctx) {
  std::lock_guard<std::mutex> lk(ctx.tables_mu);
  if (ctx.attrs_done) return CYR_OK;
  const int smem = int(kFftSmemBudget);
  CYR_CUDA(cudaFuncSetAttribute(k_fft_pass<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_CUDA(cudaFuncSetAttribute(k_fft_pass<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_CUDA(cudaFuncSetAttribute(k_fft_pass<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
#define CYR_COLS_ATTR(V, T) \
  CYR_CUDA(cudaFuncSetAttribute(k_fft_cols<V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_COLS_ATTR(32, 8)
  CYR_CUDA(cudaFuncSetAttribute(k_fft_rows<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_COLS_ATTR(4, kColsTxY) CYR_COLS_ATTR(8, kColsTxY) CYR_COLS_ATTR(16, kColsTxY)
  CYR_COLS_ATTR(4, kColsTxZ) CYR_COLS_ATTR(8, kColsTxZ) CYR_COLS_ATTR(16, kColsTxZ)
#undef CYR_COLS_ATTR
  CYR_CUDA(cudaFuncSetAttribute(k_build_fft_z<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_CUDA(cudaFuncSetAttribute(k_build_fft_z<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_CUDA(cudaFuncSetAttribute(k_build_fft_z<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
#define CYR_WARP_Z_ATTR(V, T)                                                                                     \
  CYR_CUDA(cudaFuncSetAttribute(k_build_fft_z_warp<0, true, V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));  \
  CYR_CUDA(cudaFuncSetAttribute(k_build_fft_z_warp<0, false, V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
  CYR_CUDA(cudaFuncSetAttribute(k_build_fft_z_warp<1, false, V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
#define CYR_WARP_Z_ATTR_V(V) CYR_WARP_Z_ATTR(V, 2) CYR_WARP_Z_ATTR(V, 4) CYR_WARP_Z_ATTR(V, 8)
  CYR_WARP_Z_ATTR_V(4)
  CYR_WARP_Z_ATTR_V(8)
  CYR_WARP_Z_ATTR_V(16)
#undef CYR_WARP_Z_ATTR_V
#undef CYR_WARP_Z_ATTR
  CYR_CUDA(cudaFuncSetAttribute(k_fft_cols_tma<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(cols_tma_smem(256))));
#define CYR_WS_ATTR(V, H, S)                                                                               \
  CYR_CUDA(cudaFuncSetAttribute(k_fft_cols_tma_ws<V, H, S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                int(cols_tma_ws_smem<V, H, S>())));                                         \
  CYR_CUDA(cudaFuncSetAttribute(k_fft_cols_tma_ws<V, H, S, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                int(cols_tma_ws_smem<V, H, S>())));
  CYR_WS_ATTR(16, 1, 2)
  CYR_WS_ATTR(8, 2, 3)
  CYR_WS_ATTR(8, 2, 2)
  CYR_WS_ATTR(4, 1, 2)
  CYR_WS_ATTR(4, 2, 3)
#undef CYR_WS_ATTR
  CYR_CUDA(cudaFuncSetAttribute(k_fft_cols_tma64<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(cols_tma64_smem(1024))));
#define CYR_ROWS_ATTR(M, V) \
  CYR_CUDA(cudaFuncSetAttribute(k_build_fields_rows<M, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CYR_ROWS_ATTR(0, 4) CYR_ROWS_ATTR(0, 8) CYR_ROWS_ATTR(0, 16) CYR_ROWS_ATTR(0, 32)
  CYR_ROWS_ATTR(1, 4) CYR_ROWS_ATTR(1, 8) CYR_ROWS_ATTR(1, 16) CYR_ROWS_ATTR(1, 32)
#undef CYR_ROWS_ATTR
  {
    cudaDriverEntryPointQueryResult q{};
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      ctx.encode_tiled = fn;
    cudaGetLastError();
    CYR_CUDA(cudaMalloc(&ctx.tma_error, sizeof(unsigned)));
    CYR_CUDA(cudaMemset(ctx.tma_error, 0, sizeof(unsigned)));
  }
  ctx.attrs_done = true;
  return CYR_OK;
}

int get_twiddles(DeviceContext &ctx, uint32_t n, const float2 **tw) {
  std::lock_guard<std::mutex> lk(ctx.tables_mu);
  auto it = ctx.twiddles.find(n);
  if (it != ctx.twiddles.end()) {
    *tw = it->second;
    return CYR_OK;
  }
  std::vector<float2> h(n);
  for (uint32_t m = 0; m < n; ++m) {
    const double a = -2.0 * kPi * double(m) / double(n);  // W_n^m = exp(-2 pi i m / n), in double
    h[m] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
  }
  float2 *d = nullptr;
  CYR_CUDA(cudaMalloc(&d, sizeof(float2) * n));
  CYR_CUDA(cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  ctx.twiddles[n] = d;
  *tw = d;
  return CYR_OK;
}

int make_axis(DeviceContext &ctx, uint32_t n, FftAxis &ax) {
  std::vector<uint32_t> r;
  if (!factorize(n, r)) return fail(CYR_ERR_UNSUPPORTED, "FFT length %u has a prime factor above 7", n);
  ax.n = n;
  ax.log2n = 0;
  if ((n & (n - 1)) == 0 && n > 1)
    while ((1u << ax.log2n) < n) ++ax.log2n;
  ax.nstages = uint32_t(r.size());
  ax.radix_code = 0;
  for (size_t i = 0; i < r.size(); ++i) ax.radix_code |= uint64_t(r[i]) << (4 * i);
  return get_twiddles(ctx, n, &ax.tw);
}

// Tensor map of `count` float2 volumes seen as (x, y, z, volume), volumes nvox
// elements apart, for TMA tiles of 16 columns x `box` lines along `axis`
// (1: y, 2: z), 128-byte swizzle.
int encode_cols_map(DeviceContext &ctx, CUtensorMap *map, void *data, uint32_t nx, uint32_t ny, uint32_t nz,
                    uint32_t count, size_t nvox, int axis, uint32_t box, uint32_t cols = kTmaCols) {
  const cuuint64_t dims[4] = {nx, ny, nz, count};
  const cuuint64_t strides[3] = {cuuint64_t(nx) * 8, cuuint64_t(nx) * ny * 8, cuuint64_t(nvox) * 8};
  const cuuint32_t boxd[4] = {cols, axis == 1 ? box : 1u, axis == 2 ? box : 1u, 1u};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  const CUresult r = reinterpret_cast<Encode>(ctx.encode_tiled)(
      map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, data, dims, strides, boxd, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
      cols == 16 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(CYR_ERR_CUDA, "tensor map encoding failed (%d)", int(r));
  return CYR_OK;
}

// One axis of the 3D FFT with the warp-level kernels (n = 128, 256, 512, 1024).
// zmask: the z pass's store mask (ColTmaParams::smask), used by the forms with
// a producer warp for 128-, 256- and 512-point lines; null stores every plane.
template <int V>
int warp_fft_pass_v(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, int axis,
                    cudaStream_t st, size_t nvox, uint32_t form = kFormAuto, const uint32_t *zmask = nullptr) {
  constexpr uint32_t N = 32 * V;
  const float2 *tw = nullptr;
  CYR_TRY(get_twiddles(ctx, N, &tw));
  const int slot = ctx.prof.begin(axis == 0 ? kFftRows : axis == 1 ? kFftColsY : kFftColsZ, st);
  if (axis == 0) {
    RowPassParams rp{data, uint32_t(size_t(ny) * nz * count), tw, ny * nz, nvox};
    const size_t smem = (N + 8 * N) * sizeof(float2);
    k_fft_rows<V><<<(rp.rows + 7) / 8, 256, smem, st>>>(rp);
  } else if (V == 32 && nx % 8 == 0 && ctx.encode_tiled && ctx.tma_error && form != kFormCp) {
    // 1024-point lines: 8-column tiles (k_fft_cols_tma64)
    CUtensorMap map;
    CYR_TRY(encode_cols_map(ctx, &map, data, nx, ny, nz, count, nvox, axis, 256, 8));
    ColTmaParams tp{};
    tp.nxt = nx / 8;
    tp.others = axis == 1 ? nz : ny;
    tp.ntiles = tp.nxt * tp.others * count;
    tp.axis = uint32_t(axis);
    tp.tw = tw;
    tp.error = ctx.tma_error;
    int sms = 0, per_sm = 0;
    CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
    CYR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_cols_tma64<32>, 9 * 32, cols_tma64_smem(N)));
    const unsigned grid = unsigned(std::min<size_t>(tp.ntiles, size_t(std::max(1, per_sm)) * sms));
    k_fft_cols_tma64<32><<<grid, 9 * 32, cols_tma64_smem(N), st>>>(map, tp);
  } else if ((V == 4 || V == 8 || V == 16) && nx % kTmaCols == 0 && ctx.encode_tiled && ctx.tma_error &&
             form != kFormCp) {
    CUtensorMap map, smap;
    CYR_TRY(encode_cols_map(ctx, &map, data, nx, ny, nz, count, nvox, axis, N < 256 ? N : 256));
    smap = map;
    ColTmaParams tp{};
    if (axis == 2 && zmask) {  // 8-plane boxes for the masked stores
      CYR_TRY(encode_cols_map(ctx, &smap, data, nx, ny, nz, count, nvox, axis, 8));
      tp.smask = zmask;
      tp.mwords = (N / 8 + 31) / 32;
    }
    tp.nxt = nx / kTmaCols;
    tp.others = axis == 1 ? nz : ny;
    tp.ntiles = tp.nxt * tp.others * count;
    tp.axis = uint32_t(axis);
    tp.tw = tw;
    tp.error = ctx.tma_error;
    int sms = 0, per_sm = 0;
    CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
    // 128-point lines: 32 columns in three stages (nx a multiple of 32) or 16 in two,
    // with a producer warp; 256-point lines: 32 columns with a producer warp in
    // three or two stages (nx a multiple of 32; 256-byte runs per line), else the
    // block-synchronous 16-column form; 512-point lines: 16 columns, two stages.
    // A producer-warp form: H halves of 16 columns, S stages.
    auto launch_ws = [&](auto vc, auto hc, auto sc) -> int {
      constexpr int VV = decltype(vc)::value, HH = decltype(hc)::value, SS = decltype(sc)::value;
      tp.nxt = nx / (HH * kTmaCols);
      tp.ntiles = tp.nxt * tp.others * count;
      constexpr size_t smem = cols_tma_ws_smem<VV, HH, SS>();
      // the masked form (z pass with a store mask) is its own instantiation, so
      // the unmasked passes keep the plain tile walk and its registers
      auto kern = tp.smask ? k_fft_cols_tma_ws<VV, HH, SS, true> : k_fft_cols_tma_ws<VV, HH, SS, false>;
      CYR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (8 * HH + 1) * 32, smem));
      const unsigned grid = unsigned(std::min<size_t>(tp.ntiles, size_t(std::max(1, per_sm)) * sms));
      kern<<<grid, (8 * HH + 1) * 32, smem, st>>>(map, smap, tp);
      return CYR_OK;
    };
    using I4 = std::integral_constant<int, 4>;
    using I8 = std::integral_constant<int, 8>;
    using I16 = std::integral_constant<int, 16>;
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    using I3 = std::integral_constant<int, 3>;
    if constexpr (V == 4) {
      if (nx % (2 * kTmaCols) == 0)
        CYR_TRY(launch_ws(I4{}, I2{}, I3{}));
      else
        CYR_TRY(launch_ws(I4{}, I1{}, I2{}));
    } else if constexpr (V == 8) {
      if (nx % (2 * kTmaCols) == 0 && form != kFormTmaSync) {
        if (form == kFormTmaWs2)
          CYR_TRY(launch_ws(I8{}, I2{}, I2{}));
        else
          CYR_TRY(launch_ws(I8{}, I2{}, I3{}));
      } else {
        CYR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_cols_tma<8>, kTmaWarps * 32, cols_tma_smem(N)));
        const unsigned grid = unsigned(std::min<size_t>(tp.ntiles, size_t(std::max(1, per_sm)) * sms));
        k_fft_cols_tma<8><<<grid, kTmaWarps * 32, cols_tma_smem(N), st>>>(map, tp);
      }
    } else {
      CYR_TRY(launch_ws(I16{}, I1{}, I2{}));
    }
  } else {
    ColPassParams cp{};
    cp.data = data;
    cp.nx = nx;
    cp.vstride = nvox;
    if (axis == 1) {
      cp.others = nz, cp.ostride = size_t(nx) * ny, cp.estride = nx;
    } else {
      cp.others = ny, cp.ostride = nx, cp.estride = nx * ny;
    }
    cp.tw = tw;
    auto launch = [&](auto txc) {
      constexpr uint32_t TX = decltype(txc)::value;
      const size_t smem = (N + TX * line_stride(N, TX)) * sizeof(float2);
      const dim3 grid(((nx + TX - 1) / TX) * cp.others, count);
      k_fft_cols<V, TX><<<grid, TX * 32, smem, st>>>(cp);
    };
    if (V == 32)  // 1024-point columns: 8 per block keeps the tile at 64 KB
      launch(std::integral_constant<uint32_t, 8>{});
    else if (axis == 1)
      launch(std::integral_constant<uint32_t, kColsTxY>{});
    else
      launch(std::integral_constant<uint32_t, kColsTxZ>{});
  }
  ctx.prof.end(slot, st);
  CYR_CUDA(cudaGetLastError());
  return CYR_OK;
}

int warp_fft_pass(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, int axis,
                  cudaStream_t st, size_t nvox, uint32_t form = kFormAuto, const uint32_t *zmask = nullptr) {
  const uint32_t n = axis == 0 ? nx : axis == 1 ? ny : nz;
  if (n == 128) return warp_fft_pass_v<4>(ctx, data, nx, ny, nz, count, axis, st, nvox, form, zmask);
  if (n == 256) return warp_fft_pass_v<8>(ctx, data, nx, ny, nz, count, axis, st, nvox, form, zmask);
  if (n == 512) return warp_fft_pass_v<16>(ctx, data, nx, ny, nz, count, axis, st, nvox, form, zmask);
  return warp_fft_pass_v<32>(ctx, data, nx, ny, nz, count, axis, st, nvox, form);
}

// The forms that apply to a column pass of n-point lines (axis 1 or 2) for this nx.
std::vector<uint32_t> column_forms(const DeviceContext &ctx, uint32_t n, uint32_t nx) {
  std::vector<uint32_t> f;
  const bool tma = ctx.encode_tiled && ctx.tma_error;
  if (n == 256 && tma && nx % kTmaCols == 0) {
    if (nx % (2 * kTmaCols) == 0) f.push_back(kFormTmaWs);
    if (nx % (2 * kTmaCols) == 0) f.push_back(kFormTmaWs2);
    f.push_back(kFormTmaSync);
  }
  if ((n == 128 || n == 512) && tma && nx % kTmaCols == 0) f.push_back(kFormTmaWs);
  if (n == 1024 && tma && nx % 8 == 0) f.push_back(kFormTmaWs);
  if (n == 128 || n == 256 || n == 512 || n == 1024) f.push_back(kFormCp);
  return f;
}

// One y or z pass with k_fft_thread (lines of 8..64, one thread per line).
int thread_fft_pass(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, int axis,
                    cudaStream_t st, size_t nvox) {
  const uint32_t n = axis == 1 ? ny : nz;
  const float2 *tw = nullptr;
  CYR_TRY(get_twiddles(ctx, n, &tw));
  ThreadPassParams p{};
  p.data = data;
  p.nx = nx;
  p.vstride = nvox;
  p.tw = tw;
  if (axis == 1) {
    p.others = nz, p.ostride = size_t(nx) * ny, p.estride = nx;
  } else {
    p.others = ny, p.ostride = nx, p.estride = size_t(nx) * ny;
  }
  const dim3 grid(unsigned((size_t(nx) * p.others + 127) / 128), count);
  const int slot = ctx.prof.begin(axis == 1 ? kFftColsY : kFftColsZ, st);
  if (n == 8) k_fft_thread<8><<<grid, 128, 0, st>>>(p);
  if (n == 16) k_fft_thread<16><<<grid, 128, 0, st>>>(p);
  if (n == 32) k_fft_thread<32><<<grid, 128, 0, st>>>(p);
  if (n == 64) k_fft_thread<64><<<grid, 128, 0, st>>>(p);
  ctx.prof.end(slot, st);
  CYR_CUDA(cudaGetLastError());
  return CYR_OK;
}

// Chirp c_j = exp(-i pi j^2 / n) and bhat = FFT_m(b) / m, b_j = conj(c_j) at j
// and m - j: in double (j^2 mod 2n in integers, a direct DFT with exact index
// arithmetic), rounded to float, once per length and device.
int get_blue(DeviceContext &ctx, uint32_t n, DeviceContext::BlueTables &out) {
  std::lock_guard<std::mutex> lk(ctx.tables_mu);
  auto it = ctx.blue.find(n);
  if (it != ctx.blue.end()) {
    out = it->second;
    return CYR_OK;
  }
  const uint32_t m = bluestein_length(n);
  std::vector<std::complex<double>> c(n), b(m, 0.0), w(m);
  for (uint32_t j = 0; j < n; ++j) {
    const uint64_t q = (uint64_t(j) * j) % (2 * uint64_t(n));
    c[j] = std::polar(1.0, -kPi * double(q) / double(n));
  }
  for (uint32_t j = 0; j < n; ++j) {
    b[j] = std::conj(c[j]);
    if (j) b[m - j] = std::conj(c[j]);
  }
  for (uint32_t j = 0; j < m; ++j) w[j] = std::polar(1.0, -2.0 * kPi * double(j) / double(m));
  std::vector<float2> hc(n), hb(m);
  for (uint32_t j = 0; j < n; ++j) hc[j] = make_float2(float(c[j].real()), float(c[j].imag()));
  for (uint32_t k = 0; k < m; ++k) {
    std::complex<double> acc(0.0, 0.0);
    uint64_t idx = 0;  // (j k) mod m
    for (uint32_t j = 0; j < m; ++j, idx += k) {
      if (idx >= m) idx %= m;
      acc += b[j] * w[idx];
    }
    acc /= double(m);
    hb[k] = make_float2(float(acc.real()), float(acc.imag()));
  }
  DeviceContext::BlueTables t;
  t.m = m;
  CYR_CUDA(cudaMalloc(&t.chirp, sizeof(float2) * n));
  CYR_CUDA(cudaMalloc(&t.bhat, sizeof(float2) * m));
  CYR_CUDA(cudaMemcpy(t.chirp, hc.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  CYR_CUDA(cudaMemcpy(t.bhat, hb.data(), sizeof(float2) * m, cudaMemcpyHostToDevice));
  ctx.blue[n] = t;
  out = t;
  return CYR_OK;
}

int fft_axes(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, cudaStream_t st,
             int first, int last, size_t vstride = 0, DeviceBuffer *work = nullptr, const uint32_t *forms = nullptr,
             const uint32_t *zmask = nullptr);

// One axis of length n (a prime factor above 7) as a Bluestein transform, in
// chunks of padded lines of at most 256 MB held in `work`.
int bluestein_pass(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, int axis,
                   cudaStream_t st, size_t vstride, DeviceBuffer *work) {
  const uint32_t n = axis == 0 ? nx : axis == 1 ? ny : nz;
  DeviceContext::BlueTables bt;
  CYR_TRY(get_blue(ctx, n, bt));
  const uint32_t lpv = axis == 0 ? ny * nz : axis == 1 ? nx * nz : nx * ny;
  const uint64_t total = uint64_t(lpv) * count;
  // a multiple of 32 lines per chunk, so the column pass of y and z lines can use TMA tiles
  const uint64_t cap = std::max<uint64_t>(32, (size_t(256) << 20) / (size_t(bt.m) * sizeof(float2)) / 32 * 32);
  const uint32_t chunk = uint32_t(std::min<uint64_t>(total, cap));
  CYR_TRY(work->ensure(size_t(chunk) * bt.m * sizeof(float2)));
  int sms = 0;
  CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  BlueParams p{};
  p.data = data;
  p.work = work->as<float2>();
  p.chirp = bt.chirp;
  p.bhat = bt.bhat;
  p.nx = nx, p.ny = ny, p.nz = nz;
  p.vstride = vstride;
  p.n = n, p.m = bt.m;
  p.lines_per_vol = lpv;
  for (uint64_t l0 = 0; l0 < total; l0 += chunk) {
    p.line0 = l0;
    p.nlines = uint32_t(std::min<uint64_t>(chunk, total - l0));
    const size_t elems = size_t(p.nlines) * bt.m;
    const unsigned grid = unsigned(std::min<size_t>((elems + 255) / 256, size_t(sms) * 16));
    int slot = ctx.prof.begin(kBluestein, st);
    if (axis == 0) k_blue_gather<0><<<grid, 256, 0, st>>>(p);
    if (axis == 1) k_blue_gather<1><<<grid, 256, 0, st>>>(p);
    if (axis == 2) k_blue_gather<2><<<grid, 256, 0, st>>>(p);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
    // m is 7-smooth: rows of m (x lines) or columns of m (y and z lines)
    auto padded_fft = [&]() -> int {
      if (axis == 0) return fft_axes(ctx, p.work, bt.m, p.nlines, 1, 1, st, 0, 0);
      return fft_axes(ctx, p.work, p.nlines, bt.m, 1, 1, st, 1, 1);
    };
    CYR_TRY(padded_fft());
    slot = ctx.prof.begin(kBluestein, st);
    if (axis == 0)
      k_blue_mul<0><<<grid, 256, 0, st>>>(p);
    else
      k_blue_mul<1><<<grid, 256, 0, st>>>(p);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
    CYR_TRY(padded_fft());
    slot = ctx.prof.begin(kBluestein, st);
    if (axis == 0) k_blue_scatter<0><<<grid, 256, 0, st>>>(p);
    if (axis == 1) k_blue_scatter<1><<<grid, 256, 0, st>>>(p);
    if (axis == 2) k_blue_scatter<2><<<grid, 256, 0, st>>>(p);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  }
  return CYR_OK;
}

// In-place forward FFT of `count` volumes along the axes [first, last]
// (0 x, 1 y, 2 z).  vstride (elements between volumes) defaults to the volume
// size; a larger one runs the x and y passes on nz planes of larger volumes
// (data pointing at the first plane), as the slab pipeline does.
// Lengths with a prime factor above 7 use `work` (default: the device's main
// scratch, for callers holding the context lock).
int fft_axes(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, cudaStream_t st,
             int first, int last, size_t vstride, DeviceBuffer *work, const uint32_t *forms, const uint32_t *zmask) {
  const size_t nvox = vstride ? vstride : size_t(nx) * ny * nz;
  const uint32_t dims[3] = {nx, ny, nz};
  for (int axis = first; axis <= last; ++axis) {
    const uint32_t n = dims[axis];
    if (n == 1) continue;
    if (!smooth7(n)) {
      CYR_TRY(bluestein_pass(ctx, data, nx, ny, nz, count, axis, st, nvox, work ? work : &ctx.main.blue));
      continue;
    }
    if (n == 128 || n == 256 || n == 512 || n == 1024) {
      CYR_TRY(warp_fft_pass(ctx, data, nx, ny, nz, count, axis, st, nvox, forms ? forms[axis] : kFormAuto,
                            axis == 2 ? zmask : nullptr));
      continue;
    }
    if (axis > 0 && (n == 8 || n == 16 || n == 32 || n == 64) && count <= 65535) {
      CYR_TRY(thread_fft_pass(ctx, data, nx, ny, nz, count, axis, st, nvox));
      continue;
    }
    FftPassParams p{};
    p.data = data;
    p.nx = nx, p.ny = ny, p.nz = nz;
    p.nvox = nvox;
    CYR_TRY(make_axis(ctx, n, p.ax));
    p.tx = fft_lines_per_block(n);
    const size_t smem = (size_t(2) * n * (p.tx + 1) + n) * sizeof(float2);
    if (smem > kFftSmemBudget) return fail(CYR_ERR_UNSUPPORTED, "FFT length %u too large for one block", n);
    uint32_t tiles;
    if (axis == 0) {
      tiles = (ny * nz + p.tx - 1) / p.tx;
    } else {
      const uint32_t nxt = (nx + p.tx - 1) / p.tx;
      tiles = nxt * (axis == 1 ? nz : ny);
    }
    const dim3 grid(tiles, count);
    const int slot = ctx.prof.begin(kFftX + axis, st);
    if (axis == 0) k_fft_pass<0><<<grid, kFftThreads, smem, st>>>(p);
    if (axis == 1) k_fft_pass<1><<<grid, kFftThreads, smem, st>>>(p);
    if (axis == 2) k_fft_pass<2><<<grid, kFftThreads, smem, st>>>(p);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  }
  return CYR_OK;
}

int fft3d(DeviceContext &ctx, float2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, cudaStream_t st,
          bool skip_z = false, DeviceBuffer *work = nullptr) {
  return fft_axes(ctx, data, nx, ny, nz, count, st, 0, skip_z ? 1 : 2, 0, work);
}

// ---------------------------------------------------------------------------
// Request planning
// ---------------------------------------------------------------------------
struct Plan {
  uint32_t nx, ny, nz, nmat, ne, nk, nang;
  size_t nvox, npix;
  bool material_frame, hanning, twod, interp_nn = false, euler = false;
  uint32_t nbasis, nvol;           // LAB: 2 or 3 bases; MATERIAL: 1 basis, 3 volumes
  std::vector<KFrame> frames;
  Mat3f detector;
  std::vector<float> start_inc;    // start, inc
  // host parameter arena, uploaded once
  std::vector<unsigned char> arena;
  size_t off_mc = 0, off_coef = 0, off_warp = 0, off_qx = 0, off_qy = 0, off_qz = 0, off_hx = 0, off_hy = 0, off_hz = 0;
  std::vector<WarpCoef> detector_warp;  // per k
  std::vector<float> evec;              // [k][angle][3] E = R x
  std::vector<Mat3f> rmats;             // [k][angle] (MATERIAL frame)
  std::vector<float> eangles;           // [k][angle]
  float start, inc;
  // z pruning: the spectra keep shifted planes [zlo, zlo + kz) only
  bool pruned = false;
  uint32_t zlo = 0, kz = 0, ztx = 1;
  bool zwarp = false;                   // warp-FFT form of the fused kernel
  bool zstage = false;                  // ... with the morphology tile staged in shared memory
  std::vector<ZTune> zcands;            // autotuning candidates of the warp form
  size_t vstride = 0;                   // elements per spectrum volume
  uint32_t p0 = 0, p1 = 0, pn = 0;      // planes of unshifted z bins 0, 1, nz-1
  // FIELDS strategy
  bool fields = false;
  uint32_t npk = 0;                     // packed field volumes
  uint32_t ebatch = 1;                  // energies per Ewald / rotation launch
  bool ewald_sparse = false;            // the combination coefficients keep their structural zeros
  size_t off_fcoef = 0, off_kmag = 0, off_mat = 0, off_kvec = 0;
  uint32_t mom_zstep = 1;               // z planes between the moment samples (FIELDS)
  // LAB frame, square detector: conservative per-row column ranges of the
  // Ewald output, [k][energy][row] (ewald_rows)
  bool has_rows = false;
  size_t off_rows = 0;
};

// Energies per Gram record: the FIELDS strategy packs 12 floats per pixel (4
// energies with 2 bases, 2 with 3); the per-energy path keeps one.
inline uint32_t gram_nep(const Plan &pl) { return pl.fields && !pl.material_frame ? (pl.nbasis == 2 ? 4u : 2u) : 1u; }

// Bytes of the Ewald output of nb energies: Gram records in the LAB frame
// (rotated by k_rotate_gram), per-angle images in the MATERIAL frame
// (k_rotate_average).
size_t image_bytes(const Plan &pl, uint32_t nb = 1) {
  if (pl.material_frame) return size_t(nb) * pl.nang * pl.npix * sizeof(float);
  const uint32_t nep = gram_nep(pl), ng = pl.nbasis * (pl.nbasis + 1) / 2;
  const size_t rq = (size_t(nep) * ng + 3) / 4;
  return size_t((nb + nep - 1) / nep) * gram_plane_size(int(pl.ny), int(pl.nx)) * rq * sizeof(float4);
}

// Device bytes of the FIELDS strategy: packed field spectra, per-batch images and averages.
size_t field_bytes(const Plan &pl) {
  return size_t(pl.npk) * pl.nvox * sizeof(float2) + image_bytes(pl, pl.ebatch) +
         size_t(pl.ebatch) * pl.npix * sizeof(float) + pl.arena.size() + (num_fields(pl.nmat) + 2 * pl.npk) * sizeof(float2);
}

// Dynamic shared memory of k_build_fft_z_warp: twiddles, lines, optional tile.
inline size_t zwarp_smem(uint32_t nz, uint32_t nvol, uint32_t tx, uint32_t nmat, bool stage) {
  size_t f2 = nz + size_t(nvol) * tx * line_stride(nz, tx);
  f2 += f2 & 1;  // the float4 tile starts 16-byte aligned
  return f2 * sizeof(float2) + (stage ? size_t(nmat) * nz * tx * sizeof(float4) : 0);
}

inline uint32_t igor_host(uint32_t j, uint32_t n) { return j <= n / 2 ? n / 2 - j : n + n / 2 - j; }

// Shifted z planes the Ewald projection can read, for every energy and k of
// the request.  posz = -kz + sqrt(val) grows with val = k^2 - (kx+qx)^2 -
// (ky+qy)^2, which separates in X and Y, so the extremes over the detector
// come from the extremes of two 1D arrays; val >= 0 bounds posz below by -kz.
// The range is widened by a plane on each side and always holds the planes
// of the DC neighbours.
void kept_planes(const cyr_options *o, Plan &pl) {
  const float start = -static_cast<float>(kPi / o->phys_size);
  const float dx = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nx - 1) * 1.0));
  const float dy = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.ny - 1) * 1.0));
  const float dz = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nz - 1) * 1.0));
  double tlo = 1e300, thi = -1e300;
  for (uint32_t e = 0; e < pl.ne; ++e) {
    const float kmag = static_cast<float>(2 * kPi / static_cast<float>(1239.84197 / o->energies[e]));
    for (const KFrame &f : pl.frames) {
      const double kx = kmag * f.k.x, ky = kmag * f.k.y, kz = kmag * f.k.z;
      double amin = 1e300, bmin = 1e300;
      for (uint32_t X = 0; X + 1 < pl.nx; ++X) {
        const double a = kx + double(start + X * dx);
        amin = std::min(amin, a * a);
      }
      for (uint32_t Y = 0; Y + 1 < pl.ny; ++Y) {
        const double b = ky + double(start + Y * dy);
        bmin = std::min(bmin, b * b);
      }
      const double vmax = double(kmag) * kmag - amin - bmin;
      if (vmax < 0) continue;
      tlo = std::min(tlo, (-kz - start) / dz);
      thi = std::max(thi, (-kz + std::sqrt(vmax) - start) / dz);
    }
  }
  long lo = long(pl.nz), hi = -1;
  if (tlo <= thi) {
    if (pl.interp_nn) {
      lo = long(std::floor(tlo + 0.5)) - 1, hi = long(std::floor(thi + 0.5)) + 1;
    } else {
      lo = long(std::floor(tlo)) - 1, hi = long(std::floor(thi)) + 2;
    }
    lo = std::max(lo, 0L), hi = std::min(hi, long(pl.nz) - 1);
  }
  for (uint32_t u : {0u, 1u, pl.nz - 1}) {
    const long z = long(igor_host(u % pl.nz, pl.nz));
    lo = std::min(lo, z), hi = std::max(hi, z);
  }
  pl.zlo = uint32_t(lo);
  pl.kz = uint32_t(hi - lo + 1);
  pl.p0 = igor_host(0, pl.nz) - pl.zlo;
  pl.p1 = igor_host(1 % pl.nz, pl.nz) - pl.zlo;
  pl.pn = igor_host(pl.nz - 1, pl.nz) - pl.zlo;
}

template <class T>
size_t arena_put(std::vector<unsigned char> &a, const T *src, size_t count) {
  size_t off = (a.size() + 255) & ~size_t(255);
  a.resize(off + sizeof(T) * count);
  if (count) std::memcpy(a.data() + off, src, sizeof(T) * count);
  return off;
}

// Column ranges of the Ewald output that can hold a number, per k, energy and
// detector row (LAB frame, square detector, where the rotation's image row y
// is detector row Y).  ewald_geometry marks a pixel NaN unless
// val = k^2 - (kx + qx)^2 - (ky + qy)^2 >= 0, so outside the disc
// |kx + qx| <= sqrt(k^2 - (ky + qy)^2) the pixel is NaN.  The bound takes val
// down to -1e-5 k^2 and adds two columns on each side, far beyond the float
// rounding of the device's test; a row with no such column stores [W, -1].
void ewald_rows(const cyr_options *o, Plan &pl) {
  pl.has_rows = !pl.material_frame && pl.nx == pl.ny && size_t(pl.nx) * sizeof(int2) <= 48 * 1024;
  if (!pl.has_rows) return;
  const int W = int(pl.ny), H = int(pl.nx);
  const float start = -static_cast<float>(kPi / o->phys_size);
  const float dy = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.ny - 1) * 1.0));
  const float dx = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nx - 1) * 1.0));
  std::vector<int2> rows(size_t(pl.nk) * pl.ne * H);
  for (uint32_t k = 0; k < pl.nk; ++k)
    for (uint32_t e = 0; e < pl.ne; ++e) {
      const float kmag = static_cast<float>(2 * kPi / static_cast<float>(1239.84197 / o->energies[e]));
      const double kx = double(kmag * pl.frames[k].k.x), ky = double(kmag * pl.frames[k].k.y);
      for (int Y = 0; Y < H; ++Y) {
        int lo = W, hi = -1;
        const double ay = ky + double(start + float(Y) * dy);
        const double r2 = double(kmag) * kmag * (1.0 + 1e-5) - ay * ay;
        if (r2 >= 0) {
          const double r = std::sqrt(r2);
          const double xl = (-kx - r - double(start)) / double(dx), xh = (-kx + r - double(start)) / double(dx);
          lo = int(std::max(0.0, std::floor(xl) - 2.0));
          hi = int(std::min(double(W - 1), std::ceil(xh) + 2.0));
          if (hi < lo) lo = W, hi = -1;
        }
        rows[(size_t(k) * pl.ne + e) * H + Y] = int2{lo, hi};
      }
    }
  pl.off_rows = arena_put(pl.arena, rows.data(), rows.size());
}

// make_kframe scans 100 000 candidate base angles (as the reference does per
// call); the frame depends only on k, so it is computed once per k vector.
KFrame cached_kframe(const Vec3f &k) {
  static std::mutex mu;
  static std::map<std::array<uint32_t, 3>, KFrame> cache;
  std::array<uint32_t, 3> key;
  std::memcpy(key.data(), &k.x, 4), std::memcpy(key.data() + 1, &k.y, 4), std::memcpy(key.data() + 2, &k.z, 4);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const KFrame f = make_kframe(k);
  std::lock_guard<std::mutex> lk(mu);
  cache.emplace(key, f);
  return f;
}

int validate(const cyr_options *o) {
  if (!o) return fail(CYR_ERR_ARGUMENT, "options pointer is null");
  if (o->nx < 2 || o->ny < 2 || o->nz < 1) return fail(CYR_ERR_ARGUMENT, "dimensions must be nx, ny >= 2, nz >= 1");
  if (o->num_material < 1 || o->num_material > uint32_t(kMaxMaterials))
    return fail(CYR_ERR_ARGUMENT, "num_material must be in [1, %d]", kMaxMaterials);
  if (o->num_energies < 1 || !o->energies) return fail(CYR_ERR_ARGUMENT, "no energies");
  if (!(o->phys_size > 0)) return fail(CYR_ERR_ARGUMENT, "phys_size must be positive");
  if (o->case_type > 2) return fail(CYR_ERR_ARGUMENT, "case_type must be 0, 1 or 2");
  if (o->case_type != 0 && (o->num_k < 1 || !o->k_vectors)) return fail(CYR_ERR_ARGUMENT, "k vectors missing");
  if (o->morphology_type > 1 || o->ewald_interpolation > 1 || o->windowing > 1 || o->scatter_approach > 1 ||
      o->algorithm > 1 || o->reference_frame > 1 || o->strategy > 2)
    return fail(CYR_ERR_ARGUMENT, "enumerated option out of range");
  if (o->start_angle > o->end_angle) return fail(CYR_ERR_ARGUMENT, "start angle greater than end angle");
  if (!near_equal(o->start_angle, o->end_angle) && near_equal(o->increment_angle, 0.f))
    return fail(CYR_ERR_ARGUMENT, "increment angle is 0");
  for (uint32_t e = 0; e < o->num_energies; ++e)
    if (!(o->energies[e] > 0)) return fail(CYR_ERR_ARGUMENT, "energies must be positive");
  if (size_t(o->nx) * o->ny * o->nz > kMaxVolumeVoxels)
    return fail(CYR_ERR_UNSUPPORTED, "volume of %u x %u x %u voxels exceeds the limit of 2^32 - 1 voxels", o->nx, o->ny,
                o->nz);
  const uint32_t d[3] = {o->nx, o->ny, o->nz};
  for (uint32_t n : d) {
    const char *why = "";
    if (!fft_length_ok(n, &why)) return fail(CYR_ERR_UNSUPPORTED, "dimension %u %s", n, why);
  }
  return CYR_OK;
}

int make_plan(const cyr_options *o, const float *optical, Plan &pl) {
  CYR_TRY(validate(o));
  if (!optical) return fail(CYR_ERR_ARGUMENT, "optical constants pointer is null");
  pl.nx = o->nx, pl.ny = o->ny, pl.nz = o->nz, pl.nmat = o->num_material, pl.ne = o->num_energies;
  pl.nvox = size_t(pl.nx) * pl.ny * pl.nz;
  pl.npix = size_t(pl.nx) * pl.ny;
  pl.twod = pl.nz == 1;
  pl.material_frame = o->reference_frame == 0;
  pl.hanning = o->algorithm == 0 && o->windowing == 1;
  // E-angle schedule (InputData::setEAngles, src/cudaMain.cu:393-394)
  pl.start = o->start_angle;
  pl.inc = near_equal(o->start_angle, o->end_angle) ? 1.0f : o->increment_angle;
  const float nang_f = std::round((o->end_angle - o->start_angle) / pl.inc + 1);
  if (!(nang_f >= 1) || nang_f > float(kMaxAngles)) return fail(CYR_ERR_ARGUMENT, "angle count out of range");
  pl.nang = uint32_t(nang_f);
  // k vectors and frames (src/RotationMatrix.cpp:30-51)
  std::vector<Vec3f> ks;
  if (o->case_type == 0 && (o->num_k == 0 || !o->k_vectors)) {
    ks.push_back({0.f, 0.f, 1.f});
  } else {
    for (uint32_t i = 0; i < o->num_k; ++i) ks.push_back({o->k_vectors[3 * i], o->k_vectors[3 * i + 1], o->k_vectors[3 * i + 2]});
  }
  pl.nk = uint32_t(ks.size());
  for (const Vec3f &k : ks) pl.frames.push_back(cached_kframe(k));
  const Vec3f det = o->case_type == 2 ? Vec3f{o->detector[0], o->detector[1], o->detector[2]} : Vec3f{0.f, 0.f, 1.f};
  pl.detector = rotation_between({0.f, 0.f, 1.f}, det);
  // per (k, angle): E angle, rotation, E vector
  bool any_ez = false;
  pl.evec.resize(size_t(pl.nk) * pl.nang * 3);
  pl.rmats.resize(size_t(pl.nk) * pl.nang);
  pl.eangles.resize(size_t(pl.nk) * pl.nang);
  for (uint32_t k = 0; k < pl.nk; ++k)
    for (uint32_t a = 0; a < pl.nang; ++a) {
      const float ang = e_angle(pl.frames[k], pl.start, pl.inc, a);
      const Mat3f R = e_rotation(pl.frames[k], ang);
      const size_t ka = size_t(k) * pl.nang + a;
      pl.eangles[ka] = ang;
      pl.rmats[ka] = R;
      pl.evec[ka * 3 + 0] = R(0, 0);
      pl.evec[ka * 3 + 1] = R(1, 0);
      pl.evec[ka * 3 + 2] = R(2, 0);
      if (R(2, 0) != 0.f) any_ez = true;
    }
  if (pl.material_frame) {
    pl.nbasis = 1;
    pl.nvol = 3;
  } else {
    pl.nbasis = any_ez ? 3 : 2;
    pl.nvol = any_ez ? 6 : 5;
  }
  pl.interp_nn = o->ewald_interpolation == 0;
  pl.euler = o->morphology_type == 0;
  pl.vstride = pl.nvox;
  pl.p0 = 0, pl.p1 = 1 % pl.nz, pl.pn = pl.nz - 1;
  if (!pl.twod && (pl.nz == 128 || pl.nz == 256 || pl.nz == 512)) {
    // warp-FFT form: TX columns per block, with or without the morphology
    // tile staged through shared memory.  The candidates that fit are timed
    // on the first request of this shape (run_request) and the fastest kept.
    for (bool stage : {false, true})
      for (uint32_t t : {2u, 4u, 8u})
        if (zwarp_smem(pl.nz, pl.nvol, t, pl.nmat, stage) <= (stage ? 120 : 100) * 1024)
          pl.zcands.push_back({stage, t, 0.f});
    pl.zstage = false;
    pl.ztx = 4;
    for (const ZTune &c : pl.zcands)
      if (!c.stage && c.tx <= 4) pl.ztx = c.tx;
    pl.pruned = true;
    pl.zwarp = true;
    kept_planes(o, pl);
    pl.vstride = size_t(pl.kz) * pl.npix;
  } else if (!pl.twod && smooth7(pl.nz)) {
    // fused build + z FFT: lines per block so that two 512-thread blocks fit an SM
    uint32_t tx = 16;
    while (tx > 1 && (size_t(2) * pl.nvol * pl.nz * (tx + 1) + pl.nz) * sizeof(float2) > 104 * 1024) tx /= 2;
    if ((size_t(2) * pl.nvol * pl.nz * (tx + 1) + pl.nz) * sizeof(float2) <= kFftSmemBudget) {
      pl.pruned = true;
      pl.ztx = tx;
      kept_planes(o, pl);
      pl.vstride = size_t(pl.kz) * pl.npix;
    }
  }
  // material constants per energy, in double, scaled by 1/4pi (uniaxial.h:155-162)
  std::vector<MaterialConsts> mcs(pl.ne);
  std::vector<std::complex<double>> cA(size_t(pl.ne) * pl.nmat), cB(cA.size()), cC(cA.size()), cD(cA.size());
  const double s = 1.0 / (4.0 * kPi);
  for (uint32_t e = 0; e < pl.ne; ++e) {
    MaterialConsts &mc = mcs[e];
    std::memset(&mc, 0, sizeof mc);
    for (uint32_t m = 0; m < pl.nmat; ++m) {
      const float *op = optical + (size_t(e) * pl.nmat + m) * 4;
      const std::complex<double> dpar(-double(op[0]), double(op[1]));  // n_par - 1
      const std::complex<double> dper(-double(op[2]), double(op[3]));  // n_perp - 1
      const std::complex<double> A = dpar * (dpar + 2.0);              // n^2 - 1 = (n-1)(n+1)
      const std::complex<double> B = dper * (dper + 2.0);
      const std::complex<double> dm = (dpar + 2.0 * dper) / 3.0;       // mean n - 1
      const std::complex<double> C = dm * (dm + 2.0);
      const std::complex<double> D = A - B;
      mc.A[m] = make_float2(float(A.real() * s), float(A.imag() * s));
      mc.B[m] = make_float2(float(B.real() * s), float(B.imag() * s));
      mc.C[m] = make_float2(float(C.real() * s), float(C.imag() * s));
      mc.D[m] = make_float2(float(D.real() * s), float(D.imag() * s));
      const size_t em = size_t(e) * pl.nmat + m;
      cA[em] = A * s, cB[em] = B * s, cC[em] = C * s, cD[em] = D * s;
    }
  }
  pl.arena.clear();
  pl.off_mc = arena_put(pl.arena, mcs.data(), mcs.size());
  // angle coefficients [k][angle][nbasis]
  std::vector<float> coef(size_t(pl.nk) * pl.nang * pl.nbasis);
  for (size_t ka = 0; ka < size_t(pl.nk) * pl.nang; ++ka)
    for (uint32_t b = 0; b < pl.nbasis; ++b) coef[ka * pl.nbasis + b] = pl.material_frame ? 1.f : pl.evec[ka * 3 + b];
  pl.off_coef = arena_put(pl.arena, coef.data(), coef.size());
  // per-angle image rotation coefficients [k][angle] (src/cudaMain.cu:848-855)
  std::vector<WarpCoef> wc(size_t(pl.nk) * pl.nang);
  for (size_t ka = 0; ka < wc.size(); ++ka) {
    double c[2][3];
    rotation_coeffs(pl.eangles[ka], pl.nx, pl.ny, c);
    const WarpInverse w = warp_inverse(c);
    wc[ka] = WarpCoef{w.a00, w.a01, w.a02, w.a10, w.a11, w.a12};
  }
  pl.off_warp = arena_put(pl.arena, wc.data(), wc.size());
  // detector warps per k (src/cudaMain.cu:916-940)
  pl.detector_warp.resize(pl.nk);
  for (uint32_t k = 0; k < pl.nk; ++k) {
    double c[2][3];
    detector_coeffs(pl.detector, pl.frames[k].rk, pl.nx, pl.ny, c);
    const WarpInverse w = warp_inverse(c);
    pl.detector_warp[k] = WarpCoef{w.a00, w.a01, w.a02, w.a10, w.a11, w.a12};
  }
  // q-grid tables (include/uniaxial.h:645-650, :697-702): q_j = float(-pi/L + j * float(dq))
  const double L = double(o->phys_size);
  auto qtab = [&](uint32_t n) {
    std::vector<float> q(n, 0.f);
    if (n < 2) return q;
    const float dq = static_cast<float>((2 * kPi / L) / ((n - 1) * 1.0));
    for (uint32_t j = 0; j < n; ++j) q[j] = static_cast<float>((-kPi / L) + double(float(j) * dq));
    return q;
  };
  const std::vector<float> qx = qtab(pl.nx), qy = qtab(pl.ny), qz = qtab(pl.nz);
  pl.off_qx = arena_put(pl.arena, qx.data(), qx.size());
  pl.off_qy = arena_put(pl.arena, qy.data(), qy.size());
  pl.off_qz = arena_put(pl.arena, qz.data(), qz.size());
  // Hanning tables (src/cudaMain.cu:276-295), double cos rounded to float
  auto hann = [&](uint32_t n, bool unit) {
    std::vector<float> w(n);
    for (uint32_t j = 0; j < n; ++j) w[j] = unit ? 1.f : static_cast<float>(0.5 * (1 - std::cos(2 * kPi * j / n)));
    return w;
  };
  const std::vector<float> hx = hann(pl.nx, false), hy = hann(pl.ny, false), hz = hann(pl.nz, pl.twod);
  pl.off_hx = arena_put(pl.arena, hx.data(), hx.size());
  pl.off_hy = arena_put(pl.arena, hy.data(), hy.size());
  pl.off_hz = arena_put(pl.arena, hz.data(), hz.size());

  // FIELDS strategy: choose it, then its tables
  pl.npk = num_packed(pl.nmat);
  if (o->strategy == CYR_STRATEGY_AUTO) {
    // plane-volumes moved per request (read + write of the FFT passes, morphology reads)
    const double planes = pl.pruned ? pl.kz : pl.nz;
    const double spectra = pl.material_frame ? double(pl.nk) * pl.nang * 3.0 : double(pl.nvol);
    const double per_energy = double(pl.ne) * (spectra * planes + 2.0 * pl.nmat * pl.nz);
    const double once = (1.5 * pl.npk + 2.0 * pl.nmat) * pl.nz;
    pl.fields = once < per_energy;
  } else {
    pl.fields = o->strategy == CYR_STRATEGY_FIELDS;
  }
  {
    // energies per Ewald / rotation launch: up to 64, and 256 MB of Gram records
    // (LAB) or per-angle images (MATERIAL) per batch (fewer, larger launches;
    // the rotation's reads mostly hit L1, so L2 residency of a batch matters
    // little); batches of even size, each a whole number of records
    const uint32_t nep = gram_nep(pl), cap = std::min<uint32_t>(pl.ne, 64);
    uint32_t emax = 1;
    while (emax < cap && image_bytes(pl, emax + 1) <= (size_t(256) << 20)) ++emax;
    const uint32_t nbatches = (pl.ne + emax - 1) / emax;
    const uint32_t eb = (pl.ne + nbatches - 1) / nbatches;
    pl.ebatch = nbatches == 1 ? pl.ne : std::min(pl.ne, (eb + nep - 1) / nep * nep);
  }
  if (pl.fields) {
    pl.mom_zstep = std::max(1u, pl.nz / 16);  // 16 sampled planes
    // coef[e][v][j] = (alpha, beta): Nt_v(k) = sum_j alpha Z_j(k) + beta conj Z_j(-k), where
    // Z_j = F_2j + i F_2j+1 and field g = 7 m + f (f: u_x^2 u_y^2 u_z^2 u_xu_y u_xu_z u_yu_z phi_ui), T last
    const uint32_t nf = num_fields(pl.nmat), npk = pl.npk;
    std::vector<float4> fc(size_t(pl.ne) * 6 * npk);
    std::vector<std::complex<double>> c(size_t(6) * 2 * npk);
    for (uint32_t e = 0; e < pl.ne; ++e) {
      std::fill(c.begin(), c.end(), std::complex<double>(0.0, 0.0));
      auto at = [&](int v, uint32_t g) -> std::complex<double> & { return c[size_t(v) * 2 * npk + g]; };
      std::complex<double> R(0.0, 0.0);  // common part of the diagonal coefficients
      for (uint32_t m = 0; m < pl.nmat; ++m) R += cB[size_t(e) * pl.nmat + m] + cC[size_t(e) * pl.nmat + m];
      R /= double(2 * pl.nmat);
      for (uint32_t m = 0; m < pl.nmat; ++m) {
        const size_t em = size_t(e) * pl.nmat + m;
        const uint32_t g = kFieldsPerMaterial * m;
        const std::complex<double> B = cB[em] - R, C = cC[em] - R, DB = cD[em] + cB[em] - R;
        const int diag[3] = {0, 3, 5};  // xx yy zz
        for (int i = 0; i < 3; ++i) {
          for (int f = 0; f < 3; ++f) at(diag[i], g + f) = f == i ? DB : B;
          at(diag[i], g + 6) = C;
        }
        at(1, g + 3) = cD[em];  // xy
        at(2, g + 4) = cD[em];  // xz
        at(4, g + 5) = cD[em];  // yz
      }
      for (int i : {0, 3, 5}) at(i, nf - 1) = R;
      const std::complex<double> I(0.0, 1.0);
      for (int v = 0; v < 6; ++v)
        for (uint32_t j = 0; j < npk; ++j) {
          const std::complex<double> ca = at(v, 2 * j), cb = at(v, 2 * j + 1);
          const std::complex<double> al = 0.5 * (ca - I * cb), be = 0.5 * (ca + I * cb);
          fc[(size_t(e) * 6 + v) * npk + j] =
              make_float4(float(al.real()), float(al.imag()), float(be.real()), float(be.imag()));
        }
    }
    // the Ewald kernel may skip the structural zeros (coef_used) when every one of them is exactly zero
    pl.ewald_sparse = pl.nmat <= 4;
    for (uint32_t e = 0; e < pl.ne && pl.ewald_sparse; ++e)
      for (int v = 0; v < 6; ++v)
        for (uint32_t j = 0; j < npk; ++j) {
          const float4 q = fc[(size_t(e) * 6 + v) * npk + j];
          if (!coef_used(pl.nmat, v, j) && (q.x != 0.f || q.y != 0.f || q.z != 0.f || q.w != 0.f))
            pl.ewald_sparse = false;
        }
    pl.off_fcoef = arena_put(pl.arena, fc.data(), fc.size());
    std::vector<float> km(pl.ne);
    for (uint32_t e = 0; e < pl.ne; ++e) {
      const float wavelength = static_cast<float>(1239.84197 / o->energies[e]);  // src/cudaMain.cu:607-608
      km[e] = static_cast<float>(2 * kPi / wavelength);
    }
    pl.off_kmag = arena_put(pl.arena, km.data(), km.size());
    std::vector<float> kv(size_t(pl.nk) * 3);
    for (uint32_t k = 0; k < pl.nk; ++k)
      kv[3 * k] = pl.frames[k].k.x, kv[3 * k + 1] = pl.frames[k].k.y, kv[3 * k + 2] = pl.frames[k].k.z;
    pl.off_kvec = arena_put(pl.arena, kv.data(), kv.size());
    // per (k, angle): p_c = sum_v M[c][v] Nt_v.  LAB: p = Nt E.  MATERIAL: p = R^T Nt E.
    const uint32_t sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    std::vector<float> mat(size_t(pl.nk) * pl.nang * 18, 0.f);
    for (size_t ka = 0; ka < size_t(pl.nk) * pl.nang; ++ka) {
      double M[3][6] = {};
      const float *E = &pl.evec[ka * 3];
      for (int cc = 0; cc < 3; ++cc)
        for (int b = 0; b < 3; ++b) {
          if (pl.material_frame) {
            for (int i = 0; i < 3; ++i) M[cc][sym[i][b]] += double(pl.rmats[ka].m[i * 3 + cc]) * double(E[b]);
          } else {
            M[cc][sym[cc][b]] += double(E[b]);
          }
        }
      for (int cc = 0; cc < 3; ++cc)
        for (int v = 0; v < 6; ++v) mat[ka * 18 + cc * 6 + v] = float(M[cc][v]);
    }
    pl.off_mat = arena_put(pl.arena, mat.data(), mat.size());
  }
  ewald_rows(o, pl);
  pl.arena.resize((pl.arena.size() + 255) & ~size_t(255));
  return CYR_OK;
}

size_t request_bytes(const Plan &pl) {
  if (pl.fields) return field_bytes(pl) + pl.nmat * kMoments * sizeof(double) + 64 * sizeof(float2);
  return pl.nvol * pl.vstride * sizeof(float2) + (pl.euler ? pl.nvox * pl.nmat * sizeof(float4) : 0) + image_bytes(pl) + pl.npix * sizeof(float) +
         pl.arena.size() + 64 * sizeof(float2);
}

// Ewald-kernel parameters shared by every (energy, k).
EwaldParams ewald_params(const Plan &pl, const cyr_options *o, const unsigned char *dparams, const float2 *spec,
                         const float2 *dc, float *images) {
  EwaldParams p{};
  p.spec = spec;
  p.dc = dc;
  p.nx = pl.nx, p.ny = pl.ny, p.nz = pl.nz;
  p.nvox = pl.vstride;
  p.zshifted = pl.pruned ? 1u : 0u;
  p.zlo = pl.zlo;
  p.nplanes = pl.kz;
  p.nbasis = pl.nbasis;
  if (pl.material_frame) {
    for (int c = 0; c < 3; ++c) p.vol[c][0] = c;
  } else {
    // symmetric tensor entry (c, b) -> output volume; volumes hold xx xy xz yy yz [zz]
    const uint32_t sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int c = 0; c < 3; ++c)
      for (uint32_t b = 0; b < pl.nbasis; ++b) p.vol[c][b] = sym[c][b];
  }
  p.start = -static_cast<float>(kPi / o->phys_size);
  p.dx = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nx - 1) * 1.0));
  p.dy = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.ny - 1) * 1.0));
  p.dz = pl.twod ? 0.f : static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nz - 1) * 1.0));
  p.qx = reinterpret_cast<const float *>(dparams + pl.off_qx);
  p.qy = reinterpret_cast<const float *>(dparams + pl.off_qy);
  p.qz = reinterpret_cast<const float *>(dparams + pl.off_qz);
  p.interp = o->ewald_interpolation;
  p.twod = pl.twod ? 1u : 0u;
  p.images = images;
  return p;
}

// Slab upload of a host morphology (FIELDS strategy): events[s] completes when
// planes [s * planes, (s + 1) * planes) of every material are on the device.
// Slabs are issued one ahead of the compute that needs them: from pageable
// memory a copy call returns only once its data is staged, so the kernels of
// the previous slab must already be queued for the two to overlap.
struct SlabUpload {
  uint32_t planes = 0, count = 0, issued = 0;
  std::vector<cudaEvent_t> events;
  // events to use instead of creating them (the device context's, reused across calls): the
  // sample event first, then one per slab; grown here when short, never destroyed here
  std::vector<cudaEvent_t> *pool = nullptr;
  size_t pooled = 0;
  int next_event(cudaEvent_t *ev) {
    if (pool) {
      if (pooled == pool->size()) {
        cudaEvent_t e = nullptr;
        CYR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        pool->push_back(e);
      }
      *ev = (*pool)[pooled++];
      return CYR_OK;
    }
    CYR_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    return CYR_OK;
  }
  // every sample_zstep-th plane, copied first for the means (a sample spread over the volume)
  uint32_t sample_zstep = 1;
  cudaEvent_t sample = nullptr;
  const float *host = nullptr;
  float4 *dev = nullptr;
  uint32_t nmat = 0, nz = 0;
  size_t nvox = 0, npix = 0;
  cudaStream_t stream = nullptr;
  int issue(uint32_t s) {  // queues the copies of slabs up to s
    // planes the sample already brought (every sample_zstep-th, once it was issued) are not copied again
    auto sampled = [&](uint32_t z) { return sample != nullptr && z % sample_zstep == 0; };
    for (; issued <= s && issued < count; ++issued) {
      const uint32_t z0 = issued * planes, z1 = std::min(nz, z0 + planes);
      for (uint32_t a = z0; a < z1;) {
        if (sampled(a)) {
          ++a;
          continue;
        }
        uint32_t b = a + 1;
        while (b < z1 && !sampled(b)) ++b;
        for (uint32_t m = 0; m < nmat; ++m) {
          const size_t off = size_t(m) * nvox + size_t(a) * npix;  // float4 elements
          CYR_CUDA(cudaMemcpyAsync(dev + off, host + 4 * off, size_t(b - a) * npix * sizeof(float4),
                                   cudaMemcpyHostToDevice, stream));
        }
        a = b;
      }
      cudaEvent_t ev = nullptr;
      CYR_TRY(next_event(&ev));
      events.push_back(ev);
      CYR_CUDA(cudaEventRecord(ev, stream));
    }
    return CYR_OK;
  }
  int issue_sample() {
    const size_t pitch = size_t(sample_zstep) * npix * sizeof(float4);
    for (uint32_t m = 0; m < nmat; ++m)
      CYR_CUDA(cudaMemcpy2DAsync(dev + size_t(m) * nvox, pitch, host + 4 * size_t(m) * nvox, pitch,
                                 npix * sizeof(float4), (nz + sample_zstep - 1) / sample_zstep,
                                 cudaMemcpyHostToDevice, stream));
    CYR_TRY(next_event(&sample));
    CYR_CUDA(cudaEventRecord(sample, stream));
    return CYR_OK;
  }
  ~SlabUpload() {
    if (pool) return;
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    if (sample) cudaEventDestroy(sample);
  }
};

// Fields of planes [z0, z1) and their x pass: fused (k_build_fields_rows) or
// the separate build and row pass.
int build_fields_x(DeviceContext &ctx, Scratch &sc, const cyr_options *o, const Plan &pl, FieldParams fp, uint32_t z0,
                   uint32_t z1, bool fused, const float2 *twx, cudaStream_t st) {
  const uint32_t npk = pl.npk;
  float2 *spec = sc.spec.as<float2>();
  int sms = 0;
  CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  fp.i0 = size_t(z0) * pl.npix, fp.i1 = size_t(z1) * pl.npix;
  if (fused) {
    const size_t smem = fields_rows_smem(pl.nx, npk, pl.nmat);
    const uint32_t rows = (z1 - z0) * pl.ny;
    int per_sm = 1;
    auto launch = [&](auto kern) -> int {
      CYR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
      const unsigned grid = unsigned(std::min<size_t>(rows, size_t(std::max(1, per_sm)) * sms));
      kern<<<grid, 256, smem, st>>>(fp, twx, npk);
      return CYR_OK;
    };
    const int slot = ctx.prof.begin(kBuildFieldsRows, st);
    const bool euler = o->morphology_type == 0;
    if (pl.nx == 128) CYR_TRY(launch(euler ? k_build_fields_rows<0, 4> : k_build_fields_rows<1, 4>));
    if (pl.nx == 256) CYR_TRY(launch(euler ? k_build_fields_rows<0, 8> : k_build_fields_rows<1, 8>));
    if (pl.nx == 512) CYR_TRY(launch(euler ? k_build_fields_rows<0, 16> : k_build_fields_rows<1, 16>));
    if (pl.nx == 1024) CYR_TRY(launch(euler ? k_build_fields_rows<0, 32> : k_build_fields_rows<1, 32>));
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
    return CYR_OK;
  }
  const uint32_t blocks = uint32_t(std::min<size_t>((fp.i1 - fp.i0 + 255) / 256, size_t(sms) * 8));
  const int slot = ctx.prof.begin(kBuildFields, st);
  if (o->morphology_type == 0)
    k_build_fields<0><<<blocks, 256, 0, st>>>(fp);
  else
    k_build_fields<1><<<blocks, 256, 0, st>>>(fp);
  ctx.prof.end(slot, st);
  CYR_CUDA(cudaGetLastError());
  return fft_axes(ctx, spec + fp.i0, pl.nx, pl.ny, z1 - z0, npk, st, 0, 0, pl.nvox, &sc.blue);
}

// Autotuning of the FIELDS transform for one shape (the first device-resident
// request of it on this device): the fused or separate build + x pass and the
// launch form of the y and z passes are each timed once on the packed-field
// buffer, before the build overwrites every element of it, and the fastest
// kept.  Every candidate computes the same numbers.
// Ewald geometry of a FIELDS request (k_ewald_fields); kmag, kx, ky, kz are set per energy and k.
EwaldGeom field_geometry(const cyr_options *o, const Plan &pl) {
  EwaldGeom g{};
  g.start = -static_cast<float>(kPi / o->phys_size);
  g.dx = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nx - 1) * 1.0));
  g.dy = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.ny - 1) * 1.0));
  g.dz = pl.twod ? 0.f : static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nz - 1) * 1.0));
  g.nx = pl.nx, g.ny = pl.ny, g.nz = pl.nz;
  g.interp = o->ewald_interpolation;
  g.twod = pl.twod ? 1u : 0u;
  return g;
}

// Store mask of the FIELDS z pass (k_zmask over the ne energies at d_kmag and
// the nk k vectors at d_kv) in sc.zmask; *out stays null, so every plane is
// stored, when no z-pass form of this shape takes a mask or masks are off.
int field_zmask(DeviceContext &ctx, Scratch &sc, const EwaldGeom &g, const float *d_kmag, uint32_t ne,
                const float *d_kv, uint32_t nk, cudaStream_t st, const uint32_t **out) {
  *out = nullptr;
  if (!ctx.zmask || g.twod || !(g.nz == 128 || g.nz == 256 || g.nz == 512) || g.nx % kTmaCols != 0 ||
      !ctx.encode_tiled || !ctx.tma_error)
    return CYR_OK;
  const uint32_t mw = (g.nz / 8 + 31) / 32;
  const size_t bytes = size_t(g.ny) * (g.nx / kTmaCols) * mw * sizeof(uint32_t);
  CYR_TRY(sc.zmask.ensure(bytes));
  CYR_CUDA(cudaMemsetAsync(sc.zmask.ptr, 0, bytes, st));
  ZMaskParams zp{};
  zp.g = g;
  zp.kmag = d_kmag, zp.ne = ne;
  zp.kv = d_kv, zp.nk = nk;
  zp.mwords = mw;
  zp.mask = sc.zmask.as<uint32_t>();
  const int slot = ctx.prof.begin(kZMask, st);
  k_zmask<<<unsigned((size_t(g.nx) * g.ny + 255) / 256), 256, 0, st>>>(zp);
  ctx.prof.end(slot, st);
  CYR_CUDA(cudaGetLastError());
  *out = zp.mask;
  return CYR_OK;
}

int tune_fields(DeviceContext &ctx, Scratch &sc, const cyr_options *o, const Plan &pl, const FieldParams &fp,
                bool fused_ok, const float2 *twx, cudaStream_t st, DeviceContext::FieldTune &ft,
                const uint32_t *zmask) {
  struct Cand {
    int kind;  // 0 build + x, 1 y pass, 2 z pass
    uint32_t choice;
    cudaEvent_t a, b;
  };
  std::vector<Cand> cands;
  if (fused_ok) cands.push_back({0, 1, nullptr, nullptr}), cands.push_back({0, 0, nullptr, nullptr});
  const uint32_t dims[3] = {pl.nx, pl.ny, pl.nz};
  for (int axis = 1; axis <= 2; ++axis) {
    const std::vector<uint32_t> f = column_forms(ctx, dims[axis], pl.nx);
    if (f.size() > 1)
      for (uint32_t v : f) cands.push_back({axis, v, nullptr, nullptr});
  }
  ft.fused = fused_ok;
  if (cands.empty()) return CYR_OK;
  for (Cand &c : cands) {
    CYR_CUDA(cudaEventCreate(&c.a));
    CYR_CUDA(cudaEventCreate(&c.b));
  }
  int rc = CYR_OK;
  for (Cand &c : cands) {
    CYR_CUDA(cudaEventRecord(c.a, st));
    if (c.kind == 0)
      rc = build_fields_x(ctx, sc, o, pl, fp, 0, pl.nz, c.choice == 1, twx, st);
    else
      rc = warp_fft_pass(ctx, sc.spec.as<float2>(), pl.nx, pl.ny, pl.nz, pl.npk, c.kind, st, pl.nvox, c.choice,
                         c.kind == 2 ? zmask : nullptr);
    if (rc != CYR_OK) break;
    CYR_CUDA(cudaEventRecord(c.b, st));
  }
  if (rc == CYR_OK) {
    CYR_CUDA(cudaEventSynchronize(cands.back().b));
    float best[3] = {1e30f, 1e30f, 1e30f};
    std::string rep[3];
    for (Cand &c : cands) {
      float ms = 0.f;
      CYR_CUDA(cudaEventElapsedTime(&ms, c.a, c.b));
      char buf[64];
      std::snprintf(buf, sizeof buf, " %s %.3f ms",
                    c.kind == 0 ? (c.choice ? "fused" : "separate") : form_name(c.choice), ms);
      rep[c.kind] += buf;
      if (ms < best[c.kind]) {
        best[c.kind] = ms;
        if (c.kind == 0)
          ft.fused = c.choice == 1;
        else
          ft.form[c.kind] = c.choice;
      }
    }
    ft.report = "build+x:" + (rep[0].empty() ? std::string(" -") : rep[0]) + "; y:" +
                (rep[1].empty() ? std::string(" -") : rep[1]) + "; z:" + (rep[2].empty() ? std::string(" -") : rep[2]);
  }
  for (Cand &c : cands) cudaEventDestroy(c.a), cudaEventDestroy(c.b);
  return rc;
}

// FIELDS strategy after the moments: field means, packed field spectra, then
// every energy (in batches) and k from them.
int run_fields(DeviceContext &ctx, Scratch &sc, const cyr_options *o, const Plan &pl, const unsigned char *dp,
               const float4 *d_vox, float *d_out, cudaStream_t st, size_t nsamp, const SlabUpload *up,
               bool capturing) {
  const uint32_t npk = pl.npk;
  CYR_TRY(sc.spec.ensure(size_t(npk) * pl.nvox * sizeof(float2)));
  CYR_TRY(sc.images.ensure(image_bytes(pl, pl.ebatch)));
  CYR_TRY(sc.avg.ensure(size_t(pl.ebatch) * pl.npix * sizeof(float)));
  float2 *spec = sc.spec.as<float2>();
  FieldParams fp{};
  fp.vox = d_vox;
  fp.nx = pl.nx, fp.ny = pl.ny, fp.nz = pl.nz, fp.nmat = pl.nmat;
  fp.nvox = pl.nvox;
  fp.mom = sc.moments.as<double>();  // each block forms the field means from the moments
  fp.nsamp = nsamp;
  if (pl.hanning) {
    fp.hann_x = reinterpret_cast<const float *>(dp + pl.off_hx);
    fp.hann_y = reinterpret_cast<const float *>(dp + pl.off_hy);
    fp.hann_z = reinterpret_cast<const float *>(dp + pl.off_hz);
  }
  fp.out = spec;
  // the planes the Ewald projection reads: the z pass stores only those
  const EwaldGeom geom = field_geometry(o, pl);
  const uint32_t *zmask = nullptr;
  CYR_TRY(field_zmask(ctx, sc, geom, reinterpret_cast<const float *>(dp + pl.off_kmag), pl.ne,
                      reinterpret_cast<const float *>(dp + pl.off_kvec), pl.nk, st, &zmask));
  // the field build fused with the x pass when x is a warp-FFT length and the row's lines fit
  const bool fused_ok = (pl.nx == 128 || pl.nx == 256 || pl.nx == 512 || pl.nx == 1024) &&
                        fields_rows_smem(pl.nx, npk, pl.nmat) <= kFftSmemBudget;
  const float2 *twx = nullptr;
  if (fused_ok) CYR_TRY(get_twiddles(ctx, pl.nx, &twx));
  // tuned launch forms of this shape, tuned here on its first device-resident request
  char key[96];
  std::snprintf(key, sizeof key, "%u,%u,%u,%u", pl.nx, pl.ny, pl.nz, npk);
  DeviceContext::FieldTune ft;
  bool have = false;
  {
    std::lock_guard<std::mutex> lk(ctx.tables_mu);
    auto it = ctx.ftune.find(key);
    if (it != ctx.ftune.end()) ft = it->second, have = true;
  }
  if (!have) {
    ft.fused = fused_ok;
    if (ctx.autotune && !up && !capturing && !ctx.prof.active) {
      CYR_TRY(tune_fields(ctx, sc, o, pl, fp, fused_ok, twx, st, ft, zmask));
      std::lock_guard<std::mutex> lk(ctx.tables_mu);
      ctx.ftune[key] = ft;
    }
  }
  const bool fused = fused_ok && ft.fused;
  // fields of planes [z0, z1), then their x and y passes (the axes commute; z comes last)
  const uint32_t step = up ? up->planes : pl.nz, nslab = up ? up->count : 1;
  for (uint32_t sl = 0; sl < nslab; ++sl) {
    const uint32_t z0 = sl * step, z1 = std::min(pl.nz, z0 + step);
    if (up) {
      CYR_TRY(const_cast<SlabUpload *>(up)->issue(sl));
      CYR_CUDA(cudaStreamWaitEvent(st, up->events[sl], 0));
    }
    CYR_TRY(build_fields_x(ctx, sc, o, pl, fp, z0, z1, fused, twx, st));
    CYR_TRY(fft_axes(ctx, spec + size_t(z0) * pl.npix, pl.nx, pl.ny, z1 - z0, npk, st, 1, 1, pl.nvox, &sc.blue,
                     ft.form));
    if (up) CYR_TRY(const_cast<SlabUpload *>(up)->issue(sl + 1));  // the next slab's copy, behind this slab's kernels
  }
  CYR_TRY(fft_axes(ctx, spec, pl.nx, pl.ny, pl.nz, npk, st, 2, 2, 0, &sc.blue, ft.form, zmask));
  // bin 0 of each packed volume replaced by the mean of its neighbours
  CYR_TRY(sc.dc.ensure(size_t(kMaxPacked) * sizeof(float2)));
  int slot = ctx.prof.begin(kDc, st);
  k_dc<<<1, (npk + 31) / 32 * 32, 0, st>>>(spec, npk, pl.nvox, pl.nx, pl.ny, pl.nz, 0, 1 % pl.nz, pl.nz - 1,
                                           sc.dc.as<float2>());
  ctx.prof.end(slot, st);
  CYR_CUDA(cudaGetLastError());

  FieldEwaldParams fe{};
  fe.zspec = spec;
  fe.zdc = sc.dc.as<float2>();
  fe.npk = npk;
  fe.nvox = pl.nvox;
  fe.coef = reinterpret_cast<const float4 *>(dp + pl.off_fcoef);
  fe.kmag = reinterpret_cast<const float *>(dp + pl.off_kmag);
  fe.g = geom;
  fe.qx = reinterpret_cast<const float *>(dp + pl.off_qx);
  fe.qy = reinterpret_cast<const float *>(dp + pl.off_qy);
  fe.qz = reinterpret_cast<const float *>(dp + pl.off_qz);
  fe.nangles = pl.nang;
  fe.images = sc.images.as<float>();
  fe.gram = sc.images.as<float4>();
  fe.gplane = gram_plane_size(int(pl.ny), int(pl.nx));
  const size_t fsmem = size_t(kEwaldEnergies) * 6 * npk * sizeof(float4);
  const unsigned pix_blocks = unsigned((pl.npix + 255) / 256);
  const unsigned fpix_blocks = unsigned((pl.npix + 31) / 32);  // k_ewald_fields: 32 pixels per block
  const int W = int(pl.ny), H = int(pl.nx);  // the reference hands NPP width = Ny, height = Nx
  const unsigned rot_tiles = unsigned(((W + kRotTile - 1) / kRotTile) * ((H + kRotTile - 1) / kRotTile));
  const WarpCoef *dwarp = reinterpret_cast<const WarpCoef *>(dp + pl.off_warp);
  const float *dmat = reinterpret_cast<const float *>(dp + pl.off_mat);
  const float fillv = o->rot_mask ? 0.f : std::numeric_limits<float>::quiet_NaN();
  const size_t ostride = size_t(pl.nk) * pl.npix;
  for (uint32_t k = 0; k < pl.nk; ++k) {
    const KFrame &f = pl.frames[k];
    fe.kvx = f.k.x, fe.kvy = f.k.y, fe.kvz = f.k.z;
    fe.mat = dmat + size_t(k) * pl.nang * 18;
    fe.ecoef = reinterpret_cast<const float *>(dp + pl.off_coef) + size_t(k) * pl.nang * pl.nbasis;
    RotateParams rp{};
    rp.images = sc.images.as<float>();
    rp.coef = dwarp + size_t(k) * pl.nang;
    rp.W = W, rp.H = H;
    rp.nangles = pl.nang;
    rp.rot_mask = o->rot_mask;
    rp.avg = sc.avg.as<float>();
    RotateGramParams rg{};
    rg.gram = sc.images.as<float4>();
    rg.plane = fe.gplane;
    rg.coef = rp.coef;
    rg.ecoef = fe.ecoef;
    rg.W = W, rg.H = H;
    rg.nangles = pl.nang;
    rg.rot_mask = o->rot_mask;
    rg.avg = rp.avg;
    const uint32_t nep = gram_nep(pl);
    const size_t rsm = pl.has_rows ? size_t(H) * sizeof(int2) : 0;
    for (uint32_t e0 = 0; e0 < pl.ne; e0 += pl.ebatch) {
      const uint32_t nb = std::min(pl.ebatch, pl.ne - e0);
      fe.e0 = e0;
      fe.nbatch = nb;
      rg.nenergies = nb;
      rg.rows = pl.has_rows ? reinterpret_cast<const int2 *>(dp + pl.off_rows) + (size_t(k) * pl.ne + e0) * H : nullptr;
      const dim3 rgrid(rot_tiles, (nb + nep - 1) / nep);
      slot = ctx.prof.begin(kEwaldFields, st);
      const unsigned fgrid = fpix_blocks * ((nb + kEwaldEnergies - 1) / kEwaldEnergies);
      const bool sparse = pl.ewald_sparse && ctx.sparse_ewald;
      if (pl.material_frame)
        k_ewald_fields<0><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      else if (pl.nbasis == 2 && sparse && pl.nmat == 1)
        k_ewald_fields<2, false, 1><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      else if (pl.nbasis == 2 && sparse && pl.nmat == 2)
        k_ewald_fields<2, false, 2><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      else if (pl.nbasis == 2 && sparse && pl.nmat == 3)
        k_ewald_fields<2, false, 3><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      else if (pl.nbasis == 2 && sparse && pl.nmat == 4)
        k_ewald_fields<2, false, 4><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      else if (pl.nbasis == 2)
        k_ewald_fields<2><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      else
        k_ewald_fields<3><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
      ctx.prof.end(slot, st);
      slot = ctx.prof.begin(pl.material_frame ? kRotate : kRotateGram, st);
      if (pl.material_frame)
        k_rotate_average<<<dim3(pix_blocks, nb), 256, 0, st>>>(rp);
      else if (pl.nbasis == 2)
        k_rotate_gram<2, packed_energies<2>()><<<rgrid, kRotTile * kRotTile, rsm, st>>>(rg);
      else
        k_rotate_gram<3, packed_energies<3>()><<<rgrid, kRotTile * kRotTile, rsm, st>>>(rg);
      ctx.prof.end(slot, st);
      float *dst = d_out + (size_t(e0) * pl.nk + k) * pl.npix;
      slot = ctx.prof.begin(kFill, st);
      k_fill<<<dim3(pix_blocks, nb), 256, 0, st>>>(dst, pl.npix, fillv, ostride);
      ctx.prof.end(slot, st);
      slot = ctx.prof.begin(kWarp, st);
      k_warp<<<dim3(pix_blocks, nb), 256, 0, st>>>(sc.avg.as<float>(), dst, W, H, pl.detector_warp[k], pl.npix,
                                                   ostride);
      ctx.prof.end(slot, st);
      CYR_CUDA(cudaGetLastError());
    }
  }
  return CYR_OK;
}

// How a request is enqueued.  host_arena: pinned copy of the parameter arena
// that outlives the call (required while capturing a graph: the upload node
// reads it at every replay); capturing: no host synchronisation, no device
// queries and no autotuning (a warm request of the same shape ran before).
struct RunMode {
  unsigned char *host_arena = nullptr;
  size_t host_arena_bytes = 0;
  bool capturing = false;
  const Plan *plan = nullptr;  // made by the caller for these options (strategy resolved), or null
  // host morphology to upload into d_vox first: with the FIELDS strategy in
  // z slabs on copy_stream, each slab's fields built and x/y-transformed as
  // soon as it lands, so the upload hides most of the transform
  const float *host_vox = nullptr;
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> *event_pool = nullptr;  // reused slab events, or null: made per call
};


int run_request(DeviceContext &ctx, Scratch &sc, const cyr_options *o, const float *optical, const float4 *d_vox,
                float *d_out, cudaStream_t st, const RunMode &mode = RunMode()) {
  Plan local;
  if (!mode.plan) CYR_TRY(make_plan(o, optical, local));
  Plan &pl = mode.plan ? const_cast<Plan &>(*mode.plan) : local;
  CYR_TRY(setup_attrs(ctx));
  CYR_TRY(sc.init());
  if (!mode.plan && pl.fields && o->strategy == CYR_STRATEGY_AUTO && !mode.capturing) {
    // AUTO falls back to the per-energy spectra when the field volumes do not fit
    size_t free_b = 0, total_b = 0;
    CYR_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t reusable = sc.spec.bytes + sc.images.bytes + sc.avg.bytes;
    if (field_bytes(pl) + (size_t(1) << 30) > free_b + reusable) pl.fields = false;
  }
  // scratch (grow-only); wait for the previous user of the scratch
  if (!mode.capturing) CYR_CUDA(cudaStreamWaitEvent(st, sc.last_use, 0));
  CYR_TRY(sc.errors.ensure(sizeof(unsigned)));
  CYR_CUDA(cudaMemsetAsync(sc.errors.ptr, 0, sizeof(unsigned), st));
  if (!pl.fields) {
    CYR_TRY(sc.spec.ensure(pl.nvol * pl.vstride * sizeof(float2)));
    CYR_TRY(sc.images.ensure(image_bytes(pl)));
    CYR_TRY(sc.avg.ensure(pl.npix * sizeof(float)));
    CYR_TRY(sc.dc.ensure(8 * sizeof(float2)));
  }
  CYR_TRY(sc.params.ensure(pl.arena.size()));
  if (mode.host_arena) {
    if (pl.arena.size() > mode.host_arena_bytes) return fail(CYR_ERR_ARGUMENT, "parameter arena exceeds its host buffer");
    std::memcpy(mode.host_arena, pl.arena.data(), pl.arena.size());
    CYR_CUDA(cudaMemcpyAsync(sc.params.ptr, mode.host_arena, pl.arena.size(), cudaMemcpyHostToDevice, st));
  } else {
    CYR_CUDA(cudaMemcpyAsync(sc.params.ptr, pl.arena.data(), pl.arena.size(), cudaMemcpyHostToDevice, st));
  }
  const unsigned char *dp = sc.params.as<unsigned char>();
  // host morphology: uploaded in z slabs (FIELDS) or at once (per-energy spectra)
  SlabUpload upload;
  if (mode.host_vox) {
    upload.pool = mode.event_pool;
    upload.stream = mode.copy_stream ? mode.copy_stream : st;
    if (upload.stream != st) CYR_CUDA(cudaStreamWaitEvent(upload.stream, sc.last_use, 0));
    upload.host = mode.host_vox;
    upload.dev = const_cast<float4 *>(d_vox);
    upload.nmat = pl.nmat, upload.nz = pl.nz, upload.nvox = pl.nvox, upload.npix = pl.npix;
    // slabs: after the last one lands, its fields and x/y passes are still ahead
    // of the z pass, so thinner slabs shorten that tail
    upload.count = !pl.fields ? 1u : pl.nz >= 64 ? 16u : pl.nz >= 8 ? 8u : 1u;
    upload.planes = (pl.nz + upload.count - 1) / upload.count;
    upload.count = (pl.nz + upload.planes - 1) / upload.planes;
    if (pl.fields) {
      upload.sample_zstep = std::max(1u, pl.nz / 8);
      CYR_TRY(upload.issue_sample());
      CYR_TRY(upload.issue(0));
    } else {
      CYR_TRY(upload.issue(upload.count - 1));
      CYR_CUDA(cudaStreamWaitEvent(st, upload.events.back(), 0));
    }
  }
  const bool slabs = mode.host_vox && pl.fields;
  // volume moments of the morphology -> mean of every tensor entry, per energy
  CYR_TRY(sc.moments.ensure(size_t(pl.nmat) * kMoments * sizeof(double)));
  CYR_TRY(sc.means.ensure(size_t(pl.ne) * 6 * sizeof(float2)));
  CYR_CUDA(cudaMemsetAsync(sc.moments.ptr, 0, size_t(pl.nmat) * kMoments * sizeof(double), st));
  // Euler morphologies are converted once per request to the trigonometry-free vector form
  const bool convert = o->morphology_type == 0 && !pl.fields;
  CYR_TRY(sc.flags.ensure(sizeof(unsigned)));
  CYR_CUDA(cudaMemsetAsync(sc.flags.ptr, 0, sizeof(unsigned), st));
  if (convert) CYR_TRY(sc.conv.ensure(pl.nvox * pl.nmat * sizeof(float4)));
  {
    MomentParams mp{};
    mp.vox = d_vox;
    mp.nx = pl.nx, mp.ny = pl.ny, mp.nz = pl.nz, mp.nmat = pl.nmat;
    mp.nvox = pl.nvox;
    if (pl.hanning) {
      mp.hann_x = reinterpret_cast<const float *>(dp + pl.off_hx);
      mp.hann_y = reinterpret_cast<const float *>(dp + pl.off_hy);
      mp.hann_z = reinterpret_cast<const float *>(dp + pl.off_hz);
    }
    mp.out = sc.moments.as<double>();
    mp.conv = convert ? sc.conv.as<float4>() : nullptr;
    // the conversion needs every voxel; the means alone need only a subsample of planes
    // (with a slab upload: the planes copied first for that purpose)
    mp.zstep = convert ? 1u : pl.mom_zstep;
    if (slabs) {
      mp.zstep = upload.sample_zstep;
      CYR_CUDA(cudaStreamWaitEvent(st, upload.sample, 0));
    }
    mp.neg = sc.flags.as<unsigned>();
    int nsm = 0;
    CYR_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx.device));
    // about 8 samples per thread: small volumes get few blocks (each block ends in
    // kMoments double atomics on the same addresses), large ones 4 per SM
    const size_t nsamp = pl.npix * ((pl.nz + mp.zstep - 1) / mp.zstep);
    const dim3 grid(uint32_t(std::max<size_t>(1, std::min<size_t>((nsamp + 2047) / 2048, size_t(nsm) * 4))), pl.nmat);
    int slot = ctx.prof.begin(kMom, st);
    if (o->morphology_type == 0)
      k_moments<0><<<grid, 256, 0, st>>>(mp);
    else
      k_moments<1><<<grid, 256, 0, st>>>(mp);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
    if (pl.fields) {
      const size_t nsamp = pl.npix * ((mp.nz + mp.zstep - 1) / mp.zstep);
      CYR_TRY(run_fields(ctx, sc, o, pl, dp, d_vox, d_out, st, nsamp, slabs ? &upload : nullptr, mode.capturing));
      // an event recorded inside a capture cannot be waited on outside it (slots keep order by their stream)
      if (!mode.capturing) CYR_CUDA(cudaEventRecord(sc.last_use, st));
      return CYR_OK;
    }
    slot = ctx.prof.begin(kMeans, st);
    k_entry_means<<<1, 64, 0, st>>>(sc.moments.as<double>(), pl.nmat, pl.nvox,
                                    reinterpret_cast<const MaterialConsts *>(dp + pl.off_mc), pl.ne,
                                    sc.means.as<float2>());
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  }
  float2 *spec = sc.spec.as<float2>();
  float2 *dc = sc.dc.as<float2>();
  float *images = sc.images.as<float>();
  float *avg = sc.avg.as<float>();
  const MaterialConsts *dmc = reinterpret_cast<const MaterialConsts *>(dp + pl.off_mc);

  BuildParams bp{};
  bp.vox = d_vox;
  bp.nx = pl.nx, bp.ny = pl.ny, bp.nz = pl.nz, bp.nmat = pl.nmat;
  bp.nvox = pl.nvox;
  bp.morphology = o->morphology_type;
  bp.out = spec;
  bp.conv = convert ? sc.conv.as<float4>() : nullptr;
  bp.neg = sc.flags.as<unsigned>();
  if (pl.hanning) {
    bp.hann_x = reinterpret_cast<const float *>(dp + pl.off_hx);
    bp.hann_y = reinterpret_cast<const float *>(dp + pl.off_hy);
    bp.hann_z = reinterpret_cast<const float *>(dp + pl.off_hz);
  }
  int sms = 0;
  CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  const uint32_t build_blocks = uint32_t(std::min<size_t>((pl.nvox + 255) / 256, size_t(sms) * 8));
  EwaldParams ep = ewald_params(pl, o, dp, spec, dc, images);
  ep.errors = sc.errors.as<unsigned>();
  FftAxis az{};
  if (pl.pruned) CYR_TRY(make_axis(ctx, pl.nz, az));
  // spectra of the current BuildParams (nvol volumes): pruned (build + z FFT
  // fused, then x and y on the kept planes) or full (build, then 3 passes)
  auto spectra = [&](const MaterialConsts *mce) -> int {
    int slot;
    if (pl.pruned) {
      BuildZParams zp{};
      zp.b = bp;
      zp.az = az;
      zp.tx = pl.ztx;
      zp.zlo = pl.zlo;
      zp.kz = pl.kz;
      zp.out = spec;
      if (pl.zwarp) {
        auto launch_warp = [&](const ZTune &cfg) {
          zp.stage = cfg.stage ? 1u : 0u;
          zp.tx = cfg.tx;
          const dim3 g((pl.nx + cfg.tx - 1) / cfg.tx * pl.ny);
          const size_t smem = zwarp_smem(pl.nz, bp.nvol, cfg.tx, pl.nmat, cfg.stage);
#define CYR_LAUNCH_WARP_ZT(V, T)                                                   \
  if (o->morphology_type == 0) {                                                   \
    k_build_fft_z_warp<0, true, V, T><<<g, 256, smem, st>>>(zp, mce);              \
    k_build_fft_z_warp<0, false, V, T><<<g, 256, smem, st>>>(zp, mce);             \
  } else {                                                                         \
    k_build_fft_z_warp<1, false, V, T><<<g, 256, smem, st>>>(zp, mce);             \
  }
#define CYR_LAUNCH_WARP_Z(V)         \
  if (cfg.tx == 2) {                 \
    CYR_LAUNCH_WARP_ZT(V, 2)         \
  } else if (cfg.tx == 4) {          \
    CYR_LAUNCH_WARP_ZT(V, 4)         \
  } else {                           \
    CYR_LAUNCH_WARP_ZT(V, 8)         \
  }
          if (pl.nz == 128) {
            CYR_LAUNCH_WARP_Z(4)
          } else if (pl.nz == 256) {
            CYR_LAUNCH_WARP_Z(8)
          } else {
            CYR_LAUNCH_WARP_Z(16)
          }
#undef CYR_LAUNCH_WARP_Z
#undef CYR_LAUNCH_WARP_ZT
        };
        char key[96];
        std::snprintf(key, sizeof key, "%u,%u,%u,%u,%u,%u", pl.nx, pl.ny, pl.nz, pl.nmat, bp.nvol,
                      o->morphology_type);
        ZTune tuned;
        bool have_tuned;
        {
          std::lock_guard<std::mutex> lk(ctx.tables_mu);
          auto it = ctx.ztune.find(key);
          have_tuned = it != ctx.ztune.end();
          if (have_tuned) tuned = it->second;
        }
        if (!have_tuned && pl.zcands.size() > 1 && !ctx.prof.active && !mode.capturing) {
          // autotune: time every candidate once on this energy; the last one's
          // output stays in `spec` and is used
          std::vector<cudaEvent_t> ev(2 * pl.zcands.size());
          for (auto &e : ev) CYR_CUDA(cudaEventCreate(&e));
          for (size_t c = 0; c < pl.zcands.size(); ++c) {
            CYR_CUDA(cudaEventRecord(ev[2 * c], st));
            launch_warp(pl.zcands[c]);
            CYR_CUDA(cudaEventRecord(ev[2 * c + 1], st));
          }
          CYR_CUDA(cudaGetLastError());
          CYR_CUDA(cudaEventSynchronize(ev.back()));
          ZTune best = pl.zcands[0];
          best.ms = 1e30f;
          for (size_t c = 0; c < pl.zcands.size(); ++c) {
            float ms = 0.f;
            CYR_CUDA(cudaEventElapsedTime(&ms, ev[2 * c], ev[2 * c + 1]));
            if (ms < best.ms) best = pl.zcands[c], best.ms = ms;
          }
          for (auto &e : ev) cudaEventDestroy(e);
          {
            std::lock_guard<std::mutex> lk(ctx.tables_mu);
            ctx.ztune[key] = best;
          }
          launch_warp(best);  // the kept output must come from a full, ordered launch of the chosen form
        } else {
          ZTune cfg;
          if (have_tuned) {
            cfg = tuned;
          } else {
            cfg.stage = pl.zstage;
            cfg.tx = pl.ztx;
          }
          slot = ctx.prof.begin(kBuildZ, st, o->morphology_type == 0 ? 2 : 1);
          launch_warp(cfg);
          ctx.prof.end(slot, st);
        }
      } else {
        const dim3 grid((pl.nx + pl.ztx - 1) / pl.ztx * pl.ny);
        slot = ctx.prof.begin(kBuildZ, st, o->morphology_type == 0 ? 2 : 1);
        const size_t smem = (size_t(2) * bp.nvol * pl.nz * (pl.ztx + 1) + pl.nz) * sizeof(float2);
        if (o->morphology_type == 0) {
          k_build_fft_z<0, true><<<grid, kFftThreads, smem, st>>>(zp, mce);
          k_build_fft_z<0, false><<<grid, kFftThreads, smem, st>>>(zp, mce);
        } else {
          k_build_fft_z<1, false><<<grid, kFftThreads, smem, st>>>(zp, mce);
        }
        ctx.prof.end(slot, st);
      }
      CYR_CUDA(cudaGetLastError());
      CYR_TRY(fft3d(ctx, spec, pl.nx, pl.ny, pl.kz, bp.nvol, st, true, &sc.blue));
    } else {
      slot = ctx.prof.begin(kBuild, st, o->morphology_type == 0 ? 2 : 1);
      if (o->morphology_type == 0) {
        k_build<0, true><<<build_blocks, 256, 0, st>>>(bp, mce);
        k_build<0, false><<<build_blocks, 256, 0, st>>>(bp, mce);
      } else {
        k_build<1, false><<<build_blocks, 256, 0, st>>>(bp, mce);
      }
      ctx.prof.end(slot, st);
      CYR_CUDA(cudaGetLastError());
      CYR_TRY(fft3d(ctx, spec, pl.nx, pl.ny, pl.nz, bp.nvol, st, false, &sc.blue));
    }
    slot = ctx.prof.begin(kDc, st);
    k_dc<<<1, 32, 0, st>>>(spec, bp.nvol, pl.vstride, pl.nx, pl.ny, pl.nz, pl.p0, pl.p1, pl.pn, dc);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
    return CYR_OK;
  };
  const unsigned pix_blocks = unsigned((pl.npix + 255) / 256);
  const int W = int(pl.ny), H = int(pl.nx);  // the reference hands NPP width = Ny, height = Nx
  const unsigned rot_tiles = unsigned(((W + kRotTile - 1) / kRotTile) * ((H + kRotTile - 1) / kRotTile));
  const WarpCoef *dwarp = reinterpret_cast<const WarpCoef *>(dp + pl.off_warp);
  const float *dcoef = reinterpret_cast<const float *>(dp + pl.off_coef);

  for (uint32_t e = 0; e < pl.ne; ++e) {
    const MaterialConsts *mce = dmc + e;
    const float energy = o->energies[e];
    const float wavelength = static_cast<float>(1239.84197 / energy);  // src/cudaMain.cu:607-608
    const float kmag = static_cast<float>(2 * kPi / wavelength);
    ep.kmag = kmag;
    if (!pl.material_frame) {
      // tensor entries once per energy: xx xy xz yy yz [zz]
      bp.mode = 0;
      bp.nvol = pl.nvol;
      bp.mean = sc.means.as<float2>() + size_t(e) * 6;
      CYR_TRY(spectra(mce));
    }
    for (uint32_t k = 0; k < pl.nk; ++k) {
      const KFrame &f = pl.frames[k];
      ep.kvx = f.k.x, ep.kvy = f.k.y, ep.kvz = f.k.z;
      ep.kx = kmag * f.k.x, ep.ky = kmag * f.k.y, ep.kz = kmag * f.k.z;
      if (!pl.material_frame) {
        ep.nangles = pl.nang;
        ep.coef = dcoef + size_t(k) * pl.nang * pl.nbasis;
        ep.images = images;
        ep.gram = reinterpret_cast<float4 *>(images);
        ep.gplane = gram_plane_size(int(pl.ny), int(pl.nx));
        const int slot = ctx.prof.begin(kEwald, st);
        if (pl.nbasis == 2)
          k_ewald_angles<2><<<pix_blocks, 256, 0, st>>>(ep);
        else
          k_ewald_angles<3><<<pix_blocks, 256, 0, st>>>(ep);
        ctx.prof.end(slot, st);
        CYR_CUDA(cudaGetLastError());
      } else {
        // per-angle schedule: p(angle) -> FFT -> DC -> Ewald into image slot a
        for (uint32_t a = 0; a < pl.nang; ++a) {
          const size_t ka = size_t(k) * pl.nang + a;
          bp.mode = 1;
          bp.nvol = 3;
          bp.material_frame = 1;
          bp.mean = sc.means.as<float2>() + size_t(e) * 6;
          for (int c = 0; c < 3; ++c) bp.E[c] = pl.evec[ka * 3 + c];
          std::memcpy(bp.Rm, pl.rmats[ka].m, sizeof bp.Rm);
          CYR_TRY(spectra(mce));
          ep.nangles = 1;
          ep.coef = dcoef + ka;  // nbasis == 1, coefficient 1
          ep.images = images + size_t(a) * pl.npix;
          ep.gram = nullptr;
          const int slot = ctx.prof.begin(kEwald, st);
          k_ewald_angles<1><<<pix_blocks, 256, 0, st>>>(ep);
          ctx.prof.end(slot, st);
          CYR_CUDA(cudaGetLastError());
        }
      }
      int slot = ctx.prof.begin(pl.material_frame ? kRotate : kRotateGram, st);
      if (pl.material_frame) {
        RotateParams rp{};
        rp.images = images;
        rp.coef = dwarp + size_t(k) * pl.nang;
        rp.W = W, rp.H = H;
        rp.nangles = pl.nang;
        rp.rot_mask = o->rot_mask;
        rp.avg = avg;
        k_rotate_average<<<pix_blocks, 256, 0, st>>>(rp);
      } else {
        RotateGramParams rg{};
        rg.gram = reinterpret_cast<const float4 *>(images);
        rg.plane = gram_plane_size(int(pl.ny), int(pl.nx));
        rg.coef = dwarp + size_t(k) * pl.nang;
        rg.ecoef = dcoef + size_t(k) * pl.nang * pl.nbasis;
        rg.W = W, rg.H = H;
        rg.nangles = pl.nang;
        rg.nenergies = 1;
        rg.rot_mask = o->rot_mask;
        rg.avg = avg;
        rg.rows = pl.has_rows ? reinterpret_cast<const int2 *>(dp + pl.off_rows) + (size_t(k) * pl.ne + e) * H : nullptr;
        const size_t rsm = pl.has_rows ? size_t(H) * sizeof(int2) : 0;
        if (pl.nbasis == 2)
          k_rotate_gram<2, 1><<<rot_tiles, kRotTile * kRotTile, rsm, st>>>(rg);
        else
          k_rotate_gram<3, 1><<<rot_tiles, kRotTile * kRotTile, rsm, st>>>(rg);
      }
      ctx.prof.end(slot, st);
      CYR_CUDA(cudaGetLastError());
      float *dst = d_out + (size_t(e) * pl.nk + k) * pl.npix;
      slot = ctx.prof.begin(kFill, st);
      k_fill<<<pix_blocks, 256, 0, st>>>(dst, pl.npix, o->rot_mask ? 0.f : std::numeric_limits<float>::quiet_NaN());
      ctx.prof.end(slot, st);
      slot = ctx.prof.begin(kWarp, st);
      k_warp<<<pix_blocks, 256, 0, st>>>(avg, dst, W, H, pl.detector_warp[k]);
      ctx.prof.end(slot, st);
      CYR_CUDA(cudaGetLastError());
    }
  }
  if (!mode.capturing) CYR_CUDA(cudaEventRecord(sc.last_use, st));
  return CYR_OK;
}


// ---------------------------------------------------------------------------
// FP64 pipeline (fp64.cuh): geometry from the FP32 planner (float decisions),
// amplitudes in double.
// ---------------------------------------------------------------------------
int get_tw64(DeviceContext &ctx, uint32_t n, const double2 **tw) {
  std::lock_guard<std::mutex> lk(ctx.tables_mu);
  auto it = ctx.tw64.find(n);
  if (it != ctx.tw64.end()) {
    *tw = it->second;
    return CYR_OK;
  }
  std::vector<double2> h(n);
  for (uint32_t m = 0; m < n; ++m) {
    const std::complex<double> w = std::polar(1.0, -2.0 * kPi * double(m) / double(n));
    h[m] = make_double2(w.real(), w.imag());
  }
  double2 *d = nullptr;
  CYR_CUDA(cudaMalloc(&d, sizeof(double2) * n));
  CYR_CUDA(cudaMemcpy(d, h.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
  ctx.tw64[n] = d;
  *tw = d;
  return CYR_OK;
}

constexpr size_t kFft64Smem = 192 * 1024;

// One axis of the in-place forward FFT of `count` double volumes, vstride
// elements apart (7-smooth length).
int fft64_axis(DeviceContext &ctx, double2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, int axis,
               cudaStream_t st, size_t vstride) {
  if (!ctx.attrs64) {  // once per device (the attribute belongs to the current device)
    CYR_CUDA(cudaFuncSetAttribute(k64_fft<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFft64Smem)));
    CYR_CUDA(cudaFuncSetAttribute(k64_fft<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFft64Smem)));
    CYR_CUDA(cudaFuncSetAttribute(k64_fft<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFft64Smem)));
    ctx.attrs64 = true;
  }
  const uint32_t dims[3] = {nx, ny, nz};
  {
    const uint32_t n = dims[axis];
    if (n == 1) return CYR_OK;
    std::vector<uint32_t> r;
    if (!factorize(n, r)) return fail(CYR_ERR_UNSUPPORTED, "FP64 path: length %u has a prime factor above 7", n);
    Fft64Params p{};
    p.data = data;
    p.nx = nx, p.ny = ny, p.nz = nz;
    p.vstride = vstride;
    p.n = n;
    p.nstages = uint32_t(r.size());
    for (size_t i = 0; i < r.size(); ++i) p.radix_code |= uint64_t(r[i]) << (4 * i);
    CYR_TRY(get_tw64(ctx, n, &p.tw));
    uint32_t tx = 16;
    while (tx > 1 && size_t(2) * n * tx * sizeof(double2) > 96 * 1024) tx /= 2;
    p.tx = tx;
    const size_t smem = size_t(2) * n * tx * sizeof(double2);
    if (smem > kFft64Smem) return fail(CYR_ERR_UNSUPPORTED, "FP64 path: length %u too large for one block", n);
    const uint32_t tiles = axis == 0 ? (ny * nz + tx - 1) / tx : ((nx + tx - 1) / tx) * (axis == 1 ? nz : ny);
    const dim3 grid(tiles, count);
    if (axis == 0) k64_fft<0><<<grid, 256, smem, st>>>(p);
    if (axis == 1) k64_fft<1><<<grid, 256, smem, st>>>(p);
    if (axis == 2) k64_fft<2><<<grid, 256, smem, st>>>(p);
    CYR_CUDA(cudaGetLastError());
  }
  return CYR_OK;
}

// The FP64 pipeline's Bluestein tables: the chirp and FFT_m(b) / m, formed
// on the host as for the FP32 engine (get_blue) and kept in double.
int get_blue64(DeviceContext &ctx, uint32_t n, DeviceContext::BlueTables64 &out) {
  std::lock_guard<std::mutex> lk(ctx.tables_mu);
  auto it = ctx.blue64.find(n);
  if (it != ctx.blue64.end()) {
    out = it->second;
    return CYR_OK;
  }
  const uint32_t m = bluestein_length(n);
  std::vector<std::complex<double>> c(n), b(m, 0.0), w(m);
  for (uint32_t j = 0; j < n; ++j) {
    const uint64_t q = (uint64_t(j) * j) % (2 * uint64_t(n));
    c[j] = std::polar(1.0, -kPi * double(q) / double(n));
  }
  for (uint32_t j = 0; j < n; ++j) {
    b[j] = std::conj(c[j]);
    if (j) b[m - j] = std::conj(c[j]);
  }
  for (uint32_t j = 0; j < m; ++j) w[j] = std::polar(1.0, -2.0 * kPi * double(j) / double(m));
  std::vector<double2> hc(n), hb(m);
  for (uint32_t j = 0; j < n; ++j) hc[j] = make_double2(c[j].real(), c[j].imag());
  for (uint32_t k = 0; k < m; ++k) {
    std::complex<double> acc(0.0, 0.0);
    uint64_t idx = 0;  // (j k) mod m
    for (uint32_t j = 0; j < m; ++j, idx += k) {
      if (idx >= m) idx %= m;
      acc += b[j] * w[idx];
    }
    acc /= double(m);
    hb[k] = make_double2(acc.real(), acc.imag());
  }
  DeviceContext::BlueTables64 t;
  t.m = m;
  CYR_CUDA(cudaMalloc(&t.chirp, sizeof(double2) * n));
  CYR_CUDA(cudaMalloc(&t.bhat, sizeof(double2) * m));
  CYR_CUDA(cudaMemcpy(t.chirp, hc.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
  CYR_CUDA(cudaMemcpy(t.bhat, hb.data(), sizeof(double2) * m, cudaMemcpyHostToDevice));
  ctx.blue64[n] = t;
  out = t;
  return CYR_OK;
}

// One axis of length n (a prime factor above 7) of the FP64 FFT as a
// Bluestein transform: the FP32 engine's steps (bluestein_pass) in double,
// the padded length-m transforms by fft64_axis, in chunks of padded lines of
// at most 256 MB held in `work`.
int bluestein64(DeviceContext &ctx, double2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, int axis,
                cudaStream_t st, size_t vstride, DeviceBuffer *work) {
  const uint32_t n = axis == 0 ? nx : axis == 1 ? ny : nz;
  DeviceContext::BlueTables64 bt;
  CYR_TRY(get_blue64(ctx, n, bt));
  const uint32_t lpv = axis == 0 ? ny * nz : axis == 1 ? nx * nz : nx * ny;
  const uint64_t total = uint64_t(lpv) * count;
  const uint64_t cap = std::max<uint64_t>(1, (size_t(256) << 20) / (size_t(bt.m) * sizeof(double2)));
  const uint32_t chunk = uint32_t(std::min<uint64_t>(total, cap));
  CYR_TRY(work->ensure(size_t(chunk) * bt.m * sizeof(double2)));
  int sms = 0;
  CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  BlueParamsT<double2> p{};
  p.data = data;
  p.work = work->as<double2>();
  p.chirp = bt.chirp;
  p.bhat = bt.bhat;
  p.nx = nx, p.ny = ny, p.nz = nz;
  p.vstride = vstride;
  p.n = n, p.m = bt.m;
  p.lines_per_vol = lpv;
  for (uint64_t l0 = 0; l0 < total; l0 += chunk) {
    p.line0 = l0;
    p.nlines = uint32_t(std::min<uint64_t>(chunk, total - l0));
    const size_t elems = size_t(p.nlines) * bt.m;
    const unsigned grid = unsigned(std::min<size_t>((elems + 255) / 256, size_t(sms) * 16));
    if (axis == 0) k_blue_gather<0, double2><<<grid, 256, 0, st>>>(p);
    if (axis == 1) k_blue_gather<1, double2><<<grid, 256, 0, st>>>(p);
    if (axis == 2) k_blue_gather<2, double2><<<grid, 256, 0, st>>>(p);
    CYR_CUDA(cudaGetLastError());
    // rows of m (x lines) or columns of m (y and z lines, stored lines fastest)
    auto padded_fft = [&]() -> int {
      if (axis == 0) return fft64_axis(ctx, p.work, bt.m, p.nlines, 1, 1, 0, st, elems);
      return fft64_axis(ctx, p.work, p.nlines, bt.m, 1, 1, 1, st, elems);
    };
    CYR_TRY(padded_fft());
    if (axis == 0)
      k_blue_mul<0, double2><<<grid, 256, 0, st>>>(p);
    else
      k_blue_mul<1, double2><<<grid, 256, 0, st>>>(p);
    CYR_CUDA(cudaGetLastError());
    CYR_TRY(padded_fft());
    if (axis == 0) k_blue_scatter<0, double2><<<grid, 256, 0, st>>>(p);
    if (axis == 1) k_blue_scatter<1, double2><<<grid, 256, 0, st>>>(p);
    if (axis == 2) k_blue_scatter<2, double2><<<grid, 256, 0, st>>>(p);
    CYR_CUDA(cudaGetLastError());
  }
  return CYR_OK;
}

// In-place forward FFT of `count` double volumes: 7-smooth axes by fft64_axis,
// the others as Bluestein transforms.
int fft64(DeviceContext &ctx, double2 *data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, cudaStream_t st) {
  const uint32_t dims[3] = {nx, ny, nz};
  const size_t vstride = size_t(nx) * ny * nz;
  for (int axis = 0; axis < 3; ++axis) {
    if (dims[axis] == 1) continue;
    if (smooth7(dims[axis]))
      CYR_TRY(fft64_axis(ctx, data, nx, ny, nz, count, axis, st, vstride));
    else
      CYR_TRY(bluestein64(ctx, data, nx, ny, nz, count, axis, st, vstride, &ctx.f64.blue));
  }
  return CYR_OK;
}

// The FP64 path's double tables, uploaded beside the planner's float arena:
// refractive indices per energy, Hanning tables and the E basis coefficients.
struct Plan64 {
  std::vector<unsigned char> arena;
  size_t off_mat = 0, off_hx = 0, off_hy = 0, off_hz = 0, off_e = 0;
};

int make_plan64(const cyr_options *o, const double *optical, bool window, Plan &pl, Plan64 &p64) {
  CYR_TRY(validate(o));
  if (!optical) return fail(CYR_ERR_ARGUMENT, "optical constants pointer is null");
  for (uint32_t n : {o->nx, o->ny, o->nz})
    if (n > 1 && !smooth7(n) && (n > (kMaxBluesteinPad + 1) / 2 || bluestein_length(n) > kMaxBluesteinPad))
      return fail(CYR_ERR_UNSUPPORTED, "FP64 path: dimension %u has a prime factor above 7 and exceeds the Bluestein "
                  "limit of 2048", n);
  // geometry (k frames, E rotations, q tables, warp coefficients) from the FP32 planner
  std::vector<float> of(size_t(o->num_energies) * o->num_material * 4);
  for (size_t i = 0; i < of.size(); ++i) of[i] = float(optical[i]);
  CYR_TRY(make_plan(o, of.data(), pl));
  std::vector<Mat64> mats(pl.ne);
  for (uint32_t e = 0; e < pl.ne; ++e) {
    std::memset(&mats[e], 0, sizeof(Mat64));
    for (uint32_t m = 0; m < pl.nmat; ++m) {
      const double *op = optical + (size_t(e) * pl.nmat + m) * 4;
      mats[e].npar[m] = make_double2(1.0 - op[0], op[1]);
      mats[e].nper[m] = make_double2(1.0 - op[2], op[3]);
    }
  }
  p64.arena.clear();
  p64.off_mat = arena_put(p64.arena, mats.data(), mats.size());
  auto hann = [&](uint32_t n, bool unit) {
    std::vector<double> w(n);
    for (uint32_t j = 0; j < n; ++j) w[j] = unit || !window ? 1.0 : 0.5 * (1 - std::cos(2 * kPi * j / n));
    return w;
  };
  const std::vector<double> hx = hann(pl.nx, false), hy = hann(pl.ny, false), hz = hann(pl.nz, pl.twod);
  p64.off_hx = arena_put(p64.arena, hx.data(), hx.size());
  p64.off_hy = arena_put(p64.arena, hy.data(), hy.size());
  p64.off_hz = arena_put(p64.arena, hz.data(), hz.size());
  std::vector<double> ecoef(size_t(pl.nk) * pl.nang * pl.nbasis);
  for (size_t ka = 0; ka < size_t(pl.nk) * pl.nang; ++ka)
    for (uint32_t b = 0; b < pl.nbasis; ++b)
      ecoef[ka * pl.nbasis + b] = pl.material_frame ? 1.0 : double(pl.evec[ka * 3 + b]);
  p64.off_e = arena_put(p64.arena, ecoef.data(), ecoef.size());
  p64.arena.resize((p64.arena.size() + 255) & ~size_t(255));
  return CYR_OK;
}

int run_fp64(DeviceContext &ctx, const cyr_options *o, const double *optical, const void *d_vox, bool vox64,
             double *d_out, cudaStream_t st) {
  Plan pl;
  Plan64 p64;
  CYR_TRY(make_plan64(o, optical, o->algorithm == 0 && o->windowing == 1, pl, p64));
  auto &f = ctx.f64;
  const uint32_t nvol = pl.material_frame ? 3u : pl.nvol;
  CYR_TRY(f.spec.ensure(size_t(nvol) * pl.nvox * sizeof(double2)));
  CYR_TRY(f.images.ensure(size_t(pl.nang) * pl.npix * sizeof(double)));
  CYR_TRY(f.avg.ensure(pl.npix * sizeof(double)));
  CYR_TRY(f.params.ensure(pl.arena.size()));
  CYR_TRY(f.params64.ensure(p64.arena.size()));
  CYR_CUDA(cudaMemcpyAsync(f.params.ptr, pl.arena.data(), pl.arena.size(), cudaMemcpyHostToDevice, st));
  CYR_CUDA(cudaMemcpyAsync(f.params64.ptr, p64.arena.data(), p64.arena.size(), cudaMemcpyHostToDevice, st));
  const unsigned char *dp = f.params.as<unsigned char>(), *dq = f.params64.as<unsigned char>();
  double2 *spec = f.spec.as<double2>();
  double *images = f.images.as<double>(), *avg = f.avg.as<double>();
  int sms = 0;
  CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  Build64Params bp{};
  bp.vox = d_vox;
  bp.vox_fp64 = vox64 ? 1u : 0u;
  bp.nx = pl.nx, bp.ny = pl.ny, bp.nz = pl.nz, bp.nmat = pl.nmat;
  bp.nvox = pl.nvox;
  bp.morphology = o->morphology_type;
  bp.material_frame = pl.material_frame ? 1u : 0u;
  if (pl.hanning) {
    bp.hann_x = reinterpret_cast<const double *>(dq + p64.off_hx);
    bp.hann_y = reinterpret_cast<const double *>(dq + p64.off_hy);
    bp.hann_z = reinterpret_cast<const double *>(dq + p64.off_hz);
  }
  const unsigned bgrid = unsigned(std::min<size_t>((pl.nvox + 255) / 256, size_t(sms) * 8));
  const unsigned pgrid = unsigned((pl.npix + 255) / 256);
  const int W = int(pl.ny), H = int(pl.nx);  // the reference hands NPP width = Ny, height = Nx
  const WarpCoef *dwarp = reinterpret_cast<const WarpCoef *>(dp + pl.off_warp);
  const double *dE = reinterpret_cast<const double *>(dq + p64.off_e);
  const Mat64 *dmat = reinterpret_cast<const Mat64 *>(dq + p64.off_mat);
  const double prefill = o->rot_mask ? 0.0 : std::numeric_limits<double>::quiet_NaN();
  for (uint32_t e = 0; e < pl.ne; ++e) {
    const float wavelength = static_cast<float>(1239.84197 / o->energies[e]);  // src/cudaMain.cu:607-608
    const float kmag = static_cast<float>(2 * kPi / wavelength);
    auto spectra = [&](uint32_t nv) -> int {
      bp.nvol = nv;
      bp.out = spec;
      k64_build<<<bgrid, 256, 0, st>>>(bp, dmat + e);
      CYR_CUDA(cudaGetLastError());
      CYR_TRY(fft64(ctx, spec, pl.nx, pl.ny, pl.nz, nv, st));
      k64_dc<<<1, 32, 0, st>>>(spec, nv, pl.nvox, pl.nx, pl.ny, pl.nz);
      CYR_CUDA(cudaGetLastError());
      return CYR_OK;
    };
    if (!pl.material_frame) {
      bp.mode = 0;
      CYR_TRY(spectra(nvol));
    }
    for (uint32_t k = 0; k < pl.nk; ++k) {
      const KFrame &fr = pl.frames[k];
      Ewald64Params ep{};
      ep.spec = spec;
      ep.vstride = pl.nvox;
      ep.g.start = -static_cast<float>(kPi / o->phys_size);
      ep.g.dx = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nx - 1) * 1.0));
      ep.g.dy = static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.ny - 1) * 1.0));
      ep.g.dz = pl.twod ? 0.f : static_cast<float>((2.0 * kPi / o->phys_size) / ((pl.nz - 1) * 1.0));
      ep.g.kmag = kmag;
      ep.g.kx = kmag * fr.k.x, ep.g.ky = kmag * fr.k.y, ep.g.kz = kmag * fr.k.z;
      ep.g.nx = pl.nx, ep.g.ny = pl.ny, ep.g.nz = pl.nz;
      ep.g.interp = o->ewald_interpolation;
      ep.g.twod = pl.twod ? 1u : 0u;
      ep.qx = reinterpret_cast<const float *>(dp + pl.off_qx);
      ep.qy = reinterpret_cast<const float *>(dp + pl.off_qy);
      ep.qz = reinterpret_cast<const float *>(dp + pl.off_qz);
      if (!pl.material_frame) {
        const uint32_t sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
        ep.nbasis = pl.nbasis;
        for (int c = 0; c < 3; ++c)
          for (uint32_t b = 0; b < pl.nbasis; ++b) ep.vol[c][b] = sym[c][b];
        ep.nangles = pl.nang;
        ep.E = dE + size_t(k) * pl.nang * pl.nbasis;
        ep.images = images;
        k64_ewald<<<pgrid, 256, 0, st>>>(ep);
        CYR_CUDA(cudaGetLastError());
      } else {
        // per angle, as the reference: p = R^T Nt R x -> 3 transforms -> Ewald into image a
        for (uint32_t a = 0; a < pl.nang; ++a) {
          const size_t ka = size_t(k) * pl.nang + a;
          bp.mode = 1;
          for (int c = 0; c < 3; ++c) bp.E[c] = double(pl.evec[ka * 3 + c]);
          for (int i = 0; i < 9; ++i) bp.R[i] = double(pl.rmats[ka].m[i]);
          CYR_TRY(spectra(3));
          ep.nbasis = 1;
          for (int c = 0; c < 3; ++c) ep.vol[c][0] = uint32_t(c);
          ep.nangles = 1;
          ep.E = dE + ka;  // coefficient 1
          ep.images = images + size_t(a) * pl.npix;
          k64_ewald<<<pgrid, 256, 0, st>>>(ep);
          CYR_CUDA(cudaGetLastError());
        }
      }
      Rotate64Params rp{};
      rp.images = images;
      rp.coef = dwarp + size_t(k) * pl.nang;
      rp.W = W, rp.H = H;
      rp.nangles = pl.nang;
      rp.rot_mask = o->rot_mask;
      rp.avg = avg;
      k64_rotate_average<<<pgrid, 256, 0, st>>>(rp);
      k64_warp<<<pgrid, 256, 0, st>>>(avg, d_out + (size_t(e) * pl.nk + k) * pl.npix, W, H, pl.detector_warp[k],
                                      prefill);
      CYR_CUDA(cudaGetLastError());
    }
  }
  return CYR_OK;
}

// ---------------------------------------------------------------------------
// Serving engine: continuous batching of simulation requests on one GPU.
//
// A worker thread owns S slots.  Each slot has its own stream, its own
// request scratch (stream-ordered allocations) and staging buffers, so the
// requests in different slots overlap on the device.  Requests wait in a FIFO
// queue and are admitted as soon as a slot is free and their device footprint
// (request_bytes + staging) fits in the HBM budget next to the requests in
// flight; completion is detected with one event per slot.  Optionally a slot
// replays a CUDA graph of a request signature it has already run (the same
// options and input pointers; the optical constants travel in the parameter
// arena, which each replay rewrites in the slot's pinned host copy).
// ---------------------------------------------------------------------------
using Clock = std::chrono::steady_clock;

struct ServerRequest {
  uint64_t id = 0;
  cyr_options opt{};
  std::vector<float> energies, kvecs, optical;
  const float *h_vox = nullptr;  // host buffers (caller-owned until the request is done)
  float *h_out = nullptr;
  const float4 *d_vox = nullptr;  // or device buffers
  float *d_out = nullptr;
  size_t vox_bytes = 0, out_bytes = 0, footprint = 0;
  std::string key;  // graph signature
  std::string group_key;  // requests with the same key may share launches (empty: never grouped)
  Plan plan;        // host plan (strategy resolved), made once at submit
  double work = 0;  // share of the GPU the request fills (1 = saturating)
  int status = -1;  // -1 queued or running, else a CYR_* code
  std::string error;
  Clock::time_point t_submit, t_start, t_done;
};

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  uint64_t generation = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Scratch sc;
  DeviceBuffer vox, out;  // staging for host-buffer requests
  unsigned char *host_arena = nullptr;
  size_t host_arena_bytes = 0;
  unsigned *host_errors = nullptr;  // pinned copy of the request's device error counter
  std::shared_ptr<ServerRequest> req;
  std::vector<std::shared_ptr<ServerRequest>> group;  // the other requests sharing req's launches
  std::map<std::string, GraphEntry> graphs;
  std::map<std::string, uint64_t> warm;  // signature -> scratch generation after its last uncaptured run
  uint64_t generation() const { return sc.generation; }
};

struct Server {
  DeviceContext *ctx = nullptr;
  int device = 0;
  std::vector<std::unique_ptr<Slot>> slots;
  size_t budget = 0, in_use = 0;
  double inflight_work = 0;
  bool graphs = false;
  bool groups = false;  // same-shape queued requests share one launch per kernel
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<ServerRequest>> queue;
  std::map<uint64_t, std::shared_ptr<ServerRequest>> requests;
  uint64_t next_id = 1;
  bool stop = false;
  std::atomic<uint64_t> completed{0}, failed{0}, replays{0}, captures{0}, group_runs{0}, grouped{0};
  std::thread worker;
};

// Host planning for one request: resolve the AUTO strategy (so a signature
// always means the same launch sequence) and compute its footprint.
// Voxel-materials one request needs to fill the GPU on its own; smaller
// requests leave room for others to run beside them.
constexpr double kSaturatingWork = 8.0e6;
// Requests in flight at once, in units of GPU-filling requests: beyond about
// two, concurrency only time-slices large requests and lengthens latency.
constexpr double kMaxInflightWork = 2.0;

int plan_request(ServerRequest &r, bool staged) {
  Plan &pl = r.plan;
  CYR_TRY(make_plan(&r.opt, r.optical.data(), pl));
  if (r.opt.strategy == CYR_STRATEGY_AUTO) r.opt.strategy = pl.fields ? CYR_STRATEGY_FIELDS : CYR_STRATEGY_PER_ENERGY;
  r.footprint = request_bytes(pl) + (staged ? r.vox_bytes + r.out_bytes : 0);
  r.work = std::min(1.0, double(pl.nvox) * pl.nmat / kSaturatingWork);
  char head[256];
  std::snprintf(head, sizeof head, "%u,%u,%u,%u,%u,%a,%a,%a,%a,%u,%u,%u,%u,%u,%u,%u,%u,%u,%u,%u,%a,%a,%a|%p|%p|",
                r.opt.nx, r.opt.ny, r.opt.nz, r.opt.num_material, r.opt.num_energies, double(r.opt.start_angle),
                double(r.opt.end_angle), double(r.opt.increment_angle), double(r.opt.phys_size), r.opt.case_type,
                r.opt.num_k, r.opt.morphology_type, r.opt.ewald_interpolation, r.opt.windowing,
                r.opt.scatter_approach, r.opt.algorithm, r.opt.rot_mask, r.opt.reference_frame, r.opt.strategy,
                staged ? 1u : 0u, double(r.opt.detector[0]), double(r.opt.detector[1]), double(r.opt.detector[2]),
                staged ? nullptr : static_cast<const void *>(r.d_vox), staged ? nullptr : static_cast<void *>(r.d_out));
  r.key = head;
  for (float e : r.energies) r.key += std::to_string(e) + ",";
  for (float k : r.kvecs) r.key += std::to_string(k) + ",";
  // requests that can share launches: FIELDS, LAB frame, k along z, device buffers; all but the
  // morphology, the energies and the optical constants equal
  r.group_key.clear();
  if (pl.fields && !pl.material_frame && r.opt.case_type == 0 && pl.nk == 1 && pl.nbasis == 2 && r.d_vox) {
    char g[256];
    std::snprintf(g, sizeof g, "%u,%u,%u,%u,%u,%a,%a,%a,%a,%u,%u,%u,%u,%u", r.opt.nx, r.opt.ny, r.opt.nz,
                  r.opt.num_material, r.opt.num_energies, double(r.opt.start_angle), double(r.opt.end_angle),
                  double(r.opt.increment_angle), double(r.opt.phys_size), r.opt.morphology_type,
                  r.opt.ewald_interpolation, pl.hanning ? 1u : 0u, r.opt.rot_mask, pl.has_rows ? 1u : 0u);
    r.group_key = g;
  }
  return CYR_OK;
}

// Grows the slot's pinned copy of the parameter arena (its graphs read the old one: dropped).
int ensure_host_arena(Slot &sl, size_t bytes) {
  if (bytes <= sl.host_arena_bytes) return CYR_OK;
  if (sl.host_arena) {
    CYR_CUDA(cudaStreamSynchronize(sl.stream));
    cudaFreeHost(sl.host_arena);
    sl.host_arena = nullptr;
  }
  for (auto &kv : sl.graphs) cudaGraphExecDestroy(kv.second.exec);
  sl.graphs.clear();
  sl.host_arena_bytes = std::max<size_t>(bytes, 64 * 1024);
  CYR_CUDA(cudaMallocHost(&sl.host_arena, sl.host_arena_bytes));
  return CYR_OK;
}

// Requests per group: at most 16, and their packed volumes must fit one DC block.
constexpr uint32_t kMaxGroup = 16;

// A group of same-key requests (FIELDS strategy) with one launch per kernel:
// moments, field build + x pass, y and z passes over all G npk packed volumes,
// DC, then the Ewald projection, rotation and detector warp over the G E
// "virtual energies" (request q's energy e is virtual energy q E + e), each
// request's constants in per-virtual-energy tables.  Every request computes
// exactly what it computes alone (same kernels, same arithmetic per element).
int run_group(Server &S, Slot &sl, const std::vector<std::shared_ptr<ServerRequest>> &g) {
  DeviceContext &ctx = *S.ctx;
  Scratch &sc = sl.sc;
  cudaStream_t st = sl.stream;
  const ServerRequest &r0 = *g[0];
  const Plan &p0 = r0.plan;
  const cyr_options *o = &r0.opt;
  const uint32_t G = uint32_t(g.size()), E = p0.ne, npk = p0.npk, nmat = p0.nmat;
  const int W = int(p0.ny), H = int(p0.nx);  // the reference hands NPP width = Ny, height = Nx
  CYR_TRY(setup_attrs(ctx));
  CYR_TRY(sc.init());
  // arena: request 0's (the shared geometry tables), then the per-virtual-energy and pointer tables
  std::vector<unsigned char> arena = p0.arena;
  std::vector<float4> fc;
  std::vector<float> km;
  std::vector<int2> rows;
  std::vector<const float4 *> vp;
  std::vector<float *> op;
  bool sparse = nmat <= 4 && ctx.sparse_ewald;  // every member's coefficients keep the structural zeros
  for (const auto &r : g) {
    const Plan &pl = r->plan;
    sparse = sparse && pl.ewald_sparse;
    const float4 *c = reinterpret_cast<const float4 *>(pl.arena.data() + pl.off_fcoef);
    fc.insert(fc.end(), c, c + size_t(E) * 6 * npk);
    const float *k = reinterpret_cast<const float *>(pl.arena.data() + pl.off_kmag);
    km.insert(km.end(), k, k + E);
    if (p0.has_rows) {
      const int2 *rw = reinterpret_cast<const int2 *>(pl.arena.data() + pl.off_rows);
      rows.insert(rows.end(), rw, rw + size_t(E) * H);
    }
    vp.push_back(r->d_vox);
    op.push_back(r->d_out);
  }
  const size_t off_c = arena_put(arena, fc.data(), fc.size());
  const size_t off_k = arena_put(arena, km.data(), km.size());
  const float kv0[3] = {p0.frames[0].k.x, p0.frames[0].k.y, p0.frames[0].k.z};
  const size_t off_kv = arena_put(arena, kv0, 3);
  const size_t off_r = p0.has_rows ? arena_put(arena, rows.data(), rows.size()) : 0;
  const size_t off_v = arena_put(arena, vp.data(), vp.size());
  const size_t off_o = arena_put(arena, op.data(), op.size());
  arena.resize((arena.size() + 255) & ~size_t(255));
  CYR_TRY(ensure_host_arena(sl, arena.size()));
  std::memcpy(sl.host_arena, arena.data(), arena.size());
  CYR_TRY(sc.params.ensure(arena.size()));
  CYR_CUDA(cudaMemcpyAsync(sc.params.ptr, sl.host_arena, arena.size(), cudaMemcpyHostToDevice, st));
  const unsigned char *dp = sc.params.as<unsigned char>();
  // scratch; virtual energies per Ewald / rotation launch: whole records, at most 256 MB of them
  const size_t nvox = p0.nvox, npix = p0.npix;
  const uint32_t nep = gram_nep(p0), total = G * E;
  uint32_t vb = std::min<uint32_t>(total, 512);
  while (vb > nep && image_bytes(p0, vb) > (size_t(256) << 20)) vb -= nep;
  if (vb < total) vb = std::max(nep, vb / nep * nep);
  CYR_TRY(sc.spec.ensure(size_t(G) * npk * nvox * sizeof(float2)));
  CYR_TRY(sc.images.ensure(image_bytes(p0, vb)));
  CYR_TRY(sc.avg.ensure(size_t(vb) * npix * sizeof(float)));
  CYR_TRY(sc.moments.ensure(size_t(G) * nmat * kMoments * sizeof(double)));
  CYR_TRY(sc.dc.ensure(size_t(G) * npk * sizeof(float2)));
  CYR_TRY(sc.errors.ensure(sizeof(unsigned)));
  CYR_CUDA(cudaMemsetAsync(sc.errors.ptr, 0, sizeof(unsigned), st));
  CYR_CUDA(cudaMemsetAsync(sc.moments.ptr, 0, size_t(G) * nmat * kMoments * sizeof(double), st));
  float2 *spec = sc.spec.as<float2>();
  int sms = 0;
  CYR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  const float4 *const *vox_g = reinterpret_cast<const float4 *const *>(dp + off_v);
  // moments of every request (blockIdx.z = request), over the z-plane subsample
  MomentParams mp{};
  mp.vox_g = vox_g;
  mp.nx = p0.nx, mp.ny = p0.ny, mp.nz = p0.nz, mp.nmat = nmat;
  mp.nvox = nvox;
  if (p0.hanning) {
    mp.hann_x = reinterpret_cast<const float *>(dp + p0.off_hx);
    mp.hann_y = reinterpret_cast<const float *>(dp + p0.off_hy);
    mp.hann_z = reinterpret_cast<const float *>(dp + p0.off_hz);
  }
  mp.out = sc.moments.as<double>();
  mp.zstep = p0.mom_zstep;
  const size_t nsamp = npix * ((p0.nz + mp.zstep - 1) / mp.zstep);
  {
    const dim3 grid(uint32_t(std::max<size_t>(1, std::min<size_t>((nsamp + 2047) / 2048, size_t(sms) * 4))), nmat, G);
    const int slot = ctx.prof.begin(kMom, st);
    if (o->morphology_type == 0)
      k_moments<0><<<grid, 256, 0, st>>>(mp);
    else
      k_moments<1><<<grid, 256, 0, st>>>(mp);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  }
  // field build + x pass (blockIdx.y = request), then y and z over all G npk volumes
  FieldParams fp{};
  fp.vox_g = vox_g;
  fp.nx = p0.nx, fp.ny = p0.ny, fp.nz = p0.nz, fp.nmat = nmat;
  fp.nvox = nvox;
  fp.mom = sc.moments.as<double>();
  fp.mom_stride = size_t(nmat) * kMoments;
  fp.nsamp = nsamp;
  fp.out = spec;
  fp.out_stride = size_t(npk) * nvox;
  fp.i0 = 0, fp.i1 = nvox;
  if (p0.hanning) fp.hann_x = mp.hann_x, fp.hann_y = mp.hann_y, fp.hann_z = mp.hann_z;
  const bool fused_ok = (p0.nx == 128 || p0.nx == 256 || p0.nx == 512 || p0.nx == 1024) &&
                        fields_rows_smem(p0.nx, npk, nmat) <= kFftSmemBudget;
  DeviceContext::FieldTune ft;
  {
    char key[96];
    std::snprintf(key, sizeof key, "%u,%u,%u,%u", p0.nx, p0.ny, p0.nz, npk);
    std::lock_guard<std::mutex> lk(ctx.tables_mu);
    auto it = ctx.ftune.find(key);
    if (it != ctx.ftune.end()) ft = it->second;
  }
  if (fused_ok && ft.fused) {
    const float2 *twx = nullptr;
    CYR_TRY(get_twiddles(ctx, p0.nx, &twx));
    const size_t smem = fields_rows_smem(p0.nx, npk, nmat);
    const uint32_t rws = p0.nz * p0.ny;
    int per_sm = 1;
    auto launch = [&](auto kern) -> int {
      CYR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
      const size_t want = (size_t(std::max(1, per_sm)) * sms + G - 1) / G;
      kern<<<dim3(unsigned(std::min<size_t>(rws, want)), G), 256, smem, st>>>(fp, twx, npk);
      return CYR_OK;
    };
    const int slot = ctx.prof.begin(kBuildFieldsRows, st);
    const bool euler = o->morphology_type == 0;
    if (p0.nx == 128) CYR_TRY(launch(euler ? k_build_fields_rows<0, 4> : k_build_fields_rows<1, 4>));
    if (p0.nx == 256) CYR_TRY(launch(euler ? k_build_fields_rows<0, 8> : k_build_fields_rows<1, 8>));
    if (p0.nx == 512) CYR_TRY(launch(euler ? k_build_fields_rows<0, 16> : k_build_fields_rows<1, 16>));
    if (p0.nx == 1024) CYR_TRY(launch(euler ? k_build_fields_rows<0, 32> : k_build_fields_rows<1, 32>));
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  } else {
    const uint32_t blocks =
        uint32_t(std::max<size_t>(1, std::min<size_t>((nvox + 255) / 256, (size_t(sms) * 8 + G - 1) / G)));
    const int slot = ctx.prof.begin(kBuildFields, st);
    if (o->morphology_type == 0)
      k_build_fields<0><<<dim3(blocks, G), 256, 0, st>>>(fp);
    else
      k_build_fields<1><<<dim3(blocks, G), 256, 0, st>>>(fp);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
    CYR_TRY(fft_axes(ctx, spec, p0.nx, p0.ny, p0.nz, npk * G, st, 0, 0, 0, &sc.blue, ft.form));
  }
  // the planes the Ewald projection reads for any of the G E virtual energies
  const EwaldGeom geom = field_geometry(o, p0);
  const uint32_t *zmask = nullptr;
  CYR_TRY(field_zmask(ctx, sc, geom, reinterpret_cast<const float *>(dp + off_k), G * E,
                      reinterpret_cast<const float *>(dp + off_kv), 1, st, &zmask));
  CYR_TRY(fft_axes(ctx, spec, p0.nx, p0.ny, p0.nz, npk * G, st, 1, 2, 0, &sc.blue, ft.form, zmask));
  {
    const int slot = ctx.prof.begin(kDc, st);
    k_dc<<<1, (npk * G + 31) / 32 * 32, 0, st>>>(spec, npk * G, nvox, p0.nx, p0.ny, p0.nz, 0, 1 % p0.nz, p0.nz - 1,
                                                 sc.dc.as<float2>());
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  }
  // Ewald projection, rotation and detector warp over the virtual energies
  FieldEwaldParams fe{};
  fe.zspec = spec;
  fe.zdc = sc.dc.as<float2>();
  fe.npk = npk;
  fe.nvox = nvox;
  fe.coef = reinterpret_cast<const float4 *>(dp + off_c);
  fe.kmag = reinterpret_cast<const float *>(dp + off_k);
  fe.e_per_req = E;
  fe.g = geom;
  fe.qx = reinterpret_cast<const float *>(dp + p0.off_qx);
  fe.qy = reinterpret_cast<const float *>(dp + p0.off_qy);
  fe.qz = reinterpret_cast<const float *>(dp + p0.off_qz);
  fe.nangles = p0.nang;
  fe.images = sc.images.as<float>();
  fe.gram = sc.images.as<float4>();
  fe.gplane = gram_plane_size(int(p0.ny), int(p0.nx));
  const KFrame &f = p0.frames[0];
  fe.kvx = f.k.x, fe.kvy = f.k.y, fe.kvz = f.k.z;
  fe.mat = reinterpret_cast<const float *>(dp + p0.off_mat);
  fe.ecoef = reinterpret_cast<const float *>(dp + p0.off_coef);
  RotateGramParams rg{};
  rg.gram = sc.images.as<float4>();
  rg.plane = fe.gplane;
  rg.coef = reinterpret_cast<const WarpCoef *>(dp + p0.off_warp);
  rg.ecoef = fe.ecoef;
  rg.W = W, rg.H = H;
  rg.nangles = p0.nang;
  rg.rot_mask = o->rot_mask;
  rg.avg = sc.avg.as<float>();
  const size_t fsmem = size_t(kEwaldEnergies) * 6 * npk * sizeof(float4);
  const unsigned fpix_blocks = unsigned((npix + 31) / 32), pix_blocks = unsigned((npix + 255) / 256);
  const unsigned rot_tiles = unsigned(((W + kRotTile - 1) / kRotTile) * ((H + kRotTile - 1) / kRotTile));
  const size_t rsm = p0.has_rows ? size_t(H) * sizeof(int2) : 0;
  const float fillv = o->rot_mask ? 0.f : std::numeric_limits<float>::quiet_NaN();
  float *const *out_g = reinterpret_cast<float *const *>(dp + off_o);
  for (uint32_t e0 = 0; e0 < total; e0 += vb) {
    const uint32_t nb = std::min(vb, total - e0);
    fe.e0 = e0;
    fe.nbatch = nb;
    rg.nenergies = nb;
    rg.rows = p0.has_rows ? reinterpret_cast<const int2 *>(dp + off_r) + size_t(e0) * H : nullptr;
    int slot = ctx.prof.begin(kEwaldFields, st);
    const unsigned fgrid = fpix_blocks * ((nb + kEwaldEnergies - 1) / kEwaldEnergies);
    if (sparse && nmat == 1)
      k_ewald_fields<2, true, 1><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
    else if (sparse && nmat == 2)
      k_ewald_fields<2, true, 2><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
    else if (sparse && nmat == 3)
      k_ewald_fields<2, true, 3><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
    else if (sparse && nmat == 4)
      k_ewald_fields<2, true, 4><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
    else
      k_ewald_fields<2, true><<<fgrid, kFieldEwaldThreads, fsmem, st>>>(fe);
    ctx.prof.end(slot, st);
    slot = ctx.prof.begin(kRotateGram, st);
    k_rotate_gram<2, packed_energies<2>()><<<dim3(rot_tiles, (nb + nep - 1) / nep), kRotTile * kRotTile, rsm, st>>>(rg);
    ctx.prof.end(slot, st);
    slot = ctx.prof.begin(kWarp, st);
    k_warp_group<<<dim3(pix_blocks, nb), 256, 0, st>>>(sc.avg.as<float>(), out_g, E, e0, W, H, p0.detector_warp[0],
                                                       fillv);
    ctx.prof.end(slot, st);
    CYR_CUDA(cudaGetLastError());
  }
  CYR_CUDA(cudaEventRecord(sc.last_use, st));
  return CYR_OK;
}

// Enqueues request r on slot sl (worker thread).
// Host buffers always go through the slot's staging buffers; with graphs,
// device buffers do too (device-to-device), so a signature does not depend on
// the caller's pointers and one graph serves every morphology of a shape.
bool staged_request(const Server &S, const ServerRequest &r) { return r.h_vox != nullptr || S.graphs; }

int start_request(Server &S, Slot &sl, ServerRequest &r) {
  cudaStream_t st = sl.stream;
  const float4 *d_vox = r.d_vox;
  float *d_out = r.d_out;
  const bool staged = staged_request(S, r);
  if (staged) {
    CYR_TRY(sl.vox.ensure(r.vox_bytes));
    CYR_TRY(sl.out.ensure(r.out_bytes));
    CYR_CUDA(cudaMemcpyAsync(sl.vox.ptr, r.h_vox ? static_cast<const void *>(r.h_vox) : r.d_vox, r.vox_bytes,
                             r.h_vox ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    d_vox = sl.vox.as<float4>();
    d_out = sl.out.as<float>();
  }
  const Plan &pl = r.plan;
  CYR_TRY(ensure_host_arena(sl, pl.arena.size()));  // graphs' upload nodes read the old copy: dropped on growth
  RunMode mode;
  mode.host_arena = sl.host_arena;
  mode.host_arena_bytes = sl.host_arena_bytes;
  mode.plan = &r.plan;
  auto git = S.graphs ? sl.graphs.find(r.key) : sl.graphs.end();
  if (git != sl.graphs.end() && git->second.generation == sl.generation()) {
    std::memcpy(sl.host_arena, pl.arena.data(), pl.arena.size());
    CYR_CUDA(cudaGraphLaunch(git->second.exec, st));
    ++S.replays;
  } else {
    auto wit = sl.warm.find(r.key);
    if (S.graphs && wit != sl.warm.end() && wit->second == sl.generation()) {
      // same signature ran on these buffers: capture (nothing is allocated) and replay
      if (git != sl.graphs.end()) {
        cudaGraphExecDestroy(git->second.exec);
        sl.graphs.erase(git);
      }
      mode.capturing = true;
      CYR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const int rc = run_request(*S.ctx, sl.sc, &r.opt, r.optical.data(), d_vox, d_out, st, mode);
      cudaGraph_t g = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(st, &g);
      if (rc != CYR_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ec != cudaSuccess) return fail(CYR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
      GraphEntry ge;
      const cudaError_t ei = cudaGraphInstantiate(&ge.exec, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) return fail(CYR_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ei));
      ge.generation = sl.generation();
      CYR_CUDA(cudaGraphLaunch(ge.exec, st));
      sl.graphs[r.key] = ge;
      ++S.captures;
    } else {
      CYR_TRY(run_request(*S.ctx, sl.sc, &r.opt, r.optical.data(), d_vox, d_out, st, mode));
      sl.warm[r.key] = sl.generation();
    }
  }
  CYR_CUDA(cudaMemcpyAsync(sl.host_errors, sl.sc.errors.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  if (staged)
    CYR_CUDA(cudaMemcpyAsync(r.h_out ? static_cast<void *>(r.h_out) : static_cast<void *>(r.d_out), d_out, r.out_bytes,
                             r.h_out ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
  CYR_CUDA(cudaEventRecord(sl.done, st));
  return CYR_OK;
}

// Enqueues a group of same-key requests on slot sl (worker thread).
int start_group(Server &S, Slot &sl, const std::vector<std::shared_ptr<ServerRequest>> &g) {
  CYR_TRY(run_group(S, sl, g));
  CYR_CUDA(cudaMemcpyAsync(sl.host_errors, sl.sc.errors.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, sl.stream));
  CYR_CUDA(cudaEventRecord(sl.done, sl.stream));
  ++S.group_runs;
  S.grouped += g.size();
  return CYR_OK;
}

void finish_request(Server &S, Slot &sl, int status, const std::string &err) {
  std::vector<std::shared_ptr<ServerRequest>> rs{sl.req};
  rs.insert(rs.end(), sl.group.begin(), sl.group.end());
  sl.req.reset();
  sl.group.clear();
  std::lock_guard<std::mutex> lk(S.mu);
  const Clock::time_point now = Clock::now();
  for (const auto &r : rs) {
    r->t_done = now;
    r->status = status;
    r->error = err;
    S.in_use -= std::min(S.in_use, r->footprint);
    S.inflight_work = std::max(0.0, S.inflight_work - r->work);
    if (status == CYR_OK)
      ++S.completed;
    else
      ++S.failed;
  }
  S.cv_done.notify_all();
}

void server_loop(Server *Sp) {
  Server &S = *Sp;
  cudaSetDevice(S.device);
  for (;;) {
    bool progress = false;
    // completions
    for (auto &slp : S.slots) {
      Slot &sl = *slp;
      if (!sl.req) continue;
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      progress = true;
      if (q != cudaSuccess) {
        finish_request(S, sl, CYR_ERR_CUDA, std::string("request failed on the device: ") + cudaGetErrorString(q));
      } else if (*sl.host_errors != 0) {
        char m[128];
        std::snprintf(m, sizeof m, "%u detector pixels needed z planes outside the kept range", *sl.host_errors);
        finish_request(S, sl, CYR_ERR_CUDA, m);
      } else {
        finish_request(S, sl, CYR_OK, "");
      }
    }
    // admissions (FIFO): a free slot and room in the budget; a request larger
    // than the whole budget runs alone
    for (;;) {
      std::shared_ptr<ServerRequest> r;
      Slot *free_slot = nullptr;
      bool any_active = false;
      {
        std::lock_guard<std::mutex> lk(S.mu);
        if (S.queue.empty()) break;
        r = S.queue.front();
      }
      // a free slot, preferring one that holds this signature's graph or warm state
      int best = -1;
      for (auto &slp : S.slots) {
        Slot &sl = *slp;
        if (sl.req) {
          any_active = true;
          continue;
        }
        auto g = sl.graphs.find(r->key);
        auto wm = sl.warm.find(r->key);
        const int score = (g != sl.graphs.end() && g->second.generation == sl.generation())  ? 2
                          : (wm != sl.warm.end() && wm->second == sl.generation()) ? 1
                                                                                    : 0;
        if (score > best) best = score, free_slot = &sl;
      }
      std::vector<std::shared_ptr<ServerRequest>> grp;  // requests sharing r's launches
      {
        std::lock_guard<std::mutex> lk(S.mu);
        if (!free_slot) break;
        if (any_active && (S.in_use + r->footprint > S.budget || S.inflight_work + r->work > kMaxInflightWork))
          break;
        S.queue.pop_front();
        S.in_use += r->footprint;
        S.inflight_work += r->work;
        const Clock::time_point now = Clock::now();
        r->t_start = now;
        if (S.groups && !r->group_key.empty()) {
          // queued requests of the same key join r, as far as the budget allows
          const uint32_t cap = std::min<uint32_t>(kMaxGroup, std::max<uint32_t>(1, 1024 / r->plan.npk));
          for (auto it = S.queue.begin(); it != S.queue.end() && grp.size() + 1 < cap;) {
            if ((*it)->group_key == r->group_key && S.in_use + (*it)->footprint <= S.budget) {
              S.in_use += (*it)->footprint;
              S.inflight_work += (*it)->work;
              (*it)->t_start = now;
              grp.push_back(*it);
              it = S.queue.erase(it);
            } else {
              ++it;
            }
          }
        }
      }
      progress = true;
      free_slot->req = r;
      free_slot->group = grp;
      int rc;
      if (grp.empty()) {
        rc = start_request(S, *free_slot, *r);
      } else {
        std::vector<std::shared_ptr<ServerRequest>> all{r};
        all.insert(all.end(), grp.begin(), grp.end());
        rc = start_group(S, *free_slot, all);
      }
      if (rc != CYR_OK) {
        const std::string err = g_error;
        cudaStreamSynchronize(free_slot->stream);  // let whatever was enqueued finish before the slot is reused
        cudaGetLastError();
        finish_request(S, *free_slot, rc, err);
      }
    }
    bool active = false;
    for (auto &slp : S.slots) active = active || slp->req != nullptr;
    std::unique_lock<std::mutex> lk(S.mu);
    if (S.stop && S.queue.empty() && !active) break;
    if (!active && S.queue.empty()) {
      S.cv_work.wait(lk, [&] { return S.stop || !S.queue.empty(); });
    } else if (!progress) {
      // requests in flight: poll their events again shortly
      S.cv_work.wait_for(lk, std::chrono::microseconds(20));
    }
  }
}

int server_destroy(Server *S) {
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->device);
  for (auto &slp : S->slots) {
    Slot &sl = *slp;
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (auto &kv : sl.graphs) cudaGraphExecDestroy(kv.second.exec);
    sl.sc.release();
    sl.vox.release();
    sl.out.release();
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.host_arena) cudaFreeHost(sl.host_arena);
    if (sl.host_errors) cudaFreeHost(sl.host_errors);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.sc.last_use) cudaEventDestroy(sl.sc.last_use);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete S;
  return CYR_OK;
}
}  // namespace
}  // namespace cyr

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace cyr;

extern "C" {

const char *cyr_last_error(void) { return g_error.c_str(); }

const char *cyr_version(void) { return "cyrsoxs-gb300 0.1 (sm_103a)"; }

int cyr_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return n;
}

int cyr_required_device_bytes(const cyr_options *opt, size_t *bytes) {
  if (!bytes) return fail(CYR_ERR_ARGUMENT, "bytes pointer is null");
  CYR_TRY(validate(opt));
  std::vector<float> dummy(size_t(opt->num_energies) * opt->num_material * 4, 0.f);
  Plan pl;
  CYR_TRY(make_plan(opt, dummy.data(), pl));
  *bytes = request_bytes(pl);
  return CYR_OK;
}

int cyr_plan_info(const cyr_options *opt, uint32_t *info, uint32_t n) {
  if (!info) return fail(CYR_ERR_ARGUMENT, "info pointer is null");
  CYR_TRY(validate(opt));
  std::vector<float> dummy(size_t(opt->num_energies) * opt->num_material * 4, 0.f);
  Plan pl;
  CYR_TRY(make_plan(opt, dummy.data(), pl));
  const uint32_t v[9] = {pl.nvol, pl.pruned ? pl.kz : pl.nz, pl.zlo, pl.pruned ? 1u : 0u, pl.nang, pl.nk,
                         pl.fields ? 1u : 0u, pl.npk, pl.ebatch};
  for (uint32_t i = 0; i < n && i < 9; ++i) info[i] = v[i];
  return CYR_OK;
}

int cyr_tuning_report(char *buf, size_t len) {
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->tables_mu);
  std::string r;
  for (const auto &kv : ctx->ztune) {
    char line[160];
    std::snprintf(line, sizeof line, "build_fft_z[%s]: stage=%d tx=%u %.3f ms\n", kv.first.c_str(),
                  kv.second.stage ? 1 : 0, kv.second.tx, kv.second.ms);
    r += line;
  }
  for (const auto &kv : ctx->ftune) {
    if (kv.second.report.empty()) continue;
    r += "fields[" + kv.first + "]: build+x=" + (kv.second.fused ? "fused" : "separate") +
         " y=" + form_name(kv.second.form[1]) + " z=" + form_name(kv.second.form[2]) + " (" + kv.second.report + ")\n";
  }
  if (buf && len) {
    std::strncpy(buf, r.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return CYR_OK;
}

int cyr_device_errors(uint32_t *count) {
  if (!count) return fail(CYR_ERR_ARGUMENT, "count pointer is null");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  *count = 0;
  if (!ctx->main.errors.ptr) return CYR_OK;
  CYR_CUDA(cudaDeviceSynchronize());
  unsigned h = 0;
  CYR_CUDA(cudaMemcpy(&h, ctx->main.errors.ptr, sizeof h, cudaMemcpyDeviceToHost));
  *count = h;
  return CYR_OK;
}

int cyr_release_scratch(void) {
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  CYR_CUDA(cudaDeviceSynchronize());
  ctx->main.release();
  ctx->vox_in.release();
  ctx->out_in.release();
  for (DeviceBuffer *b : {&ctx->f64.spec, &ctx->f64.images, &ctx->f64.avg, &ctx->f64.params, &ctx->f64.params64,
                          &ctx->f64.vox, &ctx->f64.out})
    b->release();
  return CYR_OK;
}

int cyr_simulate_device(const cyr_options *opt, const float *optical, const void *d_voxels, float *d_projection,
                        void *stream) {
  if (!d_voxels || !d_projection) return fail(CYR_ERR_ARGUMENT, "device pointer is null");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  return run_request(*ctx, ctx->main, opt, optical, static_cast<const float4 *>(d_voxels), d_projection,
                     static_cast<cudaStream_t>(stream));
}

static int cuda_main_impl(const cyr_options *opt, const float *optical, const float *voxels, float *projection,
                          bool streams_variant) {
  if (!voxels || !projection) return fail(CYR_ERR_ARGUMENT, "host pointer is null");
  CYR_TRY(validate(opt));
  cyr_options o = *opt;
  if (streams_variant) o.algorithm = 1;
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  const size_t nvox = size_t(o.nx) * o.ny * o.nz;
  const size_t vox_bytes = nvox * o.num_material * sizeof(float4);
  const uint32_t nk = (o.case_type == 0 && (o.num_k == 0 || !o.k_vectors)) ? 1u : o.num_k;
  const size_t out_bytes = size_t(o.num_energies) * nk * o.nx * o.ny * sizeof(float);
  CYR_TRY(ctx->vox_in.ensure(vox_bytes));
  CYR_TRY(ctx->out_in.ensure(out_bytes));
  if (!ctx->main_stream) CYR_CUDA(cudaStreamCreateWithFlags(&ctx->main_stream, cudaStreamNonBlocking));
  if (!ctx->copy_stream) CYR_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  cudaStream_t st = ctx->main_stream, cs = ctx->copy_stream;
  int rc = CYR_OK;
  do {
    // the morphology is uploaded by run_request, overlapped with the field transform (FIELDS)
    RunMode mode;
    mode.host_vox = voxels;
    mode.copy_stream = cs;
    mode.event_pool = &ctx->slab_events;
    rc = run_request(*ctx, ctx->main, &o, optical, ctx->vox_in.as<float4>(), ctx->out_in.as<float>(), st, mode);
    if (rc != CYR_OK) break;
    if (cudaMemcpyAsync(projection, ctx->out_in.ptr, out_bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "projection download failed: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "simulation failed: %s", cudaGetErrorString(e));
      break;
    }
    unsigned errs = 0;
    if (cudaMemcpy(&errs, ctx->main.errors.ptr, sizeof errs, cudaMemcpyDeviceToHost) == cudaSuccess && errs != 0)
      rc = fail(CYR_ERR_CUDA, "%u detector pixels needed z planes outside the kept range", errs);
    if (ctx->tma_error && cudaMemcpy(&errs, ctx->tma_error, sizeof errs, cudaMemcpyDeviceToHost) == cudaSuccess &&
        errs != 0)
      rc = fail(CYR_ERR_CUDA, "an FFT tile copy did not complete within its wait limit");
  } while (false);
  cudaStreamSynchronize(cs);
  cudaStreamSynchronize(st);
  return rc;
}

int cyr_cuda_main(const cyr_options *opt, const float *optical, const float *voxels, float *projection) {
  return cuda_main_impl(opt, optical, voxels, projection, false);
}

int cyr_cuda_main_streams(const cyr_options *opt, const float *optical, const float *voxels, float *projection) {
  return cuda_main_impl(opt, optical, voxels, projection, true);
}

int cyr_compute_polarization(const cyr_options *opt, const float *optical, const float *voxels, float eangle,
                             uint32_t energy_id, float *px, float *py, float *pz) {
  if (!voxels || !px || !py || !pz) return fail(CYR_ERR_ARGUMENT, "host pointer is null");
  Plan pl;
  CYR_TRY(make_plan(opt, optical, pl));
  if (opt->case_type != 0) return fail(CYR_ERR_UNSUPPORTED, "only implemented for case type 0 (as the reference)");
  if (energy_id >= pl.ne) return fail(CYR_ERR_ARGUMENT, "energy id out of range");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  CYR_TRY(setup_attrs(*ctx));
  CYR_TRY(ctx->main.init());  // the scratch's completion event (this may be the process's first call)
  const size_t vox_bytes = pl.nvox * pl.nmat * sizeof(float4);
  CYR_TRY(ctx->vox_in.ensure(vox_bytes));
  CYR_TRY(ctx->main.spec.ensure(3 * pl.nvox * sizeof(float2)));
  CYR_TRY(ctx->main.params.ensure(pl.arena.size()));
  cudaStream_t st = nullptr;
  CYR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = CYR_OK;
  do {
    if (cudaStreamWaitEvent(st, ctx->main.last_use, 0) != cudaSuccess ||
        cudaMemcpyAsync(ctx->main.params.ptr, pl.arena.data(), pl.arena.size(), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(ctx->vox_in.ptr, voxels, vox_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "polarization upload failed: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const unsigned char *dp = ctx->main.params.as<unsigned char>();
    BuildParams bp{};
    bp.vox = ctx->vox_in.as<float4>();
    bp.nx = pl.nx, bp.ny = pl.ny, bp.nz = pl.nz, bp.nmat = pl.nmat;
    bp.nvox = pl.nvox;
    bp.morphology = opt->morphology_type;
    bp.mode = 1;
    bp.nvol = 3;
    bp.out = ctx->main.spec.as<float2>();
    bp.material_frame = pl.material_frame ? 1u : 0u;
    // the debug path rotates E by EAngle radians about k (src/cudaMain.cu:1716-1721)
    const Mat3f R = e_rotation(pl.frames[0], eangle);
    for (int c = 0; c < 3; ++c) bp.E[c] = R(c, 0);
    std::memcpy(bp.Rm, R.m, sizeof bp.Rm);
    if (opt->windowing == 1) {  // the debug path windows whatever the algorithm (src/cudaMain.cu:1722-1725)
      bp.hann_x = reinterpret_cast<const float *>(dp + pl.off_hx);
      bp.hann_y = reinterpret_cast<const float *>(dp + pl.off_hy);
      bp.hann_z = reinterpret_cast<const float *>(dp + pl.off_hz);
    }
    const MaterialConsts *mce = reinterpret_cast<const MaterialConsts *>(dp + pl.off_mc) + energy_id;
    const uint32_t blocks = uint32_t(std::min<size_t>((pl.nvox + 255) / 256, 65535));
    if (opt->morphology_type == 0)
      k_build<0, false><<<blocks, 256, 0, st>>>(bp, mce);
    else
      k_build<1, false><<<blocks, 256, 0, st>>>(bp, mce);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "polarization kernel launch failed: %s", cudaGetErrorString(le));
      break;
    }
    const size_t cb = pl.nvox * sizeof(float2);
    cudaMemcpyAsync(px, ctx->main.spec.as<float2>(), cb, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(py, ctx->main.spec.as<float2>() + pl.nvox, cb, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(pz, ctx->main.spec.as<float2>() + 2 * pl.nvox, cb, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ctx->main.last_use, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(CYR_ERR_CUDA, "polarization failed: %s", cudaGetErrorString(e));
  } while (false);
  cudaStreamDestroy(st);
  return rc;
}

int cyr_cuda_main_fp64(const cyr_options *opt, const double *optical, const double *voxels, double *projection) {
  if (!voxels || !projection) return fail(CYR_ERR_ARGUMENT, "host pointer is null");
  CYR_TRY(validate(opt));
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  const size_t nvox = size_t(opt->nx) * opt->ny * opt->nz;
  const size_t vox_bytes = nvox * opt->num_material * 4 * sizeof(double);
  const uint32_t nk = (opt->case_type == 0 && (opt->num_k == 0 || !opt->k_vectors)) ? 1u : opt->num_k;
  const size_t out_bytes = size_t(opt->num_energies) * nk * opt->nx * opt->ny * sizeof(double);
  CYR_TRY(ctx->f64.vox.ensure(vox_bytes));
  CYR_TRY(ctx->f64.out.ensure(out_bytes));
  cudaStream_t st = nullptr;
  CYR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = CYR_OK;
  do {
    if (cudaMemcpyAsync(ctx->f64.vox.ptr, voxels, vox_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "voxel upload failed: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    if ((rc = run_fp64(*ctx, opt, optical, ctx->f64.vox.ptr, true, ctx->f64.out.as<double>(), st)) != CYR_OK) break;
    if (cudaMemcpyAsync(projection, ctx->f64.out.ptr, out_bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "projection download failed: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(CYR_ERR_CUDA, "FP64 simulation failed: %s", cudaGetErrorString(e));
  } while (false);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return rc;
}

int cyr_simulate_device_fp64(const cyr_options *opt, const double *optical, const void *d_voxels,
                             uint32_t voxels_fp64, double *d_projection, void *stream) {
  if (!d_voxels || !d_projection) return fail(CYR_ERR_ARGUMENT, "device pointer is null");
  if (voxels_fp64 > 1) return fail(CYR_ERR_ARGUMENT, "voxels_fp64 must be 0 (float4) or 1 (double4)");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  return run_fp64(*ctx, opt, optical, d_voxels, voxels_fp64 == 1, d_projection, static_cast<cudaStream_t>(stream));
}

int cyr_compute_polarization_fp64(const cyr_options *opt, const double *optical, const double *voxels, double eangle,
                                  uint32_t energy_id, double *px, double *py, double *pz) {
  if (!voxels || !px || !py || !pz) return fail(CYR_ERR_ARGUMENT, "host pointer is null");
  if (opt && opt->case_type != 0) return fail(CYR_ERR_UNSUPPORTED, "only implemented for case type 0 (as the reference)");
  Plan pl;
  Plan64 p64;
  // the debug path windows whatever the algorithm (src/cudaMain.cu:1722-1725)
  CYR_TRY(make_plan64(opt, optical, opt->windowing == 1, pl, p64));
  if (energy_id >= pl.ne) return fail(CYR_ERR_ARGUMENT, "energy id out of range");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto &f = ctx->f64;
  const size_t vox_bytes = pl.nvox * pl.nmat * 4 * sizeof(double);
  CYR_TRY(f.vox.ensure(vox_bytes));
  CYR_TRY(f.spec.ensure(3 * pl.nvox * sizeof(double2)));
  CYR_TRY(f.params64.ensure(p64.arena.size()));
  cudaStream_t st = nullptr;
  CYR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = CYR_OK;
  do {
    cudaMemcpyAsync(f.params64.ptr, p64.arena.data(), p64.arena.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(f.vox.ptr, voxels, vox_bytes, cudaMemcpyHostToDevice, st);
    const unsigned char *dq = f.params64.as<unsigned char>();
    Build64Params bp{};
    bp.vox = f.vox.ptr;
    bp.vox_fp64 = 1;
    bp.nx = pl.nx, bp.ny = pl.ny, bp.nz = pl.nz, bp.nmat = pl.nmat;
    bp.nvox = pl.nvox;
    bp.morphology = opt->morphology_type;
    bp.mode = 1;
    bp.nvol = 3;
    bp.material_frame = pl.material_frame ? 1u : 0u;
    // the debug path rotates E by EAngle radians about k (src/cudaMain.cu:1716-1721)
    const Mat3f R = e_rotation(pl.frames[0], float(eangle));
    for (int c = 0; c < 3; ++c) bp.E[c] = double(R.m[c * 3 + 0]);
    for (int i = 0; i < 9; ++i) bp.R[i] = double(R.m[i]);
    if (opt->windowing == 1) {
      bp.hann_x = reinterpret_cast<const double *>(dq + p64.off_hx);
      bp.hann_y = reinterpret_cast<const double *>(dq + p64.off_hy);
      bp.hann_z = reinterpret_cast<const double *>(dq + p64.off_hz);
    }
    bp.out = f.spec.as<double2>();
    const unsigned blocks = unsigned(std::min<size_t>((pl.nvox + 255) / 256, 65535));
    k64_build<<<blocks, 256, 0, st>>>(bp, reinterpret_cast<const Mat64 *>(dq + p64.off_mat) + energy_id);
    if (cudaGetLastError() != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "polarization kernel launch failed");
      break;
    }
    const size_t cb = pl.nvox * sizeof(double2);
    cudaMemcpyAsync(px, f.spec.as<double2>(), cb, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(py, f.spec.as<double2>() + pl.nvox, cb, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(pz, f.spec.as<double2>() + 2 * pl.nvox, cb, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(CYR_ERR_CUDA, "FP64 polarization failed: %s", cudaGetErrorString(e));
  } while (false);
  cudaStreamDestroy(st);
  return rc;
}

int cyr_profile_begin(uint32_t max_launches) {
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  Profiler &p = ctx->prof;
  std::lock_guard<std::mutex> plk(p.mu);
  const size_t want = std::max<uint32_t>(max_launches, 1);
  while (p.events.size() < 2 * want) {
    cudaEvent_t e;
    CYR_CUDA(cudaEventCreate(&e));
    p.events.push_back(e);
  }
  p.stage.assign(want, -1);
  p.count.assign(want, 1);
  p.used = 0;
  p.dropped = 0;
  p.active = true;
  return CYR_OK;
}

int cyr_profile_end(uint32_t *launches, uint32_t *calls, double *ms, uint32_t nstages, uint32_t *dropped) {
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  Profiler &p = ctx->prof;
  size_t used = 0;
  {
    std::lock_guard<std::mutex> plk(p.mu);
    p.active = false;
    used = p.used;
  }
  for (uint32_t i = 0; i < nstages; ++i) {
    if (launches) launches[i] = 0;
    if (calls) calls[i] = 0;
    if (ms) ms[i] = 0.0;
  }
  for (size_t i = 0; i < used; ++i) {
    float t = 0.f;
    CYR_CUDA(cudaEventSynchronize(p.events[2 * i + 1]));
    // a pair whose closing event was not recorded yet (a launch of another
    // thread still in flight when profiling stopped) is dropped
    if (cudaEventElapsedTime(&t, p.events[2 * i], p.events[2 * i + 1]) != cudaSuccess) {
      cudaGetLastError();
      p.dropped += size_t(p.count[i]);
      continue;
    }
    const int s = p.stage[i];
    if (s >= 0 && uint32_t(s) < nstages) {
      if (launches) launches[s] += uint32_t(p.count[i]);
      if (calls) calls[s] += 1;
      if (ms) ms[s] += t;
    }
  }
  std::lock_guard<std::mutex> plk(p.mu);
  if (dropped) *dropped = uint32_t(p.dropped);
  p.used = 0;
  return CYR_OK;
}

const char *cyr_stage_name(uint32_t stage) { return stage < kNumStages ? kStageNames[stage] : ""; }

uint32_t cyr_num_stages(void) { return kNumStages; }

int cyr_fft3d_device(void *d_data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count, void *stream) {
  if (!d_data || nx < 1 || ny < 1 || nz < 1 || count < 1) return fail(CYR_ERR_ARGUMENT, "bad FFT arguments");
  if (size_t(nx) * ny * nz > kMaxVolumeVoxels)
    return fail(CYR_ERR_ARGUMENT, "volume of %u x %u x %u elements exceeds the limit of 2^32 - 1", nx, ny, nz);
  for (uint32_t n : {nx, ny, nz}) {
    const char *why = "";
    if (!fft_length_ok(n, &why)) return fail(CYR_ERR_UNSUPPORTED, "FFT length %u %s", n, why);
  }
  if (count > 65535) return fail(CYR_ERR_ARGUMENT, "too many volumes in one call");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  CYR_TRY(setup_attrs(*ctx));
  return fft3d(*ctx, static_cast<float2 *>(d_data), nx, ny, nz, count, static_cast<cudaStream_t>(stream));
}

int cyr_selftest_wait_limit(int *timed_out) {
  if (!timed_out) return fail(CYR_ERR_ARGUMENT, "timed_out pointer is null");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(ctx->mu);
  CYR_TRY(setup_attrs(*ctx));
  if (!ctx->encode_tiled) return fail(CYR_ERR_UNSUPPORTED, "no tensor-map encoder in this driver");
  // one 32-column x 256-line tile; its copies deliver 16 bytes fewer than the
  // barrier expects, so the phase never completes and every wait runs out
  constexpr uint32_t nx = 32, ny = 256;
  const float2 *tw = nullptr;
  CYR_TRY(get_twiddles(*ctx, ny, &tw));
  float2 *d = nullptr;
  CYR_CUDA(cudaMalloc(&d, size_t(nx) * ny * sizeof(float2)));
  int rc = CYR_OK;
  do {
    CUtensorMap map;
    if ((rc = encode_cols_map(*ctx, &map, d, nx, ny, 1, 1, size_t(nx) * ny, 1, ny)) != CYR_OK) break;
    ColTmaParams tp{};
    tp.nxt = 1, tp.others = 1, tp.ntiles = 1, tp.axis = 1;
    tp.tw = tw;
    tp.error = ctx->tma_error;
    tp.poll_limit = 1u << 16;  // far longer than the 64 KB copies take to land
    tp.extra_tx = 16;
    if (cudaMemset(d, 0, size_t(nx) * ny * sizeof(float2)) != cudaSuccess ||
        cudaMemset(ctx->tma_error, 0, sizeof(unsigned)) != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "self-test setup failed");
      break;
    }
    k_fft_cols_tma_ws<8, 2, 3><<<1, 17 * 32, cols_tma_ws_smem<8, 2, 3>()>>>(map, map, tp);
    const cudaError_t e = cudaDeviceSynchronize();
    unsigned flag = 0;
    if (e != cudaSuccess || cudaMemcpy(&flag, ctx->tma_error, sizeof flag, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = fail(CYR_ERR_CUDA, "self-test kernel failed: %s", cudaGetErrorString(e));
      break;
    }
    *timed_out = (flag & 1u) != 0;
    if (cudaMemset(ctx->tma_error, 0, sizeof(unsigned)) != cudaSuccess) rc = fail(CYR_ERR_CUDA, "flag reset failed");
    if ((flag & 2u) != 0)
      rc = fail(CYR_ERR_TIMEOUT, "the copies of the timed-out tile did not land within the drain's wait limit");
  } while (false);
  cudaFree(d);
  return rc;
}

int cyr_warp_affine_device(const float *d_src, float *d_dst, int width, int height, const double *coeffs,
                           void *stream) {
  if (!d_src || !d_dst || !coeffs || width < 1 || height < 1) return fail(CYR_ERR_ARGUMENT, "bad warp arguments");
  const double c[2][3] = {{coeffs[0], coeffs[1], coeffs[2]}, {coeffs[3], coeffs[4], coeffs[5]}};
  const double det = c[0][0] * c[1][1] - c[0][1] * c[1][0];
  if (det == 0.0 || !std::isfinite(det)) return fail(CYR_ERR_ARGUMENT, "singular warp matrix");
  const WarpInverse w = warp_inverse(c);
  const size_t n = size_t(width) * height;
  k_warp<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_src, d_dst, width, height, WarpCoef{w.a00, w.a01, w.a02, w.a10, w.a11, w.a12});
  CYR_CUDA(cudaGetLastError());
  return CYR_OK;
}

}  // extern "C"


// ---------------------------------------------------------------------------
// Serving C ABI
// ---------------------------------------------------------------------------
struct cyr_server {
  cyr::Server *impl;
};

extern "C" {

int cyr_server_create(uint32_t slots, size_t hbm_budget, uint32_t flags, cyr_server **out) {
  if (!out) return fail(CYR_ERR_ARGUMENT, "out pointer is null");
  if (slots < 1 || slots > 64) return fail(CYR_ERR_ARGUMENT, "slots must be in [1, 64]");
  DeviceContext *ctx = nullptr;
  CYR_TRY(get_context(&ctx));
  CYR_TRY(setup_attrs(*ctx));
  std::unique_ptr<Server> S(new Server);
  S->ctx = ctx;
  S->device = ctx->device;
  S->graphs = (flags & CYR_SERVER_GRAPHS) != 0;
  S->groups = (flags & CYR_SERVER_GROUPS) != 0;
  if (hbm_budget == 0) {
    size_t free_b = 0, total_b = 0;
    CYR_CUDA(cudaMemGetInfo(&free_b, &total_b));
    hbm_budget = free_b / 100 * 85;
  }
  S->budget = hbm_budget;
  for (uint32_t i = 0; i < slots; ++i) {
    std::unique_ptr<Slot> sl(new Slot);
    CYR_CUDA(cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking));
    CYR_CUDA(cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming));
    CYR_CUDA(cudaMallocHost(&sl->host_errors, sizeof(unsigned)));
    *sl->host_errors = 0;
    sl->sc.bind(sl->stream);
    sl->vox.stream = sl->out.stream = sl->stream;
    sl->vox.generation = sl->out.generation = &sl->sc.generation;
    CYR_TRY(sl->sc.init());
    S->slots.push_back(std::move(sl));
  }
  Server *raw = S.release();
  raw->worker = std::thread(server_loop, raw);
  *out = new cyr_server{raw};
  return CYR_OK;
}

int cyr_server_submit(cyr_server *s, const cyr_options *opt, const float *optical, const void *voxels,
                      float *projection, uint32_t device_buffers, uint64_t *id) {
  if (!s || !id || !optical || !voxels || !projection) return fail(CYR_ERR_ARGUMENT, "null argument");
  CYR_TRY(validate(opt));
  auto r = std::make_shared<ServerRequest>();
  r->opt = *opt;
  r->energies.assign(opt->energies, opt->energies + opt->num_energies);
  r->opt.energies = r->energies.data();
  if (opt->k_vectors && opt->num_k) {
    r->kvecs.assign(opt->k_vectors, opt->k_vectors + size_t(3) * opt->num_k);
    r->opt.k_vectors = r->kvecs.data();
  }
  r->optical.assign(optical, optical + size_t(opt->num_energies) * opt->num_material * 4);
  const uint32_t nk = (opt->case_type == 0 && (opt->num_k == 0 || !opt->k_vectors)) ? 1u : opt->num_k;
  r->vox_bytes = size_t(opt->nx) * opt->ny * opt->nz * opt->num_material * sizeof(float4);
  r->out_bytes = size_t(opt->num_energies) * nk * opt->nx * opt->ny * sizeof(float);
  if (device_buffers) {
    r->d_vox = static_cast<const float4 *>(voxels);
    r->d_out = projection;
  } else {
    r->h_vox = static_cast<const float *>(voxels);
    r->h_out = projection;
  }
  Server &S = *s->impl;
  CYR_TRY(plan_request(*r, staged_request(S, *r)));
  {
    std::lock_guard<std::mutex> lk(S.mu);
    r->id = S.next_id++;
    r->t_submit = Clock::now();
    S.requests[r->id] = r;
    S.queue.push_back(r);
  }
  S.cv_work.notify_one();
  *id = r->id;
  return CYR_OK;
}

int cyr_server_poll(cyr_server *s, uint64_t id, int *done) {
  if (!s || !done) return fail(CYR_ERR_ARGUMENT, "null argument");
  Server &S = *s->impl;
  std::lock_guard<std::mutex> lk(S.mu);
  auto it = S.requests.find(id);
  if (it == S.requests.end()) return fail(CYR_ERR_ARGUMENT, "unknown request id %llu", (unsigned long long)id);
  *done = it->second->status >= 0 ? 1 : 0;
  return CYR_OK;
}

int cyr_server_wait(cyr_server *s, uint64_t id, double *latency_s, double *queue_s) {
  if (!s) return fail(CYR_ERR_ARGUMENT, "null server");
  Server &S = *s->impl;
  std::unique_lock<std::mutex> lk(S.mu);
  auto it = S.requests.find(id);
  if (it == S.requests.end()) return fail(CYR_ERR_ARGUMENT, "unknown request id %llu", (unsigned long long)id);
  std::shared_ptr<ServerRequest> r = it->second;
  S.cv_done.wait(lk, [&] { return r->status >= 0; });
  S.requests.erase(it);
  if (latency_s) *latency_s = std::chrono::duration<double>(r->t_done - r->t_submit).count();
  if (queue_s) *queue_s = std::chrono::duration<double>(r->t_start - r->t_submit).count();
  if (r->status != CYR_OK) return fail(r->status, "request %llu: %s", (unsigned long long)id, r->error.c_str());
  return CYR_OK;
}

int cyr_server_stats(cyr_server *s, uint64_t *completed, uint64_t *failed, uint64_t *graph_replays,
                     uint64_t *graph_captures) {
  if (!s) return fail(CYR_ERR_ARGUMENT, "null server");
  Server &S = *s->impl;
  if (completed) *completed = S.completed;
  if (failed) *failed = S.failed;
  if (graph_replays) *graph_replays = S.replays;
  if (graph_captures) *graph_captures = S.captures;
  return CYR_OK;
}

int cyr_server_group_stats(cyr_server *s, uint64_t *group_runs, uint64_t *grouped_requests) {
  if (!s) return fail(CYR_ERR_ARGUMENT, "null server");
  Server &S = *s->impl;
  if (group_runs) *group_runs = S.group_runs;
  if (grouped_requests) *grouped_requests = S.grouped;
  return CYR_OK;
}

int cyr_server_destroy(cyr_server *s) {
  if (!s) return CYR_OK;
  const int rc = server_destroy(s->impl);
  delete s;
  return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free FFT entry point.
//
// Some callers cannot allocate device memory at the point where they need the
// transform: code running inside a memory pool or arena that owns every byte
// of the device and forbids cudaMalloc/cudaFree, or a host that must not call
// allocating routines on a latency-critical path.  cyr_fft3d_device
// allocates its twiddle tables (cudaMalloc, once per length); this variant
// keeps them in a fixed file-scope device array instead.  The array is part of
// the library image: every GPU that loads the library holds its
// kStaticTwiddleBytes until the process exits.
// ---------------------------------------------------------------------------
namespace {
constexpr uint32_t kStaticMaxLength = 4096;  // per axis
constexpr size_t kStaticTwiddleBytes = size_t(3) * kStaticMaxLength * sizeof(float2);  // 96 KiB
__device__ __align__(256) float2 g_static_twiddles[3 * kStaticMaxLength];
static_assert(sizeof(g_static_twiddles) == kStaticTwiddleBytes, "static twiddle array size");

struct StaticTwiddleState {
  float2 *dev_ptr = nullptr;  // device address of g_static_twiddles on this device
  bool attrs = false;
};
std::mutex g_static_mu;
std::map<int, StaticTwiddleState> g_static_state;
}  // namespace

// W_n^m = exp(-2 pi i m / n) for the three axes, formed with sincospi in double
// and rounded to float; axis a's table starts at a * kStaticMaxLength.
__global__ void k_static_twiddles(float2 *tab, uint32_t nx, uint32_t ny, uint32_t nz) {
  const uint32_t axis = blockIdx.y;
  const uint32_t n = axis == 0 ? nx : axis == 1 ? ny : nz;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double sn, cs;
    sincospi(-2.0 * double(m) / double(n), &sn, &cs);
    tab[size_t(axis) * kStaticMaxLength + m] = make_float2(float(cs), float(sn));
  }
}

extern "C" int cyr_fft3d_device_static(void *d_data, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t count,
                                       void *stream) {
  if (!d_data || nx < 1 || ny < 1 || nz < 1 || count < 1) return fail(CYR_ERR_ARGUMENT, "bad FFT arguments");
  if (nx > kStaticMaxLength || ny > kStaticMaxLength || nz > kStaticMaxLength)
    return fail(CYR_ERR_ARGUMENT, "cyr_fft3d_device_static: every axis must be at most %u long (got %u x %u x %u)",
                kStaticMaxLength, nx, ny, nz);
  if (size_t(nx) * ny * nz > kMaxVolumeVoxels)
    return fail(CYR_ERR_ARGUMENT, "volume of %u x %u x %u elements exceeds the limit of 2^32 - 1", nx, ny, nz);
  if (count > 65535) return fail(CYR_ERR_ARGUMENT, "too many volumes in one call");
  std::vector<uint32_t> r;
  for (uint32_t n : {nx, ny, nz})
    if (n > 1 && !factorize(n, r)) return fail(CYR_ERR_UNSUPPORTED, "FFT length %u has a prime factor above 7", n);
  int dev = 0;
  CYR_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_static_mu);
  StaticTwiddleState &stt = g_static_state[dev];
  if (!stt.dev_ptr) {
    // one-time set-up on this device (must precede any stream capture): the
    // host-side name g_static_twiddles is not a device address
    void *p = nullptr;
    CYR_CUDA(cudaGetSymbolAddress(&p, g_static_twiddles));
    stt.dev_ptr = static_cast<float2 *>(p);
  }
  if (!stt.attrs) {
    // the only kernel this entry point launches with large dynamic shared memory
    const int smem = int(kFftSmemBudget);
    CYR_CUDA(cudaFuncSetAttribute(k_fft_pass<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CYR_CUDA(cudaFuncSetAttribute(k_fft_pass<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CYR_CUDA(cudaFuncSetAttribute(k_fft_pass<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    stt.attrs = true;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // The tables of this call replace the previous call's contents: a kernel on
  // `st` writes every entry the passes read, so nothing relies on zeros and no
  // host copy is involved.  Calls whose work overlaps on the GPU share the
  // array and race.
  k_static_twiddles<<<dim3(16, 3), 256, 0, st>>>(stt.dev_ptr, nx, ny, nz);
  CYR_CUDA(cudaGetLastError());
  const uint32_t dims[3] = {nx, ny, nz};
  const size_t nvox = size_t(nx) * ny * nz;
  for (int axis = 0; axis < 3; ++axis) {
    const uint32_t n = dims[axis];
    if (n == 1) continue;
    FftPassParams p{};
    p.data = static_cast<float2 *>(d_data);
    p.nx = nx, p.ny = ny, p.nz = nz;
    p.nvox = nvox;
    factorize(n, r);
    p.ax.n = n;
    p.ax.log2n = 0;
    if ((n & (n - 1)) == 0)
      while ((1u << p.ax.log2n) < n) ++p.ax.log2n;
    p.ax.nstages = uint32_t(r.size());
    p.ax.radix_code = 0;
    for (size_t i = 0; i < r.size(); ++i) p.ax.radix_code |= uint64_t(r[i]) << (4 * i);
    p.ax.tw = stt.dev_ptr + size_t(axis) * kStaticMaxLength;
    p.tx = fft_lines_per_block(n);
    const size_t smem = (size_t(2) * n * (p.tx + 1) + n) * sizeof(float2);
    if (smem > kFftSmemBudget) return fail(CYR_ERR_UNSUPPORTED, "FFT length %u too large for one block", n);
    const uint32_t tiles =
        axis == 0 ? (ny * nz + p.tx - 1) / p.tx : ((nx + p.tx - 1) / p.tx) * (axis == 1 ? nz : ny);
    const dim3 grid(tiles, count);
    if (axis == 0) k_fft_pass<0><<<grid, kFftThreads, smem, st>>>(p);
    if (axis == 1) k_fft_pass<1><<<grid, kFftThreads, smem, st>>>(p);
    if (axis == 2) k_fft_pass<2><<<grid, kFftThreads, smem, st>>>(p);
    CYR_CUDA(cudaGetLastError());
  }
  return CYR_OK;
}
