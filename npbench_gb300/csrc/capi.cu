// Library-wide C ABI helpers: version, status strings, per-thread last error.
#include <atomic>
#include <cstdarg>
#include <cstdio>

#include <mutex>

#include "npbgb_common.cuh"
#include "tma.cuh"

namespace npbgb {

static thread_local char g_last_error[512] = "";

int64_t g_cfg_f64_emulation = 1;
int64_t g_cfg_heat_chunk = 0;
int64_t g_cfg_heat_tma = 1;
int64_t g_cfg_heat_rows = 0;     // 0: per-dtype default
int64_t g_cfg_heat_hw_rows = -1; // -1: per-kernel default
int64_t g_cfg_f64_cvt = 0;
int64_t g_cfg_jacobi_hw_warps = -1;  // -1: default
int64_t g_cfg_batch_ctas_per_sm = 5;  // the persistent form takes 3 for 3 and more
int64_t g_cfg_jacobi_chunk = 0;
int64_t g_cfg_pdl = 1;
int64_t g_cfg_batch_mode = 0;
int64_t g_cfg_hdiff_emu = -1;  // -1: default mask
int64_t g_cfg_jacobi1d_ctas = 0;   // 0: default
int64_t g_cfg_jacobi1d_depth = 0;  // 0: default
int64_t g_cfg_heat_tb = 0;         // binary32 Heat-3D half-sweeps per launch (0: by size)
int64_t g_cfg_heat_tb_chunk = 0;   // 0: automatic
int64_t g_cfg_jacobi_bands = 0;    // 0, 1: chained launches; 2: bands whenever they fit
int64_t g_cfg_jacobi_bands_warps = 0;  // 0: by the grid's width
int64_t g_cfg_heat_stages = 0;         // 0: automatic (8)
int64_t g_cfg_heat_mad_rows = 0;
int64_t g_cfg_queue_whole_cells = 65536;
int64_t g_cfg_jacobi_fx_mul = 1;
int64_t g_cfg_jacobi_fx_adds = 0;
int64_t g_cfg_jacobi_tma = 1;
int64_t g_cfg_batch_tma = 0;

namespace {
std::atomic<int64_t> g_launches{0};
}  // namespace

int64_t add_launches(int64_t n) { return g_launches.fetch_add(n, std::memory_order_relaxed) + n; }
int64_t jacobi1d_effective_depth();  // jacobi1d.cu
int64_t jacobi1d_effective_ctas();

uint32_t take_heat_device_error();
uint32_t take_batch_device_error();
uint32_t take_cfd_device_error();
uint32_t take_queue_device_error();
uint32_t take_heat_tb_device_error();
uint32_t take_jacobi_bands_device_error();
uint32_t take_jacobi_tma_device_error();
int32_t launch_wait_timeout_selftest(uint64_t limit_ns, cudaStream_t st);

int32_t set_error(int32_t code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

namespace tma {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

cudaError_t encode_3d(CUtensorMap* map, int esize, const void* base, const uint64_t dims[3],
                      const uint32_t box[3]) {
  if ((esize != 4 && esize != 8) || !base) return cudaErrorInvalidValue;
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0) return cudaErrorInvalidValue;
  const uint64_t strides[2] = {dims[0] * esize, dims[0] * dims[1] * esize};
  if (strides[0] % 16 != 0 || strides[1] % 16 != 0) return cudaErrorInvalidValue;
  if ((box[0] * esize) % 16 != 0) return cudaErrorInvalidValue;
  for (int d = 0; d < 3; ++d) {
    if (box[d] == 0 || box[d] > 256) return cudaErrorInvalidValue;
    if (dims[d] == 0 || dims[d] > (uint64_t(1) << 32)) return cudaErrorInvalidValue;
  }
  if (strides[1] >= (uint64_t(1) << 40)) return cudaErrorInvalidValue;
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(map, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                        3, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace tma

}  // namespace npbgb

extern "C" {

const char* npbgb_version(void) { return "npbgb 0.1.0 sm_103a"; }

const char* npbgb_last_error(void) { return npbgb::g_last_error; }

const char* npbgb_status_string(int32_t status) {
  switch (status) {
    case NPBGB_OK: return "ok";
    case NPBGB_ERR_ARG: return "invalid argument";
    case NPBGB_ERR_DTYPE: return "unsupported dtype";
    case NPBGB_ERR_CUDA: return "CUDA error";
    case NPBGB_ERR_TIMEOUT: return "device wait timed out";
    case NPBGB_ERR_NOMEM: return "capacity or budget exceeded";
    case NPBGB_ERR_STATE: return "invalid state";
    default: return "unknown status";
  }
}

int32_t npbgb_set_config(int32_t key, int64_t value) {
  using namespace npbgb;
  switch (key) {
    case NPBGB_CFG_F64_EMULATION:
      if (value != 0 && value != 1) return set_error(NPBGB_ERR_ARG, "f64 emulation: 0 or 1");
      g_cfg_f64_emulation = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_CHUNK:
      if (value < 0 || value > (1 << 20)) return set_error(NPBGB_ERR_ARG, "heat chunk out of range");
      g_cfg_heat_chunk = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_TMA:
      if (value != 0 && value != 1) return set_error(NPBGB_ERR_ARG, "heat tma: 0 or 1");
      g_cfg_heat_tma = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_CHUNK:
      if (value < 0 || value > (1 << 20)) return set_error(NPBGB_ERR_ARG, "jacobi chunk out of range");
      g_cfg_jacobi_chunk = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_ROWS:
      if (value != 0 && value != 1 && value != 2 && value != 4)
        return set_error(NPBGB_ERR_ARG, "heat rows: 0 (automatic), 1, 2 or 4");
      g_cfg_heat_rows = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_HW_ROWS:
      if (value < -1 || value > 32) return set_error(NPBGB_ERR_ARG, "heat hw rows: -1 (automatic) .. 32");
      g_cfg_heat_hw_rows = value;
      return NPBGB_OK;
    case NPBGB_CFG_F64_CVT:
      if (value != 0 && value != 1) return set_error(NPBGB_ERR_ARG, "f64 cvt: 0 or 1");
      g_cfg_f64_cvt = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_HW_WARPS:
      if (value < -1 || value > 8) return set_error(NPBGB_ERR_ARG, "jacobi hw warps: -1 .. 8");
      g_cfg_jacobi_hw_warps = value;
      return NPBGB_OK;
    case NPBGB_CFG_BATCH_CTAS_PER_SM:
      if (value < 2 || value > 5) return set_error(NPBGB_ERR_ARG, "batch CTAs per SM: 2 .. 5");
      g_cfg_batch_ctas_per_sm = value;
      return NPBGB_OK;
    case NPBGB_CFG_PDL:
      if (value != 0 && value != 1) return set_error(NPBGB_ERR_ARG, "PDL: 0 or 1");
      g_cfg_pdl = value;
      return NPBGB_OK;
    case NPBGB_CFG_BATCH_MODE:
      if (value < 0 || value > 3) return set_error(NPBGB_ERR_ARG, "batch mode: 0, 1, 2 or 3");
      g_cfg_batch_mode = value;
      return NPBGB_OK;
    case NPBGB_CFG_HDIFF_EMU:
      if (value < -1 || value > 0xffffff) return set_error(NPBGB_ERR_ARG, "hdiff emu: -1 .. 0xffffff");
      g_cfg_hdiff_emu = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI1D_CTAS:
      if (value < 0 || value > 8) return set_error(NPBGB_ERR_ARG, "jacobi1d CTAs per SM: 0 .. 8");
      g_cfg_jacobi1d_ctas = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_TB:
      if (value < 0 || value > 2) return set_error(NPBGB_ERR_ARG, "heat TB: 0, 1 or 2");
      g_cfg_heat_tb = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_TB_CHUNK:
      if (value < 0 || value > 65535) return set_error(NPBGB_ERR_ARG, "heat TB chunk: 0 .. 65535");
      g_cfg_heat_tb_chunk = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_BANDS:
      if (value < 0 || value > 2) return set_error(NPBGB_ERR_ARG, "jacobi bands: 0, 1 or 2");
      g_cfg_jacobi_bands = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_FX_ADDS:
      if (value < 0 || value > 3) return set_error(NPBGB_ERR_ARG, "jacobi fx adds: 0 .. 3");
      g_cfg_jacobi_fx_adds = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_TMA:
      if (value < 0 || value > 2) return set_error(NPBGB_ERR_ARG, "jacobi tma: 0, 1 or 2");
      g_cfg_jacobi_tma = value;
      return NPBGB_OK;
    case NPBGB_CFG_BATCH_TMA:
      if (value != 0 && value != 1) return set_error(NPBGB_ERR_ARG, "batch tma: 0 or 1");
      g_cfg_batch_tma = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_FX_MUL:
      if (value < 0 || value > 2) return set_error(NPBGB_ERR_ARG, "jacobi fx mul: 0, 1 or 2");
      g_cfg_jacobi_fx_mul = value;
      return NPBGB_OK;
    case NPBGB_CFG_QUEUE_WHOLE_CELLS:
      if (value < 0 || value > (int64_t(1) << 40))
        return set_error(NPBGB_ERR_ARG, "queue whole cells: 0 .. 2^40");
      g_cfg_queue_whole_cells = value;
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_MAD_ROWS:
      if (value < 0 || value > 64) return set_error(NPBGB_ERR_ARG, "heat mad rows: 0 .. 64");
      g_cfg_heat_mad_rows = value;
      return NPBGB_OK;
    case NPBGB_CFG_LAUNCHES:
      if (value != 0) return set_error(NPBGB_ERR_ARG, "launch count: only 0 (reset) may be set");
      g_launches.store(0, std::memory_order_relaxed);
      return NPBGB_OK;
    case NPBGB_CFG_HEAT_STAGES:
      if (value != 0 && value != 4 && value != 6 && value != 8)
        return set_error(NPBGB_ERR_ARG, "heat stages: 0 (automatic), 4, 6 or 8");
      g_cfg_heat_stages = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI_BANDS_WARPS:
      if (value != 0 && value != 8 && value != 16 && value != 32)
        return set_error(NPBGB_ERR_ARG, "jacobi bands warps: 0, 8, 16 or 32");
      g_cfg_jacobi_bands_warps = value;
      return NPBGB_OK;
    case NPBGB_CFG_JACOBI1D_DEPTH:
      if (value < 0 || value > 64 || (value & 1))
        return set_error(NPBGB_ERR_ARG, "jacobi1d depth: 0 or an even number up to 64");
      g_cfg_jacobi1d_depth = value;
      return NPBGB_OK;
    default:
      return set_error(NPBGB_ERR_ARG, "unknown config key %d", key);
  }
}

int32_t npbgb_get_config(int32_t key, int64_t* value) {
  using namespace npbgb;
  if (!value) return set_error(NPBGB_ERR_ARG, "null output");
  switch (key) {
    case NPBGB_CFG_F64_EMULATION: *value = g_cfg_f64_emulation; return NPBGB_OK;
    case NPBGB_CFG_HEAT_CHUNK: *value = g_cfg_heat_chunk; return NPBGB_OK;
    case NPBGB_CFG_HEAT_TMA: *value = g_cfg_heat_tma; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_CHUNK: *value = g_cfg_jacobi_chunk; return NPBGB_OK;
    case NPBGB_CFG_HEAT_ROWS: *value = g_cfg_heat_rows; return NPBGB_OK;
    case NPBGB_CFG_HEAT_HW_ROWS: *value = g_cfg_heat_hw_rows; return NPBGB_OK;
    case NPBGB_CFG_F64_CVT: *value = g_cfg_f64_cvt; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_HW_WARPS: *value = g_cfg_jacobi_hw_warps; return NPBGB_OK;
    case NPBGB_CFG_BATCH_CTAS_PER_SM: *value = g_cfg_batch_ctas_per_sm; return NPBGB_OK;
    case NPBGB_CFG_PDL: *value = g_cfg_pdl; return NPBGB_OK;
    case NPBGB_CFG_BATCH_MODE: *value = g_cfg_batch_mode; return NPBGB_OK;
    case NPBGB_CFG_HDIFF_EMU: *value = g_cfg_hdiff_emu; return NPBGB_OK;
    case NPBGB_CFG_JACOBI1D_CTAS: *value = jacobi1d_effective_ctas(); return NPBGB_OK;
    case NPBGB_CFG_JACOBI1D_DEPTH: *value = jacobi1d_effective_depth(); return NPBGB_OK;
    case NPBGB_CFG_HEAT_TB: *value = g_cfg_heat_tb; return NPBGB_OK;
    case NPBGB_CFG_HEAT_TB_CHUNK: *value = g_cfg_heat_tb_chunk; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_BANDS: *value = g_cfg_jacobi_bands; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_BANDS_WARPS: *value = g_cfg_jacobi_bands_warps; return NPBGB_OK;
    case NPBGB_CFG_HEAT_STAGES: *value = g_cfg_heat_stages; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_FX_ADDS: *value = g_cfg_jacobi_fx_adds; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_TMA: *value = g_cfg_jacobi_tma; return NPBGB_OK;
    case NPBGB_CFG_BATCH_TMA: *value = g_cfg_batch_tma; return NPBGB_OK;
    case NPBGB_CFG_JACOBI_FX_MUL: *value = g_cfg_jacobi_fx_mul; return NPBGB_OK;
    case NPBGB_CFG_QUEUE_WHOLE_CELLS: *value = g_cfg_queue_whole_cells; return NPBGB_OK;
    case NPBGB_CFG_HEAT_MAD_ROWS: *value = g_cfg_heat_mad_rows; return NPBGB_OK;
    case NPBGB_CFG_LAUNCHES: *value = g_launches.load(std::memory_order_relaxed); return NPBGB_OK;
    default: return set_error(NPBGB_ERR_ARG, "unknown config key %d", key);
  }
}

int32_t npbgb_device_status(void* stream) {
  using namespace npbgb;
  cudaError_t e = stream ? cudaStreamSynchronize(as_stream(stream)) : cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_status(e, "device status");
  const uint32_t h = take_heat_device_error() | take_heat_tb_device_error();
  const uint32_t bt = take_batch_device_error();
  const uint32_t cf = take_cfd_device_error() | take_jacobi_bands_device_error();
  const uint32_t jt = take_jacobi_tma_device_error();
  const uint32_t qu = take_queue_device_error();
  if (h == 0xffffffffu || bt == 0xffffffffu || cf == 0xffffffffu || qu == 0xffffffffu || jt == 0xffffffffu)
    return set_error(NPBGB_ERR_CUDA, "reading the device error words");
  if (h) return set_error(NPBGB_ERR_TIMEOUT, "a bounded device wait gave up (heat3d)");
  if (jt) return set_error(NPBGB_ERR_TIMEOUT, "a bounded device wait gave up (jacobi2d)");
  if (bt) return set_error(NPBGB_ERR_TIMEOUT, "a batch CTA made no progress, or a batch TMA wait gave up, within its limit");
  if (cf) return set_error(NPBGB_ERR_TIMEOUT, "a band waited on its neighbours past its limit");
  if (qu & 1u) return set_error(NPBGB_ERR_TIMEOUT, "a queue worker saw no tile complete within its limit");
  if (qu) return set_error(NPBGB_ERR_STATE, "a queue worker found an invalid inbox entry");
  return NPBGB_OK;
}

int32_t npbgb_selftest_wait_timeout(int64_t limit_ns, void* stream) {
  using namespace npbgb;
  if (limit_ns <= 0 || limit_ns > 2000000000) return set_error(NPBGB_ERR_ARG, "limit out of range");
  return launch_wait_timeout_selftest(uint64_t(limit_ns), as_stream(stream));
}

}  // extern "C"
