// C ABI of one mechanism library (libmkpp_<mechanism>.so), see include/mkpp.h.
//
// Compiled once per mechanism with
//   -DMKPP_MECH_HEADER="<mechanism>.cuh" -DMKPP_MECH_NS=mkpp_<mechanism>
// The host-buffer entry points follow the reference implementation
// (src/mkpp/templates/host_api/mkpp_c_api.cpp.j2:70-374): same argument
// checks, the same "FATAL ERROR:" messages in mkpp_get_last_error and the same
// return codes.  mkpp_integrate stages the caller's host arrays to device
// memory owned by the handle, runs the GPU solve on the handle's stream and
// copies the concentrations back before returning.
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "capi_common.cuh"

using namespace mkpp_tu;

namespace {

// Attempts one integrate() call may take before the cell is reported as
// CELL_ERR_CONVERGENCE_FAILURE.  The reference has no bound (its loop only
// ends at t >= dt); a stalled cell there never returns.  20000 is four times
// the largest count of any cell that finishes in the SAPRC99 workloads.
constexpr int kDefaultMaxAttempts = 20000;

struct DeviceBuffers {
  size_t cells = 0;
  double* conc = nullptr;
  double* temp = nullptr;
  double* rho = nullptr;
  double* rh = nullptr;
  double* clw = nullptr;
  double* param = nullptr;
  double* ktab = nullptr;
  double* out = nullptr;      // rates / Jacobian staging
  size_t out_bytes = 0;
  int* status = nullptr;
  int* accepted = nullptr;
  int* rejected = nullptr;
  int* order = nullptr;        // queue position -> cell (cost ordering)
  double* dt_carry = nullptr;  // carried step size per cell (mkpp_set_dt_carryover)
  void* workspace = nullptr;
  size_t workspace_bytes = 0;  // grows when a launch-tuning change enlarges the grid
};

}  // namespace

struct mkpp_handle_s {
  size_t num_cells = 0;
  bool initialized = false;
  double* conc = nullptr;
  const double* temp = nullptr;
  const double* pressure = nullptr;
  const double* rho = nullptr;
  const double* rh = nullptr;
  const double* sa = nullptr;
  const double* clw = nullptr;
  const double* param = nullptr;
  size_t param_count = 0;
  double seed = Mech::SEED;
  int max_attempts = kDefaultMaxAttempts;
  int mode = 1;  // persistent queue
  // Cost ordering (mkpp_set_cost_order): the persistent queue hands out the
  // cells that needed the most attempts in the previous call first.
  bool cost_order = true;
  // Step-size carry-over (mkpp_set_dt_carryover): each call starts every
  // cell at the step size its previous call ended with.
  bool dt_carryover = false;
  bool dt_carry_reset = false;  // zero the carried step sizes before the next call
  std::vector<int> cost;       // attempts per cell of the previous call
  std::vector<int> rejected;   // staging for the read-back
  std::vector<int> order;      // queue position -> cell
  cudaStream_t stream = nullptr;
  DeviceBuffers dev;
  std::string last_error;

  void set_error(const std::string& msg) { last_error = msg; }
};

namespace {

// NVTX range over a scope, named as the reference's Kokkos regions
// (MKPP_C_API_<mech>: src/mkpp/templates/host_api/mkpp_c_api.cpp.j2:275;
// MKPP_Dispatch_<mech>: src/mkpp_host/include/mkpp_host/mechanism_manager.hpp:125).
// Without a profiler attached, NVTX calls do nothing.
struct NvtxRange {
  explicit NvtxRange(const std::string& name) { nvtxRangePushA(name.c_str()); }
  ~NvtxRange() { nvtxRangePop(); }
};
const std::string kApiRange = std::string("MKPP_C_API_") + Mech::NAME;
const std::string kDispatchRange = std::string("MKPP_Dispatch_") + Mech::NAME;

int device_fail(mkpp_handle_s* h, cudaError_t err, const char* what) {
  if (h) h->set_error(std::string("FATAL ERROR: ") + what + ": " + cudaGetErrorString(err));
  return MKPP_ERROR_DEVICE;
}

#define MKPP_CUDA(h, call)                                      \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return device_fail((h), e_, #call);  \
  } while (0)


// Launch configuration of the integrate kernels, process wide:
//  register_variant  launch-bounds minimum of resident blocks (2: up to 255
//                    registers per thread, 4: up to 128, more resident warps);
//  blocks_per_sm     cap on resident blocks per SM (0: as many as fit);
//  defer_after       attempts per host step of the launch after which the
//                    persistent kernel parks a cell for the warp-cooperative
//                    kernel (0: never).  A launch over S host steps parks a
//                    cell after defer_after * S attempts in all.  A
//                    cooperative SAPRC99 attempt takes ~0.37 ms against
//                    ~1 ms on one lane, but the cooperative kernel has about
//                    a fifth of the lanes' throughput, so only the tail
//                    should park.  The default, 3000, parks ~7% of the cells
//                    in the stiff first host step of the SAPRC99 workload,
//                    ~0.15% (its slowest cells) in the later ones, and none
//                    in a 24-step window (whose slowest cell needs ~22000).
// Initial values come from MKPP_REGISTER_VARIANT, MKPP_BLOCKS_PER_SM and
// MKPP_DEFER_AFTER, and mkpp_set_launch_tuning changes them.
constexpr int kDefaultDeferPerStep = 3000;
constexpr int kDefaultTailAfter = 300;

struct Tuning {
  int register_variant = 2;
  int blocks_per_sm = 0;
  int defer_after = kDefaultDeferPerStep;
  // Tail parking threshold in attempts (0: off).  300 measured on SAPRC99:
  // the 24-step window 38.3 -> 33.6 s, the 24 per-call mkpp_integrate with
  // cost ordering 218.5 -> 161.7 s, results bit-identical.
  int tail_after = kDefaultTailAfter;
  // Split launch (mkpp_set_split_launch): with a cell order, its first
  // split_cells cells go to whole warps on the first split_sms SMs, the
  // persistent body runs on the others (0: off).
  int split_cells = 0;
  int split_sms = 0;
};

Tuning& tuning() {
  static Tuning t = [] {
    Tuning x;
    if (const char* e = std::getenv("MKPP_REGISTER_VARIANT")) x.register_variant = std::atoi(e) == 4 ? 4 : 2;
    if (const char* e = std::getenv("MKPP_BLOCKS_PER_SM")) x.blocks_per_sm = std::max(0, std::atoi(e));
    if (const char* e = std::getenv("MKPP_DEFER_AFTER")) x.defer_after = std::max(0, std::atoi(e));
    if (const char* e = std::getenv("MKPP_TAIL_AFTER")) x.tail_after = std::max(0, std::atoi(e));
    return x;
  }();
  return t;
}

struct LaunchConfig {
  int minb = 0;
  int grid = 0;
  int sms = 0;
  int coop_warps = 0;
  size_t coop_smem = 0;
  bool coop_ok = false;
  bool split_ok = false;
};

template <int MINB>
int resident_blocks() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mkpp::integrate_persistent_kernel<Mech, MINB>, mkpp::kBlock, 0);
  return std::max(1, per_sm);
}

LaunchConfig g_config;

const LaunchConfig& launch_config() {
  LaunchConfig& cfg = g_config;
  if (cfg.grid == 0) {
    const Tuning& t = tuning();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cfg.sms, cudaDevAttrMultiProcessorCount, dev);
    cfg.sms = std::max(1, cfg.sms);
    cfg.minb = t.register_variant;
    int per_sm = cfg.minb == 4 ? resident_blocks4() : resident_blocks<2>();
    if (t.blocks_per_sm > 0) per_sm = std::min(per_sm, t.blocks_per_sm);
    cfg.grid = cfg.sms * per_sm;
    // Cooperative kernel: as many warps per block (at most kCoopWarps) as fit
    // in 200 KB of shared memory.  A cell store larger than that leaves the
    // cooperative kernel unused (no parking).
    const size_t per_warp = (size_t)Mech::COOP_SLOTS * sizeof(double);
    cfg.coop_warps = (int)std::min<size_t>(mkpp::kCoopWarps, (200u * 1024u) / per_warp);
    cfg.coop_smem = per_warp * (size_t)std::max(1, cfg.coop_warps);
    cfg.coop_ok = cfg.coop_warps >= 1 && set_coop_smem(cfg.coop_smem) == MKPP_SUCCESS;
    cfg.split_ok = StoreInfo::kTile;
  }
  return cfg;
}

int integrate_grid() { return launch_config().grid; }

// Workspace layout: [queue counter, parked-cell counter, active-cell counter | 256 B]
// [per-block scratch tiles][parked-cell records, one per cell].
size_t scratch_offset() { return kQueueBytes; }
size_t defer_offset() {
  const size_t end = kQueueBytes + (size_t)integrate_grid() * StoreInfo::block_bytes;
  return (end + 255) / 256 * 256;
}
size_t workspace_bytes(size_t cells) { return defer_offset() + cells * sizeof(mkpp::Deferred); }

int launch_rates(size_t cells, const double* conc, const double* temp, const double* rho,
                 const double* rh, const double* clw, const double* param, double* ktab,
                 int* status, cudaStream_t stream) {
  mkpp::RateArgs a;
  a.ncells = (int)cells;
  a.conc = conc;
  a.param = param;
  a.temp = Mech::RUNTIME_ENV ? temp : nullptr;
  a.rho = Mech::RUNTIME_ENV ? rho : nullptr;
  a.rh = rh;
  a.clw = clw;
  a.ktab = ktab;
  a.status = status;
  mkpp::rate_constant_kernel<Mech><<<launch_grid(cells, 128), 128, 0, stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

int launch_integrate(const mkpp::LaunchArgs& args, int mode, void* workspace, cudaStream_t stream) {
  mkpp::LaunchArgs a = args;
  unsigned char* ws = (unsigned char*)workspace;
  a.queue = (unsigned int*)ws;
  a.defer_count = (unsigned int*)ws + 1;
  a.active = (unsigned int*)ws + 2;
  double* scratch = StoreInfo::block_bytes ? (double*)(ws + scratch_offset()) : nullptr;
  const LaunchConfig& cfg = launch_config();
  if (cudaMemsetAsync(ws, 0, 4 * sizeof(unsigned int), stream) != cudaSuccess) return MKPP_ERROR_DEVICE;
  if (mode == 1) {
    const Tuning& t = tuning();
    // Split launch: the order's first cells on whole warps on reserved SMs,
    // in the same launch as the persistent body (255-register variant, a
    // whole warp's store fitting the block's shared memory).
    const bool split = t.split_cells > 0 && t.split_sms > 0 && t.split_sms < cfg.sms && a.order && cfg.split_ok &&
                       cfg.minb == 2 && t.tail_after == 0;
    if (split) {
      a.split_cells = (int)std::min<long long>(t.split_cells, a.ncells);
      a.split_sms = t.split_sms;
      a.split_next = (unsigned int*)ws + 3;
    }
    const long long park = (long long)t.defer_after * std::max(1, a.steps);
    a.defer_after = (int)std::min<long long>(park, INT32_MAX);
    // Tail parking runs in the 255-register variant only.
    const bool tail = t.tail_after > 0 && cfg.minb == 2;
    a.defer = (a.defer_after > 0 || tail) && cfg.coop_ok ? (mkpp::Deferred*)(ws + defer_offset()) : nullptr;
    if (!a.defer) a.defer_after = 0;
    if (tail && a.defer) {
      a.tail_after = t.tail_after;
      a.tail_cells = (unsigned)(cfg.sms * 2 * cfg.coop_warps);
      if (launch_persistent_tail(a, scratch, cfg.grid, stream) != MKPP_SUCCESS) return MKPP_ERROR_DEVICE;
    } else if (split) {
      if (launch_split(a, scratch, cfg.grid, stream) != MKPP_SUCCESS) return MKPP_ERROR_DEVICE;
    } else if (cfg.minb == 4) {
      if (launch_persistent4(a, scratch, cfg.grid, stream) != MKPP_SUCCESS) return MKPP_ERROR_DEVICE;
    } else {
      mkpp::integrate_persistent_kernel<Mech, 2><<<cfg.grid, mkpp::kBlock, 0, stream>>>(a, scratch);
    }
    if (a.defer) {
      if (launch_coop(a, cfg.sms * 2, cfg.coop_warps * 32, cfg.coop_smem, stream) != MKPP_SUCCESS) {
        return MKPP_ERROR_DEVICE;
      }
    }
  } else {
    // The plain form runs with the same grid and the 255-register variant.
    a.defer = nullptr;
    a.defer_after = 0;
    if (launch_plain(a, scratch, cfg.grid, stream) != MKPP_SUCCESS) return MKPP_ERROR_DEVICE;
  }
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}


// ---------------------------------------------------------------------------
// Allocation-free integrate (mkpp_gpu_integrate_noalloc).
//
// Its LU/stage scratch is this file-scope device array instead of a
// caller-provided workspace.  The array holds the working storage of
// MKPP_NOALLOC_MAX_CELLS cells, laid out as the plain kernel's per-block
// tiles (ceil(cells / 128) blocks of 128 threads).  Every GPU that loads the
// library keeps it allocated until the process exits.  In host code the
// name g_noalloc_scratch is only a host-side stand-in; the device address is
// obtained once per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxCells = MKPP_NOALLOC_MAX_CELLS;
// The plain launch gives every block kBlock cells of scratch, so the array
// covers the last block only when the capacity is a whole number of blocks.
static_assert(kNoAllocMaxCells % mkpp::kBlock == 0, "noalloc capacity must be a multiple of the block size");
constexpr size_t kNoAllocDoubles = StoreInfo::kTile ? (size_t)kNoAllocMaxCells * Mech::NSLOTS : 1;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, set up on the
// first call made with that device current.
int noalloc_scratch(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MKPP_ERROR_DEVICE;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    double* ptr = nullptr;
    if (cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return MKPP_ERROR_DEVICE;
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return MKPP_SUCCESS;
}

}  // namespace

extern "C" {

int mkpp_gpu_integrate_noalloc(size_t num_cells, double* conc, const double* ktab, size_t k_step_stride,
                               int steps, double dt, double seed, int max_attempts, int* status, int* accepted,
                               int* rejected, void* stream) {
  if (!conc || !ktab) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0) return MKPP_ERROR_INVALID_ARGUMENT;
  if (num_cells > (size_t)kNoAllocMaxCells) {
    std::fprintf(stderr,
                 "FATAL ERROR: mkpp_gpu_integrate_noalloc: %zu cells exceed its static scratch capacity of %d "
                 "cells; split the call or use mkpp_gpu_integrate_k with a workspace\n",
                 num_cells, kNoAllocMaxCells);
    return MKPP_ERROR_INVALID_ARGUMENT;
  }
  if (!std::isfinite(dt) || dt <= 0.0 || steps < 1 || !(seed > 0.0) || max_attempts < 1) return MKPP_ERROR_INVALID_ARGUMENT;
  if (k_step_stride != 0 && k_step_stride < num_cells * Mech::NR) return MKPP_ERROR_INVALID_ARGUMENT;
  double* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc != MKPP_SUCCESS) return rc;
  mkpp::LaunchArgs a = make_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, status, accepted, rejected);
  a.k_step_stride = k_step_stride;
  const int grid = (int)((num_cells + mkpp::kBlock - 1) / mkpp::kBlock);
  return launch_plain(a, StoreInfo::kTile ? scratch : nullptr, grid, (cudaStream_t)stream);
}

}  // extern "C"

extern "C" {

// ---- Reference host API ---------------------------------------------------

int mkpp_create_handle(mkpp_handle_t* handle_out, size_t num_cells) {
  if (!handle_out) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0) return MKPP_ERROR_INVALID_ARGUMENT;
  if (num_cells > (size_t)INT32_MAX) return MKPP_ERROR_INVALID_ARGUMENT;
  auto* h = new (std::nothrow) mkpp_handle_s();
  if (!h) return MKPP_ERROR_INVALID_STATE;
  h->num_cells = num_cells;
  *handle_out = h;
  return MKPP_SUCCESS;
}

// Frees what the handle allocated; a handle that never computed makes no
// CUDA call here.
static void free_device(DeviceBuffers& d) {
  for (void* p : {(void*)d.conc, (void*)d.temp, (void*)d.rho, (void*)d.rh, (void*)d.clw, (void*)d.param,
                  (void*)d.ktab, (void*)d.out, (void*)d.status, (void*)d.accepted, (void*)d.rejected,
                  (void*)d.order, (void*)d.dt_carry, d.workspace})
    if (p) cudaFree(p);
  d = DeviceBuffers();
}

int mkpp_destroy_handle(mkpp_handle_t handle) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  free_device(handle->dev);
  if (handle->stream) cudaStreamDestroy(handle->stream);
  delete handle;
  return MKPP_SUCCESS;
}

// Like the reference's, initialization only readies the handle: the stream
// and the device buffers are created by the first call that computes, so a
// host without a GPU gets MKPP_ERROR_DEVICE there, with a message.
int mkpp_initialize(mkpp_handle_t handle) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  handle->initialized = true;
  return MKPP_SUCCESS;
}

int mkpp_get_species_count(mkpp_handle_t handle, size_t* count_out) {
  if (!handle || !count_out) return MKPP_ERROR_NULL_POINTER;
  *count_out = Mech::NS;
  return MKPP_SUCCESS;
}

int mkpp_get_reaction_count(mkpp_handle_t handle, size_t* count_out) {
  if (!handle || !count_out) return MKPP_ERROR_NULL_POINTER;
  *count_out = Mech::NR;
  return MKPP_SUCCESS;
}

int mkpp_get_photolysis_count(mkpp_handle_t handle, size_t* count_out) {
  if (!handle || !count_out) return MKPP_ERROR_NULL_POINTER;
  *count_out = Mech::NPH;
  return MKPP_SUCCESS;
}

int mkpp_get_species_index(mkpp_handle_t handle, const char* name, int* index_out) {
  if (!handle || !name || !index_out) return MKPP_ERROR_NULL_POINTER;
  for (int s = 0; s < Mech::NS; ++s) {
    if (std::strcmp(Mech::species_name(s), name) == 0) {
      *index_out = s;
      return MKPP_SUCCESS;
    }
  }
  *index_out = -1;
  return MKPP_ERROR_NOT_FOUND;
}

int mkpp_get_photolysis_index(mkpp_handle_t handle, const char* name, int* index_out) {
  if (!handle || !name || !index_out) return MKPP_ERROR_NULL_POINTER;
  for (int p = 0; p < Mech::NPH; ++p) {
    if (std::strcmp(Mech::photolysis_name(p), name) == 0) {
      *index_out = p;
      return MKPP_SUCCESS;
    }
  }
  *index_out = -1;
  return MKPP_ERROR_NOT_FOUND;
}

static int validate_state(mkpp_handle_s& h) {
  if (!h.conc) {
    h.set_error("FATAL ERROR: species concentration pointer is not bound");
    return MKPP_ERROR_NULL_POINTER;
  }
  if (!h.temp || !h.rho || !h.pressure) {
    h.set_error("FATAL ERROR: per-cell meteorology is not bound");
    return MKPP_ERROR_NULL_POINTER;
  }
  for (size_t c = 0; c < h.num_cells; ++c) {
    if (!std::isfinite(h.temp[c]) || h.temp[c] <= 0.0 || !std::isfinite(h.rho[c]) || h.rho[c] <= 0.0 ||
        !std::isfinite(h.pressure[c]) || h.pressure[c] <= 0.0) {
      h.set_error("FATAL ERROR: cell temperature, density and pressure must be positive and finite");
      return MKPP_ERROR_INVALID_ARGUMENT;
    }
  }
  return MKPP_SUCCESS;
}

int mkpp_set_state_ptrs(mkpp_handle_t handle, double* species_conc, const double* temp,
                        const double* pressure, const double* air_density) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  if (!species_conc || !temp || !pressure || !air_density) {
    handle->set_error("FATAL ERROR: state binding requires concentration and meteorology pointers");
    return MKPP_ERROR_NULL_POINTER;
  }
  handle->conc = species_conc;
  handle->temp = temp;
  handle->pressure = pressure;
  handle->rho = air_density;
  return validate_state(*handle);
}

int mkpp_set_rate_parameter_ptrs(mkpp_handle_t handle, const double* values, size_t count) {
  if (!handle || !values) return MKPP_ERROR_NULL_POINTER;
  if (count != (size_t)Mech::NP) {
    handle->set_error("FATAL ERROR: runtime parameter count does not match the generated mechanism");
    return MKPP_ERROR_INVALID_ARGUMENT;
  }
  handle->param = values;
  handle->param_count = count;
  return MKPP_SUCCESS;
}

int mkpp_set_photolysis_ptrs(mkpp_handle_t handle, const double* photolysis_rates) {
  if (!handle || !photolysis_rates) return MKPP_ERROR_NULL_POINTER;
  if (Mech::NP > Mech::NPH) {
    handle->set_error("FATAL ERROR: use mkpp_set_rate_parameter_ptrs for the complete runtime parameter array");
    return MKPP_ERROR_INVALID_ARGUMENT;
  }
  return mkpp_set_rate_parameter_ptrs(handle, photolysis_rates, Mech::NPH);
}

int mkpp_set_cloud_water_ptr(mkpp_handle_t handle, const double* values) {
  if (!handle || !values) return MKPP_ERROR_NULL_POINTER;
  handle->clw = values;
  return MKPP_SUCCESS;
}

int mkpp_set_aerosol_ptrs(mkpp_handle_t handle, const double* relative_humidity,
                          const double* aerosol_surface_area) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  if (relative_humidity) handle->rh = relative_humidity;
  if (aerosol_surface_area) handle->sa = aerosol_surface_area;
  return MKPP_SUCCESS;
}

static int ensure_device(mkpp_handle_s* h, size_t out_bytes) {
  DeviceBuffers& d = h->dev;
  const size_t n = h->num_cells;
  if (!h->stream) MKPP_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  if (d.cells != n) {
    free_device(d);
    MKPP_CUDA(h, cudaMalloc(&d.conc, n * Mech::NS * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.temp, n * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.rho, n * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.rh, n * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.clw, n * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.param, n * std::max(1, Mech::NP) * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.ktab, n * Mech::NR * sizeof(double)));
    MKPP_CUDA(h, cudaMalloc(&d.status, n * sizeof(int)));
    MKPP_CUDA(h, cudaMalloc(&d.accepted, n * sizeof(int)));
    MKPP_CUDA(h, cudaMalloc(&d.rejected, n * sizeof(int)));
    d.cells = n;
  }
  // The integrate scratch depends on the launch grid, which
  // mkpp_set_launch_tuning can change between calls.
  const size_t ws = workspace_bytes(n);
  if (ws > d.workspace_bytes) {
    cudaFree(d.workspace);
    d.workspace = nullptr;
    d.workspace_bytes = 0;
    MKPP_CUDA(h, cudaMalloc(&d.workspace, ws));
    d.workspace_bytes = ws;
  }
  if (out_bytes > d.out_bytes) {
    cudaFree(d.out);
    d.out = nullptr;
    d.out_bytes = 0;
    MKPP_CUDA(h, cudaMalloc(&d.out, out_bytes));
    d.out_bytes = out_bytes;
  }
  return MKPP_SUCCESS;
}

// Copy the bound host inputs to the device and compute the rate constants.
static int stage_inputs(mkpp_handle_s* h) {
  DeviceBuffers& d = h->dev;
  const size_t n = h->num_cells;
  cudaStream_t s = h->stream;
  MKPP_CUDA(h, cudaMemcpyAsync(d.conc, h->conc, n * Mech::NS * sizeof(double), cudaMemcpyHostToDevice, s));
  MKPP_CUDA(h, cudaMemcpyAsync(d.temp, h->temp, n * sizeof(double), cudaMemcpyHostToDevice, s));
  MKPP_CUDA(h, cudaMemcpyAsync(d.rho, h->rho, n * sizeof(double), cudaMemcpyHostToDevice, s));
  if (h->rh) MKPP_CUDA(h, cudaMemcpyAsync(d.rh, h->rh, n * sizeof(double), cudaMemcpyHostToDevice, s));
  if (h->clw) MKPP_CUDA(h, cudaMemcpyAsync(d.clw, h->clw, n * sizeof(double), cudaMemcpyHostToDevice, s));
  if (h->param && Mech::NP > 0)
    MKPP_CUDA(h, cudaMemcpyAsync(d.param, h->param, n * Mech::NP * sizeof(double), cudaMemcpyHostToDevice, s));
  int rc = launch_rates(n, d.conc, d.temp, d.rho, h->rh ? d.rh : nullptr, h->clw ? d.clw : nullptr,
                        h->param ? d.param : nullptr, d.ktab, d.status, s);
  if (rc != MKPP_SUCCESS) return device_fail(h, cudaGetLastError(), "rate_constant_kernel launch");
  return MKPP_SUCCESS;
}

int mkpp_integrate(mkpp_handle_t handle, double dt) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  const NvtxRange range(kApiRange);
  mkpp_handle_s* h = handle;
  if (!h->initialized) {
    h->set_error("FATAL ERROR: MKPP handle must be initialized before integration");
    return MKPP_ERROR_INVALID_STATE;
  }
  const int vs = validate_state(*h);
  if (vs != MKPP_SUCCESS) return vs;
  if (!std::isfinite(dt) || dt <= 0.0) return MKPP_ERROR_INVALID_ARGUMENT;
  int rc = ensure_device(h, 0);
  if (rc != MKPP_SUCCESS) return rc;
  rc = stage_inputs(h);
  if (rc != MKPP_SUCCESS) return rc;
  DeviceBuffers& d = h->dev;
  const size_t n = h->num_cells;
  mkpp::LaunchArgs args = make_args(n, d.conc, d.ktab, 1, dt, h->seed, h->max_attempts, d.status, d.accepted,
                                    d.rejected);
  if (h->cost_order && h->cost.size() == n) {
    // Most expensive first; ties keep the cell order.
    h->order.resize(n);
    for (size_t c = 0; c < n; ++c) h->order[c] = (int)c;
    std::stable_sort(h->order.begin(), h->order.end(), [h](int x, int y) { return h->cost[x] > h->cost[y]; });
    if (!d.order) MKPP_CUDA(h, cudaMalloc(&d.order, n * sizeof(int)));
    MKPP_CUDA(h, cudaMemcpyAsync(d.order, h->order.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    args.order = d.order;
  }
  if (h->dt_carryover) {
    if (!d.dt_carry) {
      MKPP_CUDA(h, cudaMalloc(&d.dt_carry, n * sizeof(double)));
      h->dt_carry_reset = true;
    }
    if (h->dt_carry_reset) MKPP_CUDA(h, cudaMemsetAsync(d.dt_carry, 0, n * sizeof(double), h->stream));
    h->dt_carry_reset = false;
    args.dt_carry = d.dt_carry;
  }
  rc = launch_integrate(args, h->mode, d.workspace, h->stream);
  if (rc != MKPP_SUCCESS) return device_fail(h, cudaGetLastError(), "integrate kernel launch");
  MKPP_CUDA(h, cudaMemcpyAsync(h->conc, d.conc, n * Mech::NS * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  if (h->cost_order) {
    h->cost.resize(n);
    h->rejected.resize(n);
    MKPP_CUDA(h, cudaMemcpyAsync(h->cost.data(), d.accepted, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MKPP_CUDA(h, cudaMemcpyAsync(h->rejected.data(), d.rejected, n * sizeof(int), cudaMemcpyDeviceToHost,
                                 h->stream));
  }
  MKPP_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->cost_order)
    for (size_t c = 0; c < n; ++c) h->cost[c] += h->rejected[c];
  return MKPP_SUCCESS;
}

int mkpp_set_cost_order(mkpp_handle_t handle, int enable) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  handle->cost_order = enable != 0;
  handle->cost.clear();
  return MKPP_SUCCESS;
}

int mkpp_set_dt_carryover(mkpp_handle_t handle, int enable) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  handle->dt_carryover = enable != 0;
  handle->dt_carry_reset = true;
  return MKPP_SUCCESS;
}

int mkpp_evaluate_rates(mkpp_handle_t handle, double* rates_out) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  mkpp_handle_s* h = handle;
  if (!rates_out) {
    h->set_error("FATAL ERROR: rates output pointer is null");
    return MKPP_ERROR_NULL_POINTER;
  }
  if (!h->initialized) {
    h->set_error("FATAL ERROR: MKPP handle must be initialized before rates evaluation");
    return MKPP_ERROR_INVALID_STATE;
  }
  const int vs = validate_state(*h);
  if (vs != MKPP_SUCCESS) return vs;
  const size_t n = h->num_cells;
  const size_t bytes = n * Mech::NS * sizeof(double);
  int rc = ensure_device(h, bytes);
  if (rc != MKPP_SUCCESS) return rc;
  rc = stage_inputs(h);
  if (rc != MKPP_SUCCESS) return rc;
  if (launch_eval_rates(n, h->dev.conc, h->dev.ktab, h->dev.out, h->stream) != MKPP_SUCCESS)
    return device_fail(h, cudaGetLastError(), "eval_rates_kernel launch");
  MKPP_CUDA(h, cudaMemcpyAsync(rates_out, h->dev.out, bytes, cudaMemcpyDeviceToHost, h->stream));
  MKPP_CUDA(h, cudaStreamSynchronize(h->stream));
  return MKPP_SUCCESS;
}

int mkpp_evaluate_jacobian(mkpp_handle_t handle, double* jac_out) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  mkpp_handle_s* h = handle;
  if (!jac_out) {
    h->set_error("FATAL ERROR: Jacobian output pointer is null");
    return MKPP_ERROR_NULL_POINTER;
  }
  if (!h->initialized) {
    h->set_error("FATAL ERROR: MKPP handle must be initialized before Jacobian evaluation");
    return MKPP_ERROR_INVALID_STATE;
  }
  const int vs = validate_state(*h);
  if (vs != MKPP_SUCCESS) return vs;
  const size_t n = h->num_cells;
  const size_t bytes = n * Mech::NS * Mech::NS * sizeof(double);
  int rc = ensure_device(h, bytes);
  if (rc != MKPP_SUCCESS) return rc;
  rc = stage_inputs(h);
  if (rc != MKPP_SUCCESS) return rc;
  if (launch_eval_jacobian(n, h->dev.conc, h->dev.ktab, h->dev.out, h->stream) != MKPP_SUCCESS)
    return device_fail(h, cudaGetLastError(), "eval_jacobian_kernel launch");
  if (Mech::NFIX > 0 &&
      launch_fixed_columns(n, h->dev.conc, h->dev.temp, h->dev.rho, h->rh ? h->dev.rh : nullptr,
                           h->clw ? h->dev.clw : nullptr, h->param ? h->dev.param : nullptr, h->dev.out,
                           h->stream) != MKPP_SUCCESS)
    return device_fail(h, cudaGetLastError(), "fixed_columns_kernel launch");
  MKPP_CUDA(h, cudaMemcpyAsync(jac_out, h->dev.out, bytes, cudaMemcpyDeviceToHost, h->stream));
  MKPP_CUDA(h, cudaStreamSynchronize(h->stream));
  return MKPP_SUCCESS;
}

// out = J v or J^T v per cell on the dense (cells x N x N) LayoutLeft Jacobian
// jac[c + n (row + N col)]; v and out are (cells x N) LayoutLeft.
static __global__ void jac_vec_kernel(size_t n, const double* jac, const double* v, double* out, bool transpose) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t NS = Mech::NS;
  for (size_t i = 0; i < NS; ++i) {
    double acc = 0.0;
    for (size_t j = 0; j < NS; ++j) {
      const double jij = transpose ? jac[c + n * (j + NS * i)] : jac[c + n * (i + NS * j)];
      acc = fma(jij, v[c + n * j], acc);
    }
    out[c + n * i] = acc;
  }
}

// The dense Jacobian of the bound state (as mkpp_evaluate_jacobian) applied
// to a host vector, or its transpose.
static int jacobian_product(mkpp_handle_t handle, const double* vec, double* out, bool transpose) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  mkpp_handle_s* h = handle;
  if (!vec || !out) {
    h->set_error("FATAL ERROR: Jacobian product vector or output pointer is null");
    return MKPP_ERROR_NULL_POINTER;
  }
  if (!h->initialized) {
    h->set_error("FATAL ERROR: MKPP handle must be initialized before Jacobian evaluation");
    return MKPP_ERROR_INVALID_STATE;
  }
  const int vs = validate_state(*h);
  if (vs != MKPP_SUCCESS) return vs;
  const size_t n = h->num_cells;
  const size_t jbytes = n * Mech::NS * Mech::NS * sizeof(double);
  const size_t vbytes = n * Mech::NS * sizeof(double);
  int rc = ensure_device(h, jbytes + 2 * vbytes);
  if (rc != MKPP_SUCCESS) return rc;
  rc = stage_inputs(h);
  if (rc != MKPP_SUCCESS) return rc;
  DeviceBuffers& d = h->dev;
  if (launch_eval_jacobian(n, d.conc, d.ktab, d.out, h->stream) != MKPP_SUCCESS)
    return device_fail(h, cudaGetLastError(), "eval_jacobian_kernel launch");
  if (Mech::NFIX > 0 &&
      launch_fixed_columns(n, d.conc, d.temp, d.rho, h->rh ? d.rh : nullptr, h->clw ? d.clw : nullptr,
                           h->param ? d.param : nullptr, d.out, h->stream) != MKPP_SUCCESS)
    return device_fail(h, cudaGetLastError(), "fixed_columns_kernel launch");
  double* dv = d.out + n * Mech::NS * Mech::NS;
  double* dres = dv + n * Mech::NS;
  MKPP_CUDA(h, cudaMemcpyAsync(dv, vec, vbytes, cudaMemcpyHostToDevice, h->stream));
  jac_vec_kernel<<<launch_grid(n, 128), 128, 0, h->stream>>>(n, d.out, dv, dres, transpose);
  MKPP_CUDA(h, cudaGetLastError());
  MKPP_CUDA(h, cudaMemcpyAsync(out, dres, vbytes, cudaMemcpyDeviceToHost, h->stream));
  MKPP_CUDA(h, cudaStreamSynchronize(h->stream));
  return MKPP_SUCCESS;
}

int mkpp_evaluate_jacobian_vector(mkpp_handle_t handle, const double* delta, double* out) {
  return jacobian_product(handle, delta, out, false);
}

int mkpp_evaluate_jacobian_transpose_vector(mkpp_handle_t handle, const double* lambda, double* out) {
  return jacobian_product(handle, lambda, out, true);
}

int mkpp_get_last_error(mkpp_handle_t handle, char* buffer, size_t buffer_len) {
  if (!handle || !buffer || buffer_len == 0) return MKPP_ERROR_NULL_POINTER;
  std::strncpy(buffer, handle->last_error.c_str(), buffer_len - 1);
  buffer[buffer_len - 1] = '\0';
  return MKPP_SUCCESS;
}

// ---- Handle options -------------------------------------------------------

int mkpp_set_initial_step_seed(mkpp_handle_t handle, double seed) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  if (!std::isfinite(seed) || seed <= 0.0) {
    handle->set_error("FATAL ERROR: initial_step_seed must be a finite positive fraction of the chemistry interval");
    return MKPP_ERROR_INVALID_ARGUMENT;
  }
  handle->seed = seed;
  return MKPP_SUCCESS;
}

int mkpp_set_max_attempts(mkpp_handle_t handle, int max_attempts) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  if (max_attempts <= 0) return MKPP_ERROR_INVALID_ARGUMENT;
  handle->max_attempts = max_attempts;
  return MKPP_SUCCESS;
}

int mkpp_get_cell_stats(mkpp_handle_t handle, int* status, int* accepted, int* rejected) {
  if (!handle) return MKPP_ERROR_NULL_POINTER;
  mkpp_handle_s* h = handle;
  if (h->dev.cells == 0) {
    h->set_error("FATAL ERROR: no integration has run on this handle");
    return MKPP_ERROR_INVALID_STATE;
  }
  const size_t bytes = h->num_cells * sizeof(int);
  if (status) MKPP_CUDA(h, cudaMemcpyAsync(status, h->dev.status, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (accepted) MKPP_CUDA(h, cudaMemcpyAsync(accepted, h->dev.accepted, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (rejected) MKPP_CUDA(h, cudaMemcpyAsync(rejected, h->dev.rejected, bytes, cudaMemcpyDeviceToHost, h->stream));
  MKPP_CUDA(h, cudaStreamSynchronize(h->stream));
  return MKPP_SUCCESS;
}

// ---- Mechanism metadata ----------------------------------------------------

int mkpp_mechanism_name(const char** name_out) {
  if (!name_out) return MKPP_ERROR_NULL_POINTER;
  *name_out = Mech::NAME;
  return MKPP_SUCCESS;
}

int mkpp_mechanism_sizes(int* num_species, int* num_variable, int* num_reactions, int* num_rate_parameters,
                         int* num_lu_slots) {
  if (num_species) *num_species = Mech::NS;
  if (num_variable) *num_variable = Mech::NV;
  if (num_reactions) *num_reactions = Mech::NR;
  if (num_rate_parameters) *num_rate_parameters = Mech::NP;
  if (num_lu_slots) *num_lu_slots = Mech::NLU;
  return MKPP_SUCCESS;
}

int mkpp_mechanism_flags(int* runtime_environment, int* cloud_gated) {
  if (!runtime_environment && !cloud_gated) return MKPP_ERROR_NULL_POINTER;
  if (runtime_environment) *runtime_environment = Mech::RUNTIME_ENV ? 1 : 0;
  if (cloud_gated) *cloud_gated = Mech::CLOUD_GATED ? 1 : 0;
  return MKPP_SUCCESS;
}

int mkpp_mechanism_tolerances(double* atol, double* rtol) {
  if (!atol && !rtol) return MKPP_ERROR_NULL_POINTER;
  for (int s = 0; s < Mech::NS; ++s) {
    if (atol) atol[s] = Mech::ATOL[s];
    if (rtol) rtol[s] = Mech::RTOL[s];
  }
  return MKPP_SUCCESS;
}

// ---- Device-pointer entry points --------------------------------------------

size_t mkpp_gpu_workspace_bytes(size_t num_cells) { return workspace_bytes(num_cells); }

int mkpp_set_tail_parking(int min_attempts) {
  if (min_attempts < 0) return MKPP_ERROR_INVALID_ARGUMENT;
  tuning().tail_after = min_attempts;
  return MKPP_SUCCESS;
}

int mkpp_set_split_launch(int split_cells, int split_sms) {
  if (split_cells < 0 || split_sms < 0) return MKPP_ERROR_INVALID_ARGUMENT;
  Tuning& t = tuning();
  t.split_cells = split_cells;
  t.split_sms = split_sms;
  return MKPP_SUCCESS;
}

int mkpp_set_launch_tuning(int register_variant, int blocks_per_sm, int defer_after) {
  if (register_variant != 0 && register_variant != 2 && register_variant != 4) return MKPP_ERROR_INVALID_ARGUMENT;
  if (blocks_per_sm < 0 || defer_after < -1) return MKPP_ERROR_INVALID_ARGUMENT;
  Tuning& t = tuning();
  if (register_variant) t.register_variant = register_variant;
  t.blocks_per_sm = blocks_per_sm;
  if (defer_after >= 0) t.defer_after = defer_after;
  g_config = LaunchConfig();  // recomputed at the next launch
  return MKPP_SUCCESS;
}

int mkpp_gpu_rate_constants(size_t num_cells, const double* conc, const double* temp, const double* rho,
                            const double* rh, const double* clw, const double* param, size_t num_params,
                            double* ktab, int* status, void* stream) {
  if (!conc || !ktab) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0 || num_cells > (size_t)INT32_MAX) return MKPP_ERROR_INVALID_ARGUMENT;
  if (param && num_params != (size_t)Mech::NP) return MKPP_ERROR_INVALID_ARGUMENT;
  if (Mech::RUNTIME_ENV && (!temp || !rho)) return MKPP_ERROR_NULL_POINTER;
  return launch_rates(num_cells, conc, temp, rho, rh, clw, param, ktab, status, (cudaStream_t)stream);
}

static int check_integrate_args(size_t num_cells, const double* conc, const double* ktab, int steps, double dt,
                                double seed, int max_attempts, const void* workspace, size_t workspace_bytes_) {
  if (!conc || !ktab || !workspace) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0 || num_cells > (size_t)INT32_MAX) return MKPP_ERROR_INVALID_ARGUMENT;
  if (!std::isfinite(dt) || dt <= 0.0 || steps < 1 || !(seed > 0.0) || max_attempts < 1) return MKPP_ERROR_INVALID_ARGUMENT;
  if (workspace_bytes_ < workspace_bytes(num_cells)) return MKPP_ERROR_INVALID_ARGUMENT;
  if (((uintptr_t)workspace) % 256 != 0) return MKPP_ERROR_INVALID_ARGUMENT;
  return MKPP_SUCCESS;
}

int mkpp_gpu_integrate_k(size_t num_cells, double* conc, const double* ktab, size_t k_step_stride, int steps,
                         double dt, double seed, int max_attempts, int mode, const int* cell_order, int* status,
                         int* accepted, int* rejected, void* workspace, size_t workspace_bytes_, void* stream) {
  const int rc = check_integrate_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, workspace, workspace_bytes_);
  if (rc != MKPP_SUCCESS) return rc;
  const NvtxRange range(kDispatchRange);
  if (mode != 0 && mode != 1) return MKPP_ERROR_INVALID_ARGUMENT;
  if (k_step_stride != 0 && k_step_stride < num_cells * Mech::NR) return MKPP_ERROR_INVALID_ARGUMENT;
  mkpp::LaunchArgs a = make_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, status, accepted, rejected);
  a.order = cell_order;
  a.k_step_stride = k_step_stride;
  return launch_integrate(a, mode, workspace, (cudaStream_t)stream);
}

int mkpp_gpu_integrate_carry(size_t num_cells, double* conc, const double* ktab, size_t k_step_stride, int steps,
                             double dt, double seed, int max_attempts, int mode, const int* cell_order,
                             int* status, int* accepted, int* rejected, double* dt_carry, void* workspace,
                             size_t workspace_bytes_, void* stream) {
  if (!dt_carry) return MKPP_ERROR_NULL_POINTER;
  const int rc = check_integrate_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, workspace, workspace_bytes_);
  if (rc != MKPP_SUCCESS) return rc;
  const NvtxRange range(kDispatchRange);
  if (mode != 0 && mode != 1) return MKPP_ERROR_INVALID_ARGUMENT;
  if (k_step_stride != 0 && k_step_stride < num_cells * Mech::NR) return MKPP_ERROR_INVALID_ARGUMENT;
  mkpp::LaunchArgs a = make_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, status, accepted, rejected);
  a.order = cell_order;
  a.k_step_stride = k_step_stride;
  a.dt_carry = dt_carry;
  return launch_integrate(a, mode, workspace, (cudaStream_t)stream);
}

int mkpp_gpu_integrate_logged(size_t num_cells, double* conc, const double* ktab, int steps, double dt, double seed,
                              int max_attempts, int* status, int* accepted, int* rejected, double* log_h,
                              unsigned char* log_acc, int* log_n, int log_cap, void* workspace,
                              size_t workspace_bytes_, void* stream) {
  const int rc = check_integrate_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, workspace, workspace_bytes_);
  if (rc != MKPP_SUCCESS) return rc;
  if (!log_h || !log_acc || !log_n) return MKPP_ERROR_NULL_POINTER;
  if (log_cap < 1) return MKPP_ERROR_INVALID_ARGUMENT;
  mkpp::LaunchArgs a = make_args(num_cells, conc, ktab, steps, dt, seed, max_attempts, status, accepted, rejected);
  a.log_h = log_h;
  a.log_acc = log_acc;
  a.log_n = log_n;
  a.log_cap = log_cap;
  return launch_integrate(a, 0, workspace, (cudaStream_t)stream);
}

}  // extern "C"
