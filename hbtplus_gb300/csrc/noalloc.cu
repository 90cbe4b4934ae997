// noalloc.cu -- hbtu_unbind_noalloc: unbinding of one subhalo that allocates
// nothing.
//
// Some callers cannot allocate GPU memory at the point where they unbind: code
// that runs under another framework's memory pool or allocator, a process
// whose device memory is fully reserved up front, or a real-time pipeline that
// forbids allocation after start-up.  They cannot use hbtu_create (which
// allocates a stream, pinned memory and a workspace).  This entry point takes
// device-resident inputs and outputs from the caller and finds its working
// memory in a fixed array compiled into the library:
//
//   * scratch: a file-scope static __device__ array of kScratchBytes (8 MiB).
//     Every GPU that loads the library holds it until the process exits.  It
//     covers one subhalo of at most HBTU_NOALLOC_MAX_PARTICLES particles;
//     larger subhaloes are rejected with HBTU_ERR_TOO_LARGE.
//   * set-up: the first call on a device, with that device current, obtains
//     the array's device address with cudaGetSymbolAddress (the host-side name
//     of the array is not a device address) and keeps it for later calls on
//     that device.  Make that first call before any stream capture.
//   * sharing: all calls on a device use the same array and it keeps the last
//     call's contents; every buffer the loop needs zeroed is cleared by the
//     call itself.  Calls that overlap on the GPU (different streams or host
//     threads at the same time) race on the array: serialise them.
//   * no cudaMalloc, cudaFree, cudaMallocHost or allocating library routine is
//     called; host-side state lives on the stack and is copied with plain
//     cudaMemcpyAsync on the caller's stream.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "driver.h"

namespace hbtu {

void set_global_error(const char *fmt, ...);

namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mutex;
char *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once).
hbtu_status scratch_on_current_device(char **out)
{
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    set_global_error("hbtu_unbind_noalloc: no current CUDA device");
    return HBTU_ERR_NO_DEVICE;
  }
  int major = 0, minor = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
      major != 10 || minor != 3) {
    cudaGetLastError();
    set_global_error("hbtu_unbind_noalloc: device %d is not compute capability 10.3 (this "
                     "library is built for sm_103a only)",
                     dev);
    return HBTU_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      set_global_error("hbtu_unbind_noalloc: cudaGetSymbolAddress of the scratch array failed on "
                       "device %d: %s",
                       dev, cudaGetErrorString(e));
      return HBTU_ERR_CUDA;
    }
    g_scratch_ptr[dev] = (char *)p;
  }
  *out = g_scratch_ptr[dev];
  return HBTU_OK;
}

}  // namespace
}  // namespace hbtu

using namespace hbtu;

extern "C" hbtu_status hbtu_unbind_noalloc(const hbtu_params *params, const hbtu_particles *p,
                                           int64_t n, const hbtu_state *st, int64_t *order_out,
                                           float *energy_out, hbtu_result *res, void *cuda_stream)
{
  if (!params || !p || !st || !res || (n > 0 && (!order_out || !energy_out))) {
    set_global_error("hbtu_unbind_noalloc: null argument");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (p->location != HBTU_DEVICE) {
    set_global_error("hbtu_unbind_noalloc: particles and outputs must be device memory "
                     "(location HBTU_DEVICE)");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (n < 0) {
    set_global_error("hbtu_unbind_noalloc: negative particle count");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (n > HBTU_NOALLOC_MAX_PARTICLES) {
    set_global_error("hbtu_unbind_noalloc: %lld particles exceed the fixed scratch capacity of "
                     "%d particles; use hbtu_unbind",
                     (long long)n, (int)HBTU_NOALLOC_MAX_PARTICLES);
    return HBTU_ERR_TOO_LARGE;
  }
  if (n > 0 && (!p->id || !p->pos || !p->vel || !p->mass)) {
    set_global_error("hbtu_unbind_noalloc: null id, pos, vel or mass array");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (!(params->softening > 0) || !(params->open_angle >= 0) ||
      !(params->bound_mass_precision > 0 && params->bound_mass_precision <= 1) ||
      params->min_num_part < 0 || params->max_sample_size < 0 ||
      (params->periodic && !(params->box_size > 0)) || !(params->scale_factor > 0) ||
      (params->precision != HBTU_PRECISION_FP32 && params->precision != HBTU_PRECISION_FP64)) {
    set_global_error("hbtu_unbind_noalloc: invalid parameters");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (workspace_bytes(HBTU_NOALLOC_MAX_PARTICLES, 1, false) > kScratchBytes) {
    set_global_error("hbtu_unbind_noalloc: scratch array smaller than its stated capacity");
    return HBTU_ERR_TOO_LARGE;
  }
  char *base = nullptr;
  hbtu_status rc = scratch_on_current_device(&base);
  if (rc != HBTU_OK) return rc;
  const cudaStream_t stream = (cudaStream_t)cuda_stream;
  try {
    Ctx c;
    Staging sg;
    carve_workspace(base, c, sg, n, 1, false);
    PassPlan plan_host;
    c.P = derive_params(*params);
    c.N = (int)n;
    c.S = 1;
    c.st = stream;
    c.plan_host = &plan_host;
    c.pot_out = nullptr;
    c.grad_pos = c.grad_vel = c.grad_mass = nullptr;
    c.type = (int *)p->type;
    c.id = (long long *)p->id;
    c.opt_leaf_runs = 1;
    c.opt_schedule = 0;
    c.opt_layout = 0;
    c.small_cap = 0;  // every pass on the batch kernels
    c.small_per_sm = 1;
    SegState g;
    init_segment(g, 0, (int)n, *st, params->max_sample_size);
    const int segoff[2] = {0, (int)n};
    const int order[1] = {0};
    HBTU_CUDA(cudaMemcpyAsync(c.seg, &g, sizeof(SegState), cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemcpyAsync(c.seg_off, segoff, sizeof(segoff), cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemcpyAsync(c.seg_order, order, sizeof(order), cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemsetAsync(c.plan, 0, sizeof(PassPlan), c.st));
    if (n > 0) launch_init(c, p->pos, p->vel, p->mass, (const long long *)p->id);
    HBTU_CUDA(cudaStreamSynchronize(c.st));  // the stack copies above are consumed
    const int max_passes = params->max_passes > 0 ? params->max_passes : 10000;
    run_passes(c, max_passes, nullptr);
    launch_finalize(c, order_out, energy_out, res);
    int32_t status = 0;
    HBTU_CUDA(cudaMemcpyAsync(&status, &res->status, sizeof(status), cudaMemcpyDeviceToHost,
                              c.st));
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    if (status != 0) {
      set_global_error("hbtu_unbind_noalloc: max_passes reached without convergence");
      return HBTU_ERR_NOT_CONVERGED;
    }
    return HBTU_OK;
  } catch (const CudaError &e) {
    set_global_error("%s", e.what.c_str());
    // kernels already queued may still be writing the shared array: let them
    // finish, so the array is idle whenever this function returns
    cudaStreamSynchronize(stream);
    cudaGetLastError();
    return HBTU_ERR_CUDA;
  }
}
