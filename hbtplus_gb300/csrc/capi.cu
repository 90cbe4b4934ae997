// capi.cu -- the C ABI (include/hbtu.h) and the host side of the loop.
//
// The host drives one pass of the unbinding loop per iteration of a short
// loop: every kernel of a pass covers all still-active subhaloes of the batch,
// and the host reads back one small plan (active count, totals) per pass.
// The device workspace is one allocation carved into the buffers of Ctx and
// grown when a larger batch arrives.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "driver.h"
#include "handle.h"


namespace hbtu {

// Carves the workspace; with base == nullptr it only measures.
struct Carver {
  char *base;
  size_t off = 0;
  explicit Carver(char *b) : base(b) {}
  template <class T>
  T *take(size_t count)
  {
    off = (off + 255) / 256 * 256;
    T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
    off += sizeof(T) * (count ? count : 1);
    return p;
  }
};

static void carve(Carver &cv, Ctx &c, Staging &sg, long long N, long long S, bool sibling)
{
  const long long maxchunks = N / kChunk + S + 2;
  c.pm = cv.take<float4>(N);
  c.vel = cv.take<float4>(N);
  c.pseg = cv.take<int>(N);
  c.epid = cv.take<int>(N);
  c.epid2 = cv.take<int>(N);
  c.eE = cv.take<float>(N);
  c.eE2 = cv.take<float>(N);
  c.eR = cv.take<float>(N);
  c.epos_of_pid = cv.take<int>(N);
  c.coh_pid = cv.take<int>(N);
  c.seg = cv.take<SegState>(S);
  c.plan = cv.take<PassPlan>(1);
  c.seg_off = cv.take<int>(S + 1);
  c.seg_order = cv.take<int>(S);
  c.tree_base = cv.take<int>(S + 1);
  c.tgt_base = cv.take<int>(S + 1);
  c.tchunk_base = cv.take<int>(S + 1);
  c.bchunk_base = cv.take<int>(S + 1);
  c.ub_base = cv.take<int>(S + 1);
  c.plan_cnt = cv.take<int4>(S);
  c.plan_cnt2 = cv.take<int4>(S);
  c.plan_inter = cv.take<long long>(S);
  c.small_next = cv.take<int>(1);
  c.part_info = cv.take<int>(8 * S);
  c.chunk_bbox = cv.take<unsigned>(6 * maxchunks);
  c.chunk_sums = cv.take<double>(24 * maxchunks);
  c.sb.lo_a = cv.take<unsigned long long>(N);
  c.sb.lo_b = cv.take<unsigned long long>(N);
  c.sb.hi_a = cv.take<unsigned>(N);
  c.sb.hi_b = cv.take<unsigned>(N);
  c.sb.val_a = cv.take<int>(N);
  c.sb.val_b = cv.take<int>(N);
  c.sb.error = c.plan ? &c.plan->error : nullptr;
  c.sb.os_status = cv.take<unsigned>(sort_status_words(N));
  c.sb.os_ghist = cv.take<unsigned>(16 * 256);
  c.sb.os_goff = cv.take<unsigned>(16 * 256);
  c.scan_tmp = cv.take<char>(scan_tmp_bytes(N + 1));
  c.parentI = cv.take<int>(N);
  c.parentL = cv.take<int>(N);
  c.rfirst = cv.take<int>(N);
  c.rlast = cv.take<int>(N);
  c.dnode = cv.take<int>(N);
  c.iscell = cv.take<int>(N);
  c.cidx = cv.take<int>(N);
  c.cskip = cv.take<int>(N);
  c.cdepth = cv.take<int>(N);
  c.pcell = cv.take<int>(N);
  c.pending0 = cv.take<int>(N);
  c.cslot = cv.take<int>(8 * N);
  c.cell_list = cv.take<int>(N);
  c.chunk_list = cv.take<int>(N);
  c.lvl = cv.take<int>(96);
  c.pending = cv.take<int>(N);
  c.mask = cv.take<unsigned long long>(N);
  c.X = cv.take<long long>(N + 1);
  // one spare slot: the walk prefetches node cur+1 speculatively
  c.nd_abs = cv.take<float4>(2 * N + 1);
  c.nd = cv.take<WNode>(2 * N + 1);
  if (sibling) {  // the FP32 walk's copy of the nodes with each cell's children adjacent
    c.nd2 = cv.take<WNode>(2 * N + 1);
    c.newidx = cv.take<int>(2 * N + 1);
    c.X2 = cv.take<long long>(2 * N + 2);
    c.scan_tmp2 = cv.take<char>(scan_tmp_bytes(2 * N + 2));
  } else {
    c.nd2 = nullptr;
    c.newidx = nullptr;
    c.X2 = nullptr;
    c.scan_tmp2 = nullptr;
  }
  c.pcode = cv.take<long long>(N + 1);
  c.pX = cv.take<long long>(N + 1);
  c.Pk = cv.take<int>(N);
  c.Qk = cv.take<int>(N);
  sg.pos = cv.take<float>(3 * N);
  sg.vel = cv.take<float>(3 * N);
  sg.mass = cv.take<float>(N);
  sg.id = cv.take<long long>(N);
  sg.type = cv.take<int>(N);
  sg.order = cv.take<long long>(N);
  sg.energy = cv.take<float>(N);
  sg.pot = cv.take<double>(N);
  c.e_part = cv.take<double>(N);
  sg.grad = cv.take<float>(7 * N);
  sg.esum = cv.take<double>(S);
  sg.res = cv.take<hbtu_result>(S);
}

size_t workspace_bytes(long long N, long long S, bool sibling)
{
  Carver cv(nullptr);
  Ctx c;
  Staging sg;
  carve(cv, c, sg, N, S, sibling);
  return cv.off + 256;
}

void carve_workspace(char *base, Ctx &c, Staging &sg, long long N, long long S, bool sibling)
{
  Carver cv(base);
  carve(cv, c, sg, N, S, sibling);
}

// Message of the last failed call made without a handle (fixed buffer: the
// allocation-free entry point may write it).
thread_local char g_error_buf[512];

void set_global_error(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error_buf, sizeof(g_error_buf), fmt, ap);
  va_end(ap);
}

hbtu_status grow_workspace(hbtu_handle *h, size_t need)
{
  if (need <= h->ws_bytes) return HBTU_OK;
  if (h->ws) {
    cudaStreamSynchronize(h->stream);
    cudaFree(h->ws);
    h->ws = nullptr;
    h->ws_bytes = 0;
  }
  const size_t bytes = need + need / 4;  // headroom for the next, slightly larger call
  if (cudaMalloc(&h->ws, bytes) != cudaSuccess) {
    cudaGetLastError();
    h->ws = nullptr;
    h->err = "device workspace of " + std::to_string(bytes) + " bytes could not be allocated";
    return HBTU_ERR_OUT_OF_MEMORY;
  }
  h->ws_bytes = bytes;
  return HBTU_OK;
}

namespace {

int max_passes_of(const hbtu_params &p) { return p.max_passes > 0 ? p.max_passes : 10000; }


hbtu_status fail(hbtu_handle *h, hbtu_status st, const std::string &msg)
{
  if (h) h->err = msg;
  return st;
}

hbtu_status ensure_workspace(hbtu_handle *h, long long N, long long S)
{
  return grow_workspace(h, workspace_bytes(N, S));
}

void init_states(const hbtu_handle *h, long long S, const int64_t *offsets, const hbtu_state *st,
                 std::vector<SegState> &segs, std::vector<int> &segoff)
{
  const long long ms = h->params.max_sample_size;
  segs.assign(S, SegState());
  segoff.resize(S + 1);
  for (long long s = 0; s <= S; s++) segoff[s] = (int)offsets[s];
  for (long long s = 0; s < S; s++)
    init_segment(segs[s], (int)offsets[s], (int)(offsets[s + 1] - offsets[s]), st[s], ms);
}

// Shared set-up of a call: checks, workspace, staging, segment states, init kernel.
hbtu_status setup_call(hbtu_handle *h, const hbtu_particles *p, long long S, const int64_t *offsets,
                       const hbtu_state *st, Ctx &c, Staging &sg, bool &host)
{
  if (!h || !p || !offsets || !st || S < 0)
    return fail(h, HBTU_ERR_INVALID_ARGUMENT, "null handle, particles, offsets or states");
  if (p->location != HBTU_HOST && p->location != HBTU_DEVICE)
    return fail(h, HBTU_ERR_INVALID_ARGUMENT, "particles.location must be HBTU_HOST or HBTU_DEVICE");
  host = p->location == HBTU_HOST;
  if (offsets[0] != 0) return fail(h, HBTU_ERR_INVALID_ARGUMENT, "offsets[0] must be 0");
  for (long long s = 0; s < S; s++)
    if (offsets[s + 1] < offsets[s])
      return fail(h, HBTU_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
  const long long N = offsets[S];
  if (N >= HBTU_MAX_PARTICLES)
    return fail(h, HBTU_ERR_TOO_LARGE, "more than 2^30 particles in one call");
  if (S >= (1ll << 24))
    return fail(h, HBTU_ERR_TOO_LARGE, "more than 2^24 subhaloes in one call");
  if (N > 0 && (!p->id || !p->pos || !p->vel || !p->mass))
    return fail(h, HBTU_ERR_INVALID_ARGUMENT, "null id, pos, vel or mass array");
  hbtu_status rc = ensure_workspace(h, N, S);
  if (rc != HBTU_OK) return rc;
  HBTU_CUDA(cudaSetDevice(h->device));
  carve_workspace(h->ws, c, sg, N, S);
  c.P = h->dp;
  c.N = (int)N;
  c.S = (int)S;
  c.st = h->stream;
  c.plan_host = h->plan_host;
  c.pot_out = nullptr;
  c.grad_pos = c.grad_vel = c.grad_mass = nullptr;
  const float *pos = p->pos, *vel = p->vel, *mass = p->mass;
  const long long *id = (const long long *)p->id;
  c.type = (int *)p->type;
  if (host && N > 0) {
    HBTU_CUDA(cudaMemcpyAsync(sg.pos, p->pos, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemcpyAsync(sg.vel, p->vel, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemcpyAsync(sg.mass, p->mass, sizeof(float) * N, cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemcpyAsync(sg.id, p->id, sizeof(long long) * N, cudaMemcpyHostToDevice, c.st));
    if (p->type) {
      HBTU_CUDA(cudaMemcpyAsync(sg.type, p->type, sizeof(int) * N, cudaMemcpyHostToDevice, c.st));
      c.type = sg.type;
    }
    pos = sg.pos;
    vel = sg.vel;
    mass = sg.mass;
    id = sg.id;
  }
  c.id = (long long *)id;
  c.opt_leaf_runs = (int)h->opt_leaf_runs;
  c.opt_schedule = (int)h->opt_schedule;
  c.opt_layout = (int)h->opt_layout;
  std::vector<SegState> segs;
  std::vector<int> segoff, order(S);
  init_states(h, S, offsets, st, segs, segoff);
  for (long long s = 0; s < S; s++) order[s] = (int)s;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return segs[a].n > segs[b].n; });
  // the per-subhalo loop takes over small subhaloes (small.cu); the walk of
  // its blocks is the default one-target-per-lane schedule
  c.small_cap = h->opt_schedule == 0 ? (int)std::min<int64_t>(h->opt_small, kSmallCap) : 0;
  c.small_per_sm = (int)h->opt_small_per_sm;
  if (S > 0) {
    HBTU_CUDA(cudaMemcpyAsync(c.seg, segs.data(), sizeof(SegState) * S, cudaMemcpyHostToDevice,
                              c.st));
    HBTU_CUDA(cudaMemcpyAsync(c.seg_off, segoff.data(), sizeof(int) * (S + 1),
                              cudaMemcpyHostToDevice, c.st));
    HBTU_CUDA(cudaMemcpyAsync(c.seg_order, order.data(), sizeof(int) * S, cudaMemcpyHostToDevice,
                              c.st));
    // segs, segoff and order are pageable host temporaries: a copy from pageable
    // memory returns once its source has been staged, so they may go out of
    // scope now, and the host goes on queueing the call's kernels
  }
  HBTU_CUDA(cudaMemsetAsync(c.plan, 0, sizeof(PassPlan), c.st));
  if (N > 0) launch_init(c, pos, vel, mass, id);
  return HBTU_OK;
}

cudaEvent_t event_at(hbtu_handle *h, size_t k)
{
  while (h->events.size() <= k) {
    cudaEvent_t e;
    HBTU_CUDA(cudaEventCreate(&e));
    h->events.push_back(e);
  }
  return h->events[k];
}

// Phase timer: with timing on, events bracket tree / walk / loop kernels of
// each pass; elapsed times are read once the stream has passed them.
struct PhaseTimer : LoopHooks {
  hbtu_handle *h;
  cudaStream_t st;
  size_t next = 2;  // events 0, 1 bracket the whole call
  std::vector<size_t> marks;
  PhaseTimer(hbtu_handle *hh, cudaStream_t s) : h(hh), st(s) { stats = &hh->stats; }
  void mark() override
  {
    if (!h->timing) return;
    HBTU_CUDA(cudaEventRecord(event_at(h, next), st));
    marks.push_back(next++);
  }
  // the per-subhalo loop of the small subhaloes (its own pair of events)
  int small_ev[2] = {-1, -1};
  void small_begin() override
  {
    if (!h->timing) return;
    HBTU_CUDA(cudaEventRecord(event_at(h, next), st));
    small_ev[0] = (int)next++;
  }
  void small_end() override
  {
    if (!h->timing) return;
    HBTU_CUDA(cudaEventRecord(event_at(h, next), st));
    small_ev[1] = (int)next++;
  }
  // marks come in groups of 4: before tree, after tree, after walk, after loop
  int group = 0;  // pass groups collected in this call
  void collect() override
  {
    if (small_ev[0] >= 0 && small_ev[1] >= 0) {
      float ms = 0.f;
      HBTU_CUDA(cudaEventElapsedTime(&ms, h->events[small_ev[0]], h->events[small_ev[1]]));
      h->stats.small_ms += ms;
      small_ev[0] = small_ev[1] = -1;
    }
    for (size_t i = 0; i + 3 < marks.size(); i += 4) {
      float a = 0, b = 0, c = 0;
      HBTU_CUDA(cudaEventElapsedTime(&a, h->events[marks[i]], h->events[marks[i + 1]]));
      HBTU_CUDA(cudaEventElapsedTime(&b, h->events[marks[i + 1]], h->events[marks[i + 2]]));
      HBTU_CUDA(cudaEventElapsedTime(&c, h->events[marks[i + 2]], h->events[marks[i + 3]]));
      h->stats.tree_ms += a;
      h->stats.walk_ms += b;
      h->stats.loop_ms += c;
      if (group++ == 0) h->stats.walk1_ms += b;
    }
    marks.clear();
    next = 2;
  }
};

hbtu_status run_loop(hbtu_handle *h, Ctx &c)
{
  PhaseTimer pt(h, c.st);
  run_passes(c, max_passes_of(h->params), &pt);
  return HBTU_OK;
}

}  // namespace

void init_segment(SegState &g, int off, int n, const hbtu_state &st, long long maxsample)
{
  memset(&g, 0, sizeof(g));
  g.off = off;
  g.n = n;
  g.status = n <= 1 ? SEG_TRIVIAL : SEG_ACTIVE;
  g.nbound = g.nlast = n;
  g.mode = MODE_FULL;
  g.first_mb = INT_MAX;
  const bool sampling = maxsample > 0 && n > maxsample;
  g.t0 = 0;
  g.ntree = sampling ? (int)maxsample : n;
  g.mfac = sampling ? (float)n / (float)maxsample : 1.f;  // (HBTReal)Nlast/MaxSampleSize
  g.ntgt = n;
  g.tgt_mode = sampling ? 2 : 0;
  for (int j = 0; j < 3; j++) {
    g.ref_pos[j] = st.ref_pos[j];
    g.ref_vel[j] = st.ref_vel[j];
    g.mb_pos[j] = st.mostbound_pos[j];
    g.mb_vel[j] = st.mostbound_vel[j];
  }
  g.mb_id = st.mostbound_id;
}

void read_plan(Ctx &c)
{
  HBTU_CUDA(cudaMemcpyAsync(c.plan_host, c.plan, sizeof(PassPlan), cudaMemcpyDeviceToHost, c.st));
  HBTU_CUDA(cudaStreamSynchronize(c.st));
  if (c.plan_host->error) throw CudaError(cudaErrorLaunchTimeout, "radix sort look-back", __FILE__, __LINE__);
}

// One pass's tree and energies for every active subhalo.
void pass_tree_and_energies(Ctx &c, LoopHooks *hk)
{
  const PassPlan pl = *c.plan_host;
  if (hk) hk->mark();
  launch_tree_build(c, pl);
  if (hk) hk->mark();
  launch_walk(c, pl);
  if (hk && hk->stats) hk->stats->walk_launches += pl.ntgt_total > 0;
  if (hk) hk->mark();
}

// The unbinding loop of all subhaloes of a call (src/subhalo_unbind.cpp:310-422),
// then the final energy sort and RefineBindingEnergyOrder.  One host read of a
// small plan per pass.
void run_passes(Ctx &c, int max_passes, LoopHooks *hk)
{
  const int max_chunks = c.N / kChunk + c.S + 1;
  for (int pass = 0;; pass++) {
    launch_plan(c, 0);
    launch_bbox_cube(c, max_chunks);
    read_plan(c);
    if (hk) hk->collect();
    const PassPlan pl = *c.plan_host;
    if (pass == 1 && hk && hk->stats) hk->stats->walk1_interactions += pl.inter_done;
    launch_block_sort(c, pl.nsort_total, 0);  // unbound blocks of the previous pass
    if (pl.nactive == 0) break;
    if (pl.max_nlast <= c.small_cap) {
      // every active subhalo is small: one block per subhalo runs its
      // remaining passes to the end (small.cu), and the loop is done
      if (hk) hk->small_begin();
      launch_small(c, c.small_cap, pl.nactive, max_passes);
      if (hk) hk->small_end();
      if (hk && hk->stats) hk->stats->small_subhaloes += pl.nactive;
      break;
    }
    if (hk && hk->stats) hk->stats->passes++;
    pass_tree_and_energies(c, hk);
    launch_partition(c);
    launch_averages_control(c, max_passes);
    if (hk) hk->mark();
  }
  launch_plan(c, 2);
  read_plan(c);
  if (hk) hk->collect();
  const int nrefine = c.plan_host->nrefine;
  launch_block_sort(c, c.plan_host->nsort_total, 1);  // bound blocks (:405)
  if (nrefine > 0) {  // RefineBindingEnergyOrder (:406-407)
    launch_refine_mode(c, 1);
    launch_plan(c, 0);
    launch_bbox_cube(c, max_chunks);
    read_plan(c);
    pass_tree_and_energies(c, nullptr);
    launch_refine_mode(c, 0);
    launch_plan(c, 3);
    read_plan(c);
    launch_block_sort(c, c.plan_host->nsort_total, 2);
    launch_plan(c, 2);  // chunk plan of the kinematics
  }
}

DevParams derive_params(const hbtu_params &p)
{
  DevParams d;
  memset(&d, 0, sizeof(d));
  const float th = (float)p.open_angle;
  d.eps = (float)p.softening;
  d.theta2 = th * th;
  d.box = (float)p.box_size;
  d.boxhalf = (float)((double)d.box / 2.);
  d.res = (float)((double)d.eps * 0.1);
  d.reshalf = (float)((double)d.res / 2.);
  d.G = (float)p.G;
  d.Hz = (float)p.hubble;
  d.a = (float)p.scale_factor;
  d.prec = (float)p.bound_mass_precision;
  d.periodic = p.periodic != 0;
  d.refine = (p.max_sample_size > 0 && p.refine_mostbound);
  d.minpart = (int)std::min<int64_t>(p.min_num_part, INT_MAX);
  d.precision = p.precision;
  d.maxsample = p.max_sample_size;
  d.h = 2.8 * (double)d.eps;
  d.h_inv = 1.0 / d.h;
  return d;
}

}  // namespace hbtu

using namespace hbtu;

extern "C" {

int32_t hbtu_version(void) { return 10100; }

const char *hbtu_last_error(const hbtu_handle *h)
{
  return h ? h->err.c_str() : g_error_buf;
}

hbtu_status hbtu_create(const hbtu_params *params, hbtu_handle **out)
{
  if (!params || !out) {
    set_global_error("null params or output pointer");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  if (!(params->softening > 0) || !(params->open_angle >= 0) ||
      !(params->bound_mass_precision > 0 && params->bound_mass_precision <= 1) ||
      params->min_num_part < 0 || params->max_sample_size < 0 ||
      (params->periodic && !(params->box_size > 0)) || !(params->scale_factor > 0) ||
      (params->precision != HBTU_PRECISION_FP32 && params->precision != HBTU_PRECISION_FP64)) {
    set_global_error(
        "invalid parameters: need softening > 0, open_angle >= 0, 0 < bound_mass_precision <= 1, "
        "min_num_part >= 0, max_sample_size >= 0, box_size > 0 when periodic, scale_factor > 0, "
        "precision FP32 or FP64");
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= params->device || params->device < 0) {
    cudaGetLastError();
    set_global_error("no CUDA device %d", params->device);
    return HBTU_ERR_NO_DEVICE;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, params->device) != cudaSuccess || prop.major != 10 ||
      prop.minor != 3) {
    cudaGetLastError();
    set_global_error("device %d is not compute capability 10.3 (this library is built for sm_103a "
                     "only)",
                     params->device);
    return HBTU_ERR_NO_DEVICE;
  }
  hbtu_handle *h = new (std::nothrow) hbtu_handle();
  if (!h) {
    set_global_error("out of host memory");
    return HBTU_ERR_OUT_OF_MEMORY;
  }
  h->params = *params;
  h->dp = derive_params(*params);
  h->device = params->device;
  if (cudaSetDevice(h->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost(&h->plan_host, sizeof(PassPlan)) != cudaSuccess) {
    set_global_error("CUDA set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return HBTU_ERR_CUDA;
  }
  h->stream = h->own_stream;
  *out = h;
  return HBTU_OK;
}

hbtu_status hbtu_destroy(hbtu_handle *h)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->ws) cudaFree(h->ws);
  if (h->plan_host) cudaFreeHost(h->plan_host);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return HBTU_OK;
}

hbtu_status hbtu_set_option(hbtu_handle *h, const char *name, int64_t value)
{
  if (!h || !name) return HBTU_ERR_INVALID_ARGUMENT;
  const std::string n(name);
  if (n == "walk_leaf_runs") {
    if (value != 0 && value != 1) return fail(h, HBTU_ERR_INVALID_ARGUMENT, "walk_leaf_runs: 0 or 1");
    h->opt_leaf_runs = value;
    return HBTU_OK;
  }
  if (n == "walk_schedule") {
    if (value != 0 && value != 1) return fail(h, HBTU_ERR_INVALID_ARGUMENT, "walk_schedule: 0 or 1");
    h->opt_schedule = value;
    return HBTU_OK;
  }
  if (n == "walk_layout") {
    if (value != 0 && value != 1) return fail(h, HBTU_ERR_INVALID_ARGUMENT, "walk_layout: 0 or 1");
    h->opt_layout = value;
    return HBTU_OK;
  }
  if (n == "small_cutoff") {
    if (value < 0 || value > kSmallCap)
      return fail(h, HBTU_ERR_INVALID_ARGUMENT,
                  "small_cutoff: 0 (off) to " + std::to_string(kSmallCap));
    h->opt_small = value;
    return HBTU_OK;
  }
  if (n == "small_blocks_per_sm") {
    if (value < 1 || value > 8)
      return fail(h, HBTU_ERR_INVALID_ARGUMENT, "small_blocks_per_sm: 1 to 8");
    h->opt_small_per_sm = value;
    return HBTU_OK;
  }
  return fail(h, HBTU_ERR_INVALID_ARGUMENT, "unknown option " + n);
}

hbtu_status hbtu_get_option(const hbtu_handle *h, const char *name, int64_t *value)
{
  if (!h || !name || !value) return HBTU_ERR_INVALID_ARGUMENT;
  const std::string n(name);
  if (n == "walk_leaf_runs") {
    *value = h->opt_leaf_runs;
    return HBTU_OK;
  }
  if (n == "walk_schedule") {
    *value = h->opt_schedule;
    return HBTU_OK;
  }
  if (n == "walk_layout") {
    *value = h->opt_layout;
    return HBTU_OK;
  }
  if (n == "small_cutoff") {
    *value = h->opt_small;
    return HBTU_OK;
  }
  if (n == "small_blocks_per_sm") {
    *value = h->opt_small_per_sm;
    return HBTU_OK;
  }
  return HBTU_ERR_INVALID_ARGUMENT;
}

hbtu_status hbtu_set_timing(hbtu_handle *h, int32_t on)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  h->timing = on != 0;
  return HBTU_OK;
}

hbtu_status hbtu_get_stats(const hbtu_handle *h, hbtu_stats *out)
{
  if (!h || !out) return HBTU_ERR_INVALID_ARGUMENT;
  *out = h->stats;
  return HBTU_OK;
}

hbtu_status hbtu_reset_stats(hbtu_handle *h)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  memset(&h->stats, 0, sizeof(h->stats));
  return HBTU_OK;
}

hbtu_status hbtu_set_stream(hbtu_handle *h, void *cuda_stream)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  h->stream = (cudaStream_t)cuda_stream;  // NULL: the legacy default stream
  return HBTU_OK;
}

hbtu_status hbtu_unbind_batch(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                              const int64_t *offsets, const hbtu_state *st, int64_t *order_out,
                              float *energy_out, hbtu_result *res)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (nsub > 0 && (!order_out || !energy_out || !res))
    return fail(h, HBTU_ERR_INVALID_ARGUMENT, "null output array");
  try {
    Ctx c;
    Staging sg;
    bool host = true;
    const long long launches0 = g_launches;
    HBTU_CUDA(cudaSetDevice(h->device));
    HBTU_CUDA(cudaEventRecord(event_at(h, 0), h->stream));
    hbtu_status rc = setup_call(h, p, nsub, offsets, st, c, sg, host);
    if (rc != HBTU_OK) return rc;
    if (nsub == 0) return HBTU_OK;
    run_loop(h, c);
    const long long N = c.N;
    long long *ord = host ? sg.order : (long long *)order_out;
    float *en = host ? sg.energy : energy_out;
    hbtu_result *rs = host ? sg.res : res;
    launch_finalize(c, (int64_t *)ord, en, rs);
    if (host) {
      if (N > 0) {
        HBTU_CUDA(cudaMemcpyAsync(order_out, ord, sizeof(long long) * N, cudaMemcpyDeviceToHost,
                                  c.st));
        HBTU_CUDA(cudaMemcpyAsync(energy_out, en, sizeof(float) * N, cudaMemcpyDeviceToHost, c.st));
      }
      HBTU_CUDA(cudaMemcpyAsync(res, rs, sizeof(hbtu_result) * nsub, cudaMemcpyDeviceToHost, c.st));
    }
    HBTU_CUDA(cudaEventRecord(event_at(h, 1), c.st));
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    {
      float ms = 0.f;
      HBTU_CUDA(cudaEventElapsedTime(&ms, h->events[0], h->events[1]));
      h->stats.total_ms += ms;
      h->stats.calls++;
      h->stats.kernel_launches += g_launches - launches0;
      if (host)
        for (int64_t s = 0; s < nsub; s++) {
          h->stats.evaluations += res[s].evaluations;
          h->stats.interactions += res[s].interactions;
        }
    }
    if (host)
      for (int64_t s = 0; s < nsub; s++)
        if (res[s].status != 0) {
          h->err = "subhalo " + std::to_string(s) + " reached max_passes without converging";
          return HBTU_ERR_NOT_CONVERGED;
        }
    return HBTU_OK;
  } catch (const CudaError &e) {
    return fail(h, HBTU_ERR_CUDA, e.what);
  } catch (const std::bad_alloc &) {
    return fail(h, HBTU_ERR_OUT_OF_MEMORY, "out of host memory");
  }
}

hbtu_status hbtu_unbind(hbtu_handle *h, const hbtu_particles *p, int64_t n, const hbtu_state *st,
                        int64_t *order_out, float *energy_out, hbtu_result *res)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (n < 0) return fail(h, HBTU_ERR_INVALID_ARGUMENT, "negative particle count");
  const int64_t offsets[2] = {0, n};
  return hbtu_unbind_batch(h, p, 1, offsets, st, order_out, energy_out, res);
}

hbtu_status hbtu_energy_gradient(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                                 const int64_t *offsets, const hbtu_state *st, double *energy_out,
                                 float *grad_pos, float *grad_vel, float *grad_mass)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (nsub > 0 && !energy_out) return fail(h, HBTU_ERR_INVALID_ARGUMENT, "null energy_out");
  try {
    Ctx c;
    Staging sg;
    bool host = true;
    const long long launches0 = g_launches;
    // a single full pass over every particle: no sampling
    const int64_t saved = h->params.max_sample_size;
    h->params.max_sample_size = 0;
    hbtu_status rc = setup_call(h, p, nsub, offsets, st, c, sg, host);
    h->params.max_sample_size = saved;
    if (rc != HBTU_OK) return rc;
    if (nsub == 0) return HBTU_OK;
    const long long N = c.N;
    c.grad_pos = grad_pos ? (host ? sg.grad : grad_pos) : nullptr;
    c.grad_vel = grad_vel ? (host ? sg.grad + 3 * N : grad_vel) : nullptr;
    c.grad_mass = grad_mass ? (host ? sg.grad + 6 * N : grad_mass) : nullptr;
    // every subhalo with at least one particle takes part (n == 1 included)
    std::vector<SegState> segs(nsub);
    HBTU_CUDA(cudaMemcpyAsync(segs.data(), c.seg, sizeof(SegState) * nsub, cudaMemcpyDeviceToHost,
                              c.st));
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    for (auto &g : segs)
      if (g.n >= 1) g.status = SEG_ACTIVE;
    HBTU_CUDA(cudaMemcpyAsync(c.seg, segs.data(), sizeof(SegState) * nsub, cudaMemcpyHostToDevice,
                              c.st));
    if (N > 0) HBTU_CUDA(cudaMemsetAsync(c.e_part, 0, sizeof(double) * N, c.st));
    launch_plan(c, 0);
    launch_bbox_cube(c, c.N / kChunk + c.S + 1);
    read_plan(c);
    const PassPlan pl = *c.plan_host;
    launch_tree_build(c, pl);
    launch_grad_walk(c, pl);
    double *es = host ? sg.esum : energy_out;
    launch_segment_sums(c, c.e_part, es);
    if (host) {
      HBTU_CUDA(cudaMemcpyAsync(energy_out, es, sizeof(double) * nsub, cudaMemcpyDeviceToHost,
                                c.st));
      if (grad_pos)
        HBTU_CUDA(cudaMemcpyAsync(grad_pos, c.grad_pos, sizeof(float) * 3 * N,
                                  cudaMemcpyDeviceToHost, c.st));
      if (grad_vel)
        HBTU_CUDA(cudaMemcpyAsync(grad_vel, c.grad_vel, sizeof(float) * 3 * N,
                                  cudaMemcpyDeviceToHost, c.st));
      if (grad_mass)
        HBTU_CUDA(cudaMemcpyAsync(grad_mass, c.grad_mass, sizeof(float) * N,
                                  cudaMemcpyDeviceToHost, c.st));
    }
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    h->stats.kernel_launches += g_launches - launches0;
    return HBTU_OK;
  } catch (const CudaError &e) {
    return fail(h, HBTU_ERR_CUDA, e.what);
  }
}

hbtu_status hbtu_direct_potential(hbtu_handle *h, const hbtu_particles *p, int64_t n,
                                  const int64_t *targets, int64_t ntarget, double *potential_out)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (n < 0 || ntarget < 0 || (ntarget > 0 && (!targets || !potential_out)))
    return fail(h, HBTU_ERR_INVALID_ARGUMENT, "bad count, target list or output pointer");
  for (int64_t k = 0; k < ntarget; k++)
    if (targets[k] < 0 || targets[k] >= n)
      return fail(h, HBTU_ERR_INVALID_ARGUMENT, "target index out of range");
  int *d_t = nullptr;
  double *d_out = nullptr, *d_part = nullptr;
  try {
    hbtu_state st;
    memset(&st, 0, sizeof(st));
    st.mostbound_id = -1;
    const int64_t offsets[2] = {0, n};
    Ctx c;
    Staging sg;
    bool host = true;
    hbtu_status rc = setup_call(h, p, 1, offsets, &st, c, sg, host);
    if (rc != HBTU_OK) return rc;
    if (ntarget == 0) return HBTU_OK;
    const int tiles = (int)((ntarget + 127) / 128);
    const int nsplit = std::max(1, std::min(512, (16 * 152 + tiles - 1) / tiles));
    std::vector<int> t32(targets, targets + ntarget);
    if (cudaMalloc(&d_t, sizeof(int) * ntarget) != cudaSuccess ||
        cudaMalloc(&d_out, sizeof(double) * ntarget) != cudaSuccess ||
        cudaMalloc(&d_part, sizeof(double) * ntarget * nsplit) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(d_t);
      cudaFree(d_out);
      cudaFree(d_part);
      return fail(h, HBTU_ERR_OUT_OF_MEMORY, "direct potential buffers");
    }
    HBTU_CUDA(cudaMemcpyAsync(d_t, t32.data(), sizeof(int) * ntarget, cudaMemcpyHostToDevice,
                              c.st));
    direct_potential_fp64(c.P, c.pm, c.N, d_t, (int)ntarget, d_out, d_part, nsplit, c.st);
    HBTU_CUDA(cudaMemcpyAsync(potential_out, d_out, sizeof(double) * ntarget,
                              host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, c.st));
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    cudaFree(d_t);
    cudaFree(d_out);
    cudaFree(d_part);
    return HBTU_OK;
  } catch (const CudaError &e) {
    cudaFree(d_t);
    cudaFree(d_out);
    cudaFree(d_part);
    return fail(h, HBTU_ERR_CUDA, e.what);
  }
}

hbtu_status hbtu_binding_energies(hbtu_handle *h, const hbtu_particles *p, int64_t n,
                                  const float ref_pos[3], const float ref_vel[3],
                                  float *energy_out, double *potential_out)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (n < 0 || !ref_pos || !ref_vel || (n > 0 && !energy_out))
    return fail(h, HBTU_ERR_INVALID_ARGUMENT, "bad count, frame or output pointer");
  try {
    hbtu_state st;
    memset(&st, 0, sizeof(st));
    for (int j = 0; j < 3; j++) {
      st.ref_pos[j] = ref_pos[j];
      st.ref_vel[j] = ref_vel[j];
    }
    st.mostbound_id = -1;
    const int64_t offsets[2] = {0, n};
    Ctx c;
    Staging sg;
    bool host = true;
    // one exact full pass: no sampling
    const int64_t saved = h->params.max_sample_size;
    h->params.max_sample_size = 0;
    hbtu_status rc = setup_call(h, p, 1, offsets, &st, c, sg, host);
    h->params.max_sample_size = saved;
    if (rc != HBTU_OK) return rc;
    if (n == 0) return HBTU_OK;
    SegState one;
    HBTU_CUDA(cudaMemcpyAsync(&one, c.seg, sizeof(SegState), cudaMemcpyDeviceToHost, c.st));
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    one.status = SEG_ACTIVE;  // n == 1 runs the pass too
    HBTU_CUDA(cudaMemcpyAsync(c.seg, &one, sizeof(SegState), cudaMemcpyHostToDevice, c.st));
    c.pot_out = (host || !potential_out) ? sg.pot : potential_out;
    launch_plan(c, 0);
    launch_bbox_cube(c, c.N / kChunk + 2);
    read_plan(c);
    pass_tree_and_energies(c, nullptr);
    float *en = host ? sg.energy : energy_out;
    HBTU_CUDA(cudaMemcpyAsync(en, c.eE, sizeof(float) * n, cudaMemcpyDeviceToDevice, c.st));
    if (host) {
      HBTU_CUDA(cudaMemcpyAsync(energy_out, en, sizeof(float) * n, cudaMemcpyDeviceToHost, c.st));
      if (potential_out)
        HBTU_CUDA(cudaMemcpyAsync(potential_out, sg.pot, sizeof(double) * n,
                                  cudaMemcpyDeviceToHost, c.st));
    }
    HBTU_CUDA(cudaStreamSynchronize(c.st));
    return HBTU_OK;
  } catch (const CudaError &e) {
    return fail(h, HBTU_ERR_CUDA, e.what);
  }
}

}  // extern "C"
