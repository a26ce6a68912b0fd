// itn_api.cu -- the C ABI of libitn_gpu.so (declared in include/itn_gpu.h).
//
// Host-side responsibilities: validate arguments, keep the network (CSR) and the
// per-vertex op programs, own device buffers, and drive the solve loop.  The whole
// beliefpropagation solve runs on the device: each outer iteration is one sweep
// launch plus a one-thread convergence check that raises a device flag; later sweeps
// see the flag and return at once, so a fixed launch sequence (captured once as a
// CUDA graph) reproduces StopAfterIteration(maxiter) | StopWhenConverged(tol)
// without a host round trip per iteration.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/itn_gpu.h"
#include "itn_common.cuh"
#include "itn_internal.h"
#include "itn_tc.h"
#include "itn_contract.h"
#include "itn_apply.h"
#include "itn_z3.h"
#include <nvtx3/nvToolsExt.h>

using namespace itn;

namespace {

// Size classes of the two-layer parallel sweep, for networks with at least
// kSmallMinItemsPerSm items per SM: vertices of at most kClassMax[i] tensor entries (and more
// than the next bound) form class i + 1, launched after the larger ones with CTAs of
// kClassBlock[i] threads and shared staging sized for that class alone; the vertices above
// kClassMax[0] keep the tuned CTA size.  Small CTAs with small staging let many items share
// an SM (one warp: a single-warp barrier).  Batched complex64 networks (random 3-regular,
// bonds 2..8): one launch 1.12e8 updates/s; <= 256 entries in 32-thread CTAs 1.37e8 (64
// threads 1.19e8); + 257..512 in 64-thread CTAs 1.39e8; + <= 64 entries apart 1.42e8.
constexpr int kNumSubClasses = 3;
constexpr int64_t kClassMax[kNumSubClasses] = {512, 256, 64};
constexpr int kClassBlock[kNumSubClasses] = {64, 32, 32};
constexpr int kSmallMinItemsPerSm = 16;

// Device allocations that itn_inject_fault(ITN_FAULT_ALLOC) has told the calling thread to
// fail (a host-side stand-in for running out of device memory).
thread_local int64_t t_fail_allocs = 0;

// NVTX range for the lifetime of a scope: every C entry point opens one named after itself,
// and a solve opens one per chunk of sweeps (tools such as Nsight Systems show them; without
// a tool attached the calls return at once).
struct NvtxScope {
  explicit NvtxScope(const char* name) { nvtxRangePushA(name); }
  ~NvtxScope() { nvtxRangePop(); }
  NvtxScope(const NvtxScope&) = delete;
  NvtxScope& operator=(const NvtxScope&) = delete;
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;  // owns p: never copied
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (t_fail_allocs > 0) {
      --t_fail_allocs;
      return cudaErrorMemoryAllocation;
    }
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct Program {
  std::vector<uint32_t> ops;
  int nbuf = 1;
};

// Leave-one-out program generator (see bp_generic.cu): buffer 0 holds the site
// tensor; absorb chains ping-pong between two scratch buffers.
struct ProgGen {
  std::vector<uint32_t> ops;
  std::vector<int> free_list;
  int next = 1;
  int high = 1;
  int alloc() {
    int b;
    if (!free_list.empty()) {
      b = free_list.back();
      free_list.pop_back();
    } else {
      b = next++;
    }
    high = std::max(high, b + 1);
    return b;
  }
  void release(int b) {
    if (b > 0) free_list.push_back(b);
  }
  int absorb_chain(int src, const std::vector<int>& legs) {
    if (legs.empty()) return src;
    const int n = (int)legs.size();
    const int res = alloc();
    const int tmp = n > 1 ? alloc() : -1;
    int cur = src;
    for (int j = 0; j < n; ++j) {
      const int dst = ((n - 1 - j) % 2 == 0) ? res : tmp;
      ops.push_back(make_op(OP_ABSORB, cur, dst, legs[j]));
      cur = dst;
    }
    if (tmp >= 0) release(tmp);
    return res;
  }
  void loo(int cur, const std::vector<int>& L) {
    if (L.size() == 1) {
      ops.push_back(make_op(OP_FINAL, cur, 0, L[0]));
      return;
    }
    const size_t h = (L.size() + 1) / 2;
    std::vector<int> L1(L.begin(), L.begin() + h), L2(L.begin() + h, L.end());
    int b = absorb_chain(cur, L2);
    loo(b, L1);
    if (b != cur) release(b);
    b = absorb_chain(cur, L1);
    loo(b, L2);
    if (b != cur) release(b);
  }
};

// kind 0: outgoing messages for the legs in mask (leave-one-out); 1: vertex scalar
// (absorb every leg, FULL); 2: absorb every leg, DUMP (gradient of Z_u).
Program make_program(int z, uint32_t mask, int kind) {
  ProgGen g;
  if (kind != 0) {
    std::vector<int> all;
    for (int l = 0; l < z; ++l) all.push_back(l);
    int b = g.absorb_chain(0, all);
    g.ops.push_back(make_op(kind == 1 ? OP_FULL : OP_DUMP, b, 0, 0));
  } else {
    std::vector<int> others, req;
    for (int l = 0; l < z; ++l) ((mask >> l) & 1u ? req : others).push_back(l);
    int b = g.absorb_chain(0, others);
    if (!req.empty()) g.loo(b, req);
  }
  Program p;
  p.ops = g.ops;
  p.nbuf = g.high;
  return p;
}

}  // namespace

struct itn_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  int sm_count = 0;
  int smem_optin = 0;

  // network (host)
  bool have_graph = false;
  int64_t nv = 0, nslots = 0;
  int layers = 2;
  std::vector<int64_t> off, nbr, rev, toff, moff;
  std::vector<int32_t> bond, phys, net;
  int n_nets = 1;
  int max_d2 = 1;
  int64_t max_tensor = 1;
  std::vector<int> eslots;  // undirected edges: slot < rev[slot]
  bool scal_d8 = false;     // every vertex: two layers, d = 2, four legs of dimension 8
  // every vertex: two layers, three legs of dimension <= 8, at most 1024 tensor entries
  // (the grouped sweep of bp_z3.cu); items_z3 sorted by tensor size, largest first
  bool z3 = false;
  std::vector<int> items_z3;
  std::vector<double> z3_work;      // per item: entries x (D0 + D1 + D2), the sweep's cost share
  std::vector<Z3Meta> meta_z3;      // per item: tensor / message offsets and bond dimensions
  DevBuf d_items_z3, d_meta_z3;
  std::array<int, 4> z3_budget{{0, 0, 0, 0}};  // autotuned shared memory per CTA (bytes), per dtype
  std::array<int, 4> z3_mult{{0, 0, 0, 0}};    // autotuned CTAs per resident CTA slot
  std::array<int, 4> z3_k0{{0, 0, 0, 0}};      // autotuned fixed cost per vertex (work units)
  // Parallel-sweep items in size classes (items_par is sorted by tensor size, largest
  // first), in launch order: contiguous item ranges with their own staging limits and CTA
  // size; a single class uses the whole network's limits and the tuned CTA size.
  struct ItemClass {
    int begin = 0, end = 0;
    bool own = false;  // own limits (a sub-class), else the network's and the tuned size
    int64_t max_tensor = 1;
    int msg_cap = 1, max_d2 = 1, block = 0;
  };
  std::vector<ItemClass> par_classes;

  // network (device)
  DevBuf d_off, d_rev, d_bond, d_phys, d_toff, d_moff, d_eslots;
  DevBuf d_net_voff, d_net_vlist, d_net_eoff, d_net_elist;

  // programs and work lists
  std::map<std::pair<int, uint32_t>, int> prog_index;  // (z, mask|full bit) -> offset
  std::vector<uint32_t> prog_host;
  DevBuf d_prog;
  bool prog_dirty = true;
  int nbuf = 1;
  int msg_cap = 1;
  std::vector<int> items_par, items_scal, items_dump;
  DevBuf d_items_par, d_items_scal, d_items_dump;
  std::vector<int> slot_dst, slot_eidx;  // per slot: destination vertex, undirected edge index
  DevBuf d_slot_dst, d_slot_eidx;
  // gradient work buffers
  DevBuf d_grad, d_U, d_F, d_S, d_g, d_lam, d_mu, d_mu2, d_cot, d_adj, d_adjgrid, d_sweepgrid;
  bool no_persist_adj = false;     // itn_inject_fault(ITN_FAULT_NO_PERSISTENT_ADJOINT)
  bool no_persist_sweeps = false;  // itn_inject_fault(ITN_FAULT_NO_PERSISTENT_SWEEPS)
  DevBuf d_ckpt, d_seg;  // unrolled gradient: kept sweep states, recomputed segment
  std::map<std::vector<int64_t>, std::pair<std::vector<int>, std::shared_ptr<DevBuf>>> seq_plans;

  // data
  int dtype = -1;
  bool have_tensors = false, have_messages = false;
  DevBuf d_tens;
  DevBuf d_msg[2];
  int cur = 0;
  DevBuf d_zv, d_ze, d_logzv, d_logze, d_tot, d_flags, d_lspart;
  DevBuf d_scratch;
  DevBuf d_stage;  // upload staging
  // pinned host staging for small results read back together (one copy, one sync)
  void* h_pin = nullptr;
  size_t h_pin_bytes = 0;
  // a solve whose last host synchronisation was left to the caller (itn_bp_solve)
  struct {
    bool active = false;
    bool use_tol = false;
    bool tc = false;
    int launches = 0;
    float ms_before = 0.f;
  } pending;
  // a solve queued by itn_bp_solve_submit and not yet completed by itn_bp_solve_wait: it owns
  // the stream's results and the pinned staging until then
  struct {
    bool active = false;
    bool logz = false;
    itn_bp_result res{};  // the result of a solve that completed inside the submit call
  } submitted;

  // convergence state (device): dmax, nan, done, at, iters, delta, counter
  DevBuf d_slot_diff, d_state;

  // cached solve graphs and the number of kernel launches each holds
  std::map<std::string, cudaGraphExec_t> graphs;
  std::map<std::string, int> graph_launches;
  // CTA size chosen by the autotuner for the parallel sweep, per dtype (0: not tuned)
  std::vector<int> tuned_block = std::vector<int>(4, 0);
  std::vector<int> dual_block = std::vector<int>(4, 0);  // CTA size of the dual (gradient) launches
  uint64_t net_sig = 0;  // hash of the uploaded network's structure (keys the tuning cache)

  // tensor-core engine (bp_tc.cu), created on first use
  TcEngine* tc = nullptr;
  // limit of the tensor-core sweep's waits on other items' messages (itn_inject_fault)
  uint64_t wait_ns = kDefaultWaitNs;
  int stall = 0;  // itn_inject_fault(ITN_FAULT_STALL)

  ~itn_ctx() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    if (h_pin) cudaFreeHost(h_pin);
    if (tc) tc_destroy(tc);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int fail(itn_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_fail(itn_ctx* c, cudaError_t e, const char* what) {
  cudaGetLastError();
  const int code = (e == cudaErrorMemoryAllocation) ? ITN_ERR_OOM : ITN_ERR_CUDA;
  return fail(c, code, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                          \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
  } while (0)

int ensure_device(itn_ctx* c) {
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  return ITN_OK;
}

// Pinned host staging of at least `bytes` (grown, never shrunk).
int ensure_pinned(itn_ctx* c, size_t bytes) {
  if (bytes <= c->h_pin_bytes) return ITN_OK;
  if (c->h_pin) {
    CK(cudaStreamSynchronize(c->stream));
    cudaFreeHost(c->h_pin);
    c->h_pin = nullptr;
    c->h_pin_bytes = 0;
  }
  const size_t want = std::max<size_t>(bytes, 4096);
  CK(cudaMallocHost(&c->h_pin, want));
  c->h_pin_bytes = want;
  return ITN_OK;
}

template <typename T>
int upload_vec(itn_ctx* c, DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  CK(b.ensure(std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return ITN_OK;
}

int program_offset(itn_ctx* c, int z, uint32_t mask, int kind) {
  const uint32_t key = kind == 1 ? 0x80000000u : kind == 2 ? 0x40000000u : mask;
  auto it = c->prog_index.find({z, key});
  if (it != c->prog_index.end()) return it->second;
  Program p = make_program(z, mask, kind);
  const int offv = (int)c->prog_host.size();
  c->prog_host.push_back((uint32_t)p.ops.size());
  c->prog_host.insert(c->prog_host.end(), p.ops.begin(), p.ops.end());
  c->nbuf = std::max(c->nbuf, p.nbuf);
  c->prog_index[{z, key}] = offv;
  c->prog_dirty = true;
  return offv;
}

int sync_programs(itn_ctx* c) {
  if (!c->prog_dirty) return ITN_OK;
  int r = upload_vec(c, c->d_prog, c->prog_host, c->stream);
  if (r) return r;
  c->prog_dirty = false;
  return ITN_OK;
}

int block_for(itn_ctx* c) {
  if (c->dtype >= 0 && c->dtype < 4 && c->tuned_block[c->dtype] > 0) return c->tuned_block[c->dtype];
  if (c->max_tensor <= 256) return 64;
  if (c->max_tensor <= 2048) return 128;
  return 256;
}

// Staging limits and CTA size of one item class (null: the whole network's, tuned CTA size).
struct ClassLimits {
  int64_t max_tensor;
  int msg_cap, max_d2, block;
};

// Prepare GenericArgs and a launch configuration for a list of items.
int plan_generic(itn_ctx* c, GenericArgs& a, LaunchCfg& cfg, const int* d_items, int n_items,
                 const void* msg_in, void* msg_out, const ClassLimits* lim = nullptr) {
  memset(&a, 0, sizeof(a));
  a.layers = c->layers;
  a.off = c->d_off.as<int>();
  a.rev = c->d_rev.as<int>();
  a.bond = c->d_bond.as<int>();
  a.phys = c->d_phys.as<int>();
  a.toff = c->d_toff.as<long long>();
  a.moff = c->d_moff.as<long long>();
  a.tens = c->d_tens.p;
  a.msg_in = msg_in;
  a.msg_out = msg_out;
  a.items = d_items;
  a.n_items = n_items;
  a.prog = c->d_prog.as<unsigned>();
  a.nbuf = c->layers == 2 ? c->nbuf : 0;
  a.buf_elems = ((lim ? lim->max_tensor : c->max_tensor) + 15) & ~15LL;
  a.msg_cap = lim ? lim->msg_cap : c->msg_cap;
  a.max_d2 = lim ? lim->max_d2 : c->max_d2;
  a.normalize = 1;
  cfg.block = lim ? lim->block : block_for(c);
  bool in_smem = true;
  size_t smem = generic_smem_bytes(c->dtype, a, cfg.block, true);
  if (c->layers == 2 && smem > (size_t)c->smem_optin) {
    in_smem = false;
    smem = generic_smem_bytes(c->dtype, a, cfg.block, false);
    if (smem > (size_t)c->smem_optin)
      return fail(c, ITN_ERR_UNSUPPORTED, "vertex needs %zu bytes of shared staging", smem);
  }
  int per_sm = generic_max_active(c->dtype, c->layers, cfg.block, smem);
  if (per_sm <= 0) per_sm = 1;
  cfg.grid = std::max(1, std::min(n_items, c->sm_count * per_sm));
  cfg.smem = smem;
  if (!in_smem) {
    const size_t need = (size_t)cfg.grid * a.nbuf * a.buf_elems * dtype_size(c->dtype);
    CK(c->d_scratch.ensure(need));
    a.gscratch = c->d_scratch.p;
  }
  return ITN_OK;
}

ConvState* conv(itn_ctx* c) { return c->d_state.as<ConvState>(); }

// Calls that use a context's stream or staging are refused while a submitted solve is pending.
int not_busy(itn_ctx* c) {
  if (c && c->submitted.active)
    return fail(c, ITN_ERR_STATE, "a solve submitted with itn_bp_solve_submit is pending: call itn_bp_solve_wait first");
  return ITN_OK;
}

int check_ready(itn_ctx* c, bool need_msgs) {
  if (!c) return ITN_ERR_ARG;
  if (!c->have_graph) return fail(c, ITN_ERR_STATE, "no network uploaded");
  if (!c->have_tensors) return fail(c, ITN_ERR_STATE, "no site tensors uploaded");
  if (need_msgs && !c->have_messages) return fail(c, ITN_ERR_STATE, "no messages uploaded");
  return ITN_OK;
}

__global__ void copy_kernel(const int4* __restrict__ src, int4* __restrict__ dst, long long n16,
                            const ConvState* s) {
  if (s->done) return;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n16;
       j += (long long)gridDim.x * blockDim.x)
    dst[j] = src[j];
}

}  // namespace

// =====================================================================================
extern "C" {

int32_t itn_abi_version(void) { return ITN_ABI_VERSION; }

const char* itn_status_string(int32_t s) {
  switch (s) {
    case ITN_OK: return "ok";
    case ITN_ERR_ARG: return "invalid argument";
    case ITN_ERR_CUDA: return "CUDA error";
    case ITN_ERR_OOM: return "out of device memory";
    case ITN_ERR_NAN: return "non-finite value";
    case ITN_ERR_TIMEOUT: return "iteration cap reached";
    case ITN_ERR_UNSUPPORTED: return "unsupported";
    case ITN_ERR_STATE: return "invalid call order";
  }
  return "unknown status";
}

int32_t itn_create(itn_ctx** out, int32_t device, int32_t flags) {
  (void)flags;
  if (!out) return ITN_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return ITN_ERR_CUDA;
  }
  if (device < 0 || device >= n) return ITN_ERR_ARG;
  itn_ctx* c = new itn_ctx();
  c->device = device;
  if (int r = ensure_device(c)) {
    delete c;
    return r;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    delete c;
    return ITN_ERR_CUDA;
  }
  c->sm_count = prop.multiProcessorCount;
  c->smem_optin = (int)prop.sharedMemPerBlockOptin;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      c->d_state.ensure(sizeof(ConvState)) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return ITN_ERR_CUDA;
  }
  *out = c;
  return ITN_OK;
}

int32_t itn_destroy(itn_ctx* c) {
  if (!c) return ITN_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  delete c;
  return ITN_OK;
}

const char* itn_last_error(const itn_ctx* c) { return c ? c->err.c_str() : "null context"; }

int32_t itn_inject_fault(itn_ctx* c, int32_t kind, int64_t value) {
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  switch (kind) {
    case ITN_FAULT_WAIT_NS:
      c->wait_ns = value > 0 ? (uint64_t)value : kDefaultWaitNs;
      if (c->tc) tc_set_wait_limit(c->tc, c->wait_ns);
      // the limit is a kernel argument baked into the cached solve graphs
      for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
      c->graphs.clear();
      c->graph_launches.clear();
      return ITN_OK;
    case ITN_FAULT_STALL:
      c->stall = value != 0;
      if (c->tc) tc_set_stall(c->tc, c->stall);
      for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
      c->graphs.clear();
      c->graph_launches.clear();
      return ITN_OK;
    case ITN_FAULT_ALLOC:
      if (value < 0) return fail(c, ITN_ERR_ARG, "allocation failure count < 0");
      t_fail_allocs = value;
      return ITN_OK;
    case ITN_FAULT_NO_PERSISTENT_ADJOINT:
      c->no_persist_adj = value != 0;
      return ITN_OK;
    case ITN_FAULT_NO_PERSISTENT_SWEEPS:
      c->no_persist_sweeps = value != 0;
      for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
      c->graphs.clear();
      c->graph_launches.clear();
      return ITN_OK;
  }
  return fail(c, ITN_ERR_ARG, "unknown fault kind %d", kind);
}

int32_t itn_synchronize(itn_ctx* c) {
  if (!c) return ITN_ERR_ARG;
  CK(cudaStreamSynchronize(c->stream));
  return ITN_OK;
}

int32_t itn_graph_upload(itn_ctx* c, int64_t nv, const int64_t* csr_off, const int64_t* csr_nbr,
                         const int32_t* bond, const int64_t* rev, const int32_t* phys,
                         int32_t layers, const int32_t* net_id) {
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (int r = ensure_device(c)) return r;
  if (nv < 0 || nv > (1LL << 30)) return fail(c, ITN_ERR_ARG, "nv out of range");
  if (nv > 0 && (!csr_off || !csr_nbr || !bond)) return fail(c, ITN_ERR_ARG, "null CSR array");
  if (layers != 1 && layers != 2) return fail(c, ITN_ERR_ARG, "layers must be 1 or 2");
  if (nv > 0 && csr_off[0] != 0) return fail(c, ITN_ERR_ARG, "csr_off[0] must be 0");
  const int64_t ns = nv > 0 ? csr_off[nv] : 0;
  if (ns < 0 || ns > (1LL << 30)) return fail(c, ITN_ERR_ARG, "slot count out of range");
  for (int64_t u = 0; u < nv; ++u) {
    const int64_t z = csr_off[u + 1] - csr_off[u];
    if (z < 0) return fail(c, ITN_ERR_ARG, "csr_off not monotone at vertex %lld", (long long)u);
    if (z > kMaxLegs) return fail(c, ITN_ERR_UNSUPPORTED, "vertex %lld has %lld legs (max %d)",
                                  (long long)u, (long long)z, kMaxLegs);
  }
  for (int64_t s = 0; s < ns; ++s) {
    if (csr_nbr[s] < 0 || csr_nbr[s] >= nv) return fail(c, ITN_ERR_ARG, "neighbour out of range at slot %lld", (long long)s);
    if (bond[s] < 1 || bond[s] > 4096) return fail(c, ITN_ERR_ARG, "bond dimension out of range at slot %lld", (long long)s);
  }
  c->have_graph = c->have_tensors = c->have_messages = false;
  c->nv = nv;
  c->nslots = ns;
  c->layers = layers;
  c->off.assign(csr_off, csr_off + nv + 1);
  if (nv == 0) c->off.assign(1, 0);
  c->nbr.assign(csr_nbr, csr_nbr + ns);
  c->bond.assign(bond, bond + ns);
  c->phys.assign(nv, 1);
  if (phys) c->phys.assign(phys, phys + nv);
  for (int64_t u = 0; u < nv; ++u)
    if (c->phys[u] < 1) return fail(c, ITN_ERR_ARG, "physical dimension < 1 at vertex %lld", (long long)u);
  if (layers == 1)
    for (int64_t u = 0; u < nv; ++u)
      if (c->phys[u] != 1) return fail(c, ITN_ERR_UNSUPPORTED, "plain (one-layer) networks need phys = 1 (open site index at vertex %lld)", (long long)u);
  // reverse slots
  c->rev.assign(ns, -1);
  if (rev) {
    for (int64_t s = 0; s < ns; ++s) c->rev[s] = rev[s];
  } else {
    std::map<std::pair<int64_t, int64_t>, std::vector<int64_t>> pend;
    for (int64_t u = 0; u < nv; ++u)
      for (int64_t s = c->off[u]; s < c->off[u + 1]; ++s) pend[{u, c->nbr[s]}].push_back(s);
    for (auto& kv : pend) {
      auto it = pend.find({kv.first.second, kv.first.first});
      if (it == pend.end() || it->second.size() != kv.second.size())
        return fail(c, ITN_ERR_ARG, "edge %lld->%lld has no matching reverse", (long long)kv.first.first, (long long)kv.first.second);
      for (size_t k = 0; k < kv.second.size(); ++k) c->rev[kv.second[k]] = it->second[k];
    }
  }
  for (int64_t u = 0; u < nv; ++u)
    for (int64_t s = c->off[u]; s < c->off[u + 1]; ++s) {
      const int64_t r = c->rev[s];
      if (r < 0 || r >= ns || c->rev[r] != s || c->nbr[r] != u || c->bond[r] != c->bond[s] || c->nbr[s] == u)
        return fail(c, ITN_ERR_ARG, "inconsistent reverse slot for slot %lld", (long long)s);
    }
  // offsets
  c->toff.assign(nv + 1, 0);
  c->max_tensor = 1;
  c->msg_cap = 1;
  for (int64_t u = 0; u < nv; ++u) {
    int64_t n = c->phys[u];
    int64_t mc = 0;
    for (int64_t s = c->off[u]; s < c->off[u + 1]; ++s) {
      n *= c->bond[s];
      mc += (layers == 2) ? (int64_t)c->bond[s] * c->bond[s] : c->bond[s];
      if (n > (1LL << 28)) return fail(c, ITN_ERR_UNSUPPORTED, "site tensor of vertex %lld too large", (long long)u);
    }
    c->toff[u + 1] = c->toff[u] + n;
    c->max_tensor = std::max(c->max_tensor, n);
    c->msg_cap = (int)std::max<int64_t>(c->msg_cap, mc);
  }
  c->moff.assign(ns + 1, 0);
  c->max_d2 = 1;
  for (int64_t s = 0; s < ns; ++s) {
    const int64_t m = layers == 2 ? (int64_t)c->bond[s] * c->bond[s] : c->bond[s];
    c->moff[s + 1] = c->moff[s] + m;
    c->max_d2 = (int)std::max<int64_t>(c->max_d2, m);
  }
  // networks
  c->net.assign(nv, 0);
  if (net_id) c->net.assign(net_id, net_id + nv);
  int nn = 0;
  for (int64_t u = 0; u < nv; ++u) {
    if (c->net[u] < 0) return fail(c, ITN_ERR_ARG, "negative network id");
    nn = std::max(nn, c->net[u] + 1);
  }
  for (int64_t u = 0; u < nv; ++u)
    for (int64_t s = c->off[u]; s < c->off[u + 1]; ++s)
      if (c->net[c->nbr[s]] != c->net[u]) return fail(c, ITN_ERR_ARG, "edge joins two networks");
  c->n_nets = std::max(nn, 1);
  c->eslots.clear();
  for (int64_t s = 0; s < ns; ++s)
    if (s < c->rev[s]) c->eslots.push_back((int)s);
  std::vector<int> voff(c->n_nets + 1, 0), eoff(c->n_nets + 1, 0), vlist(nv), elist(c->eslots.size());
  for (int64_t u = 0; u < nv; ++u) voff[c->net[u] + 1]++;
  std::vector<int> esrc(c->eslots.size());
  for (size_t e = 0; e < c->eslots.size(); ++e) {
    int64_t s = c->eslots[e];
    int64_t u = std::upper_bound(c->off.begin(), c->off.end(), s) - c->off.begin() - 1;
    esrc[e] = (int)u;
    eoff[c->net[u] + 1]++;
  }
  for (int k = 0; k < c->n_nets; ++k) {
    voff[k + 1] += voff[k];
    eoff[k + 1] += eoff[k];
  }
  {
    std::vector<int> vp(voff.begin(), voff.end() - 1), ep(eoff.begin(), eoff.end() - 1);
    for (int64_t u = 0; u < nv; ++u) vlist[vp[c->net[u]]++] = (int)u;
    for (size_t e = 0; e < c->eslots.size(); ++e) elist[ep[c->net[esrc[e]]]++] = (int)e;
  }
  // programs & work lists
  c->prog_index.clear();
  c->prog_host.clear();
  c->nbuf = 1;
  c->items_par.clear();
  c->items_scal.clear();
  c->items_dump.clear();
  c->seq_plans.clear();
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
  // Small networks (fewer vertices than 4 per SM) get two items per vertex: the two
  // branches of the top-level leave-one-out split (legs [0, h) and [h, z)) do the same
  // absorptions as one item but give the SMs twice the CTAs; large networks keep one item
  // per vertex (one read of the site tensor).
  const bool halves = nv <= 4 * std::max(c->sm_count, 1);
  for (int64_t u = 0; u < nv; ++u) {
    const int z = (int)(c->off[u + 1] - c->off[u]);
    const uint32_t full = z >= 32 ? 0xffffffffu : ((1u << z) - 1u);
    if (layers == 2) {
      if (z >= 2 && halves) {
        const int h = (z + 1) / 2;
        const uint32_t lo = (1u << h) - 1u;
        c->items_par.push_back((int)u);
        c->items_par.push_back(program_offset(c, z, lo, 0));
        c->items_par.push_back((int)u);
        c->items_par.push_back(program_offset(c, z, full & ~lo, 0));
      } else if (z > 0) {
        c->items_par.push_back((int)u);
        c->items_par.push_back(program_offset(c, z, full, 0));
      }
      c->items_scal.push_back((int)u);
      c->items_scal.push_back(program_offset(c, z, 0, 1));
      c->items_dump.push_back((int)u);
      c->items_dump.push_back(program_offset(c, z, 0, 2));
    } else {
      if (z > 0) {
        c->items_par.push_back((int)u);
        c->items_par.push_back((int)full);
      }
      c->items_scal.push_back((int)u);
      c->items_scal.push_back(0);
    }
  }
  {
    // Largest vertices first: persistent CTAs take items round-robin, so a descending cost
    // order keeps uneven networks balanced.  Among equal sizes, items with the same bond
    // dimensions in leg order (and the same program) are adjacent, so that the CTAs running
    // at the same time execute the same D-specialised code paths.
    std::vector<std::pair<int, int>> it;
    for (size_t k = 0; k + 1 < c->items_par.size(); k += 2) it.push_back({c->items_par[k], c->items_par[k + 1]});
    auto sig_less = [&](int u, int v) {
      const int64_t zu = c->off[u + 1] - c->off[u], zv = c->off[v + 1] - c->off[v];
      if (zu != zv) return zu < zv;
      for (int64_t l = 0; l < zu; ++l) {
        const int32_t bu = c->bond[c->off[u] + l], bv = c->bond[c->off[v] + l];
        if (bu != bv) return bu < bv;
      }
      return false;
    };
    std::stable_sort(it.begin(), it.end(), [&](const std::pair<int, int>& x, const std::pair<int, int>& y) {
      const int64_t sx = c->toff[x.first + 1] - c->toff[x.first], sy = c->toff[y.first + 1] - c->toff[y.first];
      if (sx != sy) return sx > sy;
      if (sig_less(x.first, y.first)) return true;
      if (sig_less(y.first, x.first)) return false;
      return x.second < y.second;
    });
    c->items_par.clear();
    for (auto& p : it) {
      c->items_par.push_back(p.first);
      c->items_par.push_back(p.second);
    }
  }
  {
    // size classes of the two-layer parallel sweep (see kClassMax)
    const int n = (int)c->items_par.size() / 2;
    c->par_classes.clear();
    auto size_of = [&](int i) { const int u = c->items_par[2 * i]; return c->toff[u + 1] - c->toff[u]; };
    std::vector<int> cut;  // first item of each sub-class (non-increasing sizes)
    const bool split = layers == 2 && n >= kSmallMinItemsPerSm * std::max(c->sm_count, 1);
    for (int k = 0; k < kNumSubClasses; ++k) {
      int i = 0;
      while (i < n && size_of(i) > kClassMax[k]) ++i;
      cut.push_back(split ? i : n);
    }
    int begin = 0;
    for (int k = 0; k <= kNumSubClasses; ++k) {
      const int end = k < kNumSubClasses ? cut[k] : n;
      if (end <= begin) continue;
      itn_ctx::ItemClass ic;
      ic.begin = begin;
      ic.end = end;
      ic.own = k > 0;
      if (ic.own) {
        ic.block = kClassBlock[k - 1];
        for (int i = begin; i < end; ++i) {
          const int u = c->items_par[2 * i];
          ic.max_tensor = std::max<int64_t>(ic.max_tensor, size_of(i));
          int64_t mc = 0;
          for (int64_t q = c->off[u]; q < c->off[u + 1]; ++q) {
            const int64_t d2 = (int64_t)c->bond[q] * c->bond[q];
            mc += d2;
            ic.max_d2 = (int)std::max<int64_t>(ic.max_d2, d2);
          }
          ic.msg_cap = (int)std::max<int64_t>(ic.msg_cap, mc);
        }
      }
      c->par_classes.push_back(ic);
      begin = end;
    }
    // a lone sub-class covers the whole network: plan it as the single class
    if (c->par_classes.size() == 1) c->par_classes[0].own = false;
  }
  c->scal_d8 = layers == 2 && nv > 0;
  for (int64_t u = 0; u < nv && c->scal_d8; ++u) {
    if (c->off[u] != 4 * u || c->off[u + 1] != 4 * u + 4 || c->phys[u] != 2) c->scal_d8 = false;
    for (int64_t q = c->off[u]; q < c->off[u + 1] && c->scal_d8; ++q)
      if (c->bond[q] != 8) c->scal_d8 = false;
  }
  c->z3 = layers == 2 && nv > 0;
  c->items_z3.clear();
  c->z3_work.clear();
  for (int64_t u = 0; u < nv && c->z3; ++u) {
    if (c->off[u + 1] - c->off[u] != 3 || c->toff[u + 1] - c->toff[u] > kZ3MaxTensor) c->z3 = false;
    for (int64_t q = c->off[u]; q < c->off[u + 1] && c->z3; ++q)
      if (c->bond[q] > kZ3MaxBond) c->z3 = false;
  }
  if (c->z3) {
    c->items_z3.resize(nv);
    for (int64_t u = 0; u < nv; ++u) c->items_z3[u] = (int)u;
    std::stable_sort(c->items_z3.begin(), c->items_z3.end(), [&](int a, int b) {
      return c->toff[a + 1] - c->toff[a] > c->toff[b + 1] - c->toff[b];
    });
    for (int u : c->items_z3)
      c->z3_work.push_back((double)(c->toff[u + 1] - c->toff[u]) *
                           (c->bond[c->off[u]] + c->bond[c->off[u] + 1] + c->bond[c->off[u] + 2]));
    c->meta_z3.resize(nv);
    for (int64_t i = 0; i < nv; ++i) {
      const int u = c->items_z3[i];
      Z3Meta& mt = c->meta_z3[i];
      memset(&mt, 0, sizeof(mt));
      mt.t0 = c->toff[u];
      mt.n = (int)(c->toff[u + 1] - c->toff[u]);
      mt.s0 = (int)c->off[u];
      for (int l = 0; l < 3; ++l) {
        const int64_t s = c->off[u] + l;
        mt.D[l] = c->bond[s];
        mt.moff_in[l] = c->moff[c->rev[s]];
        mt.moff_out[l] = c->moff[s];
      }
    }
  } else {
    c->meta_z3.clear();
  }
  c->z3_budget = {0, 0, 0, 0};
  c->z3_mult = {0, 0, 0, 0};
  c->z3_k0 = {0, 0, 0, 0};
  c->tuned_block.assign(4, 0);
  c->dual_block.assign(4, 0);
  {
    // FNV-1a over the structure the launch shapes depend on
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
      const unsigned char* b = static_cast<const unsigned char*>(p);
      for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    };
    const int64_t hdr[3] = {c->nv, c->nslots, (int64_t)c->layers};
    mix(hdr, sizeof(hdr));
    mix(c->off.data(), c->off.size() * sizeof(int64_t));
    mix(c->nbr.data(), c->nbr.size() * sizeof(int64_t));
    mix(c->bond.data(), c->bond.size() * sizeof(int32_t));
    mix(c->phys.data(), c->phys.size() * sizeof(int32_t));
    c->net_sig = h;
  }
  if (c->prog_host.empty()) c->prog_host.push_back(0);
  c->prog_dirty = true;
  std::vector<int> off32(c->off.begin(), c->off.end()), rev32(c->rev.begin(), c->rev.end());
  std::vector<long long> toffl(c->toff.begin(), c->toff.end()), moffl(c->moff.begin(), c->moff.end());
  int r;
  if ((r = upload_vec(c, c->d_off, off32, c->stream)) || (r = upload_vec(c, c->d_rev, rev32, c->stream)) ||
      (r = upload_vec(c, c->d_bond, c->bond, c->stream)) || (r = upload_vec(c, c->d_phys, c->phys, c->stream)) ||
      (r = upload_vec(c, c->d_toff, toffl, c->stream)) || (r = upload_vec(c, c->d_moff, moffl, c->stream)) ||
      (r = upload_vec(c, c->d_eslots, c->eslots, c->stream)) ||
      (r = upload_vec(c, c->d_net_voff, voff, c->stream)) || (r = upload_vec(c, c->d_net_vlist, vlist, c->stream)) ||
      (r = upload_vec(c, c->d_net_eoff, eoff, c->stream)) || (r = upload_vec(c, c->d_net_elist, elist, c->stream)) ||
      (r = upload_vec(c, c->d_items_par, c->items_par, c->stream)) ||
      (r = upload_vec(c, c->d_items_scal, c->items_scal, c->stream)) ||
      (r = upload_vec(c, c->d_items_dump, c->items_dump, c->stream)) ||
      (r = upload_vec(c, c->d_items_z3, c->items_z3, c->stream)) ||
      (r = upload_vec(c, c->d_meta_z3, c->meta_z3, c->stream)) || (r = sync_programs(c)))
    return r;
  {
    std::vector<int> epos(ns, -1);
    for (size_t e = 0; e < c->eslots.size(); ++e) epos[c->eslots[e]] = (int)e;
    c->slot_dst.assign(ns, 0);
    c->slot_eidx.assign(ns, 0);
    for (int64_t t = 0; t < ns; ++t) {
      c->slot_dst[t] = (int)c->nbr[t];
      c->slot_eidx[t] = epos[std::min<int64_t>(t, c->rev[t])];
    }
    if ((r = upload_vec(c, c->d_slot_dst, c->slot_dst, c->stream)) ||
        (r = upload_vec(c, c->d_slot_eidx, c->slot_eidx, c->stream)))
      return r;
  }
  CK(c->d_slot_diff.ensure(std::max<int64_t>(ns, 1) * sizeof(double)));
  CK(cudaStreamSynchronize(c->stream));
  c->have_graph = true;
  c->dtype = -1;
  if (c->tc) tc_invalidate(c->tc);
  return ITN_OK;
}

int32_t itn_graph_info(const itn_ctx* c, int64_t* nv, int64_t* nslots, int64_t* tensor_elems,
                       int64_t* message_elems, int32_t* n_nets, int64_t* n_undirected) {
  if (!c) return ITN_ERR_ARG;
  if (!c->have_graph) return ITN_ERR_STATE;
  if (nv) *nv = c->nv;
  if (nslots) *nslots = c->nslots;
  if (tensor_elems) *tensor_elems = c->toff[c->nv];
  if (message_elems) *message_elems = c->moff[c->nslots];
  if (n_nets) *n_nets = c->n_nets;
  if (n_undirected) *n_undirected = (int64_t)c->eslots.size();
  return ITN_OK;
}

static int set_dtype(itn_ctx* c, int32_t dtype) {
  if (dtype < ITN_F32 || dtype > ITN_C128) return fail(c, ITN_ERR_ARG, "unknown dtype %d", dtype);
  if (c->dtype != dtype) {
    c->dtype = dtype;
    c->have_messages = false;
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
  }
  return ITN_OK;
}

int32_t itn_tensors_upload(itn_ctx* c, int32_t dtype, const void* packed) {
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (!c->have_graph) return fail(c, ITN_ERR_STATE, "upload the network first");
  if (!packed && c->toff[c->nv] > 0) return fail(c, ITN_ERR_ARG, "null tensor pointer");
  if (int r = ensure_device(c)) return r;
  if (int r = set_dtype(c, dtype)) return r;
  // a failed upload leaves no tensors behind (a failed allocation frees the old buffer)
  c->have_tensors = false;
  const size_t bytes = (size_t)c->toff[c->nv] * dtype_size(dtype);
  CK(c->d_tens.ensure(bytes));
  if (bytes) CK(cudaMemcpyAsync(c->d_tens.p, packed, bytes, cudaMemcpyHostToDevice, c->stream));
  const size_t mb = (size_t)c->moff[c->nslots] * dtype_size(dtype);
  CK(c->d_msg[0].ensure(mb));
  CK(c->d_msg[1].ensure(mb));
  CK(cudaStreamSynchronize(c->stream));
  c->have_tensors = true;
  if (c->tc) tc_invalidate(c->tc);
  return ITN_OK;
}

int32_t itn_tensors_upload_strided(itn_ctx* c, int32_t dtype, const void* const* site_ptrs,
                                   const int64_t* strides) {
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (!c->have_graph) return fail(c, ITN_ERR_STATE, "upload the network first");
  if (!site_ptrs || !strides) return fail(c, ITN_ERR_ARG, "null pointer");
  if (int r = ensure_device(c)) return r;
  if (int r = set_dtype(c, dtype)) return r;
  const size_t es = dtype_size(dtype);
  // Gather each vertex's source extent (max offset + 1) into one staging buffer.
  std::vector<long long> soff(c->nv + 1, 0), sstride;
  std::vector<int> rank_off(c->nv + 1, 0), dims;
  for (int64_t u = 0; u < c->nv; ++u) {
    const int64_t z = c->off[u + 1] - c->off[u];
    const int64_t base = c->off[u] + u;
    long long ext = 1;
    for (int64_t a = 0; a <= z; ++a) {
      const int dim = a == 0 ? c->phys[u] : c->bond[c->off[u] + a - 1];
      const long long st = strides[base + a];
      if (st < 0) return fail(c, ITN_ERR_ARG, "negative stride at vertex %lld", (long long)u);
      ext += (long long)(dim - 1) * st;
      dims.push_back(dim);
      sstride.push_back(st);
    }
    if (!site_ptrs[u]) return fail(c, ITN_ERR_ARG, "null tensor pointer at vertex %lld", (long long)u);
    soff[u + 1] = soff[u] + ext;
    rank_off[u + 1] = rank_off[u] + (int)(z + 1);
  }
  std::vector<unsigned char> host((size_t)soff[c->nv] * es);
  for (int64_t u = 0; u < c->nv; ++u)
    memcpy(host.data() + (size_t)soff[u] * es, site_ptrs[u], (size_t)(soff[u + 1] - soff[u]) * es);
  DevBuf d_soff, d_toffl, d_rank, d_dims, d_str;
  std::vector<long long> toffl(c->toff.begin(), c->toff.end());
  int r;
  if ((r = upload_vec(c, d_soff, soff, c->stream)) || (r = upload_vec(c, d_toffl, toffl, c->stream)) ||
      (r = upload_vec(c, d_rank, rank_off, c->stream)) || (r = upload_vec(c, d_dims, dims, c->stream)) ||
      (r = upload_vec(c, d_str, sstride, c->stream)))
    return r;
  CK(c->d_stage.ensure(host.size()));
  if (!host.empty()) CK(cudaMemcpyAsync(c->d_stage.p, host.data(), host.size(), cudaMemcpyHostToDevice, c->stream));
  CK(c->d_tens.ensure((size_t)c->toff[c->nv] * es));
  CK(launch_permute(dtype, (int)c->nv, d_soff.as<long long>(), d_toffl.as<long long>(), d_rank.as<int>(),
                    d_dims.as<int>(), d_str.as<long long>(), c->d_stage.p, c->d_tens.p, c->stream));
  const size_t mb = (size_t)c->moff[c->nslots] * es;
  CK(c->d_msg[0].ensure(mb));
  CK(c->d_msg[1].ensure(mb));
  CK(cudaStreamSynchronize(c->stream));
  c->have_tensors = true;
  if (c->tc) tc_invalidate(c->tc);
  return ITN_OK;
}

int32_t itn_tensors_download(itn_ctx* c, int32_t dtype, void* packed) {
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, false)) return r;
  if (dtype != c->dtype) return fail(c, ITN_ERR_ARG, "dtype differs from the uploaded tensors");
  const size_t bytes = (size_t)c->toff[c->nv] * dtype_size(dtype);
  if (bytes) CK(cudaMemcpyAsync(packed, c->d_tens.p, bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ITN_OK;
}

int32_t itn_messages_upload(itn_ctx* c, int32_t dtype, const void* packed) {
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, false)) return r;
  if (dtype != c->dtype) return fail(c, ITN_ERR_ARG, "message dtype must equal the tensor dtype");
  const size_t bytes = (size_t)c->moff[c->nslots] * dtype_size(dtype);
  if (bytes && !packed) return fail(c, ITN_ERR_ARG, "null message pointer");
  c->cur = 0;
  if (bytes) CK(cudaMemcpyAsync(c->d_msg[0].p, packed, bytes, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->have_messages = true;
  return ITN_OK;
}

int32_t itn_messages_download(itn_ctx* c, int32_t dtype, void* packed) {
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, true)) return r;
  if (dtype != c->dtype) return fail(c, ITN_ERR_ARG, "dtype differs from the uploaded data");
  const size_t bytes = (size_t)c->moff[c->nslots] * dtype_size(dtype);
  if (bytes && !packed) return fail(c, ITN_ERR_ARG, "null message pointer");
  if (bytes) CK(cudaMemcpyAsync(packed, c->d_msg[c->cur].p, bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ITN_OK;
}

int32_t itn_messages_init(itn_ctx* c, int32_t kind) {
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, false)) return r;
  if (kind < 0 || kind > 2) return fail(c, ITN_ERR_ARG, "unknown message init kind");
  c->cur = 0;
  CK(launch_init_messages(c->dtype, c->layers, kind, c->d_moff.as<long long>(), c->d_bond.as<int>(),
                          (int)c->nslots, c->d_msg[0].p, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->have_messages = true;
  return ITN_OK;
}

}  // extern "C"

// ---- solve helpers ------------------------------------------------------------------------
namespace {

// Dependency levels that make a sequential (Gauss-Seidel) sweep over `edges` exact when
// the updates of one level run concurrently: an update follows every earlier update it
// reads from (RAW), every earlier reader of the slot it writes (WAR) and every earlier
// writer of that slot (WAW).
std::vector<std::vector<int>> sequential_levels(itn_ctx* c, const int64_t* edges, int64_t n) {
  std::vector<int> last_w(c->nslots, 0), last_r(c->nslots, 0);
  std::vector<std::vector<int>> levels;
  for (int64_t e = 0; e < n; ++e) {
    const int64_t s = edges[e];
    const int64_t u = std::upper_bound(c->off.begin(), c->off.end(), s) - c->off.begin() - 1;
    int lv = std::max(last_w[s], last_r[s]);
    for (int64_t t = c->off[u]; t < c->off[u + 1]; ++t) {
      if (t == s) continue;
      lv = std::max(lv, last_w[c->rev[t]]);
    }
    lv += 1;
    last_w[s] = lv;
    for (int64_t t = c->off[u]; t < c->off[u + 1]; ++t)
      if (t != s) last_r[c->rev[t]] = std::max(last_r[c->rev[t]], lv);
    if ((int)levels.size() < lv) levels.resize(lv);
    levels[lv - 1].push_back((int)e);
  }
  return levels;
}

struct SeqPlan {
  std::vector<int> level_off;  // into items (pairs)
  std::shared_ptr<DevBuf> items;
};

int get_seq_plan(itn_ctx* c, const int64_t* edges, int64_t n, SeqPlan& plan) {
  std::vector<int64_t> key(edges, edges + n);
  auto it = c->seq_plans.find(key);
  if (it != c->seq_plans.end()) {
    plan.level_off = it->second.first;
    plan.items = it->second.second;
    return ITN_OK;
  }
  for (int64_t e = 0; e < n; ++e)
    if (edges[e] < 0 || edges[e] >= c->nslots) return fail(c, ITN_ERR_ARG, "edge slot %lld out of range", (long long)edges[e]);
  auto levels = sequential_levels(c, edges, n);
  std::vector<int> items, loff(1, 0);
  for (auto& lv : levels) {
    for (int e : lv) {
      const int64_t s = edges[e];
      const int64_t u = std::upper_bound(c->off.begin(), c->off.end(), s) - c->off.begin() - 1;
      const int z = (int)(c->off[u + 1] - c->off[u]);
      const int leg = (int)(s - c->off[u]);
      items.push_back((int)u);
      items.push_back(c->layers == 2 ? program_offset(c, z, 1u << leg, 0) : (int)(1u << leg));
    }
    loff.push_back((int)items.size() / 2);
  }
  auto buf = std::make_shared<DevBuf>();
  if (int r = upload_vec(c, *buf, items, c->stream)) return r;
  if (int r = sync_programs(c)) return r;
  c->seq_plans[key] = {loff, buf};
  plan.level_off = loff;
  plan.items = buf;
  return ITN_OK;
}

// Launch plans are computed before stream capture (no allocation or occupancy query
// happens while capturing).
struct ParPlan {
  // per item class, in launch order: a[k][i] reads buffer i, writes buffer i ^ 1
  std::vector<std::array<GenericArgs, 2>> a;
  std::vector<std::array<LaunchCfg, 2>> cfg;
};

// Process-wide cache of autotuned launch shapes, keyed by the tuner, the device, the dtype and
// the network's structure: every context that uploads the same network reuses the first
// context's choice, so solves of one network on several contexts (a serving loop's contexts,
// a context re-created per request) tune once and run the same launch shapes, which also keeps
// their results bit-identical (a different CTA size changes the order of partial sums).
std::mutex g_tune_mu;
std::map<std::string, std::array<int, 3>> g_tune_cache;

std::string tune_key(const itn_ctx* c, const char* tuner) {
  char b[160];
  snprintf(b, sizeof(b), "%s d%d t%d n%lld s%lld h%016llx", tuner, c->device, c->dtype, (long long)c->nv,
           (long long)c->nslots, (unsigned long long)c->net_sig);
  return b;
}

bool tune_lookup(const itn_ctx* c, const char* tuner, std::array<int, 3>& v) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune_cache.find(tune_key(c, tuner));
  if (it == g_tune_cache.end()) return false;
  v = it->second;
  return true;
}

void tune_store(const itn_ctx* c, const char* tuner, const std::array<int, 3>& v) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[tune_key(c, tuner)] = v;
}

// Autotuner for the parallel sweep: time one sweep per candidate CTA size (64, 128, 256
// threads; each with its own residency) from the current messages into the other
// ping-pong buffer and keep the fastest for this network and dtype.
int autotune_sweep(itn_ctx* c) {
  if (c->tuned_block[c->dtype] > 0 || c->items_par.empty()) return ITN_OK;
  if (getenv("ITN_NO_AUTOTUNE")) {
    c->tuned_block[c->dtype] = -1;
    return ITN_OK;
  }
  std::array<int, 3> cached;
  if (tune_lookup(c, "sweep", cached)) {
    c->tuned_block[c->dtype] = cached[0];
    return ITN_OK;
  }
  const int cands[3] = {64, 128, 256};
  float best = 1e30f;
  int best_b = 0;
  DevBuf scratch;  // second message buffer of the persistent trials
  for (int b : cands) {
    c->tuned_block[c->dtype] = b;
    GenericArgs a;
    LaunchCfg cfg;
    if (plan_generic(c, a, cfg, c->d_items_par.as<int>(), (int)c->items_par.size() / 2, c->d_msg[c->cur].p,
                     c->d_msg[c->cur ^ 1].p))
      continue;
    // the first launch warms the caches; the best of the next three is the candidate's time
    // (single launches of a few microseconds scatter by several percent)
    float ms = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      float t = 0.f;
      CK(cudaEventRecord(c->ev0, c->stream));
      CK(launch_generic(c->dtype, a, cfg, c->stream));
      CK(cudaEventRecord(c->ev1, c->stream));
      CK(cudaEventSynchronize(c->ev1));
      CK(cudaEventElapsedTime(&t, c->ev0, c->ev1));
      if (rep > 0) ms = std::min(ms, t);
    }
    // A shape that gives every item its own resident CTA runs the solve's sweeps as one
    // persistent launch (persistent_sweeps_fit): its time is that form's, per sweep, over
    // kTuneSweeps sweeps on copies of the current messages (the current buffer is not written).
    // The choice does not depend on ITN_FAULT_NO_PERSISTENT_SWEEPS, so both forms run one shape.
    constexpr int kTuneSweeps = 8;
    if (c->layers == 2 && c->par_classes.size() == 1 && cfg.grid == a.n_items && a.n_items > 0 &&
        (int64_t)generic_max_active(c->dtype, 2, cfg.block, cfg.smem) * c->sm_count >= a.n_items) {
      const size_t mbytes = (size_t)c->moff[c->nslots] * dtype_size(c->dtype);
      CK(scratch.ensure(mbytes));
      CK(c->d_sweepgrid.ensure(sizeof(SweepGrid)));
      GenericArgs pa = a;
      pa.conv = nullptr;
      pa.slot_diff = nullptr;
      pa.fused_step = 0;
      pa.normalize = 1;
      pa.pgrid = c->d_sweepgrid.as<SweepGrid>();
      pa.msg_buf[0] = c->d_msg[c->cur ^ 1].p;
      pa.msg_buf[1] = scratch.p;
      pa.nsweeps = kTuneSweeps;
      pa.wait_ns = c->wait_ns;
      pa.pstall = 0;
      float pms = 1e30f;
      for (int rep = 0; rep < 5; ++rep) {  // the best of four after a warm-up launch
        float t = 0.f;
        CK(cudaMemcpyAsync(c->d_msg[c->cur ^ 1].p, c->d_msg[c->cur].p, mbytes, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaEventRecord(c->ev0, c->stream));
        CK(launch_generic_persistent(c->dtype, pa, cfg, c->stream));
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaEventSynchronize(c->ev1));
        CK(cudaEventElapsedTime(&t, c->ev0, c->ev1));
        if (rep > 0) pms = std::min(pms, t / kTuneSweeps);
      }
      SweepGrid hg;
      CK(cudaMemcpy(&hg, c->d_sweepgrid.p, sizeof(hg), cudaMemcpyDeviceToHost));
      if (hg.err) return fail(c, ITN_ERR_TIMEOUT, "autotune: a grid-barrier wait of the persistent sweep gave up");
      ms = pms;
    }
    if (ms < best) {
      best = ms;
      best_b = b;
    }
  }
  c->tuned_block[c->dtype] = best_b > 0 ? best_b : -1;
  tune_store(c, "sweep", {c->tuned_block[c->dtype], 0, 0});
  if (getenv("ITN_DEBUG")) fprintf(stderr, "[itn] autotune: sweep CTA size %d (%.3f ms)\n", best_b, best);
  // cached graphs were captured with the previous launch shape
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
  return ITN_OK;
}

// FP32 parallel sweeps of a network whose vertices all have d = 2 and four legs of dimension
// 8 run on the register-blocked kernel (sweep_d8_kernel) instead of the interpreter.
bool use_sweep_d8(const itn_ctx* c) { return c->scal_d8 && c->dtype == ITN_F32; }

// Networks whose vertices all have three legs run the grouped sweep (bp_z3.cu).
bool use_sweep_z3(const itn_ctx* c) { return c->z3 && !use_sweep_d8(c); }

// Launch shape of the grouped sweep for a shared-memory budget per CTA and a CTA multiplier:
// size classes by the largest tensor (at most 1024, 682, 454, ... entries), warps per CTA of a
// class = slices of its largest vertex that fit the budget (at most 8), CTAs shared among
// the classes in proportion to their work, the total `mult` x the CTAs resident at once.
int plan_z3(itn_ctx* c, Z3Args& a, int& grid, size_t& smem, int budget, int mult, int k0, const void* in,
            void* out, int normalize, double* slot_diff, ConvState* cv) {
  memset(&a, 0, sizeof(a));
  a.meta = c->d_meta_z3.as<Z3Meta>();
  a.tens = c->d_tens.p;
  a.msg_in = in;
  a.msg_out = out;
  a.normalize = normalize;
  a.slot_diff = slot_diff;
  a.conv = cv;
  const size_t es = dtype_size(c->dtype);
  const int n = (int)c->items_z3.size();
  auto size_of = [&](int i) { const int u = c->items_z3[i]; return (int)(c->toff[u + 1] - c->toff[u]); };
  // classes: items whose tensors have (2 limit / 3, limit] entries, limit = 1024, 682, 454, ...
  // (a class's shared-memory slices are sized for its largest tensor; with halving classes the
  // smallest vertex of a class used half of its slice, and the mixed 256-network batch took
  // 9.76 ms per solve against 9.39 ms with thirds; quarters gave 9.45 ms)
  std::vector<std::pair<int, int>> ranges;
  int i = 0, limit = kZ3MaxTensor;
  auto lower = [](int l) { return (2 * l) / 3; };
  while (i < n) {
    while (lower(limit) >= size_of(i) && limit > 8 && (int)ranges.size() + 1 < kZ3MaxClasses) limit = lower(limit);
    int j = i;
    while (j < n && (size_of(j) > lower(limit) || limit <= 8 || (int)ranges.size() + 1 == kZ3MaxClasses)) ++j;
    ranges.push_back({i, j});
    i = j;
  }
  smem = (size_t)budget;
  for (auto& rg : ranges) smem = std::max(smem, (size_t)(3 * size_of(rg.first) + 448) * es);
  smem = std::min(smem, kZ3MaxSmem);
  const int per_sm = std::max(1, z3_blocks_per_sm(c->dtype, smem));
  const int total = std::max(1, c->sm_count * per_sm * std::max(mult, 1));
  // a class's CTAs are in proportion to its work: entries x (D0 + D1 + D2) per vertex plus a
  // fixed cost k0 per vertex (loading, barriers and index arithmetic, which dominate small
  // vertices; without it the classes of small vertices got too few CTAs and finished last)
  double wsum = 0;
  for (double w : c->z3_work) wsum += w + k0;
  int start = 0;
  a.n_classes = (int)ranges.size();
  for (size_t k = 0; k < ranges.size(); ++k) {
    Z3Class& cl = a.cls[k];
    cl.first = ranges[k].first;
    cl.count = ranges[k].second - ranges[k].first;
    cl.nmax = size_of(cl.first);
    cl.slice = 3 * cl.nmax + 448;
    // vertices in flight per CTA: as many slices as the budget holds (at most 8, a power of
    // two); the CTA's 8 warps are shared among them (wpi warps per vertex)
    const int fit = (int)std::max<size_t>(1, std::min<size_t>(kZ3Threads / 32, smem / ((size_t)cl.slice * es)));
    cl.groups = 1;
    while (cl.groups * 2 <= fit) cl.groups *= 2;
    cl.wpi = (kZ3Threads / 32) / cl.groups;
    double w = 0;
    for (int q = cl.first; q < cl.first + cl.count; ++q) w += c->z3_work[q] + k0;
    const int need = (cl.count + cl.groups - 1) / cl.groups;
    cl.ctas = std::max(1, std::min(need, (int)std::lround(total * w / std::max(wsum, 1.0))));
    cl.cta_start = start;
    start += cl.ctas;
  }
  grid = start;
  return ITN_OK;
}

// Autotuner of the grouped sweep: time one sweep per (shared-memory budget, CTA multiplier,
// fixed cost per vertex in the class split) candidate on the current messages (best of two
// after a warm-up launch) and keep the fastest shape for this dtype (180 launches, once per
// network and dtype).  On the 256-network complex64 batch the fixed cost took the solve from
// 15.8 to 10.4 ms, the 64 KB budget and 3-4x CTAs to 9.7 ms, size classes in thirds to 9.4 ms.
int autotune_z3(itn_ctx* c) {
  const int dt = c->dtype;
  if (c->z3_budget[dt] > 0) return ITN_OK;
  std::array<int, 3> cached;
  if (tune_lookup(c, "z3", cached)) {
    c->z3_budget[dt] = cached[0];
    c->z3_mult[dt] = cached[1];
    c->z3_k0[dt] = cached[2];
    return ITN_OK;
  }
  const int budgets[5] = {24 << 10, 48 << 10, 64 << 10, 96 << 10, 200 << 10};
  const int mults[4] = {1, 2, 3, 4};
  const int k0s[3] = {0, 5000, 20000};
  float best = 1e30f;
  int bb = budgets[1], bm = 1, bk = 0;
  for (int budget : budgets)
    for (int mult : mults)
      for (int k0 : k0s) {
        Z3Args a;
        int grid = 0;
        size_t smem = 0;
        if (int r = plan_z3(c, a, grid, smem, budget, mult, k0, c->d_msg[c->cur].p, c->d_msg[c->cur ^ 1].p, 1,
                            nullptr, nullptr))
          return r;
        float ms = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
          float t = 0.f;
          CK(cudaEventRecord(c->ev0, c->stream));
          CK(launch_sweep_z3(dt, a, grid, smem, c->stream));
          CK(cudaEventRecord(c->ev1, c->stream));
          CK(cudaEventSynchronize(c->ev1));
          CK(cudaEventElapsedTime(&t, c->ev0, c->ev1));
          if (rep > 0) ms = std::min(ms, t);
        }
        if (getenv("ITN_DEBUG"))
          fprintf(stderr, "[itn] z3 autotune: budget %d KB mult %d k0 %d grid %d smem %zu: %.4f ms\n", budget >> 10,
                  mult, k0, grid, smem, ms);
        if (ms < best) {
          best = ms;
          bb = budget;
          bm = mult;
          bk = k0;
        }
      }
  c->z3_budget[dt] = bb;
  c->z3_mult[dt] = bm;
  c->z3_k0[dt] = bk;
  tune_store(c, "z3", {bb, bm, bk});
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
  return ITN_OK;
}

int make_par_plan(itn_ctx* c, const itn_bp_opts* o, ParPlan& p) {
  const bool use_tol = o->tol >= 0;
  const size_t nc = c->par_classes.size();
  p.a.assign(nc, {});
  p.cfg.assign(nc, {});
  for (size_t k = 0; k < nc; ++k) {
    const itn_ctx::ItemClass& ic = c->par_classes[k];
    const ClassLimits lim{ic.max_tensor, ic.msg_cap, ic.max_d2, ic.block};
    for (int in = 0; in < 2; ++in) {
      GenericArgs& a = p.a[k][in];
      if (int r = plan_generic(c, a, p.cfg[k][in], c->d_items_par.as<int>() + 2 * ic.begin, ic.end - ic.begin,
                               c->d_msg[in].p, c->d_msg[in ^ 1].p, ic.own ? &lim : nullptr))
        return r;
      a.normalize = o->normalize;
      a.conv = conv(c);
      a.fused_step = k + 1 == nc ? 1 : 0;  // the last launch of a sweep steps the loop
      if (use_tol) a.slot_diff = c->d_slot_diff.as<double>();
    }
  }
  return ITN_OK;
}

// The CUDA-core sweeps of a two-layer network as one persistent cooperative launch: one item
// class, every item on its own resident CTA (small networks: the 12x12 and 16x16 lattices), and
// not switched off by itn_inject_fault(ITN_FAULT_NO_PERSISTENT_SWEEPS).
bool persistent_sweeps_fit(itn_ctx* c, const ParPlan& p, const itn_bp_opts* o) {
  if (c->no_persist_sweeps || o->precision != ITN_PREC_NATIVE || c->layers != 2 || p.a.size() != 1) return false;
  if (use_sweep_z3(c) || use_sweep_d8(c)) return false;
  const GenericArgs& a = p.a[0][0];
  const LaunchCfg& cf = p.cfg[0][0];
  return a.n_items > 0 && cf.grid == a.n_items &&
         (int64_t)generic_max_active(c->dtype, 2, cf.block, cf.smem) * c->sm_count >= a.n_items;
}

// Record `nsweeps` outer iterations of the parallel schedule onto the stream, starting
// from buffer `start`.
int record_parallel(itn_ctx* c, const ParPlan& p, int start, int nsweeps, const itn_bp_opts* o,
                    int* launches) {
  const bool use_tol = o->tol >= 0;
  if (nsweeps > 0 && c->d_sweepgrid.p && persistent_sweeps_fit(c, p, o)) {
    // sweep t reads buffer (start + t) & 1: msg_buf = {that buffer, the other}
    const int in = start & 1;
    GenericArgs a = p.a[0][in];
    a.pgrid = c->d_sweepgrid.as<SweepGrid>();
    a.msg_buf[0] = c->d_msg[in].p;
    a.msg_buf[1] = c->d_msg[in ^ 1].p;
    a.nsweeps = nsweeps;
    a.wait_ns = c->wait_ns;
    a.pstall = c->stall;
    a.fused_step = 0;
    CK(launch_generic_persistent(c->dtype, a, p.cfg[0][in], c->stream));
    *launches += 2;
    return ITN_OK;
  }
  if (o->precision != ITN_PREC_NATIVE && !use_tol) {
    // Without a convergence test the BF16 sweeps and then the split sweeps each run as
    // one persistent launch; a device that cannot host the cooperative grid gets one
    // launch per sweep.
    const int nsplit = o->precision == ITN_PREC_TF32X3 ? 0 : std::min(nsweeps, std::max(0, o->split_sweeps));
    int t = 0;
    for (int part = 0; part < 2; ++part) {
      const int n = part ? nsplit : nsweeps - nsplit;
      if (n == 0) continue;
      TcRun tr;
      tr.msg_in = c->d_msg[(start + t) & 1].p;
      tr.msg_out = c->d_msg[(start + t + n) & 1].p;
      tr.precision = o->precision;
      tr.split = part == 1;
      tr.normalize = o->normalize;
      tr.slot_diff = nullptr;
      tr.conv = conv(c);
      bool used = false;
      cudaError_t e = tc_sweeps_persistent(c->tc, tr, n, c->stream, &used);
      if (e != cudaSuccess) return cuda_fail(c, e, "persistent tensor-core sweeps");
      if (used) {
        *launches += 1;
      } else {
        for (int k = 0; k < n; ++k) {
          tr.msg_in = c->d_msg[(start + t + k) & 1].p;
          tr.msg_out = c->d_msg[((start + t + k) & 1) ^ 1].p;
          e = tc_sweep(c->tc, tr, c->stream);
          if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core sweep");
          *launches += 1;
        }
      }
      t += n;
    }
    return ITN_OK;
  }
  for (int t = 0; t < nsweeps; ++t) {
    const int in = (start + t) & 1, out = in ^ 1;
    const int prec = o->precision;
    if (prec != ITN_PREC_NATIVE) {
      TcRun tr;
      tr.msg_in = c->d_msg[in].p;
      tr.msg_out = c->d_msg[out].p;
      tr.precision = prec;
      tr.split = t >= nsweeps - o->split_sweeps;
      tr.normalize = o->normalize;
      tr.slot_diff = use_tol ? c->d_slot_diff.as<double>() : nullptr;
      tr.conv = conv(c);
      cudaError_t e = tc_sweep(c->tc, tr, c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core sweep");
    } else if (use_sweep_z3(c)) {
      Z3Args za;
      int grid = 0;
      size_t smem = 0;
      if (int r = plan_z3(c, za, grid, smem, c->z3_budget[c->dtype], c->z3_mult[c->dtype], c->z3_k0[c->dtype],
                          c->d_msg[in].p,
                          c->d_msg[out].p, o->normalize, use_tol ? c->d_slot_diff.as<double>() : nullptr, conv(c)))
        return r;
      CK(launch_sweep_z3(c->dtype, za, grid, smem, c->stream));
    } else if (use_sweep_d8(c)) {
      CK(launch_sweep_d8(c->d_rev.as<int>(), c->d_tens.as<float>(), c->d_msg[in].as<float>(),
                         c->d_msg[out].as<float>(), (int)c->nv, o->normalize,
                         use_tol ? c->d_slot_diff.as<double>() : nullptr, conv(c), c->stream));
    } else {
      for (size_t k = 0; k < p.a.size(); ++k) {
        CK(launch_generic(c->dtype, p.a[k][in], p.cfg[k][in], c->stream));
        if (k > 0) *launches += 1;
      }
    }
    *launches += 1;
  }
  return ITN_OK;
}

struct SeqLaunch {
  GenericArgs a;
  LaunchCfg cfg;
};

int make_seq_launches(itn_ctx* c, const SeqPlan& plan, const itn_bp_opts* o, std::vector<SeqLaunch>& out) {
  void* m = c->d_msg[0].p;
  out.clear();
  for (size_t lv = 0; lv + 1 < plan.level_off.size(); ++lv) {
    const int b = plan.level_off[lv], e = plan.level_off[lv + 1];
    SeqLaunch L;
    if (int r = plan_generic(c, L.a, L.cfg, plan.items->as<int>() + 2 * b, e - b, m, m)) return r;
    L.a.normalize = o->normalize;
    L.a.conv = conv(c);  // early exit once converged; the step is a separate launch
    out.push_back(L);
  }
  return ITN_OK;
}

int record_sequential(itn_ctx* c, const std::vector<SeqLaunch>& lv, int nsweeps, const itn_bp_opts* o,
                      int* launches) {
  const bool use_tol = o->tol >= 0;
  const size_t mbytes = (size_t)c->moff[c->nslots] * dtype_size(c->dtype);
  void* m = c->d_msg[0].p;
  void* prev = c->d_msg[1].p;
  for (int t = 0; t < nsweeps; ++t) {
    if (use_tol) {
      const long long n16 = (long long)(mbytes / 16);
      if (n16 > 0) {
        copy_kernel<<<(int)std::min<long long>((n16 + 255) / 256, 4096), 256, 0, c->stream>>>(
            reinterpret_cast<const int4*>(m), reinterpret_cast<int4*>(prev), n16, conv(c));
        *launches += 1;
      }
      const size_t tail = mbytes - (size_t)n16 * 16;
      if (tail) CK(cudaMemcpyAsync((char*)prev + n16 * 16, (const char*)m + n16 * 16, tail,
                                   cudaMemcpyDeviceToDevice, c->stream));
    }
    for (const SeqLaunch& L : lv) {
      CK(launch_generic(c->dtype, L.a, L.cfg, c->stream));
      *launches += 1;
    }
    if (use_tol) {
      CK(launch_iterate_diff(c->dtype, c->d_moff.as<long long>(), (int)c->nslots, m, prev,
                             c->d_slot_diff.as<double>(), conv(c), c->stream));
      *launches += 1;
    }
    CK(launch_step_check(conv(c), c->stream));
    *launches += 1;
  }
  return ITN_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// Pinned staging layout: the convergence state and the tensor-core error flag first, the
// log-norm totals and flags of itn_bp_solve after them.
constexpr size_t kPinErrAt = (sizeof(ConvState) + 15) & ~size_t(15);
constexpr size_t kPinLogzAt = kPinErrAt + 16;

// The solve behind itn_bp_run.  With `defer`, a run without a tolerance (one chunk) leaves
// its final host synchronisation to the caller: the state copies are enqueued, c->pending
// is filled, and bp_run_finish completes `res` after the caller has synchronised.
int bp_run_impl(itn_ctx* c, const itn_bp_opts* o, itn_bp_result* res, bool defer) {
  if (int r = check_ready(c, true)) return r;
  c->pending.active = false;
  if (!o) return fail(c, ITN_ERR_ARG, "null options");
  if (int r = ensure_device(c)) return r;
  if (o->maxiter < 0 && !(o->tol >= 0))
    return fail(c, ITN_ERR_ARG, "At least one of `maxiter` or `tol` must be specified.");
  if (o->schedule != ITN_SCHED_PARALLEL && o->schedule != ITN_SCHED_SEQUENTIAL)
    return fail(c, ITN_ERR_ARG, "unknown schedule");
  if (o->precision != ITN_PREC_NATIVE) {
    if (o->schedule != ITN_SCHED_PARALLEL)
      return fail(c, ITN_ERR_UNSUPPORTED, "tensor-core precision modes run the parallel schedule");
    if (c->dtype != ITN_F32) return fail(c, ITN_ERR_UNSUPPORTED, "tensor-core precision modes need float32 storage");
    if (!c->tc) {
      c->tc = tc_create();
      tc_set_wait_limit(c->tc, c->wait_ns);
      tc_set_stall(c->tc, c->stall);
    }
    const char* why = nullptr;
    cudaError_t e = tc_prepare(c->tc, c->layers, c->nv, c->off.data(), c->rev.data(), c->moff.data(),
                               c->bond.data(), c->phys.data(), c->d_off.as<int>(), c->d_rev.as<int>(),
                               c->d_moff.as<long long>(), c->d_tens.p, c->toff.data(), o->precision, c->stream,
                               &why);
    if (why) return fail(c, ITN_ERR_UNSUPPORTED, "%s", why);
    if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core prepare");
  }
  if (o->split_sweeps < 0) return fail(c, ITN_ERR_ARG, "split_sweeps < 0");
  if (c->nslots == 0) {
    // No directed edges: every sweep is empty.  iterate_diff would be a maximum over an
    // empty cache, which the reference rejects; with maxiter alone the loop just counts.
    if (o->tol >= 0) return fail(c, ITN_ERR_ARG, "iterate_diff of an empty message cache (no edges)");
    if (res) {
      res->iterations = o->maxiter;
      res->at_iteration = -1;
      res->delta = INFINITY;
      res->device_ms = 0.0;
      res->kernel_launches = 0;
    }
    return ITN_OK;
  }
  SeqPlan plan;
  if (o->schedule == ITN_SCHED_SEQUENTIAL) {
    if (!o->edges && o->n_edges > 0) return fail(c, ITN_ERR_ARG, "null edge list");
    if (int r = get_seq_plan(c, o->edges, o->n_edges, plan)) return r;
    // the sequential schedule works in place on buffer 0
    if (c->cur != 0) {
      CK(cudaMemcpyAsync(c->d_msg[0].p, c->d_msg[1].p, (size_t)c->moff[c->nslots] * dtype_size(c->dtype),
                         cudaMemcpyDeviceToDevice, c->stream));
      c->cur = 0;
    }
  }
  if (int r = sync_programs(c)) return r;
  const bool use_tol = o->tol >= 0;
  ParPlan pplan;
  std::vector<SeqLaunch> slaunch;
  if (o->schedule == ITN_SCHED_PARALLEL && o->precision == ITN_PREC_NATIVE && use_sweep_z3(c)) {
    if (int r = autotune_z3(c)) return r;
  } else if (o->schedule == ITN_SCHED_PARALLEL && o->precision == ITN_PREC_NATIVE && !use_sweep_d8(c)) {
    if (int r = autotune_sweep(c)) return r;
    if (int r = make_par_plan(c, o, pplan)) return r;
    // the persistent sweeps' barrier state (allocated here: no allocation inside a capture)
    if (persistent_sweeps_fit(c, pplan, o)) CK(c->d_sweepgrid.ensure(sizeof(SweepGrid)));
  } else if (o->schedule == ITN_SCHED_SEQUENTIAL) {
    if (int r = make_seq_launches(c, plan, o, slaunch)) return r;
  }
  CK(launch_reset_state(conv(c), use_tol ? o->tol : -1.0, use_tol ? 1 : 0, c->stream));
  int launches = 1;
  // Without a tolerance the whole run is one graph.  With one, sweeps after convergence
  // are no-op launches (~2 us each), so a CUDA-core run goes in growing chunks (16, 32,
  // 64, 64, ...) with one host check of the done flag per chunk; a persistent launch stops
  // at the converged sweep itself, so its chunks are 64 sweeps from the start.  Tensor-core
  // runs keep one graph per maxiter: their split sweeps are the last ones of the graph.
  const int64_t cap = o->maxiter >= 0 ? o->maxiter : 1000000;
  const bool grow = use_tol && (o->precision == ITN_PREC_NATIVE || o->maxiter < 0);
  const bool persistent = o->schedule == ITN_SCHED_PARALLEL && c->d_sweepgrid.p && persistent_sweeps_fit(c, pplan, o);
  int chunk = grow ? (persistent ? 64 : 16) : (o->maxiter >= 0 ? (int)std::min<int64_t>(cap, 1 << 30) : 64);
  int64_t issued = 0;
  float total_ms = 0.f;
  ConvState hs;
  memset(&hs, 0, sizeof(hs));
  // the convergence state and the tensor-core error flag come back in one pinned area
  if (int r = ensure_pinned(c, kPinErrAt + 16)) return r;
  ConvState* h_state = static_cast<ConvState*>(c->h_pin);
  int* h_tcerr = reinterpret_cast<int*>(static_cast<unsigned char*>(c->h_pin) + kPinErrAt);
  // error flag of the sweep's bounded waits: the tensor-core sweep's, or the grid barrier's
  // of persistent CUDA-core sweeps (reset by every persistent launch, so read per chunk)
  const int* d_tcerr = o->precision != ITN_PREC_NATIVE ? tc_err_ptr(c->tc)
                       : persistent ? &c->d_sweepgrid.as<SweepGrid>()->err
                                    : nullptr;
  *h_tcerr = 0;
  while (issued < cap) {
    const int n = (int)std::min<int64_t>(chunk, cap - issued);
    if (grow) chunk = std::min(2 * chunk, 64);
    if (n <= 0) break;
    // one cached graph per (schedule, start buffer, sweep count, options)
    char keyb[256];
    snprintf(keyb, sizeof(keyb), "s%d c%d n%d t%d p%d sp%d nz%d e%p:%lld", o->schedule, c->cur, n,
             use_tol ? 1 : 0, o->precision, o->split_sweeps, o->normalize,
             (const void*)plan.items.get(), (long long)o->n_edges);
    std::string key(keyb);
    if (o->precision != ITN_PREC_NATIVE && n != o->maxiter) key += " chunk";
    cudaGraphExec_t exec = nullptr;
    auto it = c->graphs.find(key);
    int rec_launches = 0;
    if (it != c->graphs.end()) {
      exec = it->second;
      rec_launches = c->graph_launches[key];
    } else {
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      itn_bp_opts oo = *o;
      if (o->precision != ITN_PREC_NATIVE && o->maxiter < 0) oo.split_sweeps = 0;
      int r = o->schedule == ITN_SCHED_PARALLEL ? record_parallel(c, pplan, c->cur, n, &oo, &rec_launches)
                                                : record_sequential(c, slaunch, n, &oo, &rec_launches);
      cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
      if (r) return r;
      if (ce != cudaSuccess) return cuda_fail(c, ce, "stream capture");
      ce = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return cuda_fail(c, ce, "graph instantiate");
      c->graphs[key] = exec;
      c->graph_launches[key] = rec_launches;
    }
    if (o->precision != ITN_PREC_NATIVE) CK(tc_note_launches(c->tc, 2, c->stream));
    char rng[96];
    snprintf(rng, sizeof(rng), "bp sweeps %lld-%lld", (long long)issued + 1, (long long)(issued + n));
    NvtxScope nvtx_chunk(rng);
    CK(cudaEventRecord(c->ev0, c->stream));
    CK(cudaGraphLaunch(exec, c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaMemcpyAsync(h_state, conv(c), sizeof(ConvState), cudaMemcpyDeviceToHost, c->stream));
    if (d_tcerr) CK(cudaMemcpyAsync(h_tcerr, d_tcerr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (defer && !use_tol && issued + n >= cap) {
      // the last (only) chunk of a run without a tolerance: every sweep runs, so the
      // messages end in buffer cur + n whatever the state says
      if (o->schedule == ITN_SCHED_PARALLEL) c->cur = (c->cur + n) & 1;
      c->pending.active = true;
      c->pending.use_tol = false;
      c->pending.tc = d_tcerr != nullptr;
      c->pending.launches = launches + rec_launches;
      c->pending.ms_before = total_ms;
      return ITN_OK;
    }
    CK(cudaStreamSynchronize(c->stream));
    hs = *h_state;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    total_ms += ms;
    launches += rec_launches;
    issued += n;
    if (hs.done || (d_tcerr && *h_tcerr)) break;
  }
  if (d_tcerr && *h_tcerr) return fail(c, ITN_ERR_TIMEOUT, "sweep: a bounded device wait gave up");
  // messages now live in buffer (cur + executed sweeps) for the parallel schedule
  if (o->schedule == ITN_SCHED_PARALLEL) c->cur = (c->cur + hs.iters) & 1;
  if (res) {
    res->iterations = hs.iters;
    res->at_iteration = hs.at_iter;
    res->delta = use_tol ? hs.delta : INFINITY;
    res->device_ms = total_ms;
    res->kernel_launches = launches;
  }
  if (o->maxiter < 0 && !hs.done) return fail(c, ITN_ERR_TIMEOUT, "no convergence within %lld iterations", (long long)cap);
  return ITN_OK;
}

// Completes a deferred run after the caller's synchronisation.
int bp_run_finish(itn_ctx* c, itn_bp_result* res) {
  if (!c->pending.active) return ITN_OK;
  c->pending.active = false;
  const ConvState* h_state = static_cast<const ConvState*>(c->h_pin);
  const int* h_tcerr = reinterpret_cast<const int*>(static_cast<const unsigned char*>(c->h_pin) + kPinErrAt);
  if (c->pending.tc && *h_tcerr) return fail(c, ITN_ERR_TIMEOUT, "sweep: a bounded device wait gave up");
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (res) {
    res->iterations = h_state->iters;
    res->at_iteration = h_state->at_iter;
    res->delta = INFINITY;
    res->device_ms = c->pending.ms_before + ms;
    res->kernel_launches = c->pending.launches;
  }
  return ITN_OK;
}

}  // namespace

extern "C" {

int32_t itn_bp_run(itn_ctx* c, const itn_bp_opts* o, itn_bp_result* res) {
  NvtxScope nvtx_("itn_bp_run");
  if (int r_ = not_busy(c)) return r_;
  return bp_run_impl(c, o, res, false);
}

int32_t itn_message_update(itn_ctx* c, int64_t slot, int32_t normalize) {
  NvtxScope nvtx_("itn_message_update");
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, true)) return r;
  if (slot < 0 || slot >= c->nslots) return fail(c, ITN_ERR_ARG, "slot out of range");
  if (int r = ensure_device(c)) return r;
  SeqPlan plan;
  const int64_t e = slot;
  if (int r = get_seq_plan(c, &e, 1, plan)) return r;
  void* m = c->d_msg[c->cur].p;
  GenericArgs a;
  LaunchCfg cfg;
  if (int r = plan_generic(c, a, cfg, plan.items->as<int>(), 1, m, m)) return r;
  a.normalize = normalize;
  CK(launch_generic(c->dtype, a, cfg, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ITN_OK;
}

int32_t itn_iterate_diff(itn_ctx* c, int32_t dtype, const void* m1, const void* m2, double* out) {
  NvtxScope nvtx_("itn_iterate_diff");
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (!c->have_graph) return fail(c, ITN_ERR_STATE, "no network uploaded");
  if (!m1 || !m2 || !out) return fail(c, ITN_ERR_ARG, "null pointer");
  if (dtype < ITN_F32 || dtype > ITN_C128) return fail(c, ITN_ERR_ARG, "unknown dtype");
  if (int r = ensure_device(c)) return r;
  const size_t bytes = (size_t)c->moff[c->nslots] * dtype_size(dtype);
  DevBuf a, b;
  CK(a.ensure(bytes));
  CK(b.ensure(bytes));
  if (bytes) {
    CK(cudaMemcpyAsync(a.p, m1, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(b.p, m2, bytes, cudaMemcpyHostToDevice, c->stream));
  }
  CK(launch_reset_state(conv(c), -1.0, 0, c->stream));
  CK(launch_iterate_diff(dtype, c->d_moff.as<long long>(), (int)c->nslots, a.p, b.p,
                         c->d_slot_diff.as<double>(), conv(c), c->stream));
  ConvState hs;
  CK(cudaMemcpyAsync(&hs, conv(c), sizeof(hs), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *out = hs.nan_flag ? nan("") : dec_double(hs.dmax);
  return ITN_OK;
}

}  // extern "C"

namespace {

// Z_u (vertex_scalar) into d_zv and Z_e (edge_scalar) into d_ze for the messages m.
int compute_scalars(itn_ctx* c, const void* m) {
  const size_t es = dtype_size(c->dtype);
  const int ne = (int)c->eslots.size();
  CK(c->d_zv.ensure(std::max<int64_t>(c->nv, 1) * es));
  CK(c->d_ze.ensure(std::max(ne, 1) * es));
  // the register-resident kernel for float / complex64 (the 8-byte types would spill)
  if (c->nv > 0 && c->scal_d8 && (c->dtype == ITN_F32 || c->dtype == ITN_C64)) {
    CK(launch_vertex_scalars_d8(c->dtype, (int)c->nv, c->d_rev.as<int>(), c->d_moff.as<long long>(),
                                c->d_toff.as<long long>(), c->d_tens.p, m, c->d_zv.p, c->stream));
  } else if (c->nv > 0) {
    GenericArgs a;
    LaunchCfg cfg;
    if (int r = plan_generic(c, a, cfg, c->d_items_scal.as<int>(), (int)c->items_scal.size() / 2, m,
                             const_cast<void*>(m)))
      return r;
    a.zv_out = c->d_zv.p;
    CK(launch_generic(c->dtype, a, cfg, c->stream));
  }
  CK(launch_edge_scalars(c->dtype, c->layers, c->d_moff.as<long long>(), c->d_rev.as<int>(),
                         c->d_eslots.as<int>(), ne, m, c->d_ze.p, c->stream));
  return ITN_OK;
}

// Launch plan of the dual-number interpreter (two planes per buffer, two message stagings).
int plan_dual(itn_ctx* c, GenericArgs& a, LaunchCfg& cfg, const int* d_items, int n_items, const void* m) {
  memset(&a, 0, sizeof(a));
  a.layers = 2;
  a.off = c->d_off.as<int>();
  a.rev = c->d_rev.as<int>();
  a.bond = c->d_bond.as<int>();
  a.phys = c->d_phys.as<int>();
  a.toff = c->d_toff.as<long long>();
  a.moff = c->d_moff.as<long long>();
  a.tens = c->d_tens.p;
  a.msg_in = m;
  a.items = d_items;
  a.n_items = n_items;
  a.prog = c->d_prog.as<unsigned>();
  a.nbuf = 2 * c->nbuf;
  a.buf_elems = (c->max_tensor + 15) & ~15LL;
  a.msg_cap = 2 * c->msg_cap;
  a.max_d2 = c->max_d2;
  cfg.block = c->dtype >= 0 && c->dtype < 4 && c->dual_block[c->dtype] > 0 ? c->dual_block[c->dtype] : block_for(c);
  bool in_smem = true;
  size_t smem = generic_smem_bytes(c->dtype, a, cfg.block, true);
  if (smem > (size_t)c->smem_optin) {
    in_smem = false;
    smem = generic_smem_bytes(c->dtype, a, cfg.block, false);
    if (smem > (size_t)c->smem_optin)
      return fail(c, ITN_ERR_UNSUPPORTED, "vertex needs %zu bytes of shared staging", smem);
  }
  int per_sm = dual_max_active(c->dtype, cfg.block, smem);
  if (per_sm <= 0) per_sm = 1;
  cfg.grid = std::max(1, std::min(n_items, c->sm_count * per_sm));
  cfg.smem = smem;
  if (!in_smem) {
    const size_t need = (size_t)cfg.grid * a.nbuf * a.buf_elems * dtype_size(c->dtype);
    CK(c->d_scratch.ensure(need));
    a.gscratch = c->d_scratch.p;
  }
  return ITN_OK;
}

// Unnormalised updates U = M(m) of one parallel sweep, their sums S and F = U / S.
int adjoint_prepare(itn_ctx* c, const void* m, int normalized) {
  const size_t mb = (size_t)c->moff[c->nslots] * dtype_size(c->dtype);
  const int ns = (int)c->nslots, np = (int)c->items_par.size() / 2;
  CK(c->d_U.ensure(std::max<size_t>(mb, 16)));
  CK(c->d_F.ensure(std::max<size_t>(mb, 16)));
  CK(c->d_mu.ensure(std::max<size_t>(mb, 16)));
  CK(c->d_cot.ensure(std::max<size_t>(mb, 16)));
  CK(c->d_S.ensure(std::max<size_t>(ns, 1) * dtype_size(c->dtype)));
  GenericArgs pa;
  LaunchCfg pcfg;
  if (int r = plan_generic(c, pa, pcfg, c->d_items_par.as<int>(), np, m, c->d_U.p)) return r;
  pa.normalize = 0;
  CK(launch_generic(c->dtype, pa, pcfg, c->stream));
  CK(launch_grad_prep(c->dtype, c->d_moff.as<long long>(), ns, c->d_U.p, c->d_F.p, c->d_S.p, normalized,
                      c->stream));
  return ITN_OK;
}

// cot = J^T lam for the sweep m -> F(m) (needs adjoint_prepare): lam is projected through
// the normalisation (mu = (lam - <lam, F>) / S) and pushed back through the products by
// the dual interpreter (tangent of the leave-one-out contraction on every leg).
// Autotuner for the dual launches (the J^T products of the adjoint iteration): time one
// launch per candidate CTA size -- 64 and 128 threads with the unrestricted kernel, 256 with
// the 128-register one (two CTAs per SM) -- on tangents from c->d_mu into c->d_cot, and keep
// the fastest for this network and dtype.  Runs outside any capture (it plans, which may size
// the global scratch, and it synchronises).
int autotune_dual(itn_ctx* c, const void* m) {
  if (c->dtype < 0 || c->dtype >= 4 || c->dual_block[c->dtype] != 0 || c->items_par.empty()) return ITN_OK;
  if (getenv("ITN_NO_AUTOTUNE")) {
    c->dual_block[c->dtype] = -1;
    return ITN_OK;
  }
  std::array<int, 3> cached;
  if (tune_lookup(c, "dual", cached)) {
    c->dual_block[c->dtype] = cached[0];
    return ITN_OK;
  }
  const int cands[3] = {64, 128, 256};
  float best = 1e30f;
  int best_b = 0;
  for (int b : cands) {
    c->dual_block[c->dtype] = b;
    GenericArgs a;
    LaunchCfg cfg;
    if (plan_dual(c, a, cfg, c->d_items_par.as<int>(), (int)c->items_par.size() / 2, m)) {
      cudaGetLastError();
      continue;
    }
    DualArgs d;
    memset(&d, 0, sizeof(d));
    d.tan_in = c->d_mu.p;
    d.tan_out = c->d_cot.p;
    float ms = 1e30f;
    for (int rep = 0; rep < 7; ++rep) {  // the first launch warms the caches; best of six
      float t = 0.f;
      CK(cudaEventRecord(c->ev0, c->stream));
      CK(launch_dual(c->dtype, a, d, cfg, c->stream));
      CK(cudaEventRecord(c->ev1, c->stream));
      CK(cudaEventSynchronize(c->ev1));
      CK(cudaEventElapsedTime(&t, c->ev0, c->ev1));
      if (rep > 0) ms = std::min(ms, t);
    }
    if (ms < best) {
      best = ms;
      best_b = b;
    }
  }
  c->dual_block[c->dtype] = best_b > 0 ? best_b : -1;
  tune_store(c, "dual", {c->dual_block[c->dtype], 0, 0});
  if (getenv("ITN_DEBUG")) fprintf(stderr, "[itn] autotune: dual CTA size %d (%.4f ms)\n", best_b, best);
  return ITN_OK;
}

int apply_jt(itn_ctx* c, const void* m, const void* lam, void* cot, int normalized, const int* done = nullptr) {
  const int ns = (int)c->nslots, np = (int)c->items_par.size() / 2;
  CK(launch_grad_mu(c->dtype, c->d_moff.as<long long>(), ns, lam, c->d_F.p, c->d_S.p, c->d_mu.p, normalized,
                    done, c->stream));
  GenericArgs da;
  LaunchCfg dcfg;
  if (int r = plan_dual(c, da, dcfg, c->d_items_par.as<int>(), np, m)) return r;
  DualArgs dd;
  memset(&dd, 0, sizeof(dd));
  dd.tan_in = c->d_mu.p;
  dd.tan_out = cot;
  dd.done = done;
  CK(launch_dual(c->dtype, da, dd, dcfg, c->stream));
  return ITN_OK;
}

// One parallel sweep in -> out of the native CUDA-core kernel over every vertex (the
// forward map of the unrolled gradient; no convergence bookkeeping).
int sweep_native(itn_ctx* c, const void* in, void* out, int normalized) {
  GenericArgs a;
  LaunchCfg cfg;
  if (int r = plan_generic(c, a, cfg, c->d_items_par.as<int>(), (int)c->items_par.size() / 2, in, out)) return r;
  a.normalize = normalized;
  CK(launch_generic(c->dtype, a, cfg, c->stream));
  return ITN_OK;
}

// grad += lambda^T dF/dA at messages m (the tangent plane of the all-legs contraction with
// mu = the projection of lambda through the normalisation); needs adjoint_prepare(m).
int add_lambda_dfda(itn_ctx* c, const void* m, const void* lam, int normalized) {
  const int ns = (int)c->nslots, nd = (int)c->items_dump.size() / 2;
  CK(launch_grad_mu(c->dtype, c->d_moff.as<long long>(), ns, lam, c->d_F.p, c->d_S.p, c->d_mu.p, normalized,
                    nullptr, c->stream));
  GenericArgs a;
  LaunchCfg cfg;
  if (int r = plan_dual(c, a, cfg, c->d_items_dump.as<int>(), nd, m)) return r;
  DualArgs d;
  memset(&d, 0, sizeof(d));
  d.grad_out = c->d_grad.p;
  d.zv = c->d_zv.p;
  d.tan_in = c->d_mu.p;
  d.dump_tangent = 1;
  for (int tr = 0; tr < 2; ++tr) {
    d.transpose = tr;
    CK(launch_dual(c->dtype, a, d, cfg, c->stream));
  }
  return ITN_OK;
}

// The direct term dlogZ_u/dA_u = (T_u(m) + T_u(m^T)) / Z_u into d_grad (zeroed first);
// computes the scalars of m.
int grad_direct(itn_ctx* c, const void* m) {
  const size_t tb = (size_t)c->toff[c->nv] * dtype_size(c->dtype);
  if (int r = compute_scalars(c, m)) return r;
  CK(c->d_grad.ensure(std::max<size_t>(tb, 16)));
  CK(cudaMemsetAsync(c->d_grad.p, 0, tb, c->stream));
  const int nd = (int)c->items_dump.size() / 2;
  GenericArgs a;
  LaunchCfg cfg;
  if (int r = plan_dual(c, a, cfg, c->d_items_dump.as<int>(), nd, m)) return r;
  DualArgs d;
  memset(&d, 0, sizeof(d));
  d.grad_out = c->d_grad.p;
  d.zv = c->d_zv.p;
  for (int tr = 0; tr < 2; ++tr) {
    d.transpose = tr;
    CK(launch_dual(c->dtype, a, d, cfg, c->stream));
  }
  return ITN_OK;
}

// Unrolled gradient (itn_grad_opts.sweeps > 0): T = sweeps parallel sweeps m_t = F(m_{t-1})
// from the current messages, then the reverse pass
//   lambda_T = dL/dm_T,  grad = dL/dA|m_T + sum_{t=T..1} lambda_t^T dF/dA(m_{t-1}),
//   lambda_{t-1} = J(m_{t-1})^T lambda_t.
// Sweep states m_s with s % k == 0 (k = checkpoint) are kept; the others of a segment
// [c0 + 1, c0 + k - 1] are recomputed from m_{c0} when the reverse pass enters it.
int grad_unrolled(itn_ctx* c, const itn_grad_opts* o, void* grad, itn_grad_result* res) {
  const int T = o->sweeps, k = std::max(1, o->checkpoint);
  const size_t es = dtype_size(c->dtype);
  const size_t tb = (size_t)c->toff[c->nv] * es, mb = (size_t)c->moff[c->nslots] * es;
  const size_t mbs = std::max<size_t>((mb + 255) & ~(size_t)255, 256);
  const int ns = (int)c->nslots;
  const int nck = (T - 1) / k + 1;  // kept states m_0, m_k, ... (indices < T)
  CK(c->d_ckpt.ensure((size_t)nck * mbs));
  CK(c->d_seg.ensure((size_t)(k + 1) * mbs));  // a segment's k - 1 states + two forward buffers
  unsigned char* ck = static_cast<unsigned char*>(c->d_ckpt.p);
  unsigned char* seg = static_cast<unsigned char*>(c->d_seg.p);
  auto ckpt = [&](int s) { return (void*)(ck + (size_t)(s / k) * mbs); };
  auto segp = [&](int j) { return (void*)(seg + (size_t)j * mbs); };  // m_{c0 + 1 + j}
  void* fwd[2] = {segp(k - 1), segp(k)};  // forward scratch (past the segment slots)
  void* cur_msg = c->d_msg[c->cur].p;
  CK(cudaEventRecord(c->ev0, c->stream));
  // forward
  if (mb) CK(cudaMemcpyAsync(ckpt(0), cur_msg, mb, cudaMemcpyDeviceToDevice, c->stream));
  const void* prev = ckpt(0);
  for (int t = 1; t <= T; ++t) {
    void* out = (t < T && t % k == 0) ? ckpt(t) : fwd[t & 1];
    if (t == T) out = cur_msg;  // the context ends holding m_T
    if (int r = sweep_native(c, prev, out, o->normalized)) return r;
    prev = out;
  }
  // direct term and lambda_T at m_T
  if (int r = grad_direct(c, cur_msg)) return r;
  CK(c->d_g.ensure(std::max<size_t>(mb, 16)));
  CK(c->d_lam.ensure(std::max<size_t>(mb, 16)));
  if (int r = adjoint_prepare(c, cur_msg, o->normalized)) return r;
  CK(launch_grad_g(c->dtype, c->d_moff.as<long long>(), c->d_rev.as<int>(), c->d_slot_dst.as<int>(),
                   c->d_slot_eidx.as<int>(), ns, c->d_U.p, cur_msg, c->d_zv.p, c->d_ze.p, c->d_lam.p, c->stream));
  // reverse pass
  int seg_base = -1;  // segment currently recomputed: states m_{seg_base + 1 ..}
  for (int t = T; t >= 1; --t) {
    const int s = t - 1;
    const void* ms;
    if (s % k == 0) {
      ms = ckpt(s);
    } else {
      const int c0 = s - s % k;
      if (seg_base != c0) {
        const void* p = ckpt(c0);
        for (int j = 0; j + 1 < k && c0 + 1 + j < T; ++j) {
          if (int r = sweep_native(c, p, segp(j), o->normalized)) return r;
          p = segp(j);
        }
        seg_base = c0;
      }
      ms = segp(s - c0 - 1);
    }
    if (int r = adjoint_prepare(c, ms, o->normalized)) return r;
    if (int r = add_lambda_dfda(c, ms, c->d_lam.p, o->normalized)) return r;
    if (t > 1) {
      if (int r = apply_jt(c, ms, c->d_lam.p, c->d_cot.p, o->normalized)) return r;
      // lambda_{t-1} is in d_cot: exchange the two buffers (pointers, not contents)
      std::swap(c->d_lam.p, c->d_cot.p);
      std::swap(c->d_lam.bytes, c->d_cot.bytes);
    }
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  if (tb) CK(cudaMemcpyAsync(grad, c->d_grad.p, tb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (res) {
    res->adjoint_iterations = T;
    res->adjoint_residual = 0.0;
    res->device_ms = ms;
  }
  return ITN_OK;
}

}  // namespace

extern "C" {

int32_t itn_sweep_vjp(itn_ctx* c, int32_t normalized, const void* cot_out, void* cot_in) {
  NvtxScope nvtx_("itn_sweep_vjp");
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, true)) return r;
  if (!cot_out || !cot_in) return fail(c, ITN_ERR_ARG, "null cotangent pointer");
  if (c->dtype != ITN_F32 && c->dtype != ITN_F64)
    return fail(c, ITN_ERR_UNSUPPORTED, "the sweep VJP is implemented for real site tensors");
  if (c->layers != 2) return fail(c, ITN_ERR_UNSUPPORTED, "the sweep VJP is implemented for norm networks");
  if (int r = ensure_device(c)) return r;
  const size_t mb = (size_t)c->moff[c->nslots] * dtype_size(c->dtype);
  const void* m = c->d_msg[c->cur].p;
  if (int r = adjoint_prepare(c, m, normalized)) return r;
  CK(c->d_lam.ensure(std::max<size_t>(mb, 16)));
  CK(c->d_g.ensure(std::max<size_t>(mb, 16)));
  if (mb) CK(cudaMemcpyAsync(c->d_lam.p, cot_out, mb, cudaMemcpyHostToDevice, c->stream));
  if (int r = apply_jt(c, m, c->d_lam.p, c->d_g.p, normalized)) return r;
  if (mb) CK(cudaMemcpyAsync(cot_in, c->d_g.p, mb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return ITN_OK;
}

int32_t itn_bp_grad(itn_ctx* c, const itn_grad_opts* o, void* grad, itn_grad_result* res) {
  NvtxScope nvtx_("itn_bp_grad");
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, true)) return r;
  if (!grad) return fail(c, ITN_ERR_ARG, "null gradient pointer");
  if (c->dtype != ITN_F32 && c->dtype != ITN_F64)
    return fail(c, ITN_ERR_UNSUPPORTED, "the gradient is implemented for real site tensors");
  if (c->layers != 2) return fail(c, ITN_ERR_UNSUPPORTED, "the gradient is implemented for norm networks");
  if (int r = ensure_device(c)) return r;
  itn_grad_opts def = {1, 200, 1e-10, 1, 0, 1, 0};
  if (!o) o = &def;
  if (o->sweeps < 0) return fail(c, ITN_ERR_ARG, "sweeps < 0");
  if (o->sweeps > 0) return grad_unrolled(c, o, grad, res);
  const int dt = c->dtype;
  const size_t es = dtype_size(dt);
  const size_t tb = (size_t)c->toff[c->nv] * es, mb = (size_t)c->moff[c->nslots] * es;
  const int ns = (int)c->nslots;
  const void* m = c->d_msg[c->cur].p;
  CK(cudaEventRecord(c->ev0, c->stream));
  if (int r = compute_scalars(c, m)) return r;
  CK(c->d_grad.ensure(std::max<size_t>(tb, 16)));
  CK(cudaMemsetAsync(c->d_grad.p, 0, tb, c->stream));
  const int nd = (int)c->items_dump.size() / 2, np = (int)c->items_par.size() / 2;
  // direct term: dlogZ_u/dA_u = (T_u(m) + T_u(m^T)) / Z_u -- here without the adjoint, after
  // the adjoint loop with its correction in the same two launches
  GenericArgs a;
  LaunchCfg cfg;
  DualArgs d;
  memset(&d, 0, sizeof(d));
  d.grad_out = c->d_grad.p;
  d.zv = c->d_zv.p;
  if (!o->adjoint) {
    if (int r = plan_dual(c, a, cfg, c->d_items_dump.as<int>(), nd, m)) return r;
    for (int tr = 0; tr < 2; ++tr) {
      d.transpose = tr;
      CK(launch_dual(dt, a, d, cfg, c->stream));
    }
  }
  int iters = 0;
  double resid = 0.0;
  if (o->adjoint) {
    CK(c->d_g.ensure(std::max<size_t>(mb, 16)));
    CK(c->d_lam.ensure(std::max<size_t>(mb, 16)));
    CK(c->d_adj.ensure(sizeof(AdjState)));
    if (int r = adjoint_prepare(c, m, o->normalized)) return r;
    // g = dL/dm, lambda_0 = g
    CK(launch_grad_g(dt, c->d_moff.as<long long>(), c->d_rev.as<int>(), c->d_slot_dst.as<int>(),
                     c->d_slot_eidx.as<int>(), ns, c->d_U.p, m, c->d_zv.p, c->d_ze.p, c->d_g.p, c->stream));
    CK(cudaMemcpyAsync(c->d_lam.p, c->d_g.p, mb, cudaMemcpyDeviceToDevice, c->stream));
    // adjoint BP: lambda <- g + J^T lambda until the relative change is below tol.  The
    // stopping rule runs on the device (AdjState); iterations are enqueued in chunks and
    // the host reads the state once per chunk (launches after the stop return at once).
    // An iteration is two launches: the dual interpreter (J^T through the products, from
    // mu) and the fused update (lambda, the next mu and the stopping rule).
    AdjState* adj = c->d_adj.as<AdjState>();
    const int maxit = std::max(o->maxiter, 0);
    CK(launch_adj_reset(adj, o->tol, maxit, c->stream));
    CK(launch_grad_mu(dt, c->d_moff.as<long long>(), ns, c->d_lam.p, c->d_F.p, c->d_S.p, c->d_mu.p,
                      o->normalized, nullptr, c->stream));
    AdjState hs;
    memset(&hs, 0, sizeof(hs));
    CK(c->d_mu2.ensure(std::max<size_t>(mb, 16)));
    // One adjoint iteration is one launch: the dual program (J^T mu through the products)
    // with the update fused into its final contractions (lambda, the next mu and, in the
    // last CTA, the device-side stopping rule).  mu alternates between two buffers (the
    // launch reads one while it writes the other), so iteration k reads buffer k & 1; a
    // chunk of kAdjChunk (even) iterations is captured once as a CUDA graph per set of
    // buffers and replayed, so the launches do not wait on the host.  The iterations after
    // convergence return at once (done flag).
    void* mu_buf[2] = {c->d_mu.p, c->d_mu2.p};
    int adj_k = 0;
    auto adj_iteration = [&]() -> int {
      if (c->items_par.empty()) {
        // no messages: the stopping rule alone (a zero change stops the loop at once)
        CK(launch_adj_step(adj, c->stream));
        return ITN_OK;
      }
      GenericArgs da;
      LaunchCfg dcfg;
      if (int r = plan_dual(c, da, dcfg, c->d_items_par.as<int>(), (int)c->items_par.size() / 2, m)) return r;
      DualArgs dd;
      memset(&dd, 0, sizeof(dd));
      dd.tan_in = mu_buf[adj_k & 1];
      dd.done = &adj->done;
      dd.adj = adj;
      dd.g = c->d_g.p;
      dd.lam = c->d_lam.p;
      dd.F = c->d_F.p;
      dd.S = c->d_S.p;
      dd.mu_next = mu_buf[(adj_k + 1) & 1];
      dd.normalize = o->normalized;
      ++adj_k;
      CK(launch_dual(c->dtype, da, dd, dcfg, c->stream));
      return ITN_OK;
    };
    constexpr int kAdjChunk = 8;
    static_assert(kAdjChunk % 2 == 0, "every chunk starts from mu buffer 0");
    // The dual program's plan, made outside the capture (it sizes the global scratch, and no
    // allocation may happen inside a capture).  The cache key holds the plan's bytes (every
    // pointer and size baked into the captured launches) and the update's buffers, so a graph
    // is replayed only on exactly the state it was captured for.
    GenericArgs pa;
    LaunchCfg pc;
    memset(&pa, 0, sizeof(pa));
    memset(&pc, 0, sizeof(pc));
    if (int r = autotune_dual(c, m)) return r;
    if (int r = plan_dual(c, pa, pc, c->d_items_par.as<int>(), (int)c->items_par.size() / 2, m)) return r;
    std::string key("adjoint ");
    key.append(reinterpret_cast<const char*>(&pa), sizeof(pa));
    key.append(reinterpret_cast<const char*>(&pc), sizeof(pc));
    char tail[320];
    snprintf(tail, sizeof(tail), " fused %d %d %d %p %p %p %p %p %p %p %p %p", dt, o->normalized, ns, m,
             c->d_mu2.p, c->d_mu.p, c->d_lam.p, c->d_g.p, c->d_F.p, c->d_S.p, (void*)adj, c->d_moff.p);
    key += tail;
    // The whole loop as one cooperative launch when every work item gets its own resident CTA:
    // the site tensors and value messages are staged once, and a grid barrier with the stopping
    // rule replaces the launch boundary and the host checks between chunks (the same
    // arithmetic, iteration for iteration).  Otherwise (or when the launch is refused) chunks
    // of captured launches as below.
    bool persisted = false;
    const int n_par = (int)c->items_par.size() / 2;
    if (!c->no_persist_adj && maxit > 0 && n_par > 0 && pc.grid == n_par &&
        (int64_t)dual_max_active(dt, pc.block, pc.smem) * c->sm_count >= n_par) {
      CK(c->d_adjgrid.ensure(sizeof(AdjGrid)));
      AdjGrid hg;
      memset(&hg, 0, sizeof(hg));
      for (int q = 0; q < 3; ++q) hg.dmax[q] = hg.lmax[q] = 0x8000000000000000ull;  // encoded 0.0
      CK(cudaMemcpyAsync(c->d_adjgrid.p, &hg, sizeof(hg), cudaMemcpyHostToDevice, c->stream));
      DualArgs dd;
      memset(&dd, 0, sizeof(dd));
      dd.done = &adj->done;
      dd.adj = adj;
      dd.g = c->d_g.p;
      dd.lam = c->d_lam.p;
      dd.F = c->d_F.p;
      dd.S = c->d_S.p;
      dd.normalize = o->normalized;
      dd.grid = c->d_adjgrid.as<AdjGrid>();
      dd.mu_buf[0] = c->d_mu.p;
      dd.mu_buf[1] = c->d_mu2.p;
      dd.wait_ns = c->wait_ns;
      dd.stall = c->stall;
      cudaError_t e = launch_dual_persistent(dt, pa, dd, pc, c->stream);
      if (e == cudaSuccess) {
        persisted = true;
        AdjGrid hgo;
        CK(cudaMemcpyAsync(&hs, adj, sizeof(hs), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(&hgo, c->d_adjgrid.p, sizeof(hgo), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (hgo.err) return fail(c, ITN_ERR_TIMEOUT, "adjoint iteration: a grid-barrier wait gave up");
      } else if (e == cudaErrorCooperativeLaunchTooLarge) {
        cudaGetLastError();
      } else {
        return cuda_fail(c, e, "persistent adjoint launch");
      }
    }
    for (int issued = 0; !persisted && issued < maxit;) {
      const int chunk = std::min(maxit - issued, kAdjChunk);
      adj_k = issued;  // even: the chunk starts reading mu buffer 0
      if (chunk == kAdjChunk) {
        auto it = c->graphs.find(key);
        if (it == c->graphs.end()) {
          cudaGraph_t graph = nullptr;
          cudaGraphExec_t exec = nullptr;
          CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
          int r = ITN_OK;
          for (int k = 0; k < chunk && r == ITN_OK; ++k) r = adj_iteration();
          cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
          if (r) {
            if (graph) cudaGraphDestroy(graph);
            return r;
          }
          if (ce != cudaSuccess) return cuda_fail(c, ce, "adjoint stream capture");
          ce = cudaGraphInstantiate(&exec, graph, 0);
          cudaGraphDestroy(graph);
          if (ce != cudaSuccess) return cuda_fail(c, ce, "adjoint graph instantiate");
          it = c->graphs.emplace(key, exec).first;
          c->graph_launches[key] = chunk;
        }
        CK(cudaGraphLaunch(it->second, c->stream));
      } else {
        for (int k = 0; k < chunk; ++k)
          if (int r = adj_iteration()) return r;
      }
      issued += chunk;
      CK(cudaMemcpyAsync(&hs, adj, sizeof(hs), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      if (hs.done) break;
    }
    iters = hs.iters;
    resid = hs.resid;
    if (hs.nan) return fail(c, ITN_ERR_NAN, "adjoint iteration produced NaN");
    // direct term + the correction lambda^T dF/dA (tangent part of the all-legs contraction
    // with mu): value plane / Z_u + tangent plane, in one launch per orientation
    CK(launch_grad_mu(dt, c->d_moff.as<long long>(), ns, c->d_lam.p, c->d_F.p, c->d_S.p, c->d_mu.p,
                      o->normalized, nullptr, c->stream));
    if (int r = plan_dual(c, a, cfg, c->d_items_dump.as<int>(), nd, m)) return r;
    d.tan_in = c->d_mu.p;
    d.dump_tangent = 2;
    for (int tr = 0; tr < 2; ++tr) {
      d.transpose = tr;
      CK(launch_dual(dt, a, d, cfg, c->stream));
    }
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  if (tb) CK(cudaMemcpyAsync(grad, c->d_grad.p, tb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (res) {
    res->adjoint_iterations = iters;
    res->adjoint_residual = resid;
    res->device_ms = ms;
  }
  if (o->adjoint && o->maxiter > 0 && !(resid < o->tol))
    return fail(c, ITN_ERR_TIMEOUT, "adjoint iteration did not reach tol %g in %d iterations (residual %g)",
                o->tol, o->maxiter, resid);
  return ITN_OK;
}

int32_t itn_tc_selftest(itn_ctx* c, int32_t* m128_ok, int32_t* m64_ok, double* max_err,
                        int32_t* lane_of_row) {
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (int r = ensure_device(c)) return r;
  int a = 0, b = 0, lr[64];
  double mx = 0;
  CK(tc_run_probe(c->stream, &a, &b, &mx, lr));
  if (m128_ok) *m128_ok = a;
  if (m64_ok) *m64_ok = b;
  if (max_err) *max_err = mx;
  if (lane_of_row)
    for (int r = 0; r < 64; ++r) lane_of_row[r] = lr[r];
  return ITN_OK;
}

}  // extern "C"

namespace {

// Enqueue the vertex / edge scalars, their FP64 logs and the per-network totals and flags
// of the current messages (no copies, no synchronisation).
int enqueue_logscalars(itn_ctx* c) {
  const int ne = (int)c->eslots.size();
  CK(c->d_logzv.ensure(std::max<int64_t>(c->nv, 1) * 2 * sizeof(double)));
  CK(c->d_logze.ensure(std::max(ne, 1) * 2 * sizeof(double)));
  CK(c->d_tot.ensure(c->n_nets * 2 * sizeof(double)));
  CK(c->d_flags.ensure(c->n_nets * sizeof(int)));
  if (int r = compute_scalars(c, c->d_msg[c->cur].p)) return r;
  const size_t part_bytes = (size_t)((c->nv + ne + 127) / 128 + 1) * 20;
  CK(c->d_lspart.ensure(part_bytes));
  CK(launch_logsum(c->dtype, c->d_zv.p, c->d_ze.p, (int)c->nv, ne, c->d_net_voff.as<int>(),
                   c->d_net_vlist.as<int>(), c->d_net_eoff.as<int>(), c->d_net_elist.as<int>(), c->n_nets,
                   c->d_logzv.as<double>(), c->d_logze.as<double>(), c->d_tot.as<double>(),
                   c->d_flags.as<int>(), c->d_lspart.p, part_bytes, c->stream));
  return ITN_OK;
}

}  // namespace

extern "C" {

int32_t itn_logscalars(itn_ctx* c, void* zv, void* ze, double* logzv, double* logze,
                       double* totals, int32_t* flags) {
  NvtxScope nvtx_("itn_logscalars");
  if (int r_ = not_busy(c)) return r_;
  if (int r = check_ready(c, true)) return r;
  if (int r = ensure_device(c)) return r;
  const size_t es = dtype_size(c->dtype);
  const int ne = (int)c->eslots.size();
  if (int r = enqueue_logscalars(c)) return r;
  // every requested result goes through one pinned staging area: the copies are queued
  // back to back and waited for once
  struct Part { void* dst; const void* src; size_t bytes; size_t at; };
  Part parts[6] = {{zv, c->d_zv.p, c->nv ? (size_t)c->nv * es : 0, 0},
                   {ze, c->d_ze.p, (size_t)ne * es, 0},
                   {logzv, c->d_logzv.p, (size_t)c->nv * 2 * sizeof(double), 0},
                   {logze, c->d_logze.p, (size_t)ne * 2 * sizeof(double), 0},
                   {totals, c->d_tot.p, (size_t)c->n_nets * 2 * sizeof(double), 0},
                   {flags, c->d_flags.p, (size_t)c->n_nets * sizeof(int), 0}};
  size_t need = 0;
  for (Part& p : parts)
    if (p.dst && p.bytes) {
      p.at = need;
      need += (p.bytes + 15) & ~size_t(15);
    }
  if (int r = ensure_pinned(c, need)) return r;
  unsigned char* h = static_cast<unsigned char*>(c->h_pin);
  for (const Part& p : parts)
    if (p.dst && p.bytes) CK(cudaMemcpyAsync(h + p.at, p.src, p.bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (const Part& p : parts)
    if (p.dst && p.bytes) memcpy(p.dst, h + p.at, p.bytes);
  return ITN_OK;
}

int32_t itn_bp_solve_submit(itn_ctx* c, int32_t dtype, const void* tensors, const void* messages_in,
                            const itn_bp_opts* o, void* messages_out, int32_t logz) {
  NvtxScope nvtx_("itn_bp_solve_submit");
  if (!c) return ITN_ERR_ARG;
  if (int r = not_busy(c)) return r;
  if (!c->have_graph) return fail(c, ITN_ERR_STATE, "upload the network first");
  if (!o) return fail(c, ITN_ERR_ARG, "null options");
  const size_t tb = (size_t)c->toff[c->nv] * (dtype >= ITN_F32 && dtype <= ITN_C128 ? dtype_size(dtype) : 0);
  if (int r = set_dtype(c, dtype)) return r;
  const size_t mb = (size_t)c->moff[c->nslots] * dtype_size(dtype);
  if ((tb && !tensors) || (mb && !messages_in)) return fail(c, ITN_ERR_ARG, "null tensor or message pointer");
  if (int r = ensure_device(c)) return r;
  // inputs: copies queued on the context's stream, no host wait
  CK(c->d_tens.ensure(tb));
  if (tb) CK(cudaMemcpyAsync(c->d_tens.p, tensors, tb, cudaMemcpyHostToDevice, c->stream));
  CK(c->d_msg[0].ensure(mb));
  CK(c->d_msg[1].ensure(mb));
  if (mb) CK(cudaMemcpyAsync(c->d_msg[0].p, messages_in, mb, cudaMemcpyHostToDevice, c->stream));
  c->cur = 0;
  c->have_tensors = true;
  c->have_messages = true;
  if (c->tc) tc_invalidate(c->tc);
  // the staging is sized before the solve queues its state copies into it (growing it
  // afterwards would move it under those copies)
  if (int r = ensure_pinned(c, kPinLogzAt + 20 * (size_t)c->n_nets + 16)) return r;
  // the solve (its last synchronisation deferred when it has no tolerance)
  c->submitted.res = itn_bp_result{};
  if (int r = bp_run_impl(c, o, &c->submitted.res, true)) return r;
  // log-norm and the messages, queued behind the solve
  unsigned char* h = static_cast<unsigned char*>(c->h_pin) + kPinLogzAt;
  if (logz) {
    if (int r = enqueue_logscalars(c)) return r;
    CK(cudaMemcpyAsync(h, c->d_tot.p, 16 * (size_t)c->n_nets, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(h + 16 * (size_t)c->n_nets, c->d_flags.p, 4 * (size_t)c->n_nets, cudaMemcpyDeviceToHost,
                       c->stream));
  }
  if (messages_out && mb)
    CK(cudaMemcpyAsync(messages_out, c->d_msg[c->cur].p, mb, cudaMemcpyDeviceToHost, c->stream));
  c->submitted.active = true;
  c->submitted.logz = logz != 0;
  return ITN_OK;
}

int32_t itn_bp_solve_wait(itn_ctx* c, itn_bp_result* res, double* totals, int32_t* flags) {
  NvtxScope nvtx_("itn_bp_solve_wait");
  if (!c) return ITN_ERR_ARG;
  if (!c->submitted.active) return fail(c, ITN_ERR_STATE, "no solve was submitted");
  c->submitted.active = false;
  CK(cudaStreamSynchronize(c->stream));
  // a run without a tolerance completes here; one with a tolerance already did in the submit
  if (res && !c->pending.active) *res = c->submitted.res;
  if (int r = bp_run_finish(c, res)) return r;
  if ((totals || flags) && !c->submitted.logz)
    return fail(c, ITN_ERR_ARG, "the solve was submitted without the log-norm");
  const unsigned char* h = static_cast<const unsigned char*>(c->h_pin) + kPinLogzAt;
  if (totals) memcpy(totals, h, 16 * (size_t)c->n_nets);
  if (flags) memcpy(flags, h + 16 * (size_t)c->n_nets, 4 * (size_t)c->n_nets);
  return ITN_OK;
}

int32_t itn_bp_solve(itn_ctx* c, int32_t dtype, const void* tensors, const void* messages_in,
                     const itn_bp_opts* o, itn_bp_result* res, void* messages_out, double* totals,
                     int32_t* flags) {
  NvtxScope nvtx_("itn_bp_solve");
  if (int r = itn_bp_solve_submit(c, dtype, tensors, messages_in, o, messages_out, (totals || flags) ? 1 : 0))
    return r;
  return itn_bp_solve_wait(c, res, totals, flags);
}

}  // extern "C"

// ---- contract_network -------------------------------------------------------------------------
namespace {

struct NetIn {
  std::vector<std::vector<int64_t>> labels, dims;
  std::map<int64_t, int64_t> dim;
};

int read_network(itn_ctx* c, int32_t n, const int32_t* ranks, const int64_t* labels, const int64_t* dims,
                 NetIn& net) {
  if (n < 1) return fail(c, ITN_ERR_ARG, "contract_network needs at least one tensor");
  if (!ranks || (!labels && n > 0) || !dims) return fail(c, ITN_ERR_ARG, "null label/dim arrays");
  std::map<int64_t, int> count;
  int64_t pos = 0;
  for (int32_t t = 0; t < n; ++t) {
    if (ranks[t] < 0 || ranks[t] > 48) return fail(c, ITN_ERR_ARG, "tensor %d has rank %d (max 48)", t, ranks[t]);
    std::vector<int64_t> l(labels + pos, labels + pos + ranks[t]), d(dims + pos, dims + pos + ranks[t]);
    for (int a = 0; a < ranks[t]; ++a) {
      if (d[a] < 1) return fail(c, ITN_ERR_ARG, "non-positive dimension");
      auto it = net.dim.find(l[a]);
      if (it != net.dim.end() && it->second != d[a])
        return fail(c, ITN_ERR_ARG, "index %lld has dimensions %lld and %lld", (long long)l[a],
                    (long long)it->second, (long long)d[a]);
      net.dim[l[a]] = d[a];
      if (++count[l[a]] > 2) return fail(c, ITN_ERR_UNSUPPORTED, "index %lld appears on more than two tensors", (long long)l[a]);
      for (int b = 0; b < a; ++b)
        if (l[b] == l[a]) return fail(c, ITN_ERR_UNSUPPORTED, "repeated index %lld within one tensor", (long long)l[a]);
    }
    net.labels.push_back(l);
    net.dims.push_back(d);
    pos += ranks[t];
  }
  return ITN_OK;
}

}  // namespace

extern "C" {

// ---- gate application (apply_gate_bp!, src/apply/apply_operators.jl:209-283) ---------------
namespace {
// host array of `dtype` -> FP64 / complex128 copy (complex data keeps (re, im) pairs)
std::vector<double> to_f64(const void* src, int64_t n, int32_t dtype) {
  const bool cx = dtype == ITN_C64 || dtype == ITN_C128;
  std::vector<double> out((size_t)n * (cx ? 2 : 1));
  const size_t m = out.size();
  if (!src) return out;
  if (dtype == ITN_F32 || dtype == ITN_C64) {
    const float* f = static_cast<const float*>(src);
    for (size_t k = 0; k < m; ++k) out[k] = f[k];
  } else {
    memcpy(out.data(), src, m * sizeof(double));
  }
  return out;
}
void from_f64(const std::vector<double>& v, void* dst, int32_t dtype) {
  if (dtype == ITN_F32 || dtype == ITN_C64) {
    float* f = static_cast<float*>(dst);
    for (size_t k = 0; k < v.size(); ++k) f[k] = (float)v[k];
  } else {
    memcpy(dst, v.data(), v.size() * sizeof(double));
  }
}
}  // namespace

int32_t itn_apply_gates(itn_ctx* c, int32_t dtype, int64_t n_gates, const itn_gate_desc* gates, const void* sites,
                        int64_t n_site_elems, const void* envs, int64_t n_env_elems, const void* ops,
                        int64_t n_op_elems, int32_t max_rank, double cutoff, int32_t normalize, void* out_sites,
                        int64_t out_capacity, double* out_s, int64_t s_capacity, int32_t* out_bond,
                        double* device_ms) {
  NvtxScope nvtx_("itn_apply_gates");
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (dtype < ITN_F32 || dtype > ITN_C128) return fail(c, ITN_ERR_ARG, "unknown dtype %d", dtype);
  if (n_gates < 0) return fail(c, ITN_ERR_ARG, "negative gate count");
  if (n_gates == 0) {
    if (device_ms) *device_ms = 0;
    return ITN_OK;
  }
  if (!gates || !sites || !ops || !out_sites || !out_bond) return fail(c, ITN_ERR_ARG, "null pointer");
  if (n_gates > (1 << 20)) return fail(c, ITN_ERR_ARG, "too many gates in one batch");
  std::vector<GateJob> jobs((size_t)n_gates);
  int64_t ws_total = 0;
  for (int64_t g = 0; g < n_gates; ++g) {
    const itn_gate_desc& G = gates[g];
    GateJob& J = jobs[(size_t)g];
    memset(&J, 0, sizeof(J));
    if (G.nsite != 1 && G.nsite != 2) return fail(c, ITN_ERR_ARG, "gate %lld: nsite must be 1 or 2", (long long)g);
    J.nsite = G.nsite;
    J.bond = G.nsite == 2 ? G.bond : 1;
    if (J.bond < 1 || J.bond > 128) return fail(c, ITN_ERR_ARG, "gate %lld: bond dimension %d", (long long)g, G.bond);
    int64_t P[2] = {1, 1};
    for (int i = 0; i < G.nsite; ++i) {
      if (G.d[i] < 1 || G.d[i] > 16) return fail(c, ITN_ERR_UNSUPPORTED, "gate %lld: site dimension %d (max 16)", (long long)g, G.d[i]);
      if (G.nleg[i] < 0 || G.nleg[i] > kGateMaxLegs)
        return fail(c, ITN_ERR_UNSUPPORTED, "gate %lld: %d other legs (max %d)", (long long)g, G.nleg[i], kGateMaxLegs);
      J.d[i] = G.d[i];
      J.nleg[i] = G.nleg[i];
      for (int j = 0; j < G.nleg[i]; ++j) {
        const int D = G.leg_dim[i][j];
        if (D < 1 || D > 64) return fail(c, ITN_ERR_UNSUPPORTED, "gate %lld: leg dimension %d (max 64)", (long long)g, D);
        J.leg_dim[i][j] = D;
        P[i] *= D;
        if (P[i] > (1 << 22)) return fail(c, ITN_ERR_UNSUPPORTED, "gate %lld: site tensor too large", (long long)g);
        J.env_off[i][j] = G.env_off[i][j];
        if (G.env_off[i][j] >= 0) {
          if (!envs || G.env_off[i][j] + (int64_t)D * D > n_env_elems)
            return fail(c, ITN_ERR_ARG, "gate %lld: environment %d of site %d out of range", (long long)g, j, i);
        }
      }
      const int64_t size = P[i] * G.d[i] * J.bond;
      if (G.site_off[i] < 0 || G.site_off[i] + size > n_site_elems)
        return fail(c, ITN_ERR_ARG, "gate %lld: site %d out of range", (long long)g, i);
      J.site_off[i] = G.site_off[i];
    }
    int64_t opn = G.nsite == 2 ? (int64_t)G.d[0] * G.d[1] * G.d[0] * G.d[1] : (int64_t)G.d[0] * G.d[0];
    if (G.op_off < 0 || G.op_off + opn > n_op_elems) return fail(c, ITN_ERR_ARG, "gate %lld: operator out of range", (long long)g);
    J.op_off = G.op_off;
    if (G.nsite == 2) {
      const int64_t n0 = (int64_t)G.d[0] * J.bond, n1 = (int64_t)G.d[1] * J.bond;
      const int64_t mcap = G.d[0] * std::min(P[0], n0), ncap = G.d[1] * std::min(P[1], n1);
      if (n0 > 128 || n1 > 128 || mcap > 128 || ncap > 128)
        return fail(c, ITN_ERR_UNSUPPORTED, "gate %lld: d * bond and d * d * bond must be <= 128", (long long)g);
      J.chi_cap = (int)std::min(mcap, ncap);
      if (!out_s || G.s_off < 0 || G.s_off + J.chi_cap > s_capacity)
        return fail(c, ITN_ERR_ARG, "gate %lld: singular values out of range", (long long)g);
      J.s_off = G.s_off;
    } else {
      J.chi_cap = 1;
    }
    for (int i = 0; i < G.nsite; ++i) {
      const int64_t need = P[i] * G.d[i] * (G.nsite == 2 ? J.chi_cap : 1);
      if (G.out_off[i] < 0 || G.out_off[i] + need > out_capacity)
        return fail(c, ITN_ERR_ARG, "gate %lld: output site %d out of range", (long long)g, i);
      J.out_off[i] = G.out_off[i];
    }
    J.ws = ws_total;
    ws_total += gate_workspace(J);
  }
  if (int r = ensure_device(c)) return r;
  const bool cx = dtype == ITN_C64 || dtype == ITN_C128;
  const size_t esz = cx ? 16 : 8;
  std::vector<double> h_sites = to_f64(sites, n_site_elems, dtype);
  std::vector<double> h_envs = to_f64(envs, envs ? n_env_elems : 0, dtype);
  std::vector<double> h_ops = to_f64(ops, n_op_elems, dtype);
  struct Buf {
    void* p = nullptr;
    cudaStream_t st;
    ~Buf() { if (p) cudaFreeAsync(p, st); }
  } b_jobs, b_sites, b_envs, b_ops, b_out, b_s, b_bond, b_ws;
  Buf* all[] = {&b_jobs, &b_sites, &b_envs, &b_ops, &b_out, &b_s, &b_bond, &b_ws};
  const size_t sizes[] = {jobs.size() * sizeof(GateJob), h_sites.size() * 8, std::max<size_t>(h_envs.size() * 8, 16),
                          h_ops.size() * 8, (size_t)out_capacity * esz, (size_t)std::max<int64_t>(s_capacity, 1) * 8,
                          jobs.size() * sizeof(int), (size_t)ws_total * esz};
  for (int k = 0; k < 8; ++k) {
    all[k]->st = c->stream;
    cudaError_t e = cudaMallocAsync(&all[k]->p, std::max<size_t>(sizes[k], 16), c->stream);
    if (e != cudaSuccess) {
      all[k]->p = nullptr;
      return e == cudaErrorMemoryAllocation ? fail(c, ITN_ERR_OOM, "apply_gates: %zu bytes", sizes[k])
                                            : cuda_fail(c, e, "apply_gates allocation");
    }
  }
  CK(cudaMemcpyAsync(b_jobs.p, jobs.data(), sizes[0], cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(b_sites.p, h_sites.data(), sizes[1], cudaMemcpyHostToDevice, c->stream));
  if (!h_envs.empty()) CK(cudaMemcpyAsync(b_envs.p, h_envs.data(), h_envs.size() * 8, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(b_ops.p, h_ops.data(), sizes[3], cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(b_out.p, 0, sizes[4], c->stream));
  CK(cudaEventRecord(c->ev0, c->stream));
  CK(launch_gates(cx, (int)n_gates, static_cast<const GateJob*>(b_jobs.p), b_sites.p, b_envs.p, b_ops.p, b_out.p,
                  static_cast<double*>(b_s.p), static_cast<int*>(b_bond.p), b_ws.p, max_rank, cutoff, normalize,
                  c->stream));
  CK(cudaEventRecord(c->ev1, c->stream));
  std::vector<double> h_out((size_t)out_capacity * (cx ? 2 : 1));
  std::vector<int> h_bond(jobs.size());
  CK(cudaMemcpyAsync(h_out.data(), b_out.p, sizes[4], cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(h_bond.data(), b_bond.p, sizes[6], cudaMemcpyDeviceToHost, c->stream));
  if (out_s && s_capacity > 0)
    CK(cudaMemcpyAsync(out_s, b_s.p, (size_t)s_capacity * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (device_ms) *device_ms = ms;
  from_f64(h_out, out_sites, dtype);
  for (size_t g = 0; g < jobs.size(); ++g) out_bond[g] = h_bond[g];
  return ITN_OK;
}

int32_t itn_contraction_order(int32_t n, const int32_t* ranks, const int64_t* labels, const int64_t* dims,
                              int32_t alg, int32_t* steps_out) {
  if (!steps_out && n > 1) return ITN_ERR_ARG;
  if (alg != 0 && alg != 1 && alg != 3) return ITN_ERR_ARG;
  NetIn net;
  if (int r = read_network(nullptr, n, ranks, labels, dims, net)) return r;
  std::vector<std::pair<int, int>> steps;
  contraction_order(net.labels, net.dim, alg, steps);
  for (size_t k = 0; k < steps.size(); ++k) {
    steps_out[2 * k] = steps[k].first;
    steps_out[2 * k + 1] = steps[k].second;
  }
  return ITN_OK;
}

int32_t itn_contract_network(itn_ctx* c, int32_t dtype, int32_t n, const int32_t* ranks, const int64_t* labels,
                             const int64_t* dims, const void* const* tensors, int32_t alg, const int32_t* steps_in,
                             int32_t precision, void* out, int64_t out_capacity, int32_t* out_rank,
                             int64_t* out_labels, int64_t* out_dims, double* device_ms) {
  NvtxScope nvtx_("itn_contract_network");
  if (int r_ = not_busy(c)) return r_;
  if (!c) return ITN_ERR_ARG;
  if (dtype < ITN_F32 || dtype > ITN_C128) return fail(c, ITN_ERR_ARG, "unknown dtype %d", dtype);
  if (precision != ITN_PREC_NATIVE &&
      !((precision == ITN_PREC_BF16 || precision == ITN_PREC_TF32X3) && dtype == ITN_F32))
    return fail(c, ITN_ERR_UNSUPPORTED,
                "contract_network precision %d needs float32 data (BF16 split or TF32 split)", precision);
  if (!tensors || !out_rank) return fail(c, ITN_ERR_ARG, "null pointer");
  if (alg < 0 || alg > 3) return fail(c, ITN_ERR_ARG, "unknown order algorithm %d", alg);
  if (int r = ensure_device(c)) return r;
  NetIn net;
  if (int r = read_network(c, n, ranks, labels, dims, net)) return r;
  std::vector<std::pair<int, int>> steps;
  if (alg == 2) {
    if (!steps_in && n > 1) return fail(c, ITN_ERR_ARG, "explicit order needs steps");
    int live = n;
    for (int k = 0; k + 1 < n; ++k) {
      const int i = steps_in[2 * k], j = steps_in[2 * k + 1];
      if (i < 0 || j < 0 || i >= live || j >= live || i == j) return fail(c, ITN_ERR_ARG, "bad contraction step %d", k);
      steps.push_back({i, j});
      --live;
    }
  } else {
    contraction_order(net.labels, net.dim, alg, steps);
  }
  const size_t es = dtype_size(dtype);
  struct Item {
    void* p;
    std::vector<int64_t> l, d;
  };
  std::vector<Item> W;
  auto numel = [](const std::vector<int64_t>& d) {
    int64_t x = 1;
    for (int64_t v : d) x *= v;
    return x;
  };
  auto release_all = [&]() {
    for (auto& it : W)
      if (it.p) cudaFreeAsync(it.p, c->stream);
    W.clear();
  };
  for (int t = 0; t < n; ++t) {
    Item it{nullptr, net.labels[t], net.dims[t]};
    const size_t bytes = (size_t)numel(it.d) * es;
    if (!tensors[t]) {
      release_all();
      return fail(c, ITN_ERR_ARG, "null tensor %d", t);
    }
    cudaError_t e = cudaMallocAsync(&it.p, std::max<size_t>(bytes, 16), c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(it.p, tensors[t], bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
      W.push_back(it);
      release_all();
      return cuda_fail(c, e, "contract_network upload");
    }
    W.push_back(it);
  }
  CK(cudaEventRecord(c->ev0, c->stream));
  for (auto& st : steps) {
    Item& A = W[st.first];
    Item& B = W[st.second];
    std::vector<int64_t> shared, fa, fb, dfa, dfb, dsh;
    std::vector<int> pa, pb;
    for (size_t a = 0; a < A.l.size(); ++a) {
      if (std::find(B.l.begin(), B.l.end(), A.l[a]) == B.l.end()) {
        fa.push_back(A.l[a]);
        dfa.push_back(A.d[a]);
        pa.push_back((int)a);
      }
    }
    // the shared indices in the larger operand's order, so that only the smaller operand's
    // permute reorders them (the larger one's keeps its shared axes in place, which is the
    // identity -- no copy -- when they lead it; in a boundary sweep the larger is the
    // running product)
    const bool b_leads = numel(B.d) > numel(A.d);
    const Item& O = b_leads ? B : A;
    const Item& P = b_leads ? A : B;
    for (size_t q = 0; q < O.l.size(); ++q)
      if (std::find(P.l.begin(), P.l.end(), O.l[q]) != P.l.end()) {
        shared.push_back(O.l[q]);
        dsh.push_back(O.d[q]);
      }
    for (int64_t x : shared) {
      pa.push_back((int)(std::find(A.l.begin(), A.l.end(), x) - A.l.begin()));
      pb.push_back((int)(std::find(B.l.begin(), B.l.end(), x) - B.l.begin()));
    }
    for (size_t b = 0; b < B.l.size(); ++b)
      if (std::find(shared.begin(), shared.end(), B.l[b]) == shared.end()) {
        fb.push_back(B.l[b]);
        dfb.push_back(B.d[b]);
        pb.push_back((int)b);
      }
    const long long M = numel(dfa), K = numel(dsh), N = numel(dfb);
    auto is_id = [](const std::vector<int>& p) {
      for (size_t k = 0; k < p.size(); ++k)
        if (p[k] != (int)k) return false;
      return true;
    };
    void *ta = A.p, *tb = B.p, *tc = nullptr;
    cudaError_t e = cudaSuccess;
    // a thin step whose long operand is not in GEMM order reads that operand in place through a
    // view (its free axes and contracted positions with their strides) instead of permuting it
    const bool thin = precision == ITN_PREC_NATIVE && contract_thin_shape(M, N, K);
    const bool small_b = thin && contract_thin_small_b(M, N);
    // (int dims in the view: tensors below 2^31 entries)
    const bool view = thin && !is_id(small_b ? pa : pb) && numel((small_b ? A : B).d) < (1LL << 31);
    ThinView tv;
    if (view) {
      const Item& Lg = small_b ? A : B;
      std::vector<long long> lstr(Lg.d.size(), 1);
      for (int q = (int)Lg.d.size() - 2; q >= 0; --q) lstr[q] = lstr[q + 1] * Lg.d[q + 1];
      std::vector<char> is_sh(Lg.l.size(), 0);
      std::vector<int> spos;
      for (int64_t x : shared) {
        const int q = (int)(std::find(Lg.l.begin(), Lg.l.end(), x) - Lg.l.begin());
        spos.push_back(q);
        is_sh[q] = 1;
      }
      // contracted positions k, row-major over `shared`
      for (int k = 0; k < (int)K; ++k) {
        long long rem = k, off = 0;
        for (int a = (int)spos.size() - 1; a >= 0; --a) {
          const long long d = Lg.d[spos[a]];
          off += (rem % d) * lstr[spos[a]];
          rem /= d;
        }
        tv.koff[k] = off;
      }
      // free axes in the operand's order, runs of adjacent free axes merged
      tv.rank = 0;
      for (int q = 0; q < (int)Lg.l.size(); ++q) {
        if (is_sh[q] || Lg.d[q] == 1) continue;
        const bool merge = tv.rank > 0 && q > 0 && !is_sh[q - 1] && tv.stride[tv.rank - 1] == lstr[q] * Lg.d[q];
        if (merge) {
          tv.dims[tv.rank - 1] = (int)(tv.dims[tv.rank - 1] * Lg.d[q]);
          tv.stride[tv.rank - 1] = lstr[q];
        } else {
          tv.dims[tv.rank] = (int)Lg.d[q];
          tv.stride[tv.rank] = lstr[q];
          ++tv.rank;
        }
      }
      if (tv.rank == 0) {
        tv.dims[0] = 1;
        tv.stride[0] = 1;
        tv.rank = 1;
      }
    }
    if (!is_id(pa) && !(view && small_b)) {
      e = cudaMallocAsync(&ta, std::max<size_t>((size_t)M * K * es, 16), c->stream);
      if (e == cudaSuccess) e = contract_permute(dtype, A.p, ta, A.d, pa, c->stream);
    }
    if (e == cudaSuccess && !is_id(pb) && !(view && !small_b)) {
      e = cudaMallocAsync(&tb, std::max<size_t>((size_t)K * N * es, 16), c->stream);
      if (e == cudaSuccess) e = contract_permute(dtype, B.p, tb, B.d, pb, c->stream);
    }
    if (e == cudaSuccess) e = cudaMallocAsync(&tc, std::max<size_t>((size_t)M * N * es, 16), c->stream);
    if (e == cudaSuccess) {
      if (precision == ITN_PREC_BF16 || precision == ITN_PREC_TF32X3)
        e = contract_gemm_tc(reinterpret_cast<const float*>(ta), reinterpret_cast<const float*>(tb),
                             reinterpret_cast<float*>(tc), M, N, K, c->stream, precision == ITN_PREC_TF32X3);
      else if (view)
        e = contract_gemm_view(dtype, ta, tb, tc, M, N, K, small_b, tv, c->stream);
      else
        e = contract_gemm(dtype, ta, tb, tc, M, N, K, c->stream);
    }
    if (ta != A.p && ta) cudaFreeAsync(ta, c->stream);
    if (tb != B.p && tb) cudaFreeAsync(tb, c->stream);
    if (e != cudaSuccess) {
      if (tc) cudaFreeAsync(tc, c->stream);
      release_all();
      return cuda_fail(c, e, "contract_network step");
    }
    Item R{tc, fa, dfa};
    R.l.insert(R.l.end(), fb.begin(), fb.end());
    R.d.insert(R.d.end(), dfb.begin(), dfb.end());
    cudaFreeAsync(A.p, c->stream);
    cudaFreeAsync(B.p, c->stream);
    const int i = st.first, j = st.second;
    std::vector<Item> nw;
    for (int k = 0; k < (int)W.size(); ++k)
      if (k != i && k != j) nw.push_back(W[k]);
    nw.push_back(R);
    W.swap(nw);
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  Item& F = W[0];
  const int64_t total = numel(F.d);
  *out_rank = (int32_t)F.l.size();
  for (size_t a = 0; a < F.l.size() && a < 48; ++a) {
    if (out_labels) out_labels[a] = F.l[a];
    if (out_dims) out_dims[a] = F.d[a];
  }
  int rc = ITN_OK;
  if (out && out_capacity >= total) {
    cudaError_t e = cudaMemcpyAsync(out, F.p, (size_t)total * es, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "contract_network download");
  } else {
    rc = fail(c, ITN_ERR_ARG, "output capacity %lld < result size %lld", (long long)out_capacity, (long long)total);
  }
  release_all();
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "contract_network");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  if (device_ms) *device_ms = ms;
  return rc;
}

}  // extern "C"
