// itn_internal.h -- declarations shared between the C-ABI layer (itn_api.cu) and the
// kernel translation units.  Not part of the public interface (that is include/itn_gpu.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "itn_conv.cuh"

namespace itn {

enum Dtype { DT_F32 = 0, DT_F64 = 1, DT_C64 = 2, DT_C128 = 3 };
inline size_t dtype_size(int dt) {
  switch (dt) {
    case DT_F32: return 4;
    case DT_F64: return 8;
    case DT_C64: return 8;
    case DT_C128: return 16;
  }
  return 0;
}

// Op-program opcodes for the two-layer vertex interpreter (bp_generic.cu).
enum OpCode { OP_ABSORB = 0, OP_FINAL = 1, OP_FULL = 2, OP_DUMP = 3 };
inline uint32_t make_op(int type, int src, int dst, int leg) {
  return ((uint32_t)type << 28) | ((uint32_t)src << 20) | ((uint32_t)dst << 12) | (uint32_t)leg;
}
constexpr int kMaxLegs = 16;
constexpr int kMaxBufs = 8;

// Arguments of one generic launch (one dtype, one list of work items).
struct GenericArgs {
  int layers;
  const int* off;          // nv + 1
  const int* rev;          // nslots
  const int* bond;         // nslots
  const int* phys;         // nv
  const long long* toff;   // nv + 1
  const long long* moff;   // nslots + 1
  const void* tens;
  const void* msg_in;
  void* msg_out;
  const int* items;        // n_items x (vertex, program offset or leg mask)
  int n_items;
  const unsigned* prog;    // programs: [n_ops, op...]
  int nbuf;                // buffers per CTA including the copy of the site tensor
  long long buf_elems;     // elements per buffer
  void* gscratch;          // non-null: buffers live in global memory (gridDim.x slots)
  int msg_cap;             // elements of incoming-message staging in shared memory
  int max_d2;              // max D*D (two-layer) or D (one-layer) over slots
  int normalize;
  void* zv_out;            // OP_FULL writes one scalar per vertex here
  double* slot_diff;       // per-slot 1 - |<m_new, m_old>|^2 (nullable)
  ConvState* conv;         // outer-loop state: early exit when done and the diff max
                           // (nullable: neither)
  int fused_step;          // non-zero: the last CTA performs the outer-loop step
  // Persistent sweeps of the two-layer interpreter (pgrid != null; one work item per CTA,
  // every CTA resident): the launch runs up to `nsweeps` parallel sweeps, sweep s reading
  // msg_buf[s & 1] and writing msg_buf[(s + 1) & 1], with the site tensor staged once, a grid
  // barrier and the outer-loop step (on every CTA, from the sweep's diff maximum) between sweeps.
  struct SweepGrid* pgrid;
  void* msg_buf[2];
  int nsweeps;
  unsigned long long wait_ns;  // limit of one grid-barrier wait (the run stops with pgrid->err)
  int pstall;                  // fault injection: CTA 0 never arrives at the first barrier
};

// Grid barrier and per-sweep diff maxima of the persistent sweeps (three rotating slots:
// slot s % 3 is filled in sweep s, read by every CTA after the barrier that ends it, and reset
// by CTA 0 for sweep s + 2).  Initialised on the stream before each launch.
struct SweepGrid {
  unsigned long long arrivals;  // grid-barrier arrivals of the launch
  unsigned long long dmax[3];
  int nanf[3];
  int err;
};

// Extra arguments of the dual-number (forward-mode) interpreter used by the gradient.
struct AdjState;
struct AdjGrid;
struct SweepGrid;

struct DualArgs {
  const void* tan_in;  // tangent per outgoing slot (mu_{u->v}); null = zero tangents
  void* tan_out;       // FINAL: tangent of the message on leg w, stored at slot rev(u->w)
  int transpose;       // stage m^T and mu^T (second orientation of the real gradient)
  void* grad_out;      // DUMP target (packed canonical tensors)
  const void* zv;      // per-vertex Z_u (DUMP of the value plane scales by 1/Z_u)
  int dump_tangent;    // DUMP: 0 the value plane / Z_u, 1 the tangent plane (unscaled), 2 both summed
  const int* done;     // adjoint loop: skip the launch once the iteration has stopped (may be null)
  // Adjoint loop with the update fused into the launch (adj != null): the FINAL of slot t
  // applies lambda_t <- g_t + (J^T mu)_t in place, writes the next iteration's
  // mu_t = (lambda_t - <lambda_t, F_t>) / S_t (lambda_t when not normalising) to mu_next
  // (not tan_in: other CTAs still read it) instead of storing the product to tan_out, and
  // folds max |lambda_new - lambda| and max |lambda_new| into *adj, whose stopping rule the
  // last CTA to finish runs.
  AdjState* adj;
  const void* g;
  void* lam;
  const void* F;
  const void* S;
  void* mu_next;
  int normalize;
  // Persistent adjoint loop (grid != null; one work item per CTA, every CTA resident): the
  // launch runs iteration after iteration of the fused update, mu alternating between mu_buf[0]
  // (read first) and mu_buf[1], with a grid barrier and the stopping rule between iterations;
  // the site tensor and the value messages are staged once.
  struct AdjGrid* grid;
  void* mu_buf[2];
  unsigned long long wait_ns;  // limit of one grid-barrier wait (the loop stops with grid->err)
  int stall;                   // fault injection: CTA 0 never arrives at the first barrier
};

// Device state of the persistent adjoint loop (zeroed before each launch): the grid barrier's
// arrival count and the maxima of the iterations in three rotating slots (slot
// k % 3 is filled in iteration k, read by every CTA after the barrier that ends it, and
// cleared by CTA 0 for iteration k + 2 -- by then every CTA has read it).
struct AdjGrid {
  unsigned long long arrivals;  // grid-barrier arrivals of the launch
  unsigned long long dmax[3], lmax[3];
  int err;  // a grid-barrier wait ran out
  int pad_;
};

// Device-side state of the adjoint fixed-point iteration lambda <- g + J^T lambda: the dual
// launch with the fused update (DualArgs::adj) folds max|lambda_new - lambda| and
// max|lambda_new| into dmax / lmax (order-encoded) and its last CTA turns them into the
// relative change and stops the loop; launches after the stop return at once.
struct AdjState {
  unsigned long long dmax, lmax;
  int done;       // stopped (converged, NaN or maxiter)
  int iters;      // iterations executed
  int nan;        // the relative change was NaN
  int maxiter;
  double tol;
  double resid;   // last relative change
  unsigned ticket;  // CTAs of the fused-update launch finished in this iteration
};

struct LaunchCfg {
  int grid;
  int block;
  size_t smem;
};

// bp_generic.cu
size_t generic_smem_bytes(int dtype, const GenericArgs& a, int block, bool buffers_in_smem);
cudaError_t launch_generic(int dtype, const GenericArgs& a, const LaunchCfg& cfg, cudaStream_t st);
// Up to a.nsweeps sweeps of a two-layer network as one cooperative launch (a.pgrid set,
// cfg.grid == a.n_items CTAs, all resident); initialises a.pgrid on the stream first.
cudaError_t launch_generic_persistent(int dtype, const GenericArgs& a, const LaunchCfg& cfg, cudaStream_t st);
int generic_max_active(int dtype, int layers, int block, size_t smem);

cudaError_t launch_edge_scalars(int dtype, int layers, const long long* moff, const int* rev,
                                const int* eslots, int n_e, const void* msgs, void* ze_out,
                                cudaStream_t st);
// Vertex scalars (float or complex64) when every vertex of a two-layer network has d = 2
// and four legs of dimension 8 (vertex u's legs are slots 4u..4u+3, its tensor 8192 entries
// at toff[u]).
cudaError_t launch_vertex_scalars_d8(int dtype, int nv, const int* rev, const long long* moff,
                                     const long long* toff, const void* tens, const void* msgs, void* zv,
                                     cudaStream_t st);
// One FP32 parallel sweep of a two-layer network whose vertices all have d = 2 and four legs
// of dimension 8 (vertex u's legs are slots 4u..4u+3, its tensor 8192 entries at 8192 u,
// slot s's message 64 entries at 64 s), CUDA cores; slot_diff / conv as in GenericArgs
// (the sweep also steps the outer loop when conv is given).
cudaError_t launch_sweep_d8(const int* rev, const float* tens, const float* msg_in, float* msg_out, int nv,
                            int normalize, double* slot_diff, ConvState* conv, cudaStream_t st);
cudaError_t launch_logsum(int dtype, const void* zv, const void* ze, int nv, int ne,
                          const int* net_voff, const int* net_vlist, const int* net_eoff,
                          const int* net_elist, int n_nets, double* logzv, double* logze,
                          double* totals, int* flags, void* scratch, size_t scratch_bytes,
                          cudaStream_t st);
cudaError_t launch_init_messages(int dtype, int layers, int kind, const long long* moff,
                                 const int* bond, int nslots, void* msgs, cudaStream_t st);
cudaError_t launch_iterate_diff(int dtype, const long long* moff, int nslots, const void* m1,
                                const void* m2, double* slot_diff, ConvState* conv, cudaStream_t st);
cudaError_t launch_permute(int dtype, int nv, const long long* soff, const long long* toff,
                           const int* rank_off, const int* dims, const long long* sstride,
                           const void* src, void* dst, cudaStream_t st);
cudaError_t launch_dual(int dtype, const GenericArgs& a, const DualArgs& d, const LaunchCfg& cfg,
                        cudaStream_t st);
int dual_max_active(int dtype, int block, size_t smem);
// The whole adjoint loop as one cooperative launch (d.grid set, cfg.grid == n_items CTAs all
// resident); cudaErrorCooperativeLaunchTooLarge when they do not fit.
cudaError_t launch_dual_persistent(int dtype, const GenericArgs& a, const DualArgs& d, const LaunchCfg& cfg,
                                   cudaStream_t st);
cudaError_t launch_grad_prep(int dtype, const long long* moff, int nslots, const void* U, void* F, void* S,
                             int normalize, cudaStream_t st);
cudaError_t launch_grad_g(int dtype, const long long* moff, const int* rev, const int* dst_vertex,
                          const int* eidx, int nslots, const void* U, const void* m, const void* zv,
                          const void* ze, void* g, cudaStream_t st);
cudaError_t launch_grad_mu(int dtype, const long long* moff, int nslots, const void* lam, const void* F,
                           const void* S, void* mu, int normalize, const int* done, cudaStream_t st);
cudaError_t launch_adj_reset(AdjState* adj, double tol, int maxiter, cudaStream_t st);
cudaError_t launch_adj_step(AdjState* adj, cudaStream_t st);
// lambda <- g + cot, then mu <- (lambda - <lambda, F>) / S (normalised) or lambda, and the
// stopping rule, in one launch (the step runs in the last block to finish).
cudaError_t launch_reset_state(ConvState* s, double tol, int use_tol, cudaStream_t st);
cudaError_t launch_step_check(ConvState* s, cudaStream_t st);

}  // namespace itn
