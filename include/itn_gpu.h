/*
 * itn_gpu.h -- C ABI of libitn_gpu.so, the GB300 (sm_103a) belief-propagation and
 * network-contraction engine behind ITensorNetworksNext.jl's hot path.
 *
 * Every entry point takes plain pointers and sizes, returns an int32 status
 * (ITN_OK = 0) and never aborts; on failure itn_last_error(ctx) holds a message.
 * A context owns one CUDA stream and all device buffers it allocates; calls are
 * synchronous at return.  A context is not thread-safe; separate contexts may be
 * used from separate threads.
 *
 * Data model (shared by every call).  A network of nv vertices is a CSR adjacency:
 *   vertex u owns leg slots csr_off[u] .. csr_off[u+1]-1; slot s is the directed edge
 *   u -> csr_nbr[s] with bond dimension bond[s]; rev[s] is the slot of the opposite
 *   direction.  All link indices shared by one pair of vertices form one leg (their
 *   dimensions multiply), exactly as linknames() intersects dim names in the reference
 *   (src/abstracttensornetwork.jl:52-73).
 *   Site tensor of u: row-major [phys][leg_0]...[leg_{z-1}] ("canonical" layout), the
 *   tensors of all vertices packed back to back in vertex order.
 *   Message on slot s: layers == 2 (norm network <psi|psi>): D x D row-major
 *   m[bra][ket] (message_environment, src/beliefpropagation/messagecache.jl:205-229);
 *   layers == 1 (plain network): a length-D vector.  Packed in slot order.
 *
 * Paths below are relative to the ITensorNetworksNext.jl source tree.
 */
#ifndef ITN_GPU_H
#define ITN_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ITN_ABI_VERSION 2

enum {
  ITN_OK = 0,
  ITN_ERR_ARG = 1,         /* bad argument: maps to ArgumentError in the Julia shim */
  ITN_ERR_CUDA = 2,        /* CUDA runtime failure */
  ITN_ERR_OOM = 3,         /* device allocation failed */
  ITN_ERR_NAN = 4,         /* NaN/Inf met where a finite value is required */
  ITN_ERR_TIMEOUT = 5,     /* iteration cap reached without meeting the tolerance */
  ITN_ERR_UNSUPPORTED = 6, /* shape / dtype / precision combination not implemented */
  ITN_ERR_STATE = 7        /* call order violated (e.g. run before upload) */
};

enum { ITN_F32 = 0, ITN_F64 = 1, ITN_C64 = 2, ITN_C128 = 3 };
enum { ITN_SCHED_PARALLEL = 0, ITN_SCHED_SEQUENTIAL = 1 };
/* ITN_PREC_NATIVE: arithmetic in the stored dtype on CUDA cores.
 * ITN_PREC_BF16 / ITN_PREC_TF32: tensor-core (tcgen05) contractions with FP32
 * accumulation for all but the last split_sweeps sweeps, which run in split
 * (hi/lo) precision; requires ITN_F32 storage.
 * ITN_PREC_TF32X3: every sweep on the tensor cores with TF32 hi/lo operands (three TF32
 * products per contraction, about FP32 accuracy); split_sweeps is ignored; ITN_F32 storage.
 * The tensor-core modes take norm networks (layers = 2) whose vertices have at most 4 legs,
 * bonds of at most 8 and a physical dimension of at most 2; anything smaller than 4 legs of
 * 8 with d = 2 is zero-padded to that frame (exact: padded products are zero) and swept with
 * one launch per sweep; other networks give ITN_ERR_UNSUPPORTED. */
enum { ITN_PREC_NATIVE = 0, ITN_PREC_BF16 = 1, ITN_PREC_TF32 = 2, ITN_PREC_TF32X3 = 3 };
enum { ITN_MSG_IDENTITY_NORMALIZED = 0, ITN_MSG_IDENTITY = 1, ITN_MSG_ONES = 2 };

typedef struct itn_ctx itn_ctx;

typedef struct {
  int32_t schedule;      /* ITN_SCHED_* */
  int32_t maxiter;       /* StopAfterIteration(maxiter); < 0 = not given */
  double tol;            /* StopWhenConverged(tol); < 0 = not given */
  int32_t normalize;     /* SimpleMessageUpdate(normalize) */
  int32_t precision;     /* ITN_PREC_* */
  int32_t split_sweeps;  /* final sweeps in split precision (tensor-core modes) */
  int32_t reserved0;
  const int64_t *edges;  /* sequential schedule: directed slots, in sweep order */
  int64_t n_edges;
} itn_bp_opts;

typedef struct {
  int32_t iterations;    /* outer iterations (sweeps) performed */
  int32_t at_iteration;  /* StopWhenConvergedState.at_iteration (-1 if not converged) */
  double delta;          /* last iterate_diff value (Inf if never computed) */
  double device_ms;      /* device time of the sweeps (CUDA events on the ctx stream) */
  int32_t kernel_launches; /* kernels launched by this call */
  int32_t reserved0;
} itn_bp_result;

/* Library/ABI identification. */
int32_t itn_abi_version(void);
const char *itn_status_string(int32_t status);

/* Context life cycle.  Replaces nothing in the reference (it has no device state);
 * the Julia shim creates one per GPU strategy object. */
int32_t itn_create(itn_ctx **out, int32_t device, int32_t flags);
int32_t itn_destroy(itn_ctx *ctx);
const char *itn_last_error(const itn_ctx *ctx);
int32_t itn_synchronize(itn_ctx *ctx);

/* Network structure.  Replaces the graph bookkeeping the reference derives from
 * shared dim names: ITensorNetwork / set!_tensornetwork (src/tensornetwork.jl:21-48,
 * 138-173), linkinds/siteinds (src/abstracttensornetwork.jl:52-95) and the directed
 * edge set of MessageCache (src/beliefpropagation/messagecache.jl:15-49).
 * rev may be NULL (computed by pairing the k-th u->w slot with the k-th w->u slot);
 * phys may be NULL (all 1); net_id (network of each vertex, for batches of
 * independent networks) may be NULL (one network).  layers: 1 = plain network
 * (factors are the tensors), 2 = norm network (factor = A * conj(A) with the site
 * index shared, src/normnetwork.jl:49-54). */
int32_t itn_graph_upload(itn_ctx *ctx, int64_t nv, const int64_t *csr_off,
                         const int64_t *csr_nbr, const int32_t *bond, const int64_t *rev,
                         const int32_t *phys, int32_t layers, const int32_t *net_id);
/* Sizes of the uploaded network. */
int32_t itn_graph_info(const itn_ctx *ctx, int64_t *nv, int64_t *nslots, int64_t *tensor_elems,
                       int64_t *message_elems, int32_t *n_nets, int64_t *n_undirected);

/* Site tensors, canonical packed layout.  Replaces the per-vertex ket tensors of
 * NormNetwork.ket / ITensorNetwork.tensors (src/normnetwork.jl:13-25). */
int32_t itn_tensors_upload(itn_ctx *ctx, int32_t dtype, const void *packed);
/* Site tensors in any strided layout (e.g. Julia column-major arrays with the
 * ITensor's own index order): site_ptrs[u] points at vertex u's array and
 * strides[(off)] lists, for vertex u, 1 + degree(u) element strides in canonical axis
 * order (phys, leg_0, ...); a vertex without a site index uses stride 0 with phys 1.
 * Strides of vertex u start at csr_off[u] + u.  Permuted on the device. */
int32_t itn_tensors_upload_strided(itn_ctx *ctx, int32_t dtype, const void *const *site_ptrs,
                                   const int64_t *strides);
/* Site tensors back in canonical packed layout. */
int32_t itn_tensors_download(itn_ctx *ctx, int32_t dtype, void *packed);

/* Messages (MessageCache contents, src/beliefpropagation/messagecache.jl:15-49). */
int32_t itn_messages_upload(itn_ctx *ctx, int32_t dtype, const void *packed);
int32_t itn_messages_download(itn_ctx *ctx, int32_t dtype, void *packed);
/* message_environment(f, nn) for f = one / ones, device side
 * (src/beliefpropagation/messagecache.jl:205-229); kind = ITN_MSG_*. */
int32_t itn_messages_init(itn_ctx *ctx, int32_t kind);

/* beliefpropagation(factors, messages; edges, stopping_criterion,
 * message_update_algorithm) (src/beliefpropagation/beliefpropagation.jl:69-92):
 * runs the whole solve on the device on the uploaded messages, in place. */
int32_t itn_bp_run(itn_ctx *ctx, const itn_bp_opts *opts, itn_bp_result *result);

/* One end-to-end call: beliefpropagation(factors, messages; ...) followed by
 * bethe_free_energy(factors, messages) (beliefpropagation.jl:69-92, messagecache.jl:185-201)
 * on host inputs.  Uploads the packed site tensors and initial messages (layouts of
 * itn_tensors_upload / itn_messages_upload, one dtype for both), runs the solve of
 * itn_bp_run with `opts`, computes the log-norm totals and flags of itn_logscalars and
 * downloads the final messages -- all queued on the context's stream with a single host
 * synchronisation at the end (one more per convergence check when opts has a tolerance).
 * messages_out, totals and flags may each be NULL.  Pinned host buffers make the copies
 * asynchronous.  The context keeps the uploaded data, as after the separate calls. */
int32_t itn_bp_solve(itn_ctx *ctx, int32_t dtype, const void *tensors, const void *messages_in,
                     const itn_bp_opts *opts, itn_bp_result *result, void *messages_out,
                     double *totals, int32_t *flags);

/* itn_bp_solve in two halves, for callers that solve many networks back to back (a serving
 * loop): itn_bp_solve_submit queues the uploads, the solve, the log-norm (when `logz` is
 * non-zero) and the download of the final messages into messages_out, and returns without
 * waiting (a solve with a tolerance still waits for its convergence checks);
 * itn_bp_solve_wait waits for that work and returns the result, totals and flags as
 * itn_bp_solve does.  Between the two the host buffers must stay valid and unchanged, and every
 * other call on the context returns ITN_ERR_STATE.  Each context has its own stream, so with two
 * contexts on one device the uploads of one network overlap the solve of the other. */
int32_t itn_bp_solve_submit(itn_ctx *ctx, int32_t dtype, const void *tensors, const void *messages_in,
                            const itn_bp_opts *opts, void *messages_out, int32_t logz);
int32_t itn_bp_solve_wait(itn_ctx *ctx, itn_bp_result *result, double *totals, int32_t *flags);

/* message_update!(SimpleMessageUpdate(normalize), cache, factors, edge)
 * (src/beliefpropagation/beliefpropagation.jl:242-257) for the directed slot. */
int32_t itn_message_update(itn_ctx *ctx, int64_t slot, int32_t normalize);

/* AIE.iterate_diff(cache1, cache2) (src/beliefpropagation/beliefpropagation.jl:261-267)
 * of two packed message sets with this context's layout, FP64 on the device. */
int32_t itn_iterate_diff(itn_ctx *ctx, int32_t dtype, const void *m1, const void *m2,
                         double *out);

/* vertex_scalars / edge_scalars / bethe_free_energy
 * (src/beliefpropagation/messagecache.jl:139-201) on the current messages.
 * zv: nv raw scalars, ze: one per undirected edge (slot < rev[slot], slot order), both
 * in the context dtype (may be NULL).  logzv / logze: (re, im) pairs in FP64 (may be
 * NULL).  totals: (re, im) of sum log Zv - sum log Ze per network.  flags per network:
 * bit0 any Re Zv < 0, bit1 any Re Ze < 0, bit2 any Ze == 0 (bethe_free_energy returns
 * -Inf then).  Every output may be NULL; only the requested ones are copied back. */
int32_t itn_logscalars(itn_ctx *ctx, void *zv, void *ze, double *logzv, double *logze,
                       double *totals, int32_t *flags);

/* contract_network ordering: contraction_order(tn; alg) (src/contract_network.jl:39-58) on
 * host data only (no device work).  Tensor t has ranks[t] indices; labels/dims list them
 * tensor after tensor; an index shared by two tensors is contracted, one on a single tensor
 * stays open.  alg 0 = Greedy (pair with the smallest growth, pairs sharing an index first),
 * 1 = LeftAssociative, 3 = sweep: the cheaper, in multiply-adds, of the Greedy order and the
 * orders in which one running product absorbs, step by step, the tensor that leaves it
 * smallest (started from every tensor, at most 64 starts) -- boundary-sweep orders on
 * lattices (no counterpart in the reference; an EvaluationOrderAlgorithm of this library).
 * steps_out (2 * (n - 1) ints): step k contracts positions
 * (steps_out[2k], steps_out[2k+1]) of a working list from which both are removed and to
 * which the result (labels: free of the first ++ free of the second) is appended. */
int32_t itn_contraction_order(int32_t n_tensors, const int32_t *ranks, const int64_t *labels,
                              const int64_t *dims, int32_t alg, int32_t *steps_out);

/* contract_network(tn; alg = Exact(order, order_alg)) (src/contract_network.jl:7-37): exact
 * contraction by pairwise GPU contractions (device permute + GEMM).  tensors[t] are host
 * row-major arrays in the order of their labels.  alg 0 = Greedy, 1 = LeftAssociative,
 * 2 = explicit `steps` (the itn_contraction_order format), 3 = sweep (see
 * itn_contraction_order).  precision: ITN_PREC_NATIVE
 * (dtype arithmetic on CUDA cores), ITN_PREC_BF16 (float32 data, tcgen05 GEMM with BF16
 * hi/lo split operands, ~16 significant bits) or ITN_PREC_TF32X3 (float32 data, tcgen05 GEMM
 * with TF32 hi/lo split operands: the accuracy of FP32 arithmetic).  The result (row-major in the order of out_labels, at most 48
 * indices) is copied to `out` if out_capacity elements suffice; device_ms (may be NULL)
 * receives the device time of the pairwise steps. */
int32_t itn_contract_network(itn_ctx *ctx, int32_t dtype, int32_t n_tensors, const int32_t *ranks,
                             const int64_t *labels, const int64_t *dims, const void *const *tensors,
                             int32_t alg, const int32_t *steps, int32_t precision, void *out,
                             int64_t out_capacity, int32_t *out_rank, int64_t *out_labels,
                             int64_t *out_dims, double *device_ms);

/* BP simple-update gate application, apply_gate_bp! (src/apply/apply_operators.jl:209-283),
 * for a batch of independent gates (e.g. one Trotter layer of gates on disjoint sites), one
 * CTA per gate, FP64 (complex128 for complex dtypes) arithmetic on the device.
 *
 * A site tensor is a row-major array with axes [other legs..., site index, shared bond];
 * a one-site gate has no shared-bond axis.  The other legs are gauged with X_e,
 * X_e^H X_e = env[e] (the D x D environment message M[bra][ket] of the edge pointing into
 * the site), which the reference obtains from gram_eigh_full(_with_pinv); env_off < 0
 * means no gauge on that leg.  Two-site gate: gauge, split each site into an isometry
 * and R (Gram eigendecomposition; the reference uses qr_compact), apply op[s1',s2',s1,s2]
 * to R1*R2, truncated SVD (the reference's svd_trunc; here from the Hermitian
 * eigendecomposition of theta theta^H, directions with sigma <= 1e-7 sigma_max dropped),
 * keep at most max_rank (> 0) values above cutoff (> 0), optionally divide S by its norm,
 * absorb sqrt(S) on both sides, undo the gauges.  The new sites have axes
 * [other legs..., site index, new bond]; out_bond[g] receives the new bond dimension chi
 * and out_s (from s_off) its singular values, which are the new environment diag(S) of
 * the bond in both directions.  One-site gate: op[s'][s] applied on the site index,
 * divided by the gauged norm when normalize.
 *
 * out_off[i] must leave room for prod(leg_dim) * d * chi_cap entries, chi_cap =
 * min(d1 * min(P1, d1 * bond), d2 * min(P2, d2 * bond)) with P_i the product of the other
 * leg dims of site i; s_off room for chi_cap values.  Limits: d <= 16, at most 6 other
 * legs of dimension <= 64 each, d * bond <= 128 and d * d * bond <= 128.  sites/envs/ops/
 * out_sites are host arrays of `dtype`; device_ms (may be NULL) receives the kernel time. */
typedef struct {
  int32_t nsite;          /* 1 or 2 */
  int32_t d[2];           /* site index dimension of each site */
  int32_t nleg[2];        /* number of other (gauged) legs of each site, <= 6 */
  int32_t bond;           /* dimension of the bond joining the two sites (2-site gates) */
  int32_t leg_dim[2][6];  /* dimensions of the other legs */
  int64_t site_off[2];    /* element offsets of the input sites in `sites` */
  int64_t env_off[2][6];  /* element offsets of each other leg's D x D message in `envs` (< 0: none) */
  int64_t op_off;         /* element offset of the operator in `ops` */
  int64_t out_off[2];     /* element offsets of the output sites in `out_sites` */
  int64_t s_off;          /* offset of the singular values in `out_s` */
} itn_gate_desc;

int32_t itn_apply_gates(itn_ctx *ctx, int32_t dtype, int64_t n_gates, const itn_gate_desc *gates,
                        const void *sites, int64_t n_site_elems, const void *envs,
                        int64_t n_env_elems, const void *ops, int64_t n_op_elems,
                        int32_t max_rank, double cutoff, int32_t normalize, void *out_sites,
                        int64_t out_capacity, double *out_s, int64_t s_capacity,
                        int32_t *out_bond, double *device_ms);

/* Gradient of the Bethe log-norm (bethe_free_energy, messagecache.jl:185-201) with
 * respect to every site tensor.  No counterpart in the reference (it has no AD); this is
 * the backward rule the Julia shim's ChainRulesCore.rrule(bp_logz) calls.
 * sweeps == 0 (implicit mode), for the converged messages currently held: the direct term
 * dlogZ_u/dA_u is always computed; with adjoint != 0 the implicit (adjoint BP) correction
 * lambda^T dF/dA is added, lambda solving lambda = dL/dm + J^T lambda by fixed-point
 * iteration until the relative change is below tol (ITN_ERR_TIMEOUT after maxiter).
 * sweeps > 0 (unrolled mode): runs `sweeps` parallel sweeps (beliefpropagation.jl:155-210)
 * from the current messages, leaves their result as the current messages, and returns the
 * exact gradient of the log-norm of that result, differentiating through every sweep in
 * reverse: lambda_T = dL/dm_T, lambda_{t-1} = J(m_{t-1})^T lambda_t, gradient = direct term
 * + sum_t lambda_t^T dF/dA(m_{t-1}).  The messages of every `checkpoint`-th sweep are kept
 * (checkpoint <= 1: every sweep) and the others recomputed from the nearest kept sweep in
 * the backward pass: device memory for about sweeps / checkpoint + checkpoint message sets
 * instead of sweeps, at the cost of one more forward pass; the result does not depend on
 * checkpoint (the recomputed sweeps are bit-identical).  adjoint, maxiter and tol are not
 * used in this mode.  normalized: the sweeps are SimpleMessageUpdate(normalize = true).
 * Real dtypes, norm networks (layers = 2). */
typedef struct {
  int32_t adjoint;
  int32_t maxiter;
  double tol;
  int32_t normalized;
  int32_t sweeps;      /* > 0: unrolled mode over this many sweeps */
  int32_t checkpoint;  /* unrolled mode: keep the messages of every checkpoint-th sweep */
  int32_t reserved0;
} itn_grad_opts;

typedef struct {
  int32_t adjoint_iterations;
  int32_t reserved0;
  double adjoint_residual;
  double device_ms;
} itn_grad_result;

int32_t itn_bp_grad(itn_ctx *ctx, const itn_grad_opts *opts, void *grad_packed,
                    itn_grad_result *result);

/* Vector-Jacobian product of one parallel sweep m -> F(m) (every message recomputed
 * by message_update!, beliefpropagation.jl:242-257, divided by its sum when normalized)
 * at the current messages: cot_in = J^T cot_out, both packed like the messages.  No
 * counterpart in the reference (no AD); it is the pullback an rrule of a BP sweep needs
 * and the inner step of the adjoint iteration of itn_bp_grad.  Real dtypes, layers = 2. */
int32_t itn_sweep_vjp(itn_ctx *ctx, int32_t normalized, const void *cot_out, void *cot_in);

/* Bethe log-norm (bethe_free_energy) of a network whose graph, tensors and messages are
 * already in device memory, computed without allocating device memory.  No counterpart
 * in the reference.  For callers whose GPU memory is owned by their own pooling allocator
 * (a CUDA.jl memory pool, a serving process that reserves HBM up front), where a library
 * cudaMalloc would fail or escape the pool.  All intermediates live in one process-wide
 * 16 MiB __device__ array: every GPU that loads the library holds it until exit, and
 * networks needing more (vertex + edge scalars + two contraction planes of
 * max_tensor_elems for one CTA) are rejected with ITN_ERR_ARG and a message in errbuf.
 * The first call on a device sets up the array's address (call it before any stream
 * capture); calls that overlap on the GPU race on the array and must be ordered.
 * Device arrays use the layout of itn_graph_upload / itn_tensors_upload: int32 d_off
 * (nv+1), d_rev, d_bond (per slot), d_phys (nv); int64 d_toff (nv+1), d_moff (nslots+1);
 * max_tensor_elems bounds every vertex's tensor.  Outputs: d_total = (re, im) of
 * sum log Zv - sum log Ze, d_flags as in itn_logscalars plus three bits for vertices the
 * call cannot contract (each makes its Z_u NaN, so the total is NaN): bit3 a tensor larger
 * than max_tensor_elems, bit4 more than 16 legs, bit5 a one-layer vertex whose physical
 * dimension is not 1 (one-layer networks need phys = 1, as in itn_graph_upload).  Work is
 * enqueued on `stream` (a cudaStream_t, may be NULL) and the outputs are ready when it
 * completes. */
int32_t itn_logz_static_scratch(int32_t device, void *stream, int32_t dtype, int32_t layers,
                                int64_t nv, int64_t nslots, int64_t max_tensor_elems,
                                const int32_t *d_off, const int32_t *d_rev, const int32_t *d_bond,
                                const int32_t *d_phys, const int64_t *d_toff,
                                const int64_t *d_moff, const void *d_tensors,
                                const void *d_messages, double *d_total, int32_t *d_flags,
                                char *errbuf, int32_t errbuf_len);

/* Fault injection for tests, with no counterpart in the reference (it has no device code
 * to fail).  ITN_FAULT_WAIT_NS: elapsed-time limit in ns of the bounded device waits of the
 * persistent launches (the tensor-core sweep's waits on other items' messages, the grid
 * barriers of the CUDA-core sweeps and of the adjoint; value <= 0 restores the default of
 * 2 s).
 * ITN_FAULT_STALL (value 1 / 0): in the persistent tensor-core sweeps, one such wait looks
 * for a message that is never written, so it runs out after the limit; the kernel then stops
 * early, waits for its own copies, releases its resources and the call returns
 * ITN_ERR_TIMEOUT, with the device and the context still usable.  ITN_FAULT_ALLOC: the next
 * `value` device allocations the library makes on the calling thread fail, so the calls
 * making them return ITN_ERR_OOM (the host-side stand-in for exhausted device memory).
 * ITN_FAULT_STALL also applies to the grid barriers of the gradient's persistent adjoint
 * launch and of the persistent CUDA-core sweeps: one CTA leaves before the first barrier,
 * the others' waits (limit ITN_FAULT_WAIT_NS) run out and itn_bp_grad / itn_bp_run return
 * ITN_ERR_TIMEOUT.  ITN_FAULT_NO_PERSISTENT_ADJOINT (value 1 / 0): the
 * adjoint iteration runs as one launch per iteration instead of one persistent launch (the
 * same arithmetic; lets a test compare the two).  ITN_FAULT_NO_PERSISTENT_SWEEPS (value 1 / 0):
 * the same for the CUDA-core parallel sweeps of small two-layer networks. */
enum {
  ITN_FAULT_WAIT_NS = 1,
  ITN_FAULT_ALLOC = 2,
  ITN_FAULT_STALL = 3,
  ITN_FAULT_NO_PERSISTENT_ADJOINT = 4,
  ITN_FAULT_NO_PERSISTENT_SWEEPS = 5
};
int32_t itn_inject_fault(itn_ctx *ctx, int32_t kind, int64_t value);

/* Diagnostic with no counterpart in the reference: runs a one-CTA tcgen05 BF16 product
 * (M = 128 and M = 64, K = 64) against exact host arithmetic.  m128_ok / m64_ok report
 * success; max_err is the largest absolute error of the M = 128 product; lane_of_row
 * (64 entries, may be NULL) receives the TMEM lane of each row of the M = 64
 * accumulator.  The tensor-core precision modes refuse to run when it fails. */
int32_t itn_tc_selftest(itn_ctx *ctx, int32_t *m128_ok, int32_t *m64_ok, double *max_err,
                        int32_t *lane_of_row);

#ifdef __cplusplus
}
#endif

#endif /* ITN_GPU_H */
