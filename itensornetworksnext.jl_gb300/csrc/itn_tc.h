// itn_tc.h -- interface of the tensor-core (tcgen05) sweep engine in bp_tc.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace itn {

struct TcEngine;
struct ConvState;

struct TcRun {
  const void* msg_in;
  void* msg_out;
  int precision;  // ITN_PREC_BF16 or ITN_PREC_TF32
  bool split;     // hi/lo split-precision sweep
  int normalize;
  double* slot_diff;  // per-slot diffs (null: no convergence test)
  ConvState* conv;    // outer-loop state (done flag, diff max, iteration step)
};

TcEngine* tc_create();
void tc_destroy(TcEngine* e);
// Drop cached operand copies (the network or the tensors changed).
void tc_invalidate(TcEngine* e);
// Check that the uploaded network fits the tensor-core kernel (a norm network whose vertices
// have at most 4 legs, bonds of at most 8 and a physical dimension of at most 2; anything but
// 4 legs of 8 with d = 2 runs zero-padded to that frame) and build its operand copies.  On an
// unsupported network *why is set and cudaSuccess returned.  off, rev, moff, bond, phys, toff:
// the host copies of the uploaded CSR graph, message and tensor offsets.
cudaError_t tc_prepare(TcEngine* e, int layers, int64_t nv, const int64_t* off, const int64_t* rev,
                       const int64_t* moff, const int32_t* bond, const int32_t* phys, const int* d_off,
                       const int* d_rev, const long long* d_moff, const void* d_tens, const int64_t* toff,
                       int precision, cudaStream_t st, const char** why);
// Enqueue one sweep (all directed messages) on the stream.
cudaError_t tc_sweep(TcEngine* e, const TcRun& r, cudaStream_t st);
// Enqueue `nsweeps` sweeps as one cooperative launch (one CTA per SM, independent 4-warp
// groups; intermediate messages travel through tagged device buffers): reads r.msg_in,
// writes r.msg_out (the two may be the same buffer).  Needs r.slot_diff == null (no
// convergence test inside).  *used = false (and nothing enqueued) when the device cannot
// host the cooperative grid, for a padded network, or for nsweeps == 2 or > 4095.
cudaError_t tc_sweeps_persistent(TcEngine* e, const TcRun& r, int nsweeps, cudaStream_t st, bool* used);
// Device address of the engine's error flag, non-zero once a bounded wait inside the
// tensor-core kernel gave up (reset by tc_prepare; null before the first prepare).
const int* tc_err_ptr(const TcEngine* e);
// Elapsed-time limit (ns) of a sweep kernel's wait on another item's message; a wait that
// runs out sets the error flag (ITN_ERR_TIMEOUT for the caller).  Applies to launches
// recorded after the call.
constexpr uint64_t kDefaultWaitNs = 2000000000ull;
void tc_set_wait_limit(TcEngine* e, uint64_t ns);
// Fault injection: in persistent launches recorded after the call, one wait (the first group's
// item in the second sweep) looks for a tag that no producer writes, so it runs out.
void tc_set_stall(TcEngine* e, int on);
// Account for up to `n` persistent launches about to be enqueued (a solve graph holds at
// most two); clears the tagged buffers and restarts the epoch on the stream before the
// 20-bit epoch could wrap onto a stale entry.
cudaError_t tc_note_launches(TcEngine* e, int n, cudaStream_t st);
// One-CTA tcgen05 self-test (cached per process): M=128 product exact, M=64
// accumulator lane map found.  lane_of_row may be null (64 entries otherwise).
cudaError_t tc_run_probe(cudaStream_t st, int* m128_ok, int* m64_ok, double* max_err, int* lane_of_row);
// The probe's exact TF32 product (kind::tf32) passed (false before the probe has run).
bool tc_tf32_ok();

}  // namespace itn
