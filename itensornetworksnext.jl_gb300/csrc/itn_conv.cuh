// itn_conv.cuh -- device-side state of the outer BP loop (StopAfterIteration(maxiter) |
// StopWhenConverged(tol), AlgorithmsInterfaceExtensions.jl:84-118, with
// iterate_diff = max over slots of 1 - |<m_new, m_old>|^2, beliefpropagation.jl:261-267).
//
// Sweep kernels fold the per-slot diffs into `dmax` (order-encoded atomicMax); the last
// CTA of a sweep (ticket counter) then advances the iteration counter, records delta
// and raises `done` when delta < tol.  Every sweep kernel returns at once when `done`
// is set, so a fixed, graph-captured launch sequence stops exactly where the reference
// loop stops.
#pragma once
#include <math.h>

#include "itn_common.cuh"

namespace itn {

struct ConvState {
  unsigned long long dmax;  // order-encoded max of this sweep's diffs
  int nan_flag;             // a diff was NaN in this sweep
  int done;                 // converged: later sweeps do nothing
  int at_iter;              // iteration at which delta < tol (-1 if never)
  int iters;                // sweeps executed
  double delta;             // last delta
  int counter;              // iteration counter
  unsigned tickets;         // CTAs finished in the current sweep
  double tol;
  int use_tol;
  int pad;
};

// One outer-loop step after a sweep (single thread).
__device__ __forceinline__ void conv_step(ConvState* s) {
  if (s->done) return;
  const int iter = ++s->counter;
  s->iters = iter;
  if (!s->use_tol) return;
  volatile unsigned long long* dm = &s->dmax;
  volatile int* nf = &s->nan_flag;
  double delta = dec_double(*dm);
  if (*nf) delta = nan("");
  s->delta = delta;
  if (delta < s->tol) {
    s->done = 1;
    s->at_iter = iter;
  }
  *dm = enc_double(-INFINITY);
  *nf = 0;
}

// Called by every CTA of a sweep kernel after its last global write (all threads);
// the last CTA performs conv_step (`steps` times for a kernel that ran several sweeps
// without a convergence test).  Threads that issued diff atomics must have executed
// __threadfence() before reaching this call.
__device__ __forceinline__ void conv_finish_cta(ConvState* s, int steps = 1) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(&s->tickets, 1u);
    if (t == gridDim.x - 1) {
      __threadfence();
      for (int k = 0; k < steps; ++k) conv_step(s);
      s->tickets = 0;
      __threadfence();
    }
  }
}

}  // namespace itn
