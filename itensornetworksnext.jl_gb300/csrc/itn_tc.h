// itn_tc.h -- interface of the tensor-core (tcgen05) sweep engine in bp_tc.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace itn {

struct TcEngine;

struct TcRun {
  const void* msg_in;
  void* msg_out;
  int precision;  // ITN_PREC_BF16 or ITN_PREC_TF32
  bool split;     // hi/lo split-precision sweep
  int normalize;
  double* slot_diff;
  unsigned long long* diff_max;
  int* nan_flag;
  const int* done;
};

TcEngine* tc_create();
void tc_destroy(TcEngine* e);
// Drop cached operand copies (the network or the tensors changed).
void tc_invalidate(TcEngine* e);
// Check that the uploaded network fits the tensor-core kernel and build its operand
// copies.  On an unsupported network *why is set and cudaSuccess returned.
cudaError_t tc_prepare(TcEngine* e, int layers, int64_t nv, const int64_t* off, const int32_t* bond,
                       const int32_t* phys, const int* d_off, const int* d_rev,
                       const long long* d_moff, const void* d_tens, const int64_t* toff,
                       int precision, cudaStream_t st, const char** why);
// Enqueue one sweep (all directed messages) on the stream.
cudaError_t tc_sweep(TcEngine* e, const TcRun& r, cudaStream_t st);

}  // namespace itn
