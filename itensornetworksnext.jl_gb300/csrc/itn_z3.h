// itn_z3.h -- the grouped sweep for networks whose vertices all have three legs (bp_z3.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "itn_conv.cuh"

namespace itn {

constexpr int kZ3Threads = 256;          // 8 warps per CTA, one vertex per warp at a time
constexpr int kZ3MaxClasses = 16;
constexpr size_t kZ3MaxSmem = 227 * 1024;
constexpr int kZ3MaxTensor = 1024;       // entries of a vertex tensor (d * D0 * D1 * D2)
constexpr int kZ3MaxBond = 8;

// One size class of the work list: items[first .. first + count) (vertices whose tensors
// have at most nmax entries) on CTAs [cta_start, cta_start + ctas); each CTA runs `groups`
// groups of `wpi` warps (one vertex per group at a time) with `slice` elements of shared
// memory each (3 nmax + 192 + 256).
struct Z3Class {
  int first, count;
  int cta_start, ctas;
  int wpi, groups;
  int nmax;
  int slice;
};

// Everything a group needs to start on one work item, in work-list order: one dependent load
// instead of the chain off -> bond / rev -> moff.
struct Z3Meta {
  long long t0;            // first tensor entry
  long long moff_in[3];    // offsets of the incoming messages on legs 0, 1, 2
  long long moff_out[3];   // offsets of the outgoing messages (slots s0, s0 + 1, s0 + 2)
  int s0;                  // first slot of the vertex
  int n;                   // tensor entries
  int D[3];                // bond dimensions of legs 0, 1, 2
  int pad;
};

struct Z3Args {
  const Z3Meta* meta;      // per work item, largest tensors first
  const void* tens;
  const void* msg_in;
  void* msg_out;
  int normalize;
  double* slot_diff;       // per-slot fidelity diffs (null: no convergence test)
  ConvState* conv;         // outer-loop state; every CTA takes part in the step
  int n_classes;
  Z3Class cls[kZ3MaxClasses];
};

// One parallel sweep msg_in -> msg_out (dtype 0..3 = float, double, complex64, complex128).
cudaError_t launch_sweep_z3(int dtype, const Z3Args& a, int grid, size_t smem, cudaStream_t st);
// CTAs of the grouped sweep resident per SM with `smem` bytes of dynamic shared memory.
int z3_blocks_per_sm(int dtype, size_t smem);

}  // namespace itn
