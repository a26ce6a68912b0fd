// itn_z3.h -- the grouped sweep for networks whose vertices all have three legs (bp_z3.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "itn_conv.cuh"

namespace itn {

constexpr int kZ3Threads = 256;          // 8 warps per CTA, one vertex per warp at a time
constexpr int kZ3MaxClasses = 8;
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

struct Z3Args {
  const int* off;          // nv + 1 (three slots per vertex)
  const int* rev;          // nslots
  const int* bond;         // nslots
  const long long* toff;   // nv + 1
  const long long* moff;   // nslots + 1
  const void* tens;
  const void* msg_in;
  void* msg_out;
  const int* items;        // vertices, largest tensors first
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
