// itn_apply.h -- device job description of the gate-application kernel (apply_gates.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace itn {

constexpr int kGateMaxLegs = 6;

// One gate as the kernel sees it: the C-ABI descriptor plus the workspace offset and the
// capacity of the new bond.  Element offsets refer to the FP64 / complex128 device copies.
struct GateJob {
  int nsite;
  int d[2];
  int nleg[2];
  int bond;
  int leg_dim[2][kGateMaxLegs];
  int64_t site_off[2];
  int64_t env_off[2][kGateMaxLegs];
  int64_t op_off;
  int64_t out_off[2];
  int64_t s_off;
  int64_t ws;   // workspace offset (elements)
  int chi_cap;  // largest possible new bond dimension (2-site gates)
};

// Workspace elements one gate needs (J.chi_cap must be set).
int64_t gate_workspace(GateJob& J);

cudaError_t launch_gates(bool complex_data, int n, const GateJob* d_jobs, const void* d_sites, const void* d_envs,
                         const void* d_ops, void* d_out, double* d_s, int* d_bond, void* d_ws, int max_rank,
                         double cutoff, int normalize, cudaStream_t st);

}  // namespace itn
