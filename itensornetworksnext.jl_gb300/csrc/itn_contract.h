// itn_contract.h -- pairwise network contraction pieces (contract.cu) used by the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <utility>
#include <vector>

namespace itn {

// Pairwise order on a working list: each step (i, j) contracts positions i and j (result
// labels: free(i) ++ free(j)), removes both and appends the result.  alg 0 = greedy
// (smallest growth, sharing pairs first), 1 = left-associative, 3 = sweep (the cheaper of the
// greedy order and running-product sweeps that absorb the neighbour leaving the product
// smallest, by multiply-adds).
int contraction_order(const std::vector<std::vector<int64_t>>& labels, const std::map<int64_t, int64_t>& dim,
                      int alg, std::vector<std::pair<int, int>>& steps);

// out = in with its axes permuted: output axis a is input axis perm[a] (row-major both).
cudaError_t contract_permute(int dtype, const void* in, void* out, const std::vector<int64_t>& in_dims,
                             const std::vector<int>& perm, cudaStream_t st);

// C[M,N] = A[M,K] B[K,N] (row-major) on CUDA cores.
cudaError_t contract_gemm(int dtype, const void* A, const void* B, void* C, long long M, long long N, long long K,
                          cudaStream_t st);

// Float32 C[M,N] = A[M,K] B[K,N] on tcgen05 with hi/lo split operands (3 MMAs per product):
// BF16 hi/lo, or TF32 hi/lo when `tf32` (FP32 accuracy).  Returns cudaErrorNotSupported when
// the tensor-core self-test has not passed.
cudaError_t contract_gemm_tc(const float* A, const float* B, float* C, long long M, long long N, long long K,
                             cudaStream_t st, bool tf32);

}  // namespace itn
