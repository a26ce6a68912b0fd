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
// Thin pairwise steps (at most 32 rows of A or columns of B, K <= 64, the long side >= 256):
// the long operand can be read in place through a view instead of being permuted first.
constexpr int kViewMaxRank = 48, kViewMaxK = 64;
struct ThinView {
  int rank;                        // free axes of the long operand (adjacent ones merged), outer first
  int dims[kViewMaxRank];
  long long stride[kViewMaxRank];  // element strides of those axes in the long operand
  long long koff[kViewMaxK];       // element offset of each contracted position k (row-major over
                                   // the contracted axes in the step's order)
};
bool contract_thin_shape(long long M, long long N, long long K);
// true: B is the thin operand (A is read through the view); false: A is thin (B through the view)
bool contract_thin_small_b(long long M, long long N);
// C[M,N] = A B with the long operand read through `v` (its pointer in its own layout) and the
// thin one contiguous ([M,K] row-major A or [K,N] row-major B).
cudaError_t contract_gemm_view(int dtype, const void* A, const void* B, void* C, long long M, long long N,
                               long long K, bool small_b, const ThinView& v, cudaStream_t st);
cudaError_t contract_gemm(int dtype, const void* A, const void* B, void* C, long long M, long long N, long long K,
                          cudaStream_t st);

// Float32 C[M,N] = A[M,K] B[K,N] on tcgen05 with hi/lo split operands (3 MMAs per product):
// BF16 hi/lo, or TF32 hi/lo when `tf32` (FP32 accuracy).  Returns cudaErrorNotSupported when
// the tensor-core self-test has not passed.
cudaError_t contract_gemm_tc(const float* A, const float* B, float* C, long long M, long long N, long long K,
                             cudaStream_t st, bool tf32);

}  // namespace itn
