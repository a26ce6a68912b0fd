/*
 * bp_oracle.c -- CPU restatement of ITensorNetworksNext.jl's belief-propagation hot
 * path (message updates, iterate_diff, vertex/edge scalars, bethe_free_energy).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU results are compared with:
 * the tests, the smoke check and the CPU-baseline leg of the benchmark call it; the GPU
 * library never links, loads or falls back to it.
 *
 * Reference semantics restated (paths inside ITensorNetworksNext.jl):
 *   src/beliefpropagation/beliefpropagation.jl:69-92   beliefpropagation entry
 *   src/beliefpropagation/beliefpropagation.jl:200-210 sequential sweep step
 *   src/beliefpropagation/beliefpropagation.jl:242-257 SimpleMessageUpdate
 *   src/beliefpropagation/beliefpropagation.jl:261-267 iterate_diff
 *   src/AlgorithmsInterfaceExtensions/AlgorithmsInterfaceExtensions.jl:73-118
 *   src/beliefpropagation/messagecache.jl:124-201       incoming messages, scalars
 *   src/normnetwork.jl:49-54,66-82                      ket * conj(bra) factor
 *
 * Data model shared with the GPU library (both sides see the same arrays):
 *   vertex u has legs off[u] .. off[u+1]-1 (CSR); slot s = off[u]+l is the directed
 *   edge u -> nbr[s], bond dim bond[s]; rev[s] is the slot of nbr[s] -> u.
 *   Site tensor of u: toff[u] .. toff[u+1], row-major [phys][leg_0]..[leg_{z-1}].
 *   Message on slot s: moff[s] .. moff[s+1]; two-layer (norm network) messages are
 *   D x D row-major [bra][ket]; single-layer messages are length-D vectors.
 *
 * Parity anchor: the reference is Julia with its arithmetic in un-vendored
 * ITensorBase 0.10 / TensorAlgebra 0.16; no Julia exists here, so this restatement is
 * pinned by the reference's own known-answer tests (tree exactness, spin ice 1.5^(n^2),
 * <psi|psi> = |psi|^2, 1D Ising) -- see tests/test_oracle_pins.py.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_MAX_LEGS 16

typedef struct {
  int64_t nv;
  const int64_t *off;  /* nv + 1 */
  const int64_t *nbr;  /* off[nv] */
  const int64_t *rev;  /* off[nv] */
  const int64_t *toff; /* nv + 1 */
  const int64_t *moff; /* off[nv] + 1 */
  const int32_t *bond; /* off[nv] */
  const int32_t *phys; /* nv */
  int32_t layers;      /* 1 = plain network, 2 = norm network */
  int32_t pad;
} orc_graph;

/* ---- float64 ---- */
#define T double
#define SUF f64
#define CONJ(x) (x)
#define ABS2(x) ((double)(x) * (double)(x))
#define REALP(x) ((double)(x))
#define IMAGP(x) (0.0)
#define IS_COMPLEX 0
#include "bp_oracle_impl.h"
#undef T
#undef SUF
#undef CONJ
#undef ABS2
#undef REALP
#undef IMAGP
#undef IS_COMPLEX

/* ---- float32 (arithmetic in float, as a plain FP32 CPU path) ---- */
#define T float
#define SUF f32
#define CONJ(x) (x)
#define ABS2(x) ((double)(x) * (double)(x))
#define REALP(x) ((double)(x))
#define IMAGP(x) (0.0)
#define IS_COMPLEX 0
#include "bp_oracle_impl.h"
#undef T
#undef SUF
#undef CONJ
#undef ABS2
#undef REALP
#undef IMAGP
#undef IS_COMPLEX

/* ---- complex128 ---- */
#define T double _Complex
#define SUF c128
#define CONJ(x) conj(x)
#define ABS2(x) (creal(x) * creal(x) + cimag(x) * cimag(x))
#define REALP(x) creal(x)
#define IMAGP(x) cimag(x)
#define IS_COMPLEX 1
#include "bp_oracle_impl.h"
#undef T
#undef SUF
#undef CONJ
#undef ABS2
#undef REALP
#undef IMAGP
#undef IS_COMPLEX

/* ---- complex64 (arithmetic in float complex) ---- */
#define T float _Complex
#define SUF c64
#define CONJ(x) conjf(x)
#define ABS2(x) ((double)crealf(x) * crealf(x) + (double)cimagf(x) * cimagf(x))
#define REALP(x) ((double)crealf(x))
#define IMAGP(x) ((double)cimagf(x))
#define IS_COMPLEX 1
#include "bp_oracle_impl.h"
#undef T
#undef SUF
#undef CONJ
#undef ABS2
#undef REALP
#undef IMAGP
#undef IS_COMPLEX

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
