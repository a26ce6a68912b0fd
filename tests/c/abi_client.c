/* A C client of libitn_gpu.so: compiled against include/itn_gpu.h and linked like any FFI
 * user would link it.  Without a GPU it checks the host-only entry points and that device
 * entry points fail with a status instead of aborting; with a GPU it runs a 2-vertex BP
 * solve and checks the log-norm against the closed form.  Prints "ok" on success. */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

#include "itn_gpu.h"

#define CHECK(cond, msg)                        \
  do {                                          \
    if (!(cond)) {                              \
      fprintf(stderr, "FAILED: %s\n", msg);     \
      return 1;                                 \
    }                                           \
  } while (0)

int main(int argc, char **argv) {
  const int want_gpu = argc > 1 && argv[1][0] == 'g';
  CHECK(itn_abi_version() == ITN_ABI_VERSION, "abi version");
  /* host-only: contraction order of a 3-tensor ring a-b, b-c, c-a */
  int32_t ranks[3] = {2, 2, 2};
  int64_t labels[6] = {0, 1, 1, 2, 2, 0};
  int64_t dims[6] = {2, 3, 3, 4, 4, 2};
  int32_t steps[4] = {-1, -1, -1, -1};
  CHECK(itn_contraction_order(3, ranks, labels, dims, 0, steps) == ITN_OK, "contraction order");
  CHECK(steps[0] >= 0 && steps[1] > steps[0], "greedy first step");
  int64_t bad_labels[6] = {0, 0, 1, 2, 2, 3}; /* repeated index on one tensor */
  int64_t bad_dims[6] = {2, 2, 3, 4, 4, 5};
  CHECK(itn_contraction_order(3, ranks, bad_labels, bad_dims, 0, steps) == ITN_ERR_UNSUPPORTED,
        "repeated index rejected");
  int64_t clash_dims[6] = {2, 3, 5, 4, 4, 2}; /* index 1 with dims 3 and 5 */
  CHECK(itn_contraction_order(3, ranks, labels, clash_dims, 0, steps) == ITN_ERR_ARG,
        "dimension clash rejected");
  /* the gate descriptor layout a ctypes / ccall binding mirrors */
  CHECK(sizeof(itn_gate_desc) == 216 && offsetof(itn_gate_desc, site_off) == 72 &&
            offsetof(itn_gate_desc, s_off) == 208,
        "itn_gate_desc layout");
  CHECK(itn_apply_gates(NULL, ITN_F64, 0, NULL, NULL, 0, NULL, 0, NULL, 0, 0, 0.0, 0, NULL, 0, NULL, 0, NULL,
                        NULL) == ITN_ERR_ARG,
        "apply_gates without a context");
  CHECK(itn_create(NULL, 0, 0) == ITN_ERR_ARG, "null out pointer");
  itn_ctx *ctx = NULL;
  const int32_t st = itn_create(&ctx, 0, 0);
  if (!want_gpu) {
    CHECK(st == ITN_OK || st == ITN_ERR_CUDA, "create status");
    if (st == ITN_OK) itn_destroy(ctx);
    printf("ok\n");
    return 0;
  }
  CHECK(st == ITN_OK, "create on a GPU");
  /* two vertices joined by one D=2 leg, phys 2: A_u = B_u = identity-like */
  int64_t off[3] = {0, 1, 2}, nbr[2] = {1, 0};
  int32_t bond[2] = {2, 2}, phys[2] = {2, 2};
  CHECK(itn_graph_upload(ctx, 2, off, nbr, bond, NULL, phys, 2, NULL) == ITN_OK, itn_last_error(ctx));
  double t[8] = {1, 0, 0, 1, 1, 0, 0, 1}; /* A[s][k] = delta(s,k) on both vertices */
  CHECK(itn_tensors_upload(ctx, ITN_F64, t) == ITN_OK, itn_last_error(ctx));
  CHECK(itn_messages_init(ctx, ITN_MSG_IDENTITY_NORMALIZED) == ITN_OK, itn_last_error(ctx));
  itn_bp_opts o = {ITN_SCHED_PARALLEL, 5, -1.0, 1, ITN_PREC_NATIVE, 0, 0, NULL, 0};
  itn_bp_result r;
  CHECK(itn_bp_run(ctx, &o, &r) == ITN_OK, itn_last_error(ctx));
  CHECK(r.iterations == 5, "iterations");
  double tot[2];
  int32_t flags[1];
  CHECK(itn_logscalars(ctx, NULL, NULL, NULL, NULL, tot, flags) == ITN_OK, itn_last_error(ctx));
  /* <psi|psi> = sum_{s,s'} (sum_k d(s,k) d(s',k))^2 = 2: BP is exact on a tree */
  CHECK(fabs(tot[0] - log(2.0)) < 1e-12, "log-norm of the two-site network");
  /* an identity two-site gate on two sites without other legs (s = 2, bond 2) leaves the
   * contracted pair unchanged */
  {
    double sites[8] = {0.3, -1.2, 0.7, 2.0, 1.1, 0.4, -0.5, 0.9}; /* psi1[s][b], psi2[s][b] */
    double op[16] = {0};
    for (int k = 0; k < 4; ++k) op[k * 5] = 1.0;
    itn_gate_desc g = {0};
    g.nsite = 2;
    g.d[0] = g.d[1] = 2;
    g.bond = 2;
    g.site_off[0] = 0;
    g.site_off[1] = 4;
    g.op_off = 0;
    g.out_off[0] = 0;
    g.out_off[1] = 4; /* chi_cap = 2 * min(1, 4) = 2 */
    g.s_off = 0;
    double out[8], s[2];
    int32_t chi = 0;
    CHECK(itn_apply_gates(ctx, ITN_F64, 1, &g, sites, 8, NULL, 0, op, 16, 0, 0.0, 0, out, 8, s, 2, &chi, NULL) ==
              ITN_OK,
          itn_last_error(ctx));
    CHECK(chi >= 1 && chi <= 2, "new bond dimension");
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        double want = 0, got = 0;
        for (int k = 0; k < 2; ++k) want += sites[a * 2 + k] * sites[4 + b * 2 + k];
        for (int k = 0; k < chi; ++k) got += out[a * chi + k] * out[4 + b * chi + k];
        CHECK(fabs(got - want) < 1e-12, "identity gate keeps the pair");
      }
  }
  itn_destroy(ctx);
  printf("ok\n");
  return 0;
}
