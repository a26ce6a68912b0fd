// bp_tc.cu -- tensor-core (tcgen05) sweep engine.  Placeholder until the kernel lands:
// every network is reported as unsupported.
#include "itn_tc.h"

namespace itn {

struct TcEngine {
  int dummy = 0;
};

TcEngine* tc_create() { return new TcEngine(); }
void tc_destroy(TcEngine* e) { delete e; }
void tc_invalidate(TcEngine* e) { (void)e; }

cudaError_t tc_prepare(TcEngine* e, int layers, int64_t nv, const int64_t* off, const int32_t* bond,
                       const int32_t* phys, const int* d_off, const int* d_rev,
                       const long long* d_moff, const void* d_tens, const int64_t* toff,
                       int precision, cudaStream_t st, const char** why) {
  (void)e; (void)layers; (void)nv; (void)off; (void)bond; (void)phys; (void)d_off; (void)d_rev;
  (void)d_moff; (void)d_tens; (void)toff; (void)precision; (void)st;
  *why = "tensor-core precision modes are not built";
  return cudaSuccess;
}

cudaError_t tc_sweep(TcEngine* e, const TcRun& r, cudaStream_t st) {
  (void)e; (void)r; (void)st;
  return cudaErrorNotSupported;
}

}  // namespace itn
