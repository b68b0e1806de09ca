/* The C ABI from plain C (what a Fortran iso_c_binding module binds): create a
   periodic 48x32x24 FP32 meshblock, upload a uniform Bz plus a small Ex ripple,
   run the prologue and 10 fused steps, download, check finiteness and that the
   uniform field is kept; then the batch and output entry points on the same
   handle.  Exit status 0 on success.  Built and run by tests/test_c_abi.py. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "ffe.h"

#define CHECK(call)                                                       \
  do {                                                                    \
    int rc_ = (call);                                                     \
    if (rc_ != FFE_OK) {                                                  \
      char msg_[256];                                                     \
      ffe_last_error(NULL, msg_, sizeof msg_);                            \
      fprintf(stderr, "%s -> %d (%s)\n", #call, rc_, msg_);               \
      return 1;                                                           \
    }                                                                     \
  } while (0)

int main(void) {
  ffe_grid_desc d;
  CHECK(ffe_desc_default(&d, 48, 32, 24));
  d.precision = FFE_FP32;
  ffe_t h = NULL;
  CHECK(ffe_create(&h, &d));
  size_t n = 0;
  CHECK(ffe_field_elems(h, &n));
  float* zero = calloc(n, sizeof(float));
  float* bz = malloc(n * sizeof(float));
  float* ex = malloc(n * sizeof(float));
  for (size_t i = 0; i < n; ++i) {
    bz[i] = 1.0f;
    ex[i] = 1e-3f * (float)sin(0.37 * (double)(i % 52));
  }
  int32_t ids[6] = {FFE_EX, FFE_EY, FFE_EZ, FFE_BX, FFE_BY, FFE_BZ};
  const void* up[6] = {ex, zero, zero, zero, zero, bz};
  CHECK(ffe_upload_many(h, 6, ids, up, n));
  CHECK(ffe_mainloop_prologue(h));
  CHECK(ffe_step(h, 10, 0));
  CHECK(ffe_synchronize(h));
  int32_t ok = 0;
  CHECK(ffe_check_finite(h, &ok));
  float* out = malloc(n * sizeof(float));
  CHECK(ffe_download(h, FFE_BZ, out, n));
  double dev = 0;
  for (size_t i = 0; i < n; ++i) dev = fmax(dev, fabs((double)out[i] - 1.0));
  if (!ok || dev > 1e-2) {
    fprintf(stderr, "finite=%d max |Bz-1|=%g\n", ok, dev);
    return 1;
  }
  ffe_batch_t b = NULL;
  CHECK(ffe_batch_create(&b, &h, 1, NULL));
  int32_t s0 = 10;
  CHECK(ffe_batch_step(b, 5, &s0));
  CHECK(ffe_batch_synchronize(b));
  CHECK(ffe_batch_destroy(b));
  int32_t dims[3];
  CHECK(ffe_output_dims(h, 2, dims));
  size_t nn = (size_t)dims[0] * dims[1] * dims[2];
  float* nodes = malloc(12 * nn * sizeof(float));
  CHECK(ffe_output(h, 2, nodes, 12 * nn));
  if (dims[0] != 24 || dims[1] != 16 || dims[2] != 12 || nodes[9 * nn + 1] != 2.0f) {
    fprintf(stderr, "output dims %d %d %d, xx[1] = %g\n", dims[0], dims[1], dims[2], nodes[9 * nn + 1]);
    return 1;
  }
  CHECK(ffe_destroy(h));
  free(zero);
  free(bz);
  free(ex);
  free(out);
  free(nodes);
  printf("c abi ok\n");
  return 0;
}
