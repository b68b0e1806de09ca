/* The C ABI from plain C (what a Fortran iso_c_binding module binds).
   Part 1: a periodic 16x12x8 FP32 meshblock on the fused-exact path, inputs
   from an exact integer formula (the same as cabi_fields in
   tests/golden/make_golden.py), the prologue and 3 steps; E and B are
   written raw to the file named by argv[1], which tests/test_c_abi.py
   compares bit for bit with the golden fixture cabi_fp32_periodic.
   Part 2: a periodic 48x32x24 FP32 meshblock, a uniform Bz plus a small Ex
   ripple, 10 fused steps, finiteness and the uniform field kept; then the
   batch and output entry points on the same handle.
   Exit status 0 on success. */
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

/* value of the golden input formula at ghosted-array position i */
static float cabi(size_t i, unsigned mul, unsigned mod, int off, float den, float base) {
  return base + (float)((int)((i * mul) % mod) - off) / den;
}

static int golden_part(const char* path) {
  ffe_grid_desc d;
  CHECK(ffe_desc_default(&d, 16, 12, 8));
  d.precision = FFE_FP32;
  d.path = FFE_PATH_FUSED_EXACT;
  ffe_t h = NULL;
  CHECK(ffe_create(&h, &d));
  size_t n = 0;
  CHECK(ffe_field_elems(h, &n));
  float* f[6];
  for (int c = 0; c < 6; ++c) f[c] = malloc(n * sizeof(float));
  for (size_t i = 0; i < n; ++i) {
    f[0][i] = cabi(i, 37, 101, 50, 4096.0f, 0.0f);
    f[1][i] = cabi(i, 53, 97, 48, 4096.0f, 0.0f);
    f[2][i] = cabi(i, 29, 89, 44, 4096.0f, 0.0f);
    f[3][i] = cabi(i, 17, 83, 41, 8192.0f, 0.0f);
    f[4][i] = cabi(i, 41, 79, 39, 8192.0f, 0.0f);
    f[5][i] = cabi(i, 13, 73, 36, 8192.0f, 1.0f);
  }
  int32_t ids[6] = {FFE_EX, FFE_EY, FFE_EZ, FFE_BX, FFE_BY, FFE_BZ};
  const void* up[6] = {f[0], f[1], f[2], f[3], f[4], f[5]};
  void* down[6] = {f[0], f[1], f[2], f[3], f[4], f[5]};
  CHECK(ffe_upload_many(h, 6, ids, up, n));
  CHECK(ffe_mainloop_prologue(h));
  CHECK(ffe_step(h, 3, 0));
  CHECK(ffe_download_many(h, 6, ids, down, n));
  CHECK(ffe_destroy(h));
  FILE* out = fopen(path, "wb");
  if (!out) {
    fprintf(stderr, "cannot write %s\n", path);
    return 1;
  }
  for (int c = 0; c < 6; ++c) {
    if (fwrite(f[c], sizeof(float), n, out) != n) {
      fclose(out);
      return 1;
    }
    free(f[c]);
  }
  fclose(out);
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 1 && golden_part(argv[1]) != 0) return 1;
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
