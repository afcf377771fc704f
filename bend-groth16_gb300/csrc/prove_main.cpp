// prove_bin: drop-in for the Bend prover binary (bend2/prove.bend:164-168).
// Reads the .bin set under $BENDG_DATA (bend2/FORMAT.md), prints `A x y`, `B x0 x1 y0 y1`,
// `C x y` (canonical big-endian 0x hex) and the `T <phase> <ms>` lines of
// bend2/prove.bend:154-162.  $BENDG_GPU is accepted for compatibility; every phase runs on
// the GPU.  $BG_DEVICE selects the CUDA device (default 0).  Exit status 1 on any error.
#include <cstdio>
#include <cstdlib>

#include "../../include/bg.h"

int main(int argc, char** argv) {
  const char* dir = getenv("BENDG_DATA");
  if (!dir) {
    fprintf(stderr, "prove_bin: BENDG_DATA is not set\n");
    return 1;
  }
  (void)argc;
  (void)argv;
  const char* dev = getenv("BG_DEVICE");
  bg_ctx* ctx = nullptr;
  int st = bg_ctx_create(dev ? atoi(dev) : 0, &ctx);
  if (st != BG_OK) {
    fprintf(stderr, "prove_bin: %s: %s\n", bg_strerror(st), bg_last_error(nullptr));
    return 1;
  }
  bg_proof proof;
  bg_phase_ms t;
  st = bg_prove_dir(ctx, dir, &proof, &t);
  if (st != BG_OK) {
    fprintf(stderr, "prove_bin: %s: %s\n", bg_strerror(st), bg_last_error(ctx));
    bg_ctx_destroy(ctx);
    return 1;
  }
  char buf[1024];
  bg_proof_format(&proof, buf, sizeof buf);
  fputs(buf, stdout);
  const char* names[9] = {"load", "evals", "qap", "msm_a", "msm_b1", "msm_b2", "msm_h", "msm_l", "total"};
  const double vals[9] = {t.load, t.evals, t.qap, t.msm_a, t.msm_b1, t.msm_b2, t.msm_h, t.msm_l, t.total};
  for (int i = 0; i < 9; i++) printf("T %s %lld\n", names[i], (long long)(vals[i] + 0.5));
  bg_ctx_destroy(ctx);
  return 0;
}
