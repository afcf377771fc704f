/* bg.h - C ABI of the GB300 Groth16/BN254 prover core.
 *
 * Drop-in boundary for the GPU seam of the bend-groth16 prover (bend2/prove.bend:21-49):
 *   Pr.g1_run(gpu, pts, scs, n) -> G1 Jacobian      => bg_msm_g1
 *   Pr.g2_run(gpu, pts, scs, n) -> G2 Jacobian      => bg_msm_g2
 *   Pr.qap_run(gpu, a, b, c, lg) -> h               => bg_qap_h
 * and for the whole prover process Pr.run (bend2/prove.bend:129-162)      => bg_prove_dir.
 *
 * Host buffers use the frozen wire layout of bend2/FORMAT.md:5-20: one field element is
 * 16 little-endian u32 words, each holding one 16-bit limb; Fq/Fr values are in Montgomery
 * form with R = 2^256 except MSM scalars, which are canonical (bend2/src/msm.bend:3-5).
 * G1 affine = x, y (32 words); G2 affine = x.c0, x.c1, y.c0, y.c1 (64 words); the point at
 * infinity is all-zero words.  Functions whose names end in _dev take device pointers in the
 * packed layout (8 x u32 limbs per element, same Montgomery convention); those pointers (and
 * bg_msm_g1_noalloc's) must be 16-byte aligned, as cudaMalloc's are (BG_E_ARG otherwise).
 *
 * Errors: every entry point returns 0 (BG_OK) or a BG_E_* status and never aborts; the
 * reference has no error channel on this path (an OOM ends the Bend process,
 * docs/bend2-idioms.md:99), so the statuses are new.  bg_last_error() gives the message.
 * Threading: a bg_ctx serialises its calls on its own CUDA stream; use one context per host
 * thread for concurrency.  The caller owns host buffers, the context owns device memory.
 */
#ifndef BG_H
#define BG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  BG_OK = 0,
  BG_E_ARG = 1,     /* bad argument (size, layout, scalar >= 2^254, ...) */
  BG_E_OOM = 2,     /* device or pinned allocation failed */
  BG_E_FORMAT = 3,  /* a .bin file disagrees with bend2/FORMAT.md or with header.bin */
  BG_E_TIMEOUT = 4, /* a bounded device wait gave up */
  BG_E_DEVICE = 5,  /* CUDA runtime error */
  BG_E_IO = 6       /* file could not be read */
};

/* NTT modes: Ntt.fft / ifft / coset_fft and the coset inverse (bend2/src/ntt.bend:431-438,
 * bend2/gen/ref_qap.py:27-65) */
enum { BG_NTT_FORWARD = 0, BG_NTT_INVERSE = 1, BG_NTT_COSET_FORWARD = 2, BG_NTT_COSET_INVERSE = 3 };

/* field / curve selectors for the primitive vector entry points */
enum { BG_FIELD_FR = 0, BG_FIELD_FQ = 1 };
enum { BG_FOP_ADD = 0, BG_FOP_SUB = 1, BG_FOP_MUL = 2, BG_FOP_NEG = 3, BG_FOP_INV = 4, BG_FOP_SQR = 5,
       BG_FOP_TO_MONT = 6, BG_FOP_FROM_MONT = 7 };
enum { BG_CURVE_G1 = 0, BG_CURVE_G2 = 1 };
enum { BG_COP_ADD = 0, BG_COP_DOUBLE = 1, BG_COP_NEG = 2, BG_COP_MUL = 3 };

typedef struct bg_ctx bg_ctx;
typedef struct bg_pk bg_pk;

/* A proof as the prover prints it, before hex formatting: affine, Montgomery, wire layout
 * (Out{a, b, c} of bend2/src/groth16.bend:24-25). */
typedef struct {
  uint32_t a[32];
  uint32_t b[64];
  uint32_t c[32];
} bg_proof;

/* Phase wall times in ms, the `T <phase> <ms>` lines of bend2/prove.bend:154-162 */
typedef struct {
  double load, evals, qap, msm_a, msm_b1, msm_b2, msm_h, msm_l, total;
} bg_phase_ms;

/* The contents of the twelve .bin files of one data/<K>/bend directory (bend2/FORMAT.md:15-23),
 * already in host memory; `*_bytes` are the file sizes. */
typedef struct {
  const void* header; size_t header_bytes;
  const void* witness; size_t witness_bytes;
  const void* r1cs_a; size_t r1cs_a_bytes;
  const void* r1cs_b; size_t r1cs_b_bytes;
  const void* r1cs_c; size_t r1cs_c_bytes;
  const void* pk_g1; size_t pk_g1_bytes;
  const void* pk_g2; size_t pk_g2_bytes;
  const void* pk_a; size_t pk_a_bytes;
  const void* pk_b1; size_t pk_b1_bytes;
  const void* pk_b2; size_t pk_b2_bytes;
  const void* pk_h; size_t pk_h_bytes;
  const void* pk_l; size_t pk_l_bytes;
  const void* rs; size_t rs_bytes;
} bg_inputs;

/* ---- context ---------------------------------------------------------------------- */
int bg_ctx_create(int device, bg_ctx** out);
void bg_ctx_destroy(bg_ctx* ctx);
const char* bg_strerror(int status);
const char* bg_last_error(const bg_ctx* ctx);
/* the cudaStream_t every launch of this context is ordered on */
void* bg_ctx_stream(bg_ctx* ctx);
/* kernels launched by this context since creation (all of them are this library's own) */
uint64_t bg_ctx_launches(const bg_ctx* ctx);
/* pinned host memory for fast host<->device copies */
int bg_host_alloc(size_t bytes, void** out);
void bg_host_free(void* p);

/* ---- the GPU seam (bend2/prove.bend:21-49) ------------------------------------------
 * bg_msm_g1 replaces Pr.g1_run -> Msm.g1 (bend2/prove.bend:24-29, bend2/src/msm.bend:297):
 * sum_{i<n} scalars[i] * points[i] over G1.  points16: n affine G1 (32 words each);
 * scalars16: n canonical Fr (16 words each, each < 2^254).  out_jac16 receives the sum as a
 * Jacobian point (x, y, z: 48 words, Montgomery) with z = 1, or (0, 1, 0) for infinity
 * (G1.infinity, bend2/src/g1.bend:16-17). */
int bg_msm_g1(bg_ctx* ctx, const uint32_t* points16, const uint32_t* scalars16, size_t n, uint32_t* out_jac16);
/* bg_msm_g2 replaces Pr.g2_run -> Msm.g2 (bend2/prove.bend:34-39, bend2/src/msm.bend:529);
 * points16: n affine G2 (64 words each); out_jac16: 96 words. */
int bg_msm_g2(bg_ctx* ctx, const uint32_t* points16, const uint32_t* scalars16, size_t n, uint32_t* out_jac16);
/* bg_qap_h replaces Pr.qap_run -> Ntt.qap_h (bend2/prove.bend:44-49, bend2/src/ntt.bend:459):
 * a, b, c: 2^log2d Fr (Montgomery) evaluation vectors; h16 receives 2^log2d Fr (Montgomery),
 * the coefficients of h(x) (the last one is 0 when the R1CS is satisfied). */
int bg_qap_h(bg_ctx* ctx, const uint32_t* a16, const uint32_t* b16, const uint32_t* c16, uint32_t log2d,
             uint32_t* h16);

/* ---- whole proofs ------------------------------------------------------------------ */
/* Pr.run (bend2/prove.bend:129-162) on the .bin files under dir (what $BENDG_DATA names). */
int bg_prove_dir(bg_ctx* ctx, const char* dir, bg_proof* out, bg_phase_ms* times);
/* The same proof from file contents already in host memory (every file copied to the device). */
int bg_prove_host(bg_ctx* ctx, const bg_inputs* in, bg_proof* out, bg_phase_ms* times);
/* Device-resident proving key: header, R1CS and the pk_*.bin points stay in HBM (packed). */
int bg_pk_upload(bg_ctx* ctx, const bg_inputs* in, bg_pk** out);
void bg_pk_release(bg_pk* pk);
/* A proof against a resident key; witness16 / rs16 are host buffers (witness.bin, rs.bin). */
int bg_prove_resident(bg_ctx* ctx, bg_pk* pk, const uint32_t* witness16, const uint32_t* rs16, bg_proof* out,
                      bg_phase_ms* times);
/* Many proofs at once against resident keys (no counterpart in the reference, which proves one
 * proof per process): `lanes` concurrent provers (1..32, each with its own streams and
 * workspace) take the proofs largest domain first; small proofs share the GPU instead of
 * leaving it idle.  out[i], times[i] (times may be NULL) and statuses[i] belong to proof i;
 * every result is bit-identical to the same proof made alone. */
int bg_prove_batch(bg_ctx* ctx, bg_pk* const* pks, const uint32_t* const* witnesses16, const uint32_t* const* rs16,
                   size_t count, int lanes, bg_proof* out, bg_phase_ms* times, int* statuses);
/* Device bytes of scratch one proof against `pk` needs (admission control, capacity planning). */
size_t bg_prove_footprint(const bg_pk* pk);

/* Serving loop (no counterpart in the reference): `lanes` provers (1..32) take prove requests
 * from one FIFO queue; the head request starts when a lane is free and the lanes' reserved
 * scratch stays within hbm_budget_bytes, so requests that arrive while others prove are
 * admitted as lanes and memory free up and run concurrently (continuous batching).  A request
 * whose footprint exceeds the budget is refused with BG_E_OOM.  witness16 / rs16 must stay
 * valid until the request completes.  bg_server_wait returns one completed request (BG_OK) or
 * BG_E_TIMEOUT; latency_ms is submit -> result, queue_ms submit -> start.  Destroying the
 * server finishes requests in flight and drops queued ones.  Keys must belong to ctx. */
typedef struct bg_server bg_server;
int bg_server_create(bg_ctx* ctx, int lanes, size_t hbm_budget_bytes, bg_server** out);
int bg_server_submit(bg_server* server, bg_pk* pk, const uint32_t* witness16, const uint32_t* rs16, uint64_t tag);
int bg_server_wait(bg_server* server, int timeout_ms, uint64_t* tag, bg_proof* out, bg_phase_ms* times,
                   double* latency_ms, double* queue_ms, int* status);
size_t bg_server_reserved_bytes(bg_server* server);
void bg_server_destroy(bg_server* server);
/* ---- verification (the role of groth16-ref verify, ref/src/verify.rs:8-27) ------------- */
/* Groth16 verifying key in the wire layout of the .bin files (16-bit limbs in u32 words,
 * Montgomery coordinates, (0, 0) = infinity): alpha_g1 (32 words), beta_g2, gamma_g2,
 * delta_g2 (64 words each), gamma_abc_g1 (n_ic x 32 words, n_ic = public inputs + 1).  The
 * reference keeps it in vk.json; the .bin set has no vk file. */
typedef struct bg_vk {
  const uint32_t* alpha_g1;
  const uint32_t* beta_g2;
  const uint32_t* gamma_g2;
  const uint32_t* delta_g2;
  const uint32_t* gamma_abc_g1;
  size_t n_ic;
} bg_vk;
/* *valid = 1 when e(A, B) = e(alpha, beta) e(vk_x, gamma) e(C, delta), vk_x = IC_0 +
 * sum_i x_i IC_i; 0 when the equation fails (a wrong proof of valid points, C at infinity
 * included).  Inputs that cannot be decoded -- a point off its curve or B outside the order-r
 * subgroup, a wire word above 16 bits, a public input not below r -- return BG_E_FORMAT with
 * *valid = 0, as the reference's verifier errors on them (ref/src/verify.rs:9-26, :47-49).
 * public16: n_public Fr elements (wire layout, Montgomery; x_1.. of z), n_public = n_ic - 1
 * (BG_E_ARG otherwise).  Host only (optimal ate pairing on the CPU, a few ms); needs no
 * context or GPU. */
int bg_verify(const bg_vk* vk, const uint32_t* public16, size_t n_public, const bg_proof* proof, int* valid);
/* e(P, Q) for P in G1 (32 words) and Q in G2 (64 words), wire layout, written as 12 Fq elements
 * (192 words) in tower order (Fq12 = Fq6[w]/(w^2 - v), Fq6 = Fq2[v]/(v^3 - (9 + u)));
 * BG_E_ARG for points off their curve or outside the order-r subgroup.  Host only. */
int bg_pairing(const uint32_t* p32, const uint32_t* q64, uint32_t* out192);

/* Proof line text exactly as the reference prints it: "A x y\nB x0 x1 y0 y1\nC x y\n"
 * (canonical big-endian 0x + 64 hex digits, bend2/FORMAT.md:33).  buf needs >= 600 bytes. */
int bg_proof_format(const bg_proof* proof, char* buf, size_t buf_bytes);

/* ---- primitives (parity tests, standalone benchmarks) ------------------------------ */
/* In-place NTT of 2^log2n Fr (Montgomery, wire layout), natural order in and out. */
int bg_ntt(bg_ctx* ctx, uint32_t* data16, uint32_t log2n, int mode);
/* Element-wise field op over n elements: out = op(a, b); unary ops ignore b.  TO_MONT and
 * FROM_MONT convert canonical <-> Montgomery; all others work on Montgomery values. */
int bg_field_op(bg_ctx* ctx, int field, int op, const uint32_t* a16, const uint32_t* b16, uint32_t* out16, size_t n);
/* Element-wise curve op over n affine points: ADD(p, q), DOUBLE(p), NEG(p), MUL(p, k) with k
 * canonical Fr (16 words); results affine in wire layout. */
int bg_curve_op(bg_ctx* ctx, int curve, int op, const uint32_t* p16, const uint32_t* q16, const uint32_t* k16,
                uint32_t* out16, size_t n);

/* Packed device-resident variants: points (16 / 32 words per G1 / G2 point), scalars
 * (8 words each), results affine packed (16 / 32 words) on the host. */
int bg_msm_g1_dev(bg_ctx* ctx, const uint32_t* d_points, const uint32_t* d_scalars, size_t n, uint32_t* out_aff32);
int bg_msm_g2_dev(bg_ctx* ctx, const uint32_t* d_points, const uint32_t* d_scalars, size_t n, uint32_t* out_aff32);
/* G1 MSM that allocates nothing (no counterpart in the reference).  For callers that may not
 * allocate device memory: a program whose GPU memory is all taken by its own pool, or a
 * latency-critical loop that cannot afford the device synchronisation cudaMalloc and cudaFree
 * imply.  Same inputs and result as bg_msm_g1_dev (device pointers to packed points and
 * canonical scalars, affine result in 16 host words) but no context: scratch is a fixed
 * 9 MiB array inside the library, held by every GPU that loads it until the process exits.
 * n <= 16384 (larger n returns BG_E_ARG).  `stream` is a cudaStream_t or NULL.  All calls
 * share the array (each clears what must start at zero); calls from one process are
 * serialised and the function returns when its work is done, and calls that overlapped on the
 * GPU would race.  The first call on a device looks up the array's address on the current
 * device.  Every call synchronises `stream` and copies to pageable host memory, so it must not
 * be called while that stream is being captured.  Errors: bg_last_error(NULL). */
int bg_msm_g1_noalloc(const uint32_t* d_points, const uint32_t* d_scalars, size_t n, void* stream,
                      uint32_t* out_aff32);
int bg_ntt_dev(bg_ctx* ctx, uint32_t* d_data, uint32_t log2n, int mode);
/* wire layout <-> packed layout for n elements (16 words -> 8 words), device pointers */
int bg_repack_to_packed_dev(bg_ctx* ctx, const uint32_t* d_wire, uint32_t* d_packed, size_t n_elems);
int bg_repack_to_wire_dev(bg_ctx* ctx, const uint32_t* d_packed, uint32_t* d_wire, size_t n_elems);

/* Seeded synthetic SquareChain(2^log2n) instance in bend2/FORMAT.md files (header, witness,
 * R1CS, proving key from a known-trapdoor setup, r and s) written under dir.  The G1/G2
 * fixed-base multiplications run on the device.  Produces inputs only; not part of proving. */
int bg_synth_square_chain(bg_ctx* ctx, uint32_t log2n, uint64_t seed, const char* dir);

/* Window width c the MSM picks for n points of `curve` (BG_CURVE_G1/G2) with one bucket set
 * per window: the committed tuning table (bend-groth16_gb300/csrc/msm_tune.h), else a size rule. */
int bg_msm_window_bits(size_t n, int curve);
/* Window width c of the window tables a resident key (bg_pk_upload) builds for a query set of
 * n points: one shared bucket set of 2^(c-1) buckets, floor(254 / c) + 1 table rows. */
int bg_msm_table_window_bits(size_t n, int curve);
/* Window width c of a bucket-set-per-window MSM of n points inside a proof whose key has no
 * window tables (bg_prove_dir, bg_prove_host): tuned on whole proofs, where the MSMs share the
 * GPU with each other's reductions and the QAP; else bg_msm_window_bits. */
int bg_msm_proof_window_bits(size_t n, int curve);
/* Tuning hook: force the window width of later MSMs of this context, layout 0 = one bucket set
 * per window (bg_msm_* and the MSMs of proofs without window tables), 1 = window tables of keys
 * uploaded afterwards; c = 0 restores the library's choice, else 2..22. */
int bg_msm_window_override(bg_ctx* ctx, int layout, int curve, int c);
/* Batch-affine pair rounds the library's cost model takes for a standalone MSM of n points of
 * `curve` (bg_msm_g1/g2 and their _dev forms): 2 for G1 MSMs of at least 2^23 entries with at
 * least 32 per bucket, else 0 (measured slower there on GB300). */
int bg_msm_pair_rounds(size_t n, int curve);
/* Tuning hook: the number of batch-affine pair rounds before each later MSM's bucket
 * accumulation on this context and its batch lanes (each round adds the points of every bucket
 * in pairs, in affine coordinates, sharing one field inversion per CTA); -1 restores the
 * library's cost model, 0 turns the rounds off, at most 12.  Results do not depend on it. */
int bg_msm_pair_rounds_override(bg_ctx* ctx, int rounds);
/* Tuning hook: the window reductions that end a critical path (standalone MSMs, a proof's last
 * MSM, every MSM of a small proof) may run each point addition on a group of 8 cooperating
 * lanes; mode -1 lets the library's latency model choose (the default), 0 never, 1 always
 * (for those reductions).  Results do not depend on it. */
int bg_msm_coop_reduce_override(bg_ctx* ctx, int mode);

/* ---- measurement (no counterpart in the reference, which prints only T lines) ------- */
/* Enable (1) / disable (0) CUDA-event timing of the library's main kernels on the streams
 * they run on; enabling clears earlier statistics. */
int bg_ctx_profile(bg_ctx* ctx, int enable);
/* Launch count and summed device time (ms) of one kernel family since profiling was enabled:
 * "msm_bucket_acc_g1", "msm_bucket_acc_g2", "msm_heavy_g1", "msm_heavy_g2", "msm_reduce_g1",
 * "msm_reduce_g2", "msm_digits", "msm_scatter", "ntt_pass", "evals", "qap".  Unknown names report
 * zero launches. */
int bg_ctx_kernel_stats(bg_ctx* ctx, const char* name, uint64_t* launches, double* total_ms);
/* Host <-> device bytes the context (and its batch lanes) copied since it was created: every
 * upload of host data (files, witnesses, randomness, tables) and every download (MSM window
 * sums, status words, results). */
int bg_ctx_transfer_bytes(bg_ctx* ctx, uint64_t* h2d, uint64_t* d2h);
/* Launch timeline: enable = 1 clears and starts recording the start and end of every timed
 * launch (the families above plus the proof phases); enable = 0 stops and writes one line
 * "family start_ms end_ms" per launch, in issue order, times relative to the first recorded
 * start, into buf (NUL-terminated; BG_E_ARG when cap is too small). */
int bg_ctx_timeline(bg_ctx* ctx, int enable, char* buf, size_t cap);
/* Integer multiply-add throughput probe: which = 0 raw 32-bit mad.lo/mad.hi chains (50/50),
 * 1 Fq Montgomery products, 2 mad.lo only, 3 mad.hi only, 4 mad.wide.u32 only.  Returns the
 * operations executed (instructions, or Fq products for 1) and the kernel time in ms. */
int bg_probe_imad(bg_ctx* ctx, int which, uint32_t iters, double* ops, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* BG_H */
