// Prover pipeline interface (see prove.cu)
#pragma once
#include "common.cuh"
#include "host_ff.hpp"
#include "msm.h"

namespace bg {

// header.bin (bend2/FORMAT.md:16; bend2/src/groth16.bend:13-14)
struct Header {
  uint32_t nc, ni, nw, lg, na, nb, nh, nl;
};

struct CsrDev {
  uint32_t nnz = 0;
  uint32_t* offs = nullptr;    // nc + 1 row offsets
  uint32_t* cols = nullptr;    // nnz column indexes
  uint32_t* coeffs = nullptr;  // nnz packed Fr coefficients (Montgomery)
};

// device-resident proving key + circuit
struct PkDev {
  Header h{};
  uint32_t *pa = nullptr, *pb1 = nullptr, *pb2 = nullptr, *ph = nullptr, *pl = nullptr;  // packed affine
  CsrDev ca, cb, cc;
  bgh::Aff<bgh::FqOps> alpha, beta, delta;
  bgh::Aff<bgh::Fq2Ops> beta2, delta2;
  // resident keys: 2^(64 j) delta and 2^(64 j) delta2 (j < 4), so that each host product of a
  // delta point by r, s or r s splits into four independent 64-bit pieces
  bool delta_pow_ready = false;
  bgh::Xyzz<bgh::FqOps> delta_pow[4];
  bgh::Xyzz<bgh::Fq2Ops> delta2_pow[4];
  // window tables of the five query sets (a, b1, b2, h, l), built for resident keys
  MsmTable tab[5];
  bool tables = false;
  // one-shot keys (pk_stage_oneshot): buffers borrowed from the context's workspace, and the
  // points of each query set (a, b1, b2, h, l) still arriving on the copy stream until ready[i]
  bool pooled = false;
  cudaEvent_t ready[5] = {};
  // one-shot keys: the R1CS matrices arrive on the copy stream too, after the first query sets
  cudaEvent_t csr_ready = nullptr;
};

Header parse_header(const bg_inputs& in);
void validate_inputs(const bg_inputs& in, const Header& h, bool need_witness);
// with build_tables, each query set also gets its 2^(c w) window table (resident keys proving
// many proofs; a one-shot proof skips them)
PkDev* pk_upload(Ctx& ctx, const bg_inputs& in, bool build_tables);
// key of a single proof: CSR and constants uploaded before it returns; the query sets are
// enqueued on the context's copy stream (ready events in the key) so that the proof's
// evaluations and QAP overlap their transfer; buffers come from the context's workspace
PkDev* pk_stage_oneshot(Ctx& ctx, const bg_inputs& in);
void pk_free(PkDev* pk);
void check_status(Ctx& ctx, cudaStream_t st);
void prove_resident(Ctx& ctx, PkDev& pk, const uint32_t* witness16, const uint32_t* rs16, bg_proof* out,
                    bg_phase_ms* times, double load_ms_before);
int format_proof(const bg_proof* p, char* buf, size_t cap);
// device bytes of scratch one proof against a key with this header needs
size_t prove_footprint(const Header& h);

// serving loop (server.cu)
class Server;
Server* server_create(int device, int lanes, size_t budget);
void server_destroy(Server* s);
void server_submit(Server* s, PkDev* pk, const uint32_t* w, const uint32_t* rs, uint64_t tag);
bool server_wait(Server* s, int timeout_ms, uint64_t* tag, bg_proof* out, bg_phase_ms* times, double* latency_ms,
                 double* queue_ms, int* status);
size_t server_reserved(Server* s);

}  // namespace bg
