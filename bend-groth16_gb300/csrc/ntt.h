// NTT / QAP interface (see ntt.cu)
#pragma once
#include "common.cuh"

namespace bg {

NttTables& ntt_tables(Ctx& ctx, int L);
// in-place transform of 2^L packed Fr, natural order in and out; mode = BG_NTT_*
void ntt_run(Ctx& ctx, cudaStream_t st, uint32_t* d_data, int L, int mode);
// h from evaluation vectors a, b, c (overwritten); d_h receives 2^L coefficients
void qap_h_run(Ctx& ctx, cudaStream_t st, uint32_t* d_a, uint32_t* d_b, uint32_t* d_c, uint32_t* d_h, int L);

}  // namespace bg
