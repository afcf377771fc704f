// Element-wise primitive kernels (see prims.cu)
#pragma once
#include "common.cuh"

namespace bg {

void wire_to_packed(cudaStream_t st, const uint32_t* d_wire, uint32_t* d_packed, size_t n, uint32_t* d_status);
void packed_to_wire(cudaStream_t st, const uint32_t* d_packed, uint32_t* d_wire, size_t n);
void fr_from_mont(cudaStream_t st, const uint32_t* d_in, uint32_t* d_out, size_t n);
void field_op(cudaStream_t st, int field, int op, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t n);
void curve_op(cudaStream_t st, int curve, int op, const uint32_t* p, const uint32_t* q, const uint32_t* k,
              uint32_t* out, size_t n);
void imad_probe(cudaStream_t st, int blocks, int threads, uint32_t iters, uint32_t* sink, int which);

}  // namespace bg
