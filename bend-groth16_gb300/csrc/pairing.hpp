// Groth16 verification on the host: the optimal ate pairing over BN254 (see pairing.cpp).
#pragma once
#include <cstddef>
#include <cstdint>
#include <stdexcept>

namespace bgh {

// Groth16 verifying key and proof in the wire layout of the .bin files (16-bit limbs in u32
// words, Montgomery coordinates, (0, 0) = infinity).
struct VkWire {
  const uint32_t* alpha_g1;      // 32 words
  const uint32_t* beta_g2;       // 64 words
  const uint32_t* gamma_g2;      // 64 words
  const uint32_t* delta_g2;      // 64 words
  const uint32_t* gamma_abc_g1;  // n_ic x 32 words
  size_t n_ic;                   // public inputs + 1
};

// A point off its curve or outside the order-r subgroup, a wire word above 16 bits or a public
// input not below r: an input that cannot be decoded, which the reference's verifier reports as
// an error rather than a rejection (ref/src/verify.rs:9-26, its test at :47-49).
struct MalformedInput : std::invalid_argument {
  using std::invalid_argument::invalid_argument;
};

// 1: e(A, B) = e(alpha, beta) e(sum_i x_i IC_i, gamma) e(C, delta) with x_0 = 1 and
// x_1.. = public16 (n_ic - 1 Fr elements, wire layout, Montgomery); 0: the equation fails.
// Throws MalformedInput for undecodable points or inputs, std::invalid_argument on malformed
// sizes.
int groth16_verify(const VkWire& vk, const uint32_t* public16, size_t n_public, const uint32_t* a32,
                   const uint32_t* b64, const uint32_t* c32);

// e(P, Q) for affine P in G1 and Q in G2 (wire layout), as 12 Fq elements (Montgomery, 16-bit
// limb wire layout, 192 words) in the tower order c0.c0.c0, c0.c0.c1, c0.c1.c0, ... (Fq12 =
// Fq6[w]/(w^2 - v), Fq6 = Fq2[v]/(v^3 - (9 + u))).  For tests of bilinearity.
void pairing_wire(const uint32_t* p32, const uint32_t* q64, uint32_t* out192);

}  // namespace bgh
