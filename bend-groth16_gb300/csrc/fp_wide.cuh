// 512-bit products without reduction, and one Montgomery reduction for a whole sum of
// products ("lazy reduction").  A CIOS product spends half of its 264 multiply-adds on the
// reduction (8 rows x 17); when a formula needs a +- b c +- d e, computing the two 16-limb
// products, combining them and reducing once saves one reduction, and the Fq2 Karatsuba product
// (three Fq products, two reductions instead of three) saves one of every six.  The 16-limb
// product itself is one level of Karatsuba over 128-bit halves (96 multiply-adds instead of
// 128), and a square computes its 28 off-diagonal limb products once and doubles them (72).
// The high half of a 32-bit product issues at half the rate of the low half on this GPU, so
// these counts are what bounds the MSM accumulation.  Bounds: every value reduced here is below p R (R = 2^256), so the reduction returns
// a value below 2p that one conditional subtraction brings below p; combinations add 2 p^2
// before subtracting, which keeps them non-negative and below 4 p^2 < p R (4p < 2^256 for the
// BN254 base field).
//
// The chains are written out limb by limb: each asm block is one carry chain.  The host test
// tests/device_emul.py executes these chains instruction by instruction on the CPU.
#pragma once
// included at the end of fp.cuh (needs Fp, Fq, Fq2 and reduce_once)

namespace bg {

struct Wide {
  uint32_t v[16];
};

// t = a b by one level of Karatsuba on 128-bit halves: a0 b0, a1 b1 and (a0 + a1)(b0 + b1)
// (three 4 x 4 limb products, 48 multiply-add pairs instead of 64); the half sums carry one
// bit each, added back as shifted copies of the other sum.
BG_DEV void wide_mul(Wide& t, const uint32_t* a, const uint32_t* b) {
  uint32_t p0[8], p2[8], p1[9], sa[4], sb[4], ca, cb;
#pragma unroll
  for (int i = 0; i < 8; i++) p0[i] = p2[i] = p1[i] = 0;
  p1[8] = 0;
  asm("add.cc.u32     %0, %5, %9;\n\t"
      "addc.cc.u32    %1, %6, %10;\n\t"
      "addc.cc.u32    %2, %7, %11;\n\t"
      "addc.cc.u32    %3, %8, %12;\n\t"
      "addc.u32       %4, 0, 0;"
      : "=r"(sa[0]), "=r"(sa[1]), "=r"(sa[2]), "=r"(sa[3]), "=r"(ca)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("add.cc.u32     %0, %5, %9;\n\t"
      "addc.cc.u32    %1, %6, %10;\n\t"
      "addc.cc.u32    %2, %7, %11;\n\t"
      "addc.cc.u32    %3, %8, %12;\n\t"
      "addc.u32       %4, 0, 0;"
      : "=r"(sb[0]), "=r"(sb[1]), "=r"(sb[2]), "=r"(sb[3]), "=r"(cb)
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p0[0]), "+r"(p0[1]), "+r"(p0[2]), "+r"(p0[3]), "+r"(p0[4])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p0[1]), "+r"(p0[2]), "+r"(p0[3]), "+r"(p0[4]), "+r"(p0[5])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[1]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p0[2]), "+r"(p0[3]), "+r"(p0[4]), "+r"(p0[5]), "+r"(p0[6])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[2]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p0[3]), "+r"(p0[4]), "+r"(p0[5]), "+r"(p0[6]), "+r"(p0[7])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[3]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p2[0]), "+r"(p2[1]), "+r"(p2[2]), "+r"(p2[3]), "+r"(p2[4])
      : "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[4]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p2[1]), "+r"(p2[2]), "+r"(p2[3]), "+r"(p2[4]), "+r"(p2[5])
      : "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[5]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p2[2]), "+r"(p2[3]), "+r"(p2[4]), "+r"(p2[5]), "+r"(p2[6])
      : "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[6]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p2[3]), "+r"(p2[4]), "+r"(p2[5]), "+r"(p2[6]), "+r"(p2[7])
      : "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[7]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p1[0]), "+r"(p1[1]), "+r"(p1[2]), "+r"(p1[3]), "+r"(p1[4])
      : "r"(sa[0]), "r"(sa[1]), "r"(sa[2]), "r"(sa[3]), "r"(sb[0]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p1[1]), "+r"(p1[2]), "+r"(p1[3]), "+r"(p1[4]), "+r"(p1[5])
      : "r"(sa[0]), "r"(sa[1]), "r"(sa[2]), "r"(sa[3]), "r"(sb[1]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p1[2]), "+r"(p1[3]), "+r"(p1[4]), "+r"(p1[5]), "+r"(p1[6])
      : "r"(sa[0]), "r"(sa[1]), "r"(sa[2]), "r"(sa[3]), "r"(sb[2]));
  asm("mad.lo.cc.u32  %0, %5, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %9, %3;\n\t"
      "madc.hi.u32    %4, %8, %9, %4;"
      : "+r"(p1[3]), "+r"(p1[4]), "+r"(p1[5]), "+r"(p1[6]), "+r"(p1[7])
      : "r"(sa[0]), "r"(sa[1]), "r"(sa[2]), "r"(sa[3]), "r"(sb[3]));
  {
    const uint32_t ma = 0u - ca, mb = 0u - cb;
    const uint32_t x0 = sb[0] & ma, x1 = sb[1] & ma, x2 = sb[2] & ma, x3 = sb[3] & ma;
    const uint32_t y0 = sa[0] & mb, y1 = sa[1] & mb, y2 = sa[2] & mb, y3 = sa[3] & mb;
  asm("add.cc.u32     %0, %0, %6;\n\t"
      "addc.cc.u32    %1, %1, %7;\n\t"
      "addc.cc.u32    %2, %2, %8;\n\t"
      "addc.cc.u32    %3, %3, %9;\n\t"
      "addc.u32       %4, %4, %14;\n\t"
      "add.cc.u32     %0, %0, %10;\n\t"
      "addc.cc.u32    %1, %1, %11;\n\t"
      "addc.cc.u32    %2, %2, %12;\n\t"
      "addc.cc.u32    %3, %3, %13;\n\t"
      "addc.u32       %4, %4, 0;"
      : "+r"(p1[4]), "+r"(p1[5]), "+r"(p1[6]), "+r"(p1[7]), "+r"(p1[8])
      : "r"(0u), "r"(x0), "r"(x1), "r"(x2), "r"(x3), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(ca & cb));
  }
  asm("sub.cc.u32     %0, %0, %9;\n\t"
      "subc.cc.u32    %1, %1, %10;\n\t"
      "subc.cc.u32    %2, %2, %11;\n\t"
      "subc.cc.u32    %3, %3, %12;\n\t"
      "subc.cc.u32    %4, %4, %13;\n\t"
      "subc.cc.u32    %5, %5, %14;\n\t"
      "subc.cc.u32    %6, %6, %15;\n\t"
      "subc.cc.u32    %7, %7, %16;\n\t"
      "subc.u32       %8, %8, 0;"
      : "+r"(p1[0]), "+r"(p1[1]), "+r"(p1[2]), "+r"(p1[3]), "+r"(p1[4]), "+r"(p1[5]), "+r"(p1[6]), "+r"(p1[7]), "+r"(p1[8])
      : "r"(p0[0]), "r"(p0[1]), "r"(p0[2]), "r"(p0[3]), "r"(p0[4]), "r"(p0[5]), "r"(p0[6]), "r"(p0[7]));
  asm("sub.cc.u32     %0, %0, %9;\n\t"
      "subc.cc.u32    %1, %1, %10;\n\t"
      "subc.cc.u32    %2, %2, %11;\n\t"
      "subc.cc.u32    %3, %3, %12;\n\t"
      "subc.cc.u32    %4, %4, %13;\n\t"
      "subc.cc.u32    %5, %5, %14;\n\t"
      "subc.cc.u32    %6, %6, %15;\n\t"
      "subc.cc.u32    %7, %7, %16;\n\t"
      "subc.u32       %8, %8, 0;"
      : "+r"(p1[0]), "+r"(p1[1]), "+r"(p1[2]), "+r"(p1[3]), "+r"(p1[4]), "+r"(p1[5]), "+r"(p1[6]), "+r"(p1[7]), "+r"(p1[8])
      : "r"(p2[0]), "r"(p2[1]), "r"(p2[2]), "r"(p2[3]), "r"(p2[4]), "r"(p2[5]), "r"(p2[6]), "r"(p2[7]));
#pragma unroll
  for (int i = 0; i < 8; i++) {
    t.v[i] = p0[i];
    t.v[8 + i] = p2[i];
  }
  asm("add.cc.u32     %0, %0, %12;\n\t"
      "addc.cc.u32    %1, %1, %13;\n\t"
      "addc.cc.u32    %2, %2, %14;\n\t"
      "addc.cc.u32    %3, %3, %15;\n\t"
      "addc.cc.u32    %4, %4, %16;\n\t"
      "addc.cc.u32    %5, %5, %17;\n\t"
      "addc.cc.u32    %6, %6, %18;\n\t"
      "addc.cc.u32    %7, %7, %19;\n\t"
      "addc.cc.u32    %8, %8, %20;\n\t"
      "addc.cc.u32    %9, %9, 0;\n\t"
      "addc.cc.u32    %10, %10, 0;\n\t"
      "addc.u32       %11, %11, 0;"
      : "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15])
      : "r"(p1[0]), "r"(p1[1]), "r"(p1[2]), "r"(p1[3]), "r"(p1[4]), "r"(p1[5]), "r"(p1[6]), "r"(p1[7]), "r"(p1[8]));
}

// t = a^2: off-diagonal products once, doubled, plus the diagonal
BG_DEV void wide_sqr(Wide& t, const uint32_t* a) {
#pragma unroll
  for (int i = 0; i < 16; i++) t.v[i] = 0;
  asm("mad.lo.cc.u32  %0, %8, %9, %0;\n\t"
      "madc.lo.cc.u32 %1, %8, %10, %1;\n\t"
      "madc.lo.cc.u32 %2, %8, %11, %2;\n\t"
      "madc.lo.cc.u32 %3, %8, %12, %3;\n\t"
      "madc.lo.cc.u32 %4, %8, %13, %4;\n\t"
      "madc.lo.cc.u32 %5, %8, %14, %5;\n\t"
      "madc.lo.cc.u32 %6, %8, %15, %6;\n\t"
      "addc.u32       %7, %7, 0;\n\t"
      "mad.hi.cc.u32  %1, %8, %9, %1;\n\t"
      "madc.hi.cc.u32 %2, %8, %10, %2;\n\t"
      "madc.hi.cc.u32 %3, %8, %11, %3;\n\t"
      "madc.hi.cc.u32 %4, %8, %12, %4;\n\t"
      "madc.hi.cc.u32 %5, %8, %13, %5;\n\t"
      "madc.hi.cc.u32 %6, %8, %14, %6;\n\t"
      "madc.hi.u32    %7, %8, %15, %7;"
      : "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("mad.lo.cc.u32  %0, %7, %8, %0;\n\t"
      "madc.lo.cc.u32 %1, %7, %9, %1;\n\t"
      "madc.lo.cc.u32 %2, %7, %10, %2;\n\t"
      "madc.lo.cc.u32 %3, %7, %11, %3;\n\t"
      "madc.lo.cc.u32 %4, %7, %12, %4;\n\t"
      "madc.lo.cc.u32 %5, %7, %13, %5;\n\t"
      "addc.u32       %6, %6, 0;\n\t"
      "mad.hi.cc.u32  %1, %7, %8, %1;\n\t"
      "madc.hi.cc.u32 %2, %7, %9, %2;\n\t"
      "madc.hi.cc.u32 %3, %7, %10, %3;\n\t"
      "madc.hi.cc.u32 %4, %7, %11, %4;\n\t"
      "madc.hi.cc.u32 %5, %7, %12, %5;\n\t"
      "madc.hi.u32    %6, %7, %13, %6;"
      : "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9])
      : "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("mad.lo.cc.u32  %0, %6, %7, %0;\n\t"
      "madc.lo.cc.u32 %1, %6, %8, %1;\n\t"
      "madc.lo.cc.u32 %2, %6, %9, %2;\n\t"
      "madc.lo.cc.u32 %3, %6, %10, %3;\n\t"
      "madc.lo.cc.u32 %4, %6, %11, %4;\n\t"
      "addc.u32       %5, %5, 0;\n\t"
      "mad.hi.cc.u32  %1, %6, %7, %1;\n\t"
      "madc.hi.cc.u32 %2, %6, %8, %2;\n\t"
      "madc.hi.cc.u32 %3, %6, %9, %3;\n\t"
      "madc.hi.cc.u32 %4, %6, %10, %4;\n\t"
      "madc.hi.u32    %5, %6, %11, %5;"
      : "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10])
      : "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("mad.lo.cc.u32  %0, %5, %6, %0;\n\t"
      "madc.lo.cc.u32 %1, %5, %7, %1;\n\t"
      "madc.lo.cc.u32 %2, %5, %8, %2;\n\t"
      "madc.lo.cc.u32 %3, %5, %9, %3;\n\t"
      "addc.u32       %4, %4, 0;\n\t"
      "mad.hi.cc.u32  %1, %5, %6, %1;\n\t"
      "madc.hi.cc.u32 %2, %5, %7, %2;\n\t"
      "madc.hi.cc.u32 %3, %5, %8, %3;\n\t"
      "madc.hi.u32    %4, %5, %9, %4;"
      : "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11])
      : "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("mad.lo.cc.u32  %0, %4, %5, %0;\n\t"
      "madc.lo.cc.u32 %1, %4, %6, %1;\n\t"
      "madc.lo.cc.u32 %2, %4, %7, %2;\n\t"
      "addc.u32       %3, %3, 0;\n\t"
      "mad.hi.cc.u32  %1, %4, %5, %1;\n\t"
      "madc.hi.cc.u32 %2, %4, %6, %2;\n\t"
      "madc.hi.u32    %3, %4, %7, %3;"
      : "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12])
      : "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("mad.lo.cc.u32  %0, %3, %4, %0;\n\t"
      "madc.lo.cc.u32 %1, %3, %5, %1;\n\t"
      "addc.u32       %2, %2, 0;\n\t"
      "mad.hi.cc.u32  %1, %3, %4, %1;\n\t"
      "madc.hi.u32    %2, %3, %5, %2;"
      : "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13])
      : "r"(a[5]), "r"(a[6]), "r"(a[7]));
  asm("mad.lo.cc.u32  %0, %2, %3, %0;\n\t"
      "addc.u32       %1, %1, 0;\n\t"
      "mad.hi.u32     %1, %2, %3, %1;"
      : "+r"(t.v[13]), "+r"(t.v[14])
      : "r"(a[6]), "r"(a[7]));
  asm("add.cc.u32     %0, %0, %0;\n\t"
      "addc.cc.u32    %1, %1, %1;\n\t"
      "addc.cc.u32    %2, %2, %2;\n\t"
      "addc.cc.u32    %3, %3, %3;\n\t"
      "addc.cc.u32    %4, %4, %4;\n\t"
      "addc.cc.u32    %5, %5, %5;\n\t"
      "addc.cc.u32    %6, %6, %6;\n\t"
      "addc.cc.u32    %7, %7, %7;\n\t"
      "addc.cc.u32    %8, %8, %8;\n\t"
      "addc.cc.u32    %9, %9, %9;\n\t"
      "addc.cc.u32    %10, %10, %10;\n\t"
      "addc.cc.u32    %11, %11, %11;\n\t"
      "addc.cc.u32    %12, %12, %12;\n\t"
      "addc.cc.u32    %13, %13, %13;\n\t"
      "addc.cc.u32    %14, %14, %14;\n\t"
      "addc.u32       %15, %15, %15;"
      : "+r"(t.v[0]), "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15])
      : );
  asm("mad.lo.cc.u32  %0, %16, %16, %0;\n\t"
      "madc.hi.cc.u32 %1, %16, %16, %1;\n\t"
      "madc.lo.cc.u32 %2, %17, %17, %2;\n\t"
      "madc.hi.cc.u32 %3, %17, %17, %3;\n\t"
      "madc.lo.cc.u32 %4, %18, %18, %4;\n\t"
      "madc.hi.cc.u32 %5, %18, %18, %5;\n\t"
      "madc.lo.cc.u32 %6, %19, %19, %6;\n\t"
      "madc.hi.cc.u32 %7, %19, %19, %7;\n\t"
      "madc.lo.cc.u32 %8, %20, %20, %8;\n\t"
      "madc.hi.cc.u32 %9, %20, %20, %9;\n\t"
      "madc.lo.cc.u32 %10, %21, %21, %10;\n\t"
      "madc.hi.cc.u32 %11, %21, %21, %11;\n\t"
      "madc.lo.cc.u32 %12, %22, %22, %12;\n\t"
      "madc.hi.cc.u32 %13, %22, %22, %13;\n\t"
      "madc.lo.cc.u32 %14, %23, %23, %14;\n\t"
      "madc.hi.u32    %15, %23, %23, %15;"
      : "+r"(t.v[0]), "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
}

// t += u (the caller keeps the sum below 2^512)
BG_DEV void wide_add(Wide& t, const Wide& u) {
  asm("add.cc.u32     %0, %0, %16;\n\t"
      "addc.cc.u32    %1, %1, %17;\n\t"
      "addc.cc.u32    %2, %2, %18;\n\t"
      "addc.cc.u32    %3, %3, %19;\n\t"
      "addc.cc.u32    %4, %4, %20;\n\t"
      "addc.cc.u32    %5, %5, %21;\n\t"
      "addc.cc.u32    %6, %6, %22;\n\t"
      "addc.cc.u32    %7, %7, %23;\n\t"
      "addc.cc.u32    %8, %8, %24;\n\t"
      "addc.cc.u32    %9, %9, %25;\n\t"
      "addc.cc.u32    %10, %10, %26;\n\t"
      "addc.cc.u32    %11, %11, %27;\n\t"
      "addc.cc.u32    %12, %12, %28;\n\t"
      "addc.cc.u32    %13, %13, %29;\n\t"
      "addc.cc.u32    %14, %14, %30;\n\t"
      "addc.u32       %15, %15, %31;"
      : "+r"(t.v[0]), "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15])
      : "r"(u.v[0]), "r"(u.v[1]), "r"(u.v[2]), "r"(u.v[3]), "r"(u.v[4]), "r"(u.v[5]), "r"(u.v[6]), "r"(u.v[7]), "r"(u.v[8]), "r"(u.v[9]), "r"(u.v[10]), "r"(u.v[11]), "r"(u.v[12]), "r"(u.v[13]), "r"(u.v[14]), "r"(u.v[15]));
}

// t -= u (the caller keeps t >= u)
BG_DEV void wide_sub(Wide& t, const Wide& u) {
  asm("sub.cc.u32     %0, %0, %16;\n\t"
      "subc.cc.u32    %1, %1, %17;\n\t"
      "subc.cc.u32    %2, %2, %18;\n\t"
      "subc.cc.u32    %3, %3, %19;\n\t"
      "subc.cc.u32    %4, %4, %20;\n\t"
      "subc.cc.u32    %5, %5, %21;\n\t"
      "subc.cc.u32    %6, %6, %22;\n\t"
      "subc.cc.u32    %7, %7, %23;\n\t"
      "subc.cc.u32    %8, %8, %24;\n\t"
      "subc.cc.u32    %9, %9, %25;\n\t"
      "subc.cc.u32    %10, %10, %26;\n\t"
      "subc.cc.u32    %11, %11, %27;\n\t"
      "subc.cc.u32    %12, %12, %28;\n\t"
      "subc.cc.u32    %13, %13, %29;\n\t"
      "subc.cc.u32    %14, %14, %30;\n\t"
      "subc.u32       %15, %15, %31;"
      : "+r"(t.v[0]), "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15])
      : "r"(u.v[0]), "r"(u.v[1]), "r"(u.v[2]), "r"(u.v[3]), "r"(u.v[4]), "r"(u.v[5]), "r"(u.v[6]), "r"(u.v[7]), "r"(u.v[8]), "r"(u.v[9]), "r"(u.v[10]), "r"(u.v[11]), "r"(u.v[12]), "r"(u.v[13]), "r"(u.v[14]), "r"(u.v[15]));
}

// t += 2 p^2 (Fq)
BG_DEV void wide_add_2p2(Wide& t) {
  asm("add.cc.u32     %0, %0, %16;\n\t"
      "addc.cc.u32    %1, %1, %17;\n\t"
      "addc.cc.u32    %2, %2, %18;\n\t"
      "addc.cc.u32    %3, %3, %19;\n\t"
      "addc.cc.u32    %4, %4, %20;\n\t"
      "addc.cc.u32    %5, %5, %21;\n\t"
      "addc.cc.u32    %6, %6, %22;\n\t"
      "addc.cc.u32    %7, %7, %23;\n\t"
      "addc.cc.u32    %8, %8, %24;\n\t"
      "addc.cc.u32    %9, %9, %25;\n\t"
      "addc.cc.u32    %10, %10, %26;\n\t"
      "addc.cc.u32    %11, %11, %27;\n\t"
      "addc.cc.u32    %12, %12, %28;\n\t"
      "addc.cc.u32    %13, %13, %29;\n\t"
      "addc.cc.u32    %14, %14, %30;\n\t"
      "addc.u32       %15, %15, %31;"
      : "+r"(t.v[0]), "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15])
      : "n"(0x4ebad362u), "n"(0x76a8b144u), "n"(0x13d58202u), "n"(0x4c040e5au), "n"(0xdb2d95b9u), "n"(0x94a03138u), "n"(0xf4248590u), "n"(0x08d13d2au), "n"(0x698d671au), "n"(0x4ddbf4b8u), "n"(0x2c6eac0cu), "n"(0x60170aa2u), "n"(0x0691a439u), "n"(0xb334def8u), "n"(0xec797f38u), "n"(0x124b8970u));
}

// r = a + b as integers (a, b < p: the sum is below 2^255)
BG_DEV void raw_add8(uint32_t* r, const uint32_t* a, const uint32_t* b) {
  asm("add.cc.u32     %0, %8, %16;\n\t"
      "addc.cc.u32    %1, %9, %17;\n\t"
      "addc.cc.u32    %2, %10, %18;\n\t"
      "addc.cc.u32    %3, %11, %19;\n\t"
      "addc.cc.u32    %4, %12, %20;\n\t"
      "addc.cc.u32    %5, %13, %21;\n\t"
      "addc.cc.u32    %6, %14, %22;\n\t"
      "addc.u32       %7, %15, %23;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

// Montgomery reduction of t < p R: returns t R^-1 mod p (below p); t is consumed.  Row I adds
// m p 2^(32 I) (m = t[I] n0'); the carries out of limb I + 8 wait in e and enter limb I + 9
// with the next row (e <= 2; it ends at zero because the result is below 2^256).
template <class P>
BG_DEV Fp<P> redc(Wide& t) {
  uint32_t e = 0;
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[0]), "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[1]), "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[2]), "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[3]), "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[4]), "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[5]), "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[6]), "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  asm("{\n\t"
      ".reg .u32 m;\n\t"
      "mul.lo.u32     m, %0, %10;\n\t"
      "mad.lo.cc.u32  %0, m, %11, %0;\n\t"
      "madc.lo.cc.u32 %1, m, %12, %1;\n\t"
      "madc.lo.cc.u32 %2, m, %13, %2;\n\t"
      "madc.lo.cc.u32 %3, m, %14, %3;\n\t"
      "madc.lo.cc.u32 %4, m, %15, %4;\n\t"
      "madc.lo.cc.u32 %5, m, %16, %5;\n\t"
      "madc.lo.cc.u32 %6, m, %17, %6;\n\t"
      "madc.lo.cc.u32 %7, m, %18, %7;\n\t"
      "addc.cc.u32    %8, %8, %9;\n\t"
      "addc.u32       %9, 0, 0;\n\t"
      "mad.hi.cc.u32  %1, m, %11, %1;\n\t"
      "madc.hi.cc.u32 %2, m, %12, %2;\n\t"
      "madc.hi.cc.u32 %3, m, %13, %3;\n\t"
      "madc.hi.cc.u32 %4, m, %14, %4;\n\t"
      "madc.hi.cc.u32 %5, m, %15, %5;\n\t"
      "madc.hi.cc.u32 %6, m, %16, %6;\n\t"
      "madc.hi.cc.u32 %7, m, %17, %7;\n\t"
      "madc.hi.cc.u32 %8, m, %18, %8;\n\t"
      "addc.u32       %9, %9, 0;\n\t"
      "}"
      : "+r"(t.v[7]), "+r"(t.v[8]), "+r"(t.v[9]), "+r"(t.v[10]), "+r"(t.v[11]), "+r"(t.v[12]), "+r"(t.v[13]), "+r"(t.v[14]), "+r"(t.v[15]), "+r"(e)
      : "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  Fp<P> r;
  reduce_once<P>(r.v, t.v + 8);
  return r;
}

// a^2 with the squaring product
template <class P>
BG_DEV Fp<P> sqr_wide(const Fp<P>& a) {
  Wide t;
  wide_sqr(t, a.v);
  return redc<P>(t);
}

// Out-of-line pieces for the curve formulas.  Every Fq and Fq2 product of the MSM kernels is
// made of three shared bodies (a 512-bit product, a 512-bit square, a reduction), so the hot
// loops stay small in the instruction cache while squares use the squaring product and sums of
// products share one reduction.
static __device__ __noinline__ Wide wide_mul_ool(Fq a, Fq b) {
  Wide t;
  wide_mul(t, a.v, b.v);
  return t;
}
static __device__ __noinline__ Wide wide_sqr_ool(Fq a) {
  Wide t;
  wide_sqr(t, a.v);
  return t;
}
static __device__ __noinline__ Fq redc_ool(Wide t) { return redc<FqParams>(t); }

// Fq2 product (Karatsuba) with two reductions:
//   c0 = a0 b0 - a1 b1,  c1 = (a0 + a1)(b0 + b1) - a0 b0 - a1 b1 = a0 b1 + a1 b0
// with the sums a0 + a1, b0 + b1 kept unreduced (below 2p) so that c1 is exact
static __device__ __noinline__ Fq2 fq2_mul_ool(Fq2 a, Fq2 b) {
  Wide t0 = wide_mul_ool(a.c0, b.c0);
  const Wide t1 = wide_mul_ool(a.c1, b.c1);
  Fq sa, sb;
  raw_add8(sa.v, a.c0.v, a.c1.v);
  raw_add8(sb.v, b.c0.v, b.c1.v);
  Wide t2 = wide_mul_ool(sa, sb);
  wide_sub(t2, t0);
  wide_sub(t2, t1);
  wide_add_2p2(t0);
  wide_sub(t0, t1);
  return {redc_ool(t0), redc_ool(t2)};
}

// a b - c d in Fq2 with two reductions (both components offset by 2 p^2, below 4 p^2)
static __device__ __noinline__ Fq2 fq2_mul_sub_mul_ool(Fq2 a, Fq2 b, Fq2 c, Fq2 d) {
  Fq s0, s1;
  // a b: re = a0 b0 - a1 b1 + 2p^2, im = (a0 + a1)(b0 + b1) - a0 b0 - a1 b1 + 2p^2
  Wide re = wide_mul_ool(a.c0, b.c0);
  Wide w1 = wide_mul_ool(a.c1, b.c1);
  raw_add8(s0.v, a.c0.v, a.c1.v);
  raw_add8(s1.v, b.c0.v, b.c1.v);
  Wide im = wide_mul_ool(s0, s1);
  wide_sub(im, re);
  wide_sub(im, w1);
  wide_add_2p2(im);
  wide_add_2p2(re);
  wide_sub(re, w1);
  // - c d: re += c1 d1 - c0 d0, im += c0 d0 + c1 d1 - (c0 + c1)(d0 + d1)
  Wide w0 = wide_mul_ool(c.c0, d.c0);
  w1 = wide_mul_ool(c.c1, d.c1);
  wide_add(re, w1);
  wide_sub(re, w0);
  wide_add(im, w0);
  wide_add(im, w1);
  raw_add8(s0.v, c.c0.v, c.c1.v);
  raw_add8(s1.v, d.c0.v, d.c1.v);
  w0 = wide_mul_ool(s0, s1);
  wide_sub(im, w0);
  return {redc_ool(re), redc_ool(im)};
}

}  // namespace bg
