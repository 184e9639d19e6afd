// bitscan.cuh -- the ALU core of the bit-parallel Jaro match count, shared by
// the evaluation kernel (kernels.cu) and the scan-rate probe (probe.cu), so
// that the probe times exactly the instructions the scan runs.
//
// State over W 32-bit words: `win`, the positions of the left string inside
// the match window of the current right character, and `mt`, the positions
// already matched.  One step with the Peq row `pe` of the right character
// (bit j set when left[j] equals it): x = pe & win & ~mt; the lowest set bit
// of x becomes matched (x & -x, the negation by a carry chain); the window
// moves one position right, growing by `grow` at its low end.
#pragma once

#include <cstdint>

namespace hbx {
namespace dev {

// n = 0 - x over W 32-bit words (two's complement of the W*32-bit number).
template <int W>
struct Neg;
template <>
struct Neg<1> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[1], uint32_t (&n)[1]) {
    n[0] = 0u - x[0];
  }
};
template <>
struct Neg<2> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[2], uint32_t (&n)[2]) {
    asm("sub.cc.u32 %0, %2, %3;\n\tsubc.u32 %1, %2, %4;"
        : "=r"(n[0]), "=r"(n[1])
        : "r"(0u), "r"(x[0]), "r"(x[1]));
  }
};
template <>
struct Neg<3> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[3], uint32_t (&n)[3]) {
    asm("sub.cc.u32 %0, %3, %4;\n\tsubc.cc.u32 %1, %3, %5;\n\tsubc.u32 %2, %3, %6;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]));
  }
};
template <>
struct Neg<4> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[4], uint32_t (&n)[4]) {
    asm("sub.cc.u32 %0, %4, %5;\n\tsubc.cc.u32 %1, %4, %6;\n\tsubc.cc.u32 %2, %4, %7;\n\t"
        "subc.u32 %3, %4, %8;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]));
  }
};
template <>
struct Neg<5> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[5], uint32_t (&n)[5]) {
    asm("sub.cc.u32 %0, %5, %6;\n\tsubc.cc.u32 %1, %5, %7;\n\tsubc.cc.u32 %2, %5, %8;\n\t"
        "subc.cc.u32 %3, %5, %9;\n\tsubc.u32 %4, %5, %10;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]));
  }
};
template <>
struct Neg<6> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[6], uint32_t (&n)[6]) {
    asm("sub.cc.u32 %0, %6, %7;\n\tsubc.cc.u32 %1, %6, %8;\n\tsubc.cc.u32 %2, %6, %9;\n\t"
        "subc.cc.u32 %3, %6, %10;\n\tsubc.cc.u32 %4, %6, %11;\n\tsubc.u32 %5, %6, %12;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4]), "=r"(n[5])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]));
  }
};
template <>
struct Neg<7> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[7], uint32_t (&n)[7]) {
    asm("sub.cc.u32 %0, %7, %8;\n\tsubc.cc.u32 %1, %7, %9;\n\tsubc.cc.u32 %2, %7, %10;\n\t"
        "subc.cc.u32 %3, %7, %11;\n\tsubc.cc.u32 %4, %7, %12;\n\tsubc.cc.u32 %5, %7, %13;\n\t"
        "subc.u32 %6, %7, %14;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4]), "=r"(n[5]), "=r"(n[6])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]),
          "r"(x[6]));
  }
};
template <>
struct Neg<8> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[8], uint32_t (&n)[8]) {
    asm("sub.cc.u32 %0, %8, %9;\n\tsubc.cc.u32 %1, %8, %10;\n\tsubc.cc.u32 %2, %8, %11;\n\t"
        "subc.cc.u32 %3, %8, %12;\n\tsubc.cc.u32 %4, %8, %13;\n\tsubc.cc.u32 %5, %8, %14;\n\t"
        "subc.cc.u32 %6, %8, %15;\n\tsubc.u32 %7, %8, %16;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4]), "=r"(n[5]), "=r"(n[6]),
          "=r"(n[7])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]),
          "r"(x[7]));
  }
};

// One character step of the bit-parallel match count (see the file comment).
template <int W, int S>
__device__ __forceinline__ void bp_update(const uint32_t (&pe)[S], uint32_t (&win)[W],
                                          uint32_t (&mt)[W], uint32_t grow) {
  uint32_t x[W], n[W];
#pragma unroll
  for (int k = 0; k < W; k++) x[k] = pe[k] & win[k] & ~mt[k];
  Neg<W>::run(x, n);
#pragma unroll
  for (int k = 0; k < W; k++) mt[k] |= x[k] & n[k];
#pragma unroll
  for (int k = W - 1; k > 0; k--) win[k] = __funnelshift_l(win[k - 1], win[k], 1);
  win[0] = (win[0] << 1) | grow;
}

}  // namespace dev
}  // namespace hbx
