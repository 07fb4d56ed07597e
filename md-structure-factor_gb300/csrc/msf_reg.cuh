// msf_reg.cuh -- in-register DFTs and two-level line FFTs (power-of-two).
//
// reg_dft<R> transforms R values held in registers (forward kernel
// e^{-2 pi i jk/R}, natural order in and out) for R = 2..64 by splitting
// R = A*B:  x[n1 + A n2]  --DFT_B over n2-->  Y[n1][k1]  --* w_R^(n1 k1)-->
// --DFT_A over n1-->  X[k1 + B k2].  Every index is a compile-time constant
// once unrolled, so the data never leaves registers and the twiddles are
// immediates: w_64^k below holds cos/sin(2 pi k/64) rounded to float.
//
// A line of length N = A*B held in shared memory is transformed in two
// register passes with one exchange through shared memory (instead of one
// pass per radix-8 stage): pass 1 reads the B samples n1 + A n2 of one n1,
// applies DFT_B and the twiddles w_N^(n1 k1) and writes them back in place;
// pass 2 reads the A values A k1 + n1 of one k1, applies DFT_A, and (after a
// barrier) writes X[k1 + B k2] in natural order.
#pragma once

#include "msf_internal.cuh"

namespace msf {
namespace reg {

__host__ __device__ constexpr float2 w64(int k) {
  switch (k & 63) {
    case 0: return make_float2(1.0f, -0.0f);
    case 1: return make_float2(0.99518472f, -0.0980171412f);
    case 2: return make_float2(0.980785251f, -0.195090324f);
    case 3: return make_float2(0.956940353f, -0.290284663f);
    case 4: return make_float2(0.923879504f, -0.382683426f);
    case 5: return make_float2(0.881921291f, -0.471396744f);
    case 6: return make_float2(0.831469595f, -0.555570245f);
    case 7: return make_float2(0.773010433f, -0.634393275f);
    case 8: return make_float2(0.707106769f, -0.707106769f);
    case 9: return make_float2(0.634393275f, -0.773010433f);
    case 10: return make_float2(0.555570245f, -0.831469595f);
    case 11: return make_float2(0.471396744f, -0.881921291f);
    case 12: return make_float2(0.382683426f, -0.923879504f);
    case 13: return make_float2(0.290284663f, -0.956940353f);
    case 14: return make_float2(0.195090324f, -0.980785251f);
    case 15: return make_float2(0.0980171412f, -0.99518472f);
    case 16: return make_float2(0.0f, -1.0f);
    case 17: return make_float2(-0.0980171412f, -0.99518472f);
    case 18: return make_float2(-0.195090324f, -0.980785251f);
    case 19: return make_float2(-0.290284663f, -0.956940353f);
    case 20: return make_float2(-0.382683426f, -0.923879504f);
    case 21: return make_float2(-0.471396744f, -0.881921291f);
    case 22: return make_float2(-0.555570245f, -0.831469595f);
    case 23: return make_float2(-0.634393275f, -0.773010433f);
    case 24: return make_float2(-0.707106769f, -0.707106769f);
    case 25: return make_float2(-0.773010433f, -0.634393275f);
    case 26: return make_float2(-0.831469595f, -0.555570245f);
    case 27: return make_float2(-0.881921291f, -0.471396744f);
    case 28: return make_float2(-0.923879504f, -0.382683426f);
    case 29: return make_float2(-0.956940353f, -0.290284663f);
    case 30: return make_float2(-0.980785251f, -0.195090324f);
    case 31: return make_float2(-0.99518472f, -0.0980171412f);
    case 32: return make_float2(-1.0f, -0.0f);
    case 33: return make_float2(-0.99518472f, 0.0980171412f);
    case 34: return make_float2(-0.980785251f, 0.195090324f);
    case 35: return make_float2(-0.956940353f, 0.290284663f);
    case 36: return make_float2(-0.923879504f, 0.382683426f);
    case 37: return make_float2(-0.881921291f, 0.471396744f);
    case 38: return make_float2(-0.831469595f, 0.555570245f);
    case 39: return make_float2(-0.773010433f, 0.634393275f);
    case 40: return make_float2(-0.707106769f, 0.707106769f);
    case 41: return make_float2(-0.634393275f, 0.773010433f);
    case 42: return make_float2(-0.555570245f, 0.831469595f);
    case 43: return make_float2(-0.471396744f, 0.881921291f);
    case 44: return make_float2(-0.382683426f, 0.923879504f);
    case 45: return make_float2(-0.290284663f, 0.956940353f);
    case 46: return make_float2(-0.195090324f, 0.980785251f);
    case 47: return make_float2(-0.0980171412f, 0.99518472f);
    case 48: return make_float2(0.0f, 1.0f);
    case 49: return make_float2(0.0980171412f, 0.99518472f);
    case 50: return make_float2(0.195090324f, 0.980785251f);
    case 51: return make_float2(0.290284663f, 0.956940353f);
    case 52: return make_float2(0.382683426f, 0.923879504f);
    case 53: return make_float2(0.471396744f, 0.881921291f);
    case 54: return make_float2(0.555570245f, 0.831469595f);
    case 55: return make_float2(0.634393275f, 0.773010433f);
    case 56: return make_float2(0.707106769f, 0.707106769f);
    case 57: return make_float2(0.773010433f, 0.634393275f);
    case 58: return make_float2(0.831469595f, 0.555570245f);
    case 59: return make_float2(0.881921291f, 0.471396744f);
    case 60: return make_float2(0.923879504f, 0.382683426f);
    case 61: return make_float2(0.956940353f, 0.290284663f);
    case 62: return make_float2(0.980785251f, 0.195090324f);
    case 63: return make_float2(0.99518472f, 0.0980171412f);
  }
  return make_float2(1.f, 0.f);
}

// w_R^m for R dividing 64
template <int R>
__host__ __device__ __forceinline__ float2 wr(int m) { return w64((m % R) * (64 / R)); }

// v * w_R^m with m a constant once unrolled: the quarter turns are a swap
// and sign changes (a product with the 0 of w = -i would cost an FMA: x * 0
// is not folded without fast math)
template <int R>
__host__ __device__ __forceinline__ float2 twiddle(float2 v, int m) {
  m %= R;
  if (m == 0) return v;
  if (4 * m == R) return cmi(v);
  if (2 * m == R) return make_float2(-v.x, -v.y);
  if (4 * m == 3 * R) return cpi(v);
  return cmul(v, wr<R>(m));
}

template <int R> struct Split {
  static constexpr int A = (R == 16) ? 4 : ((R == 32) ? 4 : 8);   // R = A * B
  static constexpr int B = R / A;
};

template <int R>
__host__ __device__ __forceinline__ void reg_dft(float2* a) {
  if constexpr (R == 1) {
  } else if constexpr (R <= 8 && R != 6) {
    Bfly<R>::run(a);
  } else {
    constexpr int A = Split<R>::A, B = Split<R>::B;
    float2 y[A][B];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) y[n1][n2] = a[n1 + A * n2];
      reg_dft<B>(y[n1]);
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) y[n1][k1] = twiddle<R>(y[n1][k1], n1 * k1);
    }
#pragma unroll
    for (int k1 = 0; k1 < B; ++k1) {
      float2 c[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) c[n1] = y[n1][k1];
      reg_dft<A>(c);
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) a[k1 + B * k2] = c[k2];
    }
  }
}

}  // namespace reg
}  // namespace msf
