// msf_mixed.cuh -- mixed-radix (2^a 3^b 5^c) two-pass register FFT of lines
// held in shared memory, every length a compile-time constant.
//
// reg_dftm<R> transforms R values in registers (forward kernel
// e^{-2 pi i jk/R}, natural order in and out) for the radices
// R in {2,3,4,5,6,8,9,10,12,15,16,18,20,25,27,32}: 2, 3, 4, 5 and 8 are the
// butterflies of msf_internal.cuh, 16 and 32 the power-of-two register DFT of
// msf_reg.cuh, the others split R = A*B the same way,
//   x[n1 + A n2] --DFT_B over n2--> * w_R^(n1 k1) --DFT_A over n1--> X[k1 + B k2],
// with the twiddles of msf_wr.cuh as immediates.
//
// A line of length N = A*B (Split2m<N>: B first, A second) is transformed
// in two register passes with one exchange through shared memory, as in
// msf_r2.cuh: pass 1 reads the B samples n1 + A n2 of one n1, applies DFT_B
// and the twiddles w_N^(n1 k1) and writes them back in place; pass 2 reads
// the A values A k1 + n1 of one k1 and applies DFT_A, giving X[k1 + B k2].
#pragma once

#include "msf_reg.cuh"
#include "msf_wr.cuh"

namespace msf {
namespace mixed {

// R = A * B for the composite register radices (A the outer, smaller factor)
template <int R> struct SplitM;
template <> struct SplitM<6> { static constexpr int A = 2, B = 3; };
template <> struct SplitM<9> { static constexpr int A = 3, B = 3; };
template <> struct SplitM<10> { static constexpr int A = 2, B = 5; };
template <> struct SplitM<12> { static constexpr int A = 4, B = 3; };
template <> struct SplitM<15> { static constexpr int A = 3, B = 5; };
template <> struct SplitM<18> { static constexpr int A = 2, B = 9; };
template <> struct SplitM<20> { static constexpr int A = 4, B = 5; };
template <> struct SplitM<25> { static constexpr int A = 5, B = 5; };
template <> struct SplitM<27> { static constexpr int A = 3, B = 9; };

// multiply by w_R^m; the axis points 1, -i, -1, i cost no arithmetic
template <int R>
__host__ __device__ __forceinline__ float2 tw_mul(float2 v, int m) {
  m %= R;
  if (m == 0) return v;
  if (4 * m == R) return cmi(v);
  if (2 * m == R) return make_float2(-v.x, -v.y);
  if (4 * m == 3 * R) return cpi(v);
  return cmul(v, WR<R>::w(m));
}

template <int R>
__host__ __device__ __forceinline__ void reg_dftm(float2* a) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2 || R == 3 || R == 4 || R == 5 || R == 8) {
    Bfly<R>::run(a);
  } else if constexpr (R == 16 || R == 32) {
    reg::reg_dft<R>(a);
  } else {
    constexpr int A = SplitM<R>::A, B = SplitM<R>::B;
    float2 y[A][B];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) y[n1][n2] = a[n1 + A * n2];
      reg_dftm<B>(y[n1]);
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) y[n1][k1] = tw_mul<R>(y[n1][k1], n1 * k1);
    }
#pragma unroll
    for (int k1 = 0; k1 < B; ++k1) {
      float2 c[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) c[n1] = y[n1][k1];
      reg_dftm<A>(c);
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) a[k1 + B * k2] = c[k2];
    }
  }
}

// N = A * B: pass-1 radix B, pass-2 radix A
template <int N> struct Split2m;
#define MSF_SPLIT2M(N_, B_, A_) \
  template <> struct Split2m<N_> { static constexpr int B = B_, A = A_; };
MSF_SPLIT2M(16, 4, 4) MSF_SPLIT2M(18, 6, 3) MSF_SPLIT2M(20, 5, 4) MSF_SPLIT2M(24, 6, 4)
MSF_SPLIT2M(25, 5, 5) MSF_SPLIT2M(27, 9, 3) MSF_SPLIT2M(30, 6, 5) MSF_SPLIT2M(32, 8, 4)
MSF_SPLIT2M(36, 6, 6) MSF_SPLIT2M(40, 8, 5) MSF_SPLIT2M(45, 9, 5) MSF_SPLIT2M(48, 8, 6)
MSF_SPLIT2M(50, 10, 5) MSF_SPLIT2M(54, 9, 6) MSF_SPLIT2M(60, 10, 6) MSF_SPLIT2M(64, 8, 8)
MSF_SPLIT2M(72, 9, 8) MSF_SPLIT2M(75, 15, 5) MSF_SPLIT2M(80, 10, 8) MSF_SPLIT2M(81, 9, 9)
MSF_SPLIT2M(90, 10, 9) MSF_SPLIT2M(96, 12, 8) MSF_SPLIT2M(100, 10, 10) MSF_SPLIT2M(108, 12, 9)
MSF_SPLIT2M(120, 12, 10) MSF_SPLIT2M(125, 25, 5) MSF_SPLIT2M(128, 16, 8) MSF_SPLIT2M(135, 15, 9)
MSF_SPLIT2M(144, 12, 12) MSF_SPLIT2M(150, 15, 10) MSF_SPLIT2M(160, 16, 10) MSF_SPLIT2M(162, 18, 9)
MSF_SPLIT2M(180, 15, 12) MSF_SPLIT2M(192, 16, 12) MSF_SPLIT2M(200, 20, 10) MSF_SPLIT2M(216, 18, 12)
MSF_SPLIT2M(225, 15, 15) MSF_SPLIT2M(240, 16, 15) MSF_SPLIT2M(243, 27, 9) MSF_SPLIT2M(250, 25, 10)
MSF_SPLIT2M(256, 16, 16) MSF_SPLIT2M(512, 32, 16)
#undef MSF_SPLIT2M

// Every supported length, for the dispatch tables of the kernels.
#define MSF_SMOOTH_SIZES(X)                                                                          \
  X(16) X(18) X(20) X(24) X(25) X(27) X(30) X(32) X(36) X(40) X(45) X(48) X(50) X(54) X(60) X(64) \
  X(72) X(75) X(80) X(81) X(90) X(96) X(100) X(108) X(120) X(125) X(128) X(135) X(144) X(150)     \
  X(160) X(162) X(180) X(192) X(200) X(216) X(225) X(240) X(243) X(250) X(256) X(512)

// Pass 1 over every (n1, l) item; sample n of line l at s[n*SM + l*SL].
// tw: w_N^k, k < N (shared memory).
template <int N, int NL, int SM, int SL, int NT>
__device__ __forceinline__ void pass1(float2* s, const float2* tw) {
  constexpr int A = Split2m<N>::A, B = Split2m<N>::B;
  constexpr int ITEMS = A * NL;
#pragma unroll 1
  for (int it = threadIdx.x; it < ITEMS; it += NT) {
    const int l = it % NL, n1 = it / NL;
    float2* p = s + l * SL + n1 * SM;
    float2 v[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) v[n2] = p[n2 * A * SM];
    reg_dftm<B>(v);
    if (n1) {
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) v[k1] = cmul(v[k1], tw[n1 * k1]);
    }
#pragma unroll
    for (int k1 = 0; k1 < B; ++k1) p[k1 * A * SM] = v[k1];
  }
}

// Full transform, natural order in and out; ends with a barrier.
template <int N, int NL, int SM, int SL, int NT>
__device__ __forceinline__ void fft2_lines(float2* s, const float2* tw) {
  constexpr int A = Split2m<N>::A, B = Split2m<N>::B;
  pass1<N, NL, SM, SL, NT>(s, tw);
  __syncthreads();
  constexpr int ITEMS = B * NL;
  constexpr int PER = (ITEMS + NT - 1) / NT;
  float2 r[PER][A];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int it = j * NT + threadIdx.x;
    if (ITEMS % NT == 0 || it < ITEMS) {
      const int l = it % NL, k1 = it / NL;
      const float2* p = s + l * SL + (A * k1) * SM;
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) r[j][n1] = p[n1 * SM];
      reg_dftm<A>(r[j]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int it = j * NT + threadIdx.x;
    if (ITEMS % NT == 0 || it < ITEMS) {
      const int l = it % NL, k1 = it / NL;
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) s[l * SL + (k1 + B * k2) * SM] = r[j][k2];
    }
  }
  __syncthreads();
}

}  // namespace mixed
}  // namespace msf
