// msf_ct.cuh -- compile-time-sized shared-memory FFT stages (power-of-two
// lengths).  Same mixed-radix schedule as the runtime engine in
// msf_internal.cuh, with every length, stride and line count a template
// constant, so index arithmetic folds to shifts and masks and every loop
// unrolls.
//
// Schedule for length N: spans N, N/R0, N/(R0 R1), ... with
//   R(span) = 8 if span % 8 == 0 and span != 16, else 4 if span % 4 == 0, else 2
// (128 = 8*4*4, 256 = 8*8*4, 512 = 8*8*8).  Stage (span, R, M = span/R)
// combines the R elements b + j + r*M of every block b of `span` elements.
//   DIF: butterfly, then twiddle w_span^{r j}; natural input, output of
//        frequency k at position pos(k) = sum_s d_s M_s (d_s the digits of k).
//   DIT: stages in reverse order, twiddle first, then butterfly; input of
//        sample k at position pos(k), natural output.
#pragma once

#include "msf_internal.cuh"

namespace msf {
namespace ct {

__host__ __device__ constexpr int radix_for(int span) {
  return (span % 8 == 0 && span != 16) ? 8 : (span % 4 == 0 ? 4 : 2);
}

__host__ __device__ constexpr bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// position of sample/frequency k in the digit-reversed layout of length N
template <int N>
__device__ __forceinline__ int pos(int k) {
  int p = 0;
  int span = N;
#pragma unroll
  for (int s = 0; s < 12; ++s) {
    if (span > 1) {
      const int R = radix_for(span);
      const int M = span / R;
      p += (k % R) * M;
      k /= R;
      span = M;
    }
  }
  return p;
}

// One stage over NL lines: element q of line l at s[q*SM + l*SL].  Threads
// walk lines fastest when LF (unit stride across lines), positions otherwise.
template <int N, int SPAN, int NL, int SM, int SL, int NT, bool LF, bool DIT>
__device__ __forceinline__ void stage(float2* s, const float2* tw) {
  constexpr int R = radix_for(SPAN);
  constexpr int M = SPAN / R;
  constexpr int NB = N / R;
  constexpr int TOTAL = NB * NL;
  constexpr int TWS = N / SPAN;
#pragma unroll 4
  for (int u = threadIdx.x; u < TOTAL; u += NT) {
    int l, q;
    if (LF) { l = u % NL; q = u / NL; }
    else    { q = u % NB; l = u / NB; }
    const int blk = q / M;
    const int j = q % M;
    float2* base = s + l * SL + (blk * SPAN + j) * SM;
    float2 a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = base[r * M * SM];
    if (DIT) {
      if (M > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) a[r] = cmul(a[r], tw[r * j * TWS]);
      }
      Bfly<R>::run(a);
#pragma unroll
      for (int r = 0; r < R; ++r) base[r * M * SM] = a[r];
    } else {
      Bfly<R>::run(a);
      base[0] = a[0];
      if (M > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) base[r * M * SM] = cmul(a[r], tw[r * j * TWS]);
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) base[r * M * SM] = a[r];
      }
    }
  }
}

template <int N, int SPAN, int NL, int SM, int SL, int NT, bool LF>
struct Dif {
  static __device__ __forceinline__ void run(float2* s, const float2* tw) {
    stage<N, SPAN, NL, SM, SL, NT, LF, false>(s, tw);
    __syncthreads();
    Dif<N, SPAN / radix_for(SPAN), NL, SM, SL, NT, LF>::run(s, tw);
  }
};
template <int N, int NL, int SM, int SL, int NT, bool LF>
struct Dif<N, 1, NL, SM, SL, NT, LF> {
  static __device__ __forceinline__ void run(float2*, const float2*) {}
};

template <int N, int SPAN, int NL, int SM, int SL, int NT, bool LF>
struct Dit {
  static __device__ __forceinline__ void run(float2* s, const float2* tw) {
    Dit<N, SPAN / radix_for(SPAN), NL, SM, SL, NT, LF>::run(s, tw);
    stage<N, SPAN, NL, SM, SL, NT, LF, true>(s, tw);
    __syncthreads();
  }
};
template <int N, int NL, int SM, int SL, int NT, bool LF>
struct Dit<N, 1, NL, SM, SL, NT, LF> {
  static __device__ __forceinline__ void run(float2*, const float2*) {}
};

// Forward FFT of NL lines, natural input -> output at pos(k); ends synced.
template <int N, int NL, int SM, int SL, int NT, bool LF>
__device__ __forceinline__ void dif(float2* s, const float2* tw) {
  Dif<N, N, NL, SM, SL, NT, LF>::run(s, tw);
}
// Forward FFT of NL lines, input at pos(k) -> natural output; ends synced.
template <int N, int NL, int SM, int SL, int NT, bool LF>
__device__ __forceinline__ void dit(float2* s, const float2* tw) {
  Dit<N, N, NL, SM, SL, NT, LF>::run(s, tw);
}

}  // namespace ct
}  // namespace msf
