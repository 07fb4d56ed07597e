// msf_r2.cuh -- two-pass register FFT of lines held in shared memory.
//
// Length N = A*B (B = first-pass radix, A = second-pass radix).  Sample n of
// line l sits at s[n*SM + l*SL].
//   pass 1, item (n1, l): the B samples n1 + A*n2 -> DFT_B -> times
//           w_N^(n1*k1) -> written back to the same B slots (n1 + A*k1);
//   pass 2, item (k1, l): the A values A*k1 + n1 -> DFT_A -> X[k1 + B*k2].
// fft2_lines writes X back in natural order (after a barrier, since the
// natural slots differ from the ones read).  Consecutive threads take
// consecutive lines, so with unit line stride (or an odd one) a warp's
// shared-memory accesses are conflict-free.  Each element crosses shared
// memory twice (one load and one store per pass) instead of once per radix
// stage.
#pragma once

#include "msf_reg.cuh"

namespace msf {
namespace r2 {

template <int N> struct Split2;
template <> struct Split2<16> { static constexpr int B = 4, A = 4; };
template <> struct Split2<32> { static constexpr int B = 8, A = 4; };
template <> struct Split2<64> { static constexpr int B = 8, A = 8; };
template <> struct Split2<128> { static constexpr int B = 16, A = 8; };
template <> struct Split2<256> { static constexpr int B = 16, A = 16; };
template <> struct Split2<512> { static constexpr int B = 32, A = 16; };

// Pass 1 over every (n1, l) item.  tw(k) = w_N^k, k < N.  With NL >= 32 the
// lanes of a warp share n1, so the twiddle index is warp-uniform (a constant
// memory table then costs no shared-memory bandwidth).
template <int N, int NL, int SM, int SL, int NT, typename TW>
__device__ __forceinline__ void pass1_fn(float2* s, TW tw) {
  constexpr int A = Split2<N>::A, B = Split2<N>::B;
  constexpr int ITEMS = A * NL;
#pragma unroll 1
  for (int base_it = 0; base_it < ITEMS; base_it += NT) {
    const int it = base_it + threadIdx.x;
    if (ITEMS % NT == 0 || it < ITEMS) {
      const int l = it % NL, n1 = it / NL;
      float2* p = s + l * SL + n1 * SM;
      float2 v[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) v[n2] = p[n2 * A * SM];
      reg::reg_dft<B>(v);
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) v[k1] = cmul(v[k1], tw(n1 * k1));
#pragma unroll
      for (int k1 = 0; k1 < B; ++k1) p[k1 * A * SM] = v[k1];
    }
  }
}

// tw: w_N^k, k < N, in shared memory.
template <int N, int NL, int SM, int SL, int NT>
__device__ __forceinline__ void pass1(float2* s, const float2* tw) {
  pass1_fn<N, NL, SM, SL, NT>(s, [tw](int k) { return tw[k]; });
}

// Full transform, natural order in and out; ends with a barrier.
template <int N, int NL, int SM, int SL, int NT, typename TW>
__device__ __forceinline__ void fft2_lines_fn(float2* s, TW tw) {
  constexpr int A = Split2<N>::A, B = Split2<N>::B;
  pass1_fn<N, NL, SM, SL, NT>(s, tw);
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
      reg::reg_dft<A>(r[j]);
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

template <int N, int NL, int SM, int SL, int NT>
__device__ __forceinline__ void fft2_lines(float2* s, const float2* tw) {
  fft2_lines_fn<N, NL, SM, SL, NT>(s, [tw](int k) { return tw[k]; });
}

// Barrier over the threads that share lines with this one.  In pass1_fn and
// fft2_lines_fn every item of thread t lies on line t % NL when NT is a
// multiple of NL, so with NL a multiple of 32 the warps split into NL/32
// groups that never touch each other's lines: a named barrier per group
// (ids 1..8; 0 is __syncthreads) orders the passes of one group without
// waiting for the others.  Otherwise a whole-block barrier.
template <int NL, int NT>
__device__ __forceinline__ void line_group_sync() {
  if constexpr (NL % 32 == 0 && NT % NL == 0 && NL / 32 > 1 && NL / 32 <= 8) {
    constexpr int G = NL / 32;
    const int g = (int)(threadIdx.x % NL) / 32;
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "n"(NT / G) : "memory");
  } else {
    __syncthreads();
  }
}

// fft2_lines_fn with its two inner barriers over line groups only; the
// caller orders the result with a whole-block barrier before another
// thread's lines are read.
template <int N, int NL, int SM, int SL, int NT, typename TW>
__device__ __forceinline__ void fft2_lines_grouped(float2* s, TW tw) {
  constexpr int A = Split2<N>::A, B = Split2<N>::B;
  pass1_fn<N, NL, SM, SL, NT>(s, tw);
  line_group_sync<NL, NT>();
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
      reg::reg_dft<A>(r[j]);
    }
  }
  line_group_sync<NL, NT>();
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int it = j * NT + threadIdx.x;
    if (ITEMS % NT == 0 || it < ITEMS) {
      const int l = it % NL, k1 = it / NL;
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) s[l * SL + (k1 + B * k2) * SM] = r[j][k2];
    }
  }
}

}  // namespace r2
}  // namespace msf
