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
      if (n1 != 0) {   // n1 = 0: every twiddle is 1
#pragma unroll
        for (int k1 = 1; k1 < B; ++k1) v[k1] = cmul(v[k1], tw(n1 * k1));
      }
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

// ------------------------------------------------ two values per access
// The plane kernel's passes with 16-byte shared-memory accesses: a thread
// moves two complex values per load or store -- the same sample of two
// adjacent lines (fft2_linepairs) or two adjacent samples of one line
// (pass1_samplepairs) -- so each pass issues half the shared-memory
// instructions.  Layout requirement: even line stride (16-byte alignment);
// with a line stride of S complex values and S*8 = 16 (mod 128) bytes, eight
// consecutive lanes cover eight different 16-byte bank groups in both
// directions, so neither pass has bank conflicts.
__device__ __forceinline__ void ld2(const float2* p, float2& a, float2& b) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  a = make_float2(t.x, t.y);
  b = make_float2(t.z, t.w);
}
__device__ __forceinline__ void st2(float2* p, float2 a, float2 b) {
  *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
}

// Full transform of NL lines (line l at s + l, unit line stride; sample n at
// n*SM), natural order in and out; thread items cover the line pairs
// (2lp, 2lp + 1).  The two inner barriers are over the warps that share line
// pairs (line_group_sync over NL/2 pairs); the caller orders the result with
// a whole-block barrier before other lines are read.
template <int N, int NL, int SM, int NT, typename TW>
__device__ __forceinline__ void fft2_linepairs(float2* s, TW tw) {
  static_assert(NL % 2 == 0 && SM % 2 == 0, "pairs of lines, 16-byte aligned");
  constexpr int A = Split2<N>::A, B = Split2<N>::B, NP = NL / 2;
  constexpr int ITEMS1 = A * NP;
#pragma unroll 1
  for (int base_it = 0; base_it < ITEMS1; base_it += NT) {
    const int it = base_it + threadIdx.x;
    if (ITEMS1 % NT == 0 || it < ITEMS1) {
      const int lp = it % NP, n1 = it / NP;
      float2* p = s + 2 * lp + n1 * SM;
      float2 u[B], v[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) ld2(p + n2 * A * SM, u[n2], v[n2]);
      reg::reg_dft<B>(u);
      reg::reg_dft<B>(v);
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) {
        const float2 w = tw(n1 * k1);
        u[k1] = cmul(u[k1], w);
        v[k1] = cmul(v[k1], w);
      }
#pragma unroll
      for (int k1 = 0; k1 < B; ++k1) st2(p + k1 * A * SM, u[k1], v[k1]);
    }
  }
  line_group_sync<NP, NT>();
  constexpr int ITEMS2 = B * NP;
  constexpr int PER = (ITEMS2 + NT - 1) / NT;
  float2 r[PER][A], q[PER][A];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int it = j * NT + threadIdx.x;
    if (ITEMS2 % NT == 0 || it < ITEMS2) {
      const int lp = it % NP, k1 = it / NP;
      const float2* p = s + 2 * lp + (A * k1) * SM;
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) ld2(p + n1 * SM, r[j][n1], q[j][n1]);
      reg::reg_dft<A>(r[j]);
      reg::reg_dft<A>(q[j]);
    }
  }
  line_group_sync<NP, NT>();
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int it = j * NT + threadIdx.x;
    if (ITEMS2 % NT == 0 || it < ITEMS2) {
      const int lp = it % NP, k1 = it / NP;
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) st2(s + 2 * lp + (k1 + B * k2) * SM, r[j][k2], q[j][k2]);
    }
  }
}

// pass1_fn over NL lines (line l at s + l*SL, unit sample stride) with the
// items (n1, l) and (n1 + 1, l) of one thread sharing their 16-byte loads.
template <int N, int NL, int SL, int NT, typename TW>
__device__ __forceinline__ void pass1_samplepairs(float2* s, TW tw) {
  static_assert(SL % 2 == 0, "16-byte aligned lines");
  constexpr int A = Split2<N>::A, B = Split2<N>::B;
  static_assert(A % 2 == 0, "pairs of first-pass items");
  constexpr int ITEMS = (A / 2) * NL;
#pragma unroll 1
  for (int base_it = 0; base_it < ITEMS; base_it += NT) {
    const int it = base_it + threadIdx.x;
    if (ITEMS % NT == 0 || it < ITEMS) {
      const int l = it % NL, n1 = 2 * (it / NL);
      float2* p = s + l * SL + n1;
      float2 u[B], v[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) ld2(p + n2 * A, u[n2], v[n2]);
      reg::reg_dft<B>(u);
      reg::reg_dft<B>(v);
      if (n1 != 0) {   // n1 = 0 (whole warps when NL >= 32): u's twiddles are 1
#pragma unroll
        for (int k1 = 1; k1 < B; ++k1) u[k1] = cmul(u[k1], tw(n1 * k1));
      }
#pragma unroll
      for (int k1 = 1; k1 < B; ++k1) v[k1] = cmul(v[k1], tw((n1 + 1) * k1));
#pragma unroll
      for (int k1 = 0; k1 < B; ++k1) st2(p + k1 * A, u[k1], v[k1]);
    }
  }
}

}  // namespace r2
}  // namespace msf
