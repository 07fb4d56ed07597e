// msf_direct.cu -- direct-sum structure factor S(q) = |sum_j f_j e^{i q.r_j}|^2
// and its adjoint, in FP32 (the continuous-position form of the gridded
// power the reference computes at dens.py:313-316).
//
// Phases are computed in turns, t = (q/2pi).r, and reduced to [-1/2, 1/2]
// before sin/cos (sincos_turns: polynomials in turns, no 2 pi scaling).
// With |q.r| up to ~25 turns a plain FP32 product loses ~1e-5 rad, so each
// q/2pi is held as an unevaluated sum hi + lo (split from FP64), each
// product q_i r_i is formed with its exact FMA residual, every component is
// reduced by its own nearest integer (exact), and the small remainders are
// summed: the phase error is then ~2e-8 turn (rms) whatever |q.r| is.
//
// Accuracy that the log(1 + S) loss needs: its gradient is dominated by the
// q vectors of small S, whose relative error is the absolute error of the
// amplitudes A, B over |F|.  Errors that add coherently over the atoms
// (a bias of the phase scale, a biased sin/cos) or a long FP32 running sum
// move A and B by ~1e-3 at 20k atoms and the gradient by ~4e-4.  Hence the
// unbiased turn-based sin/cos, and in the forward pass: each thread sums its
// q's terms over groups of kDGroup atoms in plain FP32, adds each group sum
// into the tile's FP32 partial with a compensated (Kahan) addition, and adds
// the tile partials (kDTile atoms) into FP64 running sums.  A numpy
// emulation of this arithmetic gives a gradient error of 5e-5 against FP64
// at 20k atoms (the floor is the FP32 phase rounding).  The adjoint's sums
// (no small-S amplification) stay plain FP32 per tile.
//
// Forward: A_q = sum f cos, B_q = sum f sin, S_q = A^2 + B^2.
// Adjoint (upstream g_q = dL/dS_q), recomputing the phases:
//   dL/dr_j = 2 f_j sum_q g_q q (B_q cos - A_q sin)
//   dL/df_j = 2 sum_q g_q (A_q cos + B_q sin)
#include "msf_internal.cuh"

namespace msf {

constexpr int kDThreads = 256;
constexpr int kDPerF = 4;                      // q per thread (forward)
constexpr int kDPerB = 2;                      // atoms per thread (adjoint: 4 spill at its register budget)
constexpr int kDTile = 512;                    // atoms (fwd) or q (bwd) per smem tile
constexpr int kDGroup = 16;                    // atoms per plain FP32 group sum (fwd)

// q in turns as hi + lo pairs: (hx, hy, hz) and (lx, ly, lz)
struct QTurns { float hx, hy, hz, lx, ly, lz; };

__device__ __forceinline__ QTurns q_turns(float4 q) {
  const double inv = 0.15915494309189533577;  // 1/(2 pi)
  const double tx = (double)q.x * inv, ty = (double)q.y * inv, tz = (double)q.z * inv;
  QTurns t;
  t.hx = (float)tx; t.hy = (float)ty; t.hz = (float)tz;
  t.lx = (float)(tx - (double)t.hx);
  t.ly = (float)(ty - (double)t.hy);
  t.lz = (float)(tz - (double)t.hz);
  return t;
}

// fractional turns of (hi + lo) * r, reduced per component
__device__ __forceinline__ float turn_frac(float hi, float lo, float r) {
  const float p = hi * r;
  const float e = fmaf(lo, r, fmaf(hi, r, -p));  // exact residual of hi*r, plus lo*r
  return (p - rintf(p)) + e;
}

// sin and cos of 2 pi t for t in [-1/2, 1/2] turns, without a rounded 2 pi
// scaling the phase: the quadrant k = rint(4t) is taken off exactly
// (r = t - k/4 in [-1/8, 1/8]), sin(2 pi r) and cos(2 pi r) are polynomials
// in r^2 fitted for this build (near-minimax on [0, 1/8] by iteratively
// reweighted least squares in FP64: errors 2.4e-9 and 4.7e-11 before FP32
// rounding), and the quadrant rotates them.  Errors of the rounded
// coefficients are odd (sin) or even (cos) functions of r whose means cancel
// between opposite quadrants.  The SFU form __sincosf(2 pi t) instead
// multiplies t by float(2 pi) and its own scale: a phase bias near 1e-8 of
// the same sign for every atom, whose errors add coherently in
// A = sum f cos, B = sum f sin (~1e-3 at 20k atoms); through the q of small S
// the log(1 + S) loss's gradient then moved by ~4e-4.
__device__ __forceinline__ void sincos_turns(float t, float* s, float* c) {
  // t in [-3/2, 3/2]: the quadrant k = rint(4t) (|k| <= 6) also takes off
  // the whole turns, and t - k/4 is exact (Sterbenz: t and k/4 are within a
  // factor 2 of each other for k != 0); only k mod 4 matters below.  k is
  // rounded by adding 1.5 * 2^23 (the sum's unit is 1, so the FMA rounds 4t
  // to the nearest integer, ties to even, like rintf): the sum's low bits
  // then hold k mod 4 and no float-to-int conversion is needed
  constexpr float kRound = 12582912.0f;
  const float kb = fmaf(4.0f, t, kRound);
  const float k = kb - kRound;
  const float r = fmaf(-0.25f, k, t);
  const float z = r * r;
  const float ps = r * fmaf(fmaf(fmaf(-75.40099585508018f, z, 81.5925250459675f), z, -41.34166242174424f), z,
                            6.283185287502589f);
  const float pc = fmaf(fmaf(fmaf(fmaf(59.22042251089335f, z, -85.44285258833072f), z, 64.9393162129225f), z,
                             -19.73920865037173f), z, 0.9999999999526074f);
  const int q = __float_as_int(kb) & 3;
  const float sv = (q & 1) ? pc : ps;
  const float cv = (q & 1) ? ps : pc;
  *s = (q >= 2) ? -sv : sv;                 // quadrants 2, 3
  *c = (q == 1 || q == 2) ? -cv : cv;       // quadrants 1, 2
}

__device__ __forceinline__ void phase_sincos(const QTurns& q, float4 r, float* s, float* c) {
  const float t = turn_frac(q.hx, q.lx, r.x) + turn_frac(q.hy, q.ly, r.y) + turn_frac(q.hz, q.lz, r.z);
  sincos_turns(t, s, c);
}

template <int NTH, int PER>
__global__ void __launch_bounds__(NTH, 2) k_direct_fwd(const float4* __restrict__ rf, int64_t n_atoms,
                                                      const float4* __restrict__ q, int64_t n_q,
                                                      int64_t q_sys_stride, float* S, float2* AB) {
  __shared__ float4 tile[kDTile];
  const int sys = blockIdx.y;
  const float4* R = rf + sys * n_atoms;
  const float4* Q = q + sys * q_sys_stride;
  QTurns tq[PER];
  int64_t qi[PER];
  double A[PER], B[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    qi[k] = (int64_t)blockIdx.x * NTH * PER + k * NTH + threadIdx.x;
    float4 v = qi[k] < n_q ? __ldg(Q + qi[k]) : make_float4(0.f, 0.f, 0.f, 0.f);
    tq[k] = q_turns(v);
    A[k] = 0.0; B[k] = 0.0;
  }
  for (int64_t a0 = 0; a0 < n_atoms; a0 += kDTile) {
    const int na = (int)min((int64_t)kDTile, n_atoms - a0);
    __syncthreads();
    for (int i = threadIdx.x; i < na; i += NTH) tile[i] = __ldg(R + a0 + i);
    __syncthreads();
    // tile partials with their Kahan compensations
    float pa[PER], pb[PER], ca[PER], cb[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) { pa[k] = 0.f; pb[k] = 0.f; ca[k] = 0.f; cb[k] = 0.f; }
    for (int i0 = 0; i0 < na; i0 += kDGroup) {
      const int i1 = min(i0 + kDGroup, na);
      float ga[PER], gb[PER];
#pragma unroll
      for (int k = 0; k < PER; ++k) { ga[k] = 0.f; gb[k] = 0.f; }
      for (int i = i0; i < i1; ++i) {
        const float4 r = tile[i];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
          float s, c;
          phase_sincos(tq[k], r, &s, &c);
          ga[k] = fmaf(r.w, c, ga[k]);
          gb[k] = fmaf(r.w, s, gb[k]);
        }
      }
#pragma unroll
      for (int k = 0; k < PER; ++k) {
        // compensated additions (round-to-nearest intrinsics: not contracted)
        const float ya = __fsub_rn(ga[k], ca[k]);
        const float ta = __fadd_rn(pa[k], ya);
        ca[k] = __fsub_rn(__fsub_rn(ta, pa[k]), ya);
        pa[k] = ta;
        const float yb = __fsub_rn(gb[k], cb[k]);
        const float tb = __fadd_rn(pb[k], yb);
        cb[k] = __fsub_rn(__fsub_rn(tb, pb[k]), yb);
        pb[k] = tb;
      }
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      A[k] += (double)pa[k] - (double)ca[k];
      B[k] += (double)pb[k] - (double)cb[k];
    }
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    if (qi[k] < n_q) {
      const int64_t o = sys * n_q + qi[k];
      S[o] = (float)(A[k] * A[k] + B[k] * B[k]);
      AB[o] = make_float2((float)A[k], (float)B[k]);
    }
  }
}

template <int NTH, int PER>
__global__ void __launch_bounds__(NTH) k_direct_bwd(const float4* __restrict__ rf, int64_t n_atoms,
                                                   const float4* __restrict__ q, int64_t n_q,
                                                   int64_t q_sys_stride, const float* __restrict__ g,
                                                   const float2* __restrict__ AB, float4* grad) {
  __shared__ QTurns tq[kDTile];   // q/2pi as hi + lo
  __shared__ float4 tqr[kDTile];  // q (rad)
  __shared__ float2 tg[kDTile];   // (g*A, g*B)
  const int sys = blockIdx.y;
  const float4* R = rf + sys * n_atoms;
  const float4* Q = q + sys * q_sys_stride;
  float4 r[PER];
  int64_t ai[PER];
  double gx[PER], gy[PER], gz[PER], gf[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    ai[k] = (int64_t)blockIdx.x * NTH * PER + k * NTH + threadIdx.x;
    r[k] = ai[k] < n_atoms ? __ldg(R + ai[k]) : make_float4(0.f, 0.f, 0.f, 0.f);
    gx[k] = gy[k] = gz[k] = gf[k] = 0.0;
  }
  for (int64_t q0 = 0; q0 < n_q; q0 += kDTile) {
    const int nq = (int)min((int64_t)kDTile, n_q - q0);
    __syncthreads();
    for (int i = threadIdx.x; i < nq; i += NTH) {
      const float4 v = __ldg(Q + q0 + i);
      tqr[i] = v;
      tq[i] = q_turns(v);
      const float gg = __ldg(g + sys * n_q + q0 + i);
      const float2 ab = __ldg(AB + sys * n_q + q0 + i);
      tg[i] = make_float2(gg * ab.x, gg * ab.y);
    }
    __syncthreads();
    float px[PER], py[PER], pz[PER], pf[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) px[k] = py[k] = pz[k] = pf[k] = 0.f;
    for (int i = 0; i < nq; ++i) {
      const QTurns t = tq[i];
      const float4 qq = tqr[i];
      const float2 ga = tg[i];
#pragma unroll
      for (int k = 0; k < PER; ++k) {
        float s, c;
        phase_sincos(t, r[k], &s, &c);
        const float w = fmaf(ga.y, c, -ga.x * s);   // gB cos - gA sin
        px[k] = fmaf(w, qq.x, px[k]);
        py[k] = fmaf(w, qq.y, py[k]);
        pz[k] = fmaf(w, qq.z, pz[k]);
        pf[k] = fmaf(ga.x, c, fmaf(ga.y, s, pf[k]));
      }
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      gx[k] += (double)px[k]; gy[k] += (double)py[k]; gz[k] += (double)pz[k]; gf[k] += (double)pf[k];
    }
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    if (ai[k] < n_atoms) {
      const double f2 = 2.0 * (double)r[k].w;
      grad[sys * n_atoms + ai[k]] =
          make_float4((float)(f2 * gx[k]), (float)(f2 * gy[k]), (float)(f2 * gz[k]), (float)(2.0 * gf[k]));
    }
  }
}

// multiprocessor count of the current device (cached per device)
static int sm_count() {
  static int cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cache[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = n > 0 ? n : 152;
  }
  return cache[dev];
}

}  // namespace msf

using namespace msf;

extern "C" {

int msf_direct_fwd(const void* r_f, int64_t n_atoms, const void* q, int64_t n_q, int32_t n_sys,
                   int32_t q_shared, float* S, void* AB, msf_stream_t stream) {
  if (n_atoms < 0 || n_q < 0 || n_sys < 1 || n_sys > 65535) return MSF_E_INVALID;
  if (n_q == 0) return MSF_OK;
  if (!q || !S || !AB || (n_atoms > 0 && !r_f)) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const float4* rp = static_cast<const float4*>(r_f);
  const float4* qp = static_cast<const float4*>(q);
  const int64_t qs = q_shared ? 0 : n_q;
  // few systems: one q per thread in 128-thread blocks, so that the blocks
  // still cover the SMs (the 4-per-thread form needs n_q/1024 * n_sys of them)
  const int64_t nb_big = (n_q + kDThreads * kDPerF - 1) / (kDThreads * kDPerF);
  if (nb_big * n_sys >= 2 * (int64_t)sm_count()) {
    if (nb_big > 0x7fffffff) return MSF_E_UNSUPPORTED;
    k_direct_fwd<kDThreads, kDPerF><<<dim3((unsigned)nb_big, n_sys), kDThreads, 0, st>>>(
        rp, n_atoms, qp, n_q, qs, S, static_cast<float2*>(AB));
  } else {
    const int64_t nb = (n_q + 127) / 128;
    if (nb > 0x7fffffff) return MSF_E_UNSUPPORTED;
    k_direct_fwd<128, 1><<<dim3((unsigned)nb, n_sys), 128, 0, st>>>(rp, n_atoms, qp, n_q, qs, S,
                                                                     static_cast<float2*>(AB));
  }
  return launch_status();
}

int msf_direct_bwd(const void* r_f, int64_t n_atoms, const void* q, int64_t n_q, int32_t n_sys,
                   int32_t q_shared, const float* g, const void* AB, void* grad,
                   msf_stream_t stream) {
  if (n_atoms < 0 || n_q < 0 || n_sys < 1 || n_sys > 65535) return MSF_E_INVALID;
  if (n_atoms == 0) return MSF_OK;
  if (!r_f || !grad || (n_q > 0 && (!q || !g || !AB))) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const float4* rp = static_cast<const float4*>(r_f);
  const float4* qp = static_cast<const float4*>(q);
  const int64_t qs = q_shared ? 0 : n_q;
  // few systems: one atom per thread in 64-thread blocks (more blocks over the SMs)
  const int64_t nb_big = (n_atoms + kDThreads * kDPerB - 1) / (kDThreads * kDPerB);
  if (nb_big * n_sys >= 2 * (int64_t)sm_count()) {
    if (nb_big > 0x7fffffff) return MSF_E_UNSUPPORTED;
    k_direct_bwd<kDThreads, kDPerB><<<dim3((unsigned)nb_big, n_sys), kDThreads, 0, st>>>(
        rp, n_atoms, qp, n_q, qs, g, static_cast<const float2*>(AB), static_cast<float4*>(grad));
  } else {
    const int64_t nb = (n_atoms + 63) / 64;
    if (nb > 0x7fffffff) return MSF_E_UNSUPPORTED;
    k_direct_bwd<64, 1><<<dim3((unsigned)nb, n_sys), 64, 0, st>>>(
        rp, n_atoms, qp, n_q, qs, g, static_cast<const float2*>(AB), static_cast<float4*>(grad));
  }
  return launch_status();
}

}  // extern "C"
