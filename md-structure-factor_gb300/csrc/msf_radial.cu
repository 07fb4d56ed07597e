// msf_radial.cu -- radial_integrate (plot2d.py:160-173): histogram of S over
// R = |q|^2, with R and the bin search in float16 as the reference computes
// them under numpy >= 2.
//
// The reference: R = (x**2).astype(f16) + (y**2).astype(f16) + (z**2).astype(f16)
// (plot2d.py:163), then np.histogram(R, bins=Nbins, weights=S) and
// np.histogram(R, bins=Nbins) (plot2d.py:164-165).  numpy's equal-width path
// for a float16 sample keeps every step in float16: range [min R, max R]
// (widened by 0.5 each side when empty), edges = linspace(first, last,
// Nbins + 1, dtype=float16), and per sample
//   i = int(((R - first) / (last - first)) * Nbins)       (each op rounded to f16)
//   i -= (i == Nbins);  i -= (R < edge[i]);  i += (i != Nbins-1 && R >= edge[i+1])
// then a bincount.  numpy evaluates each float16 op as one float32 op on the
// widened operands, rounded to float16; the kernels do exactly that with
// round-to-nearest intrinsics (no contraction).  The square is FP64 and its
// conversion to float16 is one round-to-nearest-even step, as numpy's.
//
// Two sources: the reference's (..., 4) kgridplt array (x, y, z, S per voxel;
// a range pass then a binning pass), or the centred S grid with its three
// axes (R from three per-axis float16 tables; the range follows from the
// tables because float16 rounding and addition are monotone; one pass).
// Histograms are privatised per CTA in shared memory (FP64 sums, u32
// counts) and flushed with global atomics.
#include <cuda_fp16.h>

#include "msf_internal.cuh"

namespace msf {
namespace {

constexpr int kRadialMaxBins = 2048;   // bin counts exact in float16

__device__ __forceinline__ float h2f(unsigned short b) { return __half2float(__ushort_as_half(b)); }
__device__ __forceinline__ unsigned short f2h(float v) { return __half_as_ushort(__float2half_rn(v)); }
__device__ __forceinline__ unsigned short d2h(double v) { return __half_as_ushort(__double2half(v)); }
__device__ __forceinline__ unsigned short hadd(unsigned short a, unsigned short b) {
  return f2h(__fadd_rn(h2f(a), h2f(b)));
}
__device__ __forceinline__ unsigned short sq16(double v) { return d2h(__dmul_rn(v, v)); }

// R of plot2d.py:163, summed left to right
__device__ __forceinline__ unsigned short r_of(double x, double y, double z) {
  return hadd(hadd(sq16(x), sq16(y)), sq16(z));
}

// Range pass over the (..., 4) array: min/max of the float16 bit patterns
// (R >= +0, so unsigned order is numeric order), and a flag for inf/NaN.
__global__ void k_radial_range(const double* __restrict__ D, int64_t nv, unsigned* __restrict__ stats) {
  unsigned lo = 0xFFFFu, hi = 0u, bad = 0u;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nv; e += (int64_t)gridDim.x * blockDim.x) {
    const double2 xy = __ldcs(reinterpret_cast<const double2*>(D + 4 * e));
    const double2 zs = __ldcs(reinterpret_cast<const double2*>(D + 4 * e + 2));
    const unsigned r = r_of(xy.x, xy.y, zs.x);
    if (r >= 0x7C00u) {
      bad = 1u;
    } else {
      lo = min(lo, r);
      hi = max(hi, r);
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
    bad |= __shfl_xor_sync(0xFFFFFFFFu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(stats, lo);
    atomicMax(stats + 1, hi);
    if (bad) atomicOr(stats + 2, 1u);
  }
}

struct RadialBins {
  const unsigned short* edges;   // nbins + 1 float16 edges
  int nbins;
  double* hist;
  unsigned long long* count;
  unsigned* status;              // bit 0: an index left [0, nbins) (clamped)
};

struct BinCtx {
  const unsigned short* es;
  int n;
  float first, den, fn;
  __device__ __forceinline__ int index(unsigned short r, unsigned& bad) const {
    const float fr = h2f(r);
    unsigned short t = f2h(__fsub_rn(fr, first));
    t = f2h(__fdiv_rn(h2f(t), den));
    t = f2h(__fmul_rn(h2f(t), fn));
    const float ft = h2f(t);   // in [0, n] for R in [first, last]; clamped before the conversion
    if (!(ft >= 0.f && ft <= (float)n)) bad = 1u;
    int i = ft >= (float)n ? n : (ft >= 0.f ? (int)ft : 0);
    if (i == n) --i;
    if (i < 0 || i > n - 1) { bad = 1u; i = i < 0 ? 0 : n - 1; }
    if (fr < h2f(es[i])) --i;
    if (i < 0) { bad = 1u; i = 0; }
    if (i != n - 1 && fr >= h2f(es[i + 1])) ++i;
    return i;
  }
};

// shared memory: sums (n doubles) | counts (n u32) | edges (n + 1 halves) | extra halves
__device__ __forceinline__ BinCtx bins_setup(const RadialBins& b, unsigned char* sm, double*& hs, unsigned*& cs) {
  const int n = b.nbins;
  hs = reinterpret_cast<double*>(sm);
  cs = reinterpret_cast<unsigned*>(hs + n);
  unsigned short* es = reinterpret_cast<unsigned short*>(cs + n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) { hs[i] = 0.0; cs[i] = 0u; }
  for (int i = threadIdx.x; i <= n; i += blockDim.x) es[i] = b.edges[i];
  __syncthreads();
  BinCtx c;
  c.es = es;
  c.n = n;
  c.first = h2f(es[0]);
  c.den = h2f(f2h(__fsub_rn(h2f(es[n]), c.first)));   // last - first, in float16
  c.fn = h2f(f2h((float)n));
  return c;
}

__device__ __forceinline__ void bins_flush(const RadialBins& b, const double* hs, const unsigned* cs, unsigned bad) {
  __syncthreads();
  for (int i = threadIdx.x; i < b.nbins; i += blockDim.x) {
    if (cs[i]) {
      atomicAdd(b.hist + i, hs[i]);
      atomicAdd(b.count + i, (unsigned long long)cs[i]);
    }
  }
  if (bad) atomicOr(b.status, 1u);
}

__global__ void k_radial_bin_points(const double* __restrict__ D, int64_t nv, RadialBins b) {
  extern __shared__ __align__(16) unsigned char sm[];
  double* hs;
  unsigned* cs;
  const BinCtx c = bins_setup(b, sm, hs, cs);
  unsigned bad = 0u;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nv; e += (int64_t)gridDim.x * blockDim.x) {
    const double2 xy = __ldcs(reinterpret_cast<const double2*>(D + 4 * e));
    const double2 zs = __ldcs(reinterpret_cast<const double2*>(D + 4 * e + 2));
    const int i = c.index(r_of(xy.x, xy.y, zs.x), bad);
    atomicAdd(hs + i, zs.y);
    atomicAdd(cs + i, 1u);
  }
  bins_flush(b, hs, cs, bad);
}

// S grid (p0, p1, p2) with per-axis float16 squares hx, hy, hz; one CTA
// iteration per (ix, iy) row, threads along z.
__global__ void k_radial_bin_grid(const double* __restrict__ S, int p0, int p1, int p2,
                                  const unsigned short* __restrict__ hx, const unsigned short* __restrict__ hy,
                                  const unsigned short* __restrict__ hz, RadialBins b) {
  extern __shared__ __align__(16) unsigned char sm[];
  double* hs;
  unsigned* cs;
  const BinCtx c = bins_setup(b, sm, hs, cs);
  unsigned bad = 0u;
  const int64_t rows = (int64_t)p0 * p1;
  for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const int ix = (int)(row / p1), iy = (int)(row % p1);
    const unsigned short rxy = hadd(__ldg(hx + ix), __ldg(hy + iy));
    const double* s = S + row * p2;
    for (int iz = threadIdx.x; iz < p2; iz += blockDim.x) {
      const int i = c.index(hadd(rxy, __ldg(hz + iz)), bad);
      atomicAdd(hs + i, __ldcs(s + iz));
      atomicAdd(cs + i, 1u);
    }
  }
  bins_flush(b, hs, cs, bad);
}

size_t bins_smem(int n) { return (size_t)n * 12 + (size_t)(n + 1) * 2; }

int grid_for(int64_t work, int threads) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (work + threads - 1) / threads;
  return (int)(want < (int64_t)sms * 4 ? (want < 1 ? 1 : want) : (int64_t)sms * 4);
}

}  // namespace
}  // namespace msf

using namespace msf;

extern "C" {

int msf_radial_range(const double* D, int64_t n_vox, uint32_t* stats, msf_stream_t stream) {
  if (!D || !stats || n_vox < 1) return MSF_E_INVALID;
  if (reinterpret_cast<uintptr_t>(D) & 15) return MSF_E_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(stats, 0xFF, 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(stats + 1, 0, 8, s);
  if (e != cudaSuccess) return cuda_status(e);
  k_radial_range<<<grid_for(n_vox, 256), 256, 0, s>>>(D, n_vox, stats);
  return launch_status();
}

int msf_radial_bin_points(const double* D, int64_t n_vox, const uint16_t* edges, int32_t nbins, double* hist,
                          int64_t* count, uint32_t* status, msf_stream_t stream) {
  if (!D || !edges || !hist || !count || !status || n_vox < 1) return MSF_E_INVALID;
  if (nbins < 1 || nbins > kRadialMaxBins) return MSF_E_UNSUPPORTED;
  if (reinterpret_cast<uintptr_t>(D) & 15) return MSF_E_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  RadialBins b{edges, nbins, hist, reinterpret_cast<unsigned long long*>(count), status};
  k_radial_bin_points<<<grid_for(n_vox, 256), 256, bins_smem(nbins), s>>>(D, n_vox, b);
  return launch_status();
}

int msf_radial_bin_grid(const double* S, int32_t p0, int32_t p1, int32_t p2, const uint16_t* hx,
                        const uint16_t* hy, const uint16_t* hz, const uint16_t* edges, int32_t nbins,
                        double* hist, int64_t* count, uint32_t* status, msf_stream_t stream) {
  if (!S || !hx || !hy || !hz || !edges || !hist || !count || !status) return MSF_E_INVALID;
  if (p0 < 1 || p1 < 1 || p2 < 1) return MSF_E_INVALID;
  if (nbins < 1 || nbins > kRadialMaxBins) return MSF_E_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  RadialBins b{edges, nbins, hist, reinterpret_cast<unsigned long long*>(count), status};
  const int threads = p2 >= 256 ? 256 : ((p2 + 31) / 32) * 32;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t rows = (int64_t)p0 * p1;
  const int blocks = (int)(rows < (int64_t)sms * 8 ? rows : (int64_t)sms * 8);
  k_radial_bin_grid<<<blocks, threads, bins_smem(nbins), s>>>(S, p0, p1, p2, hx, hy, hz, b);
  return launch_status();
}

}  // extern "C"
