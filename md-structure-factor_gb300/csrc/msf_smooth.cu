// msf_smooth.cu -- three-sweep R2C 3-D FFT with |F|^2 and the frame sum for
// grids whose axes are all 2^a 3^b 5^c lengths from 16 to 256, or 512
// (variant 4, "smooth"): the batched multi-system workload of uneven grid
// shapes and the 512^3 stress grid.  Replaces dens.py:313-318 as msf_fft.cu
// does, with every axis length a compile-time constant and every line
// transformed by the two-pass mixed-radix register FFT of msf_mixed.cuh
// (one exchange through shared memory per pass) instead of one pass per
// radix stage with runtime index arithmetic.
//
//   k_zs_bulk<n2>, k_zs<n2>
//             G row pairs (y = 2p, 2p+1 of the flattened (x, y) rows) per CTA,
//             read from the int32 grid (which is zeroed behind the read) as
//             x[2p] + i x[2p+1], z-FFT, split into the two rows' half
//             spectra; the rows arrive by one bulk copy per CTA (k_zs_bulk)
//             or by register-staged loads (float grids, unaligned bases)
//   k_ys<n1>  (x, W kz columns) per CTA: y-FFT in place in the spectra
//   k_xs<n0>  W (y, kz) columns per CTA: x-FFT of every frame of the batch
//             (the next frame's tile copied by cp.async under the current
//             one's transform where two tiles fit), |F|^2 summed in FP32 in
//             registers, one FP64 RMW of sf every kPowerFlush frames and
//             after the last
#include "msf_mixed.cuh"
#include "msf_tma.cuh"

namespace msf {

namespace {

constexpr int kSmoothThreads = 256;
constexpr int kSmoothW = 16;   // columns per CTA of the y and x sweeps

__host__ __device__ constexpr int smooth_rows(int n2) {
  // row pairs per z CTA: N2 * G <= 8192 complex, G a power of two <= 64
  return n2 <= 128 ? 64 : (n2 <= 256 ? 32 : 16);
}

struct SmZArgs {
  const void* grids;
  int kind;         // GridKind of `grids`
  int64_t V;        // elements per frame grid
  float2* C;
  int64_t Vh;       // complex elements per frame half spectrum
  int64_t rows;     // n0 * n1 rows per frame
  int zero;
  const float2* tw; // w_n2^k
  int* status;      // plan status word (bounded-wait timeout)
};

// cp.async of 8 bytes (src_bytes 0: zero fill, nothing read)
__device__ __forceinline__ void cp_async8(void* dst, const void* src, int src_bytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ float load_any(const void* g, int kind, int64_t i) {
  if (kind == kGridI32) return load_grid<kGridI32>(g, i);
  if (kind == kGridF32) return load_grid<kGridF32>(g, i);
  return load_grid<kGridF64>(g, i);
}

// z FFT of the G line pairs in buf (sample z of line g at buf[z (G+1) + g])
// and the split into the two rows' half spectra: rows 2p and 2p+1 from the
// packed line are (P[k] + conj P[-k]) / 2 and (P[k] - conj P[-k]) / (2i)
template <int N2, int G>
__device__ __forceinline__ void zs_fft_split(float2* buf, const float2* tw, const SmZArgs& a, int frame,
                                             int64_t p0) {
  constexpr int S = G + 1, NH = N2 / 2 + 1, NT = kSmoothThreads;
  mixed::fft2_lines<N2, G, S, 1, NT>(buf, tw);
  float2* out = a.C + frame * a.Vh;
  for (int e = threadIdx.x; e < G * NH; e += NT) {
    const int g = e / NH, k = e - g * NH;
    const int64_t ra = 2 * (p0 + g);
    if (ra >= a.rows) continue;
    const float2 P = buf[k * S + g];
    const float2 Q = cconj(buf[((N2 - k) % N2) * S + g]);
    out[ra * NH + k] = cscale(cadd(P, Q), 0.5f);
    if (ra + 1 < a.rows) out[(ra + 1) * NH + k] = cscale(cmi(csub(P, Q)), 0.5f);
  }
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// k_zs: the register-staged z sweep, for float grids and int32 grids at a
// base that is not 16-byte aligned (k_zs_bulk below takes the others).
// Three CTAs per SM (80 registers) for the 512-point lines, which used 94
// registers (two CTAs per SM) on their own: the 512^3 stress grid went from
// 562 to 600-700 frames/s.  The other lengths keep the compiler's choice
// (the same bound on the 256-point lines cost the batched systems 4%).
// (16-byte loads of eight z per lane with the lanes over lines, which keeps
// the shared-memory stores conflict-free, measured 4.3x slower: 1.46 ms
// against 0.34 ms for 8 frames of 192^3 -- each warp load then touches 32
// rows, and every load is followed by the zeroing store of the same bytes.)
__host__ __device__ constexpr int zs_min_blocks(int n2) { return n2 == 512 ? 3 : 1; }

template <int N2>
__global__ void __launch_bounds__(kSmoothThreads, zs_min_blocks(N2)) k_zs(SmZArgs a) {
  constexpr int G = smooth_rows(N2), S = G + 1;
  extern __shared__ __align__(16) float2 smem[];
  float2* buf = smem;              // [N2][S]: sample z of line g at buf[z*S + g]
  float2* tw = buf + N2 * S;       // N2
  const int frame = blockIdx.y;
  const int64_t p0 = (int64_t)blockIdx.x * G;
  copy_table(tw, a.tw, N2);
  void* gw = const_cast<void*>(a.grids);
  // 8 elements (16 loads) in flight per thread (12, at the same three CTAs
  // per SM, measured 3% slower on the batched systems)
  gather_batched<8, float2>(
      G * N2,
      [&](int e) {
        const int g = e / N2, z = e - g * N2;
        const int64_t ra = 2 * (p0 + g);
        float va = 0.f, vb = 0.f;
        if (ra < a.rows) {
          const int64_t ia = frame * a.V + ra * N2 + z;
          va = load_any(a.grids, a.kind, ia);
          if (a.zero) zero_grid<kGridI32>(gw, ia);
          if (ra + 1 < a.rows) {
            vb = load_any(a.grids, a.kind, ia + N2);
            if (a.zero) zero_grid<kGridI32>(gw, ia + N2);
          }
        }
        return make_float2(va, vb);
      },
      [&](int e, float2 v) {
        const int g = e / N2, z = e - g * N2;
        buf[z * S + g] = v;
      });
  __syncthreads();
  zs_fft_split<N2, G>(buf, tw, a, frame, p0);
}

// Row pairs per CTA of the bulk-copied z sweep: the line buffer plus the
// block's raw rows (8 G n2 bytes) fit three or four times per SM (32 row
// pairs of 135-192-point lines, two CTAs per SM, measured 4% slower on
// 192^3 than 16 at four).
__host__ __device__ constexpr int bulk_rows(int n2) { return n2 <= 128 ? 32 : (n2 <= 256 ? 16 : 8); }
template <int N2>
constexpr size_t zs_bulk_smem() {   // line buffer, twiddles, raw rows + 4 ints of alignment slack
  return (size_t)N2 * (bulk_rows(N2) + 2) * sizeof(float2) + ((size_t)2 * bulk_rows(N2) * N2 + 4) * sizeof(int32_t);
}

// k_zs for int32 grids at a 16-byte aligned base: the CTA's 2G rows are
// contiguous in the grid, so one cp.async.bulk copy (mbarrier, bounded wait)
// brings them into shared memory -- tens of KB in flight per CTA instead of
// 16 scalar loads per thread --, the block is zeroed by 16-byte stores
// behind the copy, and the rows are transposed into the line buffer from
// shared memory.  The block sits in shared memory at its misalignment
// (0-3 ints) so that its 16-byte aligned interior lands aligned there too;
// the fewer than four ints before and after the interior move by plain
// loads and stores, so nothing outside the block is read or written.
template <int N2>
__global__ void __launch_bounds__(kSmoothThreads) k_zs_bulk(SmZArgs a) {
  constexpr int G = bulk_rows(N2), S = G + 1, NT = kSmoothThreads;
  static_assert(G % 2 == 0, "raw rows must start 16-byte aligned");
  extern __shared__ __align__(16) float2 smem[];
  float2* buf = smem;                                   // [N2][S]
  float2* tw = buf + N2 * S;                            // N2
  int32_t* raw = reinterpret_cast<int32_t*>(tw + N2);   // [2G][N2], 16-byte aligned (G even)
  __shared__ __align__(8) uint64_t bar;
  __shared__ int failed;
  const int frame = blockIdx.y;
  const int64_t p0 = (int64_t)blockIdx.x * G, r0 = 2 * p0;
  const int nrows = (int)min((int64_t)2 * G, a.rows - r0);
  const int64_t first = frame * a.V + r0 * N2;   // int index of the block
  int32_t* src = static_cast<int32_t*>(const_cast<void*>(a.grids)) + first;
  const int n = nrows * N2;                       // ints of the block
  const int off = (int)(first & 3);               // its misalignment; block int i at raw[off + i]
  const int hn = min(off ? 4 - off : 0, n);       // ints before the aligned interior
  const int nb = (n - hn) & ~3;                   // the bulk-copied interior: a multiple of 16 bytes
  const int tn = n - hn - nb;                     // ints after it (0-3)
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0 && nb > 0) {
    mbar_expect_tx(&bar, (uint32_t)nb * 4u);
    bulk_copy_g2s(raw + off + hn, src + hn, (uint32_t)nb * 4u, &bar);
  }
  if (threadIdx.x < hn) raw[off + threadIdx.x] = __ldcg(src + threadIdx.x);
  if (threadIdx.x < tn) raw[off + hn + nb + threadIdx.x] = __ldcg(src + hn + nb + threadIdx.x);
  copy_table(tw, a.tw, N2);
  if (nb > 0) {
    long long spins = 0;
    while (!mbar_try_wait(&bar, 0))
      if (++spins > kWaitLimit) {
        failed = 1;
        break;
      }
  }
  __syncthreads();
  if (failed) {
    if (threadIdx.x == 0) {
      atomicExch(a.status + kStatErr, MSF_E_TIMEOUT);
      long long spins = 0;   // leave no copy in flight into shared memory (bounded)
      while (!mbar_try_wait(&bar, 0) && ++spins < kWaitLimit) {
      }
    }
    return;
  }
  if (a.zero) {   // the copy has landed: nothing reads these bytes any more
    int4* z4 = reinterpret_cast<int4*>(src + hn);
    for (int i = threadIdx.x; i < nb / 4; i += NT) z4[i] = make_int4(0, 0, 0, 0);
    if (threadIdx.x < hn) src[threadIdx.x] = 0;
    if (threadIdx.x < tn) src[hn + nb + threadIdx.x] = 0;
  }
  const int32_t* rb = raw + off;
  for (int e = threadIdx.x; e < G * N2; e += NT) {
    const int g = e / N2, z = e - g * N2;
    const float va = 2 * g < nrows ? (float)rb[2 * g * N2 + z] : 0.f;
    const float vb = 2 * g + 1 < nrows ? (float)rb[(2 * g + 1) * N2 + z] : 0.f;
    buf[z * S + g] = make_float2(va, vb);
  }
  __syncthreads();
  zs_fft_split<N2, G>(buf, tw, a, frame, p0);
}

struct SmYArgs {
  float2* C;
  int64_t Vh;
  int nh;
  const float2* tw; // w_n1^k
};

template <int N1>
__global__ void __launch_bounds__(kSmoothThreads) k_ys(SmYArgs a) {
  constexpr int W = kSmoothW, NT = kSmoothThreads;
  extern __shared__ __align__(16) float2 smem[];
  float2* tile = smem;             // [N1][W]
  float2* tw = tile + N1 * W;      // N1
  const int nh = a.nh;
  const int ntile = (nh + W - 1) / W;
  const int x = blockIdx.x / ntile;
  const int k0 = (blockIdx.x - x * ntile) * W;
  const int weff = min(W, nh - k0);
  float2* base = a.C + blockIdx.y * a.Vh + (int64_t)x * N1 * nh + k0;
  copy_table(tw, a.tw, N1);
  gather_batched<8, float2>(
      N1 * W,
      [&](int e) {
        const int y = e / W, w = e % W;
        return w < weff ? base[(int64_t)y * nh + w] : make_float2(0.f, 0.f);
      },
      [&](int e, float2 v) { tile[e] = v; });
  __syncthreads();
  mixed::fft2_lines<N1, W, W, 1, NT>(tile, tw);
  for (int e = threadIdx.x; e < N1 * W; e += NT) {
    const int y = e / W, w = e % W;
    if (w < weff) base[(int64_t)y * nh + w] = tile[e];
  }
}

struct SmXArgs {
  const float2* C;
  int64_t Vh;
  int nframes;
  double* sf;
  int64_t F;        // n1 * nh columns
  const float2* tw; // w_n0^k
};

// tile buffers of k_xs: two, filled by cp.async (frame b + 1's copy runs
// while frame b is transformed: 8 frames of 192^3 0.130 -> 0.073 ms, the
// batched systems 35.2k -> 37.0k frames/s) where they fit in 96 KB, else one
// filled through registers -- the 512-point lines keep two CTAs per SM (128
// registers, 70 KB): double-buffered, at one CTA per SM, the 512^3 stress
// grid fell from 709 to 550 frames/s.  The other lengths
// take no block bound (0): the compiler's own choice keeps them at 70-127
// registers, where a bound of one block took the 192-point lines from 71 to
// 137 (two CTAs per SM instead of three)
__host__ __device__ constexpr int xs_bufs(int n0) { return 2 * n0 * kSmoothW * 8 <= 96 * 1024 ? 2 : 1; }

template <int N0>
__global__ void __launch_bounds__(kSmoothThreads, xs_bufs(N0) == 1 ? 2 : 0) k_xs(SmXArgs a) {
  constexpr int W = kSmoothW, NT = kSmoothThreads;
  constexpr int A = mixed::Split2m<N0>::A, B = mixed::Split2m<N0>::B;
  constexpr int I2 = B * W, PER = (I2 + NT - 1) / NT;
  extern __shared__ __align__(16) float2 smem[];
  constexpr int NB = xs_bufs(N0);
  float2* tiles = smem;            // NB [N0][W] tiles: frame b in tile b % NB
  float2* tw = tiles + NB * N0 * W; // N0
  const int64_t f0 = (int64_t)blockIdx.x * W;
  const int weff = (int)min((int64_t)W, a.F - f0);
  copy_table(tw, a.tw, N0);
  // frame b's tile by cp.async (columns past F filled with zeros)
  auto fetch = [&](int b) {
    const float2* src = a.C + b * a.Vh + f0;
    float2* dst = tiles + (b % NB) * (N0 * W);
    for (int e = threadIdx.x; e < N0 * W; e += NT) {
      const int x = e / W, w = e % W;
      cp_async8(dst + e, src + (int64_t)x * a.F + (w < weff ? w : 0), w < weff ? 8 : 0);
    }
    cp_async_commit();
  };
  if (NB == 2 && a.nframes > 0) fetch(0);
  // pass-2 items (k1, column l) owned by this thread: X[k1 + B k2] in acc
  float acc[PER][A];
#pragma unroll
  for (int j = 0; j < PER; ++j)
#pragma unroll
    for (int k = 0; k < A; ++k) acc[j][k] = 0.f;
  for (int b = 0; b < a.nframes; ++b) {
    // two buffers: tile (b + 1) % 2 was frame b - 1's, which every thread
    // has finished (the barrier at the end of the previous iteration)
    if constexpr (NB == 1) {   // the register gather (128 registers, no spill)
      const float2* src = a.C + b * a.Vh + f0;
      gather_batched<8, float2>(
          N0 * W,
          [&](int e) {
            const int x = e / W, w = e % W;
            return w < weff ? __ldg(src + (int64_t)x * a.F + w) : make_float2(0.f, 0.f);
          },
          [&](int e, float2 v) { tiles[e] = v; });
    } else if (b + 1 < a.nframes) {
      fetch(b + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();   // every thread's copies of frame b have landed
    float2* tile = tiles + (b % NB) * (N0 * W);
    mixed::pass1<N0, W, W, 1, NT>(tile, tw);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int it = j * NT + threadIdx.x;
      if (I2 % NT == 0 || it < I2) {
        const int l = it % W, k1 = it / W;
        float2 r[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) r[n1] = tile[(A * k1 + n1) * W + l];
        mixed::reg_dftm<A>(r);
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) acc[j][k2] = fmaf(r[k2].x, r[k2].x, fmaf(r[k2].y, r[k2].y, acc[j][k2]));
      }
    }
    if (b == a.nframes - 1 || b % kPowerFlush == kPowerFlush - 1) {
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        const int it = j * NT + threadIdx.x;
        const int l = it % W, k1 = it / W;
        if ((I2 % NT == 0 || it < I2) && l < weff) {
          double* d = a.sf + (int64_t)k1 * a.F + f0 + l;
#pragma unroll
          for (int k2 = 0; k2 < A; ++k2) {
            double* dk = d + (int64_t)B * k2 * a.F;
            *dk = *dk + (double)acc[j][k2];
          }
        }
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) acc[j][k2] = 0.f;
      }
    }
    __syncthreads();   // frame b's tile is free for frame b + NB
  }
}

template <typename K>
void allow_smem_once(K kernel, bool& once, size_t bytes) {
  if (!once) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    once = true;
  }
}

template <int N2>
int launch_zs(const msf_plan* p, const void* grids, int kind, int nframes, int zero, cudaStream_t st) {
  constexpr int G = smooth_rows(N2);
  const size_t smem = ((size_t)N2 * (G + 1) + N2) * sizeof(float2);
  static bool once = false;
  allow_smem_once(k_zs<N2>, once, smem);
  SmZArgs a;
  a.grids = grids;
  a.kind = kind;
  a.V = grid_elems(p);
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.rows = (int64_t)p->n0 * p->n1;
  a.zero = kind == kGridI32 ? zero : 0;   // caller float grids are never zeroed
  a.tw = ws_ptr<float2>(p, p->off_tw[2]);
  a.status = ws_ptr<int>(p, p->off_status);
  const int64_t pairs = (a.rows + 1) / 2;
  {
    // int32 grids at a 16-byte aligned base take the bulk copies
    if (kind == kGridI32 && reinterpret_cast<uintptr_t>(grids) % 16 == 0) {
      constexpr int GB = bulk_rows(N2);
      static bool once_b = false;
      allow_smem_once(k_zs_bulk<N2>, once_b, zs_bulk_smem<N2>());
      k_zs_bulk<N2><<<dim3((unsigned)((pairs + GB - 1) / GB), nframes), kSmoothThreads, zs_bulk_smem<N2>(), st>>>(a);
      return launch_status();
    }
  }
  k_zs<N2><<<dim3((unsigned)((pairs + G - 1) / G), nframes), kSmoothThreads, smem, st>>>(a);
  return launch_status();
}

template <int N1>
int launch_ys(const msf_plan* p, int nframes, cudaStream_t st) {
  const size_t smem = ((size_t)N1 * kSmoothW + N1) * sizeof(float2);
  static bool once = false;
  allow_smem_once(k_ys<N1>, once, smem);
  SmYArgs a;
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.nh = p->nh;
  a.tw = ws_ptr<float2>(p, p->off_tw[1]);
  const int ntile = (p->nh + kSmoothW - 1) / kSmoothW;
  k_ys<N1><<<dim3(p->n0 * ntile, nframes), kSmoothThreads, smem, st>>>(a);
  return launch_status();
}

template <int N0>
int launch_xs(const msf_plan* p, int nframes, double* sf, cudaStream_t st) {
  const size_t smem = ((size_t)xs_bufs(N0) * N0 * kSmoothW + N0) * sizeof(float2);
  static bool once = false;
  allow_smem_once(k_xs<N0>, once, smem);
  SmXArgs a;
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.nframes = nframes;
  a.sf = sf;
  a.F = (int64_t)p->n1 * p->nh;
  a.tw = ws_ptr<float2>(p, p->off_tw[0]);
  k_xs<N0><<<(unsigned)((a.F + kSmoothW - 1) / kSmoothW), kSmoothThreads, smem, st>>>(a);
  return launch_status();
}

int zs_dispatch(const msf_plan* p, const void* grids, int kind, int nframes, int zero, cudaStream_t st) {
  switch (p->n2) {
#define X(N) case N: return launch_zs<N>(p, grids, kind, nframes, zero, st);
    MSF_SMOOTH_SIZES(X)
#undef X
  }
  return MSF_E_UNSUPPORTED;
}

}  // namespace

bool smooth_ok(int n) {
  switch (n) {
#define X(N) case N: return true;
    MSF_SMOOTH_SIZES(X)
#undef X
  }
  return false;
}

// z and y sweeps: grids (int32 / float32 / float64, frame-major) -> spectra
int smooth_stage_a(const msf_plan* p, const void* grids, int grid_kind, int nframes, int zero, cudaStream_t st) {
  const int s = zs_dispatch(p, grids, grid_kind, nframes, zero, st);
  if (s) return s;
  switch (p->n1) {
#define X(N) case N: return launch_ys<N>(p, nframes, st);
    MSF_SMOOTH_SIZES(X)
#undef X
  }
  return MSF_E_UNSUPPORTED;
}

// x sweep + |F|^2 + FP64 frame sum
int smooth_stage_b(const msf_plan* p, int nframes, double* sf, cudaStream_t st) {
  switch (p->n0) {
#define X(N) case N: return launch_xs<N>(p, nframes, sf, st);
    MSF_SMOOTH_SIZES(X)
#undef X
  }
  return MSF_E_UNSUPPORTED;
}

}  // namespace msf
