// msf_fused.cu -- the bucketed histogram + FFT chain for power-of-two grids.
//
// Per batch of frames (dens.py:277-318 in histogram form):
//   k_bucket_sort    every block bins its 4096 atoms (exact numpy.histogramdd
//                    search), counting-sorts them by x-plane in shared memory
//                    (lanes of a warp that share a plane merged with
//                    __match_any_sync) and writes (y*n2 + z, w) entries plus the
//                    plane offsets of its segment
//   k_plane_ct       one CTA per (frame, x): the plane's atoms, gathered from
//                    every segment, are added into the plane in shared memory
//                    (FP32 atomics on integer weights: exact and independent
//                    of order); then a two-pass register z-FFT of row pairs
//                    y = 2p, 2p+1 packed as x[2p] + i x[2p+1], a two-pass
//                    half-length y-FFT over p, and the 2-D real split
//                      E = (W[q,k] + conj W[-q,-k])/2, O = (W[q,k] - conj W[-q,-k])/(2i)
//                      Y[q,k] = E + w^q O, Y[q+P,k] = E - w^q O   (w = e^{-2 pi i/n1})
//                    written as the (n1, n2/2+1) half plane.  The density grid
//                    never goes to global memory.
//   k_xpower_tma     (msf_xtma.cu; k_xpower_ct without TMA) x-FFT of W spectrum
//                    columns for every frame of the batch, |F|^2 summed over
//                    the batch in FP32, one FP64 RMW of sf.
// All FFT lengths are template constants (msf_r2.cuh, msf_ct.cuh).
#include "msf_bins.cuh"
#include "msf_ct.cuh"
#include "msf_r2.cuh"

namespace msf {

// ------------------------------------------------------------- bucketing
// One kernel: every block takes kBucketAtoms consecutive atoms of one frame,
// bins them (exact numpy.histogramdd search), counting-sorts them by x-plane
// in shared memory and writes them to its own segment of the bucket array,
// plus the (n0 + 1) plane offsets of that segment.  No global atomics and no
// global scan: the plane kernel gathers plane x from every block's segment.
struct BucketArgs {
  DepArgs d;
  int* boff;        // (batch, nblk, n0 + 1) per-block plane offsets
  int2* bucket;     // (batch, nblk * kBucketAtoms) entries (y*n2 + z, w)
  int nblk;
};

constexpr int kBucketThreads = 256;
constexpr int kBucketIter = kBucketAtoms / kBucketThreads;

template <int MODE>
__global__ void __launch_bounds__(kBucketThreads) k_bucket_sort(BucketArgs a) {
  __shared__ int hist[kMaxN + 1];
  __shared__ int warp_sum[kBucketThreads / 32];
  const int frame = blockIdx.y;
  const int blk = blockIdx.x;
  const int n0 = a.d.n0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i <= n0; i += kBucketThreads) hist[i] = 0;
  __syncthreads();
  const int64_t a0 = (int64_t)blk * kBucketAtoms + tid;
  int key[kBucketIter], vox[kBucketIter], wt[kBucketIter];
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it) {
    const int64_t i = a0 + it * kBucketThreads;
    int b0 = -1, b1 = 0, b2 = 0, w = 0;
    const bool valid = (i < a.d.n_atoms) && atom_bins<MODE>(a.d, frame, i, b0, b1, b2, w);
    key[it] = valid ? b0 : -1;
    vox[it] = b1 * a.d.n2 + b2;
    wt[it] = w;
    if (valid) atomicAdd(&hist[b0], 1);
  }
  __syncthreads();
  // exclusive scan of hist[0..n0) -> offsets (each thread owns up to 4 consecutive planes)
  const int per = (n0 + kBucketThreads - 1) / kBucketThreads;
  int loc[kMaxN / kBucketThreads];
  int sum = 0;
#pragma unroll
  for (int j = 0; j < kMaxN / kBucketThreads; ++j) {
    const int idx = tid * per + j;
    loc[j] = (j < per && idx < n0) ? hist[idx] : 0;
    sum += loc[j];
  }
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  int before = 0;
#pragma unroll
  for (int w = 0; w < kBucketThreads / 32; ++w) before += (w < warp) ? warp_sum[w] : 0;
  int run = before + incl - sum;
  int* bo = a.boff + ((int64_t)frame * a.nblk + blk) * (n0 + 1);
  __syncthreads();                       // every thread has read its counts
#pragma unroll
  for (int j = 0; j < kMaxN / kBucketThreads; ++j) {
    const int idx = tid * per + j;
    if (j < per && idx < n0) {
      hist[idx] = run;                   // becomes the placement cursor
      bo[idx] = run;
      run += loc[j];
    }
  }
  if (tid == kBucketThreads - 1) bo[n0] = before + incl;
  __syncthreads();
  // placement: one independent shared-memory atomic per atom, so the
  // iterations of a thread overlap instead of forming a chain
  int2* bk = a.bucket + ((int64_t)frame * a.nblk + blk) * kBucketAtoms;
  int slot[kBucketIter];
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it) slot[it] = key[it] >= 0 ? atomicAdd(&hist[key[it]], 1) : -1;
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it)
    if (slot[it] >= 0) bk[slot[it]] = make_int2(vox[it], wt[it]);
}

// ----------------------------------------------------------- plane (z, y)
struct PlaneCtArgs {
  // bucket source
  const int* boff;
  const int2* bucket;
  int nblk;
  int n0;
  // grid source
  const void* grids;
  int grid_kind;
  int64_t V;
  // output
  float2* C;
  int64_t Vh;
  const float2* twz;
  const float2* twp;
  const float2* twy;
};

template <int N1, int N2>
struct PlaneShape {
  static constexpr int P = N1 / 2;
  static constexpr int SP = P + 1;      // odd line stride: conflict-free columns
  static constexpr int NH = N2 / 2 + 1;
  static constexpr int NT = (N2 * P >= 4096) ? 512 : 256;
  // plane, twiddles, then the segment tables of the bucket gather
  static constexpr size_t SMEM = (size_t)N2 * SP * sizeof(float2) + (size_t)(N2 + 2 * P) * sizeof(float2) +
                                 (size_t)(2 * NT + 1 + NT / 32) * sizeof(int);
};

// SRC 0: atoms from the plane's bucket; SRC 1: a dense grid (int32/float32/float64)
// Registers capped so that one x-pass CTA fits on the SM beside a plane CTA
// (the two kernels overlap on different streams).
template <int N1, int N2, int SRC>
__global__ void __maxnreg__((PlaneShape<N1, N2>::NT >= 512 ? 80 : 128)) k_plane_ct(PlaneCtArgs a) {
  using S = PlaneShape<N1, N2>;
  constexpr int P = S::P, SP = S::SP, NH = S::NH, NT = S::NT;
  extern __shared__ float2 smem[];
  float2* buf = smem;                 // [N2][SP], z major
  float2* twz = buf + N2 * SP;        // N2
  float2* twp = twz + N2;             // P
  float2* twy = twp + P;              // P (w^q, q < P)
  int* bufi = reinterpret_cast<int*>(buf);
  float* buff = reinterpret_cast<float*>(buf);
  const int x = blockIdx.x;
  const int frame = blockIdx.y;
  for (int i = threadIdx.x; i < N2; i += NT) twz[i] = a.twz[i];
  for (int i = threadIdx.x; i < P; i += NT) { twp[i] = a.twp[i]; twy[i] = a.twy[i]; }
  if (SRC == 0) {
    // The plane's atoms sit in one segment per bucketing block.  Thread t
    // loads segment t's bounds first (the loads overlap the zeroing below);
    // a block scan of the segment lengths then lets every thread fetch one
    // entry of the concatenated segments in a single round of loads.
    int* seg_start = reinterpret_cast<int*>(twy + P);   // NT + 1 ints
    int* seg_lo = seg_start + NT + 1;                   // NT ints
    int* warp_sum = seg_lo + NT;                        // NT / 32 ints
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool flat = a.nblk <= NT;
    int lo = 0, cnt = 0;
    if (flat && tid < a.nblk) {
      const int* bo = a.boff + ((int64_t)frame * a.nblk + tid) * (a.n0 + 1);
      lo = bo[x];
      cnt = bo[x + 1] - lo;
    }
    int4* z4 = reinterpret_cast<int4*>(buf);
    for (int i = tid; i < N2 * SP / 2; i += NT) z4[i] = make_int4(0, 0, 0, 0);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += warp_sum[w];
    seg_start[tid] = before + incl - cnt;
    seg_lo[tid] = lo;
    if (tid == NT - 1) seg_start[NT] = before + incl;
    __syncthreads();
    // integer weights summed in FP32: exact (and order-independent) while a
    // voxel's total stays below 2^24 electrons
    if (flat) {
      const int total = seg_start[NT];
      for (int e = tid; e < total; e += NT) {
        int s0 = 0, s1 = a.nblk - 1;     // last segment with seg_start <= e
        while (s0 < s1) {
          const int m = (s0 + s1 + 1) >> 1;
          if (seg_start[m] <= e) s0 = m; else s1 = m - 1;
        }
        const int2 v = a.bucket[((int64_t)frame * a.nblk + s0) * kBucketAtoms + seg_lo[s0] + (e - seg_start[s0])];
        const int y = v.x / N2, z = v.x % N2;
        atomicAdd(buff + 2 * (z * SP + (y >> 1)) + (y & 1), (float)v.y);
      }
    } else {
      for (int blk = warp; blk < a.nblk; blk += NT / 32) {
        const int* bo = a.boff + ((int64_t)frame * a.nblk + blk) * (a.n0 + 1);
        const int e0 = bo[x], e1 = bo[x + 1];
        const int2* bk = a.bucket + ((int64_t)frame * a.nblk + blk) * kBucketAtoms;
        for (int e = e0 + lane; e < e1; e += 32) {
          const int2 v = bk[e];
          const int y = v.x / N2, z = v.x % N2;
          atomicAdd(buff + 2 * (z * SP + (y >> 1)) + (y & 1), (float)v.y);
        }
      }
    }
  } else {
    const int64_t g0 = frame * a.V + (int64_t)x * N1 * N2;
    for (int e = threadIdx.x; e < N1 * N2; e += NT) {
      const int y = e / N2, z = e % N2;
      float v;
      if (a.grid_kind == kGridI32) v = (float)__ldg(static_cast<const int32_t*>(a.grids) + g0 + e);
      else if (a.grid_kind == kGridF32) v = __ldg(static_cast<const float*>(a.grids) + g0 + e);
      else v = (float)__ldg(static_cast<const double*>(a.grids) + g0 + e);
      buff[2 * (z * SP + (y >> 1)) + (y & 1)] = v;
    }
  }
  __syncthreads();
  r2::fft2_lines<N2, P, SP, 1, NT>(buf, twz);    // z: lines = pairs p, samples stride SP
  r2::fft2_lines<P, N2, 1, SP, NT>(buf, twp);    // half y: lines = kz, samples stride 1
  float2* out = a.C + frame * a.Vh + (int64_t)x * N1 * NH;
  // 2-D real split.  Columns k < N2/2: thread (k = tid % KC, g = tid / KC)
  // takes rows q = g, g + QS, ... so addresses advance by constants; a warp
  // covers consecutive k (coalesced stores, stride-SP shared loads).  The
  // Nyquist column k = N2/2 follows.
  constexpr int KC = N2 / 2 < NT ? N2 / 2 : NT;   // columns per sweep
  constexpr int QS = NT / KC;                     // rows advanced per step
  auto split = [&](int q, int k) {
    const int kn = (N2 - k) & (N2 - 1);
    const int qn = (P - q) & (P - 1);
    const float2 w = buf[k * SP + q];
    const float2 wm = cconj(buf[kn * SP + qn]);
    const float2 E = cscale(cadd(w, wm), 0.5f);
    const float2 O = cscale(cmi(csub(w, wm)), 0.5f);
    const float2 t = cmul(twy[q], O);
    out[q * NH + k] = cadd(E, t);
    out[(q + P) * NH + k] = csub(E, t);
  };
  for (int k = threadIdx.x % KC; k < N2 / 2; k += KC) {
#pragma unroll 4
    for (int q = threadIdx.x / KC; q < P; q += QS) split(q, k);
  }
  for (int q = threadIdx.x; q < P; q += NT) split(q, N2 / 2);
}

// ------------------------------------------------- x pass + |F|^2 + sum
struct XCtArgs {
  const float2* C;
  int64_t Vh;
  int nframes;
  double* sf;
  int64_t F;          // n1 * nh columns
  const float2* twx;
};

template <int N0, int W>
struct XShape {
  static constexpr int NT = 256;
  static constexpr int EPT = N0 * W / NT;
  static constexpr size_t SMEM = (size_t)(N0 * W + N0) * sizeof(float2);
};

template <int N0, int W>
__global__ void __launch_bounds__(XShape<N0, W>::NT) k_xpower_ct(XCtArgs a) {
  using S = XShape<N0, W>;
  constexpr int NT = S::NT, EPT = S::EPT;
  static_assert(EPT * NT == N0 * W, "tile must split evenly over the threads");
  extern __shared__ float2 smem[];
  float2* tile = smem;            // [N0][W]
  float2* tw = tile + N0 * W;
  const int64_t f0 = (int64_t)blockIdx.x * W;
  const int weff = (int)min((int64_t)W, a.F - f0);
  for (int i = threadIdx.x; i < N0; i += NT) tw[i] = a.twx[i];
  float acc[EPT];
#pragma unroll
  for (int i = 0; i < EPT; ++i) acc[i] = 0.f;
  for (int b = 0; b < a.nframes; ++b) {
    const float2* src = a.C + b * a.Vh + f0;
    __syncthreads();
#pragma unroll 4
    for (int e = threadIdx.x; e < N0 * W; e += NT) {
      const int x = e / W, w = e % W;
      tile[ct::pos<N0>(x) * W + w] = (w < weff) ? __ldg(src + (int64_t)x * a.F + w) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    ct::dit<N0, W, W, 1, NT, true>(tile, tw);
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const float2 v = tile[threadIdx.x + i * NT];
      acc[i] = fmaf(v.x, v.x, fmaf(v.y, v.y, acc[i]));
    }
  }
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const int e = threadIdx.x + i * NT;
    const int x = e / W, w = e % W;
    if (w < weff) {
      double* d = a.sf + (int64_t)x * a.F + f0 + w;
      *d = *d + (double)acc[i];
    }
  }
}

// ---------------------------------------------------------------- dispatch
template <typename K>
static void allow_smem_once(K kernel, bool& once) {
  if (!once) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    once = true;
  }
}

template <int N1, int N2>
static int launch_plane_ct(const PlaneCtArgs& a, int src, int n0, int nframes, cudaStream_t st) {
  using S = PlaneShape<N1, N2>;
  static bool once0 = false, once1 = false;
  dim3 grid(n0, nframes);
  if (src == 0) {
    allow_smem_once(k_plane_ct<N1, N2, 0>, once0);
    k_plane_ct<N1, N2, 0><<<grid, S::NT, S::SMEM, st>>>(a);
  } else {
    allow_smem_once(k_plane_ct<N1, N2, 1>, once1);
    k_plane_ct<N1, N2, 1><<<grid, S::NT, S::SMEM, st>>>(a);
  }
  return launch_status();
}

#define MSF_PLANE_CASES(X) \
  X(32, 32) X(64, 32) X(128, 32) X(256, 32) X(512, 32) \
  X(32, 64) X(64, 64) X(128, 64) X(256, 64) X(512, 64) \
  X(32, 128) X(64, 128) X(128, 128) X(256, 128) \
  X(32, 256) X(64, 256) X(128, 256)

static int plane_ct(const PlaneCtArgs& a, int n1, int n2, int src, int n0, int nframes, cudaStream_t st) {
#define X(A, B) if (n1 == A && n2 == B) return launch_plane_ct<A, B>(a, src, n0, nframes, st);
  MSF_PLANE_CASES(X)
#undef X
  return MSF_E_UNSUPPORTED;
}

bool ct_plane_ok(int n1, int n2) {
#define X(A, B) if (n1 == A && n2 == B) return true;
  MSF_PLANE_CASES(X)
#undef X
  return false;
}

template <int N0, int W>
static int launch_x_ct(const XCtArgs& a, cudaStream_t st) {
  using S = XShape<N0, W>;
  static bool once = false;
  allow_smem_once(k_xpower_ct<N0, W>, once);
  const unsigned nblk = (unsigned)((a.F + W - 1) / W);
  k_xpower_ct<N0, W><<<nblk, S::NT, S::SMEM, st>>>(a);
  return launch_status();
}

#define MSF_X_CASES(X) \
  X(32, 32) X(64, 32) X(64, 16) X(128, 32) X(128, 16) X(256, 16) X(256, 8) X(512, 8) X(1024, 4)

static int x_ct(const XCtArgs& a, int n0, int w, cudaStream_t st) {
#define X(A, B) if (n0 == A && w == B) return launch_x_ct<A, B>(a, st);
  MSF_X_CASES(X)
#undef X
  return MSF_E_UNSUPPORTED;
}

int ct_x_width(int n0, int requested) {
  int best = 0;
#define X(A, B) if (n0 == A && (requested == 0 ? B > best : B == requested)) best = B;
  MSF_X_CASES(X)
#undef X
  return best;
}

size_t ct_plane_smem(int n1, int n2) {
  return (size_t)n2 * (n1 / 2 + 1) * sizeof(float2) + (size_t)(n2 + n1) * sizeof(float2);
}

static BucketArgs bucket_args(const msf_plan* p) {
  BucketArgs b;
  b.d = dep_args(p);
  b.boff = ws_ptr<int>(p, p->off_offsets);
  b.bucket = ws_ptr<int2>(p, p->off_bucket);
  b.nblk = (int)((p->max_atoms + kBucketAtoms - 1) / kBucketAtoms);
  return b;
}

int fused_bucket_batch(const msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int nframes, int64_t frame_stride, const double* scale,
                       int flags, cudaStream_t st) {
  if (n_atoms > p->max_atoms) return MSF_E_WORKSPACE;
  BucketArgs b = bucket_args(p);
  b.d.pos = pos;
  b.d.w = weights;
  b.d.n_atoms = n_atoms;
  b.d.frame_stride = frame_stride;
  b.d.scale = scale;
  b.d.flags = flags;
  if (b.nblk < 1) b.nblk = 1;
  // every block of the plan's capacity runs, so blocks past n_atoms publish
  // empty segments and the plane kernel never reads stale offsets
  dim3 grid((unsigned)b.nblk, nframes);
  switch (deposit_mode(layout, scale || (flags & MSF_WRAP))) {
    case 0: k_bucket_sort<0><<<grid, kBucketThreads, 0, st>>>(b); break;
    case 1: k_bucket_sort<1><<<grid, kBucketThreads, 0, st>>>(b); break;
    case 2: k_bucket_sort<2><<<grid, kBucketThreads, 0, st>>>(b); break;
    case 3: k_bucket_sort<3><<<grid, kBucketThreads, 0, st>>>(b); break;
    default: k_bucket_sort<4><<<grid, kBucketThreads, 0, st>>>(b); break;
  }
  return launch_status();
}

// The bucketed atoms of one frame added into a dense int32 grid (one CTA per
// x-plane): what k_plane_ct deposits in shared memory, made visible.
__global__ void __launch_bounds__(256) k_bucket_to_grid(BucketArgs a, int64_t plane, int32_t* grid) {
  const int x = blockIdx.x;
  const int n0 = a.d.n0;
  for (int blk = 0; blk < a.nblk; ++blk) {
    const int* bo = a.boff + (int64_t)blk * (n0 + 1);
    const int2* bk = a.bucket + (int64_t)blk * kBucketAtoms;
    for (int e = bo[x] + threadIdx.x; e < bo[x + 1]; e += blockDim.x) {
      const int2 v = bk[e];
      atomicAdd(grid + x * plane + v.x, v.y);
    }
  }
}

int bucket_grid(const msf_plan* p, const void* pos, const int32_t* weights, int layout, int64_t n_atoms,
                const double* scale, int flags, int32_t* grid, cudaStream_t st) {
  const int64_t fstride = layout == kLayoutF32x4 ? n_atoms : 3 * n_atoms;
  int s = fused_bucket_batch(p, pos, weights, layout, n_atoms, 1, fstride, scale, flags, st);
  if (s) return s;
  BucketArgs b = bucket_args(p);
  if (b.nblk < 1) b.nblk = 1;
  k_bucket_to_grid<<<p->n0, 256, 0, st>>>(b, (int64_t)p->n1 * p->n2, grid);
  return launch_status();
}

static PlaneCtArgs plane_args(const msf_plan* p) {
  PlaneCtArgs a;
  memset(&a, 0, sizeof(a));
  a.boff = ws_ptr<int>(p, p->off_offsets);
  a.bucket = ws_ptr<int2>(p, p->off_bucket);
  a.nblk = (int)((p->max_atoms + kBucketAtoms - 1) / kBucketAtoms);
  if (a.nblk < 1) a.nblk = 1;
  a.n0 = p->n0;
  a.V = grid_elems(p);
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.twz = ws_ptr<float2>(p, p->off_tw[2]);
  a.twp = ws_ptr<float2>(p, p->off_twp);
  a.twy = ws_ptr<float2>(p, p->off_tw[1]);
  return a;
}

int fused_plane_batch(const msf_plan* p, const void* grids, int grid_kind, int nframes, cudaStream_t st,
                      int buf) {
  PlaneCtArgs a = plane_args(p);
  if (buf) a.C = ws_ptr<float2>(p, p->off_cplx2);
  a.grids = grids;
  a.grid_kind = grid_kind;
  return plane_ct(a, p->n1, p->n2, grids ? 1 : 0, p->n0, nframes, st);
}

int fused_x_batch(const msf_plan* p, int nframes, double* sf, cudaStream_t st, int buf) {
  if (p->xtma_ready) return xtma_batch(p, nframes, sf, st, buf);
  XCtArgs a;
  a.C = ws_ptr<float2>(p, buf ? p->off_cplx2 : p->off_cplx);
  a.Vh = half_elems(p);
  a.nframes = nframes;
  a.sf = sf;
  a.F = (int64_t)p->n1 * p->nh;
  a.twx = ws_ptr<float2>(p, p->off_tw[0]);
  return x_ct(a, p->n0, p->tile_w, st);
}

}  // namespace msf

using namespace msf;

extern "C" int msf_hist_bucket_grid(const msf_plan* p, int32_t layout, const void* pos,
                                    const int32_t* weights, int64_t n_atoms, const double* scale,
                                    int32_t flags, int32_t* grid, msf_stream_t stream) {
  if (!p || !grid || n_atoms < 0) return MSF_E_INVALID;
  if (layout < kLayoutF32x4 || layout > kLayoutF32xyz || (flags & ~MSF_WRAP)) return MSF_E_INVALID;
  if (n_atoms > 0 && (!pos || (layout != kLayoutF32x4 && !weights))) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  if (p->variant != 3) return MSF_E_UNSUPPORTED;
  return bucket_grid(p, pos, weights, layout, n_atoms, scale, flags, grid,
                     reinterpret_cast<cudaStream_t>(stream));
}
