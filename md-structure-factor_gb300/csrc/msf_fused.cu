// msf_fused.cu -- the bucketed histogram + FFT chain for power-of-two grids.
//
// Per batch of frames (dens.py:277-318 in histogram form):
//   k_bucket_count   bins of every atom (exact numpy.histogramdd search),
//                    per-x-plane atom counts (shared-memory histogram, one
//                    global atomic per non-empty plane per block)
//   k_bucket_scan    exclusive scan of the counts -> plane offsets
//   k_bucket_fill    bins again; each atom appends (y*n2 + z, w) to its
//                    plane's bucket, lanes of a warp that share a plane
//                    taking one atomicAdd on the cursor (__match_any_sync)
//   k_plane_ct       one CTA per (frame, x): the plane's atoms are added into
//                    an int32 plane in shared memory (integer atomics, so the
//                    grid is exact and independent of order), placed at the
//                    digit-reversed positions of both FFT axes; then a DIT
//                    z-FFT of row pairs y = 2p, 2p+1 packed as x[2p] + i x[2p+1],
//                    a DIT half-length y-FFT over p, and the 2-D real split
//                      E = (W[q,k] + conj W[-q,-k])/2, O = (W[q,k] - conj W[-q,-k])/(2i)
//                      Y[q,k] = E + w^q O, Y[q+P,k] = E - w^q O   (w = e^{-2 pi i/n1})
//                    written as the (n1, n2/2+1) half plane.  The density grid
//                    never goes to global memory.
//   k_xpower_ct      x-FFT of W spectrum columns for every frame of the batch,
//                    |F|^2 summed over the batch in FP32, one FP64 RMW of sf.
// All FFT lengths are template constants (msf_ct.cuh).
#include "msf_bins.cuh"
#include "msf_ct.cuh"

namespace msf {

// ------------------------------------------------------------- bucketing
struct BucketArgs {
  DepArgs d;
  int* counts;      // (batch, n0)
  int* offsets;     // (batch, n0 + 1)
  int* cursor;      // (batch, n0)
  int2* bucket;     // (batch, max_atoms)
  int64_t bucket_stride;
};

// Each block owns kBucketIter * 256 consecutive atoms of one frame and talks
// to the global per-plane counters once per plane (not once per atom), so the
// n0 counters see ~n_atoms / 4096 atomics each whatever the atom order.
constexpr int kBucketThreads = 256;
constexpr int kBucketIter = 16;
constexpr int kBucketAtoms = kBucketThreads * kBucketIter;

template <int MODE>
__global__ void __launch_bounds__(kBucketThreads) k_bucket_count(BucketArgs a) {
  __shared__ int hist[kMaxN];
  const int frame = blockIdx.y;
  const int n0 = a.d.n0;
  for (int i = threadIdx.x; i < n0; i += kBucketThreads) hist[i] = 0;
  __syncthreads();
  const int64_t a0 = (int64_t)blockIdx.x * kBucketAtoms + threadIdx.x;
#pragma unroll 4
  for (int it = 0; it < kBucketIter; ++it) {
    const int64_t i = a0 + it * kBucketThreads;
    int b0 = -1, b1, b2, w;
    if (i < a.d.n_atoms && atom_bins<MODE>(a.d, frame, i, b0, b1, b2, w)) atomicAdd(&hist[b0], 1);
  }
  __syncthreads();
  int* c = a.counts + (int64_t)frame * n0;
  for (int k = threadIdx.x; k < n0; k += kBucketThreads)
    if (hist[k]) atomicAdd(c + k, hist[k]);
}

// one block per frame; n0 <= kMaxN
__global__ void __launch_bounds__(1024) k_bucket_scan(BucketArgs a) {
  __shared__ int sh[kMaxN];
  __shared__ int warp_tot[32];
  const int frame = blockIdx.x;
  const int n0 = a.d.n0;
  int* c = a.counts + (int64_t)frame * n0;
  int* off = a.offsets + (int64_t)frame * (n0 + 1);
  int* cur = a.cursor + (int64_t)frame * n0;
  const int t = threadIdx.x;
  const int v = t < n0 ? c[t] : 0;
  // inclusive warp scan
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if ((t & 31) >= o) x += y;
  }
  if ((t & 31) == 31) warp_tot[t >> 5] = x;
  __syncthreads();
  if (t < 32) {
    int w = (t < (int)(blockDim.x >> 5)) ? warp_tot[t] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (t >= o) w += y;
    }
    warp_tot[t] = w;
  }
  __syncthreads();
  const int incl = x + ((t >> 5) ? warp_tot[(t >> 5) - 1] : 0);
  if (t < n0) {
    sh[t] = incl - v;
    off[t] = incl - v;
    cur[t] = incl - v;
    c[t] = 0;              // counts ready for the next batch
  }
  if (t == n0 - 1) off[n0] = incl;
}

// Same atoms per block as k_bucket_count: count the block's atoms per plane
// in shared memory, reserve one contiguous range per plane with a single
// global atomic, then place every atom with a shared-memory atomic.  Lanes of
// a warp that share a plane are first merged with __match_any_sync.
template <int MODE>
__global__ void __launch_bounds__(kBucketThreads) k_bucket_fill(BucketArgs a) {
  __shared__ int slot[kMaxN];
  const int frame = blockIdx.y;
  const int n0 = a.d.n0;
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < n0; i += kBucketThreads) slot[i] = 0;
  __syncthreads();
  const int64_t a0 = (int64_t)blockIdx.x * kBucketAtoms + threadIdx.x;
  int key[kBucketIter], vox[kBucketIter], wt[kBucketIter];
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it) {
    const int64_t i = a0 + it * kBucketThreads;
    int b0 = -1, b1 = 0, b2 = 0, w = 0;
    const bool valid = (i < a.d.n_atoms) && atom_bins<MODE>(a.d, frame, i, b0, b1, b2, w);
    key[it] = valid ? b0 : -1;
    vox[it] = b1 * a.d.n2 + b2;
    wt[it] = w;
    if (valid) atomicAdd(&slot[b0], 1);
  }
  __syncthreads();
  int* cur = a.cursor + (int64_t)frame * n0;
  for (int k = threadIdx.x; k < n0; k += kBucketThreads)
    if (slot[k]) slot[k] = atomicAdd(cur + k, slot[k]);
  __syncthreads();
  int2* bk = a.bucket + frame * a.bucket_stride;
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it) {
    const bool valid = key[it] >= 0;
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const unsigned peers = __match_any_sync(vm, key[it]);
      const int leader = __ffs(peers) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&slot[key[it]], __popc(peers));
      base = __shfl_sync(peers, base, leader);
      bk[base + __popc(peers & ((1u << lane) - 1u))] = make_int2(vox[it], wt[it]);
    }
  }
}

// ----------------------------------------------------------- plane (z, y)
struct PlaneCtArgs {
  // bucket source
  const int* offsets;
  const int2* bucket;
  int64_t bucket_stride;
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
  static constexpr int NT = (N2 * P >= 16384) ? 1024 : ((N2 * P >= 4096) ? 512 : 256);
  static constexpr size_t SMEM = (size_t)N2 * SP * sizeof(float2) + (size_t)(N2 + 2 * P) * sizeof(float2);
};

// SRC 0: atoms from the plane's bucket; SRC 1: a dense grid (int32/float32/float64)
template <int N1, int N2, int SRC>
__global__ void __launch_bounds__(PlaneShape<N1, N2>::NT) k_plane_ct(PlaneCtArgs a) {
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
    int4* z4 = reinterpret_cast<int4*>(buf);
    for (int i = threadIdx.x; i < N2 * SP / 2; i += NT) z4[i] = make_int4(0, 0, 0, 0);
    __syncthreads();
    const int* off = a.offsets + (int64_t)frame * (a.n0 + 1);
    const int e0 = off[x], e1 = off[x + 1];
    const int2* bk = a.bucket + frame * a.bucket_stride;
    for (int e = e0 + threadIdx.x; e < e1; e += NT) {
      const int2 v = bk[e];
      const int y = v.x / N2, z = v.x % N2;
      atomicAdd(bufi + 2 * (ct::pos<N2>(z) * SP + ct::pos<P>(y >> 1)) + (y & 1), v.y);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * N2 * SP; i += NT) buff[i] = (float)bufi[i];
  } else {
    const int64_t g0 = frame * a.V + (int64_t)x * N1 * N2;
    for (int e = threadIdx.x; e < N1 * N2; e += NT) {
      const int y = e / N2, z = e % N2;
      float v;
      if (a.grid_kind == kGridI32) v = (float)__ldg(static_cast<const int32_t*>(a.grids) + g0 + e);
      else if (a.grid_kind == kGridF32) v = __ldg(static_cast<const float*>(a.grids) + g0 + e);
      else v = (float)__ldg(static_cast<const double*>(a.grids) + g0 + e);
      buff[2 * (ct::pos<N2>(z) * SP + ct::pos<P>(y >> 1)) + (y & 1)] = v;
    }
  }
  __syncthreads();
  ct::dit<N2, P, SP, 1, NT, true>(buf, twz);    // z: lines = pairs p, elements stride SP
  ct::dit<P, N2, 1, SP, NT, true>(buf, twp);    // half y: lines = kz, elements stride 1
  float2* out = a.C + frame * a.Vh + (int64_t)x * N1 * NH;
  for (int e = threadIdx.x; e < P * NH; e += NT) {
    const int q = e / NH, k = e % NH;
    const int kn = (N2 - k) & (N2 - 1);
    const int qn = (P - q) & (P - 1);
    const float2 w = buf[k * SP + q];
    const float2 wm = cconj(buf[kn * SP + qn]);
    const float2 E = cscale(cadd(w, wm), 0.5f);
    const float2 O = cscale(cmi(csub(w, wm)), 0.5f);
    const float2 t = cmul(twy[q], O);
    out[q * NH + k] = cadd(E, t);
    out[(q + P) * NH + k] = csub(E, t);
  }
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
  b.counts = ws_ptr<int>(p, p->off_counts);
  b.offsets = ws_ptr<int>(p, p->off_offsets);
  b.cursor = ws_ptr<int>(p, p->off_cursor);
  b.bucket = ws_ptr<int2>(p, p->off_bucket);
  b.bucket_stride = p->max_atoms;
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
  const int64_t nb = (n_atoms + kBucketAtoms - 1) / kBucketAtoms;
  if (nb > 0x7fffffff) return MSF_E_UNSUPPORTED;
  if (nb > 0) {
    dim3 grid((unsigned)nb, nframes);
    switch (deposit_mode(layout, scale || (flags & MSF_WRAP))) {
      case 0: k_bucket_count<0><<<grid, kBucketThreads, 0, st>>>(b); break;
      case 1: k_bucket_count<1><<<grid, kBucketThreads, 0, st>>>(b); break;
      case 2: k_bucket_count<2><<<grid, kBucketThreads, 0, st>>>(b); break;
      case 3: k_bucket_count<3><<<grid, kBucketThreads, 0, st>>>(b); break;
      default: k_bucket_count<4><<<grid, kBucketThreads, 0, st>>>(b); break;
    }
  }
  k_bucket_scan<<<nframes, 1024, 0, st>>>(b);
  if (nb > 0) {
    dim3 grid((unsigned)nb, nframes);
    switch (deposit_mode(layout, scale || (flags & MSF_WRAP))) {
      case 0: k_bucket_fill<0><<<grid, kBucketThreads, 0, st>>>(b); break;
      case 1: k_bucket_fill<1><<<grid, kBucketThreads, 0, st>>>(b); break;
      case 2: k_bucket_fill<2><<<grid, kBucketThreads, 0, st>>>(b); break;
      case 3: k_bucket_fill<3><<<grid, kBucketThreads, 0, st>>>(b); break;
      default: k_bucket_fill<4><<<grid, kBucketThreads, 0, st>>>(b); break;
    }
  }
  return launch_status();
}

// The bucketed atoms of one frame added into a dense int32 grid (one CTA per
// x-plane): what k_plane_ct deposits in shared memory, made visible.
__global__ void __launch_bounds__(256) k_bucket_to_grid(const int* offsets, const int2* bucket, int n0,
                                                        int64_t plane, int32_t* grid) {
  const int x = blockIdx.x;
  for (int e = offsets[x] + threadIdx.x; e < offsets[x + 1]; e += blockDim.x) {
    const int2 v = bucket[e];
    atomicAdd(grid + x * plane + v.x, v.y);
  }
}

int bucket_grid(const msf_plan* p, const void* pos, const int32_t* weights, int layout, int64_t n_atoms,
                const double* scale, int flags, int32_t* grid, cudaStream_t st) {
  const int64_t fstride = layout == kLayoutF32x4 ? n_atoms : 3 * n_atoms;
  int s = fused_bucket_batch(p, pos, weights, layout, n_atoms, 1, fstride, scale, flags, st);
  if (s) return s;
  k_bucket_to_grid<<<p->n0, 256, 0, st>>>(ws_ptr<int>(p, p->off_offsets), ws_ptr<int2>(p, p->off_bucket),
                                           p->n0, (int64_t)p->n1 * p->n2, grid);
  return launch_status();
}

static PlaneCtArgs plane_args(const msf_plan* p) {
  PlaneCtArgs a;
  memset(&a, 0, sizeof(a));
  a.offsets = ws_ptr<int>(p, p->off_offsets);
  a.bucket = ws_ptr<int2>(p, p->off_bucket);
  a.bucket_stride = p->max_atoms;
  a.n0 = p->n0;
  a.V = grid_elems(p);
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.twz = ws_ptr<float2>(p, p->off_tw[2]);
  a.twp = ws_ptr<float2>(p, p->off_twp);
  a.twy = ws_ptr<float2>(p, p->off_tw[1]);
  return a;
}

int fused_plane_batch(const msf_plan* p, const void* grids, int grid_kind, int nframes, cudaStream_t st) {
  PlaneCtArgs a = plane_args(p);
  a.grids = grids;
  a.grid_kind = grid_kind;
  return plane_ct(a, p->n1, p->n2, grids ? 1 : 0, p->n0, nframes, st);
}

int fused_x_batch(const msf_plan* p, int nframes, double* sf, cudaStream_t st) {
  if (p->xtma_ready) return xtma_batch(p, nframes, sf, st);
  XCtArgs a;
  a.C = ws_ptr<float2>(p, p->off_cplx);
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
