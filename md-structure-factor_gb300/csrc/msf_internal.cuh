// msf_internal.cuh -- shared definitions of libmsf (GB300, sm_103a).
//
// Plan layout, workspace layout, status handling and the shared-memory
// mixed-radix FFT engine used by every FFT kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "msf.h"

namespace msf {

constexpr int kMaxStages = 12;
constexpr int kMaxN = 1024;      // largest supported axis length
constexpr int kStatusWords = 16; // device status block (int32)
// The x passes sum |F|^2 over the frames of a batch in FP32 registers and add
// that partial sum to the FP64 sf every kPowerFlush frames (and after the
// batch's last frame).  A recursive FP32 sum of k positive terms is within
// (k-1)*2^-24 of the exact sum relative to itself, so 32 frames bound the
// in-register error by 1.9e-6 of each voxel's value, whatever the batch size
// (plans accept up to 256 frames per batch); every longer sum is FP64.
constexpr int kPowerFlush = 32;
constexpr int kBucketAtoms = 2048; // atoms per bucketing block (bucketed variant)

// Device status words (latched by kernels, read by msf_plan_status).
enum StatusWord { kStatErr = 0, kStatBadAtom = 1, kStatBadIndex = 2 };

// One FFT axis: length n factored into DIF stages.  Stage s has radix R[s]
// and sub-length m[s] = span_s / R[s] (span_0 = n, span_{s+1} = m[s]).
// After all stages frequency k sits at position pos(k) = sum_s d_s * m[s],
// where d_s are the mixed-radix digits of k (least significant first).
struct AxisPlan {
  int n;
  int nst;
  int generic;             // 1 when a stage has a radix outside {2,3,4,5,8}
  int R[kMaxStages];
  int m[kMaxStages];
};

AxisPlan make_axis(int n);

}  // namespace msf

// The plan object behind the opaque C handle.
struct msf_plan {
  int n0, n1, n2, nh;
  int batch;
  double box[3];
  int variant;          // 1 fused plane, 2 split
  int tile_w;           // x-pass / y-pass columns per tile
  int rows_per_block;   // z-pass row pairs per block
  int deposit_block;    // deposit threads per block
  int plane_threads;    // threads of the fused plane kernel
  msf::AxisPlan ax[3];  // x (n0), y (n1), z (n2)
  msf::AxisPlan axp;    // y half length P = n1/2 (fused plane variant)
  // workspace layout (byte offsets)
  size_t off_status, off_tw[3], off_twp, off_pos[3], off_posp;
  size_t off_edges_d, off_edges_flo, off_edges_fhi;
  size_t off_grid, off_cplx, ws_bytes;
  char* ws;
  int bound;
  size_t plane_smem;     // dynamic smem of the fused plane kernel
  // bucketed chain (variant 3): per-x-plane atom lists
  int64_t max_atoms;
  size_t off_counts, off_offsets, off_cursor, off_bucket;
  // the entries compacted plane by plane (each plane's range padded to an
  // even count), the plane offsets, the per-plane counts (kept zero between
  // batches) and the per-plane placement cursors
  size_t off_pbucket, off_poff, off_pcount, off_pcursor, off_pnext;
  // bytes from the first copy of the bucket arrays (off_offsets ..
  // off_pcursor's end) to the second (overlap only; 0 otherwise)
  size_t bk_delta;
  int64_t pstride;      // entries per frame in the compacted array
  // TMA tensor maps over the two spectrum buffers for the x pass (CUtensorMap, 128 bytes each)
  alignas(64) unsigned char xtma_map[2][128];
  int xtma_ready;
  // overlap (bucketed variant): spectra double-buffered, the x pass of one
  // batch runs on `side` while the bucket kernels and plane FFT of the next
  // batch run on `plane_st`; both plan-owned streams of default priority,
  // forked from the caller's stream (ev_fork) and joined back into it
  // (ev_plane_st, ev_x).  Created by msf_plan_bind, released by plan_release
  int overlap;
  size_t off_cplx2;
  cudaStream_t side, plane_st, bucket_st;
  cudaEvent_t ev_plane[2], ev_x[2], ev_fork, ev_plane_st, ev_bucket[2];
  // a chain continued over several calls (MSF_CONTINUE): batches issued so
  // far, for the spectrum-buffer parity and the reuse waits; 0 when joined
  int64_t chain_k;
  // bounded device waits: the plane kernel's poll limit, and the diagnostic
  // option that makes its wait run out
  long long wait_limit;
  int diag_stall;
  // msf_plan_bind leaves the status word as it is (the allocation-free entry
  // point re-binds its plan on every call; its errors stay latched until read)
  int keep_status;
};

namespace msf {

inline int64_t grid_elems(const msf_plan* p) { return (int64_t)p->n0 * p->n1 * p->n2; }
inline int64_t half_elems(const msf_plan* p) { return (int64_t)p->n0 * p->n1 * p->nh; }

template <typename T>
inline T* ws_ptr(const msf_plan* p, size_t off) { return reinterpret_cast<T*>(p->ws + off); }

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? MSF_OK : MSF_E_CUDA; }
inline int launch_status() { return cuda_status(cudaGetLastError()); }

// Input arrays the kernels read: device (or managed) memory as is; page-locked
// host memory through its mapped device address (the kernels then read it in
// place, on GB300 over NVLink-C2C, with no staging copy); pageable host
// memory is refused (MSF_E_INVALID) instead of faulting in a kernel.  Not
// queried while `st` is being captured into a graph (captured calls take
// device pointers, as before).
inline int resolve_input(const void*& ptr, cudaStream_t st) {
  if (!ptr) return MSF_OK;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    return MSF_OK;
  }
  if (cap != cudaStreamCaptureStatusNone) return MSF_OK;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return MSF_OK;
  }
  if (at.type == cudaMemoryTypeUnregistered) return MSF_E_INVALID;
  if (at.type == cudaMemoryTypeHost) {
    if (!at.devicePointer) return MSF_E_INVALID;
    ptr = at.devicePointer;
  }
  return MSF_OK;
}
template <class T>
inline int resolve_input(T*& ptr, cudaStream_t st) {
  const void* v = ptr;
  const int s = resolve_input(v, st);
  ptr = static_cast<T*>(const_cast<void*>(v));
  return s;
}

// ---------------------------------------------------------------- complex
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by -i
__host__ __device__ __forceinline__ float2 cmi(float2 a) { return make_float2(a.y, -a.x); }
// multiply by +i
__host__ __device__ __forceinline__ float2 cpi(float2 a) { return make_float2(-a.y, a.x); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// Forward DFT butterflies (kernel e^{-2 pi i jk/R}) on R values in registers.
// Constants are cos/sin of 2 pi/R and 4 pi/5 rounded to float.
template <int R> struct Bfly;

template <> struct Bfly<2> {
  static __host__ __device__ __forceinline__ void run(float2* a) {
    float2 t = a[1];
    a[1] = csub(a[0], t);
    a[0] = cadd(a[0], t);
  }
};

template <> struct Bfly<3> {
  static __host__ __device__ __forceinline__ void run(float2* a) {
    const float s3 = 0.866025403784438647f;  // sin(2 pi/3)
    float2 t = cadd(a[1], a[2]);
    float2 u = csub(a[1], a[2]);
    float2 y0 = cadd(a[0], t);
    float2 c = make_float2(a[0].x - 0.5f * t.x, a[0].y - 0.5f * t.y);
    float2 d = cscale(cmi(u), s3);
    a[0] = y0;
    a[1] = cadd(c, d);
    a[2] = csub(c, d);
  }
};

template <> struct Bfly<4> {
  static __host__ __device__ __forceinline__ void run(float2* a) {
    float2 t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]);
    float2 t2 = cadd(a[1], a[3]), t3 = cmi(csub(a[1], a[3]));
    a[0] = cadd(t0, t2);
    a[2] = csub(t0, t2);
    a[1] = cadd(t1, t3);
    a[3] = csub(t1, t3);
  }
};

template <> struct Bfly<5> {
  static __host__ __device__ __forceinline__ void run(float2* a) {
    const float c1 = 0.309016994374947424f;   // cos(2 pi/5)
    const float c2 = -0.809016994374947424f;  // cos(4 pi/5)
    const float s1 = 0.951056516295153572f;   // sin(2 pi/5)
    const float s2 = 0.587785252292473129f;   // sin(4 pi/5)
    float2 b1 = cadd(a[1], a[4]), b2 = cadd(a[2], a[3]);
    float2 d1 = csub(a[1], a[4]), d2 = csub(a[2], a[3]);
    float2 y0 = cadd(a[0], cadd(b1, b2));
    float2 p1 = make_float2(a[0].x + c1 * b1.x + c2 * b2.x, a[0].y + c1 * b1.y + c2 * b2.y);
    float2 p2 = make_float2(a[0].x + c2 * b1.x + c1 * b2.x, a[0].y + c2 * b1.y + c1 * b2.y);
    float2 q1 = cmi(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
    float2 q2 = cmi(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
    a[0] = y0;
    a[1] = cadd(p1, q1);
    a[4] = csub(p1, q1);
    a[2] = cadd(p2, q2);
    a[3] = csub(p2, q2);
  }
};

template <> struct Bfly<8> {
  static __host__ __device__ __forceinline__ void run(float2* a) {
    const float h = 0.707106781186547524f;  // 1/sqrt(2)
    float2 e[4] = {a[0], a[2], a[4], a[6]};
    float2 o[4] = {a[1], a[3], a[5], a[7]};
    Bfly<4>::run(e);
    Bfly<4>::run(o);
    // o_k *= W8^k, W8 = (1 - i)/sqrt(2)
    float2 o1 = make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
    float2 o2 = cmi(o[2]);
    float2 o3 = make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
    a[0] = cadd(e[0], o[0]);
    a[4] = csub(e[0], o[0]);
    a[1] = cadd(e[1], o1);
    a[5] = csub(e[1], o1);
    a[2] = cadd(e[2], o2);
    a[6] = csub(e[2], o2);
    a[3] = cadd(e[3], o3);
    a[7] = csub(e[3], o3);
  }
};

// ------------------------------------------------------- shared-mem FFT
// Lines live in shared memory: element q of line l is s[q*sm + l*sl].
// `lfast` selects which index consecutive threads walk (line or position);
// pick the one with unit stride so warps touch consecutive words.
template <int R>
__device__ __forceinline__ void dif_stage(float2* s, const float2* tw, int n, int m, int nlines,
                                          int sm, int sl, bool lfast) {
  const int span = m * R;
  const int nb = n / R;
  const int twstep = n / span;
  const int total = nb * nlines;
  for (int u = threadIdx.x; u < total; u += blockDim.x) {
    int l, q;
    if (lfast) { l = u % nlines; q = u / nlines; }
    else       { q = u % nb;     l = u / nb; }
    const int blk = q / m;
    const int j = q - blk * m;
    float2* base = s + l * sl + (blk * span + j) * sm;
    const int step = m * sm;
    float2 a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = base[r * step];
    Bfly<R>::run(a);
    base[0] = a[0];
    const int jt = j * twstep;
#pragma unroll
    for (int r = 1; r < R; ++r) base[r * step] = cmul(a[r], tw[r * jt]);
  }
}

// Any radix: one output per thread iteration, written to `scratch` (same
// layout as s) and copied back.
__device__ inline void dif_stage_generic(float2* s, float2* scratch, const float2* tw, int n, int R,
                                         int m, int nlines, int sm, int sl, bool lfast) {
  const int span = m * R;
  const int twstep = n / span;
  const int wstep = n / R;
  const int total = n * nlines;
  for (int u = threadIdx.x; u < total; u += blockDim.x) {
    int l, p;
    if (lfast) { l = u % nlines; p = u / nlines; }
    else       { p = u % n;      l = u / n; }
    const int blk = p / span;
    const int rem = p - blk * span;
    const int k = rem / m;
    const int j = rem - k * m;
    const float2* base = s + l * sl + (blk * span + j) * sm;
    float2 acc = make_float2(0.f, 0.f);
    int rk = 0;
    for (int r = 0; r < R; ++r) {
      acc = cadd(acc, cmul(base[r * m * sm], tw[rk * wstep]));
      rk += k;
      if (rk >= R) rk -= R;
    }
    if (k) acc = cmul(acc, tw[k * j * twstep]);
    scratch[l * sl + p * sm] = acc;
  }
  __syncthreads();
  for (int u = threadIdx.x; u < total; u += blockDim.x) {
    int l, p;
    if (lfast) { l = u % nlines; p = u / nlines; }
    else       { p = u % n;      l = u / n; }
    s[l * sl + p * sm] = scratch[l * sl + p * sm];
  }
}

// Full forward FFT of every line (DIF, output at positions pos(k)).
// Ends with a __syncthreads.
__device__ inline void fft_lines(float2* s, float2* scratch, const AxisPlan& ap, const float2* tw,
                                 int nlines, int sm, int sl, bool lfast) {
  for (int st = 0; st < ap.nst; ++st) {
    const int R = ap.R[st], m = ap.m[st];
    switch (R) {
      case 8: dif_stage<8>(s, tw, ap.n, m, nlines, sm, sl, lfast); break;
      case 4: dif_stage<4>(s, tw, ap.n, m, nlines, sm, sl, lfast); break;
      case 2: dif_stage<2>(s, tw, ap.n, m, nlines, sm, sl, lfast); break;
      case 5: dif_stage<5>(s, tw, ap.n, m, nlines, sm, sl, lfast); break;
      case 3: dif_stage<3>(s, tw, ap.n, m, nlines, sm, sl, lfast); break;
      default: dif_stage_generic(s, scratch, tw, ap.n, R, m, nlines, sm, sl, lfast); break;
    }
    __syncthreads();
  }
}

// Block-wide copy of a table from global to shared memory.
template <typename T>
__device__ __forceinline__ void copy_table(T* dst, const T* __restrict__ src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// Fills a caller-owned plan from a descriptor (host only, no allocation).
int plan_init(msf_plan* p, const msf_plan_desc* d);
// The chain of msf_hist_sf_* over one position layout (msf_hist.cu).
int hist_sf_chain(msf_plan* p, const void* pos, const int32_t* weights, int layout, int64_t n_atoms,
                  int64_t n_frames, const double* scale, int32_t flags, double* sf, cudaStream_t st);

// Bucketed chain for power-of-two grids (msf_fused.cu).
bool ct_plane_ok(int n1, int n2);
int ct_x_width(int n0, int requested);   // 0 when no x kernel exists for n0 (and width)
size_t ct_plane_smem(int n1, int n2);
// slot: which copy of the bucket arrays (two with the overlap, so that the
// bucket sort of batch b+1 runs beside the plane FFT of batch b)
int fused_bucket_batch(const msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int nframes, int64_t frame_stride, const double* scale,
                       int flags, cudaStream_t st, int slot = 0);
int fused_plane_batch(const msf_plan* p, const void* grids, int grid_kind, int nframes, cudaStream_t st,
                      int buf = 0, int slot = 0);
// alone: no plane FFT shares the SMs with this x pass (the last batch of a
// chain, or a plan without overlap): the TMA x pass then fills every SM
int fused_x_batch(const msf_plan* p, int nframes, double* sf, cudaStream_t st, int buf = 0, bool alone = true);
// destroys the streams/events a bind created (idempotent)
void plan_release(msf_plan* p);
// x pass with TMA tile loads (msf_xtma.cu); prepared at bind time
int plane_twiddles_init();               // constant-memory twiddles of the plane kernel, once per device
// smooth variant (msf_smooth.cu): axes 2^a 3^b 5^c in 16..256, or 512
bool smooth_ok(int n);
int smooth_stage_a(const msf_plan* p, const void* grids, int grid_kind, int nframes, int zero, cudaStream_t st);
int smooth_stage_b(const msf_plan* p, int nframes, double* sf, cudaStream_t st);
bool xtma_ok(int n0, int w);
int xtma_prepare(msf_plan* p);
int xtma_batch(const msf_plan* p, int nframes, double* sf, cudaStream_t st, int buf, bool alone);
int bucket_grid(const msf_plan* p, const void* pos, const int32_t* weights, int layout, int64_t n_atoms,
                const double* scale, int flags, int32_t* grid, cudaStream_t st);

// Launch helpers implemented in msf_fft.cu, used by the chain entry points.
int fft_power_batch(msf_plan* p, const void* grids, int grid_kind, int nframes, double* sf,
                    int zero_grids, cudaStream_t st);
// the two halves of fft_power_batch: A = z (+y) passes into the workspace
// spectra, B = x pass + |F|^2 + sf accumulation
int fft_stage_a(msf_plan* p, const void* grids, int grid_kind, int nframes, int zero_grids,
                cudaStream_t st);
int fft_stage_b(msf_plan* p, int nframes, double* sf, cudaStream_t st);
int hist_deposit_batch(const msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int nframes, int64_t frame_stride_elems,
                       const double* scale, int flags, int32_t* grids, cudaStream_t st);

// position layouts for hist_deposit_batch
enum PosLayout { kLayoutF32x4 = 0, kLayoutF64 = 1, kLayoutF32xyz = 2 };

// grid kinds for fft_power_batch
enum GridKind { kGridI32 = 0, kGridF32 = 1, kGridF64 = 2 };

// L2-coherent loads: the int32 grids are zeroed by the kernel that reads them
template <int GK>
__device__ __forceinline__ float load_grid(const void* g, int64_t i) {
  if (GK == kGridI32) return (float)__ldcg(static_cast<const int32_t*>(g) + i);
  if (GK == kGridF32) return __ldcg(static_cast<const float*>(g) + i);
  return (float)__ldcg(static_cast<const double*>(g) + i);
}

// Block-strided loop over [0, total) that keeps U global loads in flight per
// thread: load(e) for U indices first, then store(e, value) for each (a loop
// that stores after every load waits a full memory latency per element).
template <int U, typename T, typename L, typename S>
__device__ __forceinline__ void gather_batched(int total, L load, S store) {
  for (int e0 = threadIdx.x; e0 < total; e0 += U * blockDim.x) {
    T v[U];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int e = e0 + j * (int)blockDim.x;
      if (e < total) v[j] = load(e);
    }
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int e = e0 + j * (int)blockDim.x;
      if (e < total) store(e, v[j]);
    }
  }
}

template <int GK>
__device__ __forceinline__ void zero_grid(void* g, int64_t i) {
  if (GK == kGridI32) static_cast<int32_t*>(g)[i] = 0;
}

}  // namespace msf
