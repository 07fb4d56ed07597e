// msf_fused.cu -- the bucketed histogram + FFT chain for power-of-two grids.
//
// Per batch of frames (dens.py:277-318 in histogram form):
//   k_bucket_sort    every block bins its 2048 atoms (exact numpy.histogramdd
//                    search), counting-sorts them by x-plane in shared memory
//                    and writes (y*n2 + z, w) entries plus the plane offsets
//                    of its segment
//   k_bucket_scan    plane offsets of the compacted entries (each plane's
//   k_bucket_compact count padded to even) and every block's segments moved
//                    to their plane's contiguous range
//   k_plane_ct       persistent, one plane (frame, x) at a time: the plane's
//                    atoms, staged by one cp.async.bulk copy under the
//                    previous plane's FFT, are added into the plane in shared
//                    memory (FP32 atomics on integer weights: exact and
//                    independent of order); then a two-pass register z-FFT of
//                    row pairs y = 2p, 2p+1 packed as x[2p] + i x[2p+1], a
//                    two-pass half-length y-FFT over p whose second pass is
//                    fused with the 2-D real split
//                      E = (W[q,k] + conj W[-q,-k])/2, O = (W[q,k] - conj W[-q,-k])/(2i)
//                      Y[q,k] = E + w^q O, Y[q+P,k] = E - w^q O   (w = e^{-2 pi i/n1})
//                    written as the (n1, n2/2+1) half plane; the weights are
//                    deposited halved (exact in FP32), which takes the 1/2
//                    out of E and O.  The density grid never goes to global
//                    memory.
//   k_xpower_tma     (msf_xtma.cu; k_xpower_ct without TMA) x-FFT of W spectrum
//                    columns for every frame of the batch, |F|^2 summed over
//                    the batch in FP32, one FP64 RMW of sf every kPowerFlush
//                    frames and after the last.
// All FFT lengths are template constants (msf_r2.cuh, msf_ct.cuh).
#include <math.h>

#include <atomic>
#include <vector>

#include "msf_bins.cuh"
#include "msf_ct.cuh"
#include "msf_r2.cuh"
#include "msf_tma.cuh"

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
  int* pcount;      // (batch, n0) atoms per plane, summed over the blocks
};

constexpr int kBucketThreads = 256;
constexpr int kBucketIter = kBucketAtoms / kBucketThreads;

// five blocks per SM (48 registers; 58 without the bound): the sort is bound
// by the latency of its position loads, so resident warps are what it needs
template <int MODE>
__global__ void __launch_bounds__(kBucketThreads, 5) k_bucket_sort(BucketArgs a) {
  constexpr bool kTab = MODE == 0 || MODE == 3;   // FP32 search: edge tables in shared memory
  __shared__ int hist[kMaxN + 1];
  __shared__ int warp_sum[kBucketThreads / 32];
  __shared__ float tab[kTab ? 3 * (kMaxN + 1) : 1];
  __shared__ float tab_hi[3];
  __shared__ int2 stage[kBucketAtoms];   // the block's entries in sorted order
  __shared__ int n_valid;
  const int frame = blockIdx.y;
  const int blk = blockIdx.x;
  const int n0 = a.d.n0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i <= n0; i += kBucketThreads) hist[i] = 0;
  if (kTab) {
    const int n1 = a.d.n1, n2 = a.d.n2;
    for (int i = tid; i <= n0; i += kBucketThreads) tab[i] = __ldg(a.d.flo0 + i);
    for (int i = tid; i <= n1; i += kBucketThreads) tab[n0 + 1 + i] = __ldg(a.d.flo1 + i);
    for (int i = tid; i <= n2; i += kBucketThreads) tab[n0 + n1 + 2 + i] = __ldg(a.d.flo2 + i);
    if (tid == 0) {
      tab_hi[0] = __ldg(a.d.fhi0 + n0);
      tab_hi[1] = __ldg(a.d.fhi1 + n1);
      tab_hi[2] = __ldg(a.d.fhi2 + n2);
    }
  }
  __syncthreads();
  const int64_t a0 = (int64_t)blk * kBucketAtoms + tid;
  int key[kBucketIter], vox[kBucketIter], wt[kBucketIter];
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it) {
    const int64_t i = a0 + it * kBucketThreads;
    int b0 = -1, b1 = 0, b2 = 0, w = 0;
    bool valid;
    if constexpr (kTab)
      valid = (i < a.d.n_atoms) && atom_bins_tab<MODE>(a.d, frame, i, tab, tab_hi, b0, b1, b2, w);
    else
      valid = (i < a.d.n_atoms) && atom_bins<MODE>(a.d, frame, i, b0, b1, b2, w);
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
      if (loc[j]) atomicAdd(a.pcount + (int64_t)frame * n0 + idx, loc[j]);
    }
  }
  if (tid == kBucketThreads - 1) {
    bo[n0] = before + incl;
    n_valid = before + incl;
  }
  __syncthreads();
  // placement: one independent shared-memory atomic per atom, so the
  // iterations of a thread overlap instead of forming a chain; the entries
  // land in shared memory and leave in one coalesced copy of the segment
  int slot[kBucketIter];
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it) slot[it] = key[it] >= 0 ? atomicAdd(&hist[key[it]], 1) : -1;
#pragma unroll
  for (int it = 0; it < kBucketIter; ++it)
    if (slot[it] >= 0) stage[slot[it]] = make_int2(vox[it], wt[it]);
  __syncthreads();
  int2* bk = a.bucket + ((int64_t)frame * a.nblk + blk) * kBucketAtoms;
  for (int i = tid; i < n_valid; i += kBucketThreads) bk[i] = stage[i];
}

// ----------------------------------------------------------- plane (z, y)
struct PlaneCtArgs {
  int n0;
  // grid source
  const void* grids;
  int grid_kind;
  int64_t V;
  // compacted entries: plane x of frame f is pbucket[f * pstride + poff[f][x] ..
  // poff[f][x + 1]) (an even count)
  const int2* pbucket;
  const int* poff;
  int64_t pstride;
  int* status;
  int* next_item;         // plane hand-out counter, zeroed before each launch
  long long wait_limit;   // bounded-wait limit (polls)
  int stall;          // MSF_PLAN_DIAG_STALL: arm the first wait for a copy never issued
  // output
  float2* C;
  int64_t Vh;
  const float2* twy;
};

// Twiddles w_N^k (k < N) of the plane kernel for N = 16, 32, ..., 512, at
// offset N - 16, in constant memory: every index the plane kernel uses is
// uniform across a warp, so the table costs no shared-memory bandwidth (the
// plane FFT is bound by shared-memory wavefronts).  Filled once per device
// by plane_twiddles_init (msf_plan_bind).
constexpr int kConstTw = 1024 - 16;
__constant__ float2 c_tw[kConstTw];

template <int N>
struct CTw {
  static_assert(N >= 16 && N <= 512 && (N & (N - 1)) == 0, "constant twiddles: N = 16..512");
  __device__ __forceinline__ float2 operator()(int k) const { return c_tw[N - 16 + k]; }
};

template <int N1, int N2>
struct PlaneShape {
  static constexpr int P = N1 / 2;
  // PAIRS: the z and y passes move two complex values per 16-byte access
  // (where the z lines' second-pass radix is at most 8: two 16-point
  // transforms of the longer z lines do not fit the register budget), with
  // an even line stride of SP*8 = 16 (mod 128) bytes (P a multiple of 16) so
  // that those accesses are free of bank conflicts along and across lines;
  // otherwise 8-byte accesses and an odd line stride.  The shapes whose pair
  // passes spill registers at the bucket kernel's register cap keep 8-byte
  // accesses.
  static constexpr bool PAIRS = r2::Split2<N2>::A <= 8 &&
                                !((N1 == 64 && N2 == 128) || (N1 == 128 && N2 == 64) || (N1 == 256 && N2 <= 64));
  static constexpr int SP = PAIRS ? P + 2 : P + 1;
  static constexpr int NH = N2 / 2 + 1;
  static constexpr int NT = (N2 * P >= 4096) ? 512 : 256;
  // plane, then the segment tables of the bucket gather
  static constexpr size_t SMEM = (size_t)N2 * SP * sizeof(float2) + (size_t)(2 * NT + 1 + NT / 32) * sizeof(int);
};

// Last pass of the half-length y FFT fused with the 2-D real split.  After
// r2::pass1_fn, DFT_A over the slots A*k1 + n1 of kz line l gives
// W[q = k1 + B*k2][l] (k2 < A).  The split pairs W[q][k] with W[-q][-k]:
// for k1 != 0 that is k2' = A-1-k2 of item (B-k1, -l), for k1 == 0 it is
// k2' = (A-k2) mod A of item (0, -l).  A unit is two items transformed in
// registers and written straight to the half plane:
//   interior line l (0 < l < n2/2): item (k1, l) and its partner on line -l
//     (only the first is an output);
//   edge line l = 0 or n2/2, 0 < k1 < B/2: items (k1, l) and (B-k1, l), each
//     the other's partner, both outputs;
//   edge line, k1 = 0 and B/2: two self-paired items in one unit.
// That is B*n2/2 units of equal transform work: exactly two per thread at
// the headline size, with no tail.  Unit u takes slot (k1 = u / (n2/2),
// l = u % (n2/2)): consecutive threads walk l with k1 fixed, so k1 -- and with
// it the twiddle index w^q, q = k1 + B*k2 -- is uniform across a warp when
// n2/2 is a multiple of 32 (one constant-cache access per twiddle), and the
// B slots with l = 0 hold the 2 x B/2 edge units (line 0 for k1 < B/2, line
// n2/2 for the others), spread over the warps instead of all in warp 0 (one
// per warp at the headline shape, with the rotation of the odd passes
// below).
template <int N1, int N2, int SP, int NT, bool ZERO = false, bool PAIRS = false>
__device__ __forceinline__ void ypass2_split(float2* buf, float2* out) {
  constexpr int P = N1 / 2, NH = N2 / 2 + 1;
  constexpr int A = r2::Split2<P>::A, B = r2::Split2<P>::B;
  constexpr int H = N2 / 2;               // interior output lines 1 .. H - 1
  constexpr int U = B * H;                // B edge units + B*(H - 1) interior units
  const CTw<N1> wq;
  // the plane holds half the weights, so E and O need no factor 1/2
  auto emit = [&](int q, int k, float2 w, float2 wm_raw) {
    const float2 wm = cconj(wm_raw);
    const float2 E = cadd(w, wm);
    const float2 O = cmi(csub(w, wm));
    const float2 t = cmul(wq(q), O);
    __stcs(out + q * NH + k, cadd(E, t));   // evict-first: keep L2 for the bucket entries
    __stcs(out + (q + P) * NH + k, csub(E, t));
  };
  // Odd passes over the units take their slots rotated by 32 within each k1
  // block (a bijection there, as NT is a multiple of H): an edge unit's extra
  // emits serialise its warp, and with two passes of NT threads (the
  // headline shape) every warp then holds one edge unit instead of the even
  // warps two and the odd ones none.
  constexpr bool ROT = H % 64 == 0 && NT % H == 0;
  for (int u = threadIdx.x; u < U; u += NT) {
    int l, lp, k1, k1p;
    const int kk = u / H, ll = ROT ? (u + ((u / NT) & 1) * 32) % H : u % H;
    const bool edge = ll == 0;
    if (edge) {                      // edge line: k1 = 0 pairs the two self-paired items
      l = lp = kk < B / 2 ? 0 : N2 / 2;
      k1 = kk % (B / 2);
      k1p = k1 ? B - k1 : B / 2;
    } else {
      k1 = kk;
      l = ll;
      lp = N2 - l;
      k1p = (B - k1) & (B - 1);
    }
    float2* pa = buf + l * SP + A * k1;
    float2* pb = buf + lp * SP + A * k1p;
    float2 a[A], b[A];
    const float2 z = make_float2(0.f, 0.f);
    if constexpr (PAIRS) {
#pragma unroll
      for (int n1 = 0; n1 < A; n1 += 2) {
        r2::ld2(pa + n1, a[n1], a[n1 + 1]);
        r2::ld2(pb + n1, b[n1], b[n1 + 1]);
      }
    } else {
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) { a[n1] = pa[n1]; b[n1] = pb[n1]; }
    }
    if (ZERO) {
      // every slot of the plane is read by exactly one unit (item and
      // partner of each unit are distinct and cover all B*N2 items once):
      // clearing what was read leaves the plane zeroed for the next deposit
      if constexpr (PAIRS) {
#pragma unroll
        for (int n1 = 0; n1 < A; n1 += 2) { r2::st2(pa + n1, z, z); r2::st2(pb + n1, z, z); }
      } else {
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) { pa[n1] = z; pb[n1] = z; }
      }
    }
    reg::reg_dft<A>(a);
    reg::reg_dft<A>(b);
    if (edge && k1 == 0) {
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) emit(B * k2, l, a[k2], a[(A - k2) & (A - 1)]);
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) emit(B / 2 + B * k2, l, b[k2], b[A - 1 - k2]);
    } else if (k1 == 0) {            // interior line, k1 = 0: partner (0, -l)
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) emit(B * k2, l, a[k2], b[(A - k2) & (A - 1)]);
    } else {
#pragma unroll
      for (int k2 = 0; k2 < A; ++k2) emit(k1 + B * k2, l, a[k2], b[A - 1 - k2]);
      if (edge) {
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) emit(k1p + B * k2, l, b[k2], a[A - 1 - k2]);
      }
    }
  }
}

// z FFT of the row pairs, then the half-length y FFT with the real split:
// the deposited plane in buf becomes the half plane at out.
template <int N1, int N2, bool ZERO = false>
__device__ __forceinline__ void plane_transform(float2* buf, float2* out) {
  using S = PlaneShape<N1, N2>;
  // z: lines = pairs p, samples stride SP, two adjacent lines per 16-byte
  // access (the two inner barriers over the warps that share lines only);
  // then pass 1 of the half y FFT (lines = kz, samples stride 1, two adjacent
  // samples per access), and its pass 2 fused with the real split
  if constexpr (S::PAIRS) {
    r2::fft2_linepairs<N2, S::P, S::SP, S::NT>(buf, CTw<N2>());
    __syncthreads();
    r2::pass1_samplepairs<S::P, N2, S::SP, S::NT>(buf, CTw<S::P>());
  } else {
    r2::fft2_lines_grouped<N2, S::P, S::SP, 1, S::NT>(buf, CTw<N2>());
    __syncthreads();
    r2::pass1_fn<S::P, N2, 1, S::SP, S::NT>(buf, CTw<S::P>());
  }
  __syncthreads();
  ypass2_split<N1, N2, S::SP, S::NT, ZERO, S::PAIRS>(buf, out);
}

// float offset of voxel y*n2 + z in the row-pair layout buf[z][p].(y & 1)
template <int N2, int SP>
__device__ __forceinline__ int pair_offset(int vx) {
  const int y = vx / N2, z = vx % N2;
  return 2 * (z * SP + (y >> 1)) + (y & 1);
}

// Registers capped so that one x-pass CTA (256 threads x 80) fits on the SM
// beside a 512-thread plane CTA (the two kernels overlap on different
// streams): 80 for the grid-source kernel, 88 for the bucket kernel, which
// also carries the next plane's entries (512 x 88 + 256 x 80 = 65536).  Not
// where the fused y pass holds two 16-point transforms (n1 = 512).
#define MSF_PLANE_MAXNREG(N1, N2, CAP) (PlaneShape<N1, N2>::NT >= 512 && r2::Split2<N1 / 2>::A < 16 ? CAP : 128)

// Dense-grid source (int32 / float32 / float64 grids of a batch): one CTA
// per (x, frame).
template <int N1, int N2>
__global__ void __maxnreg__((MSF_PLANE_MAXNREG(N1, N2, 80))) k_plane_grid(PlaneCtArgs a) {
  using S = PlaneShape<N1, N2>;
  constexpr int SP = S::SP, NT = S::NT;
  extern __shared__ float2 smem[];
  float2* buf = smem;                 // [N2][SP], z major
  float* buff = reinterpret_cast<float*>(buf);
  const int x = blockIdx.x;
  const int frame = blockIdx.y;
  const int64_t g0 = frame * a.V + (int64_t)x * N1 * N2;
  for (int e = threadIdx.x; e < N1 * N2; e += NT) {
    float v;
    if (a.grid_kind == kGridI32) v = (float)__ldg(static_cast<const int32_t*>(a.grids) + g0 + e);
    else if (a.grid_kind == kGridF32) v = __ldg(static_cast<const float*>(a.grids) + g0 + e);
    else v = (float)__ldg(static_cast<const double*>(a.grids) + g0 + e);
    buff[pair_offset<N2, SP>(e)] = 0.5f * v;   // halved: the split's 1/2 (exact)
  }
  __syncthreads();
  plane_transform<N1, N2>(buf, a.C + frame * a.Vh + (int64_t)x * N1 * S::NH);
}

// Bucket source, persistent: CTA b transforms plane (frame, x) = item b
// first, then the planes a global counter hands out (items gridDim.x, ...,
// in the order asked for): a CTA that starts late -- its SM still held by the
// CTAs of the x pass running beside on another stream -- takes fewer planes
// instead of holding the launch up.  With a fixed share per CTA, runs where
// x-pass CTAs had doubled up on some SMs when the plane kernel started took
// 30.5 instead of 23.8 us per frame.  A plane's atoms are one contiguous, even
// range of the compacted entries (k_bucket_compact); thread 0 fetches up to
// kPlanePrefetch*NT of them into shared memory with one cp.async.bulk copy
// tracked by an mbarrier, issued before the FFT of the previous plane, so the
// copy runs under that FFT.  Entries beyond the staged part are read from
// global memory at deposit time.  The wait is bounded (a.wait_limit polls):
// on timeout the kernel latches MSF_E_TIMEOUT in the plan status word and
// returns.  With a.stall (the plan's diagnostic option) the
// first wait expects 16 bytes that no copy delivers, so it runs out: the
// error path can be tested without any fault.
constexpr int kPlanePrefetch = 3;

template <int N1, int N2>
struct BucketPlaneShape {
  using S = PlaneShape<N1, N2>;
  static constexpr int CAP = kPlanePrefetch * S::NT;   // staged entries (even)
  // plane (a multiple of 16 bytes), the staged entries, then the mbarrier
  // and three ints (no static shared memory: the dynamic base keeps its
  // alignment for the 16-byte stores and the bulk copy)
  static constexpr size_t SMEM = (size_t)N2 * S::SP * sizeof(float2) + (size_t)CAP * sizeof(int2) + 32;
};

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

template <int N1, int N2>
__global__ void __maxnreg__((MSF_PLANE_MAXNREG(N1, N2, 88))) k_plane_ct(PlaneCtArgs a, int items) {
  using S = PlaneShape<N1, N2>;
  constexpr int SP = S::SP, NT = S::NT, CAP = BucketPlaneShape<N1, N2>::CAP;
  extern __shared__ __align__(16) float2 smem[];
  float2* buf = smem;                                       // [N2][SP], z major
  float* buff = reinterpret_cast<float*>(buf);
  int2* staged = reinterpret_cast<int2*>(buf + N2 * SP);    // CAP entries
  uint64_t* bar = reinterpret_cast<uint64_t*>(staged + CAP);
  int* ctl = reinterpret_cast<int*>(bar + 1);   // [0] range begin, [1] count, [2] abort flag, [3] next plane
  const int tid = threadIdx.x;
  const int G = gridDim.x;
  // thread 0: offsets (begin, end) of plane `item` in the compacted entries,
  // and the copy of its first CAP entries.  The plane after next is fetched
  // from the counter, and its offsets loaded, one plane ahead and first used
  // a plane later: a count formed right after the load stalled thread 0 --
  // and with it warp 0 and every barrier after it -- for ~3k cycles per plane
  // (measured with clock64 stamps), the latency of a global load under the
  // kernel's own traffic.
  auto fetch = [&]() { return G + atomicAdd(a.next_item, 1); };
  auto range_raw = [&](int item) {
    const int frame = item / a.n0, x = item - frame * a.n0;
    const int* po = a.poff + (int64_t)frame * (a.n0 + 1) + x;
    return make_int2(po[0], po[1]);
  };
  auto issue = [&](int item, int2 r) {
    if (a.stall) {
      mbar_expect_tx(bar, 16);
      return;
    }
    const int ns = r.y < CAP ? r.y : CAP;
    mbar_expect_tx(bar, (uint32_t)ns * sizeof(int2));
    if (ns > 0) bulk_load(staged, a.pbucket + (int64_t)(item / a.n0) * a.pstride + r.x, ns * sizeof(int2), bar);
  };
  int2 after = make_int2(0, 0);   // thread 0: offsets of plane nxt
  int nxt = items, nxt2 = items;  // thread 0: the next plane and the one after it
  int item = blockIdx.x;
  // the plane starts zeroed; afterwards the split of each plane clears what
  // it reads, so the next deposit finds it zeroed again
  {
    int4* z4 = reinterpret_cast<int4*>(buf);
    for (int i = tid; i < N2 * SP / 2; i += NT) z4[i] = make_int4(0, 0, 0, 0);
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    ctl[2] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    int2 r = make_int2(0, 0);
    if (item < items) {
      r = range_raw(item);
      r.y -= r.x;
      issue(item, r);
    }
    ctl[0] = r.x;
    ctl[1] = r.y;
    nxt = fetch();
    if (nxt < items) {
      after = range_raw(nxt);
      nxt2 = fetch();
    }
  }
  __syncthreads();
  uint32_t phase = 0;
  while (item < items) {
    const int frame = item / a.n0, x = item - frame * a.n0;
    long long spins = 0;
    while (!mbar_try_wait(bar, phase)) {
      if (++spins > a.wait_limit) { atomicExch(ctl + 2, 1); break; }
    }
    __syncthreads();   // also: the previous plane's split has read and cleared the plane
    if (ctl[2]) {
      if (tid == 0) atomicExch(a.status + kStatErr, MSF_E_TIMEOUT);
      break;
    }
    phase ^= 1u;
    // integer weights summed in FP32: exact (and order-independent) while a
    // voxel's total stays below 2^24 electrons; deposited halved, which is
    // exact too and takes the split's factor 1/2
    {
      const int n = ctl[1], ns = n < CAP ? n : CAP;
      const int2* src = a.pbucket + (int64_t)frame * a.pstride + ctl[0];
      for (int e = tid; e < n; e += NT) {
        const int2 v = e < ns ? staged[e] : src[e];
        atomicAdd(buff + pair_offset<N2, SP>(v.x), 0.5f * (float)v.y);
      }
    }
    __syncthreads();   // staging area and the range consumed
    if (tid == 0) {
      const int next = nxt;
      const int2 r = make_int2(after.x, after.y - after.x);   // loaded a plane ago
      if (next < items) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(next, r);
      }
      ctl[0] = r.x;
      ctl[1] = r.y;
      ctl[3] = next;
      nxt = nxt2;                      // fetched a plane ago
      if (nxt < items) {
        after = range_raw(nxt);
        nxt2 = fetch();
      }
    }
    plane_transform<N1, N2, true>(buf, a.C + frame * a.Vh + (int64_t)x * N1 * S::NH);
    item = ctl[3];   // written by thread 0 before the transform's barriers
  }
  // leave no copy in flight into this CTA's shared memory (bounded)
  if (tid == 0 && ctl[2]) {
    long long spins = 0;
    while (!mbar_try_wait(bar, phase) && ++spins < a.wait_limit) {
    }
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
    if (b == a.nframes - 1 || b % kPowerFlush == kPowerFlush - 1) {
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        const int e = threadIdx.x + i * NT;
        const int x = e / W, w = e % W;
        if (w < weff) {
          double* d = a.sf + (int64_t)x * a.F + f0 + w;
          *d = *d + (double)acc[i];
        }
        acc[i] = 0.f;
      }
    }
  }
}

// ---------------------------------------------------------------- dispatch
template <typename K>
static void allow_smem_once(K kernel, bool& once, size_t bytes = 227 * 1024) {
  if (!once) {
    // the exact need: with static shared memory in the kernel, 227 KB of
    // dynamic shared memory would exceed the per-block limit and be refused
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    // the whole unified L1/shared array as shared memory, so an x-pass CTA
    // finds room beside a plane CTA
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    once = true;
  }
}

template <int N1, int N2>
static int launch_plane_ct(const PlaneCtArgs& a, int src, int n0, int nframes, cudaStream_t st) {
  using S = PlaneShape<N1, N2>;
  static bool once0 = false, once1 = false;
  static int sms = 0;
  if (src == 0) {
    allow_smem_once(k_plane_ct<N1, N2>, once0, BucketPlaneShape<N1, N2>::SMEM);
    const int ms = cuda_status(cudaMemsetAsync(a.next_item, 0, sizeof(int), st));
    if (ms) return ms;
    if (!sms) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (sms <= 0) sms = 152;
    }
    const int items = n0 * nframes;
    k_plane_ct<N1, N2><<<items < sms ? items : sms, S::NT, BucketPlaneShape<N1, N2>::SMEM, st>>>(a, items);
  } else {
    allow_smem_once(k_plane_grid<N1, N2>, once1, S::SMEM);
    k_plane_grid<N1, N2><<<dim3(n0, nframes), S::NT, S::SMEM, st>>>(a);
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
  X(32, 32) X(64, 32) X(64, 16) X(128, 32) X(128, 16) X(256, 32) X(256, 16) X(256, 8) X(512, 8) X(1024, 4)

static int x_ct(const XCtArgs& a, int n0, int w, cudaStream_t st) {
#define X(A, B) if (n0 == A && w == B) return launch_x_ct<A, B>(a, st);
  MSF_X_CASES(X)
#undef X
  return MSF_E_UNSUPPORTED;
}

// the requested tile width if it is instantiated for n0, else (0) the widest
// tile of at most 2048 complex values -- the TMA x pass then runs two
// 128-thread CTAs beside a plane-FFT CTA, measured faster than one 256-thread
// CTA of 4096-value tiles beside it and alone (256-point lines: 6.68 against
// 7.45 us per frame alone, 44.8k against 44.2k frames/s for the chain) --
// or the narrowest instantiated when every tile is larger
int ct_x_width(int n0, int requested) {
  int best = 0, narrow = 0;
#define X(A, B)                                                               \
  if (n0 == A) {                                                              \
    if (requested ? B == requested : (A * B <= 2048 && B > best)) best = B;   \
    if (!narrow || B < narrow) narrow = B;                                    \
  }
  MSF_X_CASES(X)
#undef X
  return best || requested ? best : narrow;
}

// w_N^k = exp(-2 pi i k/N) rounded to float: cos/sin in double of the angle
// reduced to the first quadrant (so 0 and +-1 come out exact), then rotated.
static std::vector<float2> plane_twiddle_table() {
  std::vector<float2> t(kConstTw);
  for (int n = 16; n <= 512; n *= 2) {
    const int q4 = n / 4;
    for (int k = 0; k < n; ++k) {
      const int j = k % q4, quad = k / q4;
      const double ang = 2.0 * M_PI * (double)j / (double)n;
      const double c0 = j ? cos(ang) : 1.0, s0 = j ? sin(ang) : 0.0;
      double c, s;
      switch (quad) {
        case 0: c = c0; s = s0; break;
        case 1: c = -s0; s = c0; break;
        case 2: c = -c0; s = -s0; break;
        default: c = s0; s = -c0; break;
      }
      t[n - 16 + k] = make_float2((float)c, (float)(-s));
    }
  }
  return t;
}

int plane_twiddles_init() {
  static const std::vector<float2> table = plane_twiddle_table();
  static std::atomic<bool> ready[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MSF_E_CUDA;
  if (dev >= 0 && dev < 64 && ready[dev].load(std::memory_order_acquire)) return MSF_OK;
  if (cudaMemcpyToSymbol(c_tw, table.data(), kConstTw * sizeof(float2)) != cudaSuccess) return MSF_E_CUDA;
  if (dev >= 0 && dev < 64) ready[dev].store(true, std::memory_order_release);
  return MSF_OK;
}

size_t ct_plane_smem(int n1, int n2) {
  return (size_t)n2 * (n1 / 2 + 1) * sizeof(float2) + (size_t)(n2 + n1) * sizeof(float2);
}

// Plane offsets of the compacted entries (one CTA per frame, thread x per
// plane): plane x's count (summed over the bucketing blocks by
// k_bucket_sort, then reset to zero here for the next batch) padded to even
// with a zero-weight entry, exclusive scan over x -> poff, which also
// starts the plane's placement cursor.
__global__ void __launch_bounds__(kMaxN) k_bucket_scan(int* pcount, int n0, int* poff, int* cursor, int2* pbucket,
                                                      int64_t pstride) {
  __shared__ int wsum[kMaxN / 32];
  const int frame = blockIdx.x, x = threadIdx.x;
  const int lane = x & 31, warp = x >> 5;
  int tot = 0;
  if (x < n0) {
    tot = pcount[(int64_t)frame * n0 + x];
    pcount[(int64_t)frame * n0 + x] = 0;
  }
  const int padded = (tot + 1) & ~1;
  int incl = padded;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x / 32) ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  if (x >= n0) return;
  const int base = incl - padded + (warp ? wsum[warp - 1] : 0);
  int* po = poff + (int64_t)frame * (n0 + 1);
  po[x] = base;
  if (x == n0 - 1) po[n0] = base + padded;
  cursor[(int64_t)frame * n0 + x] = base;
  if (padded != tot) pbucket[(int64_t)frame * pstride + base + tot] = make_int2(0, 0);
}

// Every bucketing block's entries moved to their plane's range (one CTA per
// (block, frame)): each of the block's plane segments reserves its place
// with one atomic on the plane's cursor (the order of segments within a
// plane is free: the deposit sums integers exactly); entry e of the block
// belongs to the last plane x with offset <= e.
__global__ void __launch_bounds__(kBucketThreads) k_bucket_compact(BucketArgs a, int* cursor, int2* pbucket,
                                                                   int64_t pstride) {
  __shared__ int sbo[kMaxN + 1];
  __shared__ int sdst[kMaxN];
  const int blk = blockIdx.x, frame = blockIdx.y, n0 = a.d.n0;
  const int* bo = a.boff + ((int64_t)frame * a.nblk + blk) * (n0 + 1);
  for (int i = threadIdx.x; i <= n0; i += kBucketThreads) sbo[i] = bo[i];
  __syncthreads();
  for (int i = threadIdx.x; i < n0; i += kBucketThreads) {
    const int cnt = sbo[i + 1] - sbo[i];
    sdst[i] = cnt ? atomicAdd(cursor + (int64_t)frame * n0 + i, cnt) : 0;
  }
  __syncthreads();
  const int2* src = a.bucket + ((int64_t)frame * a.nblk + blk) * kBucketAtoms;
  int2* out = pbucket + (int64_t)frame * pstride;
  // warp w moves the entries of planes 32w .. 32w+31 (then w + 8, ...):
  // lane l holds plane 32w+l's segment start and destination, and an entry
  // finds its plane -- the last lane whose start is <= it -- by a 5-step
  // search over the lanes' registers (the starts ascend with the lane)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int p0 = warp * 32; p0 < n0; p0 += kBucketThreads) {
    const int pl = p0 + lane;
    const int start = pl < n0 ? sbo[pl] : sbo[n0];
    const int dst = pl < n0 ? sdst[pl] : 0;
    const int beg = sbo[p0], end = sbo[min(p0 + 32, n0)];
    for (int base = beg; base < end; base += 32) {
      const int e = base + lane;
      int lo = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int probe = __shfl_sync(0xffffffffu, start, lo + step);
        if (probe <= e) lo += step;
      }
      const int s0 = __shfl_sync(0xffffffffu, start, lo), d0 = __shfl_sync(0xffffffffu, dst, lo);
      if (e < end) out[d0 + (e - s0)] = src[e];
    }
  }
}

static BucketArgs bucket_args(const msf_plan* p, int slot = 0) {
  const size_t d = slot ? p->bk_delta : 0;
  BucketArgs b;
  b.d = dep_args(p);
  b.boff = ws_ptr<int>(p, p->off_offsets + d);
  b.bucket = ws_ptr<int2>(p, p->off_bucket + d);
  b.nblk = (int)((p->max_atoms + kBucketAtoms - 1) / kBucketAtoms);
  b.pcount = ws_ptr<int>(p, p->off_pcount + d);
  return b;
}

int fused_bucket_batch(const msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int nframes, int64_t frame_stride, const double* scale,
                       int flags, cudaStream_t st, int slot) {
  if (n_atoms > p->max_atoms) return MSF_E_WORKSPACE;
  if (slot && !p->bk_delta) return MSF_E_INVALID;
  const size_t d = slot ? p->bk_delta : 0;
  BucketArgs b = bucket_args(p, slot);
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
  int s = launch_status();
  if (s) return s;
  int2* pbucket = ws_ptr<int2>(p, p->off_pbucket + d);
  int* cursor = ws_ptr<int>(p, p->off_pcursor + d);
  k_bucket_scan<<<nframes, ((p->n0 + 31) / 32) * 32, 0, st>>>(b.pcount, p->n0, ws_ptr<int>(p, p->off_poff + d), cursor,
                                                          pbucket, p->pstride);
  s = launch_status();
  if (s) return s;
  k_bucket_compact<<<grid, kBucketThreads, 0, st>>>(b, cursor, pbucket, p->pstride);
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

static PlaneCtArgs plane_args(const msf_plan* p, int slot = 0) {
  const size_t d = slot ? p->bk_delta : 0;
  PlaneCtArgs a;
  memset(&a, 0, sizeof(a));
  a.n0 = p->n0;
  a.V = grid_elems(p);
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.twy = ws_ptr<float2>(p, p->off_tw[1]);
  a.pbucket = ws_ptr<int2>(p, p->off_pbucket + d);
  a.poff = ws_ptr<int>(p, p->off_poff + d);
  a.pstride = p->pstride;
  a.status = ws_ptr<int>(p, p->off_status);
  a.next_item = ws_ptr<int>(p, p->off_pnext);
  a.wait_limit = p->wait_limit;
  a.stall = p->diag_stall;
  return a;
}

int fused_plane_batch(const msf_plan* p, const void* grids, int grid_kind, int nframes, cudaStream_t st,
                      int buf, int slot) {
  if (slot && !p->bk_delta) return MSF_E_INVALID;
  PlaneCtArgs a = plane_args(p, slot);
  if (buf) a.C = ws_ptr<float2>(p, p->off_cplx2);
  a.grids = grids;
  a.grid_kind = grid_kind;
  return plane_ct(a, p->n1, p->n2, grids ? 1 : 0, p->n0, nframes, st);
}

int fused_x_batch(const msf_plan* p, int nframes, double* sf, cudaStream_t st, int buf, bool alone) {
  if (p->xtma_ready) return xtma_batch(p, nframes, sf, st, buf, alone);
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
  if (resolve_input(pos, reinterpret_cast<cudaStream_t>(stream)) ||
      resolve_input(weights, reinterpret_cast<cudaStream_t>(stream)) ||
      resolve_input(scale, reinterpret_cast<cudaStream_t>(stream)))
    return MSF_E_INVALID;
  return bucket_grid(p, pos, weights, layout, n_atoms, scale, flags, grid,
                     reinterpret_cast<cudaStream_t>(stream));
}
