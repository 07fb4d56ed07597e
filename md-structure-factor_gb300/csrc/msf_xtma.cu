// msf_xtma.cu -- x pass of the bucketed chain with TMA tile loads.
//
// The half spectra of a batch are one row-major matrix of B*n0 rows (frame,
// x) by F = n1*(n2/2+1) complex columns.  A persistent CTA walks work items
// (column tile of W columns, frame); each item's (n0 x W) tile is fetched by
// cp.async.bulk.tensor.2d into one of NS shared-memory buffers and tracked by
// an mbarrier, so the copies of items s+1 .. s+NS-1 run while item s is
// transformed (NS = 2: four buffers per 16 KB tile measured slower alone, as
// they cost half the CTAs per SM).  A CTA has 16 values of a tile per
// thread: 2048-value tiles take 128-thread CTAs (two beside a plane-FFT CTA
// in the overlapped launch, six per SM alone), larger ones 256.  (4-column
// tiles on four 64-thread CTAs beside the plane CTA measured slower: 8.3
// against 6.7 us per frame for the 256-point x pass alone, 32-byte box
// rows.)  x-FFT (DIF, natural input, output at pos(k)), |F|^2 summed over the frames of the tile in FP32, one FP64
// read-modify-write of sf per tile every kPowerFlush frames and after the
// last.  Waits are bounded: on timeout the kernel latches MSF_E_TIMEOUT in
// the plan status word and returns.
#include "msf_ct.cuh"
#include "msf_r2.cuh"
#include "msf_tma.cuh"

namespace msf {

struct XTmaArgs {
  int nframes;
  int64_t F;
  int ntiles;
  double* sf;
  const float2* twx;
  int* status;
};

template <int N0, int W>
struct XTmaShape {
  // 16 values per thread, 64 to 256 threads
  static constexpr int NT = N0 * W / 16 < 64 ? 64 : (N0 * W / 16 > 256 ? 256 : N0 * W / 16);
  static constexpr int EPT = N0 * W / NT;
  static constexpr int BOX_ROWS = N0 <= 256 ? N0 : 256;
  static constexpr int NBOX = N0 / BOX_ROWS;
  static constexpr uint32_t TILE_BYTES = N0 * W * sizeof(float2);
  static constexpr int NS = 2;   // tile buffers
  static constexpr size_t SMEM = 1024 + NS * (size_t)TILE_BYTES + N0 * sizeof(float2);
};

// register budget: 80 per thread, so that one 256-thread or two 128-thread
// CTAs fit beside a plane-FFT CTA (512 threads x 88)
template <int N0, int W>
__global__ void __launch_bounds__(XTmaShape<N0, W>::NT,
                                  (N0 <= 256 && N0 * W <= 4096 ? 3 * 256 / XTmaShape<N0, W>::NT : 1))
    k_xpower_tma(const __grid_constant__ CUtensorMap map, XTmaArgs a) {
  using S = XTmaShape<N0, W>;
  constexpr int NT = S::NT, EPT = S::EPT;
  static_assert(EPT * NT == N0 * W, "tile must split evenly over the threads");
  extern __shared__ unsigned char smem_raw[];
  constexpr int NS = S::NS;
  __shared__ __align__(8) uint64_t bar[NS];
  __shared__ int abort_flag, abort_at;
  // 1024-byte aligned tile buffers (TMA destination)
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  float2* buf0 = reinterpret_cast<float2*>(base);
  float2* tw = buf0 + NS * N0 * W;
  const int tid = threadIdx.x;
  const int my_tiles = (a.ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  const int total = my_tiles > 0 ? my_tiles * a.nframes : 0;
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < NS; ++k) mbar_init(&bar[k], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < N0; i += NT) tw[i] = a.twx[i];
  __syncthreads();

  auto issue = [&](int s) {
    const int tile = (int)blockIdx.x + (s / a.nframes) * (int)gridDim.x;
    const int frame = s % a.nframes;
    float2* dst = buf0 + (s % NS) * (N0 * W);
    uint64_t* b = &bar[s % NS];
    mbar_expect_tx(b, S::TILE_BYTES);
#pragma unroll
    for (int k = 0; k < S::NBOX; ++k)
      tma_load_2d(dst + k * S::BOX_ROWS * W, &map, tile * W, frame * N0 + k * S::BOX_ROWS, b);
  };
  if (tid == 0)
    for (int k = 0; k < NS && k < total; ++k) issue(k);
  uint32_t phases = 0;   // bit k: parity of buffer k's next completion
  // pass-2 items (k1, column) owned by this thread; X[k1 + B*k2] power in acc
  constexpr int A = r2::Split2<N0>::A, B = r2::Split2<N0>::B;
  constexpr int ITEMS2 = B * W;
  constexpr int PER = (ITEMS2 + NT - 1) / NT;
  // Rows narrower than 128 bytes (W < 16): the 32 / W k1 rows a warp reads
  // in pass 2 sit A * W * 8 bytes apart, on the same banks.  Group
  // g = k1 mod RG reads its A samples cyclically shifted by g rows, RG the
  // rows per 128 bytes, which spreads the groups evenly over the banks (two
  // wavefronts per 256-byte access, the least there is); a cyclic shift of a
  // DFT's input only multiplies each X[k] by a unit phase, so |X[k]|^2 is
  // unchanged.
  constexpr int RW = 128 / (W * (int)sizeof(float2));
  constexpr int RG = RW > 1 ? (RW < A ? RW : A) : 1;
  static_assert((RG & (RG - 1)) == 0, "shift groups must be a power of two");
  float acc[PER][A];
#pragma unroll
  for (int j = 0; j < PER; ++j)
#pragma unroll
    for (int k = 0; k < A; ++k) acc[j][k] = 0.f;

  for (int s = 0; s < total; ++s) {
    const int b = s % NS;
    uint64_t* bb = &bar[b];
    const uint32_t par = (phases >> b) & 1u;
    long long spins = 0;
    while (!mbar_try_wait(bb, par)) {
      if (++spins > kWaitLimit) { atomicExch(&abort_flag, 1); break; }
    }
    __syncthreads();
    if (abort_flag) {
      if (tid == 0) {
        atomicExch(a.status + kStatErr, MSF_E_TIMEOUT);
        abort_at = s;
      }
      break;
    }
    phases ^= 1u << b;
    float2* t = buf0 + b * (N0 * W);
    r2::pass1<N0, W, W, 1, NT>(t, tw);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int it = j * NT + tid;
      if (ITEMS2 % NT == 0 || it < ITEMS2) {
        const int l = it % W, k1 = it / W;
        const int g = k1 & (RG - 1);
        const float2* p = t + l + A * k1 * W;
        const float2* q = p + g * W;
        float2 r[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1)   // sample (n1 + g) mod A; only the last RG - 1 can wrap
          r[n1] = (n1 + RG - 1 < A || n1 + g < A) ? q[n1 * W] : q[(n1 - A) * W];
        reg::reg_dft<A>(r);
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) acc[j][k2] = fmaf(r[k2].x, r[k2].x, fmaf(r[k2].y, r[k2].y, acc[j][k2]));
      }
    }
    const int frame = s % a.nframes;
    if (frame == a.nframes - 1 || frame % kPowerFlush == kPowerFlush - 1) {
      const int tile = (int)blockIdx.x + (s / a.nframes) * (int)gridDim.x;
      const int64_t f0 = (int64_t)tile * W;
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        const int it = j * NT + tid;
        const int l = it % W, k1 = it / W;
        const bool ok = (ITEMS2 % NT == 0 || it < ITEMS2) && f0 + l < a.F;
        double* d = a.sf + (int64_t)k1 * a.F + f0 + l;
        // in groups of 8: the group's loads first (independent), then the adds
        // and stores (a whole column of FP64 values would not fit the
        // register budget beside the accumulators)
        constexpr int G8 = A > 8 ? 8 : A;
#pragma unroll
        for (int g = 0; g < A; g += G8) {
          double old[G8];
#pragma unroll
          for (int k2 = 0; k2 < G8; ++k2) old[k2] = ok ? __ldcg(d + (int64_t)B * (g + k2) * a.F) : 0.0;
#pragma unroll
          for (int k2 = 0; k2 < G8; ++k2) {
            if (ok) __stcg(d + (int64_t)B * (g + k2) * a.F, old[k2] + (double)acc[j][g + k2]);
            acc[j][g + k2] = 0.f;
          }
        }
      }
    }
    __syncthreads();   // every thread is done with buffer b
    if (tid == 0 && s + NS < total) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(s + NS);
    }
  }
  // leave no copy in flight into this CTA's shared memory (bounded): after an
  // abort at item s the copies still owed are those of items s .. s + NS - 1
  // (the ones issued), one per buffer
  if (tid == 0 && abort_flag) {
    for (int i = abort_at; i < abort_at + NS && i < total; ++i) {
      const int k = i % NS;
      long long spins = 0;
      while (!mbar_try_wait(&bar[k], (phases >> k) & 1u) && ++spins < kWaitLimit) {
      }
    }
  }
}

// --------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

template <int N0, int W>
static int launch_xtma(const msf_plan* p, const CUtensorMap* map, const XTmaArgs& a, cudaStream_t st, bool alone) {
  using S = XTmaShape<N0, W>;
  static int grid = 0, sms = 0;
  if (!grid) {
    cudaFuncSetAttribute(k_xpower_tma<N0, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    cudaFuncSetAttribute(k_xpower_tma<N0, W>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_xpower_tma<N0, W>, S::NT, S::SMEM);
    grid = (sms > 0 ? sms : 152) * (occ > 0 ? occ : 1);
  }
  // beside a plane FFT: 256 threads of x-pass CTAs per SM (they co-reside
  // with the plane CTA); alone: as many as fit
  const int cap = (p->overlap && !alone) ? (sms > 0 ? sms : 152) * (256 / S::NT) : grid;
  const int g = a.ntiles < cap ? a.ntiles : cap;
  k_xpower_tma<N0, W><<<g, S::NT, S::SMEM, st>>>(*map, a);
  return launch_status();
}

#define MSF_XTMA_CASES(X) X(64, 32) X(128, 16) X(128, 32) X(256, 32) X(256, 16) X(256, 8) X(512, 8)

bool xtma_ok(int n0, int w) {
#define X(A, B) if (n0 == A && w == B) return true;
  MSF_XTMA_CASES(X)
#undef X
  return false;
}

// Encodes the tensor map over the plan's spectra (after msf_plan_bind).
int xtma_prepare(msf_plan* p) {
  p->xtma_ready = 0;
  if (p->variant != 3 || !xtma_ok(p->n0, p->tile_w)) return MSF_OK;
  const int64_t F = (int64_t)p->n1 * p->nh;
  if ((F * sizeof(float2)) % 16 || (p->tile_w % 2)) return MSF_OK;
  EncodeTiledFn fn = encode_fn();
  if (!fn) return MSF_OK;
  const int box_rows = p->n0 <= 256 ? p->n0 : 256;
  cuuint64_t dims[2] = {(cuuint64_t)F, (cuuint64_t)p->batch * p->n0};
  cuuint64_t strides[1] = {(cuuint64_t)(F * sizeof(float2))};
  cuuint32_t box[2] = {(cuuint32_t)p->tile_w, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  for (int k = 0; k < (p->overlap ? 2 : 1); ++k) {
    CUtensorMap* m = reinterpret_cast<CUtensorMap*>(p->xtma_map[k]);
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, p->ws + (k ? p->off_cplx2 : p->off_cplx), dims,
                    strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return MSF_OK;   // plain loads then
  }
  p->xtma_ready = 1;
  return MSF_OK;
}

int xtma_batch(const msf_plan* p, int nframes, double* sf, cudaStream_t st, int buf, bool alone) {
  XTmaArgs a;
  a.nframes = nframes;
  a.F = (int64_t)p->n1 * p->nh;
  a.ntiles = (int)((a.F + p->tile_w - 1) / p->tile_w);
  a.sf = sf;
  a.twx = ws_ptr<float2>(p, p->off_tw[0]);
  a.status = ws_ptr<int>(p, p->off_status);
  const CUtensorMap* map = reinterpret_cast<const CUtensorMap*>(p->xtma_map[buf]);
#define X(A, B) if (p->n0 == A && p->tile_w == B) return launch_xtma<A, B>(p, map, a, st, alone);
  MSF_XTMA_CASES(X)
#undef X
  return MSF_E_UNSUPPORTED;
}

}  // namespace msf
