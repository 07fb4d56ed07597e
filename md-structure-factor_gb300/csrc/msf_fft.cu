// msf_fft.cu -- 3-D real-to-complex FFT with |F|^2 and the frame sum fused.
//
// Replaces dens.py:313-318 (np.fft.rfftn(d1); conj(F)*F; sf += dmag).
// All butterflies run in FP32 with twiddles rounded from FP64 sincospi;
// the power of the frames of one batch is summed in FP32 in registers and
// added to the FP64 accumulator `sf` once per batch.
//
// Two sweeps through global memory for grids whose (y, z) plane fits in
// shared memory ("plane" variant):
//   k_plane   one CTA per (frame, x): z-FFT of row pairs y=2p,2p+1 packed
//             as x[2p] + i x[2p+1], half-length y-FFT over p, then the
//             two-dimensional real-pair split
//               E = (W[q,k] + conj W[-q,-k])/2,  O = (W[q,k] - conj W[-q,-k])/(2i)
//               Y[q,k] = E + w^q O,  Y[q+P,k] = E - w^q O   (w = e^{-2 pi i/n1})
//             written as the (n1, n2/2+1) half plane.
//   k_xpower  one CTA per tile of W consecutive (y, kz) columns: x-FFT of
//             every frame of the batch, |F|^2 summed over frames, sf += .
// Three sweeps otherwise ("split" variant: k_zrows, k_ycols, k_xpower),
// which also covers odd n1 and radices outside {2,3,4,5,8}.
#include "msf_internal.cuh"

namespace msf {

struct PlaneArgs {
  const void* grids;
  int64_t V;       // elements per frame grid
  float2* C;
  int64_t Vh;      // complex elements per frame half spectrum
  int n1, n2, nh, P, SP;
  AxisPlan az, ap;
  const float2* twz;
  const float2* twp;
  const float2* twy;
  const int* posz;
  const int* posp;
  int zero;
};

// ----------------------------------------------------------- plane kernel
template <int GK>
__global__ void __launch_bounds__(512) k_plane(PlaneArgs a) {
  extern __shared__ float2 smem[];
  const int n1 = a.n1, n2 = a.n2, nh = a.nh, P = a.P, SP = a.SP;
  float2* buf = smem;                    // [n2][SP]
  float2* twz = buf + (size_t)n2 * SP;   // n2
  float2* twp = twz + n2;                // P
  float2* twq = twp + P;                 // P: w_{n1}^q, q < P
  int* posz = reinterpret_cast<int*>(twq + P);
  int* posp = posz + n2;
  const int x = blockIdx.x;
  const int frame = blockIdx.y;
  const int64_t plane = (int64_t)n1 * n2;
  const int64_t gbase = frame * a.V + x * plane;

  copy_table(twz, a.twz, n2);
  copy_table(twp, a.twp, P);
  copy_table(twq, a.twy, P);
  copy_table(posz, a.posz, n2);
  copy_table(posp, a.posp, P);

  // rows y = 2p, 2p+1 packed as one complex line along z
  void* gw = const_cast<void*>(a.grids);
  gather_batched<8, float2>(
      P * n2,
      [&](int e) {
        const int p = e / n2, z = e - p * n2;
        const int64_t ia = gbase + (int64_t)(2 * p) * n2 + z;
        const float2 v = make_float2(load_grid<GK>(a.grids, ia), load_grid<GK>(a.grids, ia + n2));
        if (a.zero) { zero_grid<GK>(gw, ia); zero_grid<GK>(gw, ia + n2); }
        return v;
      },
      [&](int e, float2 v) {
        const int p = e / n2, z = e - p * n2;
        buf[z * SP + p] = v;
      });
  __syncthreads();
  fft_lines(buf, nullptr, a.az, twz, P, SP, 1, true);   // z, lines = pairs
  fft_lines(buf, nullptr, a.ap, twp, n2, 1, SP, false); // half-y, lines = kz positions

  float2* out = a.C + frame * a.Vh + (int64_t)x * n1 * nh;
  for (int e = threadIdx.x; e < P * nh; e += blockDim.x) {
    const int q = e / nh;
    const int k = e - q * nh;
    const int kn = (k == 0) ? 0 : n2 - k;
    const int qn = (q == 0) ? 0 : P - q;
    const float2 w = buf[posz[k] * SP + posp[q]];
    const float2 wm = cconj(buf[posz[kn] * SP + posp[qn]]);
    const float2 E = cscale(cadd(w, wm), 0.5f);
    const float2 O = cscale(cmi(csub(w, wm)), 0.5f);
    const float2 t = cmul(twq[q], O);
    out[(int64_t)q * nh + k] = cadd(E, t);
    out[(int64_t)(q + P) * nh + k] = csub(E, t);
  }
}

// ------------------------------------------------------------ z rows pass
struct RowsArgs {
  const void* grids;
  int64_t V;
  float2* C;
  int64_t Vh;
  int64_t rows;     // n0*n1 rows per frame
  int n2, nh, G;
  AxisPlan az;
  const float2* twz;
  const int* posz;
  int zero;
};

template <int GK>
__global__ void __launch_bounds__(256) k_zrows(RowsArgs a) {
  extern __shared__ float2 smem[];
  const int n2 = a.n2, nh = a.nh, G = a.G, S = G + 1;
  const bool gen = a.az.generic;
  float2* buf = smem;                         // [n2][S]
  float2* scratch = buf + (size_t)n2 * S;     // same size when generic
  float2* twz = scratch + (gen ? (size_t)n2 * S : 0);
  int* posz = reinterpret_cast<int*>(twz + n2);
  const int frame = blockIdx.y;
  const int64_t p0 = (int64_t)blockIdx.x * G;
  copy_table(twz, a.twz, n2);
  copy_table(posz, a.posz, n2);
  void* gw = const_cast<void*>(a.grids);
  gather_batched<8, float2>(
      G * n2,
      [&](int e) {
        const int g = e / n2, z = e - g * n2;
        const int64_t ra = 2 * (p0 + g);
        float va = 0.f, vb = 0.f;
        if (ra < a.rows) {
          const int64_t ia = frame * a.V + ra * n2 + z;
          va = load_grid<GK>(a.grids, ia);
          if (a.zero) zero_grid<GK>(gw, ia);
          if (ra + 1 < a.rows) {
            vb = load_grid<GK>(a.grids, ia + n2);
            if (a.zero) zero_grid<GK>(gw, ia + n2);
          }
        }
        return make_float2(va, vb);
      },
      [&](int e, float2 v) {
        const int g = e / n2, z = e - g * n2;
        buf[z * S + g] = v;
      });
  __syncthreads();
  fft_lines(buf, scratch, a.az, twz, G, S, 1, true);
  float2* out = a.C + frame * a.Vh;
  for (int e = threadIdx.x; e < G * nh; e += blockDim.x) {
    const int g = e / nh;
    const int k = e - g * nh;
    const int64_t ra = 2 * (p0 + g);
    if (ra >= a.rows) continue;
    const int kn = (k == 0) ? 0 : n2 - k;
    const float2 P_ = buf[posz[k] * S + g];
    const float2 Q_ = cconj(buf[posz[kn] * S + g]);
    out[ra * nh + k] = cscale(cadd(P_, Q_), 0.5f);
    if (ra + 1 < a.rows) out[(ra + 1) * nh + k] = cscale(cmi(csub(P_, Q_)), 0.5f);
  }
}

// ------------------------------------------------------------- y columns
struct ColsArgs {
  float2* C;
  int64_t Vh;
  int n1, nh;
  AxisPlan ay;
  const float2* twy;
  const int* posy;
};

template <int W>
__global__ void __launch_bounds__(256) k_ycols(ColsArgs a) {
  extern __shared__ float2 smem[];
  const int n1 = a.n1, nh = a.nh;
  const bool gen = a.ay.generic;
  float2* tile = smem;                          // [n1][W]
  float2* scratch = tile + (size_t)n1 * W;
  float2* tw = scratch + (gen ? (size_t)n1 * W : 0);
  int* pos = reinterpret_cast<int*>(tw + n1);
  const int ntile = (nh + W - 1) / W;
  const int x = blockIdx.x / ntile;
  const int k0 = (blockIdx.x - x * ntile) * W;
  const int weff = min(W, nh - k0);
  float2* base = a.C + blockIdx.y * a.Vh + (int64_t)x * n1 * nh + k0;
  copy_table(tw, a.twy, n1);
  copy_table(pos, a.posy, n1);
  gather_batched<8, float2>(
      n1 * W,
      [&](int e) {
        const int y = e / W, w = e % W;
        return (w < weff) ? base[(int64_t)y * nh + w] : make_float2(0.f, 0.f);
      },
      [&](int e, float2 v) { tile[e] = v; });
  __syncthreads();
  fft_lines(tile, scratch, a.ay, tw, W, W, 1, true);
  for (int e = threadIdx.x; e < n1 * W; e += blockDim.x) {
    const int y = e / W, w = e % W;
    if (w < weff) base[(int64_t)y * nh + w] = tile[pos[y] * W + w];
  }
}

// -------------------------------------------------- x pass + power + sum
struct XArgs {
  const float2* C;
  int64_t Vh;
  int nframes;
  double* sf;
  int n0;
  int64_t F;        // n1*nh columns
  AxisPlan ax;
  const float2* twx;
  const int* posx;
};

constexpr int kXThreads = 256;
constexpr int kXEpt = 16;

template <int W>
__global__ void __launch_bounds__(kXThreads) k_xpower(XArgs a) {
  extern __shared__ float2 smem[];
  const int n0 = a.n0;
  const bool gen = a.ax.generic;
  float2* tile = smem;                          // [n0][W]
  float2* scratch = tile + (size_t)n0 * W;
  float2* tw = scratch + (gen ? (size_t)n0 * W : 0);
  int* pos = reinterpret_cast<int*>(tw + n0);
  const int64_t f0 = (int64_t)blockIdx.x * W;
  const int weff = (int)min((int64_t)W, a.F - f0);
  copy_table(tw, a.twx, n0);
  copy_table(pos, a.posx, n0);
  float acc[kXEpt];
#pragma unroll
  for (int i = 0; i < kXEpt; ++i) acc[i] = 0.f;
  const int nel = n0 * W;
  for (int b = 0; b < a.nframes; ++b) {
    const float2* src = a.C + b * a.Vh + f0;
    __syncthreads();
    gather_batched<8, float2>(
        nel,
        [&](int e) {
          const int x = e / W, w = e % W;
          return (w < weff) ? __ldg(src + (int64_t)x * a.F + w) : make_float2(0.f, 0.f);
        },
        [&](int e, float2 v) { tile[e] = v; });
    __syncthreads();
    fft_lines(tile, scratch, a.ax, tw, W, W, 1, true);
#pragma unroll
    for (int i = 0; i < kXEpt; ++i) {
      const int e = threadIdx.x + i * kXThreads;
      if (e < nel) {
        const int x = e / W, w = e % W;
        const float2 v = tile[pos[x] * W + w];
        acc[i] = fmaf(v.x, v.x, fmaf(v.y, v.y, acc[i]));
      }
    }
    if (b == a.nframes - 1 || b % kPowerFlush == kPowerFlush - 1) {
#pragma unroll
      for (int i = 0; i < kXEpt; ++i) {
        const int e = threadIdx.x + i * kXThreads;
        if (e < nel) {
          const int x = e / W, w = e % W;
          if (w < weff) {
            double* d = a.sf + (int64_t)x * a.F + f0 + w;
            *d = *d + (double)acc[i];
          }
        }
        acc[i] = 0.f;
      }
    }
  }
}

// ----------------------------------------------------------------- launch
template <typename K>
static void allow_smem(K kernel) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <int GK>
static int launch_plane(msf_plan* p, const void* grids, int nframes, int zero, cudaStream_t st) {
  static bool once = false;
  if (!once) { allow_smem(k_plane<GK>); once = true; }
  PlaneArgs a;
  a.grids = grids;
  a.V = grid_elems(p);
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.n1 = p->n1; a.n2 = p->n2; a.nh = p->nh;
  a.P = p->n1 / 2;
  a.SP = a.P + ((a.P & 1) ? 0 : 1);
  a.az = p->ax[2];
  a.ap = p->axp;
  a.twz = ws_ptr<float2>(p, p->off_tw[2]);
  a.twp = ws_ptr<float2>(p, p->off_twp);
  a.twy = ws_ptr<float2>(p, p->off_tw[1]);
  a.posz = ws_ptr<int>(p, p->off_pos[2]);
  a.posp = ws_ptr<int>(p, p->off_posp);
  a.zero = zero;
  dim3 grid(p->n0, nframes);
  k_plane<GK><<<grid, p->plane_threads, p->plane_smem, st>>>(a);
  return launch_status();
}

template <int GK>
static int launch_zrows(msf_plan* p, const void* grids, int nframes, int zero, cudaStream_t st) {
  static bool once = false;
  if (!once) { allow_smem(k_zrows<GK>); once = true; }
  RowsArgs a;
  a.grids = grids;
  a.V = grid_elems(p);
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.rows = (int64_t)p->n0 * p->n1;
  a.n2 = p->n2; a.nh = p->nh; a.G = p->rows_per_block;
  a.az = p->ax[2];
  a.twz = ws_ptr<float2>(p, p->off_tw[2]);
  a.posz = ws_ptr<int>(p, p->off_pos[2]);
  a.zero = zero;
  const int64_t pairs = (a.rows + 1) / 2;
  dim3 grid((unsigned)((pairs + a.G - 1) / a.G), nframes);
  const size_t S = a.G + 1;
  const size_t smem = (size_t)p->n2 * S * sizeof(float2) * (a.az.generic ? 2 : 1) +
                      (size_t)p->n2 * (sizeof(float2) + sizeof(int));
  k_zrows<GK><<<grid, 256, smem, st>>>(a);
  return launch_status();
}

template <int W>
static int launch_ycols_w(msf_plan* p, int nframes, cudaStream_t st) {
  static bool once = false;
  if (!once) { allow_smem(k_ycols<W>); once = true; }
  ColsArgs a;
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.n1 = p->n1; a.nh = p->nh;
  a.ay = p->ax[1];
  a.twy = ws_ptr<float2>(p, p->off_tw[1]);
  a.posy = ws_ptr<int>(p, p->off_pos[1]);
  const int ntile = (p->nh + W - 1) / W;
  dim3 grid(p->n0 * ntile, nframes);
  const size_t smem = (size_t)p->n1 * W * sizeof(float2) * (a.ay.generic ? 2 : 1) +
                      (size_t)p->n1 * (sizeof(float2) + sizeof(int));
  k_ycols<W><<<grid, 256, smem, st>>>(a);
  return launch_status();
}

static int launch_ycols(msf_plan* p, int nframes, cudaStream_t st) {
  switch (p->tile_w) {
    case 4: return launch_ycols_w<4>(p, nframes, st);
    case 8: return launch_ycols_w<8>(p, nframes, st);
    case 16: return launch_ycols_w<16>(p, nframes, st);
    default: return launch_ycols_w<32>(p, nframes, st);
  }
}

template <int W>
static int launch_xpower_w(msf_plan* p, int nframes, double* sf, cudaStream_t st) {
  static bool once = false;
  if (!once) { allow_smem(k_xpower<W>); once = true; }
  XArgs a;
  a.C = ws_ptr<float2>(p, p->off_cplx);
  a.Vh = half_elems(p);
  a.nframes = nframes;
  a.sf = sf;
  a.n0 = p->n0;
  a.F = (int64_t)p->n1 * p->nh;
  a.ax = p->ax[0];
  a.twx = ws_ptr<float2>(p, p->off_tw[0]);
  a.posx = ws_ptr<int>(p, p->off_pos[0]);
  const unsigned nblk = (unsigned)((a.F + W - 1) / W);
  const size_t smem = (size_t)p->n0 * W * sizeof(float2) * (a.ax.generic ? 2 : 1) +
                      (size_t)p->n0 * (sizeof(float2) + sizeof(int));
  k_xpower<W><<<nblk, kXThreads, smem, st>>>(a);
  return launch_status();
}

static int launch_xpower(msf_plan* p, int nframes, double* sf, cudaStream_t st) {
  switch (p->tile_w) {
    case 4: return launch_xpower_w<4>(p, nframes, sf, st);
    case 8: return launch_xpower_w<8>(p, nframes, sf, st);
    case 16: return launch_xpower_w<16>(p, nframes, sf, st);
    default: return launch_xpower_w<32>(p, nframes, sf, st);
  }
}

template <int GK>
static int stage_a_kind(msf_plan* p, const void* grids, int nframes, int zero, cudaStream_t st) {
  if (p->variant == 1) return launch_plane<GK>(p, grids, nframes, zero, st);
  int s = launch_zrows<GK>(p, grids, nframes, zero, st);
  if (!s) s = launch_ycols(p, nframes, st);
  return s;
}

int fft_stage_a(msf_plan* p, const void* grids, int kind, int nframes, int zero, cudaStream_t st) {
  if (nframes < 1 || nframes > p->batch) return MSF_E_INVALID;
  // bucketed plans read caller grids with the compile-time plane kernel (never zeroing them)
  if (p->variant == 3) return fused_plane_batch(p, grids, kind, nframes, st);
  if (p->variant == 4) return smooth_stage_a(p, grids, kind, nframes, zero, st);
  switch (kind) {
    case kGridI32: return stage_a_kind<kGridI32>(p, grids, nframes, zero, st);
    case kGridF32: return stage_a_kind<kGridF32>(p, grids, nframes, zero, st);
    default: return stage_a_kind<kGridF64>(p, grids, nframes, zero, st);
  }
}

int fft_stage_b(msf_plan* p, int nframes, double* sf, cudaStream_t st) {
  if (nframes < 1 || nframes > p->batch) return MSF_E_INVALID;
  if (p->variant == 3) return fused_x_batch(p, nframes, sf, st);
  if (p->variant == 4) return smooth_stage_b(p, nframes, sf, st);
  return launch_xpower(p, nframes, sf, st);
}

int fft_power_batch(msf_plan* p, const void* grids, int kind, int nframes, double* sf, int zero,
                    cudaStream_t st) {
  int s = fft_stage_a(p, grids, kind, nframes, zero, st);
  if (!s) s = fft_stage_b(p, nframes, sf, st);
  return s;
}

}  // namespace msf

using namespace msf;

static int power_accum_any(msf_plan* p, const void* grids, int kind, size_t esize, int n_grids,
                           double* sf, msf_stream_t stream) {
  if (!p || !grids || !sf || n_grids < 0) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const char* g = static_cast<const char*>(grids);
  for (int f = 0; f < n_grids; f += p->batch) {
    const int nb = (n_grids - f < p->batch) ? n_grids - f : p->batch;
    int s = fft_power_batch(p, g + (size_t)f * grid_elems(p) * esize, kind, nb, sf, 0, st);
    if (s) return s;
  }
  return MSF_OK;
}

extern "C" {

int msf_power_accum_i32(msf_plan* p, const int32_t* grids, int32_t n_grids, double* sf,
                        msf_stream_t stream) {
  return power_accum_any(p, grids, kGridI32, sizeof(int32_t), n_grids, sf, stream);
}

int msf_power_accum_f32(msf_plan* p, const float* grids, int32_t n_grids, double* sf,
                        msf_stream_t stream) {
  return power_accum_any(p, grids, kGridF32, sizeof(float), n_grids, sf, stream);
}

int msf_power_accum_f64(msf_plan* p, const double* grids, int32_t n_grids, double* sf,
                        msf_stream_t stream) {
  return power_accum_any(p, grids, kGridF64, sizeof(double), n_grids, sf, stream);
}

}  // extern "C"
