// msf_plan.cu -- plans, workspace layout, table initialisation, status.
//
// Replaces the grid set-up of dens.compute_sf (dens.py:181-189, 202,
// 237-263): the reference allocates numpy arrays per call; here a plan fixes
// the grid and the caller provides one device workspace that holds the FFT
// twiddle/position tables, the numpy.histogramdd bin edges, the density
// grids of one batch of frames and their half spectra.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "msf_internal.cuh"
#include "msf_tma.cuh"

namespace msf {

AxisPlan make_axis(int n) {
  AxisPlan a;
  memset(&a, 0, sizeof(a));
  a.n = n;
  int rem = n;
  int radices[kMaxStages * 2];
  int nr = 0;
  // radix 8 first (fewest passes through shared memory), then 4, 2, 5, 3,
  // then any remaining prime with the generic butterfly.
  while (rem % 8 == 0) { radices[nr++] = 8; rem /= 8; }
  while (rem % 4 == 0) { radices[nr++] = 4; rem /= 4; }
  while (rem % 2 == 0) { radices[nr++] = 2; rem /= 2; }
  while (rem % 5 == 0) { radices[nr++] = 5; rem /= 5; }
  while (rem % 3 == 0) { radices[nr++] = 3; rem /= 3; }
  for (int p = 7; rem > 1; p += 2) {
    while (rem % p == 0) { radices[nr++] = p; rem /= p; a.generic = 1; }
  }
  if (nr == 0) radices[nr++] = 1;  // n == 1: identity
  a.nst = nr;
  int span = n;
  for (int s = 0; s < nr; ++s) {
    a.R[s] = radices[s];
    a.m[s] = span / radices[s];
    span = a.m[s];
  }
  return a;
}

// Tables: twiddles exp(-2 pi i k/n) from FP64 sincospi rounded to float,
// DIF output positions, histogram edges (numpy.linspace(0, L, n+1):
// e[i] = i*(L/n), e[n] = L) and their float round-up / round-down images.
struct TabArgs {
  AxisPlan ax[4];         // x, y, z, half-y
  float2* tw[4];
  int* pos[4];
  int n[3];
  double L[3];
  double* edges;          // concatenated (n0+1, n1+1, n2+1)
  float* flo;
  float* fhi;
  int* status;    // zeroed unless NULL
};

__global__ void k_init_tables(TabArgs a) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int gs = gridDim.x * blockDim.x;
  for (int t = 0; t < 4; ++t) {
    if (!a.tw[t]) continue;
    const AxisPlan& ap = a.ax[t];
    for (int k = gt; k < ap.n; k += gs) {
      double s, c;
      sincospi(2.0 * (double)k / (double)ap.n, &s, &c);
      a.tw[t][k] = make_float2((float)c, (float)(-s));
      int kk = k, p = 0;
      for (int st = 0; st < ap.nst; ++st) {
        const int d = kk % ap.R[st];
        kk /= ap.R[st];
        p += d * ap.m[st];
      }
      a.pos[t][k] = p;
    }
  }
  int base = 0;
  for (int d = 0; d < 3; ++d) {
    const int n = a.n[d];
    const double step = __ddiv_rn(a.L[d], (double)n);
    for (int i = gt; i <= n; i += gs) {
      const double e = (i == n) ? a.L[d] : __dmul_rn((double)i, step);
      a.edges[base + i] = e;
      a.flo[base + i] = __double2float_ru(e);  // smallest float >= e
      a.fhi[base + i] = __double2float_rd(e);  // largest float <= e
    }
    base += n + 1;
  }
  if (a.status)
    for (int i = gt; i < kStatusWords; i += gs) a.status[i] = 0;
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

void plan_release(msf_plan* p) {
  for (int i = 0; i < 2; ++i) {
    if (p->ev_plane[i]) cudaEventDestroy(p->ev_plane[i]);
    if (p->ev_x[i]) cudaEventDestroy(p->ev_x[i]);
    if (p->ev_bucket[i]) cudaEventDestroy(p->ev_bucket[i]);
    p->ev_plane[i] = nullptr;
    p->ev_x[i] = nullptr;
    p->ev_bucket[i] = nullptr;
  }
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_plane_st) cudaEventDestroy(p->ev_plane_st);
  p->ev_fork = p->ev_plane_st = nullptr;
  if (p->side) cudaStreamDestroy(p->side);
  if (p->plane_st) cudaStreamDestroy(p->plane_st);
  if (p->bucket_st) cudaStreamDestroy(p->bucket_st);
  p->side = p->plane_st = p->bucket_st = nullptr;
}

}  // namespace msf

using namespace msf;

extern "C" {

const char* msf_strerror(int status) {
  switch (status) {
    case MSF_OK: return "ok";
    case MSF_E_INVALID: return "invalid argument";
    case MSF_E_UNSUPPORTED: return "unsupported size";
    case MSF_E_WORKSPACE: return "workspace missing or too small";
    case MSF_E_CUDA: return "CUDA runtime error";
    case MSF_E_RANGE: return "atom outside the padded grid";
    case MSF_E_NOT_BOUND: return "plan not bound to a workspace";
    case MSF_E_TIMEOUT: return "bounded device wait timed out";
    case MSF_E_TYPE: return "unknown atom type index";
    default: return "unknown status";
  }
}

int msf_version(void) { return 100; }

int msf_plan_create(msf_plan** out, const msf_plan_desc* d) {
  if (!out || !d) return MSF_E_INVALID;
  *out = nullptr;
  msf_plan* p = new (std::nothrow) msf_plan;
  if (!p) return MSF_E_INVALID;
  const int s = msf::plan_init(p, d);
  if (s) { delete p; return s; }
  *out = p;
  return MSF_OK;
}

}  // extern "C"

// Fills *p from *d (host only, no allocation).  Shared by msf_plan_create
// and by the entry points that keep their plan on the stack.
int msf::plan_init(msf_plan* p, const msf_plan_desc* d) {
  const int n[3] = {d->n0, d->n1, d->n2};
  for (int i = 0; i < 3; ++i)
    if (n[i] < 2 || n[i] > kMaxN) return MSF_E_UNSUPPORTED;
  for (int i = 0; i < 3; ++i)
    if (!(d->box[i] > 0.0) || !isfinite(d->box[i])) return MSF_E_INVALID;
  if (d->batch < 0 || d->batch > 256) return MSF_E_INVALID;
  if (d->variant < 0 || d->variant > 4) return MSF_E_INVALID;
  if (d->max_atoms < 0 || (d->options & ~(MSF_PLAN_NO_OVERLAP | MSF_PLAN_DIAG_STALL))) return MSF_E_INVALID;
  if (d->tile_w != 0 && d->tile_w != 4 && d->tile_w != 8 && d->tile_w != 16 && d->tile_w != 32)
    return MSF_E_INVALID;
  memset(p, 0, sizeof(*p));
  p->n0 = n[0]; p->n1 = n[1]; p->n2 = n[2];
  p->nh = n[2] / 2 + 1;
  p->batch = d->batch ? d->batch : 4;   // variant 3 default: below, once the variant is known
  for (int i = 0; i < 3; ++i) p->box[i] = d->box[i];
  for (int i = 0; i < 3; ++i) p->ax[i] = make_axis(n[i]);
  const int P = n[1] / 2;
  p->axp = make_axis(P >= 2 ? P : 2);

  // fused plane variant: n1 even, no generic radix on z or half-y, plane fits
  const int SP = P + ((P & 1) ? 0 : 1);
  // plane, z and half-y twiddles, w_{n1}^q (q < P), z and half-y positions
  const size_t plane_smem = (size_t)n[2] * SP * sizeof(float2) + (size_t)(n[2] + 2 * P) * sizeof(float2) +
                            (size_t)(n[2] + P) * sizeof(int);
  const bool plane_ok = (n[1] % 2 == 0) && P >= 2 && !p->ax[2].generic && !p->axp.generic &&
                        plane_smem <= 220 * 1024;
  const bool fused_ok = ct_plane_ok(n[1], n[2]) && ct_x_width(n[0], d->tile_w) > 0 && n[0] <= kMaxN;
  const bool smooth = smooth_ok(n[0]) && smooth_ok(n[1]) && smooth_ok(n[2]);
  int variant = d->variant;
  if (variant == 0) variant = fused_ok ? 3 : (smooth ? 4 : (plane_ok ? 1 : 2));
  if (variant == 1 && !plane_ok) return MSF_E_UNSUPPORTED;
  if (variant == 3 && !fused_ok) return MSF_E_UNSUPPORTED;
  if (variant == 4 && !smooth) return MSF_E_UNSUPPORTED;
  p->max_atoms = d->max_atoms;
  if (variant == 3 && !d->batch) {
    // the bucketed chain gains from long batches (fewer sf updates and bucket
    // launches per frame, longer overlap): as many frames as keep its two
    // spectrum buffers within 8 GiB, at most 64
    const double spectra = 2.0 * (double)n[0] * n[1] * (n[2] / 2 + 1) * sizeof(float2);
    const int64_t fit = (int64_t)((8.0 * 1024 * 1024 * 1024) / spectra);
    p->batch = (int)(fit < 1 ? 1 : (fit > 64 ? 64 : fit));
  }
  p->overlap = variant == 3 && !(d->options & MSF_PLAN_NO_OVERLAP);
  p->diag_stall = (d->options & MSF_PLAN_DIAG_STALL) ? 1 : 0;
  p->wait_limit = p->diag_stall ? kDiagWaitLimit : kWaitLimit;
  p->variant = variant;
  p->plane_smem = plane_smem;
  p->plane_threads = (n[2] * P >= 8192) ? 512 : 256;

  int w = d->tile_w;
  if (w == 0) {
    const int nmax = n[0] > n[1] ? n[0] : n[1];
    w = 16;
    while (w > 4 && nmax * w > 4096) w /= 2;
    while (w < 32 && nmax * w * 2 <= 4096) w *= 2;
  }
  // (the generic engine's column tiles hold at most 4096 values; the fused
  // chain checks its own instantiated widths)
  if (variant != 3 && (size_t)(n[0] > n[1] ? n[0] : n[1]) * w > 4096) return MSF_E_UNSUPPORTED;
  p->tile_w = w;
  if (variant == 3) p->tile_w = ct_x_width(n[0], d->tile_w);
  int g = d->rows_per_block;
  if (g == 0) {
    g = 2048 / n[2];
    if (g < 2) g = 2;
    if (g > 32) g = 32;
  }
  if (g < 1 || g > 64) return MSF_E_INVALID;
  p->rows_per_block = g;
  p->deposit_block = d->deposit_block ? d->deposit_block : 256;
  if (p->deposit_block % 32 || p->deposit_block > 1024) return MSF_E_INVALID;

  // workspace layout
  size_t o = 0;
  p->off_status = o; o = align_up(o + kStatusWords * sizeof(int));
  for (int i = 0; i < 3; ++i) { p->off_tw[i] = o; o = align_up(o + n[i] * sizeof(float2)); }
  p->off_twp = o; o = align_up(o + p->axp.n * sizeof(float2));
  for (int i = 0; i < 3; ++i) { p->off_pos[i] = o; o = align_up(o + n[i] * sizeof(int)); }
  p->off_posp = o; o = align_up(o + p->axp.n * sizeof(int));
  const int ne = n[0] + n[1] + n[2] + 3;
  p->off_edges_d = o; o = align_up(o + ne * sizeof(double));
  p->off_edges_flo = o; o = align_up(o + ne * sizeof(float));
  p->off_edges_fhi = o; o = align_up(o + ne * sizeof(float));
  // density grids: the bucketed variant never materialises them
  p->off_grid = o; o = align_up(o + (variant == 3 ? 0 : (size_t)p->batch * grid_elems(p) * sizeof(int32_t)));
  // per-block plane offsets and atom entries of the bucketed variant
  const int64_t nblk = variant == 3 ? (p->max_atoms + kBucketAtoms - 1) / kBucketAtoms : 0;
  p->off_counts = o;
  p->off_offsets = o; o = align_up(o + (size_t)p->batch * (nblk > 0 ? nblk : 1) * (n[0] + 1) * sizeof(int));
  p->off_cursor = o;
  p->off_bucket = o; o = align_up(o + (size_t)p->batch * nblk * kBucketAtoms * 8);
  p->pstride = variant == 3 ? ((p->max_atoms + n[0] + 1) & ~(int64_t)1) : 0;
  p->off_pbucket = o; o = align_up(o + (size_t)p->batch * p->pstride * 8);
  p->off_poff = o; o = align_up(o + (variant == 3 ? (size_t)p->batch * (n[0] + 1) * sizeof(int) : 0));
  p->off_pcount = o; o = align_up(o + (variant == 3 ? (size_t)p->batch * n[0] * sizeof(int) : 0));
  p->off_pcursor = o; o = align_up(o + (variant == 3 ? (size_t)p->batch * n[0] * sizeof(int) : 0));
  // with the overlap a second copy of the bucket arrays (off_offsets ..
  // here), so that one batch's bucket sort can run beside the plane FFT of
  // the batch before it
  p->bk_delta = (variant == 3 && p->overlap) ? o - p->off_offsets : 0;
  o += p->bk_delta;
  p->off_pnext = o; o = align_up(o + (variant == 3 ? sizeof(int) : 0));
  p->off_cplx = o; o = align_up(o + (size_t)p->batch * half_elems(p) * sizeof(float2));
  p->off_cplx2 = o; o = align_up(o + (p->overlap ? (size_t)p->batch * half_elems(p) * sizeof(float2) : 0));
  p->ws_bytes = o;
  return MSF_OK;
}

extern "C" {

int msf_plan_destroy(msf_plan* p) {
  if (p) plan_release(p);
  delete p;
  return MSF_OK;
}

size_t msf_plan_workspace_bytes(const msf_plan* p) { return p ? p->ws_bytes : 0; }

int msf_plan_bind(msf_plan* p, void* ws, size_t bytes, msf_stream_t stream) {
  if (!p || !ws) return MSF_E_INVALID;
  if (bytes < p->ws_bytes) return MSF_E_WORKSPACE;
  if (reinterpret_cast<uintptr_t>(ws) % 256) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  p->ws = static_cast<char*>(ws);
  TabArgs a;
  memset(&a, 0, sizeof(a));
  for (int i = 0; i < 3; ++i) {
    a.ax[i] = p->ax[i];
    a.tw[i] = ws_ptr<float2>(p, p->off_tw[i]);
    a.pos[i] = ws_ptr<int>(p, p->off_pos[i]);
    a.n[i] = p->ax[i].n;
    a.L[i] = p->box[i];
  }
  a.ax[3] = p->axp;
  a.tw[3] = ws_ptr<float2>(p, p->off_twp);
  a.pos[3] = ws_ptr<int>(p, p->off_posp);
  a.edges = ws_ptr<double>(p, p->off_edges_d);
  a.flo = ws_ptr<float>(p, p->off_edges_flo);
  a.fhi = ws_ptr<float>(p, p->off_edges_fhi);
  a.status = p->keep_status ? nullptr : ws_ptr<int>(p, p->off_status);
  k_init_tables<<<8, 256, 0, st>>>(a);
  int s = launch_status();
  if (s) return s;
  if (p->variant != 3) {
    s = cuda_status(cudaMemsetAsync(p->ws + p->off_grid, 0,
                                    (size_t)p->batch * grid_elems(p) * sizeof(int32_t), st));
    if (s) return s;
  } else {
    // per-plane counts start at zero; k_bucket_scan resets them after use
    for (int slot = 0; slot < (p->bk_delta ? 2 : 1) && !s; ++slot)
      s = cuda_status(cudaMemsetAsync(p->ws + p->off_pcount + (slot ? p->bk_delta : 0), 0,
                                      (size_t)p->batch * p->n0 * sizeof(int), st));
    if (s) return s;
  }
  if (p->overlap && !p->side) {
    // three streams, whatever the caller's stream is: the plane FFTs at the
    // device's greatest priority, so that their persistent CTAs are placed
    // first and the x passes and bucket sorts fill the room beside them; the
    // x passes and bucket sorts at the default priority
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking) != cudaSuccess) return MSF_E_CUDA;
    if (cudaStreamCreateWithPriority(&p->plane_st, cudaStreamNonBlocking, hi_prio) != cudaSuccess) return MSF_E_CUDA;
    if (cudaStreamCreateWithFlags(&p->bucket_st, cudaStreamNonBlocking) != cudaSuccess) return MSF_E_CUDA;
    for (int i = 0; i < 2; ++i) {
      if (cudaEventCreateWithFlags(&p->ev_plane[i], cudaEventDisableTiming) != cudaSuccess) return MSF_E_CUDA;
      if (cudaEventCreateWithFlags(&p->ev_x[i], cudaEventDisableTiming) != cudaSuccess) return MSF_E_CUDA;
      if (cudaEventCreateWithFlags(&p->ev_bucket[i], cudaEventDisableTiming) != cudaSuccess) return MSF_E_CUDA;
    }
    if (cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) != cudaSuccess) return MSF_E_CUDA;
    if (cudaEventCreateWithFlags(&p->ev_plane_st, cudaEventDisableTiming) != cudaSuccess) return MSF_E_CUDA;
  }
  if (p->variant == 3) {
    s = plane_twiddles_init();
    if (s) return s;
  }
  s = xtma_prepare(p);
  if (s) return s;
  p->chain_k = 0;
  p->bound = 1;
  return MSF_OK;
}

int msf_plan_status(msf_plan* p, msf_stream_t stream) {
  if (!p) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int h[kStatusWords];
  int s = cuda_status(cudaMemcpyAsync(h, p->ws + p->off_status, sizeof(h), cudaMemcpyDeviceToHost, st));
  if (s) return s;
  s = cuda_status(cudaStreamSynchronize(st));
  if (s) return s;
  if (h[kStatErr] == 0) return MSF_OK;
  s = cuda_status(cudaMemsetAsync(p->ws + p->off_status, 0, sizeof(h), st));
  if (s) return s;
  return h[kStatErr];
}

int msf_plan_query(const msf_plan* p, int32_t out[8]) {
  if (!p || !out) return MSF_E_INVALID;
  out[0] = p->variant;
  out[1] = p->tile_w;
  out[2] = p->rows_per_block;
  out[3] = p->batch;
  out[4] = p->deposit_block;
  out[5] = p->plane_threads;
  out[6] = p->xtma_ready;
  out[7] = p->nh;
  return MSF_OK;
}

}  // extern "C"
