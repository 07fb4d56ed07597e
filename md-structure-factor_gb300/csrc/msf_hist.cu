// msf_hist.cu -- electron-weighted histogram deposit and the fused chain.
//
// The reference splats a Gaussian per atom in a Python loop (dens.py:283-311);
// the plain method bins each atom's integer electron count into the voxel
// numpy.histogramdd assigns it to, so the int32 grid is bit-exact against
// np.histogramdd(pos, bins=(n0,n1,n2), range=[(0,L_i)], weights=w):
//   edges e[i] = i*(L/n), e[n] = L (numpy.linspace); bin = the largest i
//   with e[i] <= x; x == e[n] goes to bin n-1; x < 0, x > L, NaN dropped.
//
// float32 positions without rescale/wrap are binned in FP32 against two
// tables derived from the FP64 edges: flo[i] = smallest float >= e[i] and
// fhi[i] = largest float <= e[i].  For a float x, (double)x >= e[i] iff
// x >= flo[i] and (double)x <= e[i] iff x <= fhi[i], so the FP32 search
// gives exactly the FP64 answer without FP64 arithmetic (GB300 issues FP64
// at a small fraction of the FP32 rate).  Rescaled or wrapped positions and
// FP64 inputs are binned in FP64 with round-to-nearest intrinsics, so the
// compiler cannot fuse the rescale and wrap arithmetic (dens.py:58, 211-212)
// into FMAs that numpy does not do.
//
// Deposit: one atom per thread, float4 (x, y, z, w) loads, voxels of a warp
// matched with __match_any_sync and summed with __reduce_add_sync so that a
// voxel hit by several lanes takes one atomicAdd.
#include "msf_bins.cuh"

namespace msf {

// MODE 0: float4, FP32 binning; 1: float4, FP64 rescale/wrap; 2: FP64 (N,3) + int32 weights;
// 3: float (N,3) + int32 weights, FP32 binning; 4: float (N,3) + int32 weights, FP64 rescale/wrap
template <int MODE>
__global__ void k_hist_deposit(DepArgs a) {
  const int frame = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < a.n_atoms;
  int b0 = -1, b1 = -1, b2 = -1, wgt = 0;
  if (valid) {
    const double* s = a.scale ? a.scale + 3 * frame : nullptr;
    const bool wrap = a.flags & MSF_WRAP;
    if (MODE == 2) {
      const double* r = static_cast<const double*>(a.pos) + frame * a.frame_stride + 3 * i;
      wgt = __ldg(a.w + i);
      b0 = bin_f64(prep(__ldg(r + 0), s, 0, wrap, a.L0), a.n0, a.inv0, a.e0);
      b1 = bin_f64(prep(__ldg(r + 1), s, 1, wrap, a.L1), a.n1, a.inv1, a.e1);
      b2 = bin_f64(prep(__ldg(r + 2), s, 2, wrap, a.L2), a.n2, a.inv2, a.e2);
    } else if (MODE >= 3) {
      const float* r = static_cast<const float*>(a.pos) + frame * a.frame_stride + 3 * i;
      wgt = __ldg(a.w + i);
      const float x = __ldg(r + 0), y = __ldg(r + 1), z = __ldg(r + 2);
      if (MODE == 3) {
        b0 = bin_f32(x, a.n0, a.inv0, a.flo0, a.fhi0);
        b1 = bin_f32(y, a.n1, a.inv1, a.flo1, a.fhi1);
        b2 = bin_f32(z, a.n2, a.inv2, a.flo2, a.fhi2);
      } else {
        b0 = bin_f64(prep((double)x, s, 0, wrap, a.L0), a.n0, a.inv0, a.e0);
        b1 = bin_f64(prep((double)y, s, 1, wrap, a.L1), a.n1, a.inv1, a.e1);
        b2 = bin_f64(prep((double)z, s, 2, wrap, a.L2), a.n2, a.inv2, a.e2);
      }
    } else {
      const float4 v = __ldg(static_cast<const float4*>(a.pos) + frame * a.frame_stride + i);
      wgt = __float2int_rn(v.w);
      if (MODE == 0) {
        b0 = bin_f32(v.x, a.n0, a.inv0, a.flo0, a.fhi0);
        b1 = bin_f32(v.y, a.n1, a.inv1, a.flo1, a.fhi1);
        b2 = bin_f32(v.z, a.n2, a.inv2, a.flo2, a.fhi2);
      } else {
        b0 = bin_f64(prep((double)v.x, s, 0, wrap, a.L0), a.n0, a.inv0, a.e0);
        b1 = bin_f64(prep((double)v.y, s, 1, wrap, a.L1), a.n1, a.inv1, a.e1);
        b2 = bin_f64(prep((double)v.z, s, 2, wrap, a.L2), a.n2, a.inv2, a.e2);
      }
    }
    valid = (b0 >= 0) & (b1 >= 0) & (b2 >= 0);
  }
  const unsigned vm = __ballot_sync(0xffffffffu, valid);
  if (valid) {
    const int64_t key = frame * a.V + ((int64_t)b0 * a.n1 + b1) * a.n2 + b2;
    const unsigned peers = __match_any_sync(vm, (unsigned long long)key);
    const int sum = __reduce_add_sync(peers, wgt);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(a.grids + key, sum);
  }
}

int hist_deposit_batch(const msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int nframes, int64_t frame_stride, const double* scale,
                       int flags, int32_t* grids, cudaStream_t st) {
  if (n_atoms <= 0 || nframes <= 0) return MSF_OK;
  DepArgs a = dep_args(p);
  a.pos = pos;
  a.w = weights;
  a.n_atoms = n_atoms;
  a.frame_stride = frame_stride;
  a.scale = scale;
  a.flags = flags;
  a.grids = grids;
  const int bs = p->deposit_block;
  const int64_t nb = (n_atoms + bs - 1) / bs;
  if (nb > 0x7fffffff) return MSF_E_UNSUPPORTED;
  dim3 grid((unsigned)nb, nframes);
  const bool fp64_prep = scale || (flags & MSF_WRAP);
  if (layout == kLayoutF64) k_hist_deposit<2><<<grid, bs, 0, st>>>(a);
  else if (layout == kLayoutF32xyz) {
    if (fp64_prep) k_hist_deposit<4><<<grid, bs, 0, st>>>(a);
    else k_hist_deposit<3><<<grid, bs, 0, st>>>(a);
  } else {
    if (fp64_prep) k_hist_deposit<1><<<grid, bs, 0, st>>>(a);
    else k_hist_deposit<0><<<grid, bs, 0, st>>>(a);
  }
  return launch_status();
}

}  // namespace msf

using namespace msf;

static int check_flags(int flags) { return (flags & ~MSF_WRAP) ? MSF_E_INVALID : MSF_OK; }
static int check_chain_flags(int flags) {
  return (flags & ~(MSF_WRAP | MSF_CONTINUE)) ? MSF_E_INVALID : MSF_OK;
}

extern "C" {

int msf_hist_grid_f32(const msf_plan* p, const void* pos_w, int64_t n_atoms, const double* scale,
                      int32_t flags, int32_t* grid, msf_stream_t stream) {
  if (!p || !grid || n_atoms < 0 || (n_atoms > 0 && !pos_w)) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  if (check_flags(flags)) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (resolve_input(pos_w, st) || resolve_input(scale, st)) return MSF_E_INVALID;
  return hist_deposit_batch(p, pos_w, nullptr, kLayoutF32x4, n_atoms, 1, n_atoms, scale, flags, grid, st);
}

int msf_hist_grid_f32xyz(const msf_plan* p, const float* pos, const int32_t* weights,
                         int64_t n_atoms, const double* scale, int32_t flags, int32_t* grid,
                         msf_stream_t stream) {
  if (!p || !grid || n_atoms < 0 || (n_atoms > 0 && (!pos || !weights))) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  if (check_flags(flags)) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (resolve_input(pos, st) || resolve_input(weights, st) || resolve_input(scale, st)) return MSF_E_INVALID;
  return hist_deposit_batch(p, pos, weights, kLayoutF32xyz, n_atoms, 1, 3 * n_atoms, scale, flags, grid, st);
}

int msf_hist_grid_f64(const msf_plan* p, const double* pos, const int32_t* weights,
                      int64_t n_atoms, const double* scale, int32_t flags, int32_t* grid,
                      msf_stream_t stream) {
  if (!p || !grid || n_atoms < 0 || (n_atoms > 0 && (!pos || !weights))) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  if (check_flags(flags)) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (resolve_input(pos, st) || resolve_input(weights, st) || resolve_input(scale, st)) return MSF_E_INVALID;
  return hist_deposit_batch(p, pos, weights, kLayoutF64, n_atoms, 1, 3 * n_atoms, scale, flags, grid, st);
}

static int hist_sf_any(msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int64_t n_frames, const double* scale, int32_t flags,
                       double* sf, msf_stream_t stream) {
  if (!p || !sf || n_atoms < 0 || n_frames < 0) return MSF_E_INVALID;
  if (n_atoms > 0 && n_frames > 0 && (!pos || (layout != kLayoutF32x4 && !weights)))
    return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  if (check_chain_flags(flags)) return MSF_E_INVALID;
  const bool cont = flags & MSF_CONTINUE;
  flags &= ~MSF_CONTINUE;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (resolve_input(pos, st) || resolve_input(weights, st) || resolve_input(scale, st)) return MSF_E_INVALID;
  int32_t* grids = ws_ptr<int32_t>(p, p->off_grid);
  const int64_t fstride = layout == kLayoutF32x4 ? n_atoms : 3 * n_atoms;
  const size_t esize = layout == kLayoutF32x4 ? 4 * sizeof(float)
                       : (layout == kLayoutF64 ? sizeof(double) : sizeof(float));
  if (p->variant == 3 && n_atoms > p->max_atoms) return MSF_E_WORKSPACE;
  if (p->variant == 3 && p->overlap && (n_frames > p->batch || cont || p->chain_k > 0)) {
    // batch b: bucket sort into bucket slot b%2 on `bucket_st` (beside the
    // plane FFT of batch b-1), plane FFT into spectrum buffer b%2 on
    // `plane_st` (after that bucket sort), the x pass of batch b on `side`
    // (after that plane FFT), overlapping the plane FFT of batch b+1; the
    // bucket sort and plane FFT of batch b+2 wait for the plane FFT and the x
    // pass of batch b before reusing its slot and buffer.  The plan's streams
    // start after the caller's prior work and the caller's stream waits for
    // `plane_st` -- and through it every bucket sort: the positions have been
    // read -- at the end of every call; it joins `side` at the end of the
    // chain.  With MSF_CONTINUE the batch count carries over
    // to the next call and that join is left to the call that ends the
    // chain.
    int s = cuda_status(cudaEventRecord(p->ev_fork, st));
    if (!s) s = cuda_status(cudaStreamWaitEvent(p->bucket_st, p->ev_fork, 0));
    if (!s) s = cuda_status(cudaStreamWaitEvent(p->plane_st, p->ev_fork, 0));
    const cudaStream_t caller = st;
    st = p->plane_st;
    int64_t k = p->chain_k;
    // near-equal batches of at most p->batch frames: after a full batch a
    // short last one left the full batch's x pass to run on at one CTA per SM
    // once the short plane FFT beside it had ended (100 frames as 64 + 36:
    // 26.3 us per frame eager, 23.5 as 50 + 50; 160 frames as 64 + 64 + 32 in
    // a graph: 24.9 against 23.0 as 54 + 53 + 53)
    const int64_t nbat = (n_frames + p->batch - 1) / p->batch;
    for (int64_t f = 0, i = 0; f < n_frames && !s; ++i, ++k) {
      const int nb = (int)(n_frames / nbat + (i < n_frames % nbat ? 1 : 0));
      const int buf = (int)(k & 1);   // spectrum buffer and bucket slot
      const void* fp = static_cast<const char*>(pos) + (size_t)f * fstride * esize;
      // the bucket sort of batch k on its own stream, into slot buf once the
      // plane FFT of batch k-2 has read that slot: it runs beside the plane
      // FFT of batch k-1
      if (!s && k >= 2) s = cuda_status(cudaStreamWaitEvent(p->bucket_st, p->ev_plane[buf], 0));
      if (!s)
        s = fused_bucket_batch(p, fp, weights, layout, n_atoms, nb, fstride, scale ? scale + 3 * f : nullptr,
                               flags, p->bucket_st, buf);
      if (!s) s = cuda_status(cudaEventRecord(p->ev_bucket[buf], p->bucket_st));
      if (!s) s = cuda_status(cudaStreamWaitEvent(st, p->ev_bucket[buf], 0));
      if (!s && k >= 2) s = cuda_status(cudaStreamWaitEvent(st, p->ev_x[buf], 0));
      if (!s) s = fused_plane_batch(p, nullptr, kGridI32, nb, st, buf, buf);
      if (!s) s = cuda_status(cudaEventRecord(p->ev_plane[buf], st));
      if (!s) s = cuda_status(cudaStreamWaitEvent(p->side, p->ev_plane[buf], 0));
      // the last x pass of a chain has the SMs to itself
      if (!s) s = fused_x_batch(p, nb, sf, p->side, buf, !cont && f + nb >= n_frames);
      if (!s) s = cuda_status(cudaEventRecord(p->ev_x[buf], p->side));
      f += nb;
    }
    if (!s) s = cuda_status(cudaEventRecord(p->ev_plane_st, st));
    if (!s) s = cuda_status(cudaStreamWaitEvent(caller, p->ev_plane_st, 0));
    if (cont && !s) {
      p->chain_k = k;
      return MSF_OK;
    }
    p->chain_k = 0;
    // join: every x pass (recorded in order on `side`) precedes the last event
    if (k >= 1 && !s) s = cuda_status(cudaStreamWaitEvent(caller, p->ev_x[(k - 1) & 1], 0));
    return s;
  }
  for (int64_t f = 0; f < n_frames; f += p->batch) {
    const int nb = (int)((n_frames - f < p->batch) ? n_frames - f : p->batch);
    const void* fp = static_cast<const char*>(pos) + (size_t)f * fstride * esize;
    int s;
    if (p->variant == 3) {
      s = fused_bucket_batch(p, fp, weights, layout, n_atoms, nb, fstride,
                             scale ? scale + 3 * f : nullptr, flags, st);
      if (!s) s = fused_plane_batch(p, nullptr, kGridI32, nb, st);
      if (!s) s = fused_x_batch(p, nb, sf, st);
    } else {
      s = hist_deposit_batch(p, fp, weights, layout, n_atoms, nb, fstride,
                             scale ? scale + 3 * f : nullptr, flags, grids, st);
      if (!s) s = fft_power_batch(p, grids, kGridI32, nb, sf, 1, st);
    }
    if (s) return s;
  }
  return MSF_OK;
}

int msf_hist_sf_f32(msf_plan* p, const void* pos_w, int64_t n_atoms, int64_t n_frames,
                    const double* scale, int32_t flags, double* sf, msf_stream_t stream) {
  return hist_sf_any(p, pos_w, nullptr, kLayoutF32x4, n_atoms, n_frames, scale, flags, sf, stream);
}

int msf_hist_sf_f32xyz(msf_plan* p, const float* pos, const int32_t* weights, int64_t n_atoms,
                       int64_t n_frames, const double* scale, int32_t flags, double* sf,
                       msf_stream_t stream) {
  return hist_sf_any(p, pos, weights, kLayoutF32xyz, n_atoms, n_frames, scale, flags, sf, stream);
}

int msf_hist_batch_stages(msf_plan* p, int32_t stages, int32_t layout, const void* pos,
                          const int32_t* weights, int64_t n_atoms, int32_t n_frames,
                          const double* scale, int32_t flags, double* sf, msf_stream_t stream) {
  if (!p || n_atoms < 0 || n_frames < 1 || n_frames > p->batch) return MSF_E_INVALID;
  if (layout < kLayoutF32x4 || layout > kLayoutF32xyz || (stages & ~7) || check_flags(flags))
    return MSF_E_INVALID;
  if ((stages & 1) && n_atoms > 0 && (!pos || (layout != kLayoutF32x4 && !weights)))
    return MSF_E_INVALID;
  if ((stages & 4) && !sf) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (resolve_input(pos, st) || resolve_input(weights, st) || resolve_input(scale, st)) return MSF_E_INVALID;
  int32_t* grids = ws_ptr<int32_t>(p, p->off_grid);
  int s = MSF_OK;
  const bool bucketed = p->variant == 3;
  if (stages & 1) {
    const int64_t fstride = layout == kLayoutF32x4 ? n_atoms : 3 * n_atoms;
    s = bucketed ? fused_bucket_batch(p, pos, weights, layout, n_atoms, n_frames, fstride, scale, flags, st)
                 : hist_deposit_batch(p, pos, weights, layout, n_atoms, n_frames, fstride, scale, flags, grids, st);
  }
  if (!s && (stages & 2))
    s = bucketed ? fused_plane_batch(p, nullptr, kGridI32, n_frames, st)
                 : fft_stage_a(p, grids, kGridI32, n_frames, 1, st);
  if (!s && (stages & 4)) s = fft_stage_b(p, n_frames, sf, st);
  return s;
}

int msf_hist_sf_f64(msf_plan* p, const double* pos, const int32_t* weights, int64_t n_atoms,
                    int64_t n_frames, const double* scale, int32_t flags, double* sf,
                    msf_stream_t stream) {
  return hist_sf_any(p, pos, weights, kLayoutF64, n_atoms, n_frames, scale, flags, sf, stream);
}

}  // extern "C"

// The chain for callers inside the library that hold their own plan.
int msf::hist_sf_chain(msf_plan* p, const void* pos, const int32_t* weights, int layout,
                       int64_t n_atoms, int64_t n_frames, const double* scale, int32_t flags,
                       double* sf, cudaStream_t st) {
  return hist_sf_any(p, pos, weights, layout, n_atoms, n_frames, scale, flags, sf,
                     reinterpret_cast<msf_stream_t>(st));
}
