// msf_noalloc.cu -- the histogram structure-factor chain for callers that
// cannot allocate device memory.
//
// Some hosts own every byte of device memory and forbid libraries to call
// cudaMalloc once they are running: an MD engine that calls analysis hooks
// between time steps from inside its own memory pool, a process started
// under a hard per-process memory quota, or a C/Fortran host program that has no
// allocator for device buffers beyond the arrays it already passes.  For
// them msf_hist_sf_f32_noalloc runs the same kernels as msf_hist_sf_f32 but
// keeps the plan on the stack and its workspace (FFT tables, bin edges, a
// batch of int32 density grids and their half spectra) in the fixed array
// below, which lives in the library image: every GPU that loads libmsf.so
// holds these kMsfNoAllocScratchBytes bytes until the process exits, and no
// call allocates or frees anything.
//
// Loading is the one exception: the CUDA runtime loads a module (with its
// __device__ arrays) and each kernel's code on first use, which takes device
// memory.  msf_noalloc_init runs the chain once on a grid shape, with no
// atoms, so that everything the chain needs for that shape is loaded while
// the host still allows it.
#include <string.h>

#include <mutex>

#include "msf_internal.cuh"

namespace msf {

constexpr size_t kMsfNoAllocScratchBytes = 32u << 20;  // 32 MiB
constexpr int kMaxDevices = 64;
// the last 256 bytes hold the placeholder atom of msf_noalloc_init
constexpr size_t kInitAtomBytes = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kMsfNoAllocScratchBytes];

// Device address of g_noalloc_scratch for each device.  In host code the
// symbol is only a host-side stand-in, so its address is looked up with
// cudaGetSymbolAddress (with that device current) the first time a device
// is used, and cached.
static void* g_scratch_ptr[kMaxDevices];
static std::mutex g_scratch_mu;

static int scratch_for_current_device(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return MSF_E_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MSF_E_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MSF_E_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return MSF_OK;
}

// The chain on a stack plan whose workspace is the scratch array (its first
// `room` bytes).  The status word (offset 0 of every plan layout) is not
// reset by the re-bind: an error stays latched until msf_noalloc_status.
static int noalloc_chain(const void* pos_w, int64_t n_atoms, int64_t n_frames, const double* box_host,
                         int32_t n0, int32_t n1, int32_t n2, int32_t flags, double* sf, cudaStream_t st,
                         size_t room) {
  // the largest batch (frames per pass, up to 8) whose workspace fits the scratch
  msf_plan plan;
  msf_plan_desc d;
  memset(&d, 0, sizeof(d));
  d.n0 = n0; d.n1 = n1; d.n2 = n2;
  d.box[0] = box_host[0]; d.box[1] = box_host[1]; d.box[2] = box_host[2];
  d.max_atoms = n_atoms;  // per-plane atom buckets of the bucketed variant
  d.options = MSF_PLAN_NO_OVERLAP;  // no internal stream or events: nothing is created
  int fit = 0;
  for (int b = 8; b >= 1 && !fit; b /= 2) {
    d.batch = b;
    const int s = plan_init(&plan, &d);
    if (s) return s;
    fit = plan.ws_bytes <= room;
  }
  if (!fit) return MSF_E_WORKSPACE;  // grid too large for the fixed scratch
  if (plan.off_status != 0) return MSF_E_CUDA;  // the status word must sit where msf_noalloc_status reads it
  void* scratch = nullptr;
  int s = scratch_for_current_device(&scratch);
  if (s) return s;
  // the scratch keeps whatever the previous call left: rebuilding the tables
  // and zeroing the per-plane counts / density grids here (msf_plan_bind)
  // restores the state the chain starts from; the chain itself leaves them
  // zeroed again.
  plan.keep_status = 1;
  s = msf_plan_bind(&plan, scratch, room, reinterpret_cast<msf_stream_t>(st));
  if (s) return s;
  return hist_sf_chain(&plan, pos_w, nullptr, kLayoutF32x4, n_atoms, n_frames, nullptr, flags, sf, st);
}

}  // namespace msf

using namespace msf;

extern "C" size_t msf_noalloc_scratch_bytes(void) { return kMsfNoAllocScratchBytes; }

extern "C" int msf_hist_sf_f32_noalloc(const void* pos_w, int64_t n_atoms, int64_t n_frames,
                                       const double* box_host, int32_t n0, int32_t n1, int32_t n2,
                                       int32_t flags, double* sf, msf_stream_t stream) {
  if (!box_host || !sf || n_atoms < 0 || n_frames < 0) return MSF_E_INVALID;
  if (n_atoms > 0 && n_frames > 0 && !pos_w) return MSF_E_INVALID;
  // one call is one whole chain: the plan-based continuation across calls
  // (MSF_CONTINUE) has no plan to carry it here
  if (flags & ~MSF_WRAP) return MSF_E_INVALID;
  return noalloc_chain(pos_w, n_atoms, n_frames, box_host, n0, n1, n2, flags, sf,
                       reinterpret_cast<cudaStream_t>(stream), kMsfNoAllocScratchBytes - kInitAtomBytes);
}

extern "C" int msf_noalloc_init(int32_t n0, int32_t n1, int32_t n2, double* sf, msf_stream_t stream) {
  if (!sf) return MSF_E_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  int s = scratch_for_current_device(&scratch);
  if (s) return s;
  // one placeholder atom at NaN (all bits set): every binning drops it, so
  // the launches below add exactly zero to sf
  void* atom = static_cast<char*>(scratch) + (kMsfNoAllocScratchBytes - kInitAtomBytes);
  s = cuda_status(cudaMemsetAsync(atom, 0xff, 16, st));
  if (s) return s;
  const double box[3] = {1.0, 1.0, 1.0};
  for (int32_t flags : {0, (int32_t)MSF_WRAP}) {
    s = noalloc_chain(atom, 1, 1, box, n0, n1, n2, flags, sf, st, kMsfNoAllocScratchBytes - kInitAtomBytes);
    if (s) return s;
  }
  return MSF_OK;
}

extern "C" int msf_noalloc_status(msf_stream_t stream) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int h[kStatusWords];
  int s = cuda_status(cudaMemcpyFromSymbolAsync(h, g_noalloc_scratch, sizeof(h), 0, cudaMemcpyDeviceToHost, st));
  if (s) return s;
  s = cuda_status(cudaStreamSynchronize(st));
  if (s) return s;
  if (h[kStatErr] == 0) return MSF_OK;
  void* scratch = nullptr;
  s = scratch_for_current_device(&scratch);
  if (s) return s;
  s = cuda_status(cudaMemsetAsync(scratch, 0, sizeof(h), st));
  if (s) return s;
  return h[kStatErr];
}
