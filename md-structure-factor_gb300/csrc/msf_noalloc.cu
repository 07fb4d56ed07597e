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
#include <string.h>

#include <mutex>

#include "msf_internal.cuh"

namespace msf {

constexpr size_t kMsfNoAllocScratchBytes = 32u << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

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

}  // namespace msf

using namespace msf;

extern "C" size_t msf_noalloc_scratch_bytes(void) { return kMsfNoAllocScratchBytes; }

extern "C" int msf_hist_sf_f32_noalloc(const void* pos_w, int64_t n_atoms, int64_t n_frames,
                                       const double* box_host, int32_t n0, int32_t n1, int32_t n2,
                                       int32_t flags, double* sf, msf_stream_t stream) {
  if (!box_host || !sf || n_atoms < 0 || n_frames < 0) return MSF_E_INVALID;
  if (n_atoms > 0 && n_frames > 0 && !pos_w) return MSF_E_INVALID;
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
    fit = plan.ws_bytes <= kMsfNoAllocScratchBytes;
  }
  if (!fit) return MSF_E_WORKSPACE;  // grid too large for the fixed scratch
  void* scratch = nullptr;
  int s = scratch_for_current_device(&scratch);
  if (s) return s;
  // the scratch keeps whatever the previous call left: rebuilding the tables
  // and zeroing the density grids here (msf_plan_bind) restores the state the
  // chain starts from; the chain itself leaves the grids zeroed again.
  s = msf_plan_bind(&plan, scratch, kMsfNoAllocScratchBytes, stream);
  if (s) return s;
  return hist_sf_chain(&plan, pos_w, nullptr, kLayoutF32x4, n_atoms, n_frames, nullptr, flags, sf,
                       reinterpret_cast<cudaStream_t>(stream));
}
