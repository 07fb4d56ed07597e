/*
 * msf.h -- C ABI of libmsf.so, the GB300 (sm_103a) structure-factor library.
 *
 * The reference (joeyelk/MD-Structure-Factor) is pure Python: its hot path is
 * the function dens.compute_sf(r, L, typ, out_filename, rad, ucell, Sres)
 * (dens.py:166-346) and it has no FFI layer.  These entry points are what a
 * binding of that path binds: each one names the reference lines it replaces.
 *
 * Conventions (every entry point):
 *   - Every array argument is caller-owned DEVICE memory unless its name ends
 *     in _host.  Nothing here allocates device memory or synchronises the
 *     stream in a hot call; work is enqueued on `stream` (0 = legacy default).
 *   - Return value: MSF_OK (0) or a negative MSF_E* status; msf_strerror()
 *     turns it into text.  Errors detected on the GPU (e.g. an atom outside
 *     the padded grid in Gaussian mode) are latched into the plan's device
 *     status word and reported by msf_plan_status(), which synchronises.
 *   - Plans are immutable after msf_plan_bind(); one plan may be used from
 *     one stream at a time (its workspace is reused by every call).
 *   - Grid arrays are C order (x slowest, z fastest).  The half spectrum has
 *     shape (n0, n1, n2/2+1) like numpy.fft.rfftn; `sf` is FP64.
 */
#ifndef MSF_H_
#define MSF_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* msf_stream_t; /* == cudaStream_t */

enum {
  MSF_OK = 0,
  MSF_E_INVALID = -1,     /* bad argument (null pointer, bad size, bad flag) */
  MSF_E_UNSUPPORTED = -2, /* size outside what the plan supports */
  MSF_E_WORKSPACE = -3,   /* workspace missing or too small */
  MSF_E_CUDA = -4,        /* a CUDA runtime call failed */
  MSF_E_RANGE = -5,       /* an atom fell outside the grid (Gaussian mode) */
  MSF_E_NOT_BOUND = -6,   /* plan used before msf_plan_bind */
  MSF_E_TIMEOUT = -7,     /* a bounded device wait gave up */
  MSF_E_TYPE = -8         /* unknown atom type index */
};

/* Flags for the deposit / chain calls. */
enum {
  MSF_WRAP = 1,          /* periodic wrap r<L?r:r-L; r>0?r:r+L first (dens.py:204-212) */
  MSF_NO_ZERO_SF = 0,    /* (default) accumulate into sf */
  MSF_CONTINUE = 2       /* msf_hist_sf_* only: more calls on this plan, stream and sf
                            follow (e.g. chunks streamed from the host).  A bucketed plan
                            keeps its x pass overlapping across the calls and leaves the
                            last one running on its side stream; sf is complete on
                            `stream` only after a later call without this flag. */
};

const char* msf_strerror(int status);
int msf_version(void);          /* major*10000 + minor*100 + patch */

/* ------------------------------------------------------------------ plans
 * A plan fixes the grid (n0, n1, n2) and the number of frames processed per
 * batch.  It owns host-side tables only.  msf_plan_workspace_bytes() tells
 * how much device memory the caller must provide to msf_plan_bind(), which
 * fills the twiddle/edge tables on the device and zeroes the density grids.
 * Replaces: the grid set-up of dens.compute_sf (dens.py:181-189, 202,
 * 237-263) -- dims are given directly instead of from a resolution.
 */
typedef struct msf_plan msf_plan;

typedef struct msf_plan_desc {
  int32_t n0, n1, n2;     /* grid; each in [2, 1024] */
  int32_t batch;          /* frames per batch (>=1); 0 = default */
  double box[3];          /* box edges L used for binning (mean box when frames are rescaled) */
  int32_t variant;        /* 0 auto, 1 z+y plane from a global grid, 2 split rows/cols,
                             3 bucketed: atoms binned per x-plane and deposited in shared
                             memory by the plane FFT kernel (power-of-two grids),
                             4 smooth: three sweeps with compile-time mixed-radix FFTs
                             (every axis 2^a 3^b 5^c in 16..256, or 512) */
  int32_t tile_w;         /* columns per x-pass tile: 0 auto (variant 3: the widest tile of
                             at most 2048 values, 8 columns for 256-point lines), else 4..32 */
  int32_t rows_per_block; /* row pairs per z-pass block: 0 auto */
  int32_t deposit_block;  /* threads per deposit block: 0 auto */
  int64_t max_atoms;      /* atoms per frame the chain may be called with (sizes the per-plane
                             atom buckets of variant 3); 0 = no buckets */
  int32_t options;        /* MSF_PLAN_NO_OVERLAP: keep variant 3 on the caller's stream only;
                             MSF_PLAN_DIAG_STALL: diagnostic (below) */
} msf_plan_desc;

/* msf_plan_desc.options.  By default a variant-3 plan double-buffers its
 * spectra and its bucket arrays, and msf_plan_bind creates three internal
 * streams (the plane FFTs' at the device's greatest priority, the others at
 * the default) and eight events: a call over more than one batch runs each
 * batch's bucket sort beside the previous batch's plane FFT, its plane FFT,
 * and its x pass beside the next batch's plane FFT (forked from and joined
 * back to the caller's stream, so the calls stay stream-ordered and
 * graph-capturable; the caller's stream has passed the positions when the
 * call's work on it completes, with or without MSF_CONTINUE).
 * The kernels' waits on their own asynchronous copies are bounded (2^26
 * polls of the mbarrier): a wait that runs out latches MSF_E_TIMEOUT, the
 * kernel returns, and msf_plan_status() reports it.  MSF_PLAN_DIAG_STALL is
 * a diagnostic for that error path: the variant-3 plane kernel arms its
 * first wait for 16 bytes that no copy delivers and gives up after 2^14
 * polls, so every call on the plan ends in MSF_E_TIMEOUT (its sf is not
 * valid) while the context stays usable. */
enum { MSF_PLAN_NO_OVERLAP = 1, MSF_PLAN_DIAG_STALL = 2 };

int msf_plan_create(msf_plan** plan, const msf_plan_desc* desc);
int msf_plan_destroy(msf_plan* plan);
size_t msf_plan_workspace_bytes(const msf_plan* plan);
int msf_plan_bind(msf_plan* plan, void* workspace, size_t workspace_bytes, msf_stream_t stream);
/* Synchronises `stream`, returns and clears the device status word. */
int msf_plan_status(msf_plan* plan, msf_stream_t stream);
/* Effective tuning of a plan: variant, tile_w, rows_per_block, batch,
 * deposit_block, plane_threads, x pass fed by TMA (0/1), nh. */
int msf_plan_query(const msf_plan* plan, int32_t out[8]);

/* ------------------------------------------------ histogram deposit (a5)
 * One frame -> int32 grid (n0, n1, n2): grid[b] += w_j where b is the
 * numpy.histogramdd bin of atom j in [0, L) (last edge inclusive; atoms
 * outside or NaN are dropped), bit-exact with numpy.  `grid` is ADDED to:
 * zero it first for a plain histogram.
 *   pos_w:  n_atoms float4 (x, y, z, w) with w an integer electron count.
 *   scale:  NULL or 3 doubles: positions are multiplied by scale in FP64
 *           before binning (the per-frame factor of dens.py:46-62).
 * Stands in for the per-atom deposit of dens.py:283-311 (histogram form).
 */
int msf_hist_grid_f32(const msf_plan* plan, const void* pos_w, int64_t n_atoms,
                      const double* scale, int32_t flags, int32_t* grid, msf_stream_t stream);
/* float32 positions (n_atoms, 3) and int32 weights (n_atoms). */
int msf_hist_grid_f32xyz(const msf_plan* plan, const float* pos, const int32_t* weights,
                         int64_t n_atoms, const double* scale, int32_t flags, int32_t* grid,
                         msf_stream_t stream);
/* FP64 positions (n_atoms, 3) and int32 weights (n_atoms). */
int msf_hist_grid_f64(const msf_plan* plan, const double* pos, const int32_t* weights,
                      int64_t n_atoms, const double* scale, int32_t flags, int32_t* grid,
                      msf_stream_t stream);

/* ---------------------------------------- FFT power accumulate (a8, a9)
 * sf += sum over the n_grids int32 grids g of |rfftn(g)|^2.  Replaces
 * dens.py:313-318 (np.fft.rfftn, conj multiply, sf += dmag).  The grids are
 * read-only here.
 */
int msf_power_accum_i32(msf_plan* plan, const int32_t* grids, int32_t n_grids, double* sf,
                        msf_stream_t stream);
/* Same for float32 real grids (used by the Gaussian path). */
int msf_power_accum_f32(msf_plan* plan, const float* grids, int32_t n_grids, double* sf,
                        msf_stream_t stream);

/* ------------------------------------------ fused chain (a2, a4, a5, a8, a9)
 * For frames t in [0, n_frames): deposit frame t's histogram, rfftn,
 * |F|^2 and sf += -- the whole per-frame loop of dens.py:277-321 in
 * histogram form, batched at most `batch` frames per pass (a bucketed plan
 * with the overlap splits a call into ceil(n_frames / batch) near-equal
 * batches).  sf is accumulated (the reference's undivided sum,
 * dens.py:318).
 *   pos_w:  (n_frames, n_atoms) float4 (x, y, z, w).
 *   scale:  NULL or (n_frames, 3) doubles (per-frame rescale factors).
 * Input arrays (positions, weights, scale) of the deposit and chain calls
 * may be device memory or page-locked host memory (cudaHostAlloc /
 * cudaHostRegister): the kernels then read the host array in place through
 * its mapped address (on GB300 over NVLink-C2C), with no staging copy; it
 * must stay unchanged until the stream has passed the call.  Pageable host
 * memory is refused with MSF_E_INVALID before anything is launched.
 */
int msf_hist_sf_f32(msf_plan* plan, const void* pos_w, int64_t n_atoms, int64_t n_frames,
                    const double* scale, int32_t flags, double* sf, msf_stream_t stream);
/* pos: (n_frames, n_atoms, 3) floats, weights: (n_atoms) int32. */
int msf_hist_sf_f32xyz(msf_plan* plan, const float* pos, const int32_t* weights, int64_t n_atoms,
                       int64_t n_frames, const double* scale, int32_t flags, double* sf,
                       msf_stream_t stream);
/* One batch (n_frames <= the plan's batch) of the chain, stage by stage, so
 * that each stage can be timed or overlapped on its own: bit 1 = histogram
 * deposit into the workspace grids, bit 2 = z/y FFT passes into the
 * workspace spectra (zeroes the grids), bit 4 = x FFT pass, |F|^2 and
 * sf +=.  layout: 0 = float4 (x, y, z, w), 1 = FP64 (N, 3) + int32
 * weights, 2 = float32 (N, 3) + int32 weights.  Stages 1|2|4 together are
 * one batch of msf_hist_sf_*. */
int msf_hist_batch_stages(msf_plan* plan, int32_t stages, int32_t layout, const void* pos,
                          const int32_t* weights, int64_t n_atoms, int32_t n_frames,
                          const double* scale, int32_t flags, double* sf, msf_stream_t stream);
/* Verification view of the bucketed variant (variant 3): bins one frame
 * into the per-x-plane atom lists exactly as msf_hist_sf_* does and adds
 * them into the caller's int32 grid (`grid += histogram`), so the in-chain
 * binning can be compared with numpy.histogramdd bit for bit.  Layouts as
 * msf_hist_batch_stages. */
int msf_hist_bucket_grid(const msf_plan* plan, int32_t layout, const void* pos,
                         const int32_t* weights, int64_t n_atoms, const double* scale,
                         int32_t flags, int32_t* grid, msf_stream_t stream);
/* pos: (n_frames, n_atoms, 3) doubles, weights: (n_atoms) int32. */
int msf_hist_sf_f64(msf_plan* plan, const double* pos, const int32_t* weights, int64_t n_atoms,
                    int64_t n_frames, const double* scale, int32_t flags, double* sf,
                    msf_stream_t stream);

/* ------------------------------------------------ Gaussian deposit (a6, a7)
 * The reference's own density (dens.py:283-311): every atom adds
 * Nel/sigma^3 * exp(-|ucell^T (r - g)|^2 / (2 sigma^2)) on the box
 * [ir-A, ir+A) of the padded grid (ir = int(r/dr)), and the padding is
 * folded onto the periodic cell as remap_grid_tcl does (dens.py:86-108),
 * including its corner-block z destination (dens.py:107).  Computed in FP64
 * and written to `grid` (FP64, n0*n1*n2, overwritten).  An atom whose box
 * leaves the padded grid is skipped and latches MSF_E_RANGE (the reference
 * raises a numpy broadcast error there).
 *   pos:        (n_atoms, 3) doubles, already rescaled and wrapped.
 *   type_index: (n_atoms) int32 into the type table.
 *   type_tab:   (n_types, 5) doubles: c1 = Nel/sigma^3, c2 = 2*sigma^2,
 *               Ax, Ay, Az (the int() of the get_borders widths,
 *               dens.py:38-43, 287; c1, c2 as dens.py:308 computes them).
 *   geom:       16 doubles (host): dr[3], ucell[9] (row major), nborder,
 *               the largest footprint 2*max(A) over the types (0 = unknown:
 *               use the direct per-voxel exp), 0, 0.  With a footprint of at
 *               most 64 the density is evaluated in separable form (1-D and
 *               cross-term 2-D factor tables per atom; equal up to rounding).
 */
int msf_gauss_grid_f64(const msf_plan* plan, const double* pos, const int32_t* type_index,
                       int64_t n_atoms, const double* type_tab, int32_t n_types,
                       const double* geom_host, double* grid, msf_stream_t stream);
/* sf += |rfftn(grid)|^2 for FP64 grids (n_grids of them); the grid is
 * rounded to FP32 on load and transformed by the same FP32 FFT. */
int msf_power_accum_f64(msf_plan* plan, const double* grids, int32_t n_grids, double* sf,
                        msf_stream_t stream);

/* ------------------------------------------------------ plot array (a10)
 * sfplt = get_dplot(sf) (dens.py:142-163): fftshift in x and y, Hermitian
 * mirror in z, z-Nyquist dropped, DC := mean of its +x/+y/+z neighbours,
 * one voxel trimmed per face.  sf (n0, n1, nh) -> out (n0-2, n1-2, 2nh-3).
 */
int msf_sfplt(const double* sf, int32_t n0, int32_t n1, int32_t nh, double* out,
              msf_stream_t stream);

/* ---------------------------------------------------- Ewald slices (a12)
 * plot2d.Plot_Ewald_Sphere_Correction (plot2d.py:218-267): trilinear
 * interpolation (NaN outside) of the centred array D (p0, p1, p2) with axis
 * coordinates X, Y, Z at the Ewald-sphere points of the xy, xz and yz
 * planes, K = 2 pi / lambda.  Outputs (p0,p1), (p0,p2), (p1,p2).
 */
int msf_ewald(const double* D, int32_t p0, int32_t p1, int32_t p2, const double* X,
              const double* Y, const double* Z, double K, double* xy, double* xz, double* yz,
              msf_stream_t stream);

/* ------------------------------------------- cylindrical (r, z) average
 * The ring average of plot2d.PLOT_RAD_NEW (plot2d.py:601-631), the step the
 * reference CLI runs after compute_sf (main_gromacs.py:231 ->
 * plot2d.py:1008-1011): oa[ir][iz] = mean over the nth[ir] angles
 * t_i = i*2pi/nth[ir] of the trilinear interpolation (NaN outside) of the
 * centred array D (p0, p1, p2) with axes X, Y, Z at
 * (rarr[ir] cos t, rarr[ir] sin t, zar[iz]) * b_inv (b_inv_host: 9 doubles,
 * row major, host memory).  The host finishes as the reference does (NaN ->
 * smallest average, division by the mean, mirror to -r).
 */
int msf_cyl_average(const double* D, int32_t p0, int32_t p1, int32_t p2, const double* X,
                    const double* Y, const double* Z, const double* b_inv_host, const double* rarr,
                    const int32_t* nth, int32_t nr, const double* zar, int32_t nz, double* oa,
                    msf_stream_t stream);

/* ------------------------------------------------ (r, z) histograms
 * measure_intensity.py:58-120 (and plot2d.py:1035-1147): each voxel of the
 * centred S (p0, p1, p2) with axes X, Y, Z moves to
 * p = X[ix] b1 + Y[iy] b2 + Z[iz] b3 (b_host: rows b1, b2, b3, 9 doubles,
 * host memory); weight = S interpolated at p (mode 0: trilinear on the
 * original axes, NaN outside) or the voxel's own S (mode 1); r =
 * sqrt(px^2 + py^2) and pz are binned with numpy.histogram2d's explicit
 * edges (ascending; the last edge closes the last bin; outside or NaN
 * dropped) into hval (FP64 sums) and hcount (int64), both
 * (n_r_edges - 1) x (n_z_edges - 1) row major; they accumulate (zero them
 * first).
 */
int msf_rz_hist(const double* S, int32_t p0, int32_t p1, int32_t p2, const double* X, const double* Y,
                const double* Z, const double* b_host, int32_t mode, const double* r_edges, int32_t n_r_edges,
                const double* z_edges, int32_t n_z_edges, double* hval, int64_t* hcount, msf_stream_t stream);

/* ------------------------------------- nearest node of a sheared grid
 * NearestNDInterpolator over the transformed grid of plot2d.py:1087-1101
 * (the non-orthorhombic branch; a KD-tree there): out[e] = S at the node
 * p(i,j,k) = X[i] b1 + Y[j] b2 + Z[k] b3 nearest q[e] (FP64 squared
 * Euclidean distance; ties to the lowest flat index; NaN for a NaN query).
 * lattice_host (28 doubles, host): b1 b2 b3 (rows), p(0,0,0), the inverse of
 * M = rows (dX b1, dY b2, dZ b3) with the mean axis steps, a bound on the
 * distance of any node from its position in that uniform lattice (sum over
 * the axes of the largest deviation from equal steps times |b_a|), and the
 * upper Cholesky factor of M M^T (R00 R01 R02 R11 R12 R22).  The search
 * enumerates the lattice points of the distance ball (Fincke-Pohst) inside
 * the grid, so queries far outside the grid stay cheap.  index (optional, device, m int64) receives the
 * node's flat index.
 */
int msf_nearest_sheared(const double* S, int32_t p0, int32_t p1, int32_t p2, const double* X, const double* Y,
                        const double* Z, const double* lattice_host, const double* q, int64_t m, double* out,
                        int64_t* index, msf_stream_t stream);

/* --------------------------------------------- radial integrate (|q|^2)
 * plot2d.radial_integrate (plot2d.py:160-173): histograms of S over
 * R = f16(qx^2) + f16(qy^2) + f16(qz^2) with numpy's float16 equal-width bin
 * search (numpy >= 2 arithmetic: every step rounded to float16).
 * msf_radial_range: D (n_vox, 4) FP64 (qx, qy, qz, S), 16-byte aligned;
 *   stats (device, 3 u32) <- {min R bits, max R bits, 1 if any R is inf/NaN}.
 * msf_radial_bin_points: D as above; edges (device) the nbins + 1 float16
 *   edges (numpy.linspace(first, last, nbins + 1, dtype=float16), built by
 *   the caller from the range); hist (FP64) and count (int64) accumulate
 *   (zero them first); status bit 0 set if a bin index had to be clamped.
 *   1 <= nbins <= 2048, else MSF_E_UNSUPPORTED.
 * msf_radial_bin_grid: the same for the grid form of D -- S (p0, p1, p2)
 *   FP64 with qx = X[i], qy = Y[j], qz = Z[k]; hx/hy/hz (device) the float16
 *   tables f16(X^2), f16(Y^2), f16(Z^2).
 */
int msf_radial_range(const double* D, int64_t n_vox, uint32_t* stats, msf_stream_t stream);
int msf_radial_bin_points(const double* D, int64_t n_vox, const uint16_t* edges, int32_t nbins, double* hist,
                          int64_t* count, uint32_t* status, msf_stream_t stream);
int msf_radial_bin_grid(const double* S, int32_t p0, int32_t p1, int32_t p2, const uint16_t* hx,
                        const uint16_t* hy, const uint16_t* hz, const uint16_t* edges, int32_t nbins,
                        double* hist, int64_t* count, uint32_t* status, msf_stream_t stream);

/* ----------------------------------------------------- direct sum (a13)
 * S_q = |sum_j f_j exp(i q.r_j)|^2 for n_sys systems of n_atoms atoms and
 * n_q vectors each (FP32).  r_f: (n_sys, n_atoms) float4 (x, y, z, f);
 * q: (n_sys, n_q) float4 (qx, qy, qz, unused), or (n_q) shared by every
 * system when q_shared != 0; S: (n_sys, n_q) float; AB: (n_sys, n_q) float2
 * (A = sum f cos, B = sum f sin), saved for the adjoint.  No reference
 * counterpart: the continuous-position form of dens.py:313-316.
 */
int msf_direct_fwd(const void* r_f, int64_t n_atoms, const void* q, int64_t n_q, int32_t n_sys,
                   int32_t q_shared, float* S, void* AB, msf_stream_t stream);
/* Adjoint: given g = dL/dS (n_sys, n_q) float, writes (n_sys, n_atoms)
 * float4 (dL/dx, dL/dy, dL/dz, dL/df).  Recomputes the phases; no N x M
 * storage. */
int msf_direct_bwd(const void* r_f, int64_t n_atoms, const void* q, int64_t n_q, int32_t n_sys,
                   int32_t q_shared, const float* g, const void* AB, void* grad,
                   msf_stream_t stream);

/* ----------------------------------------- batched systems (CUDA graph)
 * Many independent systems -- each with its own atom count, frame count,
 * box and grid shape -- through the histogram chain of msf_hist_sf_f32 in
 * one CUDA graph.  Replaces calling dens.compute_sf (dens.py:166) once per
 * trajectory.  msf_batch_create plans every system (host only);
 * msf_batch_bind lays their workspaces out in one caller buffer of
 * msf_batch_workspace_bytes(), binds the plans and captures all chains into
 * a graph (spread over n_streams capture streams, largest systems first);
 * msf_batch_run launches it (sf += for every system).  The graph keeps the
 * device pointers given at creation: refresh positions in place between runs.
 * bind synchronises `stream` once (not a hot call).
 */
typedef struct msf_batch msf_batch;
typedef struct msf_batch_system {
  const void* pos_w;       /* device float4 (n_frames, n_atoms): x, y, z, electrons */
  const double* scale;     /* NULL or device (n_frames, 3) per-frame rescale factors */
  double* sf;              /* device FP64 (n0, n1, n2/2+1), accumulated */
  int64_t n_atoms, n_frames;
  double box[3];
  int32_t n0, n1, n2;
  int32_t flags;           /* MSF_WRAP or 0 */
  int32_t batch, variant, tile_w;   /* per-system tuning, 0 = default */
} msf_batch_system;

int msf_batch_create(msf_batch** batch, const msf_batch_system* systems, int32_t n_systems,
                     int32_t n_streams);
size_t msf_batch_workspace_bytes(const msf_batch* batch);
int msf_batch_bind(msf_batch* batch, void* workspace, size_t workspace_bytes, msf_stream_t stream);
int msf_batch_run(msf_batch* batch, msf_stream_t stream);
int msf_batch_query(const msf_batch* batch, int32_t index, int32_t out[8]);
int msf_batch_destroy(msf_batch* batch);

/* ------------------------------------------- allocation-free chain variant
 * No counterpart in the reference: an addition of this library for callers
 * that may not allocate device memory (e.g. an MD engine calling analysis
 * from inside its own memory pool, or a process under a hard device-memory
 * quota).  Same result as msf_hist_sf_f32 (sf += the frame sum of
 * |rfftn(histogram)|^2; pos_w device float4 (n_frames, n_atoms); box_host 3
 * doubles in host memory; flags 0 or MSF_WRAP -- MSF_CONTINUE is refused with
 * MSF_E_INVALID, one call is one whole chain), but the plan lives on the
 * stack and the workspace is a fixed 32 MiB array inside the library image,
 * which every GPU that loads libmsf.so holds until the process exits
 * (msf_noalloc_scratch_bytes()).  Grids whose batch-1 workspace does not fit
 * in it (e.g. 256x256x128 on the non-bucketed variants) return
 * MSF_E_WORKSPACE.  No call allocates or frees anything, with one
 * exception: loading.  The CUDA runtime loads the library's module (which
 * holds the 32 MiB array) and each kernel's code on first use, and that
 * takes device memory; so call msf_noalloc_init() once per device and grid
 * shape, while the host still allows allocation and before any stream
 * capture; calls on that shape then allocate nothing.  Every call reuses the
 * same array and re-initialises its tables, so calls that overlap on the GPU
 * (other streams, other threads) race and must be serialised by the caller.
 * Errors the kernels detect (MSF_E_TIMEOUT of a bounded wait) stay latched in
 * the array until msf_noalloc_status() reads them: check it after a call
 * whose result matters. */
int msf_hist_sf_f32_noalloc(const void* pos_w, int64_t n_atoms, int64_t n_frames,
                            const double* box_host, int32_t n0, int32_t n1, int32_t n2,
                            int32_t flags, double* sf, msf_stream_t stream);
size_t msf_noalloc_scratch_bytes(void);
/* Loads what msf_hist_sf_f32_noalloc needs on the current device for grid
 * (n0, n1, n2): looks up the array's device address and runs the chain once,
 * with and without MSF_WRAP, on one placeholder atom that every binning drops
 * (sf += 0: sf is a device FP64 (n0, n1, n2/2+1) array, left unchanged). */
int msf_noalloc_init(int32_t n0, int32_t n1, int32_t n2, double* sf, msf_stream_t stream);
/* Synchronises `stream`, returns the error latched by the allocation-free
 * calls on the current device since the last check (MSF_OK if none) and
 * clears it. */
int msf_noalloc_status(msf_stream_t stream);

/* ---------------------------------------------- trajectory ingest (host)
 * GROMACS .gro trajectories (one or more frames, fixed columns), read on the
 * host with one thread per frame group.  Replaces the .gro reading of
 * load_traj.py (process_gro_mdtraj, load_traj.py:91-110, through mdtraj:
 * coordinates nm -> Angstrom x10, unitcell lengths x10; load_gro,
 * load_traj.py:11-20: atom names from columns 11-15).
 * msf_gro_scan: atom and frame counts (MSF_E_UNSUPPORTED when the atom count
 * changes between frames).  msf_gro_read: xyz (n_frames, n_atoms, 3) float32
 * Angstrom = float32(nm field) * 10 in float32; box (n_frames, 3) the box
 * vector lengths (float32 norms) * 10; names NULL or n_atoms x 8 bytes
 * (the first frame's atom names, NUL padded); threads 0 = all cores. */
int msf_gro_scan(const char* path, int64_t* n_atoms, int64_t* n_frames);
/* GROMACS .trr trajectories (XDR, single or double precision), the
 * trajectory the reference CLI reads beside its .gro topology
 * (main_gromacs.py:95-101 -> process_gro_mdtraj, load_traj.py:91-110).
 * msf_trr_scan: atom and frame counts (MSF_E_UNSUPPORTED for a frame without
 * positions or a changing atom count).  msf_trr_read: xyz (n_frames,
 * n_atoms, 3) float32 Angstrom = float32(stored nm) * 10 in float32; box
 * (n_frames, 3) the box vector lengths (float32 norms) * 10, 0 for a frame
 * without a box; threads 0 = all cores. */
int msf_trr_scan(const char* path, int64_t* n_atoms, int64_t* n_frames);
int msf_trr_read(const char* path, int64_t n_atoms, int64_t n_frames, float* xyz, double* box, int32_t threads);
int msf_gro_read(const char* path, int64_t n_atoms, int64_t n_frames, float* xyz, double* box, char* names,
                 int32_t threads);

#ifdef __cplusplus
}
#endif
#endif /* MSF_H_ */
