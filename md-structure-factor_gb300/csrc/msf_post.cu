// msf_post.cu -- centred plot array (get_dplot) and Ewald-sphere slices.
#include "msf_internal.cuh"

namespace msf {

// dens.py:142-163.  With dmag = sf (n0, n1, nh) and the trimmed output
// (n0-2, n1-2, 2nh-3) indexed (i, j, k):
//   k >= nh-2 : sf[(i+1+n0/2) % n0, (j+1+n1/2) % n1, k-nh+2]        (shifted copy)
//   k <  nh-2 : sf[(n0-1-i+n0/2) % n0, (n1-1-j+n1/2) % n1, nh-2-k]   (z mirror)
// and the DC voxel (n0/2-1, n1/2-1, nh-2) := 1/3*((sf[1,0,0] + sf[0,1,0]) + sf[0,0,1]).
// A CTA takes kSfLines output lines (i, j) at a time, its threads along k:
// the index arithmetic is one 32-bit division per line instead of 64-bit
// divisions per voxel, the reads of a line (ascending or, mirrored,
// descending z) and its writes are contiguous, and each thread has the
// loads of all its lines in flight before it stores (the copy is bound by
// the bytes in flight: one line at a time ran at ~2 TB/s).
constexpr int kSfLines = 4;

__global__ void k_sfplt(const double* __restrict__ sf, int n0, int n1, int nh,
                        double* __restrict__ out) {
  const int m0 = n0 - 2, m1 = n1 - 2, m2 = 2 * nh - 3;
  const int lines = m0 * m1;
  for (int l0 = blockIdx.x * kSfLines; l0 < lines; l0 += gridDim.x * kSfLines) {
    for (int k = threadIdx.x; k < m2; k += blockDim.x) {
      double v[kSfLines];
#pragma unroll
      for (int u = 0; u < kSfLines; ++u) {
        const int line = l0 + u;
        v[u] = 0.0;
        if (line >= lines) continue;
        const int i = line / m1, j = line - i * m1;
        if (i == n0 / 2 - 1 && j == n1 / 2 - 1 && k == nh - 2) {
          const double a = __ldg(sf + (int64_t)1 * n1 * nh);
          const double b = __ldg(sf + nh);
          const double c = __ldg(sf + 1);
          v[u] = __dmul_rn(1.0 / 3.0, __dadd_rn(__dadd_rn(a, b), c));
        } else if (k >= nh - 2) {   // shifted copy
          const int64_t row = (int64_t)((i + 1 + n0 / 2) % n0) * n1 + (j + 1 + n1 / 2) % n1;
          v[u] = __ldg(sf + row * nh + (k - nh + 2));
        } else {                    // z mirror
          const int64_t row = (int64_t)((n0 - 1 - i + n0 / 2) % n0) * n1 + (n1 - 1 - j + n1 / 2) % n1;
          v[u] = __ldg(sf + row * nh + (nh - 2 - k));
        }
      }
#pragma unroll
      for (int u = 0; u < kSfLines; ++u)
        if (l0 + u < lines) out[(int64_t)(l0 + u) * m2 + k] = v[u];
    }
  }
}

// scipy's find_interval_ascending: i with x[i] <= v < x[i+1], the last
// interval closed on the right; -1 outside [x[0], x[n-1]] or NaN.
__device__ __forceinline__ int find_interval(const double* __restrict__ x, int n, double v) {
  const double a = __ldg(x), b = __ldg(x + n - 1);
  if (!(a <= v && v <= b)) return -1;
  if (v == b) return n - 2;
  // first guess for an evenly spaced axis, in FP32 (an FP64 division costs
  // more than the correction steps it saves), clamped before the conversion
  // (NaN -> 0), then corrected exactly: any start in [0, n-2] ends at the
  // same interval
  const float g = (float)(v - a) * ((float)(n - 1) / (float)(b - a));
  int i = g >= (float)(n - 2) ? n - 2 : (g >= 0.f ? (int)g : 0);
  while (i > 0 && v < __ldg(x + i)) --i;
  while (i < n - 2 && v >= __ldg(x + i + 1)) ++i;
  return i;
}

// RegularGridInterpolator(method='linear', bounds_error=False) at one point:
// corners in itertools.product order (lower before upper, x slowest), weight
// ((1*w0)*w1)*w2, terms summed in that order; NaN outside the grid.
__device__ double interp3(const double* __restrict__ D, int p0, int p1, int p2,
                          const double* X, const double* Y, const double* Z, double x, double y,
                          double z) {
  const int i0 = find_interval(X, p0, x);
  const int i1 = find_interval(Y, p1, y);
  const int i2 = find_interval(Z, p2, z);
  if (i0 < 0 || i1 < 0 || i2 < 0) return __longlong_as_double(0x7ff8000000000000LL);
  const double y0 = __ddiv_rn(__dsub_rn(x, __ldg(X + i0)), __dsub_rn(__ldg(X + i0 + 1), __ldg(X + i0)));
  const double y1 = __ddiv_rn(__dsub_rn(y, __ldg(Y + i1)), __dsub_rn(__ldg(Y + i1 + 1), __ldg(Y + i1)));
  const double y2 = __ddiv_rn(__dsub_rn(z, __ldg(Z + i2)), __dsub_rn(__ldg(Z + i2 + 1), __ldg(Z + i2)));
  const double w[3][2] = {{__dsub_rn(1.0, y0), y0}, {__dsub_rn(1.0, y1), y1}, {__dsub_rn(1.0, y2), y2}};
  double acc = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int a = (c >> 2) & 1, b = (c >> 1) & 1, d = c & 1;
    const double wt = __dmul_rn(__dmul_rn(__dmul_rn(1.0, w[0][a]), w[1][b]), w[2][d]);
    const double v = __ldg(D + ((int64_t)(i0 + a) * p1 + (i1 + b)) * p2 + (i2 + d));
    acc = __dadd_rn(acc, __dmul_rn(v, wt));
  }
  return acc;
}

// plot2d.py:236-263: theta = atan(sqrt(a^2 + b^2)/K); in-plane coordinates
// times cos(theta), the third K*(1 - cos(theta)).  cos(atan(t)) is computed
// as 1/sqrt(1 + t^2), the same number up to rounding (a few ulps), at a
// fraction of the FP64 cost of atan and cos.
__global__ void k_ewald(const double* __restrict__ D, int p0, int p1, int p2,
                        const double* __restrict__ X, const double* __restrict__ Y,
                        const double* __restrict__ Z, double K, double* xy, double* xz,
                        double* yz) {
  const int64_t nxy = (int64_t)p0 * p1, nxz = (int64_t)p0 * p2, nyz = (int64_t)p1 * p2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nxy + nxz + nyz;
       e += (int64_t)gridDim.x * blockDim.x) {
    int plane;
    int64_t r;
    if (e < nxy) { plane = 0; r = e; }
    else if (e < nxy + nxz) { plane = 1; r = e - nxy; }
    else { plane = 2; r = e - nxy - nxz; }
    const int nb = plane == 0 ? p1 : p2;
    const int ia = (int)(r / nb), ib = (int)(r % nb);
    const double A = plane == 2 ? __ldg(Y + ia) : __ldg(X + ia);
    const double Bv = plane == 0 ? __ldg(Y + ib) : __ldg(Z + ib);
    const double rho = sqrt(__dadd_rn(__dmul_rn(A, A), __dmul_rn(Bv, Bv)));
    const double t = __ddiv_rn(rho, K);
    const double c = __drcp_rn(__dsqrt_rn(__dadd_rn(1.0, __dmul_rn(t, t))));
    const double ua = __dmul_rn(A, c), ub = __dmul_rn(Bv, c), h = __dmul_rn(K, __dsub_rn(1.0, c));
    double v;
    if (plane == 0) { v = interp3(D, p0, p1, p2, X, Y, Z, ua, ub, h); xy[r] = v; }
    else if (plane == 1) { v = interp3(D, p0, p1, p2, X, Y, Z, ua, h, ub); xz[r] = v; }
    else { v = interp3(D, p0, p1, p2, X, Y, Z, h, ua, ub); yz[r] = v; }
  }
}

// plot2d.py:601-631 (PLOT_RAD_NEW): ring (r, z) of nth angles
// t_i = i * (2 pi / nth); the point (r cos t, r sin t, z) times b_inv (row
// vector times matrix), interpolated as RegularGridInterpolator does; the
// ring average is the mean over its angles (NaN if any sample is outside).
struct CylArgs {
  const double* D;
  int p0, p1, p2;
  const double* X;
  const double* Y;
  const double* Z;
  double b[9];
  const double* rarr;
  const int* nth;
  int nr;
  const double* zar;
  int nz;
  double* oa;
};

__global__ void k_cyl(CylArgs a) {
  const int64_t total = (int64_t)a.nr * a.nz;
  const double two_pi = 6.283185307179586232;   // the double nearest 2 pi (numpy's np.pi * 2.0)
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int ir = (int)(e / a.nz), iz = (int)(e % a.nz);
    const double r = __ldg(a.rarr + ir), z = __ldg(a.zar + iz);
    const int n = __ldg(a.nth + ir);
    const double step = __ddiv_rn(two_pi, (double)n);
    double sum = 0.0;
    for (int i = 0; i < n; ++i) {
      const double t = __dmul_rn((double)i, step);
      double s, c;
      sincos(t, &s, &c);
      const double px = __dmul_rn(r, c), py = __dmul_rn(r, s);
      const double qx = __dadd_rn(__dadd_rn(__dmul_rn(px, a.b[0]), __dmul_rn(py, a.b[3])), __dmul_rn(z, a.b[6]));
      const double qy = __dadd_rn(__dadd_rn(__dmul_rn(px, a.b[1]), __dmul_rn(py, a.b[4])), __dmul_rn(z, a.b[7]));
      const double qz = __dadd_rn(__dadd_rn(__dmul_rn(px, a.b[2]), __dmul_rn(py, a.b[5])), __dmul_rn(z, a.b[8]));
      sum = __dadd_rn(sum, interp3(a.D, a.p0, a.p1, a.p2, a.X, a.Y, a.Z, qx, qy, qz));
    }
    a.oa[e] = __ddiv_rn(sum, (double)n);
  }
}

// The (r, z) histograms of measure_intensity.py:58-120 (and the same steps
// in plot2d.py:1035-1147): every voxel (ix, iy, iz) of the centred grid is
// moved to p = X[ix] b1 + Y[iy] b2 + Z[iz] b3, accumulated per component in
// numpy's order ((X b1 + Y b2) + Z b3); its weight is S interpolated at p on
// the original axes (RegularGridInterpolator, linear, NaN outside; mode 0)
// or the voxel's own S (mode 1: the nearest-neighbour interpolator of the
// sheared grid evaluated at its own nodes, plot2d.py:1093-1101); r =
// sqrt(px^2 + py^2), z = pz; both binned with numpy.histogramdd's explicit
// edges (searchsorted right, a value equal to the last edge in the last bin,
// anything else outside -- or NaN -- dropped).  FP64 sums and int64 counts
// by global atomics.
struct RzArgs {
  const double* S;
  int p0, p1, p2;
  const double* X;
  const double* Y;
  const double* Z;
  double b[9];          // rows b1, b2, b3
  int mode;
  const double* re;     // r edges (nre)
  int nre;
  const double* ze;     // z edges (nze)
  int nze;
  double* hval;         // (nre - 1) x (nze - 1)
  unsigned long long* hcount;
};

// histogramdd's bin of v for ascending edges e[0..n-1]: -1 when dropped
__device__ __forceinline__ int edge_bin(const double* __restrict__ e, int n, double v) {
  int lo = 0, hi = n;   // count of edges <= v (searchsorted right)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(e + mid) <= v) lo = mid + 1; else hi = mid;
  }
  if (v == __ldg(e + n - 1)) lo = n - 1;
  return (lo >= 1 && lo <= n - 1) ? lo - 1 : -1;
}

__global__ void k_rz_hist(RzArgs a) {
  const int64_t total = (int64_t)a.p0 * a.p1 * a.p2;
  const int nz = a.nze - 1;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int iz = (int)(e % a.p2);
    const int64_t t = e / a.p2;
    const int iy = (int)(t % a.p1), ix = (int)(t / a.p1);
    const double xv = __ldg(a.X + ix), yv = __ldg(a.Y + iy), zv = __ldg(a.Z + iz);
    double p[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
      p[c] = __dadd_rn(__dadd_rn(__dmul_rn(xv, a.b[c]), __dmul_rn(yv, a.b[3 + c])), __dmul_rn(zv, a.b[6 + c]));
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(p[0], p[0]), __dmul_rn(p[1], p[1])));
    const int br = edge_bin(a.re, a.nre, r);
    const int bz = edge_bin(a.ze, a.nze, p[2]);
    if (br < 0 || bz < 0) continue;
    const double w = a.mode == 0 ? interp3(a.S, a.p0, a.p1, a.p2, a.X, a.Y, a.Z, p[0], p[1], p[2]) : __ldg(a.S + e);
    const int64_t bin = (int64_t)br * nz + bz;
    atomicAdd(a.hval + bin, w);
    atomicAdd(a.hcount + bin, 1ull);
  }
}

// NearestNDInterpolator over the sheared grid (plot2d.py:1087-1101): the
// nodes are p(i, j, k) = X[i] b1 + Y[j] b2 + Z[k] b3 (numpy's order per
// component, as k_rz_hist), the value at a query q is S at the node nearest
// q in FP64 squared Euclidean distance ((dx^2 + dy^2) + dz^2, scipy's
// cKDTree order).  Search (Fincke-Pohst enumeration): in the uniform-lattice
// model p = o + u M (u a real index vector, M rows dX b1, dY b2, dZ b3),
// |q - p|^2 = (u - f) G (u - f)^T with f = (q - o) M^-1 and G = M M^T =
// R^T R (R upper triangular), i.e. the sum over k of
// (sum_{j >= k} R_kj (u_j - f_j))^2.  Starting from the node nearest round(f)
// clamped to the grid, at distance rho, every node within rho lies within
// rho + delta in the model (delta bounds a node's distance from its model
// position: the axes' deviation from equal steps), so the enumeration of
// index 2, then 1 given 2, then 0 given both, each interval intersected
// with the grid, holds the nearest node; the radius shrinks as closer nodes
// are found.  Queries outside the grid enumerate only the part of the ball
// inside it.  Ties go to the lowest flat index (C order).  A query with a
// NaN or infinite coordinate gets NaN (index -1) before any index
// arithmetic.
struct NearestArgs {
  const double* S;
  int p0, p1, p2;
  const double* X;
  const double* Y;
  const double* Z;
  double b[9];      // rows b1, b2, b3
  double o[3];      // p(0, 0, 0)
  double minv[9];   // inverse of M (row major)
  double delta;     // bound on |node - its uniform-lattice model|
  double r[6];      // R00 R01 R02 R11 R12 R22
  const double* q;  // (m, 3)
  int64_t m;
  double* out;
  int64_t* index;   // optional: flat index of the nearest node
};

__device__ __forceinline__ void node_pos(const NearestArgs& a, int i, int j, int k, double* p) {
  const double xv = __ldg(a.X + i), yv = __ldg(a.Y + j), zv = __ldg(a.Z + k);
#pragma unroll
  for (int c = 0; c < 3; ++c)
    p[c] = __dadd_rn(__dadd_rn(__dmul_rn(xv, a.b[c]), __dmul_rn(yv, a.b[3 + c])), __dmul_rn(zv, a.b[6 + c]));
}

__device__ __forceinline__ double dist2(const double* p, double qx, double qy, double qz) {
  const double dx = __dsub_rn(p[0], qx), dy = __dsub_rn(p[1], qy), dz = __dsub_rn(p[2], qz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// an index from a real number, clamped to [0, n-1]; NaN gives 0 (never
// converted: a NaN to int conversion is undefined)
__device__ __forceinline__ int clamp_index(double r, int n) {
  if (!(r >= 0.0)) return 0;
  if (r >= (double)(n - 1)) return n - 1;
  return (int)r;
}

__global__ void k_nearest(NearestArgs a) {
  constexpr double kRel = 1.0 + 1e-9, kAbs = 1e-6;   // margins for the rounding of the bounds
  const double R00 = a.r[0], R01 = a.r[1], R02 = a.r[2], R11 = a.r[3], R12 = a.r[4], R22 = a.r[5];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.m; e += (int64_t)gridDim.x * blockDim.x) {
    const double qx = __ldg(a.q + 3 * e), qy = __ldg(a.q + 3 * e + 1), qz = __ldg(a.q + 3 * e + 2);
    if (!(isfinite(qx) && isfinite(qy) && isfinite(qz))) {   // no finite nearest node: NaN
      a.out[e] = __longlong_as_double(0x7ff8000000000000LL);
      if (a.index) a.index[e] = -1;
      continue;
    }
    const double d[3] = {qx - a.o[0], qy - a.o[1], qz - a.o[2]};
    double f[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] = d[0] * a.minv[c] + d[1] * a.minv[3 + c] + d[2] * a.minv[6 + c];
    const int c0 = clamp_index(rint(f[0]), a.p0), c1 = clamp_index(rint(f[1]), a.p1),
              c2 = clamp_index(rint(f[2]), a.p2);
    double p[3];
    node_pos(a, c0, c1, c2, p);
    double best = dist2(p, qx, qy, qz);
    int64_t bi = ((int64_t)c0 * a.p1 + c1) * a.p2 + c2;
    double rad = sqrt(best) + a.delta;
    const double w2 = rad * kRel / R22;
    const int lo2 = clamp_index(floor(f[2] - w2 - kAbs), a.p2), hi2 = clamp_index(ceil(f[2] + w2 + kAbs), a.p2);
    for (int i2 = lo2; i2 <= hi2; ++i2) {
      const double u2 = (double)i2 - f[2];
      const double t2 = R22 * u2;
      const double r1sq = rad * rad * kRel - t2 * t2;
      if (r1sq < 0.0) continue;
      const double r1 = sqrt(r1sq);
      const double cen1 = f[1] - R12 * u2 / R11;
      const int lo1 = clamp_index(floor(cen1 - r1 / R11 - kAbs), a.p1);
      const int hi1 = clamp_index(ceil(cen1 + r1 / R11 + kAbs), a.p1);
      for (int i1 = lo1; i1 <= hi1; ++i1) {
        const double u1 = (double)i1 - f[1];
        const double t1 = R11 * u1 + R12 * u2;
        const double r0sq = rad * rad * kRel - t2 * t2 - t1 * t1;
        if (r0sq < 0.0) continue;
        const double r0 = sqrt(r0sq);
        const double cen0 = f[0] - (R01 * u1 + R02 * u2) / R00;
        const int lo0 = clamp_index(floor(cen0 - r0 / R00 - kAbs), a.p0);
        const int hi0 = clamp_index(ceil(cen0 + r0 / R00 + kAbs), a.p0);
        for (int i0 = lo0; i0 <= hi0; ++i0) {
          node_pos(a, i0, i1, i2, p);
          const double d2 = dist2(p, qx, qy, qz);
          const int64_t fi = ((int64_t)i0 * a.p1 + i1) * a.p2 + i2;
          if (d2 < best || (d2 == best && fi < bi)) {
            best = d2;
            bi = fi;
            rad = sqrt(best) + a.delta;   // the remaining intervals shrink with it
          }
        }
      }
    }
    a.out[e] = __ldg(a.S + bi);
    if (a.index) a.index[e] = bi;
  }
}

}  // namespace msf

using namespace msf;

extern "C" int msf_nearest_sheared(const double* S, int32_t p0, int32_t p1, int32_t p2, const double* X,
                                   const double* Y, const double* Z, const double* lattice_host,
                                   const double* q, int64_t m, double* out, int64_t* index, msf_stream_t stream) {
  if (!S || !X || !Y || !Z || !lattice_host || (!q && m) || (!out && m) || m < 0) return MSF_E_INVALID;
  if (p0 < 1 || p1 < 1 || p2 < 1) return MSF_E_INVALID;
  if (m == 0) return MSF_OK;
  NearestArgs a;
  a.S = S; a.p0 = p0; a.p1 = p1; a.p2 = p2;
  a.X = X; a.Y = Y; a.Z = Z;
  for (int i = 0; i < 9; ++i) a.b[i] = lattice_host[i];
  for (int i = 0; i < 3; ++i) a.o[i] = lattice_host[9 + i];
  for (int i = 0; i < 9; ++i) a.minv[i] = lattice_host[12 + i];
  a.delta = lattice_host[21];
  if (!(a.delta >= 0.0) || a.delta > 1e300) return MSF_E_INVALID;
  for (int i = 0; i < 6; ++i) a.r[i] = lattice_host[22 + i];
  // R's diagonal positive and finite (a non-singular lattice)
  if (!(a.r[0] > 0.0 && a.r[3] > 0.0 && a.r[5] > 0.0) || !(a.r[0] < 1e300 && a.r[3] < 1e300 && a.r[5] < 1e300))
    return MSF_E_INVALID;
  a.q = q; a.m = m; a.out = out; a.index = index;
  const int blocks = (int)((m + 127) / 128 < 152 * 16 ? (m + 127) / 128 : 152 * 16);
  k_nearest<<<blocks, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(a);
  return launch_status();
}

extern "C" int msf_rz_hist(const double* S, int32_t p0, int32_t p1, int32_t p2, const double* X, const double* Y,
                           const double* Z, const double* b_host, int32_t mode, const double* r_edges,
                           int32_t n_r_edges, const double* z_edges, int32_t n_z_edges, double* hval,
                           int64_t* hcount, msf_stream_t stream) {
  if (!S || !X || !Y || !Z || !b_host || !r_edges || !z_edges || !hval || !hcount) return MSF_E_INVALID;
  if (p0 < 2 || p1 < 2 || p2 < 2 || n_r_edges < 2 || n_z_edges < 2 || (mode != 0 && mode != 1))
    return MSF_E_INVALID;
  RzArgs a;
  a.S = S; a.p0 = p0; a.p1 = p1; a.p2 = p2;
  a.X = X; a.Y = Y; a.Z = Z;
  for (int i = 0; i < 9; ++i) a.b[i] = b_host[i];
  a.mode = mode;
  a.re = r_edges; a.nre = n_r_edges; a.ze = z_edges; a.nze = n_z_edges;
  a.hval = hval;
  a.hcount = reinterpret_cast<unsigned long long*>(hcount);
  const int64_t total = (int64_t)p0 * p1 * p2;
  const int blocks = (int)((total + 255) / 256 < 152 * 8 ? (total + 255) / 256 : 152 * 8);
  k_rz_hist<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(a);
  return launch_status();
}

extern "C" int msf_cyl_average(const double* D, int32_t p0, int32_t p1, int32_t p2, const double* X,
                               const double* Y, const double* Z, const double* b_inv_host,
                               const double* rarr, const int32_t* nth, int32_t nr, const double* zar,
                               int32_t nz, double* oa, msf_stream_t stream) {
  if (!D || !X || !Y || !Z || !b_inv_host || !rarr || !nth || !zar || !oa) return MSF_E_INVALID;
  if (p0 < 2 || p1 < 2 || p2 < 2 || nr < 1 || nz < 1) return MSF_E_INVALID;
  CylArgs a;
  a.D = D; a.p0 = p0; a.p1 = p1; a.p2 = p2;
  a.X = X; a.Y = Y; a.Z = Z;
  for (int i = 0; i < 9; ++i) a.b[i] = b_inv_host[i];
  a.rarr = rarr; a.nth = nth; a.nr = nr; a.zar = zar; a.nz = nz; a.oa = oa;
  const int64_t total = (int64_t)nr * nz;
  const int blocks = (int)((total + 127) / 128 < 152 * 16 ? (total + 127) / 128 : 152 * 16);
  k_cyl<<<blocks, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(a);
  return launch_status();
}

extern "C" {

int msf_sfplt(const double* sf, int32_t n0, int32_t n1, int32_t nh, double* out,
              msf_stream_t stream) {
  if (!sf || !out) return MSF_E_INVALID;
  if (n0 < 4 || n1 < 4 || nh < 3 || (n0 & 1) || (n1 & 1)) return MSF_E_UNSUPPORTED;
  const int lines = (n0 - 2) * (n1 - 2);
  const int threads = 2 * nh - 3 <= 128 ? 128 : 256;
  const int groups = (lines + kSfLines - 1) / kSfLines;
  const int blocks = groups < 152 * 16 ? groups : 152 * 16;
  k_sfplt<<<blocks, threads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(sf, n0, n1, nh, out);
  return launch_status();
}

int msf_ewald(const double* D, int32_t p0, int32_t p1, int32_t p2, const double* X,
              const double* Y, const double* Z, double K, double* xy, double* xz, double* yz,
              msf_stream_t stream) {
  if (!D || !X || !Y || !Z || !xy || !xz || !yz) return MSF_E_INVALID;
  if (p0 < 2 || p1 < 2 || p2 < 2 || !(K > 0.0)) return MSF_E_INVALID;
  const int64_t total = (int64_t)p0 * p1 + (int64_t)p0 * p2 + (int64_t)p1 * p2;
  const int blocks = (int)((total + 255) / 256 < 152 * 8 ? (total + 255) / 256 : 152 * 8);
  k_ewald<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(D, p0, p1, p2, X, Y, Z, K,
                                                                       xy, xz, yz);
  return launch_status();
}

}  // extern "C"
