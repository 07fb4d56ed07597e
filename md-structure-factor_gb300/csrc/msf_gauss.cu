// msf_gauss.cu -- the reference's Gaussian density (drop-in mode).
//
// dens.py:283-308: for every atom, ir = int(r/dr) and on the box
// [ir-A+B, ir+A+B) of the grid padded by B = Nborder voxels it adds
//     c1 * exp(-|ucell^T (r - g)|^2 / c2),  c1 = Nel/sigma^3, c2 = 2 sigma^2,
// with g = (i - B)*dr the padded grid coordinate.  dens.py:311 then folds the
// padding onto the periodic cell (remap_grid_tcl, dens.py:86-108).  Here each
// padded voxel is mapped straight to its folded destination and added with an
// FP64 atomic, so the padded grid never exists.  The fold map is the
// reference's: faces and edges go to their periodic images; a voxel in all
// three pads (a corner block) takes its z destination from the y side --
// start N2-B when the y source is the low pad, 0 when it is the high pad --
// plus its offset inside its own z pad (dens.py:107 indexes des[2][id2]).
#include "msf_internal.cuh"

namespace msf {

struct GaussArgs {
  const double* pos;
  const int32_t* tidx;
  int64_t n_atoms;
  const double* tab;   // (n_types, 5): c1, c2, Ax, Ay, Az
  int n_types;
  double dr[3];
  double u[9];         // ucell row major: u[m*3 + l]
  int B;
  int n[3];
  double* grid;
  int* status;
};

__device__ __forceinline__ int fold_region(int P, int B, int n) {
  return P < B ? 0 : (P < B + n ? 1 : 2);
}
__device__ __forceinline__ int fold_dest(int P, int r, int B, int n) {
  return r == 0 ? n - B + P : (r == 1 ? P - B : P - B - n);
}

__global__ void __launch_bounds__(256) k_gauss(GaussArgs a) {
  const int64_t im = blockIdx.x;
  if (im >= a.n_atoms) return;
  const int t = __ldg(a.tidx + im);
  if (t < 0 || t >= a.n_types) {
    if (threadIdx.x == 0) {
      atomicExch(a.status + kStatErr, MSF_E_TYPE);
      atomicAdd(a.status + kStatBadIndex, 1);
    }
    return;
  }
  const double c1 = __ldg(a.tab + 5 * t + 0);
  const double c2 = __ldg(a.tab + 5 * t + 1);
  const int A[3] = {(int)__ldg(a.tab + 5 * t + 2), (int)__ldg(a.tab + 5 * t + 3),
                    (int)__ldg(a.tab + 5 * t + 4)};
  double r[3];
  int lo[3];
  bool ok = true;
  for (int d = 0; d < 3; ++d) {
    r[d] = __ldg(a.pos + 3 * im + d);
    const double q = __ddiv_rn(r[d], a.dr[d]);
    const int ir = (q > -2147483648.0 && q < 2147483647.0) ? (int)q : -(1 << 30);
    lo[d] = ir - A[d] + a.B;
    ok = ok && lo[d] >= 0 && ir + A[d] + a.B <= a.n[d] + 2 * a.B;
  }
  if (!ok) {
    if (threadIdx.x == 0) {
      atomicExch(a.status + kStatErr, MSF_E_RANGE);
      atomicAdd(a.status + kStatBadAtom, 1);
    }
    return;
  }
  const int ex = 2 * A[0], ey = 2 * A[1], ez = 2 * A[2];
  const int total = ex * ey * ez;
  const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2], B = a.B;
  for (int v = threadIdx.x; v < total; v += blockDim.x) {
    const int iz = v % ez;
    const int rest = v / ez;
    const int iy = rest % ey;
    const int ix = rest / ey;
    const int P0 = lo[0] + ix, P1 = lo[1] + iy, P2 = lo[2] + iz;
    // buf = r - g (dens.py:299); g = (P - B) * dr (dens.py:251-256)
    const double b0 = __dsub_rn(r[0], __dmul_rn((double)(P0 - B), a.dr[0]));
    const double b1 = __dsub_rn(r[1], __dmul_rn((double)(P1 - B), a.dr[1]));
    const double b2 = __dsub_rn(r[2], __dmul_rn((double)(P2 - B), a.dr[2]));
    // buf2_l = sum_m ucell[m][l] buf_m (dens.py:301); distSQ (dens.py:303)
    double d2 = 0.0;
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      const double s = __dadd_rn(__dadd_rn(__dmul_rn(a.u[l], b0), __dmul_rn(a.u[3 + l], b1)),
                                 __dmul_rn(a.u[6 + l], b2));
      d2 = __dadd_rn(d2, __dmul_rn(s, s));
    }
    const double val = __dmul_rn(c1, exp(-__ddiv_rn(d2, c2)));
    const int r0 = fold_region(P0, B, n0), r1 = fold_region(P1, B, n1), r2 = fold_region(P2, B, n2);
    const int D0 = fold_dest(P0, r0, B, n0);
    const int D1 = fold_dest(P1, r1, B, n1);
    int D2;
    if (r0 != 1 && r1 != 1 && r2 != 1) {
      const int off = (r2 == 0) ? P2 : P2 - B - n2;
      D2 = (r1 == 0 ? n2 - B : 0) + off;
    } else {
      D2 = fold_dest(P2, r2, B, n2);
    }
    atomicAdd(a.grid + ((int64_t)D0 * n1 + D1) * n2 + D2, val);
  }
}

// Separable form of the same density.  With b = r - g and M = U U^T
// (U = ucell), |U^T b|^2 = sum_ab M_ab b_a b_b, so
//   exp(-|U^T b|^2 / c2) = prod_a exp(-M_aa b_a^2 / c2) * prod_{a<b} exp(-2 M_ab b_a b_b / c2).
// Per atom, the 1-D factors (2A values per axis) and, where M_ab != 0, the
// 2-D cross factors ((2A_a x 2A_b) values) go to shared memory once; each
// voxel of the (2A)^3 box then costs a few FP64 multiplies instead of an
// exp.  Equal to the direct form up to rounding (~1e-15 relative).
constexpr int kSepMax = 64;   // largest footprint per axis (2A) handled here

__global__ void __launch_bounds__(256) k_gauss_sep(GaussArgs a, int cross_xy, int cross_xz, int cross_yz) {
  extern __shared__ double tabs[];
  const int64_t im = blockIdx.x;
  if (im >= a.n_atoms) return;
  const int t = __ldg(a.tidx + im);
  if (t < 0 || t >= a.n_types) {
    if (threadIdx.x == 0) {
      atomicExch(a.status + kStatErr, MSF_E_TYPE);
      atomicAdd(a.status + kStatBadIndex, 1);
    }
    return;
  }
  const double c1 = __ldg(a.tab + 5 * t + 0);
  const double c2 = __ldg(a.tab + 5 * t + 1);
  const int A[3] = {(int)__ldg(a.tab + 5 * t + 2), (int)__ldg(a.tab + 5 * t + 3),
                    (int)__ldg(a.tab + 5 * t + 4)};
  double r[3];
  int lo[3];
  bool ok = true;
  for (int d = 0; d < 3; ++d) {
    r[d] = __ldg(a.pos + 3 * im + d);
    const double q = __ddiv_rn(r[d], a.dr[d]);
    const int ir = (q > -2147483648.0 && q < 2147483647.0) ? (int)q : -(1 << 30);
    lo[d] = ir - A[d] + a.B;
    ok = ok && lo[d] >= 0 && ir + A[d] + a.B <= a.n[d] + 2 * a.B;
  }
  if (!ok) {
    if (threadIdx.x == 0) {
      atomicExch(a.status + kStatErr, MSF_E_RANGE);
      atomicAdd(a.status + kStatBadAtom, 1);
    }
    return;
  }
  const int ex = 2 * A[0], ey = 2 * A[1], ez = 2 * A[2];
  // M = U U^T
  double M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      M[i][j] = a.u[3 * i + 0] * a.u[3 * j + 0] + a.u[3 * i + 1] * a.u[3 * j + 1] + a.u[3 * i + 2] * a.u[3 * j + 2];
  double* bx = tabs;              // b_x(i) for the 2A x positions
  double* by = bx + ex;
  double* bz = by + ey;
  double* fx = bz + ez;           // exp(-M00 b_x^2 / c2)
  double* fy = fx + ex;
  double* fz = fy + ey;
  double* fxy = fz + ez;          // exp(-2 M01 b_x b_y / c2), ex * ey
  double* fxz = fxy + (cross_xy ? ex * ey : 0);
  double* fyz = fxz + (cross_xz ? ex * ez : 0);
  const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2], B = a.B;
  for (int i = threadIdx.x; i < ex + ey + ez; i += blockDim.x) {
    const int d = i < ex ? 0 : (i < ex + ey ? 1 : 2);
    const int k = i - (d == 0 ? 0 : (d == 1 ? ex : ex + ey));
    const double b = __dsub_rn(r[d], __dmul_rn((double)(lo[d] + k - B), a.dr[d]));
    bx[i] = b;
    fx[i] = exp(-__ddiv_rn(__dmul_rn(M[d][d], __dmul_rn(b, b)), c2));
  }
  __syncthreads();
  if (cross_xy)
    for (int i = threadIdx.x; i < ex * ey; i += blockDim.x)
      fxy[i] = exp(-__ddiv_rn(2.0 * M[0][1] * bx[i / ey] * by[i % ey], c2));
  if (cross_xz)
    for (int i = threadIdx.x; i < ex * ez; i += blockDim.x)
      fxz[i] = exp(-__ddiv_rn(2.0 * M[0][2] * bx[i / ez] * bz[i % ez], c2));
  if (cross_yz)
    for (int i = threadIdx.x; i < ey * ez; i += blockDim.x)
      fyz[i] = exp(-__ddiv_rn(2.0 * M[1][2] * by[i / ez] * bz[i % ez], c2));
  __syncthreads();
  const int total = ex * ey * ez;
  for (int v = threadIdx.x; v < total; v += blockDim.x) {
    const int iz = v % ez;
    const int rest = v / ez;
    const int iy = rest % ey;
    const int ix = rest / ey;
    double val = c1 * fx[ix] * fy[iy] * fz[iz];
    if (cross_xy) val *= fxy[ix * ey + iy];
    if (cross_xz) val *= fxz[ix * ez + iz];
    if (cross_yz) val *= fyz[iy * ez + iz];
    const int P0 = lo[0] + ix, P1 = lo[1] + iy, P2 = lo[2] + iz;
    const int r0 = fold_region(P0, B, n0), r1 = fold_region(P1, B, n1), r2 = fold_region(P2, B, n2);
    const int D0 = fold_dest(P0, r0, B, n0);
    const int D1 = fold_dest(P1, r1, B, n1);
    int D2;
    if (r0 != 1 && r1 != 1 && r2 != 1) {
      const int off = (r2 == 0) ? P2 : P2 - B - n2;
      D2 = (r1 == 0 ? n2 - B : 0) + off;
    } else {
      D2 = fold_dest(P2, r2, B, n2);
    }
    atomicAdd(a.grid + ((int64_t)D0 * n1 + D1) * n2 + D2, val);
  }
}

}  // namespace msf

using namespace msf;

extern "C" int msf_gauss_grid_f64(const msf_plan* p, const double* pos, const int32_t* type_index,
                                  int64_t n_atoms, const double* type_tab, int32_t n_types,
                                  const double* geom, double* grid, msf_stream_t stream) {
  if (!p || !grid || !geom || n_atoms < 0 || n_types < 1) return MSF_E_INVALID;
  if (n_atoms > 0 && (!pos || !type_index || !type_tab)) return MSF_E_INVALID;
  if (!p->bound) return MSF_E_NOT_BOUND;
  if (n_atoms > 0x7fffffffLL) return MSF_E_UNSUPPORTED;
  GaussArgs a;
  a.pos = pos;
  a.tidx = type_index;
  a.n_atoms = n_atoms;
  a.tab = type_tab;
  a.n_types = n_types;
  for (int i = 0; i < 3; ++i) a.dr[i] = geom[i];
  for (int i = 0; i < 9; ++i) a.u[i] = geom[3 + i];
  a.B = (int)geom[12];
  a.n[0] = p->n0; a.n[1] = p->n1; a.n[2] = p->n2;
  if (a.B < 0 || a.B > p->n0 || a.B > p->n1 || a.B > p->n2) return MSF_E_UNSUPPORTED;
  for (int i = 0; i < 3; ++i)
    if (!(a.dr[i] > 0.0)) return MSF_E_INVALID;
  a.grid = grid;
  a.status = ws_ptr<int>(p, p->off_status);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int s = cuda_status(cudaMemsetAsync(grid, 0, (size_t)grid_elems(p) * sizeof(double), st));
  if (s) return s;
  if (n_atoms == 0) return MSF_OK;
  // geom[13]: the largest footprint 2A over the types (0 = unknown)
  const int fmax = (int)geom[13];
  if (fmax < 1 || fmax > kSepMax) {
    k_gauss<<<(unsigned)n_atoms, 256, 0, st>>>(a);
    return launch_status();
  }
  double M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      M[i][j] = a.u[3 * i] * a.u[3 * j] + a.u[3 * i + 1] * a.u[3 * j + 1] + a.u[3 * i + 2] * a.u[3 * j + 2];
  const int cxy = M[0][1] != 0.0, cxz = M[0][2] != 0.0, cyz = M[1][2] != 0.0;
  const size_t smem = (size_t)(6 * fmax + (cxy + cxz + cyz) * fmax * fmax) * sizeof(double);
  static bool once = false;
  if (!once) {
    cudaFuncSetAttribute(k_gauss_sep, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    once = true;
  }
  k_gauss_sep<<<(unsigned)n_atoms, 256, smem, st>>>(a, cxy, cxz, cyz);
  return launch_status();
}
