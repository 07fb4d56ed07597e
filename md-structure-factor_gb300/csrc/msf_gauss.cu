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
  k_gauss<<<(unsigned)n_atoms, 256, 0, st>>>(a);
  return launch_status();
}
