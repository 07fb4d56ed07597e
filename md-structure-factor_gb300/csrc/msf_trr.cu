// msf_trr.cu -- GROMACS .trr trajectory reader (host code, multithreaded).
//
// The reference CLI processes a .gro topology with a .trr trajectory
// (main_gromacs.py:95-101 -> load_traj.process_gro_mdtraj(top, traj, out),
// load_traj.py:91-110, through mdtraj's md.load): coordinates in nm as
// float32, times 10 to Angstrom; unitcell lengths times 10.  mdtraj and its
// xdrfile library are not part of this library; the frame layout follows
// the published .trr (XDR, big-endian) format:
//
//   int magic (1993), int string length + 1, XDR string "GMX_trn_file"
//   (uint length, bytes padded to 4), then 13 ints: ir_size, e_size,
//   box_size, vir_size, pres_size, top_size, sym_size, x_size, v_size,
//   f_size, natoms, step, nre; then t and lambda as reals; then box (9),
//   virial (9), pressure (9), x (natoms*3), v, f -- each present when its
//   size is non-zero.  A real is a float or a double: box_size / 9 or
//   x_size / (3 natoms) bytes.
//
// Arithmetic as the .gro reader's: a coordinate is the float32 nearest the
// stored value (a float, or a double rounded once), times 10 in float32; a
// box length is the float32 norm of its box vector, times 10 in float32.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "msf.h"

namespace {

constexpr int32_t kTrrMagic = 1993;

struct TrrFrame {
  size_t off;        // byte offset of the frame's data (after the header)
  int prec;          // 4 or 8
  int64_t natoms;
  int has_box, has_x;
  size_t box_off, x_off;   // offsets from `off`
  size_t end;        // byte offset of the next frame
};

uint32_t be32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

float be_float(const unsigned char* p) {
  const uint32_t u = be32(p);
  float f;
  memcpy(&f, &u, 4);
  return f;
}

double be_double(const unsigned char* p) {
  const uint64_t u = ((uint64_t)be32(p) << 32) | (uint64_t)be32(p + 4);
  double d;
  memcpy(&d, &u, 8);
  return d;
}

int load(const char* path, std::vector<unsigned char>& data) {
  FILE* f = fopen(path, "rb");
  if (!f) return MSF_E_INVALID;
  if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return MSF_E_INVALID; }
  const long n = ftell(f);
  if (n < 0) { fclose(f); return MSF_E_INVALID; }
  rewind(f);
  data.resize((size_t)n);
  const size_t got = n ? fread(data.data(), 1, (size_t)n, f) : 0;
  fclose(f);
  return got == (size_t)n ? MSF_OK : MSF_E_INVALID;
}

// header of the frame at `pos`; MSF_E_INVALID on a malformed or truncated frame
int parse_header(const std::vector<unsigned char>& d, size_t pos, TrrFrame& fr) {
  const size_t n = d.size();
  auto need = [&](size_t k) { return pos + k <= n; };
  if (!need(8)) return MSF_E_INVALID;
  if ((int32_t)be32(&d[pos]) != kTrrMagic) return MSF_E_INVALID;
  pos += 4;
  const uint32_t slen = be32(&d[pos]);   // string length + 1
  pos += 4;
  if (slen == 0 || slen > 1024 || !need(4)) return MSF_E_INVALID;
  const uint32_t xl = be32(&d[pos]);     // XDR string: length, bytes padded to 4
  pos += 4;
  if (xl > 1024) return MSF_E_INVALID;
  const size_t padded = ((size_t)xl + 3) & ~(size_t)3;
  if (!need(padded + 13 * 4)) return MSF_E_INVALID;
  pos += padded;
  int32_t h[13];
  for (int i = 0; i < 13; ++i) h[i] = (int32_t)be32(&d[pos + 4 * (size_t)i]);
  pos += 13 * 4;
  const int32_t ir = h[0], e = h[1], box = h[2], vir = h[3], pres = h[4], top = h[5], sym = h[6];
  const int32_t xs = h[7], vs = h[8], fs = h[9], natoms = h[10];
  for (int i = 0; i < 11; ++i)
    if (h[i] < 0) return MSF_E_INVALID;
  int prec = 0;
  if (box) prec = box / 9;
  else if (natoms > 0 && xs) prec = (int)(xs / (3 * (int64_t)natoms));
  else if (natoms > 0 && vs) prec = (int)(vs / (3 * (int64_t)natoms));
  else if (natoms > 0 && fs) prec = (int)(fs / (3 * (int64_t)natoms));
  else if (vir) prec = vir / 9;
  else if (pres) prec = pres / 9;
  else prec = 4;
  if (prec != 4 && prec != 8) return MSF_E_UNSUPPORTED;
  if ((box && box != 9 * prec) || (vir && vir != 9 * prec) || (pres && pres != 9 * prec)) return MSF_E_INVALID;
  const int64_t vec = 3 * (int64_t)natoms * prec;
  if ((xs && xs != vec) || (vs && vs != vec) || (fs && fs != vec)) return MSF_E_INVALID;
  if (ir || e || top || sym) return MSF_E_UNSUPPORTED;   // not written into trajectories
  if (!need(2 * (size_t)prec)) return MSF_E_INVALID;
  pos += 2 * (size_t)prec;                // t, lambda
  fr.off = pos;
  fr.prec = prec;
  fr.natoms = natoms;
  fr.has_box = box != 0;
  fr.box_off = 0;
  size_t o = (size_t)box + (size_t)vir + (size_t)pres;
  fr.has_x = xs != 0;
  fr.x_off = o;
  o += (size_t)xs + (size_t)vs + (size_t)fs;
  if (!need(o)) return MSF_E_INVALID;
  fr.end = pos + o;
  return MSF_OK;
}

int scan(const std::vector<unsigned char>& d, std::vector<TrrFrame>& frames, int64_t& n_atoms) {
  frames.clear();
  n_atoms = -1;
  size_t pos = 0;
  while (pos < d.size()) {
    TrrFrame fr;
    const int s = parse_header(d, pos, fr);
    if (s) return s;
    if (!fr.has_x) return MSF_E_UNSUPPORTED;                 // a frame without positions
    if (n_atoms >= 0 && fr.natoms != n_atoms) return MSF_E_UNSUPPORTED;
    n_atoms = fr.natoms;
    frames.push_back(fr);
    pos = fr.end;
  }
  return frames.empty() ? MSF_E_INVALID : MSF_OK;
}

void parse_frame(const std::vector<unsigned char>& d, const TrrFrame& fr, float* xyz, double* box) {
  const unsigned char* p = d.data() + fr.off;
  const int pr = fr.prec;
  auto real = [&](const unsigned char* q) -> float {
    return pr == 4 ? be_float(q) : (float)be_double(q);
  };
  const unsigned char* x = p + fr.x_off;
  for (int64_t i = 0; i < 3 * fr.natoms; ++i) xyz[i] = real(x + (size_t)i * pr) * 10.0f;
  if (fr.has_box) {
    for (int a = 0; a < 3; ++a) {
      const float v0 = real(p + (size_t)(3 * a + 0) * pr), v1 = real(p + (size_t)(3 * a + 1) * pr),
                  v2 = real(p + (size_t)(3 * a + 2) * pr);
      // each product rounded to float32 before the sums (no fused multiply-add)
      volatile float q0 = v0 * v0, q1 = v1 * v1, q2 = v2 * v2;
      const float s2 = (q0 + q1) + q2;
      box[a] = (double)(sqrtf(s2) * 10.0f);
    }
  } else {
    box[0] = box[1] = box[2] = 0.0;
  }
}

}  // namespace

extern "C" {

int msf_trr_scan(const char* path, int64_t* n_atoms, int64_t* n_frames) {
  if (!path || !n_atoms || !n_frames) return MSF_E_INVALID;
  std::vector<unsigned char> d;
  int s = load(path, d);
  if (s) return s;
  std::vector<TrrFrame> frames;
  s = scan(d, frames, *n_atoms);
  if (s) return s;
  *n_frames = (int64_t)frames.size();
  return MSF_OK;
}

int msf_trr_read(const char* path, int64_t n_atoms, int64_t n_frames, float* xyz, double* box, int32_t threads) {
  if (!path || !xyz || !box || n_atoms < 0 || n_frames < 1) return MSF_E_INVALID;
  std::vector<unsigned char> d;
  int s = load(path, d);
  if (s) return s;
  std::vector<TrrFrame> frames;
  int64_t na;
  s = scan(d, frames, na);
  if (s) return s;
  if (na != n_atoms || (int64_t)frames.size() != n_frames) return MSF_E_INVALID;
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  nt = (int)std::max<int64_t>(1, std::min<int64_t>(nt, n_frames));
  auto work = [&](int t) {
    for (int64_t f = t; f < n_frames; f += nt)
      parse_frame(d, frames[(size_t)f], xyz + f * n_atoms * 3, box + 3 * f);
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(work, t);
    for (auto& th : pool) th.join();
  }
  return MSF_OK;
}

}  // extern "C"
