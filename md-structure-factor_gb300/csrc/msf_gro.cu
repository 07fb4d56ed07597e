// msf_gro.cu -- GROMACS .gro trajectory reader (host code, multithreaded).
//
// Replaces the trajectory ingest of load_traj.py for .gro files:
// process_gro_mdtraj (load_traj.py:91-110: positions in nm from the
// trajectory reader, times 10 to Angstrom; unitcell lengths times 10) and
// load_gro (load_traj.py:11-20: atom names from columns 11-15).  mdtraj, which
// the reference uses for this, is not part of this library.
//
// Format, per frame: a title line; the atom count; one fixed-column line per
// atom -- residue number (5), residue name (5), atom name (5), atom number
// (5), then x, y, z (and optionally vx, vy, vz) in fields of equal width w
// with d decimals, where w is the distance between the first two decimal
// points from column 21 -- and the box line: v1(x) v2(y) v3(z) and, for
// triclinic boxes, v1(y) v1(z) v2(x) v2(z) v3(x) v3(y).
//
// Arithmetic follows the reference's reader: each coordinate is the float32
// nearest the decimal field, then multiplied by 10 in float32; a box length
// is the float32 norm of its box vector, times 10 in float32.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "msf.h"

namespace {

struct GroFile {
  std::vector<char> data;
  std::vector<size_t> line;   // start offset of every line
};

int worker_count(int threads, int64_t work) {
  const int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  return (int)std::max<int64_t>(1, std::min<int64_t>(nt, work));
}

template <class F>
void run_threads(int nt, F&& fn) {
  if (nt == 1) {
    fn(0);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t) pool.emplace_back(fn, t);
  for (auto& th : pool) th.join();
}

// Whole file plus the start offset of every line.  The line index is built in
// two parallel passes over equal byte ranges: count the line starts of each
// range, then write them after the prefix count of the ranges before.
int load_file(const char* path, GroFile& g, int threads) {
  FILE* f = fopen(path, "rb");
  if (!f) return MSF_E_INVALID;
  if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return MSF_E_INVALID; }
  const long n = ftell(f);
  if (n < 0) { fclose(f); return MSF_E_INVALID; }
  rewind(f);
  g.data.resize((size_t)n + 1);
  const size_t got = fread(g.data.data(), 1, (size_t)n, f);
  fclose(f);
  if (got != (size_t)n) return MSF_E_INVALID;
  g.data[(size_t)n] = '\n';
  g.line.clear();
  if (n == 0) return MSF_OK;
  const int nt = worker_count(threads, (int64_t)n / (1 << 20) + 1);
  const char* d = g.data.data();
  const size_t sz = (size_t)n;
  std::vector<size_t> cnt((size_t)nt + 1, 0);
  // line starts: offset 0 and every offset after a '\n' that is < n
  auto each_start = [&](int t, auto&& emit) {
    const size_t a = sz * (size_t)t / (size_t)nt, b = sz * (size_t)(t + 1) / (size_t)nt;
    const char* q = d + a;
    while (q < d + b) {
      q = static_cast<const char*>(memchr(q, '\n', (size_t)(d + b - q)));
      if (!q) break;
      const size_t s = (size_t)(q - d) + 1;
      if (s < sz) emit(s);
      ++q;
    }
  };
  run_threads(nt, [&](int t) {
    size_t c = 0;
    each_start(t, [&](size_t) { ++c; });
    cnt[(size_t)t + 1] = c;
  });
  for (int t = 0; t < nt; ++t) cnt[(size_t)t + 1] += cnt[(size_t)t];
  g.line.resize(cnt[(size_t)nt] + 1);
  g.line[0] = 0;
  run_threads(nt, [&](int t) {
    size_t k = cnt[(size_t)t] + 1;
    each_start(t, [&](size_t s) { g.line[k++] = s; });
  });
  return MSF_OK;
}

size_t line_len(const GroFile& g, size_t i) {
  const size_t a = g.line[i];
  size_t b = (i + 1 < g.line.size()) ? g.line[i + 1] : g.data.size() - 1;
  while (b > a && (g.data[b - 1] == '\n' || g.data[b - 1] == '\r')) --b;
  return b - a;
}

// Decimal field [p, p + w) (may hold surrounding blanks); false when empty
// or malformed.  Plain fixed-point fields ([-]ddd.ddd, at most 15 digits)
// take the exact path m / 10^d: m and 10^d (d <= 15) are exact doubles and
// IEEE division rounds their quotient correctly, the same double strtod
// returns (Clinger's fast path); anything else goes through strtod.
const double kPow10[16] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11, 1e12, 1e13, 1e14, 1e15};

bool parse_field_slow(const char* p, int w, double& out) {
  char buf[64];
  if (w <= 0 || w >= (int)sizeof(buf)) return false;
  memcpy(buf, p, (size_t)w);
  buf[w] = '\0';
  char* end = nullptr;
  out = strtod(buf, &end);
  if (end == buf) return false;
  for (char* c = end; *c; ++c)
    if (*c != ' ' && *c != '\t') return false;
  return true;
}

bool parse_field(const char* p, int w, double& out) {
  int i = 0;
  while (i < w && p[i] == ' ') ++i;
  bool neg = false;
  if (i < w && (p[i] == '-' || p[i] == '+')) neg = p[i++] == '-';
  uint64_t m = 0;
  int digits = 0, frac = 0;
  bool dot = false;
  for (; i < w; ++i) {
    const unsigned char c = (unsigned char)p[i];
    if (c >= '0' && c <= '9') {
      if (digits < 16) m = m * 10 + (c - '0');
      ++digits;
      frac += dot;
    } else if (c == '.' && !dot) {
      dot = true;
    } else {
      break;
    }
  }
  int j = i;
  while (j < w && p[j] == ' ') ++j;
  if (j < w || digits == 0 || digits > 15) return parse_field_slow(p, w, out);
  const double v = (double)m / kPow10[frac];
  out = neg ? -v : v;
  return true;
}

// the atom count of the frame starting at line l
bool frame_atoms(const GroFile& g, size_t l, int64_t& n) {
  if (l + 1 >= g.line.size()) return false;
  const char* p = g.data.data() + g.line[l + 1];
  char* end = nullptr;
  const long long v = strtoll(p, &end, 10);
  if (end == p || v < 0) return false;
  n = v;
  return true;
}

// coordinate field width from the first atom line of a frame
int field_width(const GroFile& g, size_t atom_line) {
  const char* p = g.data.data() + g.line[atom_line];
  const size_t len = line_len(g, atom_line);
  if (len < 21) return 0;
  const char* d1 = static_cast<const char*>(memchr(p + 20, '.', len - 20));
  if (!d1) return 0;
  const size_t off = (size_t)(d1 - p) + 1;
  const char* d2 = static_cast<const char*>(memchr(d1 + 1, '.', len - off));
  return d2 ? (int)(d2 - d1) : 0;
}

bool blank_from(const GroFile& g, size_t l) {
  for (size_t k = l; k < g.line.size(); ++k) {
    const char* p = g.data.data() + g.line[k];
    const size_t len = line_len(g, k);
    for (size_t c = 0; c < len; ++c)
      if (p[c] != ' ' && p[c] != '\t') return false;
  }
  return true;
}

int scan(const GroFile& g, int64_t& n_atoms, int64_t& n_frames) {
  n_atoms = -1;
  n_frames = 0;
  size_t l = 0;
  while (l < g.line.size()) {
    if (blank_from(g, l)) break;   // trailing blank lines end the file
    int64_t n;
    if (!frame_atoms(g, l, n)) return MSF_E_INVALID;
    if (n_atoms >= 0 && n != n_atoms) return MSF_E_UNSUPPORTED;  // changing atom counts
    n_atoms = n;
    if (l + 2 + (size_t)n >= g.line.size()) return MSF_E_INVALID;
    l += 3 + (size_t)n;
    ++n_frames;
  }
  if (n_frames == 0) return MSF_E_INVALID;
  return MSF_OK;
}

int parse_frame(const GroFile& g, size_t l0, int64_t n, int w, float* xyz, double* box, char* names) {
  for (int64_t i = 0; i < n; ++i) {
    const size_t li = l0 + 2 + (size_t)i;
    const char* p = g.data.data() + g.line[li];
    if (line_len(g, li) < (size_t)(20 + 3 * w)) return MSF_E_INVALID;
    for (int c = 0; c < 3; ++c) {
      double v;
      if (!parse_field(p + 20 + c * w, w, v)) return MSF_E_INVALID;
      xyz[3 * i + c] = (float)v * 10.0f;
    }
    if (names) {
      char* nm = names + 8 * i;
      memset(nm, 0, 8);
      int a = 10, b = 15;
      while (a < b && (p[a] == ' ' || p[a] == '\t')) ++a;
      while (b > a && (p[b - 1] == ' ' || p[b - 1] == '\t')) --b;
      memcpy(nm, p + a, (size_t)(b - a));
    }
  }
  // box line: 3 or 9 numbers
  const size_t lb = l0 + 2 + (size_t)n;
  const size_t len = line_len(g, lb);
  std::vector<char> buf(g.data.data() + g.line[lb], g.data.data() + g.line[lb] + len);
  buf.push_back('\0');
  double v[9];
  int k = 0;
  char* s = buf.data();
  while (k < 9) {
    char* end = nullptr;
    const double x = strtod(s, &end);
    if (end == s) break;
    v[k++] = x;
    s = end;
  }
  while (*s == ' ' || *s == '\t') ++s;
  if ((k != 3 && k != 9) || *s) return MSF_E_INVALID;
  float vec[3][3] = {{(float)v[0], 0.f, 0.f}, {0.f, (float)v[1], 0.f}, {0.f, 0.f, (float)v[2]}};
  if (k == 9) {
    vec[0][1] = (float)v[3]; vec[0][2] = (float)v[4];
    vec[1][0] = (float)v[5]; vec[1][2] = (float)v[6];
    vec[2][0] = (float)v[7]; vec[2][1] = (float)v[8];
  }
  for (int a = 0; a < 3; ++a) {
    // each product rounded to float32 before the sums (no fused multiply-add,
    // which Arm compilers would otherwise form), summed left to right
    volatile float p0 = vec[a][0] * vec[a][0], p1 = vec[a][1] * vec[a][1], p2 = vec[a][2] * vec[a][2];
    const float s2 = (p0 + p1) + p2;
    box[a] = (double)(sqrtf(s2) * 10.0f);
  }
  return MSF_OK;
}

}  // namespace

extern "C" {

int msf_gro_scan(const char* path, int64_t* n_atoms, int64_t* n_frames) {
  if (!path || !n_atoms || !n_frames) return MSF_E_INVALID;
  GroFile g;
  int s = load_file(path, g, 0);
  if (s) return s;
  return scan(g, *n_atoms, *n_frames);
}

int msf_gro_read(const char* path, int64_t n_atoms, int64_t n_frames, float* xyz, double* box, char* names,
                 int32_t threads) {
  if (!path || !xyz || !box || n_atoms < 0 || n_frames < 1) return MSF_E_INVALID;
  GroFile g;
  int s = load_file(path, g, threads);
  if (s) return s;
  int64_t na, nf;
  s = scan(g, na, nf);
  if (s) return s;
  if (na != n_atoms || nf != n_frames) return MSF_E_INVALID;
  const int w = n_atoms > 0 ? field_width(g, 2) : 8;
  if (w <= 0) return MSF_E_INVALID;
  const int nt = worker_count(threads, n_frames);
  std::vector<int> status((size_t)nt, MSF_OK);
  run_threads(nt, [&](int t) {
    for (int64_t f = t; f < n_frames; f += nt) {
      const size_t l0 = (size_t)f * (size_t)(n_atoms + 3);
      const int r = parse_frame(g, l0, n_atoms, w, xyz + f * n_atoms * 3, box + 3 * f, f == 0 ? names : nullptr);
      if (r) { status[(size_t)t] = r; return; }
    }
  });
  for (int r : status)
    if (r) return r;
  return MSF_OK;
}

}  // extern "C"
