// Host-side clustering of tagged blocks into patch boxes (regridding).
//
// The reference hands this to SAMRAI's BergerRigoutsos box generator
// (main.C:261-265, input.txt:123-127).  This is the published signature
// algorithm of Berger & Rigoutsos (IEEE Trans. SMC 21(5), 1991) with the
// cut rules and tie-breaks of enlightning_gb300/cluster.py, which stays the
// readable specification; tests compare the two box for box.  Summed-area
// tables of the tags and of the disallowed cells make every box sum, row or
// column test O(1), so a regrid of a 2048 x 1024 block map costs
// milliseconds instead of the tens of milliseconds of the array version.
// Host code only; no device memory is touched.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "enlightning_gpu.h"

namespace {

// Summed-area table of a window (x0, y0, nx, ny) of a row-major byte map
// with row pitch `pitch`: s[j*(nx+1) + i] = count over window rows < j and
// columns < i of cells that are set (or clear, with invert).  Coordinates
// passed to sum() are window coordinates.
struct Sat {
  int nx = 0, ny = 0;
  std::vector<int32_t> s;
  void build(const unsigned char* m, size_t pitch, int x0, int y0, int nx_, int ny_, bool invert) {
    nx = nx_;
    ny = ny_;
    s.resize((size_t)(nx + 1) * (ny + 1));
    std::fill(s.begin(), s.begin() + (nx + 1), 0);
    for (int j = 0; j < ny; ++j) {
      const unsigned char* r = m + (size_t)(y0 + j) * pitch + x0;
      int32_t* prev = s.data() + (size_t)j * (nx + 1);
      int32_t* cur = prev + (nx + 1);
      int32_t row = 0;
      cur[0] = 0;
      if (invert)
        for (int i = 0; i < nx; ++i) cur[i + 1] = prev[i + 1] + (row += (r[i] == 0));
      else
        for (int i = 0; i < nx; ++i) cur[i + 1] = prev[i + 1] + (row += (r[i] != 0));
    }
  }
  // sum over cols [i0, i1], rows [j0, j1] (inclusive)
  int64_t sum(int i0, int i1, int j0, int j1) const {
    const size_t w = (size_t)nx + 1;
    return (int64_t)s[(size_t)(j1 + 1) * w + (i1 + 1)] - s[(size_t)j0 * w + (i1 + 1)] -
           s[(size_t)(j1 + 1) * w + i0] + s[(size_t)j0 * w + i0];
  }
};

struct Box {
  int ilo, ihi, jlo, jhi;
};

// Bounding box of the tags inside b; false when there are none.
bool shrink(const Sat& T, Box& b) {
  if (T.sum(b.ilo, b.ihi, b.jlo, b.jhi) == 0) return false;
  while (T.sum(b.ilo, b.ihi, b.jlo, b.jlo) == 0) ++b.jlo;
  while (T.sum(b.ilo, b.ihi, b.jhi, b.jhi) == 0) --b.jhi;
  while (T.sum(b.ilo, b.ilo, b.jlo, b.jhi) == 0) ++b.ilo;
  while (T.sum(b.ihi, b.ihi, b.jlo, b.jhi) == 0) --b.ihi;
  return true;
}

int sgn(int64_t v) { return (v > 0) - (v < 0); }

// Cut position c (the box splits into [0, c) and [c, n)), or -1: a zero of
// the signature nearest the middle, else the strongest inflection, else the
// middle (cluster.py _cut).
int cut_signature(const std::vector<int64_t>& sig, int min_size) {
  const int n = (int)sig.size();
  const int lo = min_size, hi = n - min_size;
  if (hi < lo) return -1;
  const double mid = (n - 1) / 2.0;
  int best = -1;
  double bestd = 0.0;
  for (int q = lo; q <= hi && q < n; ++q) {
    if (sig[q] != 0) continue;
    const double d = std::fabs((double)q - mid);
    if (best < 0 || d < bestd) {
      best = q;
      bestd = d;
    }
  }
  if (best >= 0) return best < lo ? lo : (best > hi ? hi : best);
  if (n >= 4) {
    std::vector<int64_t> lap(n - 2);
    for (int q = 0; q < n - 2; ++q) lap[q] = sig[q] - 2 * sig[q + 1] + sig[q + 2];
    int64_t bj = -1;
    int bc = -1;
    for (int q = 0; q < n - 3; ++q) {
      const int cand = q + 2;
      const bool ok = cand >= lo && cand <= hi && sgn(lap[q]) != sgn(lap[q + 1]);
      const int64_t jv = ok ? std::llabs(lap[q + 1] - lap[q]) : -1;
      if (jv > bj) {
        bj = jv;
        bc = cand;
      }
    }
    if (bj > 0) return bc;
  }
  return (n / 2 >= lo && n / 2 <= hi) ? n / 2 : -1;
}

// Cut separating columns (rows) that hold disallowed cells from those that
// do not, longer side first (cluster.py _nesting_cut); axis 0 = x, 1 = y.
bool nesting_cut(const Sat& B, const Box& b, int& axis, int& c) {
  const int nx = b.ihi - b.ilo + 1, ny = b.jhi - b.jlo + 1;
  const int order[2] = {ny > nx ? 1 : 0, ny > nx ? 0 : 1};  // stable: x first on ties
  for (int o = 0; o < 2; ++o) {
    const int ax = order[o];
    const int n = ax == 0 ? nx : ny;
    if (n < 2) continue;
    auto bad = [&](int q) {
      return ax == 0 ? B.sum(b.ilo + q, b.ilo + q, b.jlo, b.jhi) > 0 : B.sum(b.ilo, b.ihi, b.jlo + q, b.jlo + q) > 0;
    };
    int best = -1;
    double bestd = 0.0;
    bool prev = bad(0);
    for (int q = 1; q < n; ++q) {
      const bool cur = bad(q);
      if (cur != prev) {
        const double d = std::fabs((double)q - n / 2.0);
        if (best < 0 || d < bestd) {
          best = q;
          bestd = d;
        }
      }
      prev = cur;
    }
    if (best >= 0) {
      axis = ax;
      c = best;
      return true;
    }
  }
  if (nx >= ny && nx >= 2) {
    axis = 0;
    c = nx / 2;
    return true;
  }
  if (ny >= 2) {
    axis = 1;
    c = ny / 2;
    return true;
  }
  return false;
}

void push_halves(std::vector<Box>& st, const Box& b, int axis, int c) {
  if (axis == 0) {
    st.push_back({b.ilo, b.ilo + c - 1, b.jlo, b.jhi});
    st.push_back({b.ilo + c, b.ihi, b.jlo, b.jhi});
  } else {
    st.push_back({b.ilo, b.ihi, b.jlo, b.jlo + c - 1});
    st.push_back({b.ilo, b.ihi, b.jlo + c, b.jhi});
  }
}

// Split points of [lo, hi + 1) into k nearly equal parts, rounded half to
// even like numpy's linspace(...).round().
std::vector<int> split_points(int lo, int hi, int k) {
  std::vector<int> p(k + 1);
  const double step = (double)(hi + 1 - lo) / (double)k;
  for (int q = 0; q < k; ++q) p[q] = (int)std::nearbyint((double)q * step + (double)lo);
  p[k] = hi + 1;
  return p;
}

// `passes` binary erosions by the 3x3 square, cells outside the map counting
// as set (scipy.ndimage.binary_erosion with border_value=1); separable: a
// row minimum, then a column minimum.
void erode3x3(std::vector<unsigned char>& a, int nx, int ny, int passes) {
  // values are 0/1; bitwise and keeps the loops branch-free
  std::vector<unsigned char> r((size_t)nx * ny);
  for (int it = 0; it < passes; ++it) {
    for (int j = 0; j < ny; ++j) {
      const unsigned char* src = a.data() + (size_t)j * nx;
      unsigned char* dst = r.data() + (size_t)j * nx;
      if (nx == 1) {
        dst[0] = src[0];
        continue;
      }
      dst[0] = src[0] & src[1];
      int i = 1;
      for (; i + 8 <= nx - 1; i += 8) {  // eight cells per 64-bit word
        uint64_t l, c, r;
        std::memcpy(&l, src + i - 1, 8);
        std::memcpy(&c, src + i, 8);
        std::memcpy(&r, src + i + 1, 8);
        const uint64_t v = l & c & r;
        std::memcpy(dst + i, &v, 8);
      }
      for (; i < nx - 1; ++i) dst[i] = src[i - 1] & src[i] & src[i + 1];
      dst[nx - 1] = src[nx - 2] & src[nx - 1];
    }
    for (int j = 0; j < ny; ++j) {
      const unsigned char* mid = r.data() + (size_t)j * nx;
      const unsigned char* up = j > 0 ? mid - nx : mid;
      const unsigned char* dn = j < ny - 1 ? mid + nx : mid;
      unsigned char* dst = a.data() + (size_t)j * nx;
      int i = 0;
      for (; i + 8 <= nx; i += 8) {
        uint64_t u, m, d;
        std::memcpy(&u, up + i, 8);
        std::memcpy(&m, mid + i, 8);
        std::memcpy(&d, dn + i, 8);
        const uint64_t v = u & m & d;
        std::memcpy(dst + i, &v, 8);
      }
      for (; i < nx; ++i) dst[i] = up[i] & mid[i] & dn[i];
    }
  }
}

}  // namespace

extern "C" int enl_cluster_tags(const unsigned char* tags, const unsigned char* allowed_in, int nx, int ny,
                                int nest_erode, double efficiency, int min_size, int max_size, int* boxes,
                                int max_boxes, int* nboxes) {
  if (!tags || nx < 1 || ny < 1 || nest_erode < 0 || min_size < 1 || max_size < 1 || !nboxes || max_boxes < 0 ||
      (max_boxes > 0 && !boxes)) {
    return ENL_ERR_ARG;
  }
  std::vector<unsigned char> eroded;
  const unsigned char* allowed = allowed_in;
  if (allowed_in && nest_erode > 0) {
    eroded.resize((size_t)nx * ny);
    for (size_t q = 0; q < eroded.size(); ++q) eroded[q] = (unsigned char)(allowed_in[q] != 0);
    erode3x3(eroded, nx, ny, nest_erode);
    allowed = eroded.data();
  }
  // tags outside the allowed region are dropped first; everything after
  // works inside the bounding box of what is left (window coordinates)
  std::vector<unsigned char> t((size_t)nx * ny);
  int bx0 = nx, bx1 = -1, by0 = ny, by1 = -1;
  for (int j = 0; j < ny; ++j) {
    const size_t o = (size_t)j * nx;
    unsigned char* tr = t.data() + o;
    unsigned char any = 0;
    if (allowed)
      for (int i = 0; i < nx; ++i) any |= tr[i] = (unsigned char)((tags[o + i] != 0) & (allowed[o + i] != 0));
    else
      for (int i = 0; i < nx; ++i) any |= tr[i] = (unsigned char)(tags[o + i] != 0);
    if (!any) continue;
    by0 = std::min(by0, j);
    by1 = j;
    int a = 0, b = nx - 1;
    while (!tr[a]) ++a;
    while (!tr[b]) --b;
    bx0 = std::min(bx0, a);
    bx1 = std::max(bx1, b);
  }
  if (bx1 < 0) {
    *nboxes = 0;
    return ENL_OK;
  }
  const int wx = bx1 - bx0 + 1, wy = by1 - by0 + 1;
  Sat T, B;
  T.build(t.data(), (size_t)nx, bx0, by0, wx, wy, false);
  if (allowed) B.build(allowed, (size_t)nx, bx0, by0, wx, wy, true);
  std::vector<Box> out, st;
  st.push_back(Box{0, wx - 1, 0, wy - 1});
  std::vector<int64_t> sig;
  while (!st.empty()) {
    Box b = st.back();
    st.pop_back();
    if (!shrink(T, b)) continue;
    const int nxb = b.ihi - b.ilo + 1, nyb = b.jhi - b.jlo + 1;
    if (allowed && B.sum(b.ilo, b.ihi, b.jlo, b.jhi) > 0) {
      int ax, c;
      if (nesting_cut(B, b, ax, c)) push_halves(st, b, ax, c);
      continue;
    }
    const double eff = (double)T.sum(b.ilo, b.ihi, b.jlo, b.jhi) / (double)((double)nxb * nyb);
    if (eff >= efficiency) {
      out.push_back(b);
      continue;
    }
    // longer side first; on equal sides y first (cluster.py sorts (n, axis) descending)
    const int order[2] = {nxb > nyb ? 0 : 1, nxb > nyb ? 1 : 0};
    bool done = false;
    for (int o = 0; o < 2 && !done; ++o) {
      const int ax = order[o];
      const int n = ax == 0 ? nxb : nyb;
      sig.resize(n);
      for (int q = 0; q < n; ++q)
        sig[q] = ax == 0 ? T.sum(b.ilo + q, b.ilo + q, b.jlo, b.jhi) : T.sum(b.ilo, b.ihi, b.jlo + q, b.jlo + q);
      const int c = cut_signature(sig, min_size);
      if (c <= 0 || c >= n) continue;
      push_halves(st, b, ax, c);
      done = true;
    }
    if (!done) out.push_back(b);
  }
  // chop: no side longer than max_size
  int n = 0;
  for (const Box& b : out) {
    const int bw = b.ihi - b.ilo + 1, bh = b.jhi - b.jlo + 1;
    const int kx = (bw + max_size - 1) / max_size, ky = (bh + max_size - 1) / max_size;
    const std::vector<int> xs = split_points(b.ilo, b.ihi, kx), ys = split_points(b.jlo, b.jhi, ky);
    for (int a = 0; a < kx; ++a)
      for (int c = 0; c < ky; ++c) {
        if (n < max_boxes) {  // back to map coordinates
          boxes[4 * n + 0] = bx0 + xs[a];
          boxes[4 * n + 1] = bx0 + xs[a + 1] - 1;
          boxes[4 * n + 2] = by0 + ys[c];
          boxes[4 * n + 3] = by0 + ys[c + 1] - 1;
        }
        ++n;
      }
  }
  *nboxes = n;
  return n <= max_boxes ? ENL_OK : ENL_ERR_ARG;
}
