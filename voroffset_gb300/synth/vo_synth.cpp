// Seeded synthetic inputs for the dexel morphology path (host C++).
//
// Volumes: unions of spheres and flat-capped cylinders, evaluated per column
// at the dexel centre (i + 0.5, j + 0.5) in FP64, clipped to [0, zmax] and
// merged per column with the same closed-interval rule as the reference's
// appendSegment (src/vor3d/MorphologyOperators.cpp:15-34: touching merges).
// Meshes: a watertight torus with per-vertex normal noise.
//
// The random stream is splitmix64 so every input is reproducible from its seed
// on any machine (x86 build container and the aarch64 GPU host alike).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "voroffset_synth.h"

namespace {

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [0, 1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal() {
    // Box-Muller; u1 in (0, 1]
    double u1 = 1.0 - uniform();
    double u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

struct Hit {
  int32_t col;
  double lo, hi;
};

struct Sphere {
  double cx, cy, cz, r;
};

struct Cylinder {
  double a[3], b[3], r;
};

void sphere_hits(const Sphere &s, int nx, int ny, double zmax, std::vector<Hit> &out) {
  int j0 = std::max(0, (int)std::floor(s.cy - s.r - 0.5));
  int j1 = std::min(ny - 1, (int)std::ceil(s.cy + s.r - 0.5));
  int i0 = std::max(0, (int)std::floor(s.cx - s.r - 0.5));
  int i1 = std::min(nx - 1, (int)std::ceil(s.cx + s.r - 0.5));
  const double r2 = s.r * s.r;
  for (int j = j0; j <= j1; ++j) {
    const double dy = (j + 0.5) - s.cy;
    if (dy * dy >= r2) continue;
    for (int i = i0; i <= i1; ++i) {
      const double dx = (i + 0.5) - s.cx;
      const double d2 = dx * dx + dy * dy;
      if (d2 >= r2) continue;
      const double h = std::sqrt(r2 - d2);
      double lo = s.cz - h, hi = s.cz + h;
      if (lo < 0) lo = 0;
      if (hi > zmax) hi = zmax;
      if (lo < hi) out.push_back({(int32_t)(i + nx * j), lo, hi});
    }
  }
}

// Vertical line (px, py, t) against the flat-capped cylinder a-b of radius r.
bool cylinder_column(const Cylinder &c, double px, double py, double &tlo, double &thi) {
  double u[3] = {c.b[0] - c.a[0], c.b[1] - c.a[1], c.b[2] - c.a[2]};
  const double L = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  if (!(L > 0)) return false;
  for (double &x : u) x /= L;
  const double w0[3] = {px - c.a[0], py - c.a[1], -c.a[2]};
  const double wu = w0[0] * u[0] + w0[1] * u[1] + w0[2] * u[2];
  const double ww = w0[0] * w0[0] + w0[1] * w0[1] + w0[2] * w0[2];
  // radial^2(t) = A t^2 + 2 B t + C
  const double A = 1.0 - u[2] * u[2];
  const double B = w0[2] - wu * u[2];
  const double C = ww - wu * wu;
  double lo, hi;
  if (A < 1e-12) {
    if (C > c.r * c.r) return false;
    lo = -INFINITY;
    hi = INFINITY;
  } else {
    const double disc = B * B - A * (C - c.r * c.r);
    if (disc <= 0) return false;
    const double sq = std::sqrt(disc);
    lo = (-B - sq) / A;
    hi = (-B + sq) / A;
  }
  // axial coordinate s(t) = wu + t*u2 must lie in [0, L]
  if (std::fabs(u[2]) < 1e-15) {
    if (wu < 0 || wu > L) return false;
  } else {
    double s0 = (0 - wu) / u[2], s1 = (L - wu) / u[2];
    if (s0 > s1) std::swap(s0, s1);
    lo = std::max(lo, s0);
    hi = std::min(hi, s1);
  }
  if (!(lo < hi)) return false;
  tlo = lo;
  thi = hi;
  return true;
}

void cylinder_hits(const Cylinder &c, int nx, int ny, double zmax, std::vector<Hit> &out) {
  const double ax = c.a[0], ay = c.a[1], dx = c.b[0] - c.a[0], dy = c.b[1] - c.a[1];
  const double ymin = std::min(c.a[1], c.b[1]) - c.r, ymax = std::max(c.a[1], c.b[1]) + c.r;
  int j0 = std::max(0, (int)std::floor(ymin - 0.5));
  int j1 = std::min(ny - 1, (int)std::ceil(ymax - 0.5));
  for (int j = j0; j <= j1; ++j) {
    const double py = j + 0.5;
    // parameter range of the projected axis within r of this row
    double t0 = 0, t1 = 1;
    if (std::fabs(dy) > 1e-12) {
      double ta = (py - c.r - ay) / dy, tb = (py + c.r - ay) / dy;
      if (ta > tb) std::swap(ta, tb);
      t0 = std::max(0.0, ta);
      t1 = std::min(1.0, tb);
      if (t0 > t1) continue;
    } else if (std::fabs(py - ay) > c.r) {
      continue;
    }
    double xa = ax + t0 * dx, xb = ax + t1 * dx;
    if (xa > xb) std::swap(xa, xb);
    int i0 = std::max(0, (int)std::floor(xa - c.r - 0.5));
    int i1 = std::min(nx - 1, (int)std::ceil(xb + c.r - 0.5));
    for (int i = i0; i <= i1; ++i) {
      double lo, hi;
      if (!cylinder_column(c, i + 0.5, py, lo, hi)) continue;
      if (lo < 0) lo = 0;
      if (hi > zmax) hi = zmax;
      if (lo < hi) out.push_back({(int32_t)(i + nx * j), lo, hi});
    }
  }
}

template <typename F>
void parallel_chunks(int n, int nthreads, F f) {
  if (nthreads <= 1 || n < 2) {
    f(0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  const int per = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    int b = t * per, e = std::min(n, b + per);
    if (b >= e) break;
    th.emplace_back(f, b, e, t);
  }
  for (auto &x : th) x.join();
}

int host_threads() {
  int n = (int)std::thread::hardware_concurrency();
  return n > 0 ? std::min(n, 64) : 1;
}

}  // namespace

extern "C" int vo_synth_volume(const vo_synth_params *p, int32_t *offs, double **z_out,
                               int64_t *nseg_out) {
  if (!p || !offs || !z_out || p->nx <= 0 || p->ny <= 0 || !(p->zmax > 0)) return VO_EINVAL;
  const int nx = p->nx, ny = p->ny;
  const int64_t ncols = (int64_t)nx * ny;
  SplitMix64 rng(p->seed);
  std::vector<Sphere> spheres((size_t)std::max(0, p->n_spheres));
  for (auto &s : spheres) {
    s.cx = rng.uniform(0, nx);
    s.cy = rng.uniform(0, ny);
    s.cz = rng.uniform(0, p->zmax);
    double r;
    if (p->sphere_dist == 1) {
      r = p->s_median * std::exp(p->s_sigma * rng.normal());
    } else {
      r = rng.uniform(p->s_rmin, p->s_rmax);
    }
    s.r = std::min(std::max(r, p->s_rmin), p->s_rmax);
  }
  std::vector<Cylinder> cyls((size_t)std::max(0, p->n_cyl));
  for (auto &c : cyls) {
    c.a[0] = rng.uniform(0, nx);
    c.a[1] = rng.uniform(0, ny);
    c.a[2] = rng.uniform(0, p->zmax);
    c.b[0] = rng.uniform(0, nx);
    c.b[1] = rng.uniform(0, ny);
    c.b[2] = rng.uniform(0, p->zmax);
    c.r = rng.uniform(p->c_rmin, p->c_rmax);
  }
  const int T = host_threads();
  const int nobj = (int)(spheres.size() + cyls.size());
  std::vector<std::vector<Hit>> hits((size_t)T);
  parallel_chunks(nobj, T, [&](int b, int e, int t) {
    for (int o = b; o < e; ++o) {
      if (o < (int)spheres.size())
        sphere_hits(spheres[o], nx, ny, p->zmax, hits[t]);
      else
        cylinder_hits(cyls[o - spheres.size()], nx, ny, p->zmax, hits[t]);
    }
  });
  // counting sort by column
  std::vector<int64_t> start((size_t)ncols + 1, 0);
  for (auto &hv : hits)
    for (const Hit &h : hv) start[(size_t)h.col + 1]++;
  for (int64_t c = 0; c < ncols; ++c) start[c + 1] += start[c];
  const int64_t nh = start[ncols];
  std::vector<double> lo((size_t)std::max<int64_t>(nh, 1)), hi((size_t)std::max<int64_t>(nh, 1));
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (auto &hv : hits) {
      for (const Hit &h : hv) {
        int64_t k = fill[h.col]++;
        lo[k] = h.lo;
        hi[k] = h.hi;
      }
      std::vector<Hit>().swap(hv);
    }
  }
  // per column: sort by lo, merge closed intervals (touching merges)
  std::vector<int32_t> cnt((size_t)ncols, 0);
  parallel_chunks((int)std::min<int64_t>(ncols, 1 << 30), T, [&](int b, int e, int) {
    std::vector<std::pair<double, double>> tmp;
    for (int c = b; c < e; ++c) {
      int64_t s0 = start[c], s1 = start[c + 1];
      tmp.clear();
      for (int64_t k = s0; k < s1; ++k) tmp.emplace_back(lo[k], hi[k]);
      std::sort(tmp.begin(), tmp.end());
      int64_t w = s0;
      for (auto &iv : tmp) {
        if (w > s0 && !(hi[w - 1] < iv.first)) {
          if (iv.second > hi[w - 1]) hi[w - 1] = iv.second;
        } else {
          lo[w] = iv.first;
          hi[w] = iv.second;
          ++w;
        }
      }
      cnt[c] = (int32_t)(w - s0);
    }
  });
  int64_t total = 0;
  offs[0] = 0;
  for (int64_t c = 0; c < ncols; ++c) {
    total += cnt[c];
    if (total > 2147483647LL) return VO_ERANGE;
    offs[c + 1] = (int32_t)total;
  }
  double *z = (double *)std::malloc(sizeof(double) * 2 * (size_t)std::max<int64_t>(total, 1));
  if (!z) return VO_ENOMEM;
  parallel_chunks((int)ncols, T, [&](int b, int e, int) {
    for (int c = b; c < e; ++c) {
      int64_t s0 = start[c];
      for (int k = 0; k < cnt[c]; ++k) {
        z[2 * ((int64_t)offs[c] + k)] = lo[s0 + k];
        z[2 * ((int64_t)offs[c] + k) + 1] = hi[s0 + k];
      }
    }
  });
  *z_out = z;
  if (nseg_out) *nseg_out = total;
  return VO_OK;
}

extern "C" int vo_synth_torus(int nu, int nv, double major, double minor, double noise,
                              uint64_t seed, double **verts_out, int *nverts_out,
                              int32_t **tris_out, int *ntris_out) {
  if (nu < 3 || nv < 3 || !verts_out || !tris_out || !nverts_out || !ntris_out) return VO_EINVAL;
  SplitMix64 rng(seed);
  const int nvert = nu * nv, ntri = 2 * nu * nv;
  double *V = (double *)std::malloc(sizeof(double) * 3 * (size_t)nvert);
  int32_t *F = (int32_t *)std::malloc(sizeof(int32_t) * 3 * (size_t)ntri);
  if (!V || !F) {
    std::free(V);
    std::free(F);
    return VO_ENOMEM;
  }
  const double twopi = 6.283185307179586;
  for (int i = 0; i < nu; ++i)
    for (int j = 0; j < nv; ++j) {
      const double th = twopi * i / nu, ph = twopi * j / nv;
      const double n[3] = {std::cos(ph) * std::cos(th), std::cos(ph) * std::sin(th), std::sin(ph)};
      const double ring = major + minor * std::cos(ph);
      const double e = noise * rng.uniform(-1.0, 1.0);
      double *v = V + 3 * (i * nv + j);
      v[0] = 0.5 + ring * std::cos(th) + e * n[0];
      v[1] = 0.5 + ring * std::sin(th) + e * n[1];
      v[2] = 0.5 + minor * std::sin(ph) + e * n[2];
    }
  int32_t *f = F;
  for (int i = 0; i < nu; ++i)
    for (int j = 0; j < nv; ++j) {
      const int i1 = (i + 1) % nu, j1 = (j + 1) % nv;
      const int a = i * nv + j, b = i1 * nv + j, c = i1 * nv + j1, d = i * nv + j1;
      f[0] = a; f[1] = b; f[2] = c;
      f[3] = a; f[4] = c; f[5] = d;
      f += 6;
    }
  *verts_out = V;
  *nverts_out = nvert;
  *tris_out = F;
  *ntris_out = ntri;
  return VO_OK;
}

extern "C" void vo_host_free(void *p) { std::free(p); }
