// Host-side C++ mirror of the reference's method layer over the C ABI.
#include "voroffset_host.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <unordered_map>

namespace voroffset3d {

namespace {

void check(vo_ctx *ctx, int rc, const char *what) {
  if (rc != VO_OK) {
    std::ostringstream os;
    os << what << " failed (" << rc << "): " << (ctx ? vo_last_error(ctx) : "");
    throw std::runtime_error(os.str());
  }
}

}  // namespace

// ------------------------------------------------------------ CompressedVolume

CompressedVolume::CompressedVolume(Vec3 origin, Vec3 extent, Scalar voxel_size, int padding) {
  origin_ = origin;
  extent_ = extent;
  spacing_ = voxel_size;
  padding_ = padding;
  for (auto &o : origin_) o -= padding * voxel_size;
  nx_ = (int)(std::ceil(extent[0] / spacing_) + 2 * padding);
  ny_ = (int)(std::ceil(extent[1] / spacing_) + 2 * padding);
  data_.assign((size_t)nx_ * ny_, {});
}

void CompressedVolume::reset(Vec3 origin, Vec3 extent, Scalar voxel_size, int padding, int xsize, int ysize) {
  origin_ = origin;
  extent_ = extent;
  spacing_ = voxel_size;
  padding_ = padding;
  reshape(xsize, ysize);
}

void CompressedVolume::reshape(int xsize, int ysize) {
  nx_ = xsize;
  ny_ = ysize;
  data_.assign((size_t)nx_ * ny_, {});
}

std::array<double, 2> CompressedVolume::dexelCenter(int x, int y) const {
  return {(x + 0.5) * spacing_ + origin_[0], (y + 0.5) * spacing_ + origin_[1]};
}

int CompressedVolume::numSegments() const {
  int n = 0;
  for (const auto &c : data_) n += (int)(c.size() / 2);
  return n;
}

double CompressedVolume::get_volume() const {
  double vol = 0, h = spacing_;
  for (int x = 0; x < nx_; ++x)
    for (int y = 0; y < ny_; ++y) {
      const auto &c = at(x, y);
      for (size_t k = 0; k + 1 < c.size(); k += 2) vol = vol + h * h * h * (c[k + 1] - c[k]);
    }
  return vol;
}

void CompressedVolume::save(std::ostream &out) const {
  out << origin_[0] << ' ' << origin_[1] << ' ' << origin_[2] << "\n";
  out << extent_[0] << ' ' << extent_[1] << ' ' << extent_[2] << "\n";
  out << nx_ << ' ' << ny_ << "\n" << padding_ << "\n" << spacing_ << "\n";
  for (const auto &row : data_) {
    out << row.size();
    for (double v : row) out << ' ' << v;
    out << "\n";
  }
}

void CompressedVolume::load(std::istream &in) {
  in >> origin_[0] >> origin_[1] >> origin_[2] >> extent_[0] >> extent_[1] >> extent_[2];
  in >> nx_ >> ny_ >> padding_ >> spacing_;
  if (!in || nx_ < 0 || ny_ < 0) throw std::runtime_error("CompressedVolume::load: bad header");
  data_.assign((size_t)nx_ * ny_, {});
  for (auto &row : data_) {
    size_t n;
    in >> n;
    row.resize(n);
    for (auto &v : row) in >> v;
  }
  if (!in) throw std::runtime_error("CompressedVolume::load: truncated");
}

namespace {
constexpr char kCsrMagic[8] = {'V', 'O', 'C', 'S', 'R', '0', '0', '1'};
}

void CompressedVolume::save_csr(const std::string &filename) const {
  std::vector<int32_t> offs;
  std::vector<double> z;
  to_csr(offs, z);
  std::ofstream out(filename, std::ios::binary);
  if (!out) throw std::runtime_error("cannot write " + filename);
  const int32_t head[3] = {nx_, ny_, padding_};
  const double geo[7] = {origin_[0], origin_[1], origin_[2], extent_[0], extent_[1], extent_[2], spacing_};
  const int64_t nseg = (int64_t)z.size() / 2;
  out.write(kCsrMagic, 8);
  out.write(reinterpret_cast<const char *>(head), sizeof head);
  out.write(reinterpret_cast<const char *>(geo), sizeof geo);
  out.write(reinterpret_cast<const char *>(&nseg), sizeof nseg);
  out.write(reinterpret_cast<const char *>(offs.data()), (std::streamsize)(sizeof(int32_t) * offs.size()));
  out.write(reinterpret_cast<const char *>(z.data()), (std::streamsize)(sizeof(double) * z.size()));
  if (!out) throw std::runtime_error("write failed: " + filename);
}

void CompressedVolume::load_csr(const std::string &filename) {
  std::ifstream in(filename, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + filename);
  char magic[8];
  int32_t head[3];
  double geo[7];
  int64_t nseg = 0;
  in.read(magic, 8);
  in.read(reinterpret_cast<char *>(head), sizeof head);
  in.read(reinterpret_cast<char *>(geo), sizeof geo);
  in.read(reinterpret_cast<char *>(&nseg), sizeof nseg);
  if (!in || std::memcmp(magic, kCsrMagic, 8) != 0 || head[0] < 0 || head[1] < 0 || nseg < 0)
    throw std::runtime_error("not a CSR volume: " + filename);
  vo_grid g;
  g.nx = head[0];
  g.ny = head[1];
  g.padding = head[2];
  for (int k = 0; k < 3; ++k) {
    g.origin[k] = geo[k];
    g.extent[k] = geo[3 + k];
  }
  g.spacing = geo[6];
  std::vector<int32_t> offs((size_t)g.nx * g.ny + 1);
  std::vector<double> z(2 * (size_t)nseg);
  in.read(reinterpret_cast<char *>(offs.data()), (std::streamsize)(sizeof(int32_t) * offs.size()));
  in.read(reinterpret_cast<char *>(z.data()), (std::streamsize)(sizeof(double) * z.size()));
  if (!in || offs[0] != 0 || offs.back() != nseg) throw std::runtime_error("truncated CSR volume: " + filename);
  for (size_t c = 0; c + 1 < offs.size(); ++c)
    if (offs[c + 1] < offs[c]) throw std::runtime_error("bad CSR offsets: " + filename);
  from_csr(g, offs.data(), z.data());
}

vo_grid CompressedVolume::grid() const {
  vo_grid g;
  g.nx = nx_;
  g.ny = ny_;
  for (int k = 0; k < 3; ++k) {
    g.origin[k] = origin_[k];
    g.extent[k] = extent_[k];
  }
  g.spacing = spacing_;
  g.padding = padding_;
  return g;
}

void CompressedVolume::to_csr(std::vector<int32_t> &offs, std::vector<double> &z) const {
  offs.assign(data_.size() + 1, 0);
  size_t total = 0;
  for (size_t c = 0; c < data_.size(); ++c) {
    total += data_[c].size() / 2;  // a trailing unpaired value is ignored, as iterate() does
    offs[c + 1] = (int32_t)total;
  }
  z.resize(2 * total);
  size_t k = 0;
  for (const auto &col : data_)
    for (size_t i = 0; i + 1 < col.size(); i += 2) {
      z[k++] = col[i];
      z[k++] = col[i + 1];
    }
}

void CompressedVolume::from_csr(const vo_grid &g, const int32_t *offs, const double *z) {
  origin_ = {g.origin[0], g.origin[1], g.origin[2]};
  extent_ = {g.extent[0], g.extent[1], g.extent[2]};
  spacing_ = g.spacing;
  padding_ = g.padding;
  reshape(g.nx, g.ny);
  for (size_t c = 0; c < data_.size(); ++c) data_[c].assign(z + 2 * (size_t)offs[c], z + 2 * (size_t)offs[c + 1]);
}

// ------------------------------------------------------------ VoronoiMorphoGpu

VoronoiMorphoGpu::VoronoiMorphoGpu(int method, int device) : method_(method) {
  check(nullptr, vo_create(&ctx_, device), "vo_create");
}

VoronoiMorphoGpu::~VoronoiMorphoGpu() { vo_destroy(ctx_); }

void VoronoiMorphoGpu::apply(int op, const CompressedVolume &input, CompressedVolume &result, double radius,
                             double &time_1, double &time_2) {
  std::vector<int32_t> offs;
  std::vector<double> z;
  input.to_csr(offs, z);
  const vo_grid g = input.grid();
  vo_volume *in = nullptr, *out = nullptr;
  check(ctx_, vo_volume_upload(ctx_, &g, offs.data(), z.data(), &in), "vo_volume_upload");
  vo_timings t;
  int rc = vo_morph(ctx_, op, method_, radius, in, &out, &t);
  vo_volume_free(ctx_, in);
  check(ctx_, rc, "vo_morph");
  vo_grid og;
  int64_t nseg = 0;
  vo_volume_info(ctx_, out, &og, &nseg);
  std::vector<int32_t> ooffs((size_t)og.nx * og.ny + 1);
  std::vector<double> oz((size_t)std::max<int64_t>(2 * nseg, 1));
  rc = vo_volume_download(ctx_, out, ooffs.data(), oz.data());
  vo_volume_free(ctx_, out);
  check(ctx_, rc, "vo_volume_download");
  result.from_csr(og, ooffs.data(), oz.data());
  time_1 = t.pass1_ms;
  time_2 = t.pass2_ms;
}

void VoronoiMorphoGpu::dilation(CompressedVolume input, CompressedVolume &result, double radius, double &time_1,
                                double &time_2) {
  apply(VO_DILATION, input, result, radius, time_1, time_2);
}

void VoronoiMorphoGpu::erosion(CompressedVolume input, CompressedVolume &result, double radius, double &time_1,
                               double &time_2) {
  apply(VO_EROSION, input, result, radius, time_1, time_2);
}

double VoronoiMorphoGpu::calculateXor(const CompressedVolume &a, const CompressedVolume &b) {
  std::vector<int32_t> oa, ob;
  std::vector<double> za, zb;
  a.to_csr(oa, za);
  b.to_csr(ob, zb);
  const vo_grid ga = a.grid(), gb = b.grid();
  vo_volume *va = nullptr, *vb = nullptr;
  check(ctx_, vo_volume_upload(ctx_, &ga, oa.data(), za.data(), &va), "vo_volume_upload");
  int rc = vo_volume_upload(ctx_, &gb, ob.data(), zb.data(), &vb);
  if (rc) vo_volume_free(ctx_, va);
  check(ctx_, rc, "vo_volume_upload");
  double vol = 0;
  rc = vo_xor_volume(ctx_, va, vb, &vol);
  vo_volume_free(ctx_, va);
  vo_volume_free(ctx_, vb);
  check(ctx_, rc, "vo_xor_volume");
  return vol;
}

// ------------------------------------------------------------ mesh I/O

namespace {

bool ends_with(const std::string &s, const std::string &suf) {
  return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

void add_polygon(TriMesh &m, const std::vector<int32_t> &poly) {
  for (size_t k = 1; k + 1 < poly.size(); ++k) {
    m.tris.push_back(poly[0]);
    m.tris.push_back(poly[k]);
    m.tris.push_back(poly[k + 1]);
  }
}

}  // namespace

TriMesh load_mesh(const std::string &filename) {
  std::ifstream in(filename);
  if (!in) throw std::runtime_error("cannot open " + filename);
  TriMesh m;
  if (ends_with(filename, ".off")) {
    std::string head;
    in >> head;
    if (head != "OFF") throw std::runtime_error("not an OFF file: " + filename);
    int nv, nf, ne;
    in >> nv >> nf >> ne;
    m.verts.resize(3 * (size_t)nv);
    for (auto &v : m.verts) in >> v;
    for (int f = 0; f < nf; ++f) {
      int k;
      in >> k;
      std::vector<int32_t> poly(k);
      for (auto &i : poly) in >> i;
      add_polygon(m, poly);
    }
  } else {  // Wavefront OBJ: v and f records
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string tag;
      ls >> tag;
      if (tag == "v") {
        double x, y, zz;
        ls >> x >> y >> zz;
        m.verts.insert(m.verts.end(), {x, y, zz});
      } else if (tag == "f") {
        std::vector<int32_t> poly;
        std::string tok;
        while (ls >> tok) {
          int i = std::stoi(tok.substr(0, tok.find('/')));
          poly.push_back(i > 0 ? i - 1 : (int32_t)(m.verts.size() / 3) + i);
        }
        add_polygon(m, poly);
      }
    }
  }
  if (!in.eof() && in.fail()) throw std::runtime_error("malformed mesh " + filename);
  return m;
}

CompressedVolume create_dexels(VoronoiMorphoGpu &gpu, const std::string &filename, double &voxel_size, int padding,
                               int num_voxels) {
  TriMesh m = load_mesh(filename);
  vo_ctx *ctx = gpu.context();
  vo_volume *v = nullptr;
  double sp = voxel_size;
  check(ctx, vo_dexelize(ctx, m.verts.data(), (int)(m.verts.size() / 3), m.tris.data(), (int)(m.tris.size() / 3),
                         &sp, padding, num_voxels, &v),
        "vo_dexelize");
  voxel_size = sp;
  vo_grid g;
  int64_t nseg = 0;
  vo_volume_info(ctx, v, &g, &nseg);
  std::vector<int32_t> offs((size_t)g.nx * g.ny + 1);
  std::vector<double> z((size_t)std::max<int64_t>(2 * nseg, 1));
  int rc = vo_volume_download(ctx, v, offs.data(), z.data());
  vo_volume_free(ctx, v);
  check(ctx, rc, "vo_volume_download");
  CompressedVolume out;
  out.from_csr(g, offs.data(), z.data());
  return out;
}

namespace {

// Closed intervals of column list a minus those of b (both sorted, disjoint;
// flat [z0, z1, z2, z3, ...]); pieces of zero length are dropped.
std::vector<double> interval_minus(const std::vector<double> &a, const std::vector<double> *b) {
  std::vector<double> out;
  for (size_t i = 0; i + 1 < a.size(); i += 2) {
    double lo = a[i];
    const double hi = a[i + 1];
    if (b)
      for (size_t j = 0; j + 1 < b->size() && lo < hi; j += 2) {
        const double blo = (*b)[j], bhi = (*b)[j + 1];
        if (bhi <= lo) continue;
        if (blo >= hi) break;
        if (blo > lo) {
          out.push_back(lo);
          out.push_back(blo);
        }
        lo = bhi;
      }
    if (lo < hi) {
      out.push_back(lo);
      out.push_back(hi);
    }
  }
  return out;
}

// OBJ writer with vertices merged by (lattice x, lattice y, z).
struct ObjWriter {
  std::ostream &out;
  double ox, oy, h;
  std::unordered_map<std::string, size_t> ids;
  std::vector<std::array<size_t, 4>> faces;
  size_t next = 1;
  size_t vertex(int ix, int iy, double z) {
    char key[64];
    uint64_t zb;
    std::memcpy(&zb, &z, sizeof zb);
    std::snprintf(key, sizeof key, "%d:%d:%llx", ix, iy, (unsigned long long)zb);
    auto it = ids.find(key);
    if (it != ids.end()) return it->second;
    out << "v " << ox + ix * h << ' ' << oy + iy * h << ' ' << z * h << "\n";
    ids.emplace(key, next);
    return next++;
  }
  void quad(size_t a, size_t b, size_t c, size_t d) { faces.push_back({a, b, c, d}); }
  void finish() {
    for (const auto &f : faces) out << "f " << f[0] << ' ' << f[1] << ' ' << f[2] << ' ' << f[3] << "\n";
  }
};

}  // namespace

void dexel_dump(const std::string &filename, const CompressedVolume &dexels) {
  std::ofstream out(filename);
  if (!out) throw std::runtime_error("cannot write " + filename);
  out.precision(17);
  const auto gs = dexels.gridSize();
  const auto o = dexels.origin();
  const double h = dexels.spacing();
  if (ends_with(filename, ".xyz")) {  // points_dump (Dexelize.cpp:289-310)
    for (int y = 0; y < gs[1]; ++y)
      for (int x = 0; x < gs[0]; ++x) {
        const auto &c = dexels.at(x, y);
        for (size_t i = 0; i + 1 < c.size(); i += 2)
          for (int e = 0; e < 2; ++e)
            out << o[0] + (x + 0.5) * h << ' ' << o[1] + (y + 0.5) * h << ' ' << c[i + e] * h << "\n";
      }
    return;
  }
  ObjWriter w{out, o[0], o[1], h, {}, {}, 1};
  for (int y = 0; y < gs[1]; ++y)
    for (int x = 0; x < gs[0]; ++x) {
      const auto &c = dexels.at(x, y);
      // bottom and top faces; a face shared by two touching segments is interior
      for (size_t i = 0; i + 1 < c.size(); i += 2) {
        const double z0 = c[i], z1 = c[i + 1];
        if (!(i >= 2 && c[i - 1] == z0))
          w.quad(w.vertex(x, y, z0), w.vertex(x, y + 1, z0), w.vertex(x + 1, y + 1, z0), w.vertex(x + 1, y, z0));
        if (!(i + 2 < c.size() && c[i + 2] == z1))
          w.quad(w.vertex(x, y, z1), w.vertex(x + 1, y, z1), w.vertex(x + 1, y + 1, z1), w.vertex(x, y + 1, z1));
      }
      // sides: the column's intervals minus the neighbour's, facing the neighbour
      const std::vector<double> *nb[4] = {
          x > 0 ? &dexels.at(x - 1, y) : nullptr, x + 1 < gs[0] ? &dexels.at(x + 1, y) : nullptr,
          y > 0 ? &dexels.at(x, y - 1) : nullptr, y + 1 < gs[1] ? &dexels.at(x, y + 1) : nullptr};
      for (int s = 0; s < 4; ++s) {
        const std::vector<double> open = interval_minus(c, nb[s]);
        for (size_t i = 0; i + 1 < open.size(); i += 2) {
          const double z0 = open[i], z1 = open[i + 1];
          if (s == 0)
            w.quad(w.vertex(x, y, z0), w.vertex(x, y, z1), w.vertex(x, y + 1, z1), w.vertex(x, y + 1, z0));
          else if (s == 1)
            w.quad(w.vertex(x + 1, y, z0), w.vertex(x + 1, y + 1, z0), w.vertex(x + 1, y + 1, z1),
                   w.vertex(x + 1, y, z1));
          else if (s == 2)
            w.quad(w.vertex(x, y, z0), w.vertex(x + 1, y, z0), w.vertex(x + 1, y, z1), w.vertex(x, y, z1));
          else
            w.quad(w.vertex(x, y + 1, z0), w.vertex(x, y + 1, z1), w.vertex(x + 1, y + 1, z1),
                   w.vertex(x + 1, y + 1, z0));
        }
      }
    }
  w.finish();
}

void dexel_dump_boxes(const std::string &filename, const CompressedVolume &dexels) {
  std::ofstream out(filename);
  if (!out) throw std::runtime_error("cannot write " + filename);
  out.precision(17);
  const auto gs = dexels.gridSize();
  const auto o = dexels.origin();
  const double h = dexels.spacing();
  // one box per segment (Dexelize.cpp:320-343), written as six quads each
  size_t base = 1;
  for (int y = 0; y < gs[1]; ++y)
    for (int x = 0; x < gs[0]; ++x) {
      const auto &c = dexels.at(x, y);
      for (size_t i = 0; i + 1 < c.size(); i += 2) {
        const double x0 = o[0] + x * h, x1 = o[0] + (x + 1) * h;
        const double y0 = o[1] + y * h, y1 = o[1] + (y + 1) * h;
        const double z0 = c[i] * h, z1 = c[i + 1] * h;
        const double P[8][3] = {{x0, y0, z0}, {x1, y0, z0}, {x1, y1, z0}, {x0, y1, z0},
                                {x0, y0, z1}, {x1, y0, z1}, {x1, y1, z1}, {x0, y1, z1}};
        for (auto &p : P) out << "v " << p[0] << ' ' << p[1] << ' ' << p[2] << "\n";
        static const int F[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                    {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
        for (auto &f : F)
          out << "f " << base + f[0] << ' ' << base + f[1] << ' ' << base + f[2] << ' ' << base + f[3] << "\n";
        base += 8;
      }
    }
}

}  // namespace voroffset3d
