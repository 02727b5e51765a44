// C++ host side of the GB300 dexel morphology library: the reference's method
// layer interface (src/vor3d/Voronoi.h:13-44) and dexel container
// (src/vor3d/CompressedVolume.h:11-41) restated over the C ABI of
// include/voroffset_gpu.h, so code written against VoronoiMorpho can select
// the GPU method beside "ours" and "brute_force" (app/cli3d/offset3d.cpp:104-112).
#pragma once

#include <array>
#include <cstdint>
#include <iosfwd>
#include <stdexcept>
#include <string>
#include <vector>

#include "voroffset_gpu.h"

namespace voroffset3d {

typedef double Scalar;

// Dexel grid: nx*ny columns, column (x, y) at index x + nx*y, each a flat
// sorted list [z0, z1, z2, z3, ...] of segment endpoints in dexel units
// (CompressedVolume.h:28-29). The origin is stored already shifted by
// -padding*spacing (CompressedVolume.cpp:11-23).
class CompressedVolume {
 public:
  typedef std::array<double, 3> Vec3;

  CompressedVolume() = default;
  // CompressedVolume.cpp:11-23: origin -= padding*voxel_size;
  // grid = ceil(extent / voxel_size) + 2*padding in x and y.
  CompressedVolume(Vec3 origin, Vec3 extent, Scalar voxel_size, int padding);

  void reset(Vec3 origin, Vec3 extent, Scalar voxel_size, int padding, int xsize, int ysize);
  void reshape(int xsize, int ysize);

  std::vector<Scalar> &at(int x, int y) { return data_[(size_t)x + (size_t)nx_ * y]; }
  const std::vector<Scalar> &at(int x, int y) const { return data_[(size_t)x + (size_t)nx_ * y]; }

  std::array<int, 2> gridSize() const { return {nx_, ny_}; }
  int numDexels() const { return nx_ * ny_; }
  Vec3 origin() const { return origin_; }
  Vec3 extent() const { return extent_; }
  Scalar spacing() const { return spacing_; }
  int padding() const { return padding_; }
  std::array<double, 2> dexelCenter(int x, int y) const;  // CompressedVolumeBase.cpp:5-11

  int numSegments() const;  // CompressedVolume.cpp:76-83
  double get_volume() const;  // CompressedVolume.cpp:61-74

  // Text marshalling (CompressedVolume.cpp:116-152).
  void save(std::ostream &out) const;
  void load(std::istream &in);
  // Binary CSR dump (no reference counterpart; exact, for golden files and
  // large volumes): "VOCSR001", int32 nx, ny, padding, FP64 origin[3],
  // extent[3], spacing, int64 segment count, int32 offsets[nx*ny+1], FP64
  // endpoint pairs, all little-endian.
  void save_csr(const std::string &filename) const;
  void load_csr(const std::string &filename);

  // CSR packing for the C ABI.
  vo_grid grid() const;
  void to_csr(std::vector<int32_t> &offs, std::vector<double> &z) const;
  void from_csr(const vo_grid &g, const int32_t *offs, const double *z);

 private:
  Vec3 origin_{{0, 0, 0}}, extent_{{0, 0, 0}};
  Scalar spacing_ = 1;
  int padding_ = 0;
  int nx_ = 0, ny_ = 0;
  std::vector<std::vector<Scalar>> data_;
};

// The method interface of src/vor3d/Voronoi.h:13-44.
class VoronoiMorpho {
 public:
  virtual ~VoronoiMorpho() = default;
  virtual void dilation(CompressedVolume input, CompressedVolume &result, double radius, double &time_1,
                        double &time_2) = 0;
  virtual void erosion(CompressedVolume input, CompressedVolume &result, double radius, double &time_1,
                       double &time_2) = 0;
};

// GPU method: every operation runs on one sm_103 device through the C ABI.
// Errors surface as std::runtime_error carrying vo_last_error(), the way the
// reference reports failed assertions (Common.cpp:8-18).
class VoronoiMorphoGpu : public VoronoiMorpho {
 public:
  explicit VoronoiMorphoGpu(int method = VO_METHOD_FAST, int device = 0);
  ~VoronoiMorphoGpu() override;
  VoronoiMorphoGpu(const VoronoiMorphoGpu &) = delete;
  VoronoiMorphoGpu &operator=(const VoronoiMorphoGpu &) = delete;

  void dilation(CompressedVolume input, CompressedVolume &result, double radius, double &time_1,
                double &time_2) override;
  void erosion(CompressedVolume input, CompressedVolume &result, double radius, double &time_1,
               double &time_2) override;
  // opening / closing in one call (offset3d.cpp:124-133 chains them on the host)
  void apply(int op, const CompressedVolume &input, CompressedVolume &result, double radius, double &time_1,
             double &time_2);
  // Xor volume (Voronoi.cpp:91-111).
  double calculateXor(const CompressedVolume &a, const CompressedVolume &b);

  vo_ctx *context() { return ctx_; }

 private:
  vo_ctx *ctx_ = nullptr;
  int method_;
};

// Triangle mesh (vertices and 0-based triangles); quads are split on load.
struct TriMesh {
  std::vector<double> verts;   // 3 per vertex
  std::vector<int32_t> tris;   // 3 per triangle
};
TriMesh load_mesh(const std::string &filename);  // .obj or .off

// create_dexels (Dexelize.h:25-28) on the GPU: voxel_size is updated when
// num_voxels > 0 (spacing = longest bbox side / num_voxels).
CompressedVolume create_dexels(VoronoiMorphoGpu &gpu, const std::string &filename, double &voxel_size,
                               int padding = 0, int num_voxels = -1);

// dexel_dump (Dexelize.cpp:281-351): the dexel boxes of a volume, one per
// segment. ".xyz" writes the segment endpoints at the dexel centres
// (points_dump). Otherwise a Wavefront OBJ of the boxes' boundary: the faces
// no neighbouring box covers (top and bottom of every segment, and each side
// minus the neighbouring column's segments there), with vertices merged, the
// effect of compute_borders / connect / remove_isolated on the box cells.
// Side faces are split only at the z values of the two columns they separate,
// so vertices of other columns may lie on their edges (T-junctions).
void dexel_dump(const std::string &filename, const CompressedVolume &dexels);
// The six faces of every box, eight unshared vertices per box.
void dexel_dump_boxes(const std::string &filename, const CompressedVolume &dexels);

}  // namespace voroffset3d
