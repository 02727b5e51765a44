// C-ABI bridge over the reference's own vor3d classes, compiled together with
// the unmodified reference sources into oracle/_ref/libvor3d_ref.so.
//
// TEST INFRASTRUCTURE ONLY. It exists so tests can pin the oracle restatement
// against the reference itself, and so bench.py's reference arm can time the
// reference's multithreaded `ours` path. Nothing in the product links it.
//
// Follows app/cli3d/offset3d.cpp:104-136: the method is chosen by name
// ("ours" = VoronoiMorphoVorPower, "brute_force" = VoronoiMorphoBruteForce),
// closing = dilation then erosion, opening = erosion then dilation, and the
// wall-clock timer surrounds each call (including the by-value input copy).
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>

#include "tbb/task_scheduler_init.h"
#include "vor3d/CompressedVolume.h"
#include "vor3d/VoronoiBruteForce.h"
#include "vor3d/VoronoiVorPower.h"

using voroffset3d::CompressedVolume;

namespace {

CompressedVolume make_volume(int nx, int ny, const double *origin, const double *extent,
                             double spacing, int padding, const int32_t *offs,
                             const double *z) {
  CompressedVolume v;
  // reset() stores the origin as given (already shifted by -padding*spacing),
  // exactly as the CompressedVolume constructor leaves it (CompressedVolume.cpp:11-23).
  v.reset(Eigen::Vector3d(origin[0], origin[1], origin[2]),
          Eigen::Vector3d(extent[0], extent[1], extent[2]), spacing, padding, nx, ny);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const int c = x + nx * y;
      auto &col = v.at(x, y);
      col.assign(z + 2 * (int64_t)offs[c], z + 2 * (int64_t)offs[c + 1]);
    }
  return v;
}

int export_volume(CompressedVolume &v, int32_t **out_offs, double **out_z, int *out_nx,
                  int *out_ny) {
  const int nx = v.gridSize()(0), ny = v.gridSize()(1);
  int64_t total = 0;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) total += (int64_t)v.at(x, y).size();
  if (total % 2) return -3;
  int32_t *offs = (int32_t *)std::malloc(sizeof(int32_t) * ((size_t)nx * ny + 1));
  double *z = (double *)std::malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
  if (!offs || !z) return -4;
  int64_t k = 0;
  offs[0] = 0;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const auto &col = v.at(x, y);
      std::memcpy(z + k, col.data(), sizeof(double) * col.size());
      k += (int64_t)col.size();
      offs[x + nx * y + 1] = (int32_t)(k / 2);
    }
  *out_offs = offs;
  *out_z = z;
  *out_nx = nx;
  *out_ny = ny;
  return 0;
}

}  // namespace

extern "C" {

// method: 0 = ours (VoronoiMorphoVorPower), 1 = brute_force.
// op: 0 = dilation, 1 = erosion, 2 = opening, 3 = closing.
// Returns 0 on success, negative on failure (exceptions never cross the ABI).
int ref_morph(int method, int op, int nx, int ny, const double *origin, const double *extent,
              double spacing, int padding, const int32_t *offs, const double *z, double radius,
              int nthreads, int32_t **out_offs, double **out_z, int *out_nx, int *out_ny,
              double *time_ms, double *time_1, double *time_2) {
  try {
    tbb::task_scheduler_init init(nthreads);
    CompressedVolume input = make_volume(nx, ny, origin, extent, spacing, padding, offs, z);
    CompressedVolume output;
    std::unique_ptr<voroffset3d::VoronoiMorpho> m;
    if (method == 0)
      m.reset(new voroffset3d::VoronoiMorphoVorPower());
    else if (method == 1)
      m.reset(new voroffset3d::VoronoiMorphoBruteForce());
    else
      return -1;
    double t1 = 0, t2 = 0;
    auto t0 = std::chrono::steady_clock::now();
    if (op == 0) {
      m->dilation(input, output, radius, t1, t2);
    } else if (op == 1) {
      m->erosion(input, output, radius, t1, t2);
    } else if (op == 2) {
      CompressedVolume tmp;
      m->erosion(input, tmp, radius, t1, t2);
      m->dilation(tmp, output, radius, t1, t2);
    } else if (op == 3) {
      CompressedVolume tmp;
      m->dilation(input, tmp, radius, t1, t2);
      m->erosion(tmp, output, radius, t1, t2);
    } else {
      return -2;
    }
    auto t3 = std::chrono::steady_clock::now();
    if (time_ms) *time_ms = std::chrono::duration<double, std::milli>(t3 - t0).count();
    if (time_1) *time_1 = t1;
    if (time_2) *time_2 = t2;
    return export_volume(output, out_offs, out_z, out_nx, out_ny);
  } catch (const std::exception &) {
    return -10;
  }
}

// Xor volume of two volumes with the same grid (Voronoi.cpp:91-111).
double ref_xor_volume(int nx, int ny, const double *origin, const double *extent, double spacing,
                      int padding, const int32_t *offs_a, const double *za,
                      const int32_t *offs_b, const double *zb) {
  try {
    CompressedVolume a = make_volume(nx, ny, origin, extent, spacing, padding, offs_a, za);
    CompressedVolume b = make_volume(nx, ny, origin, extent, spacing, padding, offs_b, zb);
    CompressedVolume r;
    voroffset3d::VoronoiMorphoVorPower m;
    return m.calculateXor(a, b, r);
  } catch (const std::exception &) {
    return -1.0;
  }
}

void ref_free(void *p) { std::free(p); }

}  // extern "C"
