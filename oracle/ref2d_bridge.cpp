// C bridge to the reference's own 2D morphology (src/vor2d, CompressedImage),
// compiled unmodified into oracle/_ref/libvor2d_ref.so. TEST INFRASTRUCTURE
// ONLY: it pins the oracle's 2D restatement; the product never links it.
//
// An image is `height` rows of `width` pixels; row i holds sorted half-open
// spans as event pairs [a0, b0, a1, b1, ...] (the rows of CompressedImage,
// CompressedImage.h:32-41), given in CSR form: offs[height + 1] counts events.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "vor2d/CompressedImage.h"

extern "C" int ref2d_morph(int op, int width, int height, const int32_t *offs, const int32_t *events, double radius,
                           int32_t **out_offs, int32_t **out_events) {
  try {
    // CompressedImage::load's text layout (CompressedImage.cpp:84-99): width, row count, then per
    // row its event count and events
    std::ostringstream in;
    in << width << ' ' << height << '\n';
    for (int i = 0; i < height; ++i) {
      in << (offs[i + 1] - offs[i]);
      for (int k = offs[i]; k < offs[i + 1]; ++k) in << ' ' << events[k];
      in << '\n';
    }
    std::istringstream is(in.str());
    voroffset::CompressedImage img(is);
    switch (op) {
      case 0: img.dilate(radius); break;
      case 1: img.erode(radius); break;
      case 2: img.open(radius); break;
      case 3: img.close(radius); break;
      default: return -1;
    }
    std::ostringstream os;
    img.save(os);
    std::istringstream rs(os.str());
    int w2 = 0;
    unsigned h2 = 0;
    rs >> w2 >> h2;
    std::vector<int32_t> o(1, 0), e;
    for (unsigned i = 0; i < h2; ++i) {
      size_t n = 0;
      rs >> n;
      for (size_t k = 0; k < n; ++k) {
        int v;
        rs >> v;
        e.push_back(v);
      }
      o.push_back((int32_t)e.size());
    }
    if (!rs || (int)h2 != height) return -2;
    *out_offs = (int32_t *)std::malloc(sizeof(int32_t) * o.size());
    *out_events = (int32_t *)std::malloc(sizeof(int32_t) * (e.size() + 1));
    if (!*out_offs || !*out_events) return -3;
    std::memcpy(*out_offs, o.data(), sizeof(int32_t) * o.size());
    if (!e.empty()) std::memcpy(*out_events, e.data(), sizeof(int32_t) * e.size());
    return 0;
  } catch (...) {
    return -4;
  }
}

extern "C" void ref2d_free(void *p) { std::free(p); }

// The FP64 twin, DoubleCompressedImage (DoubleCompressedImage.cpp:680-720):
// rows of closed spans with FP64 events; dilate scales its radius by the row
// count, erode does not (as the reference does).
#include "vor2d/DoubleCompressedImage.h"

extern "C" int ref2d_morph_f64(int op, int width, int height, const int32_t *offs, const double *events,
                               double radius, int32_t **out_offs, double **out_events) {
  try {
    std::ostringstream in;
    in.precision(17);
    in << width << ' ' << height << '\n';
    for (int i = 0; i < height; ++i) {
      in << (offs[i + 1] - offs[i]);
      for (int k = offs[i]; k < offs[i + 1]; ++k) in << ' ' << events[k];
      in << '\n';
    }
    std::istringstream is(in.str());
    voroffset::DoubleCompressedImage img(is);
    switch (op) {
      case 0: img.dilate(radius); break;
      case 1: img.erode(radius); break;
      case 2: img.open(radius); break;
      case 3: img.close(radius); break;
      default: return -1;
    }
    std::vector<int32_t> o(1, 0);
    std::vector<double> e;
    for (int i = 0; i < img.height(); ++i) {
      const auto &row = img.at(i);
      e.insert(e.end(), row.begin(), row.end());
      o.push_back((int32_t)e.size());
    }
    *out_offs = (int32_t *)std::malloc(sizeof(int32_t) * o.size());
    *out_events = (double *)std::malloc(sizeof(double) * (e.size() + 1));
    if (!*out_offs || !*out_events) return -3;
    std::memcpy(*out_offs, o.data(), sizeof(int32_t) * o.size());
    if (!e.empty()) std::memcpy(*out_events, e.data(), sizeof(double) * e.size());
    return 0;
  } catch (...) {
    return -4;
  }
}
