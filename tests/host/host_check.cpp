// Drives the C++ host layer (voroffset_gb300/host) for the tests: volume I/O,
// the mesh writers, and VoronoiMorphoGpu called directly.
//   host_check roundtrip IN.txt OUT.txt        load + save of the text format
//   host_check csr IN.txt OUT.csr OUT2.txt     text -> binary CSR -> text (17 digits)
//   host_check stats IN.txt                    numSegments and get_volume
//   host_check surface IN.txt OUT.obj          boundary mesh (dexel_dump)
//   host_check boxes IN.txt OUT.obj            six quads per box (dexel_dump_boxes)
//   host_check morph OP METHOD R IN.txt OUT.txt  OP: dilation|erosion|opening|closing (GPU)
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>

#include "voroffset_host.h"

using namespace voroffset3d;

static CompressedVolume load_text(const char *f) {
  std::ifstream in(f);
  if (!in) throw std::runtime_error(std::string("cannot open ") + f);
  CompressedVolume v;
  v.load(in);
  return v;
}

static void save_text(const CompressedVolume &v, const char *f, int precision) {
  std::ofstream out(f);
  if (precision > 0) out.precision(precision);
  v.save(out);
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const std::string cmd = argv[1];
  try {
    if (cmd == "roundtrip" && argc == 4) {
      save_text(load_text(argv[2]), argv[3], 0);
    } else if (cmd == "csr" && argc == 5) {
      load_text(argv[2]).save_csr(argv[3]);
      CompressedVolume v;
      v.load_csr(argv[3]);
      save_text(v, argv[4], 17);
    } else if (cmd == "stats" && argc == 3) {
      CompressedVolume v = load_text(argv[2]);
      std::printf("%d %.17g\n", v.numSegments(), v.get_volume());
    } else if (cmd == "surface" && argc == 4) {
      dexel_dump(argv[3], load_text(argv[2]));
    } else if (cmd == "boxes" && argc == 4) {
      dexel_dump_boxes(argv[3], load_text(argv[2]));
    } else if (cmd == "morph" && argc == 7) {
      const std::string op = argv[2], method = argv[3];
      const double r = std::atof(argv[4]);
      const int m = method == "separable" ? VO_METHOD_SEPARABLE : method == "brute" ? VO_METHOD_BRUTE : VO_METHOD_FAST;
      VoronoiMorphoGpu gpu(m, 0);
      CompressedVolume in = load_text(argv[5]), out;
      double t1 = 0, t2 = 0;
      if (op == "dilation") gpu.dilation(in, out, r, t1, t2);         // the VoronoiMorpho interface
      else if (op == "erosion") gpu.erosion(in, out, r, t1, t2);
      else if (op == "opening") gpu.apply(VO_OPENING, in, out, r, t1, t2);
      else if (op == "closing") gpu.apply(VO_CLOSING, in, out, r, t1, t2);
      else return 2;
      save_text(out, argv[6], 17);
    } else {
      return 2;
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "host_check: %s\n", e.what());
    return 1;
  }
  return 0;
}
