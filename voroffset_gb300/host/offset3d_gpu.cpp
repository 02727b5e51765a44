// offset3d_gpu: the reference's 3D offsetting CLI (app/cli3d/offset3d.cpp)
// with the GPU methods: mesh -> dexels -> dilation / erosion / opening /
// closing -> dexel mesh and JSON timings. Same flags:
//   input (-i), -o output mesh, -j json, -d dexel size, -n num dexels (-1: use
//   -d), -p padding, -t threads (recorded only), -r radius, -m method,
//   -x operation, -f force overwrite, -u radius in mm.
// Methods: gpu (FP32-guarded exact, default), gpu_envelope (the two envelope
// sweeps in FP64), gpu_separable (the painter form, FP64 kernels), gpu_brute
// (lattice-disc brute force).
// Additions: -s/--save-volume FILE writes the output volume (the text format of
// CompressedVolume::save, or the exact binary CSR dump when FILE ends in .csr);
// --boxes writes six quads per dexel box instead of the boundary surface.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "voroffset_host.h"

using namespace voroffset3d;

namespace {

struct Args {
  std::string input, output_mesh = "output.obj", output_json, method = "gpu", operation = "dilation";
  std::string save_volume;
  bool boxes = false;
  double radius = 8, dexels_size = 1;
  int padding = 0, num_dexels = 256, num_thread = 1;
  bool force = false, radius_in_mm = false;
};

[[noreturn]] void usage(const char *msg) {
  std::fprintf(stderr,
               "%s\nusage: offset3d_gpu input [-o out.obj] [-j out.json] [-d size] [-n num_dexels] [-p padding]\n"
               "       [-r radius] [-m gpu|gpu_envelope|gpu_separable|gpu_brute] [-x noop|dilation|erosion|closing|opening]\n"
               "       [-f] [-u] [-s volume.txt|volume.csr] [--boxes]\n",
               msg);
  std::exit(2);
}

Args parse(int argc, char **argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string s = argv[i];
    auto val = [&](const char *name) -> std::string {
      if (i + 1 >= argc) usage((std::string("missing value for ") + name).c_str());
      return argv[++i];
    };
    if (s == "-i" || s == "--input") a.input = val("-i");
    else if (s == "-o" || s == "--output") a.output_mesh = val("-o");
    else if (s == "-j" || s == "--json") a.output_json = val("-j");
    else if (s == "-d" || s == "--dexels_size") a.dexels_size = std::atof(val("-d").c_str());
    else if (s == "-n" || s == "--num_dexels") a.num_dexels = std::atoi(val("-n").c_str());
    else if (s == "-p" || s == "--padding") a.padding = std::atoi(val("-p").c_str());
    else if (s == "-t" || s == "--num_thread") a.num_thread = std::atoi(val("-t").c_str());
    else if (s == "-r" || s == "--radius") a.radius = std::atof(val("-r").c_str());
    else if (s == "-m" || s == "--method") a.method = val("-m");
    else if (s == "-x" || s == "--apply") a.operation = val("-x");
    else if (s == "-f" || s == "--force") a.force = true;
    else if (s == "-u" || s == "--radius_in_mm") a.radius_in_mm = true;
    else if (s == "-s" || s == "--save-volume") a.save_volume = val("-s");
    else if (s == "--boxes") a.boxes = true;
    else if (!s.empty() && s[0] != '-' && a.input.empty()) a.input = s;
    else if (!s.empty() && s[0] != '-') a.output_mesh = s;
    else usage(("unknown option " + s).c_str());
  }
  if (a.input.empty()) usage("an input mesh is required");
  return a;
}

bool exists(const std::string &f) { return std::ifstream(f).good(); }

}  // namespace

int main(int argc, char **argv) {
  Args args = parse(argc, argv);
  int method;
  if (args.method == "gpu") method = VO_METHOD_FAST;
  else if (args.method == "gpu_envelope") method = VO_METHOD_ENVELOPE;
  else if (args.method == "gpu_separable") method = VO_METHOD_SEPARABLE;
  else if (args.method == "gpu_brute") method = VO_METHOD_BRUTE;
  else usage(("invalid method: " + args.method).c_str());
  int op;
  if (args.operation == "noop") op = -1;
  else if (args.operation == "dilation") op = VO_DILATION;
  else if (args.operation == "erosion") op = VO_EROSION;
  else if (args.operation == "opening") op = VO_OPENING;
  else if (args.operation == "closing") op = VO_CLOSING;
  else usage(("invalid operation: " + args.operation).c_str());

  try {
    auto t0 = std::chrono::steady_clock::now();
    VoronoiMorphoGpu gpu(method, 0);
    CompressedVolume input = create_dexels(gpu, args.input, args.dexels_size, args.padding, args.num_dexels);
    if (args.radius_in_mm) args.radius /= input.spacing();
    std::fprintf(stderr, "grid %d x %d, spacing %g, radius %g dexels, %d segments\n", input.gridSize()[0],
                 input.gridSize()[1], input.spacing(), args.radius, input.numSegments());
    CompressedVolume output;
    double t1 = 0, t2 = 0;
    if (op < 0)
      output = input;
    else
      gpu.apply(op, input, output, args.radius, t1, t2);
    if (!args.output_mesh.empty()) {
      if (exists(args.output_mesh) && !args.force)
        std::fprintf(stderr, "Output mesh already exists. Please use -f to force overwriting.\n");
      else if (args.boxes)
        dexel_dump_boxes(args.output_mesh, output);
      else
        dexel_dump(args.output_mesh, output);
    }
    if (!args.save_volume.empty()) {
      const std::string &f = args.save_volume;
      if (f.size() >= 4 && f.compare(f.size() - 4, 4, ".csr") == 0) {
        output.save_csr(f);
      } else {
        std::ofstream vo(f);
        vo.precision(17);
        output.save(vo);
      }
    }
    const double total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (!args.output_json.empty()) {
      if (exists(args.output_json) && !args.force) {
        std::fprintf(stderr, "Output json already exists. Please use -f to force overwriting.\n");
      } else {
        std::ofstream o(args.output_json);
        o.precision(17);
        o << "{\n    \"method\": \"" << args.method << "\",\n    \"num_threads\": " << args.num_thread
          << ",\n    \"model_name\": \"" << args.input << "\",\n    \"voxel_size\": " << input.spacing()
          << ",\n    \"padding\": " << input.padding() << ",\n    \"num_dexels\": " << args.num_dexels
          << ",\n    \"radius\": " << args.radius << ",\n    \"grid_size\": [" << input.gridSize()[0] << ", "
          << input.gridSize()[1] << "],\n    \"num_segments\": " << input.numSegments()
          << ",\n    \"operation\": \"" << args.operation << "\",\n    \"time\": " << total
          << ",\n    \"time_first_pass\": " << t1 << ",\n    \"time_second_pass\": " << t2
          << ",\n    \"output_segments\": " << output.numSegments() << "\n}\n";
      }
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "offset3d_gpu: %s\n", e.what());
    return 1;
  }
  return 0;
}
