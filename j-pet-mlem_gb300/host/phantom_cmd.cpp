// 2d_strip_phantom: list-mode event generator for the 2D strip scanner with the
// options, phantom description format and outputs of the reference tool
// (src/2d/strip/phantom_cmd.cpp:136-444, src/2d/strip/options.cpp:78-103),
// running the Monte Carlo on the GPU through libjpet_strip
// (jpet_strip_generate_host).
//
// Outputs: the smeared responses (z_u, z_d, dl) to --output, binary float
// triples or, for a .txt name, one text line each; <base>.cfg with the options;
// the int32 count images <base>_emitted, <base>_detected and <base>_naive with
// their .nrrd headers; with --tan-bins also <base>_tan_bins (int32, the naive
// points binned by tangent) and <base>_tan_kernel (float, the analytic kernel
// of each voxel at --kernel-point), 3D maps of n_z x n_y x tan_bins.  The
// events follow a deterministic counter-based stream selected by --seed (the
// reference seeds std::mt19937 per OpenMP thread, so its output is not
// reproducible).  --no-responses skips the responses file and keeps the rest;
// --full adds <base>_wo_error and <base>_full_response (the exact responses)
// and <base>_events (emission point and direction), each with the output's
// extension and format.  Not supported: PNG previews.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "jpet_cmdline.hpp"
#include "jpet_strip.h"

using jpet::cmd::Kind;
using jpet::cmd::Parser;
namespace cmd = jpet::cmd;

namespace {

// add_phantom_options (src/2d/strip/options.cpp:13-46,78-103) plus --seed and
// --cuda-device.
void add_options(Parser& cl) {
  cl.add("config", 'c', "load config file", Kind::Path, cmd::kDontSave, "", false, true);
  cl.add("radius", 'r', "R distance between scintillator", Kind::Doubles, cmd::kOptional, "0.5");
  cl.add("length", 'l', "scintillator length", Kind::Double, cmd::kOptional, "1");
  cl.add("s-pixel", 'p', "pixel size", Kind::Double, cmd::kOptional, "0.01");
  cl.add("n-pixels", 'n', "number of pixels", Kind::Int, cmd::kDontSave, "0");
  cl.add("n-z-pixels", 0, "number of z pixels", Kind::Int, cmd::kOptional, "0");
  cl.add("n-y-pixels", 0, "number of y pixels", Kind::Int, cmd::kOptional, "0");
  cl.add("s-z", 0, "TOF sigma along z axis", Kind::Double, cmd::kAlwaysSave, "0.015");
  cl.add("s-dl", 0, "TOF sigma delta-l", Kind::Double, cmd::kAlwaysSave, "0.06");
  cl.add("n-emissions", 'e', "number of emissions", Kind::Size, cmd::kOptional, "0");
  cl.add_flag("verbose", 'v', "print progress information (-v) or benchmark (-vv)");
  cl.add("n-threads", 'T', "number of OpenMP threads", Kind::Int, cmd::kDontSave, "0");
  cl.add("scale", 0, "Scale phantom with given constant", Kind::Double, cmd::kAlwaysSave, "1");
  cl.add_flag("additive", 0, "phantom regions are additive, not disjunctive");
  cl.add("tan-bins", 0, "Bin reconstructed events using given number of tangent bins",
         Kind::Int, cmd::kDontSave, "0");
  cl.add("kernel-point", 0, "Point to evaluate kernel in", Kind::Doubles, cmd::kDontSave, "");
  cl.add_flag("full", 0, "Emit additional full information");
  cl.add_flag("no-responses", 0, "Do not emit responses");
  cl.add("point", 0, "Add point phantom x,y[,intensity]", Kind::Doubles, cmd::kOptional, "");
  cl.footer("phantom_description\nbuild: GB300 (sm_103a)");
  cl.add("output", 'o', "responses file", Kind::Path, cmd::kOptional, "phantom.bin", true);
  cl.add_flag("detected", 0, "collects detected emissions");
  cl.add("image-origin", 0, "Image origin x,y (default 0,0)", Kind::Doubles, cmd::kDontSave, "");
  cl.add("seed", 0, "seed of the counter-based random stream", Kind::Size, cmd::kDontSave, "1");
  cl.add("cuda-device", 'D', "CUDA device", Kind::Int, cmd::kDontSave, "0");
}

// calculate_scanner_options (src/2d/strip/options.cpp:106-124).
void calculate_scanner_options(Parser& cl) {
  if (cl.exist("n-pixels")) {
    cl.set("n-z-pixels", cl.get_path("n-pixels"));
    cl.set("n-y-pixels", cl.get_path("n-pixels"));
  } else {
    auto radius = cl.get_doubles("radius");
    if (radius.empty()) throw "at least one --radius has to be specified";
    if (radius.size() > 1)
      std::cerr << "warning: more than one radius specified with --radius" << std::endl;
    double L = cl.get_double("length"), p = cl.get_double("s-pixel");
    if (!cl.exist("n-z-pixels"))
      cl.set("n-z-pixels", std::to_string(static_cast<int>(std::ceil(L / p))));
    if (!cl.exist("n-y-pixels"))
      cl.set("n-y-pixels", std::to_string(static_cast<int>(std::ceil(2 * radius[0] / p))));
  }
}

// Phantom::operator<< (src/2d/geometry/phantom.h:137-181): "ellipse x y a b
// angle intensity", "rectangle x y a b intensity", "point x y intensity"; the
// scale applies to ellipses and rectangles; a malformed line ends the file.
void read_phantom(std::istream& in, double scale, std::vector<jpet_strip_region>& out) {
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream iss(line);
    std::string type;
    iss >> type;
    jpet_strip_region r{};
    if (type == "ellipse") {
      double x, y, a, b, angle, intensity;
      if (!(iss >> x >> y >> a >> b >> angle >> intensity)) break;
      r.kind = JPET_REGION_ELLIPSE;
      r.x = x * scale;
      r.y = y * scale;
      r.a = a * scale;
      r.b = b * scale;
      r.angle_deg = angle;
      r.intensity = intensity;
    } else if (type == "rectangle") {
      double x, y, a, b, intensity;
      if (!(iss >> x >> y >> a >> b >> intensity)) break;
      r.kind = JPET_REGION_RECTANGLE;
      r.x = x * scale;
      r.y = y * scale;
      r.a = a * scale;
      r.b = b * scale;
      r.intensity = intensity;
    } else if (type == "point") {
      double x, y, intensity;
      if (!(iss >> x >> y >> intensity)) break;
      r.kind = JPET_REGION_POINT;
      r.x = x;
      r.y = y;
      r.intensity = intensity;
    } else {
      throw "unknown phantom type: " + type;
    }
    out.push_back(r);
  }
}

// rows of `width` floats, as text lines ("a b c") or raw binary
void write_floats(const std::string& fn, const std::vector<float>& v, int64_t rows, int width,
                  bool text) {
  if (text) {
    std::ofstream o(fn);
    for (int64_t i = 0; i < rows; ++i)
      for (int k = 0; k < width; ++k) o << v[width * i + k] << (k + 1 < width ? ' ' : '\n');
    if (!o) throw "cannot write " + fn;
  } else {
    std::ofstream o(fn, std::ios::binary);
    o.write(reinterpret_cast<const char*>(v.data()), rows * width * sizeof(float));
    if (!o) throw "cannot write " + fn;
  }
}

const char* nrrd_type(const int32_t*) { return "int"; }
const char* nrrd_type(const float*) { return "float"; }

// raw map plus its NRRD header (nrrd_writer.h:18-27): 2D for depth 0, else 3D
template <typename T>
void write_image(const std::string& base, const char* suffix, const std::vector<T>& img, int n_z,
                 int n_y, int depth = 0) {
  const std::string raw = base + suffix;
  std::ofstream o(raw, std::ios::binary);
  o.write(reinterpret_cast<const char*>(img.data()), img.size() * sizeof(T));
  if (!o) throw "cannot write " + raw;
  std::ofstream h(raw + ".nrrd");
  h << "NRRD0001\ntype: " << nrrd_type(img.data())
    << "\nendian: little\ndimension: " << (depth > 0 ? 3 : 2) << "\nsizes: " << n_z << " "
    << n_y;
  if (depth > 0) h << " " << depth;
  h << "\ndata file: ./" << raw << "\nencoding: raw\n";
}

int run(int argc, char* argv[]) {
  Parser cl;
  add_options(cl);
  cl.parse_check(argc, argv);
  calculate_scanner_options(cl);
  if (cl.rest().empty() && !cl.exist("point")) {
    if (argc == 1) {
      std::cerr << cl.usage();
      return 0;
    }
    throw "at least one input phantom description expected, consult --help";
  }
  const int tan_bins = cl.get_int("tan-bins");
  if (tan_bins < 0) throw "--tan-bins must not be negative";
  double kernel_x = 0, kernel_y = 0;
  if (cl.exist("kernel-point")) {
    auto kp = cl.get_doubles("kernel-point");
    if (kp.size() != 2) throw "--kernel-point must supply exactly 2 values for x, y";
    kernel_x = kp[0];
    kernel_y = kp[1];
  }

  const uint64_t n = cl.get_size("n-emissions");
  const int verbose = cl.count("verbose");
  const double scale = cl.get_double("scale");
  std::vector<jpet_strip_region> regions;
  for (const auto& fn : cl.rest()) {
    std::ifstream in(fn);
    if (!in) throw "cannot open phantom description " + fn;
    read_phantom(in, scale, regions);
  }
  if (cl.exist("point")) {
    auto pt = cl.get_doubles("point");
    if (pt.size() < 2 || pt.size() > 3) throw "--point must specifcy 2 or 3 values x,y[,intensity]";
    jpet_strip_region r{};
    r.kind = JPET_REGION_POINT;
    r.x = pt[0];
    r.y = pt[1];
    r.intensity = pt.size() == 3 ? pt[2] : 1.0;
    regions.push_back(r);
  }
  if (regions.empty()) throw "must specify at least one region";

  jpet_strip_geom g{};
  g.radius = cl.get_doubles("radius").at(0);
  g.scintillator_length = cl.get_double("length");
  g.n_z_pixels = cl.get_int("n-z-pixels");
  g.n_y_pixels = cl.get_int("n-y-pixels");
  g.pixel_width = g.pixel_height = cl.get_double("s-pixel");
  g.sigma_z = cl.get_double("s-z");
  g.sigma_dl = cl.get_double("s-dl");
  jpet_strip_gen_images im{};
  if (cl.exist("image-origin")) {
    auto o = cl.get_doubles("image-origin");
    if (o.size() != 2) throw "--image-origin must specify two values for x,y";
    im.origin_x = o[0];
    im.origin_y = o[1];
  }
  const size_t n_pix = static_cast<size_t>(g.n_z_pixels) * static_cast<size_t>(g.n_y_pixels);
  std::vector<int32_t> emitted(n_pix), det(n_pix), naive(n_pix), tan_map;
  im.emitted = emitted.data();
  im.detected = det.data();
  im.naive = naive.data();
  if (tan_bins > 0) {
    tan_map.resize(n_pix * static_cast<size_t>(tan_bins));
    im.tan_bins = tan_bins;
    im.tan_map = tan_map.data();
  }
  std::vector<float> ev(static_cast<size_t>(std::max<uint64_t>(n, 1)) * 3);
  const bool full = cl.exist("full") && !cl.exist("no-responses");
  std::vector<float> exact, events;
  if (full) {
    exact.resize(ev.size());
    events.resize(static_cast<size_t>(std::max<uint64_t>(n, 1)) * 4);
    im.exact_responses = exact.data();
    im.events = events.data();
  }
  int64_t written = 0;
  const int32_t flags = (cl.exist("detected") ? JPET_GEN_DETECTED : 0) |
                        (cl.exist("additive") ? JPET_GEN_ADDITIVE : 0);
  if (verbose) {
    std::cerr << "    image size: " << g.n_z_pixels << " x " << g.n_y_pixels << std::endl
              << "    pixel size: " << g.pixel_width << " x " << g.pixel_height << std::endl;
  }
  const int rc = jpet_strip_generate_host(&g, regions.data(), static_cast<int32_t>(regions.size()),
                                          static_cast<int64_t>(n), cl.get_size("seed"), flags,
                                          ev.data(), static_cast<int64_t>(n), &written, &im,
                                          cl.get_int("cuda-device"));
  if (rc != JPET_OK) throw std::string(jpet_strip_last_error(nullptr));
  if (verbose) {
    int64_t n_emit = 0;
    for (int32_t v : emitted) n_emit += v;
    std::cerr << " emitted: " << (flags & JPET_GEN_DETECTED ? n_emit : static_cast<int64_t>(n))
              << " events" << std::endl
              << "detected: " << written << " events" << std::endl;
  }

  const std::string output = cl.get_path("output");
  const std::string base = cmd::path_wo_ext(output), ext = cmd::path_ext(output);
  if (cl.exist("no-responses")) {
    // the reference writes no responses file (phantom_cmd.cpp:210-232)
  } else if (ext == ".txt") {
    std::ofstream o(output);
    for (int64_t i = 0; i < written; ++i)
      o << ev[3 * i] << ' ' << ev[3 * i + 1] << ' ' << ev[3 * i + 2] << '\n';
    if (!o) throw "cannot write " + output;
  } else {
    std::ofstream o(output, std::ios::binary);
    o.write(reinterpret_cast<const char*>(ev.data()), written * 3 * sizeof(float));
    if (!o) throw "cannot write " + output;
  }
  if (full) {
    // phantom_cmd.cpp:210-219,300-333: the same stream format as the responses;
    // FullResponse is the exact Response for the strip scanner (scanner.h:35,252-254)
    write_floats(base + "_wo_error" + ext, exact, written, 3, ext == ".txt");
    write_floats(base + "_full_response" + ext, exact, written, 3, ext == ".txt");
    write_floats(base + "_events" + ext, events, written, 4, ext == ".txt");
  }
  {
    std::ofstream cfg(base + ".cfg");
    cl.save(cfg);
  }
  write_image(base, "_detected", det, g.n_z_pixels, g.n_y_pixels);
  write_image(base, "_emitted", emitted, g.n_z_pixels, g.n_y_pixels);
  write_image(base, "_naive", naive, g.n_z_pixels, g.n_y_pixels);
  if (tan_bins > 0) {
    write_image(base, "_tan_bins", tan_map, g.n_z_pixels, g.n_y_pixels, tan_bins);
    if (verbose) std::cerr << "generating kernel map..." << std::endl;
    std::vector<float> kmap(n_pix * static_cast<size_t>(tan_bins));
    if (jpet_strip_tan_kernel_map(&g, tan_bins, kernel_x, kernel_y, im.origin_x, im.origin_y,
                                  (flags & JPET_GEN_DETECTED) ? 1 : 0, kmap.data(),
                                  cl.get_int("cuda-device")) != JPET_OK)
      throw std::string(jpet_strip_last_error(nullptr));
    write_image(base, "_tan_kernel", kmap, g.n_z_pixels, g.n_y_pixels, tan_bins);
  }
  return 0;
}

}  // namespace

int main(int argc, char* argv[]) {
  try {
    return run(argc, argv);
  } catch (const cmd::Error& ex) {
    std::cerr << "error: " << ex.what() << std::endl;
  } catch (const std::string& ex) {
    std::cerr << "error: " << ex << std::endl;
  } catch (const char* ex) {
    std::cerr << "error: " << ex << std::endl;
  } catch (const std::exception& ex) {
    std::cerr << "error: " << ex.what() << std::endl;
  }
  return 1;
}
