// 3d_tool_convert: converts detector-hit lists of real or simulated J-PET data
// into the list-mode responses "d1 d2 z_u z_d dl" that 2d_strip_reconstruction
// reads with --3d-response.  Options and behaviour of the reference tool
// (src/3d/tool/convert_cmd.cpp:53-211, src/3d/tool/options.cpp:32-65): the
// barrel scanner options and their defaults (src/2d/barrel/options.cpp:16-49,
// 225-348), the ring of square detectors (src/2d/barrel/scanner_builder.h:
// 35-220, square_detector.h:18-25) and the point-in-detector test
// (src/2d/geometry/polygon.h:70-83), all in float as the reference builds them.
//
//   --warsaw (default)  "x1 y1 z1 t1 x2 y2 z2 t2 ... scatter" per line, positions
//                       in cm, times in ps: the hits are assigned to detectors,
//                       z and dl get Gaussian smearing (std::mt19937_64 seeded
//                       by --seed, std::normal_distribution, the reference's
//                       draw order), hits with |z| > length / 2 are dropped
//   --tbednarski        "du dd t_ul t_ur t_dl t_dr" per line (1-based detectors,
//                       times in ps): z from the left/right time differences at
//                       the scintillator's light speed, dl at the speed of light;
//                       --relative-time prints the times relative to their minimum
//
// Host code only (text in, text out on stdout); the detector shape is always a
// square, as in the reference tool.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "jpet_cmdline.hpp"

using jpet::cmd::Kind;
using jpet::cmd::Parser;
namespace cmd = jpet::cmd;

namespace {

using F = float;
constexpr int kMaxDetectors = 400;  // the reference build's MAX_DETECTORS
const double kCm = 0.01;
const double kLightMPerPs = 299792458.0e-12;
const double kScintLightMPerPs = 126000000.0e-12;

struct Point {
  F x, y;
};
using Detector = std::array<Point, 4>;

// Point::rotate (src/2d/geometry/point.h:65-73)
Point rotated(Point p, F phi) {
  const F s = std::sin(phi), c = std::cos(phi);
  return Point{p.x * c - p.y * s, p.x * s + p.y * c};
}

// Polygon::contains (src/2d/geometry/polygon.h:70-83): p lies on the inner
// side of every edge, within tol
bool contains(const Detector& d, Point p, F tol) {
  Point start = d[3];
  for (int i = 0; i < 4; ++i) {
    const Point end = d[i];
    const F ex = end.x - start.x, ey = end.y - start.y;
    // edge.cw_perpendicular() = (ey, -ex)
    if (ey * (p.x - start.x) + -ex * (p.y - start.y) < -tol) return false;
    start = end;
  }
  return true;
}

// ScannerBuilder::build_single_ring (scanner_builder.h:35-92) for square detectors
std::vector<Detector> single_ring(F radius, int n_detectors, F w, F h, F d) {
  if (n_detectors > kMaxDetectors) {
    std::stringstream ss;
    ss << "buld single ring: too many detectors: " << n_detectors;
    throw ss.str();
  }
  if (radius <= 0) throw "invalid radius";
  if (w > 0 && h == 0) h = w;  // SquareDetector::default_height_for_width
  if (w <= 0 || h <= 0) throw "invalid detector size";
  if (n_detectors > 4 && n_detectors % 4 != 0) throw "number of detectors must be multiple of 4";
  Detector base{Point{w / 2, h / 2}, Point{w / 2, -h / 2}, Point{-w / 2, -h / 2},
                Point{-w / 2, h / 2}};
  const F shift = radius + (d > 0 ? d : h) / 2;
  for (auto& p : base) p.y += shift;
  std::vector<Detector> ring;
  for (int n = 0; n < n_detectors; ++n) {
    Detector det = base;
    const F phi = 2 * F(M_PI) * n / n_detectors - F(M_PI_2);
    for (auto& p : det) p = rotated(p, phi);
    ring.push_back(det);
  }
  return ring;
}

// ScannerBuilder::build_multiple_rings (scanner_builder.h:94-220): geometry
// only (the symmetry descriptor plays no part in the conversion)
std::vector<Detector> multiple_rings(std::vector<F> radius, std::vector<F> rotation,
                                     std::vector<int> n_detectors, F w, F h, F d) {
  if (radius.empty()) throw "must specify at least one radius";
  if (n_detectors.empty()) throw "must specify at least one number of detectors";
  if (n_detectors.size() < rotation.size()) throw "too many rotation values";
  if (radius.size() < n_detectors.size() || radius.size() < rotation.size())
    throw "must specify all radiuses";
  for (size_t i = 0; i < radius.size(); ++i) {
    if (i && radius[i] < radius[i - 1]) throw "radiuses must be specified in incrementing order";
    if (i && n_detectors.size() == i) n_detectors.push_back(n_detectors[i - 1]);
    if (rotation.size() == i) rotation.push_back(0);
  }
  const F eps = std::numeric_limits<F>::epsilon();
  for (size_t i = 0; i < radius.size(); ++i)
    if (std::abs(rotation[i]) >= eps && std::abs(rotation[i] - F(0.5)) > eps)
      throw "broken symmetry";
  std::vector<Detector> all = single_ring(radius[0], n_detectors[0], w, h, d);
  for (size_t i = 1; i < radius.size(); ++i) {
    if (!radius[i]) break;
    if (!n_detectors[i]) n_detectors[i] = n_detectors[i - 1];
    if (n_detectors[i] + static_cast<int>(all.size()) > kMaxDetectors)
      throw "build multiple rings: too many detectors";
    auto ring = single_ring(radius[i], n_detectors[i], w, h, d);
    const F phi = 2 * F(M_PI) * rotation[i] / static_cast<F>(ring.size());
    for (auto& det : ring) {
      for (auto& p : det) p = rotated(p, phi);
      all.push_back(det);
    }
  }
  return all;
}

// add_convert_options (src/3d/tool/options.cpp:32-65) with add_config_option and
// add_scanner_options (src/2d/barrel/options.cpp:16-49)
void add_options(Parser& cl) {
  cl.footer("means");
  cl.add("config", 'c', "load config file", Kind::Path, cmd::kDontSave, "", false, true);
  cl.add("shape", 0, "detector shape (square, circle, triangle, hexagon)", Kind::Path,
         cmd::kOptional, "square");
  cl.add("w-detector", 'w', "detector width", Kind::Double, cmd::kOptional, "0");
  cl.add("h-detector", 'h', "detector height", Kind::Double, cmd::kOptional, "0");
  cl.add("d-detector", 0, "inscribe detector shape into circle of given diameter", Kind::Double,
         cmd::kOptional, "0");
  cl.add("radius", 'r', "inner detector ring radius(es)", Kind::Doubles, cmd::kOptional, "");
  cl.add("rotation", 0, "ring rotation(s) (0-1)", Kind::Doubles, cmd::kOptional, "");
  cl.add("n-detectors", 'd', "number of detectors in ring(s)", Kind::Doubles, cmd::kOptional, "");
  cl.add("fov-radius", 0, "field of view radius", Kind::Double, cmd::kOptional, "0");
  cl.add("s-dl", 0, "TOF sigma delta-l", Kind::Double, cmd::kAlwaysSave, "0.06");
  cl.add("s-z", 0, "TOF sigma along z axis", Kind::Double, cmd::kAlwaysSave, "0.015");
  cl.add("length", 'l', "scintillator length", Kind::Double, cmd::kOptional, "1");
  cl.add_flag("verbose", 'v', "prints the iterations information on std::out");
  cl.add("seed", 'S', "random number generator seed", Kind::Size, cmd::kDontSave, "0");
  cl.add_flag("warsaw", 0, "Warsaw data format");
  cl.add_flag("tbednarski", 0, "T.Bednarski data format");
  cl.add("only", 0, "limit event (scattering) type, eg. 1 for non-scattered", Kind::Int,
         cmd::kOptional, "0");
  cl.add_flag("relative-time", 0, "output relative time instead z_u, z_d, dl");
}

// calculate_scanner_options (src/2d/barrel/options.cpp:225-348) without the
// pixel and model parts
void calculate_scanner_options(Parser& cl, int argc) {
  if (!cl.exist("w-detector") && !cl.exist("d-detector") && !cl.exist("n-detectors")) {
    if (argc == 1) {
      std::cerr << cl.usage() << "requires one of following options specified:" << std::endl
                << "  --w-detector, --d-detector, --n-detectors" << std::endl;
      std::exit(0);
    }
    throw "need to specify either --w-detector, --d-detector, --n-detectors";
  }
  std::stringstream assumed;
  std::vector<double> radius = cl.get_doubles("radius");
  std::vector<double> n_det = cl.get_doubles("n-detectors");
  const double d_detector = cl.get_double("d-detector");
  const std::string shape = cl.get_path("shape");
  auto exact = [](double v) {
    std::ostringstream o;
    o.precision(17);
    o << v;
    return o.str();
  };
  if (radius.empty()) {
    radius.push_back(M_SQRT2);
    assumed << "--radius=" << radius[0] << std::endl;
    cl.set("radius", exact(radius[0]));
  }
  if (!cl.exist("fov-radius")) {
    const double fov = radius[0] / M_SQRT2;
    assumed << "--fov-radius=" << fov << std::endl;
  }
  if (!cl.exist("w-detector")) {
    double w = 0;
    if (!n_det.empty()) {
      w = 2 * M_PI * .9 * radius[0] / static_cast<int>(n_det[0]);
    } else if (cl.exist("d-detector")) {
      if (shape == "circle") {
        w = d_detector;
      } else {
        double mult = 1., sides = 0.;
        if (shape == "triangle") {
          sides = 3.;
        } else if (shape == "square") {
          sides = 4.;
        } else if (shape == "hexagon") {
          sides = 6.;
          mult = 2.;
        } else {
          throw "cannot determine detector width for given shape";
        }
        w = d_detector * std::sin(M_PI / sides) * mult;
      }
    }
    cl.set("w-detector", exact(w));
    assumed << "--w-detector=" << w << std::endl;
  }
  if (n_det.empty()) {
    const double w = cl.get_double("w-detector");
    int n;
    if (cl.exist("d-detector"))
      n = (static_cast<int>(std::floor(M_PI / std::atan2(d_detector, 2 * radius[0] + d_detector / 2))) /
           4) * 4;
    else
      n = (static_cast<int>(std::floor(M_PI / std::atan2(w, 2 * radius[0]))) / 4) * 4;
    cl.set("n-detectors", std::to_string(n));
    assumed << "--n-detectors=" << n << std::endl;
  }
  if (cl.exist("verbose") && assumed.str().size())
    std::cerr << "assumed:" << std::endl << assumed.str();
}

std::vector<Detector> build_scanner(const Parser& cl) {
  std::vector<F> radius, rotation;
  std::vector<int> n_det;
  for (double r : cl.get_doubles("radius")) radius.push_back(static_cast<F>(r));
  for (double r : cl.get_doubles("rotation")) rotation.push_back(static_cast<F>(r));
  for (double n : cl.get_doubles("n-detectors")) n_det.push_back(static_cast<int>(n));
  return multiple_rings(radius, rotation, n_det, static_cast<F>(cl.get_double("w-detector")),
                        static_cast<F>(cl.get_double("h-detector")),
                        static_cast<F>(cl.get_double("d-detector")));
}

// convert_warsaw (convert_cmd.cpp:86-158)
void convert_warsaw(const Parser& cl) {
  const F sigma_z = static_cast<F>(cl.get_double("s-z"));
  const F sigma_dl = static_cast<F>(cl.get_double("s-dl"));
  const F length = static_cast<F>(cl.get_double("length"));
  const int verbose = cl.count("verbose");
  std::normal_distribution<double> z_error(0, sigma_z);
  std::normal_distribution<double> dl_error(0, sigma_dl);
  std::mt19937_64 rng(static_cast<long>(cl.get_size("seed")));
  const std::vector<Detector> scanner = build_scanner(cl);
  const int only = cl.get_int("only");
  for (const auto& fn : cl.rest()) {
    std::ifstream in_means(fn);
    if (!in_means.is_open()) throw "cannot open input means file: " + fn;
    std::string line;
    size_t no_columns = 0;
    while (std::getline(in_means, line)) {
      // the column count of the first line (files differ in their middle
      // columns; the first 8 and the last are used)
      if (!no_columns) {
        std::stringstream in(line);
        std::string el;
        while (in >> el) ++no_columns;
        if (verbose) std::cerr << "reading " << no_columns << " column: " << fn << std::endl;
        if (!no_columns) break;
      }
      std::stringstream in(line);
      double x1, y1, z1, t1, x2, y2, z2, t2;
      int scatter;
      in >> x1 >> y1 >> z1 >> t1 >> x2 >> y2 >> z2 >> t2;
      for (size_t i = 0; i + 9 < no_columns; ++i) {
        std::string el;
        in >> el;
      }
      in >> scatter;
      if (std::abs(z1 * kCm) > length / 2 || std::abs(z2 * kCm) > length / 2) continue;
      if (only != 0 && only != scatter) continue;
      const Point p1{static_cast<F>(x1 * kCm), static_cast<F>(y1 * kCm)};
      const Point p2{static_cast<F>(x2 * kCm), static_cast<F>(y2 * kCm)};
      int d1 = -1, d2 = -1;
      for (size_t i = 0; i < scanner.size(); ++i) {
        if (contains(scanner[i], p1, F(0.0001))) d1 = static_cast<int>(i);
        if (contains(scanner[i], p2, F(0.0001))) d2 = static_cast<int>(i);
      }
      if (d1 >= 0 && d2 >= 0) {
        if (d1 < d2) {
          std::swap(d1, d2);
          std::swap(z1, z2);
          std::swap(t1, t2);
        }
        const double dl = (t1 - t2) * kLightMPerPs;
        // the reference's output expression draws z_u, z_d, dl in this order
        const double zu = z1 * kCm + z_error(rng);
        const double zd = z2 * kCm + z_error(rng);
        const double dle = dl + dl_error(rng);
        std::cout << d1 << " " << d2 << " " << zu << " " << zd << " " << dle << "\n";
      } else if (verbose) {
        std::cerr << "point (" << p1.x << ' ' << p1.y << ") or (" << p2.x << ' ' << p2.y
                  << ") outside detector - skiping\n";
      }
    }
  }
}

// convert_tbednarski (convert_cmd.cpp:160-211)
void convert_tbednarski(const Parser& cl) {
  const bool output_relative = cl.exist("relative-time");
  for (const auto& fn : cl.rest()) {
    std::ifstream in_means(fn);
    if (!in_means.is_open()) throw "cannot open input means file: " + fn;
    std::string line;
    while (std::getline(in_means, line)) {
      std::stringstream in(line);
      int du = 0, dd = 0;
      double tul = 0, tur = 0, tdl = 0, tdr = 0;
      in >> du >> dd >> tul >> tur >> tdl >> tdr;
      if (output_relative) {
        const double tmin = std::min(std::min(tur, tul), std::min(tdr, tdl));
        tul -= tmin;
        tur -= tmin;
        tdl -= tmin;
        tdr -= tmin;
        std::cout << du << ' ' << dd << ' ' << tul << ' ' << tur << ' ' << tdl << ' ' << tdr
                  << '\n';
        continue;
      }
      if (du < dd) {
        std::swap(du, dd);
        std::swap(tul, tdl);
        std::swap(tur, tdr);
      }
      du -= 1;
      dd -= 1;
      const double zu = 0.5 * kScintLightMPerPs * (tul - tur);
      const double zd = 0.5 * kScintLightMPerPs * (tdl - tdr);
      const double dl = 0.5 * kLightMPerPs * ((tul + tur) - (tdl + tdr));
      std::cout << du << ' ' << dd << ' ' << zu << ' ' << zd << ' ' << dl << '\n';
    }
  }
}

int run(int argc, char* argv[]) {
  Parser cl;
  add_options(cl);
  cl.parse_check(argc, argv);
  cl.load_accompanying_config(false);
  calculate_scanner_options(cl, argc);
  if (cl.exist("tbednarski") && !cl.exist("warsaw"))
    convert_tbednarski(cl);
  else
    convert_warsaw(cl);  // the reference falls back to the Warsaw format
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
