// Test-only harness: the reference's own 3D hybrid reconstruction,
// PET3D::Hybrid::Reconstruction<Scanner, PET2D::Strip::GaussianKernel<float>>
// (src/3d/hybrid/reconstruction.h), instantiated from the reference headers and
// driven the way 3d_hybrid_reconstruction drives it
// (src/3d/hybrid/reconstruction_cmd.cpp:340-358, 462-541): calculate_weight
// (unless the weights are given, as with --system, one matrix per plane half
// for a multi-plane geometry), the external 3D sensitivity (--sensitivity),
// set_sensitivity_to_one (--sens-to-one) or calculate_sensitivity,
// normalize_geometry_weights, the responses read through operator<<
// (translate_to_frame and the bounding-box filter), then operator() once per
// iteration.
//
// The scanner is a harness class exposing the three things Reconstruction
// reads from it (sigma_z(), sigma_dl(), length) and the Response type of
// src/3d/hybrid/scanner.h:71-87; the geometry is a GeometrySOA filled from the
// case file, which stands in for the barrel system matrix or geometry file.
//
// usage: ref_hybrid case.txt out.bin
//   case.txt (text):
//     n_detectors n_pixel_infos n_columns n_rows n_planes
//     pixel_size lower_left_x lower_left_y z_left sigma_z sigma_dl length
//     weights_given sens_to_one n_iterations [n_planes_half sens_given_3d]
//     n_lors lines: 12 LineSegment fields (start, end, mid_point, direction,
//                   normal, length, distance_from_origin), width, begin, end
//     n_pixel_infos lines: x y position weight (n_planes_half weights: plane 0, 1, ...)
//     with sens_given_3d: the sensitivity, (n_planes_half > 1 ? n_planes_half :
//                   n_planes / 2) * n_rows * n_columns values, x fastest
//     n_responses, then that many lines: first second z_up z_dn dl
//   out.bin (little-endian):
//     int64 n_events, then per event the FrameEvent fields
//       int16 first, second; float up, right, tan, sec; uint64 begin, end;
//       int16 plane_begin, plane_end
//     float32 normalized weights [n_planes_half * n_pixel_infos]
//     float32 sensitivity [depth * n_columns * n_rows]
//     per iteration: float32 rho [n_voxels], int64 used_events, used_pixels,
//       used_voxels
//
// Built by oracle/build_ref.sh without OpenMP (one event thread, so the
// summation order is the event order) and without FP contraction (the source's
// evaluation order); never linked into the product.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <vector>

#include "2d/barrel/lor.h"
#include "2d/strip/gaussian_kernel.h"
#include "3d/hybrid/reconstruction.h"

struct HarnessScanner {
  using F = float;
  using S = short;
  struct Response {
    PET2D::Barrel::LOR<S> lor;
    F z_up, z_dn, dl;
    Response() = default;
    Response(std::istream& in)
        : lor(in), z_up(util::read<F>(in)), z_dn(util::read<F>(in)), dl(util::read<F>(in)) {}
  };
  F sigma_z_, sigma_dl_, length;
  F sigma_z() const { return sigma_z_; }
  F sigma_dl() const { return sigma_dl_; }
};

using Kernel = PET2D::Strip::GaussianKernel<float>;
using Rec = PET3D::Hybrid::Reconstruction<HarnessScanner, Kernel>;

template <typename T> static void put(std::FILE* f, T v) { std::fwrite(&v, sizeof v, 1, f); }

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s case.txt out.bin\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  int n_detectors, n_columns, n_rows, n_planes, weights_given, sens_to_one, n_iterations;
  long long n_infos;
  float pixel_size, llx, lly, z_left, sigma_z, sigma_dl, length;
  if (!(in >> n_detectors >> n_infos >> n_columns >> n_rows >> n_planes)) return 3;
  if (!(in >> pixel_size >> llx >> lly >> z_left >> sigma_z >> sigma_dl >> length)) return 3;
  if (!(in >> weights_given >> sens_to_one >> n_iterations)) return 3;
  int n_planes_half = 1, sens_given_3d = 0;
  {
    std::string rest;
    std::getline(in, rest);
    std::istringstream rs(rest);
    if (rs >> n_planes_half) rs >> sens_given_3d;
    if (n_planes_half < 1) n_planes_half = 1;
  }

  using Geometry = Rec::Geometry;
  Geometry geometry((short)n_detectors, (size_t)n_infos, (size_t)n_planes_half);
  for (size_t l = 0; l < geometry.n_lors; ++l) {
    float v[12], width;
    unsigned long long b, e;
    for (float& x : v)
      if (!(in >> x)) return 3;
    if (!(in >> width >> b >> e)) return 3;
    auto& s = geometry.lor_line_segments[l];
    s.start = PET2D::Point<float>(v[0], v[1]);
    s.end = PET2D::Point<float>(v[2], v[3]);
    s.mid_point = PET2D::Point<float>(v[4], v[5]);
    s.direction = PET2D::Vector<float>(v[6], v[7]);
    s.normal = PET2D::Vector<float>(v[8], v[9]);
    s.length = v[10];
    s.distance_from_origin = v[11];
    geometry.lor_widths[l] = width;
    geometry.lor_pixel_info_begin[l] = (size_t)b;
    geometry.lor_pixel_info_end[l] = (size_t)e;
  }
  for (long long i = 0; i < n_infos; ++i) {
    int x, y;
    float pos;
    if (!(in >> x >> y >> pos)) return 3;
    geometry.pixels[i] = PET2D::Pixel<short>((short)x, (short)y);
    geometry.pixel_positions[i] = pos;
    for (int plane = 0; plane < n_planes_half; ++plane) {
      float w;
      if (!(in >> w)) return 3;
      geometry.pixel_weights[i + n_infos * plane] = w;
    }
  }

  HarnessScanner scanner{sigma_z, sigma_dl, length};
  Rec::PixelGrid pixel_grid((short)n_columns, (short)n_rows, pixel_size,
                            PET2D::Point<float>(llx, lly));
  Rec::Grid grid(pixel_grid, z_left, (short)n_planes);
  Rec rec(scanner, grid, geometry, sens_given_3d != 0);
  if (!weights_given) rec.calculate_weight();
  const size_t n_sens = (size_t)rec.sensitivity.width * rec.sensitivity.height *
                        rec.sensitivity.depth;
  if (sens_given_3d) {
    for (size_t i = 0; i < n_sens; ++i)
      if (!(in >> rec.sensitivity.data[i])) return 3;
  } else if (sens_to_one) {
    rec.set_sensitivity_to_one();
  } else {
    rec.calculate_sensitivity();
  }
  rec.normalize_geometry_weights();

  long long n_responses;
  if (!(in >> n_responses)) return 3;
  std::stringstream responses;
  std::string line;
  std::getline(in, line);
  for (long long i = 0; i < n_responses; ++i) {
    if (!std::getline(in, line)) return 3;
    responses << line << '\n';
  }
  rec << responses;

  std::FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 4;
  put<int64_t>(out, rec.n_events());
  for (const auto& e : rec.events()) {
    put<int16_t>(out, e.lor.first);
    put<int16_t>(out, e.lor.second);
    put<float>(out, e.up);
    put<float>(out, e.right);
    put<float>(out, e.tan);
    put<float>(out, e.sec);
    put<uint64_t>(out, e.pixel_info_begin);
    put<uint64_t>(out, e.pixel_info_end);
    put<int16_t>(out, e.plane_begin);
    put<int16_t>(out, e.plane_end);
  }
  std::fwrite(geometry.pixel_weights, sizeof(float), (size_t)n_infos * n_planes_half, out);
  std::fwrite(rec.sensitivity.data, sizeof(float), n_sens, out);
  for (int it = 0; it < n_iterations; ++it) {
    rec();
    std::fwrite(rec.rho.data, sizeof(float), (size_t)grid.n_voxels, out);
    const auto& st = rec.statistics();
    put<int64_t>(out, (int64_t)st.used_events);
    put<int64_t>(out, (int64_t)st.used_pixels);
    put<int64_t>(out, (int64_t)st.used_voxels);
  }
  std::fclose(out);
  return 0;
}
