// Test-only harness: the reference's own AnalyticKernel<F>::operator()
// (src/2d/strip/analytic_kernel.h:28-62) and Scanner<F, short>::pixel_sensitivity
// (src/2d/strip/scanner.h:174-185), the two pieces of the reference GPU path's
// semantics, instantiated at float and at double from the reference headers.
// The reference's own known answers for the analytic kernel are disabled
// (kernel_test.cpp:66-79), so these values are what pins the restatement.
//
// usage: ref_analytic cases.txt
//   cases.txt: "R L n_y n_z pixel_height pixel_width sigma_z sigma_dl", then a
//   count and that many lines "y tan sec dz dy" (kernel cases), then a count and
//   that many lines "px py" (pixels).
// Prints one line per kernel case, "float_value double_value", then one line
// per pixel, "float_sensitivity double_sensitivity" (%.9g / %.17g).
//
// Built by oracle/build_ref.sh from the reference sources without FP contraction
// (the source's evaluation order); never linked into the product.
#include <cstdio>
#include <fstream>
#include <vector>

#include "2d/strip/analytic_kernel.h"
#include "2d/strip/scanner.h"

template <typename F>
F kernel_value(F sigma_z, F sigma_dl, F y, F tan, F sec, F R, F dz, F dy) {
  PET2D::Strip::AnalyticKernel<F> k(sigma_z, sigma_dl);
  return k(y, tan, sec, R, PET2D::Vector<F>(dz, dy));
}

template <typename F>
F pixel_sensitivity(double R, double L, int n_y, int n_z, double ph, double pw, double sz,
                    double sdl, int px, int py) {
  const F fR = F(R), fL = F(L), fph = F(ph), fpw = F(pw), fsz = F(sz), fsdl = F(sdl);
  const short sy = short(n_y), sz_ = short(n_z);
  const PET2D::Strip::Scanner<F, short> s(fR, fL, sy, sz_, fph, fpw, fsz, fsdl);
  return s.pixel_sensitivity(PET2D::Pixel<short>(short(px), short(py)));
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s cases.txt\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  double R, L, ph, pw, sz, sdl;
  int n_y, n_z;
  if (!(in >> R >> L >> n_y >> n_z >> ph >> pw >> sz >> sdl)) return 3;
  int nk = 0;
  in >> nk;
  for (int i = 0; i < nk; ++i) {
    double y, t, sec, dz, dy;
    if (!(in >> y >> t >> sec >> dz >> dy)) return 3;
    const float vf = kernel_value<float>(float(sz), float(sdl), float(y), float(t), float(sec),
                                         float(R), float(dz), float(dy));
    const double vd = kernel_value<double>(sz, sdl, y, t, sec, R, dz, dy);
    std::printf("%.9g %.17g\n", double(vf), vd);
  }
  int np = 0;
  in >> np;
  for (int i = 0; i < np; ++i) {
    int px, py;
    if (!(in >> px >> py)) return 3;
    const float sf = pixel_sensitivity<float>(R, L, n_y, n_z, ph, pw, sz, sdl, px, py);
    const double sd = pixel_sensitivity<double>(R, L, n_y, n_z, ph, pw, sz, sdl, px, py);
    std::printf("%.9g %.17g\n", double(sf), sd);
  }
  return 0;
}
