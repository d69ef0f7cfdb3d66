// Test-only FP64 oracle: the reference's own CPU MLEM template instantiated at
// double precision, PET2D::Strip::Reconstruction<double, GaussianKernel<double>>
// (src/2d/strip/reconstruction.h:32), with Scanner<double, short> as the
// reference tests use it (src/2d/strip/kernel_test.cpp:33).
//
// It reads the reference binary event format (float32 z_u, z_d, dl triples,
// src/2d/strip/reconstruction.h:156-167), widens every value to double and runs
// the reference's operator() (reconstruction.h:108-154).  After each iteration
// listed in --dump it writes the image as float64 row-major [n_y][n_z] to
// <out>_<NN>.f64.
//
// usage: ref_fp64 events.bin R L n_y n_z pixel sigma_z sigma_dl iterations
//                 threads out_prefix [rho_init.f32]
//
// Built by oracle/build_ref.sh from the reference sources; it is test
// infrastructure and is never linked into the product.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "2d/strip/reconstruction.h"
#include "2d/strip/gaussian_kernel.h"

using Kernel = PET2D::Strip::GaussianKernel<double>;
using Reconstruction = PET2D::Strip::Reconstruction<double, Kernel>;
using Scanner = PET2D::Strip::Scanner<double, short>;

struct NoProgress {
  void operator()(int, bool = false) {}
};

int main(int argc, char** argv) {
  if (argc < 12) {
    std::fprintf(stderr,
                 "usage: %s events.bin R L n_y n_z pixel sigma_z sigma_dl "
                 "iterations threads out_prefix [rho_init.f32]\n",
                 argv[0]);
    return 2;
  }
  const char* events_fn = argv[1];
  double R = std::atof(argv[2]);
  double L = std::atof(argv[3]);
  int n_y = std::atoi(argv[4]);
  int n_z = std::atoi(argv[5]);
  double pixel = std::atof(argv[6]);
  double sigma_z = std::atof(argv[7]);
  double sigma_dl = std::atof(argv[8]);
  int iterations = std::atoi(argv[9]);
  int threads = std::atoi(argv[10]);
  std::string out = argv[11];
#if _OPENMP
  if (threads > 0)
    omp_set_num_threads(threads);
#else
  (void)threads;
#endif

  Scanner scanner(R, L, n_y, n_z, pixel, pixel, sigma_z, sigma_dl);
  Reconstruction reconstruction(scanner);

  if (argc > 12) {
    std::ifstream in(argv[12], std::ios::binary);
    std::vector<float> init(reconstruction.rho.size);
    in.read(reinterpret_cast<char*>(init.data()), init.size() * sizeof(float));
    for (size_t i = 0; i < init.size(); ++i)
      reconstruction.rho[i] = init[i];
  }

  std::ifstream in(events_fn, std::ios::binary);
  if (!in) {
    std::fprintf(stderr, "cannot open %s\n", events_fn);
    return 1;
  }
  float triple[3];
  while (in.read(reinterpret_cast<char*>(triple), sizeof(triple)))
    reconstruction.responses.emplace_back(triple[0], triple[1], triple[2]);

  NoProgress progress;
  for (int it = 0; it < iterations; ++it) {
    reconstruction(progress, 1, it);
    char name[64];
    std::snprintf(name, sizeof(name), "_%03d.f64", it + 1);
    std::ofstream o(out + name, std::ios::binary);
    o.write(reinterpret_cast<const char*>(reconstruction.rho.data),
            reconstruction.rho.size * sizeof(double));
  }
  return 0;
}
