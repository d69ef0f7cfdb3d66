// 2d_strip_reconstruction: list-mode TOF MLEM reconstruction for the 2D strip
// scanner, with the options, input/output formats and output naming of the
// reference tool (src/2d/strip/reconstruction_cmd.cpp:105-301), running every
// iteration on the GPU through libjpet_strip.
//
//   without --gpu: the reference's CPU float semantics (GaussianKernel, no
//                  sensitivity), one output per iteration block;
//   with --gpu:    the reference GPU backend's semantics and output protocol
//                  (AnalyticKernel, sensitivity-weighted denominator, the
//                  <base>_sensitivity image and the intermediate iterations).
//
// PNG previews are not written: the reference writes them through libpng only.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "jpet_cmdline.hpp"
#include "jpet_strip_host.hpp"

using jpet::cmd::Kind;
using jpet::cmd::Parser;
namespace cmd = jpet::cmd;
using Reconstruction = PET2D::Strip::Reconstruction<float>;
using Scanner = PET2D::Strip::Scanner<float, short>;

namespace {

// Options of add_reconstruction_options (src/2d/strip/options.cpp:13-76,
// src/common/options.cpp:5-23) plus --rho / --rho-is-int.
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
  cl.add("n-emissions", 'e', "number of emissions", Kind::Size, cmd::kOptional, "0", true);
  cl.add_flag("verbose", 'v', "print progress information (-v) or benchmark (-vv)");
  cl.add("n-threads", 'T', "number of OpenMP threads", Kind::Int, cmd::kDontSave, "0");
  cl.footer("response ...\nbuild: GB300 (sm_103a)\n"
            "note: All length options below should be expressed in milimeters.");
  cl.add_flag("3d-response", 0, "input response contains additional LOR information");
  cl.add_flag("dl-is-time", 0, "delta is time, convert using speed of light");
  cl.add("speed-of-light", 0, "speed of light", Kind::Double, cmd::kOptional, "299792458.");
  cl.add("scale-length", 0, "scale input length values", Kind::Double, cmd::kOptional, "1.");
  cl.add("scale-time", 0, "scale input time values", Kind::Double, cmd::kOptional, "1.");
  cl.add("blocks", 'i', "number of iteration blocks", Kind::Int, cmd::kOptional, "0");
  cl.add("iterations", 'I', "number of iterations (per block)", Kind::Int, cmd::kOptional, "1");
  cl.add("output", 'o', "output files prefix (png)", Kind::Path, cmd::kOptional, "", true);
  cl.add("png-max", 0, "maximum value mapped to 255 in PNG", Kind::Double, cmd::kOptional, "0");
  cl.add_flag("gpu", 'G', "run on GPU (via CUDA)");
  cl.add("cuda-device", 'D', "CUDA device", Kind::Int, cmd::kDontSave, "0");
  cl.add("cuda-blocks", 'B', "CUDA blocks", Kind::Int, cmd::kDontSave, "64");
  cl.add("cuda-threads", 'W', "CUDA threads per block", Kind::Int, cmd::kDontSave, "512");
  cl.add("rho", 0, "start rho (eg. existing iteration)", Kind::Path, cmd::kOptional, "");
  cl.add_flag("rho-is-int", 0, "start rho uses integer representation (not float)");
  cl.add("kernel", 0,
         "GPU kernel variant: 0 fast (batch-union), 1 exact (reference operation order), "
         "2 warp per event, 3 row-owned",
         Kind::Int, cmd::kDontSave, "0");
  cl.add("precision", 0,
         "accumulation: 0 float, 1 compensated tiles, 2 compensated + FP64 denominators, "
         "3 fixed-point tiles",
         Kind::Int, cmd::kDontSave, "0");
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

// util::progress (src/util/progress.h:17-155): -v estimate line, -vv per
// iteration milliseconds and an average.
class Progress {
 public:
  Progress(int verbosity, size_t total) : verbosity_(verbosity), total_(total) {
    size_t reasonable = total / 1000;
    while (mask_ < reasonable && mask_ < 1) mask_ <<= 1;
    --mask_;
    if (verbosity_ >= 2) std::cout << "# it     time (ms)" << std::endl;
    start_ = clock::now();
  }
  void operator()(size_t completed, bool finished = false) {
    if (!(verbosity_ && ((completed == total_ - 1 && finished) || (completed & mask_) == 0)))
      return;
    if (verbosity_ >= 2) {
      if (!finished) {
        start_ = clock::now();
      } else {
        double ms = elapsed() * 1000;
        total_ms_ += ms;
        std::cout << std::fixed << std::setprecision(2) << std::setw(4) << (completed + 1) << ' '
                  << std::setw(10) << ms << std::endl;
        if (completed == total_ - 1)
          std::cout << "# av " << std::setw(10) << total_ms_ / total_ << "   total "
                    << total_ms_ << std::endl;
        std::cout.unsetf(std::ios::fixed);
        std::cout << std::setprecision(6);
      }
      return;
    }
    if (finished) {
      if (completed < total_ - 1) return;
      ++completed;
    }
    if (completed == last_) return;
    last_ = completed;
    std::cerr << ' ' << std::round(static_cast<double>(completed) / total_ * 100.0) << "% "
              << completed << "/" << total_;
    if (finished && completed == total_)
      std::cerr << std::endl;
    else
      std::cerr << "\r";
  }

 private:
  using clock = std::chrono::high_resolution_clock;
  double elapsed() const {
    return std::chrono::duration<double>(clock::now() - start_).count();
  }
  int verbosity_;
  size_t total_;
  size_t mask_ = 1;
  size_t last_ = static_cast<size_t>(-1);
  double total_ms_ = 0;
  clock::time_point start_;
};

void write_outputs(const std::string& fn, const std::string& ext, bool txt,
                   const PET2D::PixelMap<PET2D::Pixel<short>, float>& img) {
  if (txt) {
    PET2D::Strip::write_text_image(fn + ".txt", img.data, img.width, img.height);
  } else if (ext != ".png") {
    PET2D::Strip::write_binary_image(fn + ext, img.data, img.size);
  }
  PET2D::Strip::write_nrrd(fn + ".nrrd", cmd::path_wo_path(fn) + (txt ? ".txt" : ext), img.width,
                           img.height, txt);
}

int run(int argc, char* argv[]) {
  Parser cl;
  add_options(cl);
  cl.parse_check(argc, argv);
  calculate_scanner_options(cl);
  if (cl.rest().empty()) {
    if (argc == 1) {
      std::cerr << cl.usage();
      return 0;
    }
    throw "at least one responses input file expected, consult --help";
  }
  cl.load_accompanying_config();

  auto radius = cl.get_doubles("radius");
  Scanner scanner(static_cast<float>(radius.at(0)), static_cast<float>(cl.get_double("length")),
                  static_cast<short>(cl.get_int("n-y-pixels")),
                  static_cast<short>(cl.get_int("n-z-pixels")),
                  static_cast<float>(cl.get_double("s-pixel")),
                  static_cast<float>(cl.get_double("s-pixel")),
                  static_cast<float>(cl.get_double("s-z")),
                  static_cast<float>(cl.get_double("s-dl")));
  const bool gpu_semantics = cl.exist("gpu");
  PET2D::Strip::RunOptions ro;
  ro.device = cl.get_int("cuda-device");
  ro.mode = gpu_semantics ? JPET_MODE_GPU_REFERENCE : JPET_MODE_CPU_REFERENCE;
  ro.variant = cl.get_int("kernel");
  ro.precision = cl.get_int("precision");
  Reconstruction reconstruction(scanner, ro);

  const int verbose = cl.count("verbose");
  if (verbose)
    std::cout << "# image: " << scanner.n_y_pixels << "x" << scanner.n_z_pixels << std::endl;

  if (cl.exist("rho")) {
    std::string rho_name = cl.get_path("rho");
    PET2D::Strip::read_image(rho_name, reconstruction.rho.data, reconstruction.rho.size,
                             cmd::path_ext(rho_name) == ".txt", cl.exist("rho-is-int"));
  }

  const bool is_3d = cl.exist("3d-response");
  for (const auto& fn : cl.rest()) {
    if (cmd::path_ext(fn) == ".txt") {
      reconstruction.fast_load_txt_events(fn.c_str(), is_3d);
    } else {
      if (is_3d) throw "3D input must have .txt extension";
      PET2D::Strip::read_binary_responses(fn, reconstruction.responses);
    }
    if (verbose)
      std::cerr << "# read " << reconstruction.responses.size() << " responsess from " << fn
                << std::endl;
    // the reference rescales every response read so far after each file
    // (reconstruction_cmd.cpp:194-210)
    const bool dl_is_time = cl.exist("dl-is-time");
    if (cl.exist("scale-length")) {
      double scale = cl.get_double("scale-length");
      for (auto& r : reconstruction.responses) {
        r.z_u *= scale;
        r.z_d *= scale;
        if (!dl_is_time) r.dl *= scale;
      }
    }
    if (dl_is_time) {
      double scale = cl.get_double("scale-time");
      double c = cl.get_double("speed-of-light");
      for (auto& r : reconstruction.responses) r.dl = r.dl * c * scale;
    }
  }

  const int n_blocks = cl.get_int("blocks");
  const int n_in_block = cl.get_int("iterations");
  const int n_iterations = n_blocks * n_in_block;
  const std::string output_name = cl.get_path("output");
  const std::string base = cmd::path_wo_ext(output_name);
  const std::string ext = cmd::path_ext(output_name);
  const bool output_txt = ext == ".txt";
  Progress progress(verbose, static_cast<size_t>(n_iterations));

  if (gpu_semantics) {
    PET2D::Strip::GPU::Reconstruction::run<float>(
        scanner, reconstruction.responses.data(),
        static_cast<int>(reconstruction.responses.size()), reconstruction.rho, n_blocks,
        n_in_block,
        [&](int iteration, const PET2D::Strip::GPU::Reconstruction::Output& output) {
          if (!base.length()) return;
          std::string fn = iteration >= 0 ? cmd::path_add_index(base, iteration, n_iterations)
                                          : base + "_sensitivity";
          write_outputs(fn, ext, output_txt, output);
        },
        [&](int completed, bool finished) { progress(completed, finished); },
        cl.get_int("cuda-device"), cl.get_int("cuda-blocks"), cl.get_int("cuda-threads"),
        [=](const char* device_name) {
          if (verbose) std::cerr << "# device: " << device_name << std::endl;
        });
  } else {
    for (int block = 0; block < n_blocks; ++block) {
      reconstruction(progress, n_in_block, block * n_in_block);
      if (!base.length()) continue;
      std::string fn = cmd::path_add_index(base, (block + 1) * n_in_block, n_iterations);
      if (output_txt) {
        std::ofstream txt(fn + ".txt");
        txt.precision(12);
        txt << std::fixed;
        reconstruction.output_tuples(txt);
      } else if (ext != ".png") {
        PET2D::Strip::write_binary_image(fn + ext, reconstruction.rho.data,
                                         reconstruction.rho.size);
        PET2D::Strip::write_nrrd(fn + ".nrrd", cmd::path_wo_path(fn) + ext,
                                 reconstruction.rho.width, reconstruction.rho.height, false);
      }
    }
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
