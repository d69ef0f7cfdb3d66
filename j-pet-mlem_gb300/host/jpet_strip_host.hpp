// Host-side mirror of the reference's strip reconstruction interface, built on
// the C ABI (include/jpet_strip.h).  Same names, argument meaning and error
// behaviour as the reference's classes:
//
//   PET2D::Strip::Scanner<F, S>          src/2d/strip/scanner.h:26-291
//   PET2D::Strip::Response<F>            src/2d/strip/response.h:13-45
//   PET2D::PixelMap<Pixel, F> (images)   src/2d/geometry/pixel_map.h:15-162
//   PET2D::Strip::Reconstruction<F, K>   src/2d/strip/reconstruction.h:32-213
//   PET2D::Strip::GPU::Reconstruction::run<F>   src/2d/strip/cuda/reconstruction.h:32-44
//
// The iteration itself always runs on the GPU through the C ABI; a failing
// library call throws std::string, which the reference's CMDLINE_CATCH prints
// (src/util/cmdline_hooks.h:30-58).
#pragma once

#include <cstdint>
#include <functional>
#include <iosfwd>
#include <string>
#include <vector>

#include "jpet_strip.h"

namespace PET2D {

template <typename SType>
struct Pixel {
  using S = SType;
  S x, y;
  Pixel() = default;
  Pixel(S x, S y) : x(x), y(y) {}
  int index(S width) const { return static_cast<int>(y) * width + x; }
};

template <typename FType>
struct Point {
  FType x, y;
  Point() = default;
  Point(FType x, FType y) : x(x), y(y) {}
};

// Row-major image, index y * width + x (pixel_map.h:15-162).
template <typename PixelType, typename ValueType>
class PixelMap {
 public:
  using Pixel = PixelType;
  using S = typename Pixel::S;
  using Value = ValueType;
  PixelMap(S width, S height, Value v = Value())
      : width(width), height(height), size(static_cast<int>(width) * height),
        storage(static_cast<size_t>(size), v), data(storage.data()) {}
  // wraps caller-owned storage
  PixelMap(S width, S height, Value* ext)
      : width(width), height(height), size(static_cast<int>(width) * height), data(ext) {}
  PixelMap(const PixelMap& o)
      : width(o.width), height(o.height), size(o.size), storage(o.data, o.data + o.size),
        data(storage.data()) {}
  PixelMap& operator=(const PixelMap&) = delete;
  Value& operator[](int i) { return data[i]; }
  const Value& operator[](int i) const { return data[i]; }
  void assign(Value v) {
    for (int i = 0; i < size; ++i) data[i] = v;
  }
  Value* begin() { return data; }
  Value* end() { return data + size; }
  const Value* begin() const { return data; }
  const Value* end() const { return data + size; }

  const S width, height;
  const int size;

 private:
  std::vector<Value> storage;

 public:
  Value* const data;
};

namespace Strip {

// Strip response (response.h:13-45).
template <typename FType>
struct Response {
  using F = FType;
  F z_u, z_d, dl;
  Response() = default;
  Response(F z_u, F z_d, F dl) : z_u(z_u), z_d(z_d), dl(dl) {}
  void calculate_tan_y_z(F R, F& tan, F& y, F& z) const;
};

// Strip scanner (scanner.h:26-291): geometry as the reference stores it.
template <typename FType, typename SType>
class Scanner {
 public:
  using F = FType;
  using S = SType;
  using Pixel = PET2D::Pixel<S>;
  using Point = PET2D::Point<F>;
  Scanner(F radius, F scintillator_length, S n_y_pixels, S n_z_pixels, F pixel_height,
          F pixel_width, F sigma_z, F sigma_dl, F center_y = 0, F center_z = 0);

  Point pixel_center(Pixel p) const;
  Pixel pixel_at(Point p) const;
  F sensitivity(Point p) const;
  F pixel_sensitivity(Pixel p) const;
  jpet_strip_geom geom() const;

  const F radius, scintillator_length;
  const S n_y_pixels, n_z_pixels;
  const int total_n_pixels;
  const F pixel_width, pixel_height, sigma_z, sigma_dl, center_y, center_z;
  const F size_y, size_z, tl_y, tl_z, tl_y_half_h, tl_z_half_w;

 private:
  const F half_scintillator_length;
};

// Options of the GPU run that the reference passes as loose arguments.
struct RunOptions {
  int device = 0;
  int mode = JPET_MODE_CPU_REFERENCE;
  int variant = JPET_VARIANT_FAST;
  int precision = JPET_PRECISION_FP32;
};

// Reconstruction<F, GaussianKernel<F>> with the reference's members
// (reconstruction.h:32-213); the iterations run on the GPU.
template <typename FType>
class Reconstruction {
 public:
  using F = FType;
  using Scanner = Strip::Scanner<F, short>;
  using Pixel = typename Scanner::Pixel;
  using Output = PET2D::PixelMap<Pixel, F>;

  explicit Reconstruction(const Scanner& scanner, RunOptions opts = RunOptions());
  ~Reconstruction();
  Reconstruction(const Reconstruction&) = delete;
  Reconstruction& operator=(const Reconstruction&) = delete;

  // n_iterations of list-mode MLEM (reconstruction.h:108-154); the progress
  // callback is called as progress(iteration) and progress(iteration, true).
  template <typename ProgressCallback>
  void operator()(ProgressCallback& progress, int n_iterations, int n_iterations_so_far = 0) {
    upload();
    for (int it = 0; it < n_iterations; ++it) {
      progress(it + n_iterations_so_far);
      iterate(1);
      download();
      progress(it + n_iterations_so_far, true);
    }
  }

  // Binary responses: float triples until end of stream (reconstruction.h:156-167).
  Reconstruction& operator<<(std::istream& in);
  // Text responses, 3 values per line or `i j z_u z_d dl` (reconstruction.h:170-195),
  // parsed with the reference's text-parser arithmetic (util/text_parser.h).
  void fast_load_txt_events(const char* fn, bool is_3d = false);
  // Writes rho as binary floats (reconstruction.h:198-200).
  std::ostream& operator>>(std::ostream& out);
  // `x y value` lines for values >= 1e-12 (reconstruction.h:202-213).
  void output_tuples(std::ostream& out, bool output_sensitivity = false);

  // GPU handle operations used by operator() and the command-line tool
  void upload();            // responses -> device (once per change of responses)
  void iterate(int n);      // n iterations on the device
  void download();          // device image -> rho
  jpet_strip_counters counters() const;

  Scanner scanner;
  Output rho;
  Output sensitivity;
  std::vector<Response<F>> responses;

 private:
  jpet_strip_t* handle_ = nullptr;
  size_t uploaded_ = static_cast<size_t>(-1);
  const void* uploaded_ptr_ = nullptr;
};

namespace GPU {
namespace Reconstruction {

using Pixel = PET2D::Pixel<short>;
using Output = PET2D::PixelMap<Pixel, float>;

// The reference GPU entry point (cuda/reconstruction.h:32-44) with its callback
// protocol (cuda/reconstruction.cu:54-112).  `n_blocks` and
// `n_threads_per_block` are accepted for compatibility; the launch shape is
// chosen by the library.  Runs the reference GPU kernel's semantics
// (AnalyticKernel, sensitivity-weighted denominator).
template <typename F>
void run(Strip::Scanner<F, short>& scanner, Response<F>* responses, int n_responses,
         Output& rho_output, int n_iteration_blocks, int n_iterations_in_block,
         std::function<void(int iteration, const Output& output)> output,
         std::function<void(int completed, bool finished)> progress, int device, int n_blocks,
         int n_threads_per_block, std::function<void(const char* device_name)> device_name,
         int mode = JPET_MODE_GPU_REFERENCE);

}  // namespace Reconstruction
}  // namespace GPU

// ---- IO in the reference's formats ---------------------------------------------

// Parses one float as util::text_parser::parse_fp<float> does (text_parser.h:116-160).
float parse_fp_float(const char*& p);
// Reads float32 triples; a trailing partial triple is dropped.
void read_binary_responses(const std::string& fn, std::vector<Response<float>>& out);
void write_binary_image(const std::string& fn, const float* data, int n);
// PixelMap text output: values separated by ' ', one row per line (pixel_map.h:134-147).
void write_text_image(const std::string& fn, const float* data, int width, int height);
// NRRD header (src/util/nrrd_writer.h:18-27).
void write_nrrd(const std::string& fn, const std::string& raw_fn, int width, int height,
                bool textual);
// Reads an image (binary floats, or text values) into data[n].
void read_image(const std::string& fn, float* data, int n, bool text, bool is_int);

}  // namespace Strip
}  // namespace PET2D
