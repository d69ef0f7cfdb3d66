// Host-side mirror of the reference's strip reconstruction classes on the C ABI.
#include "jpet_strip_host.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>

namespace PET2D {
namespace Strip {

namespace {

void check(int rc, const jpet_strip_t* h, const char* what) {
  if (rc != JPET_OK)
    throw std::string(what) + ": " + jpet_strip_last_error(h);
}

}  // namespace

// ---- Response / Scanner --------------------------------------------------------

template <typename F>
void Response<F>::calculate_tan_y_z(F R, F& tan, F& y, F& z) const {
  tan = (z_u - z_d) / (2 * R);
  y = -F(0.5) * (dl / std::sqrt(1 + tan * tan));
  z = F(0.5) * (z_u + z_d + (2 * y * tan));
}

template <typename F, typename S>
Scanner<F, S>::Scanner(F radius, F scintillator_length, S n_y_pixels, S n_z_pixels,
                       F pixel_height, F pixel_width, F sigma_z, F sigma_dl, F center_y,
                       F center_z)
    : radius(radius),
      scintillator_length(scintillator_length),
      n_y_pixels(n_y_pixels),
      n_z_pixels(n_z_pixels),
      total_n_pixels(static_cast<int>(n_y_pixels) * n_z_pixels),
      pixel_width(pixel_width),
      pixel_height(pixel_height),
      sigma_z(sigma_z),
      sigma_dl(sigma_dl),
      center_y(center_y),
      center_z(center_z),
      size_y(n_y_pixels * pixel_height),
      size_z(n_z_pixels * pixel_width),
      tl_y(center_y + size_y / 2),
      tl_z(center_z - size_z / 2),
      tl_y_half_h(tl_y - pixel_height / 2),
      tl_z_half_w(tl_z + pixel_width / 2),
      half_scintillator_length(scintillator_length / 2) {}

template <typename F, typename S>
typename Scanner<F, S>::Point Scanner<F, S>::pixel_center(Pixel p) const {
  return Point(tl_z_half_w + p.x * pixel_width, tl_y_half_h - p.y * pixel_height);
}

template <typename F, typename S>
typename Scanner<F, S>::Pixel Scanner<F, S>::pixel_at(Point p) const {
  return Pixel(static_cast<S>((p.x - tl_z) / pixel_width),
               static_cast<S>((tl_y - p.y) / pixel_height));
}

template <typename F, typename S>
F Scanner<F, S>::sensitivity(Point p) const {
  F L_plus = half_scintillator_length + p.x;
  F L_minus = half_scintillator_length - p.x;
  F R_plus = radius + p.y;
  F R_minus = radius - p.y;
  if (R_plus <= 0) R_plus = 1;
  if (R_minus <= 0) R_minus = 1;
  F a = std::min(L_minus / R_minus, L_plus / R_plus);
  F b = std::max(-L_plus / R_minus, -L_minus / R_plus);
  return F(M_1_PI) * (std::atan(a) - std::atan(b));
}

template <typename F, typename S>
F Scanner<F, S>::pixel_sensitivity(Pixel p) const {
  Point c = pixel_center(p);
  F hw = pixel_width / 2, hh = pixel_height / 2;
  return sensitivity(c) / 3 + sensitivity(Point(c.x + hw, c.y + hh)) / 6 +
         sensitivity(Point(c.x - hw, c.y - hh)) / 6 + sensitivity(Point(c.x - hw, c.y + hh)) / 6 +
         sensitivity(Point(c.x + hw, c.y - hh)) / 6;
}

template <typename F, typename S>
jpet_strip_geom Scanner<F, S>::geom() const {
  jpet_strip_geom g;
  g.radius = radius;
  g.scintillator_length = scintillator_length;
  g.n_y_pixels = n_y_pixels;
  g.n_z_pixels = n_z_pixels;
  g.pixel_height = pixel_height;
  g.pixel_width = pixel_width;
  g.sigma_z = sigma_z;
  g.sigma_dl = sigma_dl;
  return g;
}

template struct Response<float>;
template class Scanner<float, short>;

// ---- text parsing --------------------------------------------------------------
//
// util::text_parser (src/util/text_parser.h:19-176) parses a float as
//   whole + fraction * 10^-n_fraction_digits, then scales by the exponent,
// with every power of ten built by repeated multiplication in float and
// integer parts accumulated in int.  That arithmetic is restated here so that a
// text event file yields exactly the reference's float values; this includes
// the reference's scaling of positive exponents by 10 * 10^-(e-1).

namespace {

float pow10_negative_f(int e) {
  static float cache[300] = {1.0f};
  if (e < 0 || e >= 300) return 0.0f;
  float res = cache[e];
  if (!res) {
    res = 0.1f * pow10_negative_f(e - 1);
    cache[e] = res;
  }
  return res;
}

float pow10_positive_f(int e) {
  static float cache[300] = {1.0f};
  if (e < 0 || e >= 300) return 0.0f;
  float res = cache[e];
  if (!res) {
    res = 10.0f * pow10_negative_f(e - 1);
    cache[e] = res;
  }
  return res;
}

int parse_integer(const char*& p, int& n_digits) {
  n_digits = 0;
  uint32_t sum = 0;  // the reference accumulates in int; wraps identically
  while (*p >= '0' && *p <= '9') {
    sum = sum * 10u + static_cast<uint32_t>(*p - '0');
    ++p;
    ++n_digits;
  }
  return static_cast<int>(sum);
}

int parse_sign(const char*& p) {
  if (*p == '-') {
    ++p;
    return -1;
  }
  if (*p == '+') ++p;
  return 1;
}

}  // namespace

float parse_fp_float(const char*& p) {
  while (*p == ' ') ++p;
  int n_whole;
  int sign = parse_sign(p);
  int whole = parse_integer(p, n_whole);
  float val = static_cast<float>(whole);
  if (*p == '.') {
    ++p;
    int n_frac = 0;
    int frac = parse_integer(p, n_frac);
    if (n_whole == 0 && n_frac == 0) throw "period with no digits either before or after";
    if (n_frac > 0) val += frac * pow10_negative_f(n_frac);
  } else if (n_whole == 0) {
    throw "neither whole part nor period";
  }
  if (*p == 'e' || *p == 'E') {
    ++p;
    int n_exp;
    int ex = parse_sign(p);
    ex *= parse_integer(p, n_exp);
    if (n_exp == 0) throw "found exponent char but no exponent";
    if (ex > 300 || ex < -300) throw "exponent out of range";
    if (ex > 0) val *= pow10_positive_f(ex);
    if (ex < 0) val *= pow10_negative_f(-ex);
  }
  return val * sign;
}

namespace {

int parse_signed_int(const char*& p) {
  while (*p == ' ') ++p;
  int n;
  int s = parse_sign(p);
  return s * parse_integer(p, n);
}

// util::text_parser::read_lines: every '\n'-terminated line; a final line
// without '\n' is not delivered (text_parser.h:29-71).
template <typename Fn>
void read_lines(const char* fn, Fn&& got_line) {
  std::ifstream in(fn, std::ios::binary);
  if (!in) throw std::string("cannot open input file: ") + fn;
  std::string buf((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  size_t start = 0;
  for (;;) {
    size_t nl = buf.find('\n', start);
    if (nl == std::string::npos) break;
    buf[nl] = 0;
    got_line(buf.c_str() + start);
    start = nl + 1;
  }
}

}  // namespace

void read_binary_responses(const std::string& fn, std::vector<Response<float>>& out) {
  std::ifstream in(fn, std::ios::binary);
  if (!in.is_open()) throw std::string("cannot open phantom responses: ") + fn;
  float t[3];
  while (in.read(reinterpret_cast<char*>(t), sizeof(t))) out.emplace_back(t[0], t[1], t[2]);
}

void write_binary_image(const std::string& fn, const float* data, int n) {
  std::ofstream o(fn, std::ios::binary);
  if (!o) throw std::string("cannot create output file: ") + fn;
  o.write(reinterpret_cast<const char*>(data), static_cast<std::streamsize>(n) * sizeof(float));
}

void write_text_image(const std::string& fn, const float* data, int width, int height) {
  std::ofstream o(fn);
  if (!o) throw std::string("cannot create output file: ") + fn;
  const int n = width * height;
  for (int c = 1; c <= n; ++c) {
    o << data[c - 1];
    o << ((c % width == 0) ? "\n" : " ");
  }
}

void write_nrrd(const std::string& fn, const std::string& raw_fn, int width, int height,
                bool textual) {
  std::ofstream o(fn);
  o << "NRRD0001" << std::endl
    << "type: float" << std::endl
    << "endian: little" << std::endl
    << "dimension: 2" << std::endl
    << "sizes: " << width << " " << height << std::endl
    << "data file: ./" << raw_fn << std::endl
    << "encoding: " << (textual ? "ascii" : "raw") << std::endl;
}

void read_image(const std::string& fn, float* data, int n, bool text, bool is_int) {
  if (text) {
    std::ifstream in(fn);
    if (!in) throw std::string("cannot open ") + fn;
    for (int i = 0; i < n && (in >> data[i]); ++i) {
    }
    return;
  }
  std::ifstream in(fn, std::ios::binary);
  if (!in) throw std::string("cannot open ") + fn;
  if (is_int) {
    // integer maps get +1000 (reconstruction_cmd.cpp:154-160)
    std::vector<int32_t> tmp(n, 0);
    in.read(reinterpret_cast<char*>(tmp.data()), static_cast<std::streamsize>(n) * 4);
    for (int i = 0; i < n; ++i) data[i] = static_cast<float>(tmp[i] + 1000);
  } else {
    in.read(reinterpret_cast<char*>(data), static_cast<std::streamsize>(n) * 4);
  }
}

// ---- Reconstruction ------------------------------------------------------------

template <typename F>
Reconstruction<F>::Reconstruction(const Scanner& s, RunOptions o)
    : scanner(s),
      rho(s.n_z_pixels, s.n_y_pixels, F(1)),
      sensitivity(s.n_z_pixels, s.n_y_pixels, F(0)) {
  jpet_strip_geom g = scanner.geom();
  jpet_strip_opts opts;
  jpet_strip_default_opts(&opts);
  opts.device = o.device;
  opts.mode = o.mode;
  opts.variant = o.variant;
  opts.precision = o.precision;
  check(jpet_strip_create(&g, &opts, &handle_), nullptr, "jpet_strip_create");
  // point sensitivity at pixel centres (reconstruction.h:67-73)
  check(jpet_strip_get_sensitivity(handle_, 0, sensitivity.data), handle_, "sensitivity");
}

template <typename F>
Reconstruction<F>::~Reconstruction() {
  jpet_strip_destroy(handle_);
}

template <typename F>
Reconstruction<F>& Reconstruction<F>::operator<<(std::istream& in) {
  for (;;) {
    F t[3];
    in.read(reinterpret_cast<char*>(t), sizeof(t));
    if (!in) break;
    responses.emplace_back(t[0], t[1], t[2]);
  }
  return *this;
}

template <typename F>
void Reconstruction<F>::fast_load_txt_events(const char* fn, bool is_3d) {
  read_lines(fn, [&](const char* line) {
    const char* p = line;
    try {
      if (is_3d) {
        parse_signed_int(p);
        parse_signed_int(p);
      }
      F z_u = parse_fp_float(p);
      F z_d = parse_fp_float(p);
      F dl = parse_fp_float(p);
      responses.emplace_back(z_u, z_d, dl);
    } catch (const char* ex) {
      std::cerr << "error line: " << line << std::endl;
      throw;
    }
  });
}

template <typename F>
std::ostream& Reconstruction<F>::operator>>(std::ostream& out) {
  out.write(reinterpret_cast<const char*>(rho.data), static_cast<std::streamsize>(rho.size) * 4);
  return out;
}

template <typename F>
void Reconstruction<F>::output_tuples(std::ostream& out, bool output_sensitivity) {
  auto& o = output_sensitivity ? sensitivity : rho;
  for (int y = 0; y < scanner.n_y_pixels; ++y)
    for (int x = 0; x < scanner.n_z_pixels; ++x) {
      F v = o[y * scanner.n_z_pixels + x];
      if (v >= F(0.000000000001)) out << x << ' ' << y << ' ' << v << std::endl;
    }
}

template <typename F>
void Reconstruction<F>::upload() {
  if (uploaded_ != responses.size() || uploaded_ptr_ != responses.data()) {
    static_assert(sizeof(Response<F>) == 3 * sizeof(float), "Response layout");
    check(jpet_strip_set_events(handle_, reinterpret_cast<const float*>(responses.data()),
                                static_cast<int64_t>(responses.size())),
          handle_, "jpet_strip_set_events");
    uploaded_ = responses.size();
    uploaded_ptr_ = responses.data();
  }
  check(jpet_strip_set_image(handle_, rho.data), handle_, "jpet_strip_set_image");
}

template <typename F>
void Reconstruction<F>::iterate(int n) {
  check(jpet_strip_iterate(handle_, n), handle_, "jpet_strip_iterate");
}

template <typename F>
void Reconstruction<F>::download() {
  check(jpet_strip_get_image(handle_, rho.data), handle_, "jpet_strip_get_image");
}

template <typename F>
jpet_strip_counters Reconstruction<F>::counters() const {
  jpet_strip_counters c;
  check(jpet_strip_get_counters(handle_, &c), handle_, "jpet_strip_get_counters");
  return c;
}

template class Reconstruction<float>;

// ---- GPU::Reconstruction::run --------------------------------------------------

namespace GPU {
namespace Reconstruction {

namespace {
struct RunCallbacks {
  std::function<void(int, const Output&)>* output;
  std::function<void(int, bool)>* progress;
  Output* rho;
};

void output_tramp(int iteration, const float* image, int n_z, int n_y, void* user) {
  auto* cb = static_cast<RunCallbacks*>(user);
  if (!*cb->output) return;
  if (image == cb->rho->data) {
    (*cb->output)(iteration, *cb->rho);
  } else {
    Output view(static_cast<short>(n_z), static_cast<short>(n_y), const_cast<float*>(image));
    (*cb->output)(iteration, view);
  }
}

void progress_tramp(int completed, int finished, void* user) {
  auto* cb = static_cast<RunCallbacks*>(user);
  if (*cb->progress) (*cb->progress)(completed, finished != 0);
}
}  // namespace

template <typename F>
void run(Strip::Scanner<F, short>& scanner, Response<F>* responses, int n_responses,
         Output& rho_output, int n_iteration_blocks, int n_iterations_in_block,
         std::function<void(int, const Output&)> output, std::function<void(int, bool)> progress,
         int device, int n_blocks, int n_threads_per_block,
         std::function<void(const char*)> device_name, int mode) {
  (void)n_blocks;
  (void)n_threads_per_block;
  jpet_strip_geom g = scanner.geom();
  jpet_strip_opts opts;
  jpet_strip_default_opts(&opts);
  opts.device = device;
  opts.mode = mode;
  RunCallbacks cb{&output, &progress, &rho_output};
  char name[256] = {0};
  int rc = jpet_strip_run(&g, &opts, reinterpret_cast<const float*>(responses), n_responses,
                          rho_output.data, n_iteration_blocks, n_iterations_in_block,
                          output_tramp, progress_tramp, &cb, name, sizeof(name));
  if (rc != JPET_OK) throw std::string("GPU reconstruction: ") + jpet_strip_last_error(nullptr);
  if (device_name) device_name(name);
}

template void run<float>(Strip::Scanner<float, short>&, Response<float>*, int, Output&, int, int,
                         std::function<void(int, const Output&)>, std::function<void(int, bool)>,
                         int, int, int, std::function<void(const char*)>, int);

}  // namespace Reconstruction
}  // namespace GPU

}  // namespace Strip
}  // namespace PET2D
