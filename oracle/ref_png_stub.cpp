// Test-only stand-in for the reference's util::png_writer (src/util/png_writer.h:10-63).
//
// The reference CPU tool writes a PNG preview of every image through libpng,
// which this machine does not have; with libpng absent the reference's own
// writer throws on every `-o` run (src/util/png_writer.cpp:43-46).  This file
// provides the same four members as a no-op so the reference tool links and
// writes its .bin/.nrrd images.  It is part of the oracle recipe only and is
// never linked into the product.
#include <string>

#include "util/png_writer.h"

namespace util {

png_writer::png_writer(std::string fn, double scale_max)
    : priv(nullptr), scale_max(scale_max) {
  (void)fn;
}

png_writer::~png_writer() {}

void png_writer::priv_write_header(unsigned int, unsigned int, unsigned int) {}

void png_writer::priv_write_row(unsigned char*) {}

}  // namespace util
