// Minimal OpenEXR writer for the thickness frames.
#pragma once

#include <string>
#include <vector>

namespace sb {

// Writes a single-part scanline EXR, no compression, three HALF channels
// B, G, R all equal to `img` (row-major, height rows of width pixels), the
// layout the reference writes through tinyexr (kernel/solver.cu:338-385).
bool write_exr_gray3(const char* path, int width, int height, const float* img);

// As write_exr_gray3 with three planes for the channels B, G and R (the
// velocity frames of Solver::write_velocity_image, kernel/solver.cu:388-497).
bool write_exr_bgr(const char* path, int width, int height, const float* b, const float* g,
                   const float* r);

// IEEE 754 binary32 -> binary16, round to nearest even.
unsigned short float_to_half(float f);

// binary16 -> binary32 (exact).
float half_to_float(unsigned short h);

// One channel of a single-part scanline EXR without compression (the
// layout of the reference's init/*.exr textures and of tinyexr's
// uncompressed output): HALF, FLOAT or UINT samples, as FP32, row-major
// over the data window.  Returns false with a message in `err` for other
// files (tiles, compression, a missing channel).
bool read_exr_channel(const char* path, const char* channel, int* width, int* height,
                      std::vector<float>& out, std::string& err);

// Bilinear resampling with half-pixel centres and clamped edges: the
// destination pixel x samples the source at (x + 0.5) sw / dw - 0.5 (the
// published definition of OpenCV's cv::resize with INTER_LINEAR on float
// images, which the reference applies to its textures).
void resize_linear(const float* src, int sw, int sh, float* dst, int dw, int dh);

}  // namespace sb
