// Minimal OpenEXR writer for the thickness frames.
#pragma once

namespace sb {

// Writes a single-part scanline EXR, no compression, three HALF channels
// B, G, R all equal to `img` (row-major, height rows of width pixels), the
// layout the reference writes through tinyexr (kernel/solver.cu:338-385).
bool write_exr_gray3(const char* path, int width, int height, const float* img);

// IEEE 754 binary32 -> binary16, round to nearest even.
unsigned short float_to_half(float f);

}  // namespace sb
