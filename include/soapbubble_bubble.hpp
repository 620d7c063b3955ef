// C++ drop-in for the reference's Bubble class (include/bubble.cuh:36-89):
// same constructor arguments (the 17 config.txt keys, kernel/main.cu:20-36)
// and run() (kernel/bubble.cu:2607-2704), implemented over the C ABI of
// soapbubble.h.  Errors throw std::runtime_error instead of exiting.
#pragma once

#include <cstddef>
#include <string>

#include "soapbubble.h"

class Bubble {
public:
    Bubble(double radius = 0.05, double H = 0.0000005, double U = 1.0, double c_m = 0.5,
           double Gamma_m = 0.000001, double T = 298.15, double Ds = 0.01,
           double rm = 0.000000005, size_t nTheta = 128, double dt = 0.005,
           double DT = 1.0 / 24.0, int frames = 1000,
           std::string outputDir = "../output/test/", std::string thicknessImage = "",
           int device = 0, std::string AMGconfig = "", double blendCoeff = 0.5);
    ~Bubble();
    Bubble(const Bubble&) = delete;
    Bubble& operator=(const Bubble&) = delete;

    /* Runs all frames, writing frameNNNN.exr into outputDir. */
    void run();

    sb_bubble* handle() { return handle_; }
    const sb_params& params() const { return params_; }

private:
    sb_params params_;
    std::string outputDir_, thicknessImage_, AMGconfig_;
    sb_bubble* handle_ = nullptr;
};

/* Reads the reference's positional config.txt (17 "key value" pairs in the
 * order of kernel/main.cu:20-36; key names are not checked, as there).
 * "null" for thicknessInit means no image. Throws on a short file. */
struct BubbleConfig {
    sb_params params;
    std::string outputDir, thicknessImage, AMGconfig;
};
BubbleConfig read_bubble_config(const std::string& path);
