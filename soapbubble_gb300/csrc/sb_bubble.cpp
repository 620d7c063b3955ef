// Bubble class and config.txt reader over the C ABI.
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <sys/stat.h>

#include "../../include/soapbubble_bubble.hpp"

namespace {

void check(int rc, const char* what) {
    if (rc != SB_OK) throw std::runtime_error(std::string(what) + ": " + sb_last_error());
}

}  // namespace

Bubble::Bubble(double radius, double H, double U, double c_m, double Gamma_m, double T,
               double Ds, double rm, size_t nTheta, double dt, double DT, int frames,
               std::string outputDir, std::string thicknessImage, int device,
               std::string AMGconfig, double blendCoeff)
    : outputDir_(std::move(outputDir)), thicknessImage_(std::move(thicknessImage)),
      AMGconfig_(std::move(AMGconfig)) {
    sb_default_params(&params_);
    params_.radius = radius;
    params_.H = H;
    params_.U = U;
    params_.c_m = c_m;
    params_.Gamma_m = Gamma_m;
    params_.T = T;
    params_.Ds = Ds;
    params_.rm = rm;
    params_.nTheta = (int)nTheta;
    params_.dt = dt;
    params_.DT = DT;
    params_.frames = frames;
    params_.device = device;
    params_.blendCoeff = blendCoeff;
    check(sb_create(&params_, &handle_), "sb_create");
}

Bubble::~Bubble() { sb_destroy(handle_); }

void Bubble::run() {
    // Bubble::run initialises from the textures first (kernel/bubble.cu:2640-2641);
    // like the reference, a missing texture leaves the defaults in place
    if (sb_init_thickness_from_exr(handle_, thicknessImage_.c_str()) != SB_OK)
        std::fprintf(stderr, "No thickness image provided, initialize with eta = 0.5 (%s)\n",
                     sb_last_error());
    if (sb_init_airflow_from_exr(handle_, "../init/velocityfield_512.exr") != SB_OK)
        std::fprintf(stderr, "No airflow image provided, initialize with zero (%s)\n",
                     sb_last_error());
    if (!outputDir_.empty()) {
        // create the output directory (one level), as the reference does
        mkdir(outputDir_.c_str(), 0755);
    }
    check(sb_run(handle_, outputDir_.empty() ? nullptr : outputDir_.c_str(), 0), "sb_run");
}

BubbleConfig read_bubble_config(const std::string& path) {
    std::ifstream fin(path);
    if (!fin) throw std::runtime_error("cannot open " + path);
    BubbleConfig c;
    sb_default_params(&c.params);
    std::string key;
    double r, H, U, c_m, Gm, T, Ds, rm, dt, DT, blend;
    size_t nTheta;
    int frames, device;
    std::string outputDir, thick, amg;
    fin >> key >> r >> key >> H >> key >> U >> key >> c_m >> key >> Gm >> key >> T >> key >> Ds >>
        key >> rm >> key >> nTheta >> key >> dt >> key >> DT >> key >> frames >> key >>
        outputDir >> key >> thick >> key >> amg >> key >> blend >> key >> device;
    if (!fin) throw std::runtime_error("config " + path + " is missing keys");
    if (thick == "null") thick = "";
    c.params.radius = r; c.params.H = H; c.params.U = U; c.params.c_m = c_m;
    c.params.Gamma_m = Gm; c.params.T = T; c.params.Ds = Ds; c.params.rm = rm;
    c.params.nTheta = (int)nTheta; c.params.dt = dt; c.params.DT = DT;
    c.params.frames = frames; c.params.blendCoeff = blend; c.params.device = device;
    c.outputDir = outputDir;
    c.thicknessImage = thick;
    c.AMGconfig = amg;
    return c;
}
