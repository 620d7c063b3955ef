// soapBubble CLI: ./soapBubble config.txt (kernel/main.cu:4-56).
#include <cstdio>
#include <exception>

#include "../../include/soapbubble_bubble.hpp"

int main(int argc, char** argv) {
    if (argc != 2) {
        std::printf("Please provide the path to config.txt as an argument.\n");
        std::printf("Usage example: ./soapBubble ../config.txt\n");
        std::printf("Configuration file was missing, exiting.\n");
        return -1;
    }
    try {
        BubbleConfig c = read_bubble_config(argv[1]);
        Bubble bubble(c.params.radius, c.params.H, c.params.U, c.params.c_m, c.params.Gamma_m,
                      c.params.T, c.params.Ds, c.params.rm, (size_t)c.params.nTheta, c.params.dt,
                      c.params.DT, c.params.frames, c.outputDir, c.thicknessImage,
                      c.params.device, c.AMGconfig, c.params.blendCoeff);
        bubble.run();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "soapBubble: %s\n", e.what());
        return 1;
    }
    return 0;
}
