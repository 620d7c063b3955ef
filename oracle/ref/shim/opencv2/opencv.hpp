// Host execution shim of the OpenCV calls in the reference's texture
// initialisers (kernel/initializer.cu:50-135): cv::imread returns an image
// the test driver registered under that path (three float channels B, G, R),
// cv::resize only copies (the driver registers images at the grid's size).
#pragma once
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
namespace cv {
struct Size {
    int width, height;
    Size(int w = 0, int h = 0) : width(w), height(h) {}
};
template <class T>
struct Point3_ {
    T x, y, z;
};
enum { IMREAD_UNCHANGED = -1 };
class Mat {
  public:
    int rows = 0, cols = 0;
    std::vector<float> pix;  // rows x cols x 3 (B, G, R)
    unsigned char* data = nullptr;
    template <class T>
    T* ptr(int r, int c) {
        return reinterpret_cast<T*>(&pix[3 * ((size_t)r * cols + c)]);
    }
    void attach() { data = pix.empty() ? nullptr : reinterpret_cast<unsigned char*>(pix.data()); }
};
Mat imread(const std::string& path, int flags);
void resize(const Mat& in, Mat& out, Size size);
}  // namespace cv
