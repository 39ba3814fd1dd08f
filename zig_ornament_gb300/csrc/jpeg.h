// jpeg.h — sequential (baseline / extended Huffman) JPEG parsing and entropy
// decoding on the host (jpeg.cpp); the GPU stage (jpeg.cu) dequantises,
// inverse-transforms, upsamples and colour-converts the coefficient planes.
//
// This is the texture path of the reference's example app: textures are
// loaded with zstbi (stb_image) as 4-component images, flipped vertically
// (glfw_example/examples.zig:492-503 loadTexture; app_no_interop.zig:17
// setFlipVerticallyOnLoad(true)) and handed to Scene.createTexture
// (src/scene.zig:339-351).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace orn {
namespace jpeg {

constexpr int kMaxComponents = 3;

struct Component {
    uint32_t id = 0;
    uint32_t h = 1, v = 1;       // sampling factors
    uint32_t tq = 0;             // quantisation table
    uint32_t bw = 0, bh = 0;     // coefficient plane in 8x8 blocks (MCU-padded)
    bool decoded = false;
    std::vector<int16_t> coef;   // [bh][bw][64], natural (row-major) order, not dequantised
};

struct Image {
    uint32_t width = 0, height = 0, ncomp = 0;
    uint32_t hmax = 1, vmax = 1;
    uint32_t mcux = 0, mcuy = 0;
    bool ycbcr = true;           // false: the three components are R, G, B
    Component comp[kMaxComponents];
    uint16_t quant[4][64] = {};  // natural order
    bool quant_present[4] = {};
};

// Status codes are the library's ORN_* values.  With header_only the scan
// data is not decoded (width, height and components only).
int parse(const uint8_t* data, size_t len, bool header_only, Image* out, std::string* err);

// The calling thread's last error message of the orn_jpeg_* entry points.
std::string& last_error();

}  // namespace jpeg
}  // namespace orn
