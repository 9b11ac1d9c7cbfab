// Declaration-only stand-in for the png++ header, which is not installed here. The reference's
// framebuffer header names png::image<png::rgb_pixel> in one member declaration; the test that
// compiles the drop-in adapter against the reference's CUDA platform headers needs the names,
// never an implementation. Test infrastructure, not part of the product.
#pragma once
namespace png {
struct rgb_pixel {
    unsigned char red, green, blue;
};
template <typename Pixel> class image;
}  // namespace png
