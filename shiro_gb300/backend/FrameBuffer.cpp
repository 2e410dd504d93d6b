// FrameBuffer.cpp - implementation of the FrameBuffer stand-in (in the Shiro
// tree the application's own src/render/FrameBuffer.cpp provides it).
#include "shiro/render/FrameBuffer.h"

#include <algorithm>
#include <limits>

namespace shiro::render {

void FrameBuffer::Resize(uint32_t width, uint32_t height) {
    width_ = width;
    height_ = height;
    const size_t n = static_cast<size_t>(width) * height;
    beauty_.assign(n, Vec4f{});
    albedo_.assign(n, Vec3f{});
    normal_.assign(n, Vec3f{});
    depth_.assign(n, std::numeric_limits<float>::infinity());
}

void FrameBuffer::Clear() {
    std::fill(beauty_.begin(), beauty_.end(), Vec4f{});
    std::fill(albedo_.begin(), albedo_.end(), Vec3f{});
    std::fill(normal_.begin(), normal_.end(), Vec3f{});
    std::fill(depth_.begin(), depth_.end(), std::numeric_limits<float>::infinity());
}

void FrameBuffer::SetBeauty(uint32_t x, uint32_t y, const Vec4f& v) { beauty_[static_cast<size_t>(y) * width_ + x] = v; }
void FrameBuffer::SetAlbedo(uint32_t x, uint32_t y, const Vec3f& v) { albedo_[static_cast<size_t>(y) * width_ + x] = v; }
void FrameBuffer::SetNormal(uint32_t x, uint32_t y, const Vec3f& v) { normal_[static_cast<size_t>(y) * width_ + x] = v; }
void FrameBuffer::SetDepth(uint32_t x, uint32_t y, float v) { depth_[static_cast<size_t>(y) * width_ + x] = v; }

}  // namespace shiro::render
