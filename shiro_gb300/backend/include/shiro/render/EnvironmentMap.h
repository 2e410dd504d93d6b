// Interface stand-in for shiro/render/EnvironmentMap.h: the accessors the GPU
// adapter reads (decoded pixels, size, layout).  FromPixels exists only in
// this stand-in, for tests that have no image loader.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "shiro/render/Renderer.h"
#include "shiro/render/Types.h"

namespace shiro::render {

class EnvironmentMap {
public:
    static std::shared_ptr<EnvironmentMap> FromPixels(uint32_t width, uint32_t height, std::vector<Vec3f> pixels,
                                                      EnvironmentMapLayout layout) {
        auto env = std::shared_ptr<EnvironmentMap>(new EnvironmentMap());
        env->width_ = width;
        env->height_ = height;
        env->layout_ = layout == EnvironmentMapLayout::Automatic ? EnvironmentMapLayout::LatLong : layout;
        env->pixels_ = std::move(pixels);
        return env;
    }

    uint32_t Width() const { return width_; }
    uint32_t Height() const { return height_; }
    EnvironmentMapLayout Layout() const { return layout_; }
    const std::vector<Vec3f>& Pixels() const { return pixels_; }

private:
    EnvironmentMap() = default;
    uint32_t width_ = 0;
    uint32_t height_ = 0;
    EnvironmentMapLayout layout_ = EnvironmentMapLayout::Automatic;
    std::vector<Vec3f> pixels_;
};

}  // namespace shiro::render
