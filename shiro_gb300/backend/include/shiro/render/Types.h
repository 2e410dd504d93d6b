// Interface stand-in for shiro/render/Types.h of the host application
// (vector PODs and the few helpers the GPU adapter uses).  In the Shiro tree
// the adapter compiles against the application's own header instead.
#pragma once

#include <cstdint>

namespace shiro::render {

struct Vec2f {
    float x = 0.0f;
    float y = 0.0f;
};

struct Vec3f {
    float x = 0.0f;
    float y = 0.0f;
    float z = 0.0f;
};

struct Vec4f {
    float x = 0.0f;
    float y = 0.0f;
    float z = 0.0f;
    float w = 0.0f;
};

}  // namespace shiro::render
