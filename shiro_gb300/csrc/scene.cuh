// scene.cuh - device-resident scene snapshot.
//
// Layout in HBM (all arrays owned by the context, built by
// shiro_gpu_upload_scene):
//   nodes      BVH2 nodes, 64 B each (4 x float4): both children's boxes plus
//              child links; a negative link is a leaf ~((first << 3) | (n-1))
//   tris       3 x float4 per triangle in leaf order: (v0, gid), (e1, 0),
//              (e2, 0) with e1 = p1 - p0, e2 = p2 - p0 exactly as the
//              reference's Moller-Trumbore test forms them
//   triVerts   per global triangle: global vertex indices + mesh index
//   normals    per global vertex, float4 (xyz, 0); meshes without normals
//              fall back to the geometric normal (meshHasNormals = 0)
//   materials  ShiroMaterialDesc, the PbrMaterial fields verbatim
//   envs       per dome texture: texels (rgb, pixel probability mass),
//              row / conditional CDFs, alias table, and per texel the result
//              of sampling it (centre direction, pdf, radiance there)
//   emissive   the emissive triangles in mesh / primitive order with the
//              float running sums of their selection weights (area x
//              luminance), as BuildAccelerationScene forms them
#pragma once

#include "../../include/shiro_gpu.h"
#include "common.cuh"

namespace shiro_gpu {

struct DevEnv {
    const float4* texels;   // (r, g, b, rowMass * columnMass)
    const float* rowCdf;    // h + 1
    const float* condCdf;   // h * (w + 1)
    const uint2* alias;     // (acceptance threshold bits, alias index), w * h
    const float4* samples;  // 2 per texel: (centre direction, pdf), (radiance at the centre, 0)
    uint32_t w, h;
    uint32_t latlong;       // 1: lat-long, 0: angular
    uint32_t hasTable;      // importance table present (lat-long, non-empty)
};

struct DevDome {
    V3 radiance, right, up, forward;
    int32_t env;  // index into envs, -1: constant dome
    uint32_t pad;
};

struct DevDistant {
    V3 direction, radiance;
};

// Shading record of a triangle (make_surface): everything a hit needs past
// the intersection, indexed by global triangle, so the hit's normal and
// material come from one 64-byte record instead of triangle -> vertex
// indices -> normals / mesh -> material chains.  The material index is the
// mesh's (mapped to the default material when out of range); bit 31 says
// the mesh carries vertex normals.
constexpr int kShadeRec = 4;
constexpr uint32_t kShadeNormals = 0x80000000u;

struct DevScene {
    const float4* nodes;
    const float4* nodes8;           // 8-wide quantised BVH (bvh_build.h); NULL: traverse the binary BVH
    const float4* tris;
    const uint4* triVerts;
    const float4* positions;
    const float4* shade;            // kShadeRec per global triangle: (unit geometric normal, material | kShadeNormals),
                                    // then its three vertex normals (zero when the mesh has none)
    const ShiroMaterialDesc* materials;
    const float4* bsdfRecs;         // kBsdfRec per material: the BSDF's material-only quantities (bsdf.cuh)
    const DevDistant* distant;
    const DevDome* domes;
    const DevEnv* envs;
    uint32_t* error;                // device error word (kErr* bits)
    uint32_t nodeCount;
    uint32_t triCount;
    uint32_t distantCount;
    uint32_t domeCount;
    V3 envTop, envBottom;
    V3 boundsLo, boundsHi;          // box of all triangles (queue binning by ray origin)
    uint32_t rootIsLeaf;            // scene of <= 8 triangles: node 0 holds them all
    uint32_t emissiveCount;         // emissive triangles (AccelerationScene::emissiveTriangles)
    const float4* emissive;         // 3 per emissive triangle: (area, selection weight, running sum, gid bits),
                                    // (radiance, 0), (unit geometric normal, 0)
    const float* emissiveCdf;       // running sums of the selection weights
    const int32_t* emissiveOf;      // per global triangle: its emissive entry or -1
    float emissiveSum;
    uint32_t extended;              // some material uses transmission, opacity or emission
};

// Per-request constants.
struct DevRequest {
    V3 camPos, camForward, camRight, camUp;
    float tanHalfFov;   // std::tan(fov * 0.5 * pi / 180) evaluated on the host
    float aspect;
    uint32_t width, height;
    uint32_t sampleStart, sampleCount;
    uint32_t maxDepth, diffuseDepth, specularDepth;
    uint32_t domeSamples;        // max(1, domeLightSamples)
    uint32_t backgroundVisible;
    uint32_t flags;              // SHIRO_RENDER_*
};

}  // namespace shiro_gpu
