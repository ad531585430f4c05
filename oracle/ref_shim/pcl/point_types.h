/* Minimal stand-in for PCL's point types: just enough for the reference's
 * octree, entropy and slice-IO sources to compile (test oracle only). */
#pragma once
#include <cmath>
#include <cstdint>
namespace pcl {
struct PointXYZ {
    float x, y, z;
    PointXYZ() : x(0.f), y(0.f), z(0.f) {}
    PointXYZ(float a, float b, float c) : x(a), y(b), z(c) {}
};
struct PointXYZRGB {
    float x, y, z;
    uint8_t r, g, b, a;
    PointXYZRGB() : x(0.f), y(0.f), z(0.f), r(0), g(0), b(0), a(255) {}
};
struct Normal {
    float normal_x, normal_y, normal_z, curvature;
};
struct PointNormal {
    float x, y, z, normal_x, normal_y, normal_z, curvature;
};
struct PointXYZRGBNormal {
    float x, y, z;
    uint8_t r, g, b, a;
    float normal_x, normal_y, normal_z, curvature;
};
}  // namespace pcl
