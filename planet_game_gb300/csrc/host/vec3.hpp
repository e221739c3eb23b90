// Plain double-precision 3-vectors for the host-side mesh builder.
//
// The mesh must come out bit-identical to the reference builder
// (sim/planet/mesh/icosphere.cpp:200-419, sim/core/math/vec3d.hpp:8-52), so every
// operation here evaluates in the same order as the reference's: dot products as
// (x*x' + y*y') + z*z', normalisation as a per-component division by the
// length. This file is compiled with -ffp-contract=off so that no multiply-add
// is fused on either x86-64 or aarch64.
#pragma once

#include <cmath>
#include <stdexcept>

namespace psgb {

struct V3 {
    double x, y, z;
};

inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 unit(const V3& a) {
    const double m = std::sqrt(dot(a, a));
    if (!(m > 0.0) || !std::isfinite(m)) {
        throw std::invalid_argument("cannot normalise a zero or non-finite vector");
    }
    return {a.x / m, a.y / m, a.z / m};
}

}  // namespace psgb
