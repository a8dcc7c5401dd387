// Stand-in for OSL/oslconfig.h, enough to compile kazen_proto's header-only
// vector and closure math (src/base/vec.h converts to and from OSL's Imath
// vector types). TEST INFRASTRUCTURE: used only to build the reference-code
// harness under oracle/_ref.
#pragma once

namespace OSL {
// Imath's vectors: named components, also indexable
struct Vec2 {
    float x = 0.f, y = 0.f;
    float operator[](unsigned long i) const { return i == 0 ? x : y; }
};
struct Vec3 {
    float x = 0.f, y = 0.f, z = 0.f;
    float operator[](unsigned long i) const { return i == 0 ? x : i == 1 ? y : z; }
};
}  // namespace OSL
