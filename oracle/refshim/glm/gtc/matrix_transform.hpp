// Project-written stand-in (see glm/glm.hpp): translate and rotate of a 4x4
// column-major matrix, m * T and m * R with R the rotation by `angle` radians
// about the normalised axis (Rodrigues' formula).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../glm.hpp"

namespace glm {

inline mat4 translate(const mat4 &m, vec3 t) {
    mat4 r = m;
    r[3] = ((m[0] * t.x + m[1] * t.y) + m[2] * t.z) + m[3];
    return r;
}

inline mat4 rotate(const mat4 &m, float angle, vec3 axis) {
    const vec3 a = normalize(axis);
    const float c = std::cos(angle), s = std::sin(angle), k = 1.0f - c;
    // R's columns: R e_j = e_j cos + (a x e_j) sin + a (a . e_j)(1 - cos)
    const float R[3][3] = {{c + k * a.x * a.x, k * a.x * a.y + s * a.z, k * a.x * a.z - s * a.y},
                           {k * a.y * a.x - s * a.z, c + k * a.y * a.y, k * a.y * a.z + s * a.x},
                           {k * a.z * a.x + s * a.y, k * a.z * a.y - s * a.x, c + k * a.z * a.z}};
    mat4 r;
    for (int j = 0; j < 3; ++j) r[j] = (m[0] * R[j][0] + m[1] * R[j][1]) + m[2] * R[j][2];
    r[3] = m[3];
    return r;
}

} // namespace glm
