// Project-written stand-in for glm::vec4 (see vec3.hpp).
#pragma once
#include "vec3.hpp"
namespace glm
{
    struct vec4
    {
        float x = 0.f, y = 0.f, z = 0.f, w = 0.f;
        vec4() = default;
        vec4( float a, float b, float c, float d ) : x( a ), y( b ), z( c ), w( d ) {}
    };
} // namespace glm
