// Project-written stand-in for the few glm types the reference's headers name
// (glm is an empty git submodule in the reference checkout). Only what is needed
// to parse the reference's CUDA sources for the device-code build is provided.
#pragma once
#include <cmath>
namespace glm
{
    struct vec3
    {
        float x = 0.f, y = 0.f, z = 0.f;
        vec3() = default;
        explicit vec3( float s ) : x( s ), y( s ), z( s ) {}
        vec3( float a, float b, float c ) : x( a ), y( b ), z( c ) {}
        template<class V> explicit vec3( const V & v ) : x( v.x ), y( v.y ), z( v.z ) {}
    };
    inline vec3 operator+( vec3 a, float s ) { return { a.x + s, a.y + s, a.z + s }; }
    inline vec3 operator-( vec3 a, float s ) { return { a.x - s, a.y - s, a.z - s }; }
    inline vec3 operator-( vec3 a, vec3 b ) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
    inline vec3 operator/( vec3 a, float s ) { return { a.x / s, a.y / s, a.z / s }; }
    inline vec3 abs( vec3 a ) { return { std::fabs( a.x ), std::fabs( a.y ), std::fabs( a.z ) }; }
    inline vec3 min( vec3 a, vec3 b ) { return { std::fmin( a.x, b.x ), std::fmin( a.y, b.y ), std::fmin( a.z, b.z ) }; }
    inline vec3 max( vec3 a, vec3 b ) { return { std::fmax( a.x, b.x ), std::fmax( a.y, b.y ), std::fmax( a.z, b.z ) }; }
} // namespace glm
