// bcs/core/math.hpp -- vector and box types of the drop-in API.
// Mirrors sesdf/include/bcs/core/math.hpp of the reference: Vec4f/Vec3f are glm
// vectors when glm is available, otherwise plain float structs with the same
// member names and layout (x, y, z[, w]).
#ifndef BCS_CORE_MATH_HPP
#define BCS_CORE_MATH_HPP

#include <cstddef>
#include <cstdint>

#if defined( __has_include )
#if __has_include( <glm/vec4.hpp> ) && !defined( SESGB_NO_GLM )
#define SESGB_HAVE_GLM 1
#include <glm/vec3.hpp>
#include <glm/vec4.hpp>
#endif
#endif

namespace bcs
{
    constexpr float Pif    = 3.141592654f;
    constexpr float TwoPif = 6.283185307f;

#ifdef SESGB_HAVE_GLM
    using Vec4f = glm::vec4;
    using Vec3f = glm::vec3;
#else
    struct Vec3f
    {
        float x = 0.f, y = 0.f, z = 0.f;
        Vec3f() = default;
        Vec3f( float a, float b, float c ) : x( a ), y( b ), z( c ) {}
        explicit Vec3f( float s ) : x( s ), y( s ), z( s ) {}
    };
    struct Vec4f
    {
        float x = 0.f, y = 0.f, z = 0.f, w = 0.f;
        Vec4f() = default;
        Vec4f( float a, float b, float c, float d ) : x( a ), y( b ), z( c ), w( d ) {}
    };
#endif
    static_assert( sizeof( Vec4f ) == 16, "atoms are float4 (x, y, z, vdW radius)" );

    struct Aabb
    {
        Vec3f min;
        Vec3f max;
    };

    // nextPowerOfTwoValue / nextPowerOfTwoExponent (sesdf/include/bcs/core/math.inl:5-19)
    constexpr std::size_t nextPowerOfTwoValue( const std::size_t baseNumber ) noexcept
    {
        std::size_t i = 1;
        while ( baseNumber > i )
            i <<= 1;
        return i;
    }
    constexpr std::size_t nextPowerOfTwoExponent( std::size_t baseNumber ) noexcept
    {
        std::size_t exponent = 0;
        while ( baseNumber >>= 1 )
            exponent++;
        return exponent;
    }
} // namespace bcs

#endif // BCS_CORE_MATH_HPP
