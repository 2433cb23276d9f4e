// bcs/ssesdf/graphics.hpp -- output structs of the exterior-only build, field for
// field those of sesdf/include/bcs/ssesdf/graphics.hpp:10-50 of the reference.
#ifndef BCS_SSESDF_GRAPHICS_HPP
#define BCS_SSESDF_GRAPHICS_HPP

#include <cstdint>

#include <vector_types.h>

#include "bcs/core/type.hpp"

using GLuint = unsigned int;
namespace bcs::ssesdf
{
    struct SsesdfGraphics
    {
        uint32_t           atomNb = 0;
        HandleSpan<GLuint> atoms;

        uint32_t           circlePatchNb = 0;
        HandleSpan<GLuint> circlePosition;
        HandleSpan<GLuint> circleAxis;
        HandleSpan<GLuint> circleVs;

        uint32_t           concavePatchNb = 0;
        HandleSpan<GLuint> concavePatchesPosition;
        HandleSpan<GLuint> concavePatchesId;
        HandleSpan<GLuint> concavePatchesNeighbors;

        float    probeRadius         = 0.f;
        uint16_t maxConcaveNeighbors = 0;
    };

    struct SsesdfData
    {
        uint32_t atomNb = 0;
        float4 * atoms  = nullptr;

        uint32_t circlePatchNb  = 0;
        float4 * circlePosition = nullptr;
        float4 * circleAxis     = nullptr;
        float4 * circleVs       = nullptr;

        uint32_t concavePatchNb          = 0;
        float4 * concavePatchesPosition  = nullptr;
        int4 *   concavePatchesId        = nullptr;
        float4 * concavePatchesNeighbors = nullptr;

        float    probeRadius         = 0.f;
        uint16_t maxConcaveNeighbors = 0;
    };
} // namespace bcs::ssesdf

#endif // BCS_SSESDF_GRAPHICS_HPP
