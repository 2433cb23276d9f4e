// bcs/sesdf/graphics.hpp -- output structs of the full-surface build, field for
// field those of sesdf/include/bcs/sesdf/graphics.hpp:10-66 of the reference.
#ifndef BCS_SESDF_GRAPHICS_HPP
#define BCS_SESDF_GRAPHICS_HPP

#include <cstdint>

#include <vector_types.h>

#include "bcs/core/type.hpp"

using GLuint = unsigned int;
namespace bcs::sesdf
{
    // OpenGL buffer handles: no graphics stack is used by this build, so every
    // handle is 0; offsets and sizes are filled as in the reference.
    struct SesdfGraphics
    {
        uint32_t           atomNb = 0;
        HandleSpan<GLuint> atoms;

        uint32_t           convexPatchNb = 0;
        HandleSpan<GLuint> convexPatches;

        uint32_t           sectorNb = 0;
        HandleSpan<GLuint> sectors;

        uint32_t           segmentPatchNb = 0;
        HandleSpan<GLuint> segmentPatches;

        uint32_t           circlePatchNb = 0;
        HandleSpan<GLuint> circlePatches;

        uint32_t           concavePatchNb = 0;
        HandleSpan<GLuint> concavePatchesPosition;
        HandleSpan<GLuint> concavePatchesId;
        HandleSpan<GLuint> concavePatchesNeighbors;

        float    probeRadius         = 0.f;
        uint16_t maxConcaveNeighbors = 0;
    };

    struct SesdfData
    {
        uint32_t atomNb = 0;
        float4 * atoms  = nullptr;

        uint32_t convexPatchNb = 0;
        uint2 *  convexPatches = nullptr;

        uint32_t sectorNb = 0;
        float4 * sectors  = nullptr;

        uint32_t segmentPatchNb = 0;
        uint4 *  segmentPatches = nullptr;

        uint32_t circlePatchNb = 0;
        uint2 *  circlePatches = nullptr;

        uint32_t concavePatchNb          = 0;
        float4 * concavePatchesPosition  = nullptr;
        int4 *   concavePatchesId        = nullptr;
        float4 * concavePatchesNeighbors = nullptr;

        float    probeRadius         = 0.f;
        uint16_t maxConcaveNeighbors = 0;
    };
} // namespace bcs::sesdf

#endif // BCS_SESDF_GRAPHICS_HPP
