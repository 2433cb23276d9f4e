// Device-code build of the reference's SES kernels (PlathC/SESDF), compiled from
// the reference's own sources where they lie (the include path is given by the
// recipe in oracle/Makefile). Nothing here restates the reference: this unit only
// pulls in its kernel translation units and instantiates the kernel templates the
// reference's host code launches, so that one sm_103a cubin holds them all.
//
// Kernels instantiated (reference file:line):
//   bcs::computeHashes, bcs::buildAccelerationGrid        sesdf/src/cuda/grid.cu:15-89
//   bcs::sesdf::findCirclesBetweenAtoms                   sesdf/src/sesdf/operations.cu:68-124
//   bcs::sesdf::computeCirclesVisibilityStatus            sesdf/src/sesdf/operations.cu:126-204
//   bcs::sesdf::fillIntersections                         sesdf/src/sesdf/operations.cu:206-269
//   bcs::sesdf::findIntersectionsNeighbors                sesdf/src/sesdf/operations.cu:271-338
//   bcs::sesdf::buildConvexPatchesSectors<128>            sesdf/include/bcs/sesdf/operations.inl:175-228
//   bcs::sesdf::findIntersectionsBetweenCircles<128>      sesdf/include/bcs/sesdf/operations.inl:230-486
//   bcs::sesdf::buildSegments<256,16>                     sesdf/include/bcs/sesdf/operations.inl:552-668
//   bcs::ssesdf::* (exterior twins)                       sesdf/src/ssesdf/operations.cu, sesdf/include/bcs/ssesdf/operation.inl
// The templates are instantiated for both capacities the reference builds (sesdf/CMakeLists.txt:96-117:
// the default library with 128 neighbour slots per atom, sesdf288 with 288).
#include "src/cuda/grid.cu"
#include "src/sesdf/operations.cu"
#include "src/ssesdf/operations.cu"

namespace bcs
{
    namespace sesdf
    {
        template __global__ void findIntersectionsBetweenCircles<128u>( SesdfContext, int4 * );
        template __global__ void buildConvexPatchesSectors<128u>( SesdfContext, const uint32_t * const, uint2 *, float4 * );
        template __global__ void findIntersectionsBetweenCircles<288u>( SesdfContext, int4 * );
        template __global__ void buildConvexPatchesSectors<288u>( SesdfContext, const uint32_t * const, uint2 *, float4 * );
        template __global__ void buildSegments<256, 16>( const SesdfContext,
                                                         const uint32_t,
                                                         const uint32_t *,
                                                         const float4 * const,
                                                         const int4 * const,
                                                         const uint32_t * const,
                                                         uint4 * );
    } // namespace sesdf
    namespace ssesdf
    {
        template __global__ void findIntersectionsBetweenCircles<128u>( SsesdfContext, int4 * );
        template __global__ void findIntersectionsBetweenCircles<288u>( SsesdfContext, int4 * );
    } // namespace ssesdf
} // namespace bcs
