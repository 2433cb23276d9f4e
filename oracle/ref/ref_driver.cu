// ref_driver.cu -- TEST INFRASTRUCTURE ONLY (reference arm and parity pin).
//
// Runs the reference's own CUDA kernels (PlathC/SESDF), compiled from its
// sources into oracle/_ref/ref_kernels.cubin by oracle/Makefile, under a host
// driver that restates the reference's build orchestration:
//   bcs::Sesdf::build   sesdf/src/sesdf/sesdf.cu:172-264
//     findCircles       sesdf/include/bcs/sesdf/operations.inl:14-93
//     findIntersections sesdf/include/bcs/sesdf/operations.inl:106-173
//     buildConicPatches sesdf/include/bcs/sesdf/operations.inl:488-541
//     handleIntersectionSingularities sesdf/src/sesdf/operations.cu:14-32
//   bcs::Ssesdf::build  sesdf/src/ssesdf/ssesdf.cu:133-187 (+ ssesdf/operations.cu:25-75,
//                       ssesdf/operation.inl:28-98)
//   AccelerationGrid::build sesdf/src/cuda/grid.cu:99-132
// The reference's own host code cannot be built for the GPU host (its sources
// are not available there), so this file repeats its sequence of launches,
// library calls (thrust), stream-ordered allocations and blocking read-backs on
// the legacy default stream. Deviations, each needed to run it safely:
//   * launches with zero elements are skipped (KernelConfig::From divides by
//     zero for them, sesdf/include/bcs/cuda/setup.inl:21-25);
//   * the temporary intersection buffer is sized N*(slots per atom) instead of C1*2 and the
//     intersection buffer gets a tail of Q*16 bytes, so that the reference
//     kernels' unchecked writes stay inside allocations;
//   * the exterior status buffer is zeroed once at construction (the
//     reference leaves its j < i slots as whatever cudaMalloc returned).
// One harness serves both libraries the reference builds (128 and 288 neighbour
// slots per atom, sesdf/CMakeLists.txt:96-117): the capacity is chosen per build.
// The structs below mirror the reference's kernel parameter layouts
// (sesdf/include/bcs/cuda/grid.cuh:9-16, sesdf/include/bcs/sesdf/data.cuh:27-115,
// sesdf/include/bcs/ssesdf/data.cuh:27-92); their sizes are checked against the
// kernels' parameter info at load time.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cxxabi.h>
#include <thrust/copy.h>
#include <thrust/count.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/transform.h>
#include <thrust/transform_scan.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace
{
    struct GridInfoRef
    {
        float3 worldOrigin;
        float3 cellSize;
        int3   size;
    };

    struct alignas( 16 ) SesdfContextRef
    {
        float      probeRadius;
        uint32_t   atomNb;
        uint32_t * dIntersectedCircleNb;
        uint32_t * hIntersectedCircleNb;
        uint32_t * dIntersectionNb;
        uint32_t * hIntersectionNb;
        uint32_t * dFullCircleNb;
        uint32_t * hFullCircleNb;
        uint32_t * dSegmentCount;
        uint32_t * hSegmentCount;
        uint32_t * hVisibleCircleNb;
        uint32_t   maxNeighborPerAtom;
        uint32_t   maxIntersectionsPerCircles;
        uint32_t   maxIntersectionNeighbors;
        float4 *   atoms;
        uint32_t * sortedToInitialIndices;
        uint32_t   intersectionWithNeighborNb;
        uint32_t * neighborNb;
        uint32_t * neighborIds;
        uint8_t *  visibilityStatus;
        uint32_t * circlesIntersectionNb;
        uint32_t * circlesIntersectionStartId;
        uint32_t * circlesIntersectionIds;
        uint32_t * trimmedToGlobalId;
        uint32_t * globalToTrimmedId;
    };

    struct alignas( 16 ) SsesdfContextRef
    {
        float      probeRadius;
        uint32_t   atomNb;
        uint32_t * dIntersectionNb;
        uint32_t * hIntersectionNb;
        uint32_t * hVisibleCircleNb;
        uint32_t   intersectedCircleNb;
        uint32_t   maxNeighborPerAtom;
        uint32_t   maxIntersectionsPerCircles;
        uint32_t   maxIntersectionNeighbors;
        float4 *   atoms;
        uint32_t * sortedToInitialIndices;
        uint32_t   intersectionWithNeighborNb;
        uint32_t * neighborNb;
        uint32_t * neighborIds;
        uint8_t *  visibilityStatus;
    };

    // BCS_SESDF_MAXNEIGHBORPERATOM of the two libraries the reference builds (sesdf/CMakeLists.txt:96-117)
    constexpr uint32_t kMaxNbr       = 128;
    constexpr uint32_t kMaxNbr288    = 288;
    constexpr uint32_t kMaxIntNbr    = 32;
    constexpr uint32_t kMeanIntPerC  = 2;

    enum K
    {
        kHashes,
        kBuildGrid,
        kFindCircles,
        kVisibility,
        kSectors,
        kFindIntersections,
        kFillIntersections,
        kSegments,
        kIntNeighbors,
        kXFindCircles,
        kXVisibility,
        kXFindIntersections,
        kXFillIntersections,
        kXFillCircles,
        kXIntNeighbors,
        kSectors288,
        kFindIntersections288,
        kXFindIntersections288,
        kCount
    };

    // demangled-name prefixes of the reference kernels
    const char * kNames[ kCount ] = {
        "bcs::computeHashes(",
        "bcs::buildAccelerationGrid(",
        "bcs::sesdf::findCirclesBetweenAtoms(",
        "bcs::sesdf::computeCirclesVisibilityStatus(",
        "bcs::sesdf::buildConvexPatchesSectors<128u>(",
        "bcs::sesdf::findIntersectionsBetweenCircles<128u>(",
        "bcs::sesdf::fillIntersections(",
        "bcs::sesdf::buildSegments<(unsigned short)256, (unsigned short)16>(",
        "bcs::sesdf::findIntersectionsNeighbors(",
        "bcs::ssesdf::findCirclesBetweenAtoms(",
        "bcs::ssesdf::computeCirclesVisibilityStatus(",
        "bcs::ssesdf::findIntersectionsBetweenCircles<128u>(",
        "bcs::ssesdf::fillIntersections(",
        "bcs::ssesdf::fillCircles(",
        "bcs::ssesdf::findIntersectionsNeighbors(",
        "bcs::sesdf::buildConvexPatchesSectors<288u>(",
        "bcs::sesdf::findIntersectionsBetweenCircles<288u>(",
        "bcs::ssesdf::findIntersectionsBetweenCircles<288u>(",
    };

    CUlibrary  g_lib = nullptr;
    CUfunction g_fn[ kCount ] {};
    std::string g_err;

    bool check( CUresult r, const char * what )
    {
        if ( r == CUDA_SUCCESS )
            return true;
        const char * s = nullptr;
        cuGetErrorString( r, &s );
        g_err = std::string( what ) + ": " + ( s ? s : "?" );
        return false;
    }
    bool checkRt( cudaError_t r, const char * what )
    {
        if ( r == cudaSuccess )
            return true;
        g_err = std::string( what ) + ": " + cudaGetErrorString( r );
        return false;
    }

    // KernelConfig::From (sesdf/include/bcs/cuda/setup.inl:21-25)
    void kernelConfig( uint32_t n, uint32_t blockDim, uint32_t & grid, uint32_t & block )
    {
        block = std::min( blockDim, n );
        grid  = n / block + std::min( n / block, 1u );
    }

    template<class... Args> bool launch( K k, uint32_t grid, uint32_t block, uint32_t smem, const Args &... args )
    {
        if ( grid == 0 || block == 0 )
            return true;
        void * params[] = { const_cast<void *>( static_cast<const void *>( &args ) )... };
        return check( cuLaunchKernel( g_fn[ k ], grid, 1, 1, block, 1, 1, smem, nullptr, params, nullptr ), kNames[ k ] );
    }

    // stream-ordered device buffer on the legacy default stream (DeviceBuffer,
    // sesdf/src/cuda/memory.cu:108-143)
    struct DBuf
    {
        void * p    = nullptr;
        size_t size = 0;
        DBuf()      = default;
        explicit DBuf( size_t s, bool zero = false ) : size( s )
        {
            cudaMallocAsync( &p, s ? s : 1, 0 );
            if ( zero )
                cudaMemset( p, 0, s ? s : 1 );
        }
        DBuf( const DBuf & )             = delete;
        DBuf & operator=( const DBuf & ) = delete;
        DBuf( DBuf && o ) noexcept { std::swap( p, o.p ), std::swap( size, o.size ); }
        DBuf & operator=( DBuf && o ) noexcept
        {
            std::swap( p, o.p );
            std::swap( size, o.size );
            return *this;
        }
        ~DBuf()
        {
            if ( p )
                cudaFreeAsync( p, 0 );
        }
        template<class T> T * get( size_t byteOffset = 0 ) const { return reinterpret_cast<T *>( (char *)p + byteOffset ); }
    };

    template<class T> void d2h( T * dst, const T * src, size_t n ) { cudaMemcpy( dst, src, n * sizeof( T ), cudaMemcpyDeviceToHost ); }
    template<class T> void d2d( T * dst, const T * src, size_t n )
    {
        if ( n )
            cudaMemcpyAsync( dst, src, n * sizeof( T ), cudaMemcpyDeviceToDevice, 0 );
    }

    // functors of the reference's thrust calls (operations.inl:95-104, ssesdf/operation.inl:13-26)
    struct HasNeighborsComparator
    {
        __device__ bool operator()( const int4 a, const int4 b ) const { return abs( a.w ) > abs( b.w ); }
    };
    struct HasNeighbors
    {
        __device__ bool operator()( const int4 a ) const { return abs( a.w ) == 2; }
    };
    struct NonZeroU8
    {
        __host__ __device__ uint32_t operator()( uint8_t x ) const { return uint32_t( x != 0 ); }
    };
    struct IsCompleteU8
    {
        __host__ __device__ bool operator()( uint8_t x ) const { return x == 2; }
    };
    struct NonZeroU32
    {
        __host__ __device__ bool operator()( uint32_t x ) const { return x != 0; }
    };
    struct U8ToU32
    {
        __host__ __device__ uint32_t operator()( uint8_t c ) const { return static_cast<uint32_t>( c ); }
    };
    struct HalfU8
    {
        __host__ __device__ uint32_t operator()( uint8_t c ) const { return c / 2u; }
    };
    struct Identity
    {
        __host__ __device__ uint32_t operator()( uint32_t x ) const { return x; }
    };

    // AccelerationGrid (sesdf/src/cuda/grid.cu:91-132)
    struct Grid
    {
        GridInfoRef info {};
        uint32_t    cells = 0;
        DBuf        start, end, hashes, indices, sorted;
        size_t      capacity = 0;

        void init( GridInfoRef g )
        {
            info  = g;
            cells = (uint32_t)( g.size.x * g.size.y * g.size.z );
            start = DBuf( sizeof( uint32_t ) * cells );
            end   = DBuf( sizeof( uint32_t ) * cells );
        }
        bool build( uint32_t n, const float4 * positions )
        {
            cudaMemset( start.p, 0xff, sizeof( uint32_t ) * cells );
            if ( capacity < n )
            {
                hashes   = DBuf( sizeof( uint32_t ) * n );
                indices  = DBuf( sizeof( uint32_t ) * n );
                sorted   = DBuf( sizeof( float4 ) * n );
                capacity = n;
            }
            if ( n == 0 )
                return true;
            uint32_t g, b;
            kernelConfig( n, 256, g, b );
            uint32_t * h  = hashes.get<uint32_t>();
            uint32_t * ix = indices.get<uint32_t>();
            if ( !launch( kHashes, g, b, 0, info, n, positions, h, ix ) )
                return false;
            thrust::sort_by_key( thrust::device, h, h + n, ix );
            uint32_t * cs = start.get<uint32_t>();
            uint32_t * ce = end.get<uint32_t>();
            float4 *   sp = sorted.get<float4>();
            return launch( kBuildGrid, g, b, sizeof( uint32_t ) * ( b + 1 ), n, h, ix, positions, cs, ce, sp );
        }
    };

    struct Ref
    {
        int            mode = 0; // 0 full, 1 exterior
        uint32_t       maxNbr = kMaxNbr; // neighbour slots per atom: 128 or 288 (the library the kernels come from)
        const float *  hostAtoms = nullptr;
        uint32_t       n  = 0;
        float          rp = 1.4f;
        GridInfoRef    gridInfo {};
        Grid           grid;

        // counters (pinned host + device)
        uint32_t *dIntersectedCircleNb = nullptr, *dIntersectionNb = nullptr, *dFullCircleNb = nullptr,
                 *dSegmentCount = nullptr;
        uint32_t *hIntersectedCircleNb = nullptr, *hIntersectionNb = nullptr, *hFullCircleNb = nullptr,
                 *hSegmentCount = nullptr, *hVisibleCircleNb = nullptr;

        // preallocated (ctor)
        DBuf atoms, atomIndices, nbrCount, nbrIds, status, globalToTrimmed, convexPatches;

        // per build results
        DBuf     fCircleAndSectors, trimmedToGlobal, intersections, segments, circles, startAndIds, circleIntCount;
        uint32_t convexPatchNb = 0, fullCircleNb = 0, sectorNb = 0, intersectionNb = 0, intersectionWithNbr = 0,
                 segmentNb = 0, circleNb = 0, trimmedNb = 0, visibleNb = 0;
    };

    // Sesdf::Sesdf / Ssesdf::Ssesdf (sesdf/src/sesdf/sesdf.cu:20-75; sesdf/src/ssesdf/ssesdf.cu:19-66)
    void construct( Ref * r, const float * aabb )
    {
        const float maxVdw = 3.48f;
        float       origin[ 3 ], size[ 3 ];
        for ( int a = 0; a < 3; a++ )
        {
            origin[ a ] = ( aabb[ a ] - maxVdw ) - r->rp;
            size[ a ]   = std::fabs( ( ( aabb[ 3 + a ] + maxVdw ) + r->rp ) - origin[ a ] );
        }
        uint64_t e = 0, v = r->n;
        while ( v >>= 1 )
            e++;
        uint32_t gs = 1;
        while ( e > gs )
            gs <<= 1;
        r->gridInfo.worldOrigin = make_float3( origin[ 0 ], origin[ 1 ], origin[ 2 ] );
        r->gridInfo.cellSize    = make_float3( size[ 0 ] / (float)gs, size[ 1 ] / (float)gs, size[ 2 ] / (float)gs );
        r->gridInfo.size        = make_int3( (int)gs, (int)gs, (int)gs );

        cudaMallocHost( &r->hIntersectedCircleNb, 4 );
        cudaMallocHost( &r->hIntersectionNb, 4 );
        cudaMallocHost( &r->hFullCircleNb, 4 );
        cudaMallocHost( &r->hSegmentCount, 4 );
        cudaMallocHost( &r->hVisibleCircleNb, 4 );
        cudaMalloc( &r->dIntersectedCircleNb, 4 );
        cudaMalloc( &r->dIntersectionNb, 4 );
        cudaMalloc( &r->dFullCircleNb, 4 );
        cudaMalloc( &r->dSegmentCount, 4 );

        const size_t N = r->n;
        r->atoms       = DBuf( sizeof( float4 ) * N );
        if ( r->mode == 0 )
            r->convexPatches = DBuf( sizeof( uint2 ) * N );
        r->atomIndices = DBuf( sizeof( uint32_t ) * N );
        r->nbrCount    = DBuf( sizeof( uint32_t ) * N );
        r->nbrIds      = DBuf( sizeof( uint32_t ) * r->maxNbr * N );
        r->status      = DBuf( r->maxNbr * N + 1, r->mode == 1 );
        if ( r->mode == 0 )
            r->globalToTrimmed = DBuf( sizeof( uint32_t ) * ( r->maxNbr * N + 1 ) );

        cudaMemPool_t pool;
        int           dev = 0;
        cudaGetDevice( &dev );
        cudaDeviceGetDefaultMemPool( &pool, dev );
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute( pool, cudaMemPoolAttrReleaseThreshold, &threshold );
        r->grid.init( r->gridInfo );
    }

    SesdfContextRef fullContext( Ref * r )
    {
        SesdfContextRef c {};
        c.probeRadius                = r->rp;
        c.atomNb                     = r->n;
        c.atoms                      = r->atoms.get<float4>();
        c.sortedToInitialIndices     = r->atomIndices.get<uint32_t>();
        c.neighborNb                 = r->nbrCount.get<uint32_t>();
        c.neighborIds                = r->nbrIds.get<uint32_t>();
        c.visibilityStatus           = r->status.get<uint8_t>();
        c.maxNeighborPerAtom         = r->maxNbr;
        c.maxIntersectionsPerCircles = kMeanIntPerC;
        c.maxIntersectionNeighbors   = kMaxIntNbr;
        c.globalToTrimmedId          = r->globalToTrimmed.get<uint32_t>();
        c.dIntersectedCircleNb       = r->dIntersectedCircleNb;
        c.hIntersectedCircleNb       = r->hIntersectedCircleNb;
        c.dIntersectionNb            = r->dIntersectionNb;
        c.hIntersectionNb            = r->hIntersectionNb;
        c.dFullCircleNb              = r->dFullCircleNb;
        c.hFullCircleNb              = r->hFullCircleNb;
        c.dSegmentCount              = r->dSegmentCount;
        c.hSegmentCount              = r->hSegmentCount;
        c.hVisibleCircleNb           = r->hVisibleCircleNb;
        return c;
    }

    // Sesdf::build (sesdf/src/sesdf/sesdf.cu:172-264)
    bool buildFull( Ref * r )
    {
        SesdfContextRef ctx = fullContext( r );
        cudaMemset( ctx.dIntersectedCircleNb, 0, 4 );
        *ctx.hIntersectedCircleNb = 0;
        cudaMemset( ctx.dIntersectionNb, 0, 4 );
        *ctx.hIntersectionNb = 0;
        cudaMemset( ctx.dFullCircleNb, 0, 4 );
        *ctx.hFullCircleNb = 0;
        cudaMemset( ctx.dSegmentCount, 0, 4 );
        *ctx.hSegmentCount    = 0;
        *ctx.hVisibleCircleNb = 0;
        const uint32_t N      = r->n;
        const uint64_t slots  = (uint64_t)N * r->maxNbr;

        // #1 H2D
        cudaMemcpy( ctx.atoms, r->hostAtoms, sizeof( float4 ) * N, cudaMemcpyHostToDevice );

        // #2 findCircles (operations.inl:14-93)
        if ( !r->grid.build( N, ctx.atoms ) )
            return false;
        d2d( ctx.atoms, r->grid.sorted.get<float4>(), N );
        d2d( ctx.sortedToInitialIndices, r->grid.indices.get<uint32_t>(), N );
        {
            uint32_t         g, b;
            const uint32_t * cs = r->grid.start.get<uint32_t>();
            const uint32_t * ce = r->grid.end.get<uint32_t>();
            kernelConfig( N, r->maxNbr, g, b );
            if ( N && !launch( kFindCircles, g, b, 0, r->gridInfo, cs, ce, ctx ) )
                return false;
        }
        DBuf       temp( slots * sizeof( uint2 ) + ( slots + 1 ) * sizeof( uint32_t ), true );
        uint32_t * mask            = temp.get<uint32_t>( slots * sizeof( uint2 ) );
        uint2 *    tempFullCircles = temp.get<uint2>();
        if ( N && !launch( kVisibility, N, r->maxNbr, r->maxNbr * sizeof( float4 ), ctx, tempFullCircles, mask ) )
            return false;

        // prefixSumCount (memory.inl:26-49)
        thrust::exclusive_scan( thrust::device, mask, mask + slots + 1, ctx.globalToTrimmedId );
        d2h( ctx.hIntersectedCircleNb, ctx.globalToTrimmedId + slots, 1 );

        r->trimmedToGlobal = DBuf( sizeof( uint32_t ) * *ctx.hIntersectedCircleNb );
        thrust::copy_if( thrust::device, thrust::make_counting_iterator<uint32_t>( 0 ),
                         thrust::make_counting_iterator<uint32_t>( (uint32_t)slots ), mask,
                         r->trimmedToGlobal.get<uint32_t>(), Identity() );
        thrust::transform_exclusive_scan( thrust::device, ctx.visibilityStatus, ctx.visibilityStatus + slots + 1, mask,
                                          NonZeroU8(), 0u, thrust::plus<uint32_t>() );
        d2h( ctx.hVisibleCircleNb, mask + slots, 1 );
        const uint32_t visibleCirclesNb = *ctx.hVisibleCircleNb;
        d2h( ctx.hFullCircleNb, ctx.dFullCircleNb, 1 );

        const size_t alignment = ( *ctx.hFullCircleNb * sizeof( uint2 ) ) % sizeof( float4 );
        r->fCircleAndSectors   = DBuf( *ctx.hFullCircleNb * sizeof( uint2 ) + alignment + visibleCirclesNb * sizeof( float4 ) );
        if ( visibleCirclesNb > 0 )
        {
            uint2 *  convex  = r->convexPatches.get<uint2>();
            float4 * sectors = r->fCircleAndSectors.get<float4>( *ctx.hFullCircleNb * sizeof( uint2 ) + alignment );
            if ( !launch( r->maxNbr == kMaxNbr288 ? kSectors288 : kSectors, N, r->maxNbr, 0, ctx, mask, convex, sectors ) )
                return false;
        }
        if ( *ctx.hFullCircleNb > 0 )
            d2d( r->fCircleAndSectors.get<uint2>(), tempFullCircles, *ctx.hFullCircleNb );

        ctx.trimmedToGlobalId = r->trimmedToGlobal.get<uint32_t>();
        r->convexPatchNb      = N;
        r->fullCircleNb       = *ctx.hFullCircleNb;
        r->sectorNb           = visibleCirclesNb;
        r->trimmedNb          = *ctx.hIntersectedCircleNb;
        r->visibleNb          = visibleCirclesNb;
        r->intersectionNb = r->intersectionWithNbr = r->segmentNb = 0;

        if ( *ctx.hIntersectedCircleNb > 0 )
        {
            const uint32_t C1  = *ctx.hIntersectedCircleNb;
            r->circleIntCount  = DBuf( sizeof( uint32_t ) * C1, true );
            ctx.circlesIntersectionNb = r->circleIntCount.get<uint32_t>();

            // findIntersections (operations.inl:106-173)
            {
                DBuf   tempIds( sizeof( int4 ) * std::max<uint64_t>( (uint64_t)C1 * kMeanIntPerC, slots ) );
                int4 * tids = tempIds.get<int4>();
                if ( !launch( r->maxNbr == kMaxNbr288 ? kFindIntersections288 : kFindIntersections, N, r->maxNbr, 0, ctx, tids ) )
                    return false;
                d2h( ctx.hIntersectionNb, ctx.dIntersectionNb, 1 );
                const uint32_t I = *ctx.hIntersectionNb;
                thrust::sort( thrust::device, tids, tids + I, HasNeighborsComparator() );
                ctx.intersectionWithNeighborNb
                    = (uint32_t)thrust::count_if( thrust::device, tids, tids + I, HasNeighbors() );
                const uint32_t Q  = ctx.intersectionWithNeighborNb;
                r->intersections  = DBuf( (size_t)I * ( sizeof( int4 ) + sizeof( float4 ) )
                                         + (size_t)Q * sizeof( float4 ) * kMaxIntNbr + (size_t)Q * sizeof( float4 ) );
                d2d( r->intersections.get<int4>(), tids, I );
            }
            const uint32_t I    = *ctx.hIntersectionNb;
            r->startAndIds      = DBuf( sizeof( uint32_t ) * ( C1 + (size_t)I * 3 ) );
            uint32_t * startIds = r->startAndIds.get<uint32_t>();
            uint32_t * ids      = startIds + C1;
            thrust::transform_exclusive_scan( thrust::device, ctx.circlesIntersectionNb, ctx.circlesIntersectionNb + C1,
                                              startIds, U8ToU32(), 0u, thrust::plus<uint32_t>() );
            {
                DBuf stencil( sizeof( uint32_t ) * C1, true );
                uint32_t g, b;
                kernelConfig( I, 256, g, b );
                int4 *     iids    = r->intersections.get<int4>();
                uint32_t * st      = stencil.get<uint32_t>();
                float4 *   ipos    = r->intersections.get<float4>( sizeof( int4 ) * (size_t)I );
                if ( I && !launch( kFillIntersections, g, b, 0, ctx, startIds, iids, st, ids, ipos ) )
                    return false;
            }
            r->intersectionNb      = I;
            r->intersectionWithNbr = ctx.intersectionWithNeighborNb;
            ctx.circlesIntersectionStartId = startIds;
            ctx.circlesIntersectionIds     = ids;

            // buildConicPatches<16> (operations.inl:488-541)
            {
                const float4 * ipos        = r->intersections.get<float4>( sizeof( int4 ) * (size_t)I );
                const int4 *   iids        = r->intersections.get<int4>();
                const size_t   buffer1Size = (size_t)C1 + 1;
                DBuf           temp2( sizeof( uint32_t ) * ( buffer1Size + C1 ), true );
                uint32_t *     segmentIds  = temp2.get<uint32_t>();
                uint32_t *     withSegIds  = segmentIds + buffer1Size;
                thrust::transform( thrust::device, ctx.circlesIntersectionNb, ctx.circlesIntersectionNb + C1, segmentIds,
                                   HalfU8() );
                uint32_t * last = thrust::copy_if( thrust::device, thrust::make_counting_iterator<uint32_t>( 0 ),
                                                   thrust::make_counting_iterator<uint32_t>( C1 ), segmentIds, withSegIds,
                                                   NonZeroU32() );
                const uint32_t cws = (uint32_t)( last - withSegIds );
                thrust::exclusive_scan( thrust::device, segmentIds, segmentIds + buffer1Size, segmentIds );
                d2h( ctx.hSegmentCount, segmentIds + buffer1Size - 1, 1 );
                r->segmentNb = *ctx.hSegmentCount;
                if ( *ctx.hSegmentCount > 0 )
                {
                    r->segments = DBuf( sizeof( uint4 ) * *ctx.hSegmentCount );
                    uint32_t g, b;
                    kernelConfig( cws, 256, g, b );
                    if ( b % 16 != 0 )
                        b = cws + 16 - cws % 16;
                    uint4 * segs = r->segments.get<uint4>();
                    if ( !launch( kSegments, g, b, 0, ctx, cws, withSegIds, ipos, iids, segmentIds, segs ) )
                        return false;
                }
            }

            // handleIntersectionSingularities (operations.cu:14-32)
            if ( ctx.intersectionWithNeighborNb > 0 )
            {
                const float4 * ipos = r->intersections.get<float4>( sizeof( int4 ) * (size_t)I );
                int4 *         iids = r->intersections.get<int4>();
                float4 *       nbrs = r->intersections.get<float4>( (size_t)I * ( sizeof( int4 ) + sizeof( float4 ) ) );
                if ( !r->grid.build( ctx.intersectionWithNeighborNb, ipos ) )
                    return false;
                uint32_t g, b;
                kernelConfig( ctx.intersectionWithNeighborNb, 256, g, b );
                const float4 *   sp = r->grid.sorted.get<float4>();
                const uint32_t * si = r->grid.indices.get<uint32_t>();
                const uint32_t * cs = r->grid.start.get<uint32_t>();
                const uint32_t * ce = r->grid.end.get<uint32_t>();
                if ( !launch( kIntNeighbors, g, b, 0, r->gridInfo, ctx, sp, si, cs, ce, ipos, iids, nbrs ) )
                    return false;
            }
        }
        return checkRt( cudaGetLastError(), "build" );
    }

    // Ssesdf::build (sesdf/src/ssesdf/ssesdf.cu:133-187)
    bool buildExterior( Ref * r )
    {
        SsesdfContextRef ctx {};
        ctx.probeRadius                = r->rp;
        ctx.atomNb                     = r->n;
        ctx.atoms                      = r->atoms.get<float4>();
        ctx.sortedToInitialIndices     = r->atomIndices.get<uint32_t>();
        ctx.neighborNb                 = r->nbrCount.get<uint32_t>();
        ctx.neighborIds                = r->nbrIds.get<uint32_t>();
        ctx.visibilityStatus           = r->status.get<uint8_t>();
        ctx.maxNeighborPerAtom         = r->maxNbr;
        ctx.maxIntersectionsPerCircles = 2;
        ctx.maxIntersectionNeighbors   = kMaxIntNbr;
        ctx.dIntersectionNb            = r->dIntersectionNb;
        cudaMemset( ctx.dIntersectionNb, 0, 4 );
        ctx.hIntersectionNb  = r->hIntersectionNb;
        *ctx.hIntersectionNb = 0;
        ctx.hVisibleCircleNb  = r->hVisibleCircleNb;
        *ctx.hVisibleCircleNb = 0;
        const uint32_t N      = r->n;
        const uint64_t slots  = (uint64_t)N * r->maxNbr;

        cudaMemcpy( ctx.atoms, r->hostAtoms, sizeof( float4 ) * N, cudaMemcpyHostToDevice );

        // findCircles (ssesdf/operations.cu:25-55)
        if ( !r->grid.build( N, ctx.atoms ) )
            return false;
        d2d( ctx.atoms, r->grid.sorted.get<float4>(), N );
        d2d( ctx.sortedToInitialIndices, r->grid.indices.get<uint32_t>(), N );
        {
            uint32_t         g, b;
            const uint32_t * cs = r->grid.start.get<uint32_t>();
            const uint32_t * ce = r->grid.end.get<uint32_t>();
            kernelConfig( N, r->maxNbr, g, b );
            if ( N && !launch( kXFindCircles, g, b, 0, r->gridInfo, cs, ce, ctx ) )
                return false;
        }
        if ( N && !launch( kXVisibility, N, r->maxNbr, r->maxNbr * sizeof( float4 ), ctx ) )
            return false;
        *ctx.hVisibleCircleNb
            = (uint32_t)thrust::count_if( thrust::device, ctx.visibilityStatus, ctx.visibilityStatus + slots, NonZeroU8() );
        ctx.intersectedCircleNb
            = (uint32_t)thrust::count_if( thrust::device, ctx.visibilityStatus, ctx.visibilityStatus + slots, NonZeroU8() );
        r->visibleNb = *ctx.hVisibleCircleNb;
        r->circleNb  = *ctx.hVisibleCircleNb;
        r->intersectionNb = r->intersectionWithNbr = 0;

        if ( r->circleNb > 0 )
        {
            // findIntersections (ssesdf/operation.inl:28-98)
            {
                DBuf   tempIds( sizeof( int4 ) * std::max<uint64_t>( (uint64_t)ctx.intersectedCircleNb * 2, slots ) );
                int4 * tids = tempIds.get<int4>();
                if ( !launch( r->maxNbr == kMaxNbr288 ? kXFindIntersections288 : kXFindIntersections, N, r->maxNbr, 0, ctx, tids ) )
                    return false;
                d2h( ctx.hIntersectionNb, ctx.dIntersectionNb, 1 );
                const uint32_t I = *ctx.hIntersectionNb;
                thrust::sort( thrust::device, tids, tids + I, HasNeighborsComparator() );
                ctx.intersectionWithNeighborNb
                    = (uint32_t)thrust::count_if( thrust::device, tids, tids + I, HasNeighbors() );
                const uint32_t Q = ctx.intersectionWithNeighborNb;
                r->intersections = DBuf( (size_t)I * ( sizeof( int4 ) + sizeof( float4 ) )
                                         + (size_t)Q * sizeof( float4 ) * kMaxIntNbr + (size_t)Q * sizeof( float4 ) );
                d2d( r->intersections.get<int4>() + I, tids, I );
            }
            const uint32_t I = *ctx.hIntersectionNb;
            {
                uint32_t g, b;
                kernelConfig( I, 256, g, b );
                int4 *   iids = r->intersections.get<int4>() + I;
                float4 * ipos = r->intersections.get<float4>();
                if ( I && !launch( kXFillIntersections, g, b, 0, ctx, iids, ipos ) )
                    return false;
            }
            const uint32_t T = (uint32_t)thrust::count_if( thrust::device, ctx.visibilityStatus,
                                                           ctx.visibilityStatus + slots, IsCompleteU8() );
            DBuf patchesIds( sizeof( uint32_t ) * T );
            thrust::copy_if( thrust::device, thrust::make_counting_iterator<uint32_t>( 0 ),
                             thrust::make_counting_iterator<uint32_t>( (uint32_t)slots ), ctx.visibilityStatus,
                             patchesIds.get<uint32_t>(), IsCompleteU8() );
            r->circles = DBuf( sizeof( float4 ) * 3 * (size_t)T );
            {
                uint32_t g, b;
                kernelConfig( T, 256, g, b );
                const uint32_t * pid  = patchesIds.get<uint32_t>();
                float4 *         pos  = r->circles.get<float4>();
                float4 *         axis = pos + T;
                float4 *         vs   = pos + 2ull * T;
                if ( T && !launch( kXFillCircles, g, b, 0, ctx, T, pid, pos, axis, vs ) )
                    return false;
            }
            r->circleNb            = T;
            r->intersectionNb      = I;
            r->intersectionWithNbr = ctx.intersectionWithNeighborNb;

            // handleIntersectionSingularities (ssesdf/operations.cu:57-75)
            if ( ctx.intersectionWithNeighborNb > 0 )
            {
                float4 * ipos = r->intersections.get<float4>();
                int4 *   iids = r->intersections.get<int4>() + I;
                float4 * nbrs = r->intersections.get<float4>() + 2ull * I;
                if ( !r->grid.build( ctx.intersectionWithNeighborNb, ipos ) )
                    return false;
                uint32_t g, b;
                kernelConfig( ctx.intersectionWithNeighborNb, 256, g, b );
                const float4 *   sp = r->grid.sorted.get<float4>();
                const uint32_t * si = r->grid.indices.get<uint32_t>();
                const uint32_t * cs = r->grid.start.get<uint32_t>();
                const uint32_t * ce = r->grid.end.get<uint32_t>();
                if ( !launch( kXIntNeighbors, g, b, 0, r->gridInfo, ctx, sp, si, cs, ce, ipos, iids, nbrs ) )
                    return false;
            }
        }
        return checkRt( cudaGetLastError(), "build" );
    }
} // namespace

extern "C"
{
    const char * sesref_error() { return g_err.c_str(); }

    // Loads the reference cubin and resolves its kernels; checks the host
    // mirror structs against the kernels' parameter sizes.
    int sesref_init( const char * cubinPath )
    {
        if ( g_lib )
            return 0;
        cudaFree( nullptr ); // create the primary context
        if ( !check( cuLibraryLoadFromFile( &g_lib, cubinPath, nullptr, nullptr, 0, nullptr, nullptr, 0 ), "load" ) )
            return -1;
        unsigned int count = 0;
        if ( !check( cuLibraryGetKernelCount( &count, g_lib ), "count" ) )
            return -1;
        std::vector<CUkernel> kernels( count );
        if ( !check( cuLibraryEnumerateKernels( kernels.data(), count, g_lib ), "enumerate" ) )
            return -1;
        for ( CUkernel k : kernels )
        {
            const char * mangled = nullptr;
            if ( cuKernelGetName( &mangled, k ) != CUDA_SUCCESS || !mangled )
                continue;
            int    st        = 0;
            char * demangled = abi::__cxa_demangle( mangled, nullptr, nullptr, &st );
            if ( !demangled )
                continue;
            std::string name( demangled );
            std::free( demangled );
            if ( name.rfind( "void ", 0 ) == 0 )
                name = name.substr( 5 );
            for ( int i = 0; i < kCount; i++ )
                if ( name.rfind( kNames[ i ], 0 ) == 0 )
                {
                    CUfunction f;
                    if ( !check( cuKernelGetFunction( &f, k ), "function" ) )
                        return -1;
                    g_fn[ i ] = f;
                }
        }
        for ( int i = 0; i < kCount; i++ )
            if ( !g_fn[ i ] )
            {
                g_err = std::string( "kernel not found: " ) + kNames[ i ];
                return -2;
            }
        // parameter layout checks
        struct
        {
            K      k;
            int    idx;
            size_t size;
        } checks[] = { { kFindCircles, 0, sizeof( GridInfoRef ) },        { kFindCircles, 3, sizeof( SesdfContextRef ) },
                       { kXFindCircles, 3, sizeof( SsesdfContextRef ) }, { kVisibility, 0, sizeof( SesdfContextRef ) },
                       { kXVisibility, 0, sizeof( SsesdfContextRef ) },  { kIntNeighbors, 1, sizeof( SesdfContextRef ) } };
        for ( auto & c : checks )
        {
            size_t off = 0, sz = 0;
            if ( cuFuncGetParamInfo( g_fn[ c.k ], c.idx, &off, &sz ) == CUDA_SUCCESS && sz != c.size )
            {
                char buf[ 256 ];
                snprintf( buf, sizeof( buf ), "parameter %d of %s has %zu bytes, mirror has %zu", c.idx, kNames[ c.k ], sz,
                          c.size );
                g_err = buf;
                return -3;
            }
        }
        return 0;
    }

    // Constructs the reference object (the host atoms are borrowed, as the
    // reference's ConstSpan is).
    void * sesref_create_cap( const float * atoms, uint32_t n, const float * aabb, float rp, int mode, uint32_t maxNbr )
    {
        if ( maxNbr != kMaxNbr && maxNbr != kMaxNbr288 )
        {
            g_err = "neighbour slots per atom: 128 or 288";
            return nullptr;
        }
        Ref * r       = new Ref();
        r->maxNbr     = maxNbr;
        r->mode       = mode;
        r->hostAtoms  = atoms;
        r->n          = n;
        r->rp         = rp;
        construct( r, aabb );
        cudaDeviceSynchronize();
        return r;
    }

    void * sesref_create( const float * atoms, uint32_t n, const float * aabb, float rp, int mode )
    {
        return sesref_create_cap( atoms, n, aabb, rp, mode, kMaxNbr );
    }

    int sesref_build( void * h )
    {
        Ref * r  = static_cast<Ref *>( h );
        bool  ok = r->mode == 0 ? buildFull( r ) : buildExterior( r );
        return ok ? 0 : -1;
    }

    // Times `iterations` builds with CUDA events on the legacy default stream
    // (app/benchmarks/main.cu:37-56); writes per-build milliseconds.
    int sesref_time( void * h, int iterations, float * ms )
    {
        cudaEvent_t a, b;
        cudaEventCreate( &a );
        cudaEventCreate( &b );
        for ( int it = 0; it < iterations; it++ )
        {
            cudaEventRecord( a, 0 );
            if ( sesref_build( h ) )
                return -1;
            cudaEventRecord( b, 0 );
            cudaEventSynchronize( b );
            cudaEventElapsedTime( ms + it, a, b );
        }
        cudaEventDestroy( a );
        cudaEventDestroy( b );
        return 0;
    }

    // Counts: n, F, V, C1, I, Q, S, T (exterior tori), visible circles.
    void sesref_counts( void * h, uint64_t * out )
    {
        Ref * r  = static_cast<Ref *>( h );
        out[ 0 ] = r->n;
        out[ 1 ] = r->fullCircleNb;
        out[ 2 ] = r->sectorNb;
        out[ 3 ] = r->trimmedNb;
        out[ 4 ] = r->intersectionNb;
        out[ 5 ] = r->intersectionWithNbr;
        out[ 6 ] = r->segmentNb;
        out[ 7 ] = r->mode == 1 ? r->circleNb : 0;
        out[ 8 ] = r->visibleNb;
    }

    // Copies a named output to host memory (bytes must match the buffer's size).
    int sesref_get( void * h, const char * name, void * dst, uint64_t bytes )
    {
        Ref *          r  = static_cast<Ref *>( h );
        const uint64_t I  = r->intersectionNb, Q = r->intersectionWithNbr, N = r->n;
        const void *   src = nullptr;
        uint64_t       need = 0;
        const size_t   align = ( r->fullCircleNb * sizeof( uint2 ) ) % sizeof( float4 );
        std::string    s( name );
        if ( s == "atoms" )
            src = r->atoms.p, need = 16 * N;
        else if ( s == "atom_indices" )
            src = r->atomIndices.p, need = 4 * N;
        else if ( s == "nbr_count" )
            src = r->nbrCount.p, need = 4 * N;
        else if ( s == "nbr_ids" )
            src = r->nbrIds.p, need = 4 * N * r->maxNbr;
        else if ( s == "status" )
            src = r->status.p, need = N * r->maxNbr;
        else if ( s == "global_to_trimmed" && r->mode == 0 )
            src = r->globalToTrimmed.p, need = 4 * ( N * r->maxNbr + 1 );
        else if ( s == "convex" && r->mode == 0 )
            src = r->convexPatches.p, need = 8 * N;
        else if ( s == "full_circles" && r->mode == 0 )
            src = r->fCircleAndSectors.p, need = 8ull * r->fullCircleNb;
        else if ( s == "sectors" && r->mode == 0 )
            src = r->fCircleAndSectors.get<char>( r->fullCircleNb * sizeof( uint2 ) + align ), need = 16ull * r->sectorNb;
        else if ( s == "segments" && r->mode == 0 )
            src = r->segments.p, need = 16ull * r->segmentNb;
        else if ( s == "int_ids" )
            src = r->mode == 0 ? r->intersections.p : r->intersections.get<char>( 16 * I ), need = 16 * I;
        else if ( s == "int_pos" )
            src = r->mode == 0 ? r->intersections.get<char>( 16 * I ) : r->intersections.p, need = 16 * I;
        else if ( s == "int_nbrs" )
            src = r->intersections.get<char>( 32 * I ), need = 16 * kMaxIntNbr * Q;
        else if ( s == "tori" && r->mode == 1 )
            src = r->circles.p, need = 48ull * r->circleNb;
        else
        {
            g_err = "unknown output " + s;
            return -1;
        }
        if ( bytes != need )
        {
            g_err = "size mismatch for " + s;
            return -2;
        }
        if ( need == 0 )
            return 0;
        return checkRt( cudaMemcpy( dst, src, need, cudaMemcpyDeviceToHost ), "get" ) ? 0 : -3;
    }

    void sesref_destroy( void * h )
    {
        Ref * r = static_cast<Ref *>( h );
        cudaDeviceSynchronize();
        cudaFreeHost( r->hIntersectedCircleNb );
        cudaFreeHost( r->hIntersectionNb );
        cudaFreeHost( r->hFullCircleNb );
        cudaFreeHost( r->hSegmentCount );
        cudaFreeHost( r->hVisibleCircleNb );
        cudaFree( r->dIntersectedCircleNb );
        cudaFree( r->dIntersectionNb );
        cudaFree( r->dFullCircleNb );
        cudaFree( r->dSegmentCount );
        delete r;
        cudaDeviceSynchronize();
    }
}
