// bcs_sesdf.cpp -- the drop-in classes bcs::Sesdf and bcs::Ssesdf over the C ABI.
//
// Constructor, build(), getData(), getGraphics() and the analysis getters keep
// the reference's signatures and meaning (sesdf/src/sesdf/sesdf.cu:20-358,
// sesdf/src/ssesdf/ssesdf.cu:19-245): the molecule span is borrowed and re-read
// by every build(), results are device buffers owned by the object and valid
// until the next build(), build() reports problems without throwing.
#include <cstring>
#include <utility>

#include "bcs/sesdf/sesdf.hpp"
#include "bcs/ssesdf/ssesdf.hpp"
#include "sesgb.h"

namespace bcs
{
    Aabb getAabb( ConstSpan<Vec4f> molecule )
    {
        Aabb r;
        r.min = Vec3f( 3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f );
        r.max = Vec3f( -3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f );
        for ( std::size_t i = 0; i < molecule.size; i++ )
        {
            const Vec4f & a = molecule.ptr[ i ];
            r.min.x = std::min( r.min.x, a.x - a.w ), r.min.y = std::min( r.min.y, a.y - a.w ), r.min.z = std::min( r.min.z, a.z - a.w );
            r.max.x = std::max( r.max.x, a.x + a.w ), r.max.y = std::max( r.max.y, a.y + a.w ), r.max.z = std::max( r.max.z, a.z + a.w );
        }
        return r;
    }

    namespace
    {
        void box( const Aabb & aabb, float out[ 6 ] )
        {
            out[ 0 ] = aabb.min.x, out[ 1 ] = aabb.min.y, out[ 2 ] = aabb.min.z;
            out[ 3 ] = aabb.max.x, out[ 4 ] = aabb.max.y, out[ 5 ] = aabb.max.z;
        }

        sesgb_ctx * make( ConstSpan<Vec4f> molecule, const Aabb & aabb, float probeRadius, int mode, uint32_t cap, int & status )
        {
            float          b[ 6 ];
            sesgb_options  o {};
            sesgb_ctx *    ctx = nullptr;
            box( aabb, b );
            o.max_neighbor_per_atom = cap;
            o.device                = -1;
            o.flags                 = SESGB_FLAG_GRAPH; // rebuilds replay the captured launch sequence
            status = sesgb_create( reinterpret_cast<const float *>( molecule.ptr ), (uint32_t)molecule.size, b, probeRadius, mode,
                                   &o, &ctx );
            return ctx;
        }

        DeviceBuffer & view( sesgb_ctx * ctx, int which, DeviceBuffer & slot )
        {
            void *   p = nullptr;
            uint64_t n = 0;
            if ( ctx && sesgb_analysis_buffer( ctx, which, &p, &n ) == SESGB_OK )
                slot = DeviceBuffer( p, (std::size_t)n );
            else
                slot = DeviceBuffer();
            return slot;
        }

        std::vector<uint32_t> indices( sesgb_ctx * ctx )
        {
            sesgb_counts c {};
            if ( !ctx || sesgb_get_counts( ctx, &c ) != SESGB_OK )
                return {};
            std::vector<uint32_t> out( c.atoms );
            sesgb_atom_indices( ctx, out.data() );
            return out;
        }
    } // namespace

    // ---- Sesdf ---------------------------------------------------------------
    Sesdf::Sesdf( ConstSpan<Vec4f> molecule, const Aabb & aabb, const float probeRadius, bool buildSurface, bool )
    {
        int st = 0;
        m_ctx  = make( molecule, aabb, probeRadius, SESGB_MODE_FULL, BCS_SESDF_MAXNEIGHBORPERATOM, st );
        record( st );
        if ( buildSurface && m_ctx )
            build();
    }
    Sesdf::Sesdf( Sesdf && o ) noexcept { *this = std::move( o ); }
    Sesdf & Sesdf::operator=( Sesdf && o ) noexcept
    {
        std::swap( m_ctx, o.m_ctx );
        std::swap( m_status, o.m_status );
        std::swap( m_error, o.m_error );
        for ( int k = 0; k < 5; k++ )
            std::swap( m_views[ k ], o.m_views[ k ] );
        return *this;
    }
    Sesdf::~Sesdf() { sesgb_destroy( m_ctx ); }

    void Sesdf::record( int status )
    {
        m_status = status;
        m_error  = status == SESGB_OK ? std::string() : std::string( sesgb_error_string( status ) ) + ": " + sesgb_last_error( m_ctx );
    }

    void Sesdf::build() { record( m_ctx ? sesgb_build( m_ctx, nullptr ) : SESGB_ERR_INVALID ); }

    sesdf::SesdfData Sesdf::getData()
    {
        sesgb_full_data d {};
        sesdf::SesdfData r {};
        if ( !m_ctx || sesgb_get_full( m_ctx, &d ) != SESGB_OK )
            return r;
        r.atomNb                  = d.atomNb;
        r.atoms                   = static_cast<float4 *>( d.atoms );
        r.convexPatchNb           = d.convexPatchNb;
        r.convexPatches           = static_cast<uint2 *>( d.convexPatches );
        r.sectorNb                = d.sectorNb;
        r.sectors                 = static_cast<float4 *>( d.sectors );
        r.segmentPatchNb          = d.segmentPatchNb;
        r.segmentPatches          = static_cast<uint4 *>( d.segmentPatches );
        r.circlePatchNb           = d.circlePatchNb;
        r.circlePatches           = static_cast<uint2 *>( d.circlePatches );
        r.concavePatchNb          = d.concavePatchNb;
        r.concavePatchesPosition  = static_cast<float4 *>( d.concavePatchesPosition );
        r.concavePatchesId        = static_cast<int4 *>( d.concavePatchesId );
        r.concavePatchesNeighbors = static_cast<float4 *>( d.concavePatchesNeighbors );
        r.probeRadius             = d.probeRadius;
        r.maxConcaveNeighbors     = d.maxConcaveNeighbors;
        return r;
    }

    // The reference packs complete circles and sectors in one GL buffer
    // (sesdf/src/sesdf/sesdf.cu:266-299); offsets and sizes follow that layout.
    sesdf::SesdfGraphics Sesdf::getGraphics() const
    {
        sesgb_full_data d {};
        sesdf::SesdfGraphics g {};
        if ( !m_ctx || sesgb_get_full( m_ctx, &d ) != SESGB_OK )
            return g;
        const std::size_t F = d.circlePatchNb, I = d.concavePatchNb;
        sesgb_counts      c {};
        sesgb_get_counts( m_ctx, &c );
        g.atomNb                  = d.atomNb;
        g.atoms                   = { 0u, d.atomNb * 16ull };
        g.convexPatchNb           = d.convexPatchNb;
        g.convexPatches           = { 0u, d.atomNb * 8ull };
        g.sectorNb                = d.sectorNb;
        g.sectors                 = { 0u, F * 8 + ( ( F * 8 ) % 16 ), d.sectorNb * 16ull };
        g.segmentPatchNb          = d.segmentPatchNb;
        g.segmentPatches          = { 0u, d.segmentPatchNb * 16ull };
        g.circlePatchNb           = d.circlePatchNb;
        g.circlePatches           = { 0u, F * 8 };
        g.concavePatchNb          = d.concavePatchNb;
        g.concavePatchesPosition  = { 0u, I * 16, I * 16 };
        g.concavePatchesId        = { 0u, I * 16 };
        g.concavePatchesNeighbors = { 0u, I * 32, (std::size_t)c.singular_probes * 32 * 16 };
        g.probeRadius             = d.probeRadius;
        g.maxConcaveNeighbors     = d.maxConcaveNeighbors;
        return g;
    }

    uint16_t              Sesdf::getMaxNeighborPerAtom() const { return sesgb_max_neighbor_per_atom( m_ctx ); }
    uint16_t              Sesdf::getMaxIntersectionsPerCircles() const { return 16; }
    uint16_t              Sesdf::getMaxIntersectionNeighbors() const { return sesgb_max_intersection_neighbors( m_ctx ); }
    std::vector<uint32_t> Sesdf::getAtomIndices() { return indices( m_ctx ); }
    DeviceBuffer &        Sesdf::getDAtomIndices() { return view( m_ctx, SESGB_BUF_ATOM_INDICES, m_views[ 0 ] ); }
    DeviceBuffer &        Sesdf::getDAtomNeighborsCount() { return view( m_ctx, SESGB_BUF_NEIGHBOR_COUNT, m_views[ 1 ] ); }
    DeviceBuffer &        Sesdf::getDAtomNeighborsIndices() { return view( m_ctx, SESGB_BUF_NEIGHBOR_IDS, m_views[ 2 ] ); }
    DeviceBuffer &        Sesdf::getDCircleVisibilityStatus() { return view( m_ctx, SESGB_BUF_VISIBILITY_STATUS, m_views[ 3 ] ); }
    DeviceBuffer &        Sesdf::getDGlobalToTrimmedId() { return view( m_ctx, SESGB_BUF_GLOBAL_TO_TRIMMED, m_views[ 4 ] ); }

    // ---- Ssesdf --------------------------------------------------------------
    Ssesdf::Ssesdf( ConstSpan<Vec4f> molecule, const Aabb & aabb, const float probeRadius, bool buildSurface, bool )
    {
        int st = 0;
        m_ctx  = make( molecule, aabb, probeRadius, SESGB_MODE_EXTERIOR, BCS_SSESDF_MAXNEIGHBORPERATOM, st );
        record( st );
        if ( buildSurface && m_ctx )
            build();
    }
    Ssesdf::Ssesdf( Ssesdf && o ) noexcept { *this = std::move( o ); }
    Ssesdf & Ssesdf::operator=( Ssesdf && o ) noexcept
    {
        std::swap( m_ctx, o.m_ctx );
        std::swap( m_status, o.m_status );
        std::swap( m_error, o.m_error );
        for ( int k = 0; k < 4; k++ )
            std::swap( m_views[ k ], o.m_views[ k ] );
        return *this;
    }
    Ssesdf::~Ssesdf() { sesgb_destroy( m_ctx ); }

    void Ssesdf::record( int status )
    {
        m_status = status;
        m_error  = status == SESGB_OK ? std::string() : std::string( sesgb_error_string( status ) ) + ": " + sesgb_last_error( m_ctx );
    }

    void Ssesdf::build() { record( m_ctx ? sesgb_build( m_ctx, nullptr ) : SESGB_ERR_INVALID ); }

    ssesdf::SsesdfData Ssesdf::getData()
    {
        sesgb_exterior_data d {};
        ssesdf::SsesdfData  r {};
        if ( !m_ctx || sesgb_get_exterior( m_ctx, &d ) != SESGB_OK )
            return r;
        r.atomNb                  = d.atomNb;
        r.atoms                   = static_cast<float4 *>( d.atoms );
        r.circlePatchNb           = d.circlePatchNb;
        r.circlePosition          = static_cast<float4 *>( d.circlePosition );
        r.circleAxis              = static_cast<float4 *>( d.circleAxis );
        r.circleVs                = static_cast<float4 *>( d.circleVs );
        r.concavePatchNb          = d.concavePatchNb;
        r.concavePatchesPosition  = static_cast<float4 *>( d.concavePatchesPosition );
        r.concavePatchesId        = static_cast<int4 *>( d.concavePatchesId );
        r.concavePatchesNeighbors = static_cast<float4 *>( d.concavePatchesNeighbors );
        r.probeRadius             = d.probeRadius;
        r.maxConcaveNeighbors     = d.maxConcaveNeighbors;
        return r;
    }

    // buffer layout of sesdf/src/ssesdf/ssesdf.cu:189-210
    ssesdf::SsesdfGraphics Ssesdf::getGraphics() const
    {
        sesgb_exterior_data    d {};
        ssesdf::SsesdfGraphics g {};
        if ( !m_ctx || sesgb_get_exterior( m_ctx, &d ) != SESGB_OK )
            return g;
        sesgb_counts c {};
        sesgb_get_counts( m_ctx, &c );
        const std::size_t T = d.circlePatchNb, I = d.concavePatchNb;
        g.atomNb                  = d.atomNb;
        g.atoms                   = { 0u, 0, d.atomNb * 16ull };
        g.circlePatchNb           = d.circlePatchNb;
        g.circlePosition          = { 0u, 0, T * 16 };
        g.circleAxis              = { 0u, T * 16, T * 16 };
        g.circleVs                = { 0u, T * 32, T * 16 };
        g.concavePatchNb          = d.concavePatchNb;
        g.concavePatchesPosition  = { 0u, 0, I * 16 };
        g.concavePatchesId        = { 0u, I * 16, I * 16 };
        g.concavePatchesNeighbors = { 0u, I * 32, (std::size_t)c.singular_probes * 32 * 16 };
        g.probeRadius             = d.probeRadius;
        g.maxConcaveNeighbors     = d.maxConcaveNeighbors;
        return g;
    }

    uint16_t              Ssesdf::getMaxNeighborPerAtom() const { return sesgb_max_neighbor_per_atom( m_ctx ); }
    uint16_t              Ssesdf::getMaxIntersectionsPerCircles() const { return 2; }
    uint16_t              Ssesdf::getMaxIntersectionNeighbors() const { return sesgb_max_intersection_neighbors( m_ctx ); }
    std::vector<uint32_t> Ssesdf::getAtomIndices() { return indices( m_ctx ); }
    DeviceBuffer &        Ssesdf::getDAtomIndices() { return view( m_ctx, SESGB_BUF_ATOM_INDICES, m_views[ 0 ] ); }
    DeviceBuffer &        Ssesdf::getDAtomNeighborsCount() { return view( m_ctx, SESGB_BUF_NEIGHBOR_COUNT, m_views[ 1 ] ); }
    DeviceBuffer &        Ssesdf::getDAtomNeighborsIndices() { return view( m_ctx, SESGB_BUF_NEIGHBOR_IDS, m_views[ 2 ] ); }
    DeviceBuffer &        Ssesdf::getDCircleVisibilityStatus() { return view( m_ctx, SESGB_BUF_VISIBILITY_STATUS, m_views[ 3 ] ); }
} // namespace bcs
