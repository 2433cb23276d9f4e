// bcs/ssesdf/ssesdf.hpp -- drop-in bcs::Ssesdf (exterior-only SES build).
// Same public interface as sesdf/include/bcs/ssesdf/ssesdf.hpp:14-77 of the reference.
#ifndef BCS_SSESDF_SSESDF_HPP
#define BCS_SSESDF_SSESDF_HPP

#include <string>
#include <vector>

#include "bcs/core/molecule.hpp"
#include "bcs/core/type.hpp"
#include "bcs/cuda/memory.hpp"
#include "bcs/ssesdf/graphics.hpp"

#ifndef BCS_SSESDF_MAXNEIGHBORPERATOM
#define BCS_SSESDF_MAXNEIGHBORPERATOM 128u
#endif // BCS_SSESDF_MAXNEIGHBORPERATOM

struct sesgb_ctx;

namespace bcs
{
    class Ssesdf
    {
      public:
        Ssesdf( ConstSpan<Vec4f> molecule, const Aabb & aabb, const float probeRadius = 1.4f, bool buildSurface = true,
                bool graphics = true );

        Ssesdf( const Ssesdf & )             = delete;
        Ssesdf & operator=( const Ssesdf & ) = delete;

        Ssesdf( Ssesdf && ) noexcept;
        Ssesdf & operator=( Ssesdf && ) noexcept;

        ~Ssesdf();

        void build();

        ssesdf::SsesdfGraphics getGraphics() const;
        ssesdf::SsesdfData     getData();

        uint16_t              getMaxNeighborPerAtom() const;
        uint16_t              getMaxIntersectionsPerCircles() const;
        uint16_t              getMaxIntersectionNeighbors() const;
        std::vector<uint32_t> getAtomIndices();
        DeviceBuffer &        getDAtomIndices();
        DeviceBuffer &        getDAtomNeighborsCount();
        DeviceBuffer &        getDAtomNeighborsIndices();
        DeviceBuffer &        getDCircleVisibilityStatus();

        int                 lastStatus() const { return m_status; }
        const std::string & lastError() const { return m_error; }
        sesgb_ctx *         handle() const { return m_ctx; }

      private:
        void record( int status );

        sesgb_ctx *  m_ctx    = nullptr;
        int          m_status = 0;
        std::string  m_error;
        DeviceBuffer m_views[ 4 ];
    };
} // namespace bcs

#endif // BCS_SSESDF_SSESDF_HPP
