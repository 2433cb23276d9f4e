// bcs/sesdf/sesdf.hpp -- drop-in bcs::Sesdf (full Solvent-Excluded Surface build).
// Same public interface as sesdf/include/bcs/sesdf/sesdf.hpp:15-88 of the reference;
// the build runs on the GB300 engine behind include/sesgb.h.
#ifndef BCS_SESDF_SESDF_HPP
#define BCS_SESDF_SESDF_HPP

#include <string>
#include <vector>

#include "bcs/core/molecule.hpp"
#include "bcs/core/type.hpp"
#include "bcs/cuda/memory.hpp"
#include "bcs/sesdf/graphics.hpp"

#ifndef BCS_SESDF_MAXNEIGHBORPERATOM
#define BCS_SESDF_MAXNEIGHBORPERATOM 128u
#endif // BCS_SESDF_MAXNEIGHBORPERATOM

struct sesgb_ctx;

namespace bcs
{
    class Sesdf
    {
      public:
        // The molecule span is borrowed: the caller keeps the atoms alive; every
        // build() uploads them again. `graphics` is accepted and ignored (no GL).
        Sesdf( ConstSpan<Vec4f> molecule, const Aabb & aabb, const float probeRadius = 1.4f, bool buildSurface = true,
               bool graphics = true );

        Sesdf( const Sesdf & )             = delete;
        Sesdf & operator=( const Sesdf & ) = delete;

        Sesdf( Sesdf && ) noexcept;
        Sesdf & operator=( Sesdf && ) noexcept;

        ~Sesdf();

        void build();

        sesdf::SesdfGraphics getGraphics() const;
        sesdf::SesdfData     getData();

        uint16_t              getMaxNeighborPerAtom() const;
        uint16_t              getMaxIntersectionsPerCircles() const;
        uint16_t              getMaxIntersectionNeighbors() const;
        std::vector<uint32_t> getAtomIndices();
        DeviceBuffer &        getDAtomIndices();
        DeviceBuffer &        getDAtomNeighborsCount();
        DeviceBuffer &        getDAtomNeighborsIndices();
        DeviceBuffer &        getDCircleVisibilityStatus();
        DeviceBuffer &        getDGlobalToTrimmedId();

        // status of the last call (0 = ok, see include/sesgb.h) and its message;
        // build() does not throw, like the reference's
        int                lastStatus() const { return m_status; }
        const std::string & lastError() const { return m_error; }
        sesgb_ctx *        handle() const { return m_ctx; }

      private:
        void record( int status );

        sesgb_ctx * m_ctx    = nullptr;
        int         m_status = 0;
        std::string m_error;
        DeviceBuffer m_views[ 5 ];
    };
} // namespace bcs

#endif // BCS_SESDF_SESDF_HPP
