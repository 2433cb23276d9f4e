// bcs/core/molecule.hpp -- Molecule and getAabb of the drop-in API
// (sesdf/include/bcs/core/molecule.hpp:11,138).
#ifndef BCS_MOLECULE_HPP
#define BCS_MOLECULE_HPP

#include <vector>

#include "bcs/core/math.hpp"
#include "bcs/core/type.hpp"

namespace bcs
{
    using Molecule = std::vector<Vec4f>;

    // Axis-aligned box of the atoms' vdW spheres (min of xyz - r, max of xyz + r, float32).
    Aabb getAabb( ConstSpan<Vec4f> molecule );
} // namespace bcs

#endif // BCS_MOLECULE_HPP
