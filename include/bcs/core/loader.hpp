// bcs/core/loader.hpp -- bcs::load of the drop-in API (sesdf/include/bcs/core/loader.hpp,
// sesdf/src/core/loader.cpp:14-71), for MMTF files.
#ifndef BCS_LOADER_HPP
#define BCS_LOADER_HPP

#include <string>

#include "bcs/core/molecule.hpp"

namespace bcs
{
    // Atoms (x, y, z, vdW radius) of the first model of an MMTF file, as the reference's loader
    // builds them: residues in file order, the radius of each atom's element (an unknown element
    // takes 1.2 A). Throws std::runtime_error on a file it cannot read (gzip-compressed files
    // included: decompress them first).
    Molecule load( const std::string & path );
} // namespace bcs

#endif // BCS_LOADER_HPP
