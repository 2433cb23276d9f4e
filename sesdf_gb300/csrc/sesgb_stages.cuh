// sesgb_stages.cuh -- parameter block of the SES build kernels and their launchers.
#pragma once
#include "sesgb_internal.h"

namespace sesgb
{
    constexpr int kWarpsPerBlock = 8;               // warp-per-item kernels: 256 threads
    constexpr int kNbrBuf        = 512;             // per-warp candidate buffer of the neighbour search
    constexpr int kSegBuf        = 64;              // probes per circle the segment stage can hold
    constexpr int kSnbrBuf       = 256;             // per-warp candidate buffer of the singular-probe search
    constexpr uint32_t kMaxProbeNbr = 32;           // MaxIntersectionNeighbors (sesdf.cu:18)
    // per-molecule record of a batch build (molCounts)
    enum MolField : uint32_t
    {
        kMolAtoms = 0, kMolSectors, kMolFull, kMolC1, kMolProbes, kMolSingular, kMolSegments, kMolTori,
        kMolAtomBase, kMolSectorBase, kMolFullBase, kMolC1Base, kMolProbeBase, kMolSingularBase, kMolSegmentBase,
        kMolToriBase, kMolFields
    };

    // Everything a kernel of the build needs, passed by value.
    struct Build
    {
        // configuration
        uint32_t n;      // atoms
        uint32_t cap;    // neighbour slots per atom (MaxNeighborPerAtom)
        uint32_t segCap; // probes per circle used for segments
        int      mode;   // 0 full surface, 1 exterior only
        float    rp;
        GridRef  grid;
        int      nbrSpan; // neighbour-search grid: cells of the pair cutoff / nbrSpan (1 or 2)
        // block shapes (warps per block) of the neighbour search, the visibility pass and the probe
        // screen, and the resident blocks of the persistent probe screen (0: one block per atom group)
        int      nbrWarps, visWarps, probeWarps;
        uint32_t probeQueueBlocks;

        // batches: nMol molecules built together (nMol = 1 for a single molecule). Sort
        // keys carry the molecule above molShift, so every molecule keeps its own
        // reference-grid order and atoms stay molecule-major in sorted order.
        uint32_t         nMol;
        uint32_t         molShift;
        const uint32_t * molStart;  // nMol + 1: first atom of each molecule (input and sorted order)
        const GridRef *  gridM;     // nMol: reference grid of each molecule
        const uint32_t * cellBase;  // nMol + 1: first cell of each molecule's neighbour grid
        uint32_t *       singList;  // capProbes: probe index of each singular probe (batches)
        uint32_t *       molCounts; // nMol * kMolFields: per-molecule counts and bases (batches)

        // capacities of the count-dependent buffers
        uint32_t capSectors, capFull, capC1, capProbes, capSeg, capTori, capCells;

        // atoms
        float4 *       atomsIn; // input order (device copy)
        float4 *       atoms;   // reference-grid order (the output "atoms")
        uint32_t *     perm;    // sorted id -> input id
        uint32_t *     keys;    // sort keys scratch (n)

        // neighbour grid (one per molecule)
        FineGrid * fine;
        uint32_t * cellCount; // capCells + 1
        uint32_t * cellStart; // capCells + 1
        uint32_t * cellCursor;
        uint32_t * cellItems; // n (or Q) item ids in cell order
        float4 *   cellPos;   // positions in cell order

        // neighbour lists and circles, slot = i * cap + s (the reference layout)
        uint32_t * nbr;
        uint32_t * nbrCount;
        uint8_t *  status;   // n * cap + 4 (whole 32-bit words for the flag updates)
        uint2 *    visBand;  // capVisBand: visibility tests left to double precision (i, s | k << 16)
        uint32_t   capVisBand;
        uint32_t * pairOff;  // n + 1: first pair of each atom (exclusive count of the neighbour lists)
        uint64_t * touch;    // capPairs, at pairOff[i] + s: neighbours that may hold a point of circle (i, s)
        uint32_t   capPairs;
        uint32_t * slotTrim; // partial-circle number of each slot (exclusive count)

        // per-atom counts and offsets
        uint32_t *visCnt, *partCnt, *fullCnt, *torCnt;
        uint32_t *visOff, *partOff, *fullOff, *torOff;

        // convex patches
        float4 * sectors;
        uint2 *  convex;
        uint2 *  fullCircles;

        // partial circles
        uint32_t * trimSlot; // C1

        // probes of each atom, staged as one chunk per atom (capProbes)
        float4 *   stagePos;
        int4 *     stageCid;
        int4 *     stageIds;
        uint32_t * chunkStart; // n
        uint32_t * chunkLen;   // n
        uint4 *    jobs;       // capProbes: double-precision jobs
        uint32_t * singCnt;    // n + 1
        uint32_t * regCnt;     // n + 1
        uint32_t * singOff;    // n + 1
        uint32_t * regOff;     // n + 1

        // probes, final order (singular first)
        int4 *     probeIds;  // capProbes: output ids
        float4 *   probePos;  // capProbes: output positions
        int4 *     probeCid;  // capProbes: circle ids (full: partial-circle numbers; exterior: slots)
        float4 *   probeNbrs; // capProbes * 32
        uint32_t * probeNbrIdx; // capProbes * 32: singular index of each listed neighbour
        uint32_t * ccount;    // C1 + 1
        uint32_t * cstart;    // C1 + 1
        uint32_t * ccursor;   // C1
        uint32_t * clist;     // 3 capProbes
        uint32_t * segCnt;    // C1 + 1
        uint32_t * segOff;    // C1 + 1
        uint32_t * segList;   // C1: circles with at least two probes
        uint4 *    segments;  // capSeg

        // exterior tori
        float4 *torPos, *torAxis, *torVs;

        DeviceCounts * counts;
    };

    // ---- launchers (sesgb_stages.cu) ---------------------------------------
    void launch_hash( const Build & b, cudaStream_t s );
    // neighbour-grid geometry: cells of cutoff / span (span 1 or 2), coarsened until they fit the capacity
    void launch_fine_params( const Build & b, float cutoff, uint32_t items, cudaStream_t s, int span = 1 );
    void launch_gather( const Build & b, cudaStream_t s );
    // zeroes a[0, n] and c[0, n] (c may be null) with n = min(*nDevice, nHost), or nHost without nDevice
    void launch_zero2( uint32_t * a, uint32_t * c, uint32_t nHost, const uint32_t * nDevice, cudaStream_t s );
    // kind 0: the sorted atoms (n); kind 1: the singular probes (count read from *nDevice); kind 2: the
    // sorted atoms with the radius negated for atoms without accessible surface (SDF queries)
    void launch_cells( const Build & b, int kind, uint32_t nHost, const uint32_t * nDevice, void * scanScratch,
                       cudaStream_t s );
    void launch_batch_finish( const Build & b, cudaStream_t s );
    // signed distance to the SES at float3 query points (needs the atom grid of reach
    // rmax + 2 rp + band built by launch_fine_params + launch_cells first)
    size_t sdf_scratch_bytes( uint32_t m );
    void   launch_sdf( const Build & b, const float * queries, uint32_t m, float band, float * sdf, int * kind, void * scratch,
                       cudaStream_t s );
    void   launch_sdf_backward( const Build & b, const float * queries, uint32_t m, float band, const float * gradSdf,
                                float * gradSorted, float * gradInput, void * scratch, cudaStream_t s );
    // headless image: every pixel's ray sphere-traced against the signed distance (same grid as the SDF)
    struct TraceParams
    {
        double   eye[ 3 ], forward[ 3 ], right[ 3 ], up[ 3 ];
        double   tanHalfFov, tNear, tFar, eps, normalStep;
        uint32_t width, height, maxSteps;
    };
    void launch_trace( const Build & b, const TraceParams & p, float band, float * depth, float * normals, cudaStream_t s );
    // components of the probe-accessible space on a voxel grid (sesgb_cavities.cu)
    struct CavGrid
    {
        double   lo[ 3 ]; // centre of voxel (0, 0, 0)
        double   h;
        double   rp;
        uint32_t dims[ 3 ];
    };
    // out (device double[6]): min and max of c -+ (r + rp) over the build's atoms
    void launch_cavity_bounds( const Build & b, double rp, double * out, cudaStream_t s );
    // occupancy bits, union-find labels (root = smallest voxel index), roots collected into roots
    // (scalars[0] = count, scalars[1] = error bits)
    void launch_cavity_labels( const Build & b, const CavGrid & g, uint32_t * bits, int32_t * labels, uint32_t * roots,
                               uint32_t rootCap, uint32_t * scalars, cudaStream_t s );
    // labels 1..nRoots by the rank of their root in the sorted roots; voxel counts and border flags
    // per label; the label of each of k probes (probeLabel may be null)
    void launch_cavity_relabel( const CavGrid & g, int32_t * labels, const uint32_t * roots, uint32_t nRoots, uint32_t * voxels,
                                uint8_t * border, const float4 * probes, uint32_t k, int32_t * probeLabel, cudaStream_t s );
    // SES area of the primitives of a full-surface build (sesgb_area.cu): parts (device
    // double[3]: convex, toroidal, concave), atomArea (optional, float[n], input order)
    size_t area_scratch_bytes( const Build & b );
    void   launch_area( const Build & b, double * parts, float * atomArea, cudaStream_t s );
    // gradient of gParts . parts into gradInput (float4[n], input order); gradSorted
    // (float4[n]) and scratch (area_scratch_bytes) are work buffers
    void launch_area_backward( const Build & b, const float gParts[ 3 ], float * gradSorted, float * gradInput, void * scratch,
                               cudaStream_t s );
    void launch_neighbors( const Build & b, cudaStream_t s );
    void launch_visibility( const Build & b, cudaStream_t s );
    void launch_visibility_resolve( const Build & b, cudaStream_t s );
    void launch_emit( const Build & b, cudaStream_t s );
    void launch_probes( const Build & b, cudaStream_t s );
    void launch_probe_jobs( const Build & b, cudaStream_t s );
    void launch_place( const Build & b, cudaStream_t s );
    void launch_lists( const Build & b, cudaStream_t s );
    void launch_segment_counts( const Build & b, cudaStream_t s );
    void launch_segments( const Build & b, cudaStream_t s );
    void launch_probe_neighbors( const Build & b, cudaStream_t s );
    void launch_tori( const Build & b, cudaStream_t s );
    void launch_tori_emit( const Build & b, cudaStream_t s );
    cudaError_t configure_kernels( const Build & b );
    uint32_t    probe_queue_blocks( const Build & b, int warps );
    uint64_t    launch_count();
    void launch_reference_fill( const Build & b, uint32_t * globalToTrimmed, cudaStream_t s );
} // namespace sesgb
