// sesgb_internal.h -- host-side declarations shared by the CUDA translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "sesgb_device.cuh"

namespace sesgb
{
    // Launches kernel k on stream s as a programmatic dependent of the work before
    // it: the grid may be scheduled while the previous kernel drains and waits in
    // pdl_begin() for its completion. Captured into a CUDA graph, the dependency
    // becomes a programmatic edge.
    template<typename... P, typename... A>
    inline void pdl_launch( void ( *k )( P... ), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args )
    {
        cudaLaunchConfig_t  cfg {};
        cudaLaunchAttribute attr[ 1 ];
        attr[ 0 ].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[ 0 ].val.programmaticStreamSerializationAllowed = 1;
        cfg.gridDim                                          = grid;
        cfg.blockDim                                         = block;
        cfg.dynamicSmemBytes                                 = smem;
        cfg.stream                                           = s;
        cfg.attrs                                            = attr;
        cfg.numAttrs                                         = 1;
        cudaLaunchKernelEx( &cfg, k, static_cast<P>( args )... );
    }

    // Counters written by the kernels and read back once at the end of a build.
    struct DeviceCounts
    {
        uint32_t P;        // neighbour pairs (directed circles) kept
        uint32_t V;        // visible directed circles (convex sectors)
        uint32_t F;        // complete circles with i < j
        uint32_t C1;       // partial circles with i < j
        uint32_t cand;     // (i, j, k) candidates of the probe solve
        uint32_t I;        // probes (concave patches)
        uint32_t Q;        // singular probes
        uint32_t S;        // segments
        uint32_t T;        // exterior tori
        uint32_t maxNbr;   // largest neighbour count seen (before truncation)
        uint32_t overflow; // bitmask, see Overflow
        uint32_t outside;  // atoms outside the reference grid
        uint32_t fp64[ 7 ]; // predicate evaluations settled in double precision, see Fp64Stage
        uint32_t bandJobs;  // probe candidates whose float32 screen hit the band (jobs from the top)
        uint32_t nbrTruncated;
        uint32_t segTruncated;
        uint32_t snbrTruncated;
        uint32_t torusDegenerate;
        uint32_t fineCells;  // cells of the neighbour grid in use
        float    fineCell;   // edge of a neighbour-grid cell (A)
        float    rmax;       // largest vdW radius
        uint32_t regTotal;   // regular (non-singular) probes
        // staged and jobs form one 8-byte word: k_probes advances both with one 64-bit atomic
        uint32_t staged;     // probes written to the staging chunks
        uint32_t jobs;       // double-precision probe jobs
        uint32_t segCircles; // circles carrying at least two probes
        uint32_t visBand;    // visibility tests queued for double precision
        uint32_t probeCursor; // work counter of the persistent probe screen
    };
    static_assert( offsetof( DeviceCounts, staged ) % 8 == 0 && offsetof( DeviceCounts, jobs ) == offsetof( DeviceCounts, staged ) + 4,
                   "staged and jobs form one 8-byte word" );

    enum Overflow : uint32_t
    {
        kOverflowNbr     = 1u << 0, // an atom has more neighbours than the per-atom capacity
        kOverflowSectors = 1u << 1,
        kOverflowFull    = 1u << 2,
        kOverflowC1      = 1u << 3,
        kOverflowCand    = 1u << 4,
        kOverflowProbes  = 1u << 5,
        kOverflowSeg     = 1u << 6,
        kOverflowTori    = 1u << 7,
        kOverflowCells   = 1u << 8,
        kOverflowList    = 1u << 9,
        kOverflowAtomProbes = 1u << 10, // an atom owns more probes than one warp holds (128)
        kOverflowVisBand    = 1u << 11, // more visibility tests in the float32 band than the queue holds
        kOverflowPairs      = 1u << 12, // more neighbour pairs than the touch-mask buffer holds
        kOverflowSdfList    = 1u << 13, // a query point had more atoms within reach than the SDF search holds
        kOverflowArea       = 1u << 14, // an area region had more constraints or cuts than the kernel holds
    };

    enum Fp64Stage : uint32_t
    {
        kFp64Neighbor = 0,
        kFp64Visibility,
        kFp64Occlusion,
        kFp64SingularNbr,
        kFp64Solve,    // probe candidates whose float32 screen hit the band
        kFp64Segments, // circles whose float32 angle order was ambiguous
        kFp64Positions, // kept probes whose float-float position was too close to a rounding boundary
        kFp64Count
    };

    // neighbour grid (a uniform grid whose cell is at least the largest pair cutoff)
    struct FineGrid
    {
        float3   origin;
        float    h;
        int3     dims;
        uint32_t cells;
        int      span; // cells the search stencil reaches on each side: 1 (cell >= cutoff) or 2 (cell >= cutoff / 2)
    };

    // ---- primitives (sesgb_sort.cu) ------------------------------------------
    // scratch bytes needed by exclusive_scan for n elements
    size_t scan_scratch_bytes( uint64_t n );
    // out[i] = sum_{k<i} in[k] for i < n (n read from *nDevice when given, else nHost);
    // out[n] = total; *total (device) = total when non-null. in == out allowed.
    void exclusive_scan( const uint32_t * in, uint32_t * out, uint64_t nHost, const uint32_t * nDevice, uint32_t * total,
                         void * scratch, cudaStream_t stream );
    // up to three scans of the same length in two launches
    struct ScanJob
    {
        const uint32_t * in;
        uint32_t *       out;
        uint32_t *       total;
    };
    void exclusive_scan_many( const ScanJob * jobs, int count, uint64_t nHost, const uint32_t * nDevice, void * scratch,
                              cudaStream_t stream );

    // host-side count of kernel launches (sesgb_launch_count)
    void count_launches( uint32_t k );

    size_t radix_scratch_bytes( uint32_t n );
    // stable LSD radix sort of (keys, vals) on the low `bits` bits; result in keys/vals
    void radix_sort( uint32_t * keys, uint32_t * vals, uint32_t n, int bits, void * scratch, cudaStream_t stream );
} // namespace sesgb
