// sesgb_api.cu -- host orchestration of the SES build and the C ABI of include/sesgb.h.
//
// One build is a fixed sequence of launches on one stream with no host
// synchronisation until the final read of the counters (the reference reads
// counts back seven times per build and allocates its outputs per build,
// sesdf/src/sesdf/sesdf.cu:172-264). Count-dependent buffers are allocated
// with a capacity; every kernel bounds its writes by it and raises an overflow
// bit instead. After a build whose counters show an overflow, the affected
// buffers are regrown to the exact counts (plus a margin) and the build is
// run again, so the first build of a new molecule may run twice.
#include <algorithm>
#include <initializer_list>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sesgb.h"
#include "sesgb_stages.cuh"

using namespace sesgb;

struct sesgb_ctx
{
    int           device = -1;
    int           mode   = 0;
    uint32_t      n      = 0;
    float         rp     = 1.4f;
    uint32_t      flags  = 0;
    const float * hostAtoms = nullptr;
    float         aabb[ 6 ] {};
    int           gridBits = 0; // radix-sort key bits

    // batches (sesgb_create_batch): molecules, their first atoms, per-molecule records
    uint32_t              nMol = 1;
    std::vector<uint32_t> molStart;
    std::vector<GridRef>  molGrid;
    std::vector<uint32_t> molCells;
    uint32_t *            hMol = nullptr; // pinned copy of Build::molCounts

    // SDF queries: gradient scratch in sorted atom order, query-order scratch (grow-only)
    float * gradSorted = nullptr;
    void *  sdfScratch = nullptr;
    size_t  sdfScratchBytes = 0;
    double * areaParts  = nullptr; // device double[3]
    void *   areaScratch = nullptr;
    size_t   areaScratchBytes = 0;

    // cavities (sesgb_cavities): one grow-only allocation carved into the grid's parts
    void *   cavMem = nullptr;
    size_t   cavBytes = 0;
    int32_t * cavLabels = nullptr;
    uint32_t * cavVoxels = nullptr;
    uint8_t *  cavBorder = nullptr;
    uint64_t   cavV = 0;
    uint32_t   cavComponents = 0;

    Build          b {};
    DeviceCounts * hCounts = nullptr;
    void *         scanScratch = nullptr;
    size_t         scanScratchBytes = 0;
    void *         radixScratch = nullptr;
    uint32_t *     g2t = nullptr;

    std::vector<void *> fixedAllocs, dynAllocs;
    bool                built = false;
    uint32_t            rebuilds = 0;
    std::string         err;

    // per-stage events (SESGB_FLAG_PROFILE)
    static constexpr int kStages = 10;
    cudaEvent_t          ev[ kStages + 1 ] {};
    float                stageMs[ kStages ] {};
    bool                 profiled = false;

    // graph replay
    cudaGraph_t     graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    uint32_t        graphKernels = 0; // kernel launches in one replay
    bool            lastUsedGraph = false;

    // build in flight (sesgb_build_async .. sesgb_finish)
    cudaStream_t pendingStream = nullptr;
    bool         pendingUpload = false;
    const void * pendingAtoms  = nullptr;
};

namespace
{
    const char * kStatusNames[] = { "ok", "invalid argument", "CUDA error", "capacity overflow", "not built", "timeout",
                                    "wrong mode",
                                    "input exceeds a fixed limit (the no-allocation limit SESGB_NOALLOC_MAX_ATOMS, or 2^28 "
                                    "cavity-grid voxels)" };

    bool cuda_ok( sesgb_ctx * c, cudaError_t e, const char * what )
    {
        if ( e == cudaSuccess )
            return true;
        c->err = std::string( what ) + ": " + cudaGetErrorString( e );
        return false;
    }

    template<class T> T * dalloc( sesgb_ctx * c, std::vector<void *> & list, size_t count, bool & ok )
    {
        void * p = nullptr;
        if ( !ok )
            return nullptr;
        if ( !cuda_ok( c, cudaMalloc( &p, std::max<size_t>( count, 1 ) * sizeof( T ) ), "cudaMalloc" ) )
        {
            ok = false;
            return nullptr;
        }
        list.push_back( p );
        return static_cast<T *>( p );
    }

    void free_list( std::vector<void *> & list )
    {
        for ( void * p : list )
            cudaFree( p );
        list.clear();
    }

    uint32_t floor_log2( uint64_t v )
    {
        uint32_t e = 0;
        while ( v >>= 1 )
            e++;
        return e;
    }
    uint32_t next_pow2( uint64_t v )
    {
        uint64_t i = 1;
        while ( v > i )
            i <<= 1;
        return (uint32_t)i;
    }

    // getAabb (sesdf/src/core/molecule.cpp:132-143)
    void host_aabb( const float * atoms, uint32_t n, float * out )
    {
        for ( int a = 0; a < 3; a++ )
        {
            out[ a ]     = 3.402823466e+38f;
            out[ 3 + a ] = -3.402823466e+38f;
        }
        for ( uint32_t i = 0; i < n; i++ )
            for ( int a = 0; a < 3; a++ )
            {
                out[ a ]     = std::min( out[ a ], atoms[ 4 * i + a ] - atoms[ 4 * i + 3 ] );
                out[ 3 + a ] = std::max( out[ 3 + a ], atoms[ 4 * i + a ] + atoms[ 4 * i + 3 ] );
            }
    }

    // reference grid of Sesdf::Sesdf (sesdf/src/sesdf/sesdf.cu:23-33)
    void setup_grid( sesgb_ctx * c )
    {
        const float maxVdw = 3.48f;
        const uint32_t gs  = next_pow2( floor_log2( c->n ) );
        for ( int a = 0; a < 3; a++ )
        {
            const float origin = ( c->aabb[ a ] - maxVdw ) - c->rp;
            const float size   = std::fabs( ( ( c->aabb[ 3 + a ] + maxVdw ) + c->rp ) - origin );
            ( &c->b.grid.origin.x )[ a ] = origin;
            ( &c->b.grid.cell.x )[ a ]   = size / (float)gs;
        }
        c->b.grid.size = (int)gs;
        c->gridBits    = 3 * (int)floor_log2( gs );
    }

    uint32_t grow( uint64_t need ) { return (uint32_t)std::min<uint64_t>( need + need / 4 + 1024, 0xfffffff0ull ); }

    bool allocate_fixed( sesgb_ctx * c )
    {
        Build &        b  = c->b;
        const size_t   n  = c->n;
        bool           ok = true;
        auto &         L  = c->fixedAllocs;
        b.atomsIn         = dalloc<float4>( c, L, n, ok );
        b.atoms           = dalloc<float4>( c, L, n, ok );
        b.perm            = dalloc<uint32_t>( c, L, n, ok );
        b.keys            = dalloc<uint32_t>( c, L, n, ok );
        b.fine            = dalloc<FineGrid>( c, L, c->nMol, ok );
        b.nMol            = c->nMol;
        if ( c->nMol > 1 )
        {
            // per-molecule neighbour grids side by side: molecule m owns cells [cellBase[m], cellBase[m + 1])
            std::vector<uint32_t> cellBase( c->nMol + 1, 0 );
            for ( uint32_t m = 0; m < c->nMol; m++ )
                cellBase[ m + 1 ] = cellBase[ m ] + c->molCells[ m ];
            b.capCells        = cellBase[ c->nMol ];
            uint32_t * start  = dalloc<uint32_t>( c, L, c->nMol + 1, ok );
            uint32_t * base   = dalloc<uint32_t>( c, L, c->nMol + 1, ok );
            GridRef *  grids  = dalloc<GridRef>( c, L, c->nMol, ok );
            b.molCounts       = dalloc<uint32_t>( c, L, (size_t)c->nMol * kMolFields, ok );
            if ( ok && !cuda_ok( c, cudaMallocHost( &c->hMol, sizeof( uint32_t ) * c->nMol * kMolFields ), "cudaMallocHost" ) )
                ok = false;
            if ( ok )
            {
                cudaMemcpy( start, c->molStart.data(), sizeof( uint32_t ) * ( c->nMol + 1 ), cudaMemcpyHostToDevice );
                cudaMemcpy( base, cellBase.data(), sizeof( uint32_t ) * ( c->nMol + 1 ), cudaMemcpyHostToDevice );
                cudaMemcpy( grids, c->molGrid.data(), sizeof( GridRef ) * c->nMol, cudaMemcpyHostToDevice );
            }
            b.molStart = start;
            b.cellBase = base;
            b.gridM    = grids;
        }
        else
            // a half-cutoff grid over a sparse molecule needs room: cells are coarsened until they fit
            b.capCells = (uint32_t)std::min<size_t>( std::max<size_t>( 1u << 16, ( b.nbrSpan == 2 ? 16 : 4 ) * n ), 1u << 28 );
        b.cellCount       = dalloc<uint32_t>( c, L, b.capCells + 1ull, ok );
        b.cellStart       = dalloc<uint32_t>( c, L, b.capCells + 1ull, ok );
        b.cellCursor      = dalloc<uint32_t>( c, L, b.capCells + 1ull, ok );
        b.nbr             = dalloc<uint32_t>( c, L, n * b.cap, ok );
        b.nbrCount        = dalloc<uint32_t>( c, L, n + 1, ok );
        b.status          = dalloc<uint8_t>( c, L, n * b.cap + 4, ok );
        b.slotTrim        = dalloc<uint32_t>( c, L, n * b.cap, ok );
        uint32_t ** per[] = { &b.visCnt,  &b.partCnt, &b.fullCnt, &b.torCnt,  &b.visOff,    &b.partOff, &b.fullOff,
                              &b.torOff,  &b.singCnt, &b.regCnt,  &b.singOff, &b.regOff,    &b.chunkStart,
                              &b.chunkLen, &b.pairOff };
        for ( uint32_t ** p : per )
            *p = dalloc<uint32_t>( c, L, n + 1, ok );
        b.convex = dalloc<uint2>( c, L, n, ok );
        b.counts = dalloc<DeviceCounts>( c, L, 1, ok );
        if ( ok && !cuda_ok( c, cudaMallocHost( &c->hCounts, sizeof( DeviceCounts ) ), "cudaMallocHost" ) )
            ok = false;
        c->radixScratch = dalloc<char>( c, L, radix_scratch_bytes( c->n ), ok );
        if ( ok )
        {
            cudaMemset( b.status, 0, n * b.cap + 4 );
            cudaMemset( b.nbrCount, 0, sizeof( uint32_t ) * ( n + 1 ) );
        }
        return ok;
    }

    bool allocate_dynamic( sesgb_ctx * c )
    {
        free_list( c->dynAllocs );
        Build &      b  = c->b;
        bool         ok = true;
        auto &       L  = c->dynAllocs;
        const size_t C1 = b.capC1, PR = b.capProbes;
        b.sectors     = dalloc<float4>( c, L, b.capSectors, ok );
        b.fullCircles = dalloc<uint2>( c, L, b.capFull, ok );
        b.trimSlot    = dalloc<uint32_t>( c, L, C1, ok );
        b.stagePos    = dalloc<float4>( c, L, PR, ok );
        b.stageCid    = dalloc<int4>( c, L, PR, ok );
        b.stageIds    = dalloc<int4>( c, L, PR, ok );
        b.jobs        = dalloc<uint4>( c, L, PR, ok );
        b.probeIds    = dalloc<int4>( c, L, PR, ok );
        b.probePos    = dalloc<float4>( c, L, PR, ok );
        b.probeCid    = dalloc<int4>( c, L, PR, ok );
        b.probeNbrs   = dalloc<float4>( c, L, PR * kMaxProbeNbr, ok );
        b.probeNbrIdx = dalloc<uint32_t>( c, L, PR * kMaxProbeNbr, ok );
        b.singList    = c->nMol > 1 ? dalloc<uint32_t>( c, L, PR, ok ) : nullptr;
        b.ccount      = dalloc<uint32_t>( c, L, C1 + 1, ok );
        b.cstart      = dalloc<uint32_t>( c, L, C1 + 1, ok );
        b.ccursor     = dalloc<uint32_t>( c, L, C1 + 1, ok );
        b.clist       = dalloc<uint32_t>( c, L, 3 * PR, ok );
        b.segCnt      = dalloc<uint32_t>( c, L, C1 + 1, ok );
        b.segOff      = dalloc<uint32_t>( c, L, C1 + 1, ok );
        b.segList     = dalloc<uint32_t>( c, L, C1 + 1, ok );
        b.segments    = dalloc<uint4>( c, L, b.capSeg, ok );
        b.visBand     = dalloc<uint2>( c, L, b.capVisBand, ok );
        b.touch       = dalloc<uint64_t>( c, L, b.capPairs, ok );
        b.torPos      = dalloc<float4>( c, L, b.capTori, ok );
        b.torAxis     = dalloc<float4>( c, L, b.capTori, ok );
        b.torVs       = dalloc<float4>( c, L, b.capTori, ok );
        const size_t items = std::max<size_t>( c->n, PR );
        b.cellItems = dalloc<uint32_t>( c, L, items, ok );
        b.cellPos   = dalloc<float4>( c, L, items, ok );
        const uint64_t scanMax = std::max<uint64_t>( { (uint64_t)c->n + 1, C1 + 1, (uint64_t)b.capCells + 1 } );
        c->scanScratchBytes    = scan_scratch_bytes( scanMax );
        c->scanScratch         = dalloc<char>( c, L, c->scanScratchBytes, ok );
        return ok;
    }

    void destroy_graph( sesgb_ctx * c )
    {
        if ( c->graphExec )
            cudaGraphExecDestroy( c->graphExec );
        if ( c->graph )
            cudaGraphDestroy( c->graph );
        c->graphExec = nullptr;
        c->graph     = nullptr;
    }

    const char * kStageNames[] = { "grid",       "neighbors", "visibility", "circles",         "probes",
                                   "probe_jobs", "place",     "segments",   "probe_neighbors", "tori" };

    // all launches of one build; no host synchronisation inside
    void enqueue( sesgb_ctx * c, cudaStream_t s, bool profile, bool capturing = false )
    {
        Build &     b    = c->b;
        const auto  n    = c->n;
        void *      sc   = c->scanScratch;
        DeviceCounts * d = b.counts;
        auto mark = [ & ]( int k ) {
            // in a capture, an external record node keeps the event observable after replays
            if ( profile )
                cudaEventRecordWithFlags( c->ev[ k ], s, capturing ? cudaEventRecordExternal : cudaEventRecordDefault );
        };
        cudaMemsetAsync( d, 0, sizeof( DeviceCounts ), s );
        if ( n == 0 )
            return;

        // A: reference-grid order, neighbour grid, neighbour lists
        mark( 0 );
        launch_hash( b, s );
        radix_sort( b.keys, b.perm, n, c->gridBits, c->radixScratch, s );
        launch_fine_params( b, -1.f, n, s, b.nbrSpan );
        launch_gather( b, s );
        launch_cells( b, 0, n, nullptr, sc, s );
        mark( 1 );
        launch_neighbors( b, s );
        exclusive_scan( b.nbrCount, b.pairOff, n, nullptr, &d->P, sc, s );

        // B, C: visibility, sectors, complete and partial circles
        mark( 2 );
        launch_visibility( b, s );
        mark( 3 );
        launch_visibility_resolve( b, s );
        {
            const ScanJob jobs[] = { { b.visCnt, b.visOff, &d->V }, { b.partCnt, b.partOff, &d->C1 }, { b.fullCnt, b.fullOff, &d->F } };
            exclusive_scan_many( jobs, 3, n, nullptr, sc, s );
        }
        launch_emit( b, s );

        // D, E: probes
        mark( 4 );
        launch_probes( b, s );
        mark( 5 );
        launch_probe_jobs( b, s );
        mark( 6 );
        {
            const ScanJob jobs[] = { { b.singCnt, b.singOff, &d->Q }, { b.regCnt, b.regOff, &d->regTotal } };
            exclusive_scan_many( jobs, 2, n, nullptr, sc, s );
        }
        launch_zero2( b.ccount, b.ccursor, b.capC1, &d->C1, s ); // per-circle probe counts and list cursors
        launch_place( b, s );
        mark( 7 );

        // F: segments
        if ( c->mode == SESGB_MODE_FULL )
        {
            exclusive_scan( b.ccount, b.cstart, b.capC1, &d->C1, nullptr, sc, s );
            launch_lists( b, s );
            launch_segment_counts( b, s );
            exclusive_scan( b.segCnt, b.segOff, b.capC1, &d->C1, &d->S, sc, s );
            launch_segments( b, s );
        }

        // G: neighbours of singular probes
        mark( 8 );
        // singular probes are sparse in the atoms' box: their grid stays on cutoff cells (a half-cutoff
        // grid hits the cell capacity and is coarsened; measured slower)
        launch_fine_params( b, 2.f * c->rp + 0.01f, 0, s, 1 );
        launch_cells( b, 1, b.capProbes, &d->Q, sc, s );
        launch_probe_neighbors( b, s );

        // H: exterior tori
        mark( 9 );
        if ( c->mode == SESGB_MODE_EXTERIOR )
        {
            launch_tori( b, s );
            exclusive_scan( b.torCnt, b.torOff, n, nullptr, &d->T, sc, s );
            launch_tori_emit( b, s );
        }
        // batches: per-molecule records, molecule-local ids
        launch_batch_finish( b, s );
        mark( 10 );
    }

    // first capacities: protein-like ratios to the atom count (regrown on demand), or the
    // minimum with SESGB_FLAG_MIN_CAPACITY
    void initial_capacities( sesgb_ctx * c )
    {
        Build &        b   = c->b;
        const uint64_t n   = ( c->flags & SESGB_FLAG_MIN_CAPACITY ) ? 0 : c->n;
        b.capSectors       = grow( 40ull * n );
        b.capFull          = grow( 4ull * n );
        b.capC1            = grow( 24ull * n );
        b.capProbes        = grow( 8ull * n );
        b.capVisBand       = grow( n ? std::max<uint64_t>( 1u << 16, n / 2 ) : 0 );
        b.capPairs         = grow( 40ull * n );
        b.capSeg           = grow( 8ull * n );
        b.capTori          = grow( 16ull * n );
    }

    // regrows the buffers whose counts exceeded their capacity; true if any
    bool regrow( sesgb_ctx * c )
    {
        Build &              b = c->b;
        const DeviceCounts & h = *c->hCounts;
        bool                 g = false;
        auto fix = [ & ]( uint32_t & cap, uint64_t need ) {
            if ( need > cap )
            {
                cap = grow( need );
                g   = true;
            }
        };
        fix( b.capSectors, h.V );
        fix( b.capFull, h.F );
        fix( b.capC1, h.C1 );
        fix( b.capProbes, h.staged );
        fix( b.capProbes, h.I );
        fix( b.capSeg, h.S );
        fix( b.capTori, h.T );
        fix( b.capVisBand, h.visBand );
        fix( b.capPairs, h.P );
        if ( h.overflow & ( kOverflowProbes | kOverflowList ) )
        {
            // sizes follow I; a list overflow means a circle with more probes than one
            // thread can order, which regrowing does not cure
            if ( h.overflow & kOverflowProbes )
                fix( b.capProbes, (uint64_t)b.capProbes * 2 );
        }
        return g;
    }

    // enqueues one build (upload, kernels, counter read-back) without waiting
    int enqueue_build( sesgb_ctx * c, cudaStream_t s, bool upload, const void * deviceAtoms )
    {
        if ( upload && c->n )
        {
            if ( !c->hostAtoms )
            {
                c->err = "no host atoms";
                return SESGB_ERR_INVALID;
            }
            if ( !cuda_ok( c, cudaMemcpyAsync( c->b.atomsIn, c->hostAtoms, sizeof( float4 ) * c->n, cudaMemcpyHostToDevice, s ),
                           "upload" ) )
                return SESGB_ERR_CUDA;
        }
        else if ( deviceAtoms && c->n )
        {
            if ( !cuda_ok( c, cudaMemcpyAsync( c->b.atomsIn, deviceAtoms, sizeof( float4 ) * c->n, cudaMemcpyDeviceToDevice, s ),
                           "copy" ) )
                return SESGB_ERR_CUDA;
        }
        c->pendingStream = s;
        c->pendingUpload = upload;
        c->pendingAtoms  = deviceAtoms;
        const bool useGraph = ( c->flags & SESGB_FLAG_GRAPH ) && c->built;
        const bool profile  = ( c->flags & SESGB_FLAG_PROFILE ) && c->n;
        if ( profile && !c->ev[ 0 ] )
            for ( auto & e : c->ev )
                cudaEventCreate( &e );
        c->lastUsedGraph = useGraph;
        if ( useGraph )
        {
            bool replayed = true;
            if ( !c->graphExec )
            {
                replayed = false; // the capture counted this build's kernels already
                const uint64_t l0 = launch_count();
                cudaStream_t cap;
                if ( !cuda_ok( c, cudaStreamCreateWithFlags( &cap, cudaStreamNonBlocking ), "stream" ) )
                    return SESGB_ERR_CUDA;
                cudaStreamBeginCapture( cap, cudaStreamCaptureModeThreadLocal );
                enqueue( c, cap, profile, true ); // stage events become event-record nodes of the graph
                cudaMemcpyAsync( c->hCounts, c->b.counts, sizeof( DeviceCounts ), cudaMemcpyDeviceToHost, cap );
                if ( c->nMol > 1 )
                    cudaMemcpyAsync( c->hMol, c->b.molCounts, sizeof( uint32_t ) * c->nMol * kMolFields, cudaMemcpyDeviceToHost, cap );
                const cudaError_t e = cudaStreamEndCapture( cap, &c->graph );
                cudaStreamDestroy( cap );
                if ( !cuda_ok( c, e, "capture" ) )
                    return SESGB_ERR_CUDA;
                if ( !cuda_ok( c, cudaGraphInstantiate( &c->graphExec, c->graph, 0 ), "instantiate" ) )
                    return SESGB_ERR_CUDA;
                c->graphKernels = (uint32_t)( launch_count() - l0 );
            }
            if ( replayed )
                count_launches( c->graphKernels );
            if ( !cuda_ok( c, cudaGraphLaunch( c->graphExec, s ), "graph launch" ) )
                return SESGB_ERR_CUDA;
            c->profiled = profile;
        }
        else
        {
            enqueue( c, s, profile );
            cudaMemcpyAsync( c->hCounts, c->b.counts, sizeof( DeviceCounts ), cudaMemcpyDeviceToHost, s );
            if ( c->nMol > 1 )
                cudaMemcpyAsync( c->hMol, c->b.molCounts, sizeof( uint32_t ) * c->nMol * kMolFields, cudaMemcpyDeviceToHost, s );
            c->profiled = profile;
        }
        return cuda_ok( c, cudaGetLastError(), "launch" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    bool counts_fit( const sesgb_ctx * c )
    {
        const DeviceCounts & h = *c->hCounts;
        const Build &        b = c->b;
        return ( h.overflow & ~(uint32_t)kOverflowNbr ) == 0 && h.V <= b.capSectors && h.F <= b.capFull && h.C1 <= b.capC1
               && h.staged <= b.capProbes && h.I <= b.capProbes && h.S <= b.capSeg && h.T <= b.capTori
               && h.visBand <= b.capVisBand && h.P <= b.capPairs;
    }

    // waits for the enqueued build; on a capacity overflow regrows and builds again
    int finish_build( sesgb_ctx * c )
    {
        cudaStream_t s = c->pendingStream;
        for ( int attempt = 0; attempt < 6; attempt++ )
        {
            if ( !cuda_ok( c, cudaStreamSynchronize( s ), "build" ) )
                return SESGB_ERR_CUDA;
            if ( c->profiled )
                for ( int k = 0; k < sesgb_ctx::kStages; k++ )
                    cudaEventElapsedTime( &c->stageMs[ k ], c->ev[ k ], c->ev[ k + 1 ] );
            const DeviceCounts & h = *c->hCounts;
            if ( counts_fit( c ) )
            {
                if ( h.overflow & kOverflowNbr )
                {
                    c->err = "an atom has more than 512 neighbour candidates passing the test";
                    return SESGB_ERR_OVERFLOW;
                }
                c->built = true;
                return SESGB_OK;
            }
            if ( ( h.overflow & kOverflowList ) )
            {
                c->err = "a circle carries more probes than the segment stage holds";
                return SESGB_ERR_OVERFLOW;
            }
            if ( ( h.overflow & kOverflowAtomProbes ) )
            {
                c->err = "an atom owns more than 128 probes (the reference's per-atom limit as well)";
                return SESGB_ERR_OVERFLOW;
            }
            regrow( c );
            destroy_graph( c );
            c->rebuilds++;
            if ( !allocate_dynamic( c ) )
                return SESGB_ERR_CUDA;
            const int st = enqueue_build( c, s, c->pendingUpload, c->pendingAtoms );
            if ( st != SESGB_OK )
                return st;
        }
        c->err = "capacities still exceeded after regrowing";
        return SESGB_ERR_OVERFLOW;
    }

    int run_build( sesgb_ctx * c, cudaStream_t s, bool upload, const void * deviceAtoms )
    {
        const int st = enqueue_build( c, s, upload, deviceAtoms );
        return st != SESGB_OK ? st : finish_build( c );
    }
} // namespace

extern "C"
{
    int sesgb_create( const float * atoms, uint32_t n, const float * aabb, float probe_radius, int mode,
                      const sesgb_options * options, sesgb_ctx ** out )
    {
        if ( !out || ( mode != SESGB_MODE_FULL && mode != SESGB_MODE_EXTERIOR ) || !( probe_radius >= 0.f ) )
            return SESGB_ERR_INVALID;
        if ( !aabb && n && !atoms )
            return SESGB_ERR_INVALID;
        *out             = nullptr;
        sesgb_ctx * c    = new sesgb_ctx();
        c->mode          = mode;
        c->n             = n;
        c->rp            = probe_radius;
        c->hostAtoms     = atoms;
        sesgb_options o  = options ? *options : sesgb_options {};
        c->b.cap         = o.max_neighbor_per_atom ? o.max_neighbor_per_atom : 128u;
        c->b.segCap      = o.max_intersections_per_circle ? o.max_intersections_per_circle : 32u;
        c->flags         = o.flags;
        c->b.nbrSpan    = ( o.flags & SESGB_FLAG_CUTOFF_CELLS ) ? 1 : 2;
        c->b.nbrWarps   = 8;
        c->b.visWarps   = 1;
        c->b.probeWarps = 1;
        c->b.mode        = mode;
        c->b.rp          = probe_radius;
        c->b.n           = n;
        if ( c->b.cap > 4096 || c->b.segCap > (uint32_t)kSegBuf )
        {
            delete c;
            return SESGB_ERR_INVALID;
        }
        if ( o.device >= 0 && !cuda_ok( c, cudaSetDevice( o.device ), "cudaSetDevice" ) )
        {
            delete c;
            return SESGB_ERR_CUDA;
        }
        cudaGetDevice( &c->device );
        if ( aabb )
            std::memcpy( c->aabb, aabb, sizeof( c->aabb ) );
        else
            host_aabb( atoms, n, c->aabb );
        setup_grid( c );

        // first capacities from protein-like ratios; regrown on demand
        Build & b    = c->b;
        initial_capacities( c );
        if ( !allocate_fixed( c ) || !allocate_dynamic( c ) || !cuda_ok( c, configure_kernels( c->b ), "configure" ) )
        {
            const int st = SESGB_ERR_CUDA;
            sesgb_destroy( c );
            return st;
        }
        *out = c;
        return SESGB_OK;
    }

    int sesgb_set_tuning( sesgb_ctx * c, const sesgb_tuning * t )
    {
        if ( !c || !t )
            return SESGB_ERR_INVALID;
        auto one_of = []( uint32_t v, std::initializer_list<uint32_t> ok ) {
            for ( uint32_t x : ok )
                if ( v == x )
                    return true;
            return false;
        };
        if ( !one_of( t->neighbor_cell_span, { 1, 2 } ) || !one_of( t->neighbor_warps, { 2, 4, 8, 16 } )
             || !one_of( t->visibility_warps, { 1, 2, 4 } ) || !one_of( t->probe_warps, { 1, 2, 4 } ) || t->probe_queue > 1 )
        {
            c->err = "tuning value out of range";
            return SESGB_ERR_INVALID;
        }
        Build & b          = c->b;
        b.nbrSpan          = (int)t->neighbor_cell_span;
        b.nbrWarps         = (int)t->neighbor_warps;
        b.visWarps         = (int)t->visibility_warps;
        b.probeWarps       = (int)t->probe_warps;
        b.probeQueueBlocks = t->probe_queue ? probe_queue_blocks( b, b.probeWarps ) : 0u;
        destroy_graph( c );
        return SESGB_OK;
    }

    int sesgb_get_tuning( const sesgb_ctx * c, sesgb_tuning * t )
    {
        if ( !c || !t )
            return SESGB_ERR_INVALID;
        t->neighbor_cell_span = (uint32_t)c->b.nbrSpan;
        t->neighbor_warps     = (uint32_t)c->b.nbrWarps;
        t->visibility_warps   = (uint32_t)c->b.visWarps;
        t->probe_warps        = (uint32_t)c->b.probeWarps;
        t->probe_queue        = c->b.probeQueueBlocks ? 1u : 0u;
        return SESGB_OK;
    }

    int sesgb_set_host_atoms( sesgb_ctx * c, const float * atoms )
    {
        if ( !c )
            return SESGB_ERR_INVALID;
        c->hostAtoms = atoms;
        return SESGB_OK;
    }

    int sesgb_build( sesgb_ctx * c, void * stream )
    {
        if ( !c )
            return SESGB_ERR_INVALID;
        return run_build( c, static_cast<cudaStream_t>( stream ), true, nullptr );
    }

    int sesgb_build_device( sesgb_ctx * c, const void * device_atoms, void * stream )
    {
        if ( !c || ( c->n && !device_atoms ) )
            return SESGB_ERR_INVALID;
        return run_build( c, static_cast<cudaStream_t>( stream ), false, device_atoms );
    }

    int sesgb_build_async( sesgb_ctx * c, const void * device_atoms, void * stream )
    {
        if ( !c )
            return SESGB_ERR_INVALID;
        return enqueue_build( c, static_cast<cudaStream_t>( stream ), device_atoms == nullptr, device_atoms );
    }

    int sesgb_finish( sesgb_ctx * c )
    {
        if ( !c )
            return SESGB_ERR_INVALID;
        return finish_build( c );
    }

    int sesgb_get_full( sesgb_ctx * c, sesgb_full_data * o )
    {
        if ( !c || !o )
            return SESGB_ERR_INVALID;
        if ( c->mode != SESGB_MODE_FULL )
            return SESGB_ERR_MODE;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        const DeviceCounts & h      = *c->hCounts;
        o->atomNb                   = c->n;
        o->atoms                    = c->b.atoms;
        o->convexPatchNb            = c->n;
        o->convexPatches            = c->b.convex;
        o->sectorNb                 = h.V;
        o->sectors                  = c->b.sectors;
        o->segmentPatchNb           = h.S;
        o->segmentPatches           = c->b.segments;
        o->circlePatchNb            = h.F;
        o->circlePatches            = c->b.fullCircles;
        o->concavePatchNb           = h.I;
        o->concavePatchesPosition   = c->b.probePos;
        o->concavePatchesId         = c->b.probeIds;
        o->concavePatchesNeighbors  = c->b.probeNbrs;
        o->probeRadius              = c->rp;
        o->maxConcaveNeighbors      = (uint16_t)kMaxProbeNbr;
        return SESGB_OK;
    }

    int sesgb_get_exterior( sesgb_ctx * c, sesgb_exterior_data * o )
    {
        if ( !c || !o )
            return SESGB_ERR_INVALID;
        if ( c->mode != SESGB_MODE_EXTERIOR )
            return SESGB_ERR_MODE;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        const DeviceCounts & h     = *c->hCounts;
        o->atomNb                  = c->n;
        o->atoms                   = c->b.atoms;
        o->circlePatchNb           = h.T;
        o->circlePosition          = c->b.torPos;
        o->circleAxis              = c->b.torAxis;
        o->circleVs                = c->b.torVs;
        o->concavePatchNb          = h.I;
        o->concavePatchesPosition  = c->b.probePos;
        o->concavePatchesId        = c->b.probeIds;
        o->concavePatchesNeighbors = c->b.probeNbrs;
        o->probeRadius             = c->rp;
        o->maxConcaveNeighbors     = (uint16_t)kMaxProbeNbr;
        return SESGB_OK;
    }

    int sesgb_get_counts( sesgb_ctx * c, sesgb_counts * o )
    {
        if ( !c || !o )
            return SESGB_ERR_INVALID;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        const DeviceCounts & h          = *c->hCounts;
        *o                              = sesgb_counts {};
        o->atoms                        = c->n;
        o->pairs                        = h.P;
        o->sectors                      = c->mode == SESGB_MODE_FULL ? h.V : 0;
        o->full_circles                 = c->mode == SESGB_MODE_FULL ? h.F : 0;
        o->partial_circles              = h.C1;
        o->candidates                   = h.cand;
        o->probes                       = h.I;
        o->singular_probes              = h.Q;
        o->segments                     = h.S;
        o->tori                         = h.T;
        o->max_neighbors                = h.maxNbr;
        o->truncated_atoms              = h.nbrTruncated;
        o->truncated_circles            = h.segTruncated;
        o->truncated_probe_neighbors    = h.snbrTruncated;
        o->degenerate_tori              = h.torusDegenerate;
        o->outside_atoms                = h.outside;
        for ( int k = 0; k < 7; k++ )
            o->fp64_decisions[ k ] = h.fp64[ k ];
        o->rebuilds = c->rebuilds;
        return SESGB_OK;
    }

    int sesgb_atom_indices( sesgb_ctx * c, uint32_t * host )
    {
        if ( !c || ( c->n && !host ) )
            return SESGB_ERR_INVALID;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        return cuda_ok( c, cudaMemcpy( host, c->b.perm, sizeof( uint32_t ) * c->n, cudaMemcpyDeviceToHost ), "copy" )
                   ? SESGB_OK
                   : SESGB_ERR_CUDA;
    }

    int sesgb_analysis_buffer( sesgb_ctx * c, int which, void ** ptr, uint64_t * bytes )
    {
        if ( !c || !ptr || !bytes )
            return SESGB_ERR_INVALID;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        const uint64_t slots = (uint64_t)c->n * c->b.cap;
        switch ( which )
        {
        case SESGB_BUF_ATOM_INDICES: *ptr = c->b.perm, *bytes = 4ull * c->n; return SESGB_OK;
        case SESGB_BUF_NEIGHBOR_COUNT: *ptr = c->b.nbrCount, *bytes = 4ull * c->n; return SESGB_OK;
        case SESGB_BUF_NEIGHBOR_IDS: *ptr = c->b.nbr, *bytes = 4ull * slots; return SESGB_OK;
        case SESGB_BUF_VISIBILITY_STATUS:
        case SESGB_BUF_GLOBAL_TO_TRIMMED:
        {
            if ( which == SESGB_BUF_GLOBAL_TO_TRIMMED )
            {
                if ( c->mode != SESGB_MODE_FULL )
                    return SESGB_ERR_MODE;
                if ( !c->g2t && !cuda_ok( c, cudaMalloc( &c->g2t, 4ull * ( slots + 1 ) ), "cudaMalloc" ) )
                    return SESGB_ERR_CUDA;
            }
            launch_reference_fill( c->b, which == SESGB_BUF_GLOBAL_TO_TRIMMED ? c->g2t : nullptr, nullptr );
            if ( !cuda_ok( c, cudaDeviceSynchronize(), "fill" ) )
                return SESGB_ERR_CUDA;
            if ( which == SESGB_BUF_VISIBILITY_STATUS )
                *ptr = c->b.status, *bytes = slots + 1;
            else
                *ptr = c->g2t, *bytes = 4ull * ( slots + 1 );
            return SESGB_OK;
        }
        default: return SESGB_ERR_INVALID;
        }
    }

    int sesgb_copy_to_host( sesgb_ctx * c, const void * dptr, void * host, uint64_t bytes )
    {
        if ( !c || ( bytes && ( !dptr || !host ) ) )
            return SESGB_ERR_INVALID;
        if ( !bytes )
            return SESGB_OK;
        return cuda_ok( c, cudaMemcpy( host, dptr, bytes, cudaMemcpyDeviceToHost ), "copy" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    uint16_t sesgb_max_neighbor_per_atom( const sesgb_ctx * c ) { return c ? (uint16_t)c->b.cap : 0; }
    uint16_t sesgb_max_intersections_per_circle( const sesgb_ctx * c ) { return c ? (uint16_t)c->b.segCap : 0; }
    uint16_t sesgb_max_intersection_neighbors( const sesgb_ctx * ) { return (uint16_t)kMaxProbeNbr; }

    int sesgb_stage_times( sesgb_ctx * c, float * ms, uint32_t capacity, uint32_t * count )
    {
        if ( !c || ( capacity && !ms ) )
            return SESGB_ERR_INVALID;
        if ( !c->profiled )
            return SESGB_ERR_NOT_BUILT;
        for ( uint32_t k = 0; k < capacity && k < (uint32_t)sesgb_ctx::kStages; k++ )
            ms[ k ] = c->stageMs[ k ];
        if ( count )
            *count = sesgb_ctx::kStages;
        return SESGB_OK;
    }

    const char * sesgb_stage_name( uint32_t stage )
    {
        return stage < (uint32_t)sesgb_ctx::kStages ? kStageNames[ stage ] : "";
    }

    uint64_t sesgb_launch_count( void ) { return launch_count(); }

    const char * sesgb_error_string( int status )
    {
        const int k = -status;
        if ( k < 0 || k >= (int)( sizeof( kStatusNames ) / sizeof( kStatusNames[ 0 ] ) ) )
            return "unknown status";
        return kStatusNames[ k ];
    }

    const char * sesgb_last_error( const sesgb_ctx * c ) { return c ? c->err.c_str() : "no context"; }

    void sesgb_destroy( sesgb_ctx * c )
    {
        if ( !c )
            return;
        cudaDeviceSynchronize();
        destroy_graph( c );
        for ( auto & e : c->ev )
            if ( e )
                cudaEventDestroy( e );
        free_list( c->dynAllocs );
        free_list( c->fixedAllocs );
        if ( c->g2t )
            cudaFree( c->g2t );
        if ( c->hCounts )
            cudaFreeHost( c->hCounts );
        if ( c->hMol )
            cudaFreeHost( c->hMol );
        if ( c->gradSorted )
            cudaFree( c->gradSorted );
        if ( c->sdfScratch )
            cudaFree( c->sdfScratch );
        if ( c->areaParts )
            cudaFree( c->areaParts );
        if ( c->areaScratch )
            cudaFree( c->areaScratch );
        if ( c->cavMem )
            cudaFree( c->cavMem );
        delete c;
    }

    // ---- signed distance at query points ---------------------------------------
    static int sdf_prepare( sesgb_ctx * c, uint32_t m, cudaStream_t s )
    {
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        const size_t need = sdf_scratch_bytes( m );
        if ( need > c->sdfScratchBytes )
        {
            if ( c->sdfScratch )
            {
                cudaStreamSynchronize( s );
                cudaFree( c->sdfScratch );
                c->sdfScratch = nullptr;
            }
            if ( !cuda_ok( c, cudaMalloc( &c->sdfScratch, need ), "cudaMalloc" ) )
            {
                c->sdfScratchBytes = 0;
                return SESGB_ERR_CUDA;
            }
            c->sdfScratchBytes = need;
        }
        if ( c->mode != SESGB_MODE_FULL || c->nMol != 1 )
        {
            c->err = "the SDF needs a full-surface build of one molecule";
            return SESGB_ERR_MODE;
        }
        const float reach = c->hCounts->rmax + 2.f * c->rp + SESGB_SDF_BAND;
        launch_fine_params( c->b, reach, c->n, s );
        launch_cells( c->b, 2, c->n, nullptr, c->scanScratch, s );
        return cuda_ok( c, cudaGetLastError(), "sdf grid" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    int sesgb_sdf( sesgb_ctx * c, const float * device_queries, uint32_t m, float * device_sdf, int * device_kind, void * stream )
    {
        if ( !c || ( m && ( !device_queries || !device_sdf ) ) )
            return SESGB_ERR_INVALID;
        cudaStream_t s  = static_cast<cudaStream_t>( stream );
        int          st = sdf_prepare( c, m, s );
        if ( st != SESGB_OK )
            return st;
        launch_sdf( c->b, device_queries, m, SESGB_SDF_BAND, device_sdf, device_kind, c->sdfScratch, s );
        return cuda_ok( c, cudaGetLastError(), "sdf" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    int sesgb_sdf_backward( sesgb_ctx * c, const float * device_queries, uint32_t m, const float * device_grad_sdf,
                            float * device_grad_atoms, void * stream )
    {
        if ( !c || !device_grad_atoms || ( m && ( !device_queries || !device_grad_sdf ) ) )
            return SESGB_ERR_INVALID;
        cudaStream_t s  = static_cast<cudaStream_t>( stream );
        int          st = sdf_prepare( c, m, s );
        if ( st != SESGB_OK )
            return st;
        if ( !c->gradSorted && !cuda_ok( c, cudaMalloc( &c->gradSorted, sizeof( float ) * 4 * std::max<size_t>( c->n, 1 ) ), "cudaMalloc" ) )
            return SESGB_ERR_CUDA;
        launch_sdf_backward( c->b, device_queries, m, SESGB_SDF_BAND, device_grad_sdf, c->gradSorted, device_grad_atoms,
                             c->sdfScratch, s );
        return cuda_ok( c, cudaGetLastError(), "sdf backward" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    int sesgb_render( sesgb_ctx * c, const sesgb_camera * cam, float * device_depth, float * device_normals, void * stream )
    {
        if ( !c || !cam || !device_depth || !cam->width || !cam->height || (uint64_t)cam->width * cam->height > ( 1ull << 28 )
             || cam->max_steps > ( 1u << 20 ) || !( cam->eps > 0.0 ) || !( cam->normal_step > 0.0 ) )
            return SESGB_ERR_INVALID;
        cudaStream_t s  = static_cast<cudaStream_t>( stream );
        int          st = sdf_prepare( c, 0, s );
        if ( st != SESGB_OK )
            return st;
        TraceParams p;
        for ( int a = 0; a < 3; a++ )
        {
            p.eye[ a ]     = cam->eye[ a ];
            p.forward[ a ] = cam->forward[ a ];
            p.right[ a ]   = cam->right[ a ];
            p.up[ a ]      = cam->up[ a ];
        }
        p.tanHalfFov = cam->tan_half_fov;
        p.tNear      = cam->t_near;
        p.tFar       = cam->t_far;
        p.eps        = cam->eps;
        p.normalStep = cam->normal_step;
        p.width      = cam->width;
        p.height     = cam->height;
        p.maxSteps   = cam->max_steps;
        launch_trace( c->b, p, SESGB_SDF_BAND, device_depth, device_normals, s );
        return cuda_ok( c, cudaGetLastError(), "render" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    // ---- exterior and cavities ---------------------------------------------------
    int sesgb_cavities( sesgb_ctx * c, double voxel, sesgb_cavity_info * info, int32_t * device_probe_component, void * stream )
    {
        if ( !c || !info || !( voxel >= 0.05 ) || !( voxel <= 100.0 ) )
            return SESGB_ERR_INVALID;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        if ( c->nMol != 1 || c->n == 0 )
        {
            c->err = "cavities need a build of one molecule with atoms";
            return SESGB_ERR_MODE;
        }
        cudaStream_t s   = static_cast<cudaStream_t>( stream );
        const double rp  = (double)c->rp;
        const double h   = voxel;
        // grid: bounds of the SAS spheres on the device, then the grid shape on the host
        auto carve = []( char *& p, size_t bytes ) {
            char * q = p;
            p += ( bytes + 255 ) & ~(size_t)255;
            return q;
        };
        const size_t small = 256;
        if ( c->cavBytes < small )
        {
            if ( c->cavMem )
                cudaFree( c->cavMem );
            c->cavMem   = nullptr;
            c->cavBytes = 0;
            if ( !cuda_ok( c, cudaMalloc( &c->cavMem, small ), "cudaMalloc" ) )
                return SESGB_ERR_CUDA;
            c->cavBytes = small;
        }
        double bounds[ 6 ];
        launch_cavity_bounds( c->b, rp, static_cast<double *>( c->cavMem ), s );
        if ( !cuda_ok( c, cudaMemcpyAsync( bounds, c->cavMem, sizeof( bounds ), cudaMemcpyDeviceToHost, s ), "bounds" )
             || !cuda_ok( c, cudaStreamSynchronize( s ), "bounds" ) )
            return SESGB_ERR_CUDA;
        CavGrid  g;
        uint64_t V = 1;
        for ( int a = 0; a < 3; a++ )
        {
            const double lo = bounds[ a ] - 2.0 * h, hi = bounds[ 3 + a ] + 2.0 * h;
            const double d  = std::ceil( ( hi - lo ) / h ) + 1.0;
            if ( !( d >= 1.0 ) || d > (double)( 1u << 28 ) )
            {
                c->err = "the cavity grid is too large for this voxel size";
                return SESGB_ERR_TOO_LARGE;
            }
            g.lo[ a ]   = lo;
            g.dims[ a ] = (uint32_t)d;
            V *= g.dims[ a ];
        }
        g.h  = h;
        g.rp = rp;
        if ( V > ( 1ull << 28 ) )
        {
            c->err = "the cavity grid exceeds 2^28 voxels: use a larger voxel size";
            return SESGB_ERR_TOO_LARGE;
        }
        const uint32_t rootCap = (uint32_t)std::min<uint64_t>( V, 1u << 22 );
        const size_t   need    = small + ( ( ( V + 31 ) / 32 * 4 + 255 ) & ~(size_t)255 ) + ( ( V * 4 + 255 ) & ~(size_t)255 )
                            + 2 * ( ( (size_t)rootCap * 4 + 255 ) & ~(size_t)255 ) + ( ( ( rootCap + 1ull ) * 4 + 255 ) & ~(size_t)255 )
                            + ( ( rootCap + 1ull + 255 ) & ~(size_t)255 ) + radix_scratch_bytes( rootCap ) + 256;
        if ( need > c->cavBytes )
        {
            cudaFree( c->cavMem );
            c->cavMem   = nullptr;
            c->cavBytes = 0;
            if ( !cuda_ok( c, cudaMalloc( &c->cavMem, need ), "cudaMalloc" ) )
                return SESGB_ERR_CUDA;
            c->cavBytes = need;
        }
        char *     p       = static_cast<char *>( c->cavMem );
        uint32_t * scalars = reinterpret_cast<uint32_t *>( carve( p, small ) );
        uint32_t * bits    = reinterpret_cast<uint32_t *>( carve( p, ( V + 31 ) / 32 * 4 ) );
        int32_t *  labels  = reinterpret_cast<int32_t *>( carve( p, V * 4 ) );
        uint32_t * roots   = reinterpret_cast<uint32_t *>( carve( p, (size_t)rootCap * 4 ) );
        uint32_t * order   = reinterpret_cast<uint32_t *>( carve( p, (size_t)rootCap * 4 ) );
        uint32_t * voxels  = reinterpret_cast<uint32_t *>( carve( p, ( rootCap + 1ull ) * 4 ) );
        uint8_t *  border  = reinterpret_cast<uint8_t *>( carve( p, rootCap + 1ull ) );
        void *     radix   = carve( p, radix_scratch_bytes( rootCap ) );
        launch_cavity_labels( c->b, g, bits, labels, roots, rootCap, scalars, s );
        uint32_t hs[ 2 ];
        if ( !cuda_ok( c, cudaMemcpyAsync( hs, scalars, sizeof( hs ), cudaMemcpyDeviceToHost, s ), "labels" )
             || !cuda_ok( c, cudaStreamSynchronize( s ), "labels" ) )
            return SESGB_ERR_CUDA;
        if ( hs[ 1 ] )
        {
            c->err = ( hs[ 1 ] & 4u ) ? "more than 2^22 components in the cavity grid" : "cavity labelling did not converge";
            return SESGB_ERR_OVERFLOW;
        }
        const uint32_t nRoots = hs[ 0 ];
        radix_sort( roots, order, nRoots, 28, radix, s ); // voxel indices are below 2^28
        const uint32_t nProbes = device_probe_component ? c->hCounts->I : 0u;
        launch_cavity_relabel( g, labels, roots, nRoots, voxels, border, c->b.probePos, nProbes, device_probe_component, s );
        std::vector<uint8_t> hb( nRoots + 1ull );
        if ( !cuda_ok( c, cudaMemcpyAsync( hb.data(), border, hb.size(), cudaMemcpyDeviceToHost, s ), "components" )
             || !cuda_ok( c, cudaStreamSynchronize( s ), "components" ) )
            return SESGB_ERR_CUDA;
        uint32_t ext = 0;
        for ( uint32_t k = 1; k <= nRoots; k++ )
            ext += hb[ k ] != 0;
        c->cavLabels     = labels;
        c->cavVoxels     = voxels;
        c->cavBorder     = border;
        c->cavV          = V;
        c->cavComponents = nRoots;
        for ( int a = 0; a < 3; a++ )
        {
            info->origin[ a ] = g.lo[ a ];
            info->dims[ a ]   = g.dims[ a ];
        }
        info->voxel      = h;
        info->components = nRoots;
        info->exterior   = ext;
        info->cavities   = nRoots - ext;
        info->probes     = nProbes;
        return SESGB_OK;
    }

    int sesgb_cavity_labels( sesgb_ctx * c, const int32_t ** device_labels, uint64_t * voxels )
    {
        if ( !c || !device_labels || !voxels )
            return SESGB_ERR_INVALID;
        if ( !c->cavLabels )
            return SESGB_ERR_NOT_BUILT;
        *device_labels = c->cavLabels;
        *voxels        = c->cavV;
        return SESGB_OK;
    }

    int sesgb_cavity_components( sesgb_ctx * c, uint32_t * host_voxels, uint8_t * host_border, uint32_t capacity )
    {
        if ( !c )
            return SESGB_ERR_INVALID;
        if ( !c->cavLabels )
            return SESGB_ERR_NOT_BUILT;
        if ( capacity < c->cavComponents + 1u )
            return SESGB_ERR_OVERFLOW;
        if ( host_voxels && !cuda_ok( c, cudaMemcpy( host_voxels, c->cavVoxels, 4ull * ( c->cavComponents + 1ull ), cudaMemcpyDeviceToHost ), "components" ) )
            return SESGB_ERR_CUDA;
        if ( host_border && !cuda_ok( c, cudaMemcpy( host_border, c->cavBorder, c->cavComponents + 1ull, cudaMemcpyDeviceToHost ), "components" ) )
            return SESGB_ERR_CUDA;
        return SESGB_OK;
    }

    // ---- SES area of the primitives ---------------------------------------------
    static int area_prepare( sesgb_ctx * c, cudaStream_t s )
    {
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        if ( c->mode != SESGB_MODE_FULL || c->nMol != 1 )
        {
            c->err = "the SES area needs a full-surface build of one molecule";
            return SESGB_ERR_MODE;
        }
        if ( !c->areaParts && !cuda_ok( c, cudaMalloc( &c->areaParts, 4 * sizeof( double ) ), "cudaMalloc" ) )
            return SESGB_ERR_CUDA;
        const size_t need = area_scratch_bytes( c->b );
        if ( need > c->areaScratchBytes )
        {
            if ( c->areaScratch )
            {
                cudaStreamSynchronize( s );
                cudaFree( c->areaScratch );
                c->areaScratch = nullptr;
            }
            if ( !cuda_ok( c, cudaMalloc( &c->areaScratch, need ), "cudaMalloc" ) )
            {
                c->areaScratchBytes = 0;
                return SESGB_ERR_CUDA;
            }
            c->areaScratchBytes = need;
        }
        // the overflow word of the build is free once its counts are on the host
        cudaMemsetAsync( &c->b.counts->overflow, 0, sizeof( uint32_t ), s );
        return SESGB_OK;
    }

    int sesgb_ses_area( sesgb_ctx * c, double * host_parts, float * device_atom_area, void * stream )
    {
        if ( !c || !host_parts )
            return SESGB_ERR_INVALID;
        cudaStream_t s  = static_cast<cudaStream_t>( stream );
        int          st = area_prepare( c, s );
        if ( st != SESGB_OK )
            return st;
        launch_area( c->b, c->areaParts, device_atom_area, s );
        uint32_t ovf = 0;
        cudaMemcpyAsync( host_parts, c->areaParts, 3 * sizeof( double ), cudaMemcpyDeviceToHost, s );
        cudaMemcpyAsync( &ovf, &c->b.counts->overflow, sizeof( uint32_t ), cudaMemcpyDeviceToHost, s );
        if ( !cuda_ok( c, cudaStreamSynchronize( s ), "ses area" ) )
            return SESGB_ERR_CUDA;
        if ( ovf & kOverflowArea )
        {
            c->err = "an area region held more constraints than the kernel does (more than 128 neighbours)";
            return SESGB_ERR_OVERFLOW;
        }
        return SESGB_OK;
    }

    int sesgb_ses_area_backward( sesgb_ctx * c, const float * host_grad_parts, float * device_grad_atoms, void * stream )
    {
        if ( !c || !host_grad_parts || !device_grad_atoms )
            return SESGB_ERR_INVALID;
        cudaStream_t s  = static_cast<cudaStream_t>( stream );
        int          st = area_prepare( c, s );
        if ( st != SESGB_OK )
            return st;
        if ( !c->gradSorted && !cuda_ok( c, cudaMalloc( &c->gradSorted, sizeof( float ) * 4 * std::max<size_t>( c->n, 1 ) ), "cudaMalloc" ) )
            return SESGB_ERR_CUDA;
        launch_area_backward( c->b, host_grad_parts, c->gradSorted, device_grad_atoms, c->areaScratch, s );
        return cuda_ok( c, cudaGetLastError(), "ses area backward" ) ? SESGB_OK : SESGB_ERR_CUDA;
    }

    int sesgb_create_batch( const float * atoms, const uint32_t * molecule_start, uint32_t molecules, float probe_radius,
                            int mode, const sesgb_options * options, sesgb_ctx ** out )
    {
        if ( !out || !molecule_start || molecules == 0 || ( mode != SESGB_MODE_FULL && mode != SESGB_MODE_EXTERIOR )
             || !( probe_radius >= 0.f ) || molecule_start[ 0 ] != 0 )
            return SESGB_ERR_INVALID;
        for ( uint32_t m = 0; m < molecules; m++ )
            if ( molecule_start[ m + 1 ] < molecule_start[ m ] )
                return SESGB_ERR_INVALID;
        const uint32_t n = molecule_start[ molecules ];
        if ( n && !atoms )
            return SESGB_ERR_INVALID;
        if ( molecules == 1 )
            return sesgb_create( atoms, n, nullptr, probe_radius, mode, options, out );
        *out            = nullptr;
        sesgb_ctx * c   = new sesgb_ctx();
        c->mode         = mode;
        c->n            = n;
        c->rp           = probe_radius;
        c->hostAtoms    = atoms;
        sesgb_options o = options ? *options : sesgb_options {};
        c->b.cap        = o.max_neighbor_per_atom ? o.max_neighbor_per_atom : 128u;
        c->b.segCap     = o.max_intersections_per_circle ? o.max_intersections_per_circle : 32u;
        c->flags        = o.flags;
        c->b.nbrSpan    = ( o.flags & SESGB_FLAG_CUTOFF_CELLS ) ? 1 : 2;
        c->b.nbrWarps   = 8;
        c->b.visWarps   = 1;
        c->b.probeWarps = 1;
        c->b.mode       = mode;
        c->b.rp         = probe_radius;
        c->b.n          = n;
        if ( c->b.cap > 4096 || c->b.segCap > (uint32_t)kSegBuf )
        {
            delete c;
            return SESGB_ERR_INVALID;
        }
        if ( o.device >= 0 && !cuda_ok( c, cudaSetDevice( o.device ), "cudaSetDevice" ) )
        {
            delete c;
            return SESGB_ERR_CUDA;
        }
        cudaGetDevice( &c->device );
        // each molecule keeps the reference grid of its own construction (getAabb of its atoms)
        c->nMol = molecules;
        c->molStart.assign( molecule_start, molecule_start + molecules + 1 );
        c->molGrid.resize( molecules );
        c->molCells.resize( molecules );
        int molShift = 1;
        for ( uint32_t m = 0; m < molecules; m++ )
        {
            const uint32_t cnt = molecule_start[ m + 1 ] - molecule_start[ m ];
            float          box[ 6 ];
            host_aabb( atoms + 4ull * molecule_start[ m ], cnt, box );
            const uint32_t gs     = next_pow2( floor_log2( cnt ) );
            const float    maxVdw = 3.48f;
            for ( int a = 0; a < 3; a++ )
            {
                const float origin = ( box[ a ] - maxVdw ) - probe_radius;
                const float size   = std::fabs( ( ( box[ 3 + a ] + maxVdw ) + probe_radius ) - origin );
                ( &c->molGrid[ m ].origin.x )[ a ] = origin;
                ( &c->molGrid[ m ].cell.x )[ a ]   = size / (float)gs;
            }
            c->molGrid[ m ].size = (int)gs;
            molShift             = std::max( molShift, 3 * (int)floor_log2( gs ) );
            c->molCells[ m ]     = std::max<uint32_t>( 1024u, 4u * cnt );
        }
        const int molBits = (int)floor_log2( molecules - 1 ) + 1;
        if ( molShift + molBits > 32 )
        {
            delete c;
            return SESGB_ERR_INVALID;
        }
        c->b.molShift = (uint32_t)molShift;
        c->gridBits   = molShift + molBits;
        c->b.grid     = c->molGrid[ 0 ];
        host_aabb( atoms, n, c->aabb );

        Build & b    = c->b;
        initial_capacities( c );
        if ( !allocate_fixed( c ) || !allocate_dynamic( c ) || !cuda_ok( c, configure_kernels( c->b ), "configure" ) )
        {
            const int st = SESGB_ERR_CUDA;
            sesgb_destroy( c );
            return st;
        }
        *out = c;
        return SESGB_OK;
    }

    uint32_t sesgb_batch_molecules( const sesgb_ctx * c ) { return c ? c->nMol : 0u; }

    int sesgb_molecule_record( const sesgb_ctx * c, uint32_t molecule, uint32_t * record )
    {
        if ( !c || !record || molecule >= c->nMol )
            return SESGB_ERR_INVALID;
        if ( !c->built )
            return SESGB_ERR_NOT_BUILT;
        if ( c->nMol == 1 )
        {
            const DeviceCounts & h = *c->hCounts;
            const uint32_t       r[ kMolFields ] = { c->n, h.V, h.F, h.C1, h.I, h.Q, h.S, h.T, 0, 0, 0, 0, 0, 0, 0, 0 };
            std::memcpy( record, r, sizeof( r ) );
            return SESGB_OK;
        }
        std::memcpy( record, c->hMol + (size_t)molecule * kMolFields, sizeof( uint32_t ) * kMolFields );
        return SESGB_OK;
    }

    int sesgb_get_full_molecule( sesgb_ctx * c, uint32_t molecule, sesgb_full_data * o )
    {
        uint32_t r[ kMolFields ];
        int      st = sesgb_molecule_record( c, molecule, r );
        if ( st != SESGB_OK )
            return st;
        if ( ( st = sesgb_get_full( c, o ) ) != SESGB_OK )
            return st;
        const Build & b            = c->b;
        o->atomNb                  = r[ kMolAtoms ];
        o->atoms                   = b.atoms + r[ kMolAtomBase ];
        o->convexPatchNb           = r[ kMolAtoms ];
        o->convexPatches           = b.convex + r[ kMolAtomBase ];
        o->sectorNb                = r[ kMolSectors ];
        o->sectors                 = b.sectors + r[ kMolSectorBase ];
        o->segmentPatchNb          = r[ kMolSegments ];
        o->segmentPatches          = b.segments + r[ kMolSegmentBase ];
        o->circlePatchNb           = r[ kMolFull ];
        o->circlePatches           = b.fullCircles + r[ kMolFullBase ];
        o->concavePatchNb          = r[ kMolProbes ];
        o->concavePatchesPosition  = b.probePos + r[ kMolProbeBase ];
        o->concavePatchesId        = b.probeIds + r[ kMolProbeBase ];
        o->concavePatchesNeighbors = b.probeNbrs + (size_t)kMaxProbeNbr * r[ kMolSingularBase ];
        return SESGB_OK;
    }

    int sesgb_get_exterior_molecule( sesgb_ctx * c, uint32_t molecule, sesgb_exterior_data * o )
    {
        uint32_t r[ kMolFields ];
        int      st = sesgb_molecule_record( c, molecule, r );
        if ( st != SESGB_OK )
            return st;
        if ( ( st = sesgb_get_exterior( c, o ) ) != SESGB_OK )
            return st;
        const Build & b            = c->b;
        o->atomNb                  = r[ kMolAtoms ];
        o->atoms                   = b.atoms + r[ kMolAtomBase ];
        o->circlePatchNb           = r[ kMolTori ];
        o->circlePosition          = b.torPos + r[ kMolToriBase ];
        o->circleAxis              = b.torAxis + r[ kMolToriBase ];
        o->circleVs                = b.torVs + r[ kMolToriBase ];
        o->concavePatchNb          = r[ kMolProbes ];
        o->concavePatchesPosition  = b.probePos + r[ kMolProbeBase ];
        o->concavePatchesId        = b.probeIds + r[ kMolProbeBase ];
        o->concavePatchesNeighbors = b.probeNbrs + (size_t)kMaxProbeNbr * r[ kMolSingularBase ];
        return SESGB_OK;
    }
}
