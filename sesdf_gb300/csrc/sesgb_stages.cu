// sesgb_stages.cu -- the kernels of the SES build (full surface and exterior only).
//
// Stage map (reference functions restated, file:line of PlathC/SESDF):
//   k_hash / radix sort / k_gather   AccelerationGrid::build, computeHashes, buildAccelerationGrid
//                            (sesdf/src/cuda/grid.cu:15-132) -- same cell hash and stable order
//   k_neighbors              findCirclesBetweenAtoms (sesdf/src/sesdf/operations.cu:34-124)
//   k_visibility (+ _band, _final)   computeCirclesVisibilityStatus (operations.cu:126-204; ssesdf :169-244)
//   k_emit                   scans of findCircles + buildConvexPatchesSectors
//                            (sesdf/include/bcs/sesdf/operations.inl:46-93,175-228)
//   k_probes / k_probe_jobs  findIntersectionsBetweenCircles (operations.inl:230-486; ssesdf operation.inl:100-351)
//   k_place/k_lists          thrust::sort by |w| + fillIntersections (operations.inl:128-141; operations.cu:206-269;
//                            ssesdf/operations.cu:287-329)
//   k_segment_counts/k_segments      buildConicPatches + buildSegments (operations.inl:488-668)
//   k_probe_neighbors        handleIntersectionSingularities + findIntersectionsNeighbors (operations.cu:14-32,271-338)
//   k_tori_count/k_tori      fillCircles (ssesdf/operations.cu:246-285)
//   k_sdf                    signed distance at query points and its adjoint (no reference counterpart)
//
// Every predicate is first evaluated in float32 in coordinates relative to the
// owning atom; when its margin is inside a conservative band (kRel times the
// magnitudes involved, about 30x the float32 error bound) it is decided again,
// in float-float (pairs of float32 with an a-priori error bound) where that
// settles it and otherwise by the double-precision twin in sesgb_device.cuh,
// which evaluates the reference's formula exactly as the FP64 oracle does.
#include <atomic>
#include <cfloat>

#include "sesgb_stages.cuh"

namespace sesgb
{
    namespace
    {
        constexpr float kRel = 1.0f / 65536.0f;

        __device__ __forceinline__ int3 fine_cell( const FineGrid & g, float x, float y, float z )
        {
            int cx = (int)floorf( ( x - g.origin.x ) / g.h );
            int cy = (int)floorf( ( y - g.origin.y ) / g.h );
            int cz = (int)floorf( ( z - g.origin.z ) / g.h );
            cx     = cx < 0 ? 0 : ( cx >= g.dims.x ? g.dims.x - 1 : cx );
            cy     = cy < 0 ? 0 : ( cy >= g.dims.y ? g.dims.y - 1 : cy );
            cz     = cz < 0 ? 0 : ( cz >= g.dims.z ? g.dims.z - 1 : cz );
            return make_int3( cx, cy, cz );
        }
        __device__ __forceinline__ uint32_t fine_key( const FineGrid & g, int3 c )
        {
            return ( (uint32_t)c.z * (uint32_t)g.dims.y + (uint32_t)c.y ) * (uint32_t)g.dims.x + (uint32_t)c.x;
        }

        // The 27 cells around c as 9 rows of up to three x-adjacent cells, each a
        // contiguous range of the cell-ordered item array. Lane r < 9 computes row r;
        // every lane receives all nine (start, exclusive prefix) pairs.
        struct Rows
        {
            uint32_t start[ 9 ];
            uint32_t pre[ 9 ];
            uint32_t total;
        };
        __device__ __forceinline__ void stencil_rows( const FineGrid & g, const uint32_t * cellStart, int3 c, Rows & rows )
        {
            const uint32_t lane = lane_id();
            uint32_t       st = 0, len = 0;
            if ( lane < 9 )
            {
                const int y = c.y + (int)( lane % 3 ) - 1;
                const int z = c.z + (int)( lane / 3 ) - 1;
                if ( y >= 0 && z >= 0 && y < g.dims.y && z < g.dims.z )
                {
                    const int      x0 = c.x > 0 ? c.x - 1 : 0;
                    const int      x1 = c.x + 1 < g.dims.x ? c.x + 1 : g.dims.x - 1;
                    const uint32_t c0 = fine_key( g, make_int3( x0, y, z ) );
                    const uint32_t c1 = fine_key( g, make_int3( x1, y, z ) );
                    st                = cellStart[ c0 ];
                    len               = cellStart[ c1 + 1 ] - st;
                }
            }
            uint32_t       total;
            const uint32_t pre = warp_exclusive_sum( len, total );
#pragma unroll
            for ( int r = 0; r < 9; r++ )
            {
                rows.start[ r ] = __shfl_sync( 0xffffffffu, st, r );
                rows.pre[ r ]   = __shfl_sync( 0xffffffffu, pre, r );
            }
            rows.total = total;
        }
        __device__ __forceinline__ uint32_t row_item( const Rows & rows, uint32_t f )
        {
            int r = 0;
#pragma unroll
            for ( int q = 1; q < 9; q++ )
                r = rows.pre[ q ] <= f ? q : r;
            return rows.start[ r ] + ( f - rows.pre[ r ] );
        }

        template<class T> __device__ void warp_bitonic_sort( T * a, uint32_t count, uint32_t capacity, T pad )
        {
            const uint32_t lane = lane_id();
            uint32_t       n2   = 32;
            while ( n2 < count )
                n2 <<= 1;
            if ( n2 > capacity )
                n2 = capacity;
            for ( uint32_t idx = count + lane; idx < n2; idx += 32 )
                a[ idx ] = pad;
            __syncwarp();
            for ( uint32_t k = 2; k <= n2; k <<= 1 )
                for ( uint32_t j = k >> 1; j > 0; j >>= 1 )
                {
                    for ( uint32_t idx = lane; idx < n2; idx += 32 )
                    {
                        const uint32_t ixj = idx ^ j;
                        if ( ixj > idx )
                        {
                            const bool asc = ( idx & k ) == 0;
                            const T    x   = a[ idx ];
                            const T    y   = a[ ixj ];
                            if ( ( x > y ) == asc )
                            {
                                a[ idx ] = y;
                                a[ ixj ] = x;
                            }
                        }
                    }
                    __syncwarp();
                }
        }

        // Bitonic sort of up to 64 keys held in registers, two per lane: key
        // index lane + 32 r is held in v[r]; ascending on return. The network is
        // unrolled at compile time for 32 and for 64 keys (the partner distance and
        // direction of every step are constants): the loop form with a run-time size
        // cost the neighbour search ~54 us per 100k atoms, most of it loop control.
        template<class T, bool kTwo> __device__ __forceinline__ void warp_sort_net( T & v0, T & v1 )
        {
            const uint32_t     lane = lane_id();
            constexpr uint32_t top  = kTwo ? 64u : 32u;
#pragma unroll
            for ( uint32_t k = 2; k <= top; k <<= 1 )
            {
#pragma unroll
                for ( uint32_t j = k >> 1; j > 0; j >>= 1 )
                {
                    if ( j == 32 )
                    {
                        // partner in the lane's other register; k == 64: ascending
                        const T lo = min( v0, v1 ), hi = max( v0, v1 );
                        v0         = lo;
                        v1         = hi;
                        continue;
                    }
                    const bool lower = ( lane & j ) == 0;
                    {
                        const T    p   = __shfl_xor_sync( 0xffffffffu, v0, j );
                        const bool asc = ( lane & k ) == 0;
                        v0             = ( lower == asc ) ? min( v0, p ) : max( v0, p );
                    }
                    if ( kTwo )
                    {
                        const T    p   = __shfl_xor_sync( 0xffffffffu, v1, j );
                        const bool asc = ( ( lane + 32u ) & k ) == 0;
                        v1             = ( lower == asc ) ? min( v1, p ) : max( v1, p );
                    }
                }
            }
        }
        template<class T> __device__ __forceinline__ void warp_sort64( T & v0, T & v1, bool two )
        {
            if ( two )
                warp_sort_net<T, true>( v0, v1 );
            else
                warp_sort_net<T, false>( v0, v1 );
        }

        // ---- molecules of a batch ---------------------------------------------
        __device__ __forceinline__ uint32_t mol_of( const Build & b, uint32_t sortedAtom )
        {
            return b.nMol > 1 ? b.keys[ sortedAtom ] >> b.molShift : 0u;
        }
        __device__ __forceinline__ GridRef grid_of( const Build & b, uint32_t m ) { return b.nMol > 1 ? b.gridM[ m ] : b.grid; }
        __device__ __forceinline__ uint32_t cell_base( const Build & b, uint32_t m ) { return b.nMol > 1 ? b.cellBase[ m ] : 0u; }
        // last molecule whose first atom is <= a (empty molecules are skipped)
        __device__ __forceinline__ uint32_t mol_of_index( const Build & b, uint32_t a )
        {
            uint32_t lo = 0, hi = b.nMol;
            while ( hi - lo > 1 )
            {
                const uint32_t mid = ( lo + hi ) >> 1;
                if ( b.molStart[ mid ] <= a )
                    lo = mid;
                else
                    hi = mid;
            }
            return lo;
        }

        // ------------------------------------------------------------------
        __global__ void k_hash( Build b )
        {
            pdl_begin();
            const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
            if ( i >= b.n )
                return;
            const float4   a = b.atomsIn[ i ];
            const uint32_t m = b.nMol > 1 ? mol_of_index( b, i ) : 0u;
            const GridRef  g = grid_of( b, m );
            const int3     p = ref_grid_position( g, a.x, a.y, a.z );
            if ( p.x < 0 || p.y < 0 || p.z < 0 || p.x >= g.size || p.y >= g.size || p.z >= g.size )
                atomicAdd( &b.counts->outside, 1u );
            b.keys[ i ] = ( m << b.molShift ) | ref_grid_hash( g, p );
            b.perm[ i ] = i;
            atomicMax( reinterpret_cast<int *>( &b.counts->rmax ), __float_as_int( fmaxf( a.w, 0.f ) ) );
        }

        // thread per molecule: neighbour-grid geometry from the molecule's reference grid box
        __global__ void k_fine_params( Build b, float cutoff, int span )
        {
            pdl_begin();
            if ( cutoff < 0.f )
                cutoff = 2.f * ( b.counts->rmax + b.rp ) + 0.01f;
            for ( uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < b.nMol; m += gridDim.x * blockDim.x )
            {
                const GridRef  gr  = grid_of( b, m );
                const uint32_t cap = b.nMol > 1 ? b.cellBase[ m + 1 ] - b.cellBase[ m ] : b.capCells;
                const float    ex = gr.cell.x * gr.size, ey = gr.cell.y * gr.size, ez = gr.cell.z * gr.size;
                float          h  = cutoff / (float)span;
                int3           d;
                for ( int it = 0; it < 200; it++ )
                {
                    d = make_int3( max( 1, (int)ceilf( ex / h ) ), max( 1, (int)ceilf( ey / h ) ), max( 1, (int)ceilf( ez / h ) ) );
                    if ( (uint64_t)d.x * d.y * d.z <= cap )
                        break;
                    h *= 1.1f;
                }
                FineGrid g;
                g.origin    = gr.origin;
                g.h         = h;
                g.dims      = d;
                g.cells     = (uint32_t)( (uint64_t)d.x * d.y * d.z );
                g.span      = span;
                b.fine[ m ] = g;
                if ( m == 0 )
                {
                    b.counts->fineCells = g.cells;
                    b.counts->fineCell  = h;
                }
            }
        }

        // zeroes a[0, n] and c[0, n] (c may be null), n = min(*nDevice, nHost) or nHost
        __global__ void k_zero2( uint32_t * a, uint32_t * c, uint32_t nHost, const uint32_t * nDevice )
        {
            pdl_begin();
            const uint32_t n = ( nDevice ? min( *nDevice, nHost ) : nHost ) + 1u;
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x )
            {
                a[ q ] = 0u;
                if ( c )
                    c[ q ] = 0u;
            }
        }

        __global__ void k_gather( Build b )
        {
            pdl_begin();
            const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
            if ( s >= b.n )
                return;
            b.atoms[ s ] = b.atomsIn[ b.perm[ s ] ];
        }

        // item q of a cell sort: kind 0 the sorted atom q, kind 1 the singular probe q
        __device__ __forceinline__ float4 cell_item( const Build & b, int kind, uint32_t q, uint32_t & key )
        {
            float4   p;
            uint32_t m = 0;
            if ( kind == 0 || kind == 2 )
            {
                p = b.atoms[ q ];
                m = mol_of( b, q );
                // kind 2 (SDF queries): the sign of the radius marks an atom without any
                // accessible surface (neighbours present, every circle buried)
                if ( kind == 2 && b.visCnt[ q ] == 0 && b.nbrCount[ q ] > 0 )
                    p.w = -p.w;
            }
            else
            {
                const uint32_t pi = b.nMol > 1 ? b.singList[ q ] : q;
                p                 = b.probePos[ pi ];
                if ( b.nMol > 1 )
                    m = mol_of( b, (uint32_t)b.probeIds[ pi ].x );
                // singular probes: w holds the reference-grid hash of the position, the
                // sort key of the probe in its neighbours' lists (k_probe_neighbors)
                const GridRef gr = grid_of( b, m );
                p.w              = __uint_as_float( ref_grid_hash( gr, ref_grid_position( gr, p.x, p.y, p.z ) ) );
            }
            const FineGrid g = b.fine[ m ];
            key              = cell_base( b, m ) + fine_key( g, fine_cell( g, p.x, p.y, p.z ) );
            return p;
        }

        __global__ void k_cell_count( Build b, int kind, uint32_t nHost, const uint32_t * nDevice )
        {
            pdl_begin();
            const uint32_t n = nDevice ? min( *nDevice, nHost ) : nHost;
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x )
            {
                uint32_t key;
                cell_item( b, kind, q, key );
                atomicAdd( &b.cellCount[ key ], 1u );
            }
        }

        __global__ void k_cell_scatter( Build b, int kind, uint32_t nHost, const uint32_t * nDevice )
        {
            pdl_begin();
            const uint32_t n = nDevice ? min( *nDevice, nHost ) : nHost;
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x )
            {
                uint32_t       key;
                const float4   p   = cell_item( b, kind, q, key );
                const uint32_t idx = b.cellStart[ key ] + atomicAdd( &b.cellCursor[ key ], 1u );
                b.cellItems[ idx ] = q;
                b.cellPos[ idx ]   = p;
            }
        }

        // ---- neighbour lists ---------------------------------------------
        // The double-precision twins of the float32 screens below are out of line: their
        // float-to-double conversions then run only in the rare band branch instead of
        // being hoisted into every warp (the FP64 pipe of GB300 issues one warp
        // instruction per 64 cycles).
        __device__ __noinline__ bool neighbor_d( float4 ai, float4 aj, float rp )
        {
            return dneighbor( D3( ai ), ai.w, D3( aj ), aj.w, (double)rp );
        }
        __device__ __noinline__ bool probe_pair_d( float4 pq, float4 pp, float rp )
        {
            const d3 dd = dsub( D3( pq ), D3( pp ) );
            return __dsqrt_rn( ddot( dd, dd ) ) < 2.0 * (double)rp;
        }

        // The 25 rows of a span-2 stencil (cells of at least half the largest pair cutoff) around
        // atom position p, each cut to the x-range that can hold a neighbour of the atom: a
        // neighbour j lies within cut = R_i + R_max (+ margins) of p, so a row (y, z) whose cells
        // keep |dy|, |dz| >= ey, ez from p only needs x within sqrt(cut^2 - ey^2 - ez^2) of p.
        // Lane r < 25 computes row r; the rows' first items and exclusive prefixes go to shared
        // memory (start[25], pre[26] with pre[25] = total), and the total is returned. A cell two
        // beyond the atom's own along any axis starts at least 2h >= the largest pair cutoff away.
        __device__ __forceinline__ uint32_t stencil_rows_span2( const FineGrid & g, const uint32_t * cellStart, float4 p,
                                                                float cut, uint32_t * start, uint32_t * pre )
        {
            const uint32_t lane = lane_id();
            const int3     c    = fine_cell( g, p.x, p.y, p.z );
            uint32_t       st = 0, len = 0;
            if ( lane < 25u )
            {
                const int y = c.y + (int)( lane % 5u ) - 2;
                const int z = c.z + (int)( lane / 5u ) - 2;
                if ( y >= 0 && z >= 0 && y < g.dims.y && z < g.dims.z )
                {
                    const float ylo = g.origin.y + (float)y * g.h, zlo = g.origin.z + (float)z * g.h;
                    const float ey  = fmaxf( 0.f, fmaxf( ylo - p.y, p.y - ( ylo + g.h ) ) );
                    const float ez  = fmaxf( 0.f, fmaxf( zlo - p.z, p.z - ( zlo + g.h ) ) );
                    const float w2  = cut * cut - ey * ey - ez * ez;
                    if ( w2 >= 0.f )
                    {
                        const float w  = sqrtf( w2 ) + 0.01f;
                        int         x0 = (int)floorf( ( p.x - w - g.origin.x ) / g.h );
                        int         x1 = (int)floorf( ( p.x + w - g.origin.x ) / g.h );
                        x0             = max( x0, max( c.x - 2, 0 ) );
                        x1             = min( x1, min( c.x + 2, g.dims.x - 1 ) );
                        if ( x0 <= x1 )
                        {
                            st  = cellStart[ fine_key( g, make_int3( x0, y, z ) ) ];
                            len = cellStart[ fine_key( g, make_int3( x1, y, z ) ) + 1 ] - st;
                        }
                    }
                }
            }
            uint32_t       total;
            const uint32_t ex = warp_exclusive_sum( len, total );
            if ( lane < 25u )
            {
                start[ lane ] = st;
                pre[ lane ]   = ex;
            }
            if ( lane == 0 )
                pre[ 25 ] = total;
            __syncwarp();
            return total;
        }
        // cell-item index of stencil item f (f < total): the last row whose prefix is <= f
        __device__ __forceinline__ uint32_t row_item_span2( const uint32_t * start, const uint32_t * pre, uint32_t f )
        {
            uint32_t r = 0;
#pragma unroll
            for ( uint32_t step = 16; step > 0; step >>= 1 )
                if ( r + step < 25u && pre[ r + step ] <= f )
                    r += step;
            return start[ r ] + ( f - pre[ r ] );
        }

        template<int W>
        __global__ void __launch_bounds__( 32 * W ) k_neighbors( Build b )
        {
            pdl_begin();
            __shared__ uint32_t buf[ W ][ kNbrBuf ];
            __shared__ uint32_t rowStart[ W ][ 25 ], rowPre[ W ][ 26 ];
            const uint32_t      warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t      i    = blockIdx.x * W + warp;
            if ( i >= b.n )
                return;
            const uint32_t   m     = mol_of( b, i );
            const FineGrid   g     = b.fine[ m ];
            const float4     ai    = b.atoms[ i ];
            const uint32_t * cells = b.cellStart + cell_base( b, m );
            const bool       span2 = g.span == 2;
            Rows             rows;
            uint32_t         total;
            if ( span2 )
                total = stencil_rows_span2( g, cells, ai, ( ai.w + b.rp ) + ( b.counts->rmax + b.rp ) + 0.01f, rowStart[ warp ],
                                            rowPre[ warp ] );
            else
            {
                stencil_rows( g, cells, fine_cell( g, ai.x, ai.y, ai.z ), rows );
                total = rows.total;
            }
            const float Ri    = ai.w + b.rp;
            uint32_t    count = 0, fp64 = 0;
            for ( uint32_t base0 = 0; base0 < total; base0 += 64 )
            {
                // two rows of 32 items: the loads of both issued before their use
                uint32_t jj[ 2 ] = { 0u, 0u };
                float4   pp[ 2 ];
#pragma unroll
                for ( int h = 0; h < 2; h++ )
                {
                    const uint32_t f = base0 + 32 * h + lane;
                    if ( f < total )
                    {
                        const uint32_t idx = span2 ? row_item_span2( rowStart[ warp ], rowPre[ warp ], f ) : row_item( rows, f );
                        jj[ h ]            = b.cellItems[ idx ];
                        pp[ h ]            = b.cellPos[ idx ];
                    }
                }
#pragma unroll
                for ( int h = 0; h < 2; h++ )
                {
                    const uint32_t base = base0 + 32 * h;
                    if ( base >= total )
                        break;
                    const uint32_t f    = base + lane;
                    bool           pass = false;
                    const uint32_t j    = jj[ h ];
                    if ( f < total && j != i )
                    {
                        const float4 aj = pp[ h ];
                        const f3     dj = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
                        const float  d  = dot( dj, dj );
                        const float  R  = Ri + ( aj.w + b.rp );
                        const float  m  = d - R * R - 1e-4f;
                        const float  e  = kRel * ( d + R * R + 1.f );
                        if ( m < -e )
                            pass = true;
                        else if ( m <= e )
                        {
                            pass = neighbor_d( ai, aj, b.rp );
                            fp64++;
                        }
                    }
                    const uint32_t mask = __ballot_sync( 0xffffffffu, pass );
                    const uint32_t pos  = count + __popc( mask & lanemask_lt() );
                    if ( pass && pos < kNbrBuf )
                        buf[ warp ][ pos ] = j;
                    count += __popc( mask );
                }
            }
            __syncwarp();
            const uint32_t held = count < kNbrBuf ? count : kNbrBuf;
            const uint32_t kept = held < b.cap ? held : b.cap;
            if ( held <= 64 )
            {
                // in registers (the common case)
                uint32_t v0 = lane < held ? buf[ warp ][ lane ] : 0xffffffffu;
                uint32_t v1 = lane + 32 < held ? buf[ warp ][ lane + 32 ] : 0xffffffffu;
                warp_sort64( v0, v1, held > 32 );
                if ( lane < kept )
                    b.nbr[ (size_t)i * b.cap + lane ] = v0;
                if ( lane + 32 < kept )
                    b.nbr[ (size_t)i * b.cap + lane + 32 ] = v1;
            }
            else
            {
                warp_bitonic_sort<uint32_t>( buf[ warp ], held, kNbrBuf, 0xffffffffu );
                for ( uint32_t s = lane; s < kept; s += 32 )
                    b.nbr[ (size_t)i * b.cap + s ] = buf[ warp ][ s ];
            }
            for ( int o = 16; o > 0; o >>= 1 )
                fp64 += __shfl_xor_sync( 0xffffffffu, fp64, o );
            if ( lane == 0 )
            {
                b.nbrCount[ i ] = kept;
                // every warp updating one counter serialised the kernel's ends on its L2 atomics:
                // a warp whose count is not above the maximum already seen skips the update
                if ( count > *(volatile uint32_t *)&b.counts->maxNbr )
                    atomicMax( &b.counts->maxNbr, count );
                if ( count > b.cap )
                    atomicAdd( &b.counts->nbrTruncated, 1u );
                if ( count > kNbrBuf )
                    atomicOr( &b.counts->overflow, (uint32_t)kOverflowNbr );
                if ( fp64 )
                    atomicAdd( &b.counts->fp64[ kFp64Neighbor ], fp64 );
            }
        }

        // slot of target in an ascending neighbour row, or -1
        __device__ __forceinline__ int find_in_row( const uint32_t * row, uint32_t len, uint32_t target )
        {
            uint32_t lo = 0, hi = len;
            while ( lo < hi )
            {
                const uint32_t mid = ( lo + hi ) >> 1;
                if ( row[ mid ] < target )
                    lo = mid + 1;
                else
                    hi = mid;
            }
            return ( lo < len && row[ lo ] == target ) ? (int)lo : -1;
        }

        // ---- circle visibility ----------------------------------------------
        // Warp per atom i, lane per circle (i, s): every lane tests its circle
        // against the same k in turn. The neighbourhood is staged in shared memory
        // as (d_k, K_k, |d_k|^2) relative to atom i; a test is then sqrt- and
        // division-free: with t the axial offset of the circle (centre c = t d_j),
        // g = d_j . d_k and p^2 = |d_k|^2 - g^2 / |d_j|^2 (k's distance from the
        // circle axis, squared)
        //     A = R_i^2 + |d_k|^2 - R_k^2 - 1e-4 - 2 t g      (= |c - d_k|^2 + r^2 - R_k^2 - 1e-4)
        //     G = A^2 - 4 r^2 p^2,
        // k holds the whole circle iff A < 0 and G > 0 and touches it iff A < 0
        // or G < 0 (the two extremes A +- 2 r p of computeCirclesVisibilityStatus,
        // operations.cu:164-197). Tests inside the float32 error band go to a
        // queue that k_visibility_band decides in double precision with full
        // warps; k_visibility_final turns the flags into statuses and counts.
        constexpr int kVisQueue   = 128;            // band tests a warp holds before they go to the global queue
        constexpr int kMaskSlots  = 64;             // atoms with at most this many neighbours keep touch masks

        // status flags between the three visibility kernels
        enum : uint8_t
        {
            kVisBuried    = 1,
            kVisTouched   = 2,
            kVisEvaluated = 4,
            kVisUpper     = 8,  // circle (i, j) with i < j: its touch mask is kept
            kVisMirror    = 16, // circle (i, j), j < i, of two complete lists: takes the status of (j, i)
        };

        __host__ __device__ inline uint32_t staged_rows( uint32_t cap ) { return cap < (uint32_t)kNbrBuf ? cap : (uint32_t)kNbrBuf; }

        struct VisSmem
        {
            float4 *   rel;   // rows + 32: d_k, R_i^2 + |d_k|^2 - R_k^2 - 1e-4 (padding: never touches)
            float *    dd;    // rows + 32: |d_k|^2
            uint8_t *  res;   // rows: kVis* flags
            uint16_t * list;  // rows: circles to evaluate
            uint32_t * queue; // kVisQueue: s | k << 16
        };

        __host__ __device__ inline size_t vis_smem_per_warp( uint32_t cap )
        {
            const size_t r = staged_rows( cap ) + 32;
            return ( ( r * ( 16 + 4 + 1 + 2 ) + 15 ) & ~(size_t)15 ) + kVisQueue * 4;
        }

        __device__ inline VisSmem vis_smem( unsigned char * base, uint32_t cap )
        {
            const size_t r = staged_rows( cap ) + 32;
            VisSmem      m;
            m.rel   = reinterpret_cast<float4 *>( base );
            m.dd    = reinterpret_cast<float *>( base + r * 16 );
            m.res   = base + r * 20;
            m.list  = reinterpret_cast<uint16_t *>( base + ( ( r * 21 + 1 ) & ~(size_t)1 ) );
            m.queue = reinterpret_cast<uint32_t *>( base + ( ( r * 23 + 15 ) & ~(size_t)15 ) );
            return m;
        }

        // Per-circle constants of the test, with the error bands: every float32
        // rounding of A stays below eA = kRel Mc and every rounding of G below
        // alpha |A| + beta p^2 + gamma, Mc bounding R_i^2 + |d_k|^2 + R_k^2 + 2 |c| |d_k| + 1
        // over the atom's neighbours. theta: k closer to the axis than that is
        // left to double precision (infinite for a nearly tangent circle).
        struct VisCircle
        {
            f3    dj;
            float m2t, inv, r2x4, eA, alpha, beta, gamma, theta;
        };

        __device__ __forceinline__ VisCircle vis_circle( float Ri, float Mc, float theta, const float4 & q, float dJ )
        {
            VisCircle   v;
            v.dj              = F3( q.x, q.y, q.z );
            const float t     = __fdividef( q.w + 1e-4f, 2.f * dJ ); // (R_i^2 - R_j^2 + |d_j|^2) / (2 |d_j|^2)
            const f3    c     = v.dj * t;
            const float r2raw = Ri * Ri - dot( c, c );
            const float r2    = fmaxf( r2raw, 0.f );
            // (nearly) tangent SAS spheres: the reference's circle radius is
            // sqrt of a negative number (NaN) and every test of the circle is
            // false; the double-precision twin decides whether that happens
            v.theta = r2raw <= 4.f * kRel * Ri * Ri ? __int_as_float( 0x7f800000 ) : theta;
            v.m2t   = -2.f * t;
            v.inv   = __fdividef( 1.f, dJ );
            v.r2x4  = 4.f * r2;
            v.eA    = kRel * Mc;
            v.alpha = 3.f * kRel * Mc;
            v.beta  = 4.f * kRel * ( r2 + Mc );
            v.gamma = 4.f * kRel * Mc * r2;
            return v;
        }

        // double-precision twin of one test (computeCirclesVisibilityStatus in IEEE double)
        __device__ __noinline__ int circle_test_d( const Build & b, const float4 & ai, uint32_t i, uint32_t s, uint32_t k )
        {
            const float4  aj = b.atoms[ b.nbr[ (size_t)i * b.cap + s ] ];
            const float4  ak = b.atoms[ b.nbr[ (size_t)i * b.cap + k ] ];
            const dcircle dc = dcircle_geometry( D3( ai ), ai.w, D3( aj ), aj.w, (double)b.rp );
            return dcircle_vs_atom( dc, D3( ak ), __dadd_rn( (double)ak.w, (double)b.rp ) );
        }

        // circle_test_d in float-float: the same quantities (circle geometry of
        // getCircleGeometry, then the two extremes first = r +- p, complete =
        // first^2 + second^2 of computeCirclesVisibilityStatus, operations.cu:164-197)
        // with a bound on their distance from the exact values that also covers the
        // double-precision twin's own rounding (its sqrt(1 - cos^2) loses half the
        // digits next to the axis). Returns the bits when both tests are farther than
        // that from the 1e-4 threshold, -1 otherwise (the caller then decides in
        // double precision).
        __device__ int circle_test_ff( const float4 & ai, const float4 & aj, const float4 & ak, float rp )
        {
            const ff R1 = two_sum( ai.w, rp ), R2 = two_sum( aj.w, rp ), Rk = two_sum( ak.w, rp );
            const ff dx = two_sum( aj.x, -ai.x ), dy = two_sum( aj.y, -ai.y ), dz = two_sum( aj.z, -ai.z ); // c_j - c_i
            const ff d  = ff_add( ff_add( ff_mul( dx, dx ), ff_mul( dy, dy ) ), ff_mul( dz, dz ) );
            if ( !( d.hi > 0.f ) )
                return -1;
            const ff R12 = ff_mul( R1, R1 );
            const ff tt  = ff_div( ff_add( ff_sub( R12, ff_mul( R2, R2 ) ), d ), ff_scale( d, 2.f ) );
            // circle centre relative to c_i: t (c_j - c_i); radius^2 = R1^2 - t^2 d
            const ff ccx = ff_mul( dx, tt ), ccy = ff_mul( dy, tt ), ccz = ff_mul( dz, tt );
            const ff r2  = ff_sub( R12, ff_mul( ff_mul( tt, tt ), d ) );
            if ( !( r2.hi > 0.f ) )
                return -1;
            const ff rad = ff_sqrt( r2 );
            const ff inv = ff_div( ff_of( 1.f ), ff_sqrt( d ) );
            const ff nx = ff_mul( dx, inv ), ny = ff_mul( dy, inv ), nz = ff_mul( dz, inv );
            // centre - c_k
            const ff kx = ff_add( ccx, two_sum( ai.x, -ak.x ) ), ky = ff_add( ccy, two_sum( ai.y, -ak.y ) ), kz = ff_add( ccz, two_sum( ai.z, -ak.z ) );
            const ff k2   = ff_add( ff_add( ff_mul( kx, kx ), ff_mul( ky, ky ) ), ff_mul( kz, kz ) );
            if ( !( k2.hi > 0.f ) )
                return -1;
            const ff dist = ff_sqrt( k2 );
            const ff sec  = ff_add( ff_add( ff_mul( kx, nx ), ff_mul( ky, ny ) ), ff_mul( kz, nz ) );
            const ff cs   = ff_div( sec, dist );
            const ff s2   = ff_sub( ff_of( 1.f ), ff_mul( cs, cs ) );
            if ( !( s2.hi > 0.f ) )
                return -1;
            const ff sn   = ff_sqrt( s2 );
            const ff p    = ff_mul( sn, dist ); // distance of c_k from the circle's axis
            const ff sec2 = ff_mul( sec, sec );
            const ff Rk2  = ff_mul( Rk, Rk );
            const ff tol  = ff_of( 1e-4f );
            const ff fp = ff_add( p, rad ), fm = ff_add( ff_neg( p ), rad );
            const ff vp = ff_sub( ff_sub( ff_add( ff_mul( fp, fp ), sec2 ), Rk2 ), tol );
            const ff vm = ff_sub( ff_sub( ff_add( ff_mul( fm, fm ), sec2 ), Rk2 ), tol );
            // bound: u per operation on the magnitudes involved (u = 2^-42 covers the
            // float-float chain, far more than the double one), plus the conditioning
            // of the radius (cancellation in R1^2 - t^2 d) and of sin(theta) near the
            // axis, for float-float (u / sin, at most 2 sqrt(u)) and for double
            // (2^-50 / sin, at most 2^-24)
            const float u   = 2.2737367544323206e-13f;
            const float F   = fabsf( fp.hi ), D = dist.hi, R = rad.hi, S = sn.hi;
            const float mag = F * F + sec2.hi + Rk2.hi + R12.hi + d.hi + 2.f * F * D;
            const float eSin = fminf( 4.f * u / S, 2.f * sqrtf( u ) ) + fminf( 8.8817842e-16f / S, 5.9604645e-08f );
            const float E    = 64.f * u * mag + 2.f * F * ( 64.f * u * R12.hi / R ) + 2.f * F * D * eSin;
            if ( !( fabsf( vp.hi ) > E && fabsf( vm.hi ) > E ) )
                return -1;
            return ( vp.hi < 0.f ? 1 : 0 ) | ( vm.hi < 0.f ? 2 : 0 );
        }

        // one test to the global double-precision queue (capacity exceeded: the build is redone larger)
        __device__ __forceinline__ void band_push( const Build & b, uint32_t i, uint32_t sk )
        {
            const uint32_t at = atomicAdd( &b.counts->visBand, 1u );
            if ( at < b.capVisBand )
                b.visBand[ at ] = make_uint2( i, sk );
            else
                atomicOr( &b.counts->overflow, (uint32_t)kOverflowVisBand );
        }

        struct UnitStride
        {
        };
        __device__ __forceinline__ uint32_t operator*( UnitStride, uint32_t u ) { return u; }

        // W warps (atoms) per block; one by default, as k_probes: a slot is freed when its atom is done
        template<int W>
        __global__ void __launch_bounds__( 32 * W, 32 / W ) k_visibility( Build b )
        {
            pdl_begin();
            extern __shared__ __align__( 16 ) unsigned char smemRaw[];
            const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t i    = blockIdx.x * W + warp;
            if ( i >= b.n )
                return;
            const VisSmem  m   = vis_smem( smemRaw + warp * vis_smem_per_warp( b.cap ), b.cap );
            const uint32_t ni  = b.nbrCount[ i ];
            const float4   ai  = b.atoms[ i ];
            const float    Ri  = ai.w + b.rp;
            const size_t   row = (size_t)i * b.cap;

            // stage the neighbourhood (padded by 32 far slots) and the list of
            // circles to evaluate: circles (i, j) with i < j, and in the full build
            // also the circles (i, j), j < i, of a list cut at the capacity on either
            // side. Circles (i, j) and (j, i) are one circle, and every atom that can
            // touch it is in both complete lists, so that the other lower circles take
            // the status of (j, i) in k_visibility_final (the reference evaluates both,
            // operations.cu:126-204; the two differ only inside its float32 band)
            float    d2max = 0.f, r2max = 0.f;
            uint32_t nc    = 0;
            for ( uint32_t base = 0; base < ni + 32; base += 32 )
            {
                const uint32_t s    = base + lane;
                bool           eval = false;
                if ( s < ni )
                {
                    const uint32_t j  = b.nbr[ row + s ];
                    const float4   aj = b.atoms[ j ];
                    const bool     mirror = b.mode == 0 && j < i && ni < b.cap && b.nbrCount[ j ] < b.cap;
                    const f3       d  = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
                    const float    dd = dot( d, d );
                    const float    Rk = aj.w + b.rp;
                    m.rel[ s ]        = make_float4( d.x, d.y, d.z, ( ( Ri * Ri + dd ) - Rk * Rk ) - 1e-4f );
                    m.dd[ s ]         = dd;
                    eval              = b.mode == 0 ? !mirror : i < j;
                    m.res[ s ]        = ( eval ? kVisEvaluated : 0 ) | ( i < j ? kVisUpper : 0 ) | ( mirror ? kVisMirror : 0 );
                    // the slot of i in the list of j (both complete; the neighbour predicate is
                    // symmetric), kept for k_visibility_final in slotTrim, which k_emit fills later
                    if ( mirror )
                        b.slotTrim[ row + s ] = (uint32_t)find_in_row( b.nbr + (size_t)j * b.cap, b.nbrCount[ j ], i );
                    d2max             = fmaxf( d2max, dd );
                    r2max             = fmaxf( r2max, Rk * Rk );
                }
                else if ( s < ni + 32 )
                {
                    // padding for the rounded-up test loops: far away, never undecided
                    m.rel[ s ] = make_float4( 0.f, 0.f, 0.f, 1e15f );
                    m.dd[ s ]  = 1e15f;
                }
                const uint32_t mk = __ballot_sync( 0xffffffffu, eval );
                if ( eval )
                    m.list[ nc + __popc( mk & lanemask_lt() ) ] = (uint16_t)s;
                nc += __popc( mk );
            }
            for ( int o = 16; o > 0; o >>= 1 )
            {
                d2max = fmaxf( d2max, __shfl_xor_sync( 0xffffffffu, d2max, o ) );
                r2max = fmaxf( r2max, __shfl_xor_sync( 0xffffffffu, r2max, o ) );
            }
            const float Mc    = Ri * Ri + d2max + r2max + 2.f * Ri * sqrtf( d2max ) * ( 1.f + kRel ) + 1.f;
            const float theta = kRel * ( d2max + 1.f );
            __syncwarp();

            uint32_t nq = 0;
            // Circles go 32 at a time, one per lane, each lane looping over all k
            // (the same k in every lane: shared-memory broadcasts). A last step with
            // at most 16 circles spreads the k of each circle over a group of G lanes
            // (k = lane in group + G u). (Steps of 8 or 16 circles with every lane
            // busy, instead of one step with idle lanes, measured slower on GB300.)
            for ( uint32_t c0 = 0; c0 < nc; )
            {
                const uint32_t rem = nc - c0;
                uint32_t       G   = 1;
                if ( rem < 32 )
                    while ( rem * G * 2 <= 32 )
                        G <<= 1;
                const uint32_t grp = lane / G, gl = lane % G;
                const uint32_t gmask = ( G == 32 ? 0xffffffffu : ( ( 1u << G ) - 1u ) ) << ( grp * G );
                const uint32_t ci    = c0 + grp;
                const bool     valid = grp < 32 / G && ci < nc;
                const uint32_t s     = m.list[ valid ? ci : c0 ];
                const uint32_t U     = ( ni + G - 1 ) / G; // tests per lane
                bool           bur = false, tch = false;
                uint32_t       und[ 2 ] = { 0, 0 }, tou[ 2 ] = { 0, 0 }; // bit u of word w: k = gl + G (32 w + u)
                {
                    const VisCircle v = vis_circle( Ri, Mc, theta, m.rel[ s ], m.dd[ s ] );
                    for ( uint32_t u0 = 0; u0 < U; u0 += 32 )
                    {
                        const uint32_t uN = U - u0 < 32 ? U - u0 : 32;
                        const float4 * qp = m.rel + gl + G * u0;
                        const float *  dp = m.dd + gl + G * u0;
                        uint32_t       uw = 0, tw = 0, bw = 0;
                        auto           run = [ & ]( auto stride ) {
#pragma unroll 8
                        for ( uint32_t u = 0; u < uN; u++ )
                        {
                            const float4 q  = qp[ stride * u ];
                            const float  dk = dp[ stride * u ];
                            const float  g  = v.dj.x * q.x + v.dj.y * q.y + v.dj.z * q.z;
                            const float  A  = fmaf( v.m2t, g, q.w );
                            const float  p2 = fmaf( -g * v.inv, g, dk );
                            const float  G2 = fmaf( A, A, -v.r2x4 * p2 );
                            const float  eG = fmaf( v.alpha, fabsf( A ), fmaf( v.beta, p2, v.gamma ) );
                            // false on NaN: the test is then left to double precision
                            const bool ok = ( p2 > v.theta ) & ( fabsf( A ) > v.eA ) & ( fabsf( G2 ) > eG );
                            // bits shifted in (the bit of test u ends at position uN - 1 - u); the
                            // sign bits of A and G2 go in without a compare: a decided test has
                            // A != 0 and G2 != 0, so they are A < 0 and G2 < 0 there (undecided
                            // bits are masked by uw below)
                            const uint32_t ab = __float_as_uint( A ), gb = __float_as_uint( G2 );
                            uw                = ( uw << 1 ) | (uint32_t)!ok;
                            tw                = __funnelshift_l( ab | gb, tw, 1 );  // A < 0 or G2 < 0: touches
                            bw                = __funnelshift_l( ab & ~gb, bw, 1 ); // A < 0 and G2 > 0: buries
                        }
                        };
                        if ( G == 1 )
                            run( UnitStride {} );
                        else
                            run( G );
                        // into place (bit u for test u); a decided test touches when its tw bit is set
                        uw  = __brev( uw ) >> ( 32u - uN );
                        tw  = __brev( tw ) >> ( 32u - uN );
                        bw  = __brev( bw ) >> ( 32u - uN );
                        tch = tch | ( ( tw & ~uw ) != 0u );
                        bur = bur | ( ( bw & ~uw ) != 0u );
                        tw |= uw; // an undecided test may touch (the touch mask is conservative)
                        // the circle's own j is always undecided and never tested
                        const uint32_t us = s / G;
                        if ( gl == s % G && us >= u0 && us < u0 + uN )
                            uw &= ~( 1u << ( us - u0 ) );
                        if ( !valid )
                            uw = 0;
                        if ( u0 < 64 )
                        {
                            und[ u0 / 32 ] = uw;
                            tou[ u0 / 32 ] = tw;
                        }
                        else if ( __any_sync( 0xffffffffu, uw != 0 ) )
                        {
                            // more than 64 tests per lane: these go out now (no buried filter)
                            uint32_t tot;
                            uint32_t at = nq + warp_exclusive_sum( (uint32_t)__popc( uw ), tot );
                            for ( uint32_t w = uw; w; w &= w - 1 )
                            {
                                const uint32_t k = gl + G * ( u0 + (uint32_t)( __ffs( w ) - 1 ) );
                                if ( at < (uint32_t)kVisQueue )
                                    m.queue[ at ] = s | ( k << 16 );
                                else
                                    band_push( b, i, s | ( k << 16 ) );
                                at++;
                            }
                            nq = min( nq + tot, (uint32_t)kVisQueue );
                        }
                    }
                }
                const bool gb = ( __ballot_sync( 0xffffffffu, bur ) & gmask ) != 0;
                const bool gt = ( __ballot_sync( 0xffffffffu, tch ) & gmask ) != 0;
                if ( ni <= (uint32_t)kMaskSlots )
                {
                    // touch mask of the circle over slots 0..63: the atoms that may hold
                    // a point of it (k_probes tests only those)
                    uint64_t x = 0;
                    if ( G == 1 )
                        x = (uint64_t)tou[ 0 ] | ( (uint64_t)tou[ 1 ] << 32 );
                    else
                        for ( uint32_t w = tou[ 0 ]; w; w &= w - 1 )
                            x |= 1ull << ( gl + G * (uint32_t)( __ffs( w ) - 1 ) );
                    for ( uint32_t o = 1; o < G; o <<= 1 )
                        x |= __shfl_xor_sync( 0xffffffffu, x, o );
                    if ( valid && gl == 0 && ( m.res[ s ] & kVisUpper ) )
                    {
                        const uint32_t at = b.pairOff[ i ] + s;
                        if ( at < b.capPairs )
                            b.touch[ at ] = x;
                        else
                            atomicOr( &b.counts->overflow, (uint32_t)kOverflowPairs );
                    }
                }
                if ( valid && gl == 0 && ( gb || gt ) )
                    atomicOr( reinterpret_cast<uint32_t *>( m.res ) + ( s >> 2 ),
                              (uint32_t)( ( gb ? kVisBuried : 0 ) | ( gt ? kVisTouched : 0 ) ) << ( 8 * ( s & 3 ) ) );
                // queue the undecided tests of circles not buried in float32
                if ( gb )
                    und[ 0 ] = und[ 1 ] = 0;
                if ( __any_sync( 0xffffffffu, ( und[ 0 ] | und[ 1 ] ) != 0 ) )
                {
                    uint32_t tot;
                    uint32_t at = nq + warp_exclusive_sum( (uint32_t)( __popc( und[ 0 ] ) + __popc( und[ 1 ] ) ), tot );
                    for ( uint32_t h = 0; h < 2; h++ )
                        for ( uint32_t w = und[ h ]; w; w &= w - 1 )
                        {
                            const uint32_t k = gl + G * ( 32 * h + (uint32_t)( __ffs( w ) - 1 ) );
                            if ( at < (uint32_t)kVisQueue )
                                m.queue[ at ] = s | ( k << 16 );
                            else
                                band_push( b, i, s | ( k << 16 ) ); // the warp's queue is full
                            at++;
                        }
                    nq = min( nq + tot, (uint32_t)kVisQueue );
                }
                c0 += 32 / G;
            }
            __syncwarp();
            // hand the band tests of circles not buried in float32 to the double-precision pass
            uint32_t nKeep = 0;
            for ( uint32_t e0 = 0; e0 < nq; e0 += 32 )
            {
                const uint32_t e    = e0 + lane;
                const uint32_t q    = e < nq ? m.queue[ e ] : 0u;
                const bool     keep = e < nq && !( m.res[ q & 0xffffu ] & kVisBuried );
                nKeep += __popc( __ballot_sync( 0xffffffffu, keep ) );
            }
            uint32_t qbase = 0;
            if ( lane == 0 && nKeep )
                qbase = atomicAdd( &b.counts->visBand, nKeep );
            qbase = __shfl_sync( 0xffffffffu, qbase, 0 );
            for ( uint32_t e0 = 0; e0 < nq; e0 += 32 )
            {
                const uint32_t e    = e0 + lane;
                const uint32_t q    = e < nq ? m.queue[ e ] : 0u;
                const bool     keep = e < nq && !( m.res[ q & 0xffffu ] & kVisBuried );
                const uint32_t mk   = __ballot_sync( 0xffffffffu, keep );
                const uint32_t at   = qbase + __popc( mk & lanemask_lt() );
                if ( keep && at < b.capVisBand )
                    b.visBand[ at ] = make_uint2( i, q );
                else if ( keep )
                    atomicOr( &b.counts->overflow, (uint32_t)kOverflowVisBand );
                qbase += __popc( mk );
            }
            __syncwarp();
            for ( uint32_t s = lane; s < ni; s += 32 )
                b.status[ row + s ] = m.res[ s ];
        }

        // Band tests, one per thread with full warps: float-float first, the double
        // precision twin only where that cannot decide (counted); the result bits go
        // into the circle's status flags.
        __global__ void __launch_bounds__( 128 ) k_visibility_band( Build b )
        {
            pdl_begin();
            const uint32_t nb   = min( b.counts->visBand, b.capVisBand );
            uint32_t       fp64 = 0;
            for ( uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x )
            {
                const uint2    e   = b.visBand[ t ];
                const uint32_t i   = e.x, s = e.y & 0xffffu, k = e.y >> 16;
                if ( i >= b.n || s >= b.nbrCount[ i ] || k >= b.nbrCount[ i ] )
                    continue; // not written by k_visibility
                const size_t pos = (size_t)i * b.cap + s;
                if ( b.status[ pos ] & kVisBuried )
                    continue;
                const float4 ai = b.atoms[ i ];
                const float4 aj = b.atoms[ b.nbr[ (size_t)i * b.cap + s ] ];
                const float4 ak = b.atoms[ b.nbr[ (size_t)i * b.cap + k ] ];
                int          rd = circle_test_ff( ai, aj, ak, b.rp );
                if ( rd < 0 )
                {
                    rd = circle_test_d( b, ai, i, s, k );
                    fp64++;
                }
                if ( rd & 3 )
                    atomicOr( reinterpret_cast<uint32_t *>( b.status + ( pos & ~(size_t)3 ) ), (uint32_t)( rd & 3 ) << ( 8 * ( pos & 3 ) ) );
            }
            for ( int o = 16; o > 0; o >>= 1 )
                fp64 += __shfl_xor_sync( 0xffffffffu, fp64, o );
            if ( lane_id() == 0 && fp64 )
                atomicAdd( &b.counts->fp64[ kFp64Visibility ], fp64 );
        }

        // statuses (0 buried, 1 partial, 2 complete; circles not evaluated 0) and
        // the per-atom counts; four atoms per warp, eight lanes per atom. A lane holds
        // up to eight slots of its atom in registers, so that their loads (and those
        // of the mirrored circles' statuses) are in flight together.
        __global__ void __launch_bounds__( 32 * kWarpsPerBlock ) k_visibility_final( Build b )
        {
            pdl_begin();
            constexpr uint32_t kHeld = 8;
            const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t grp = lane / 8, gl = lane % 8;
            const uint32_t i    = ( blockIdx.x * kWarpsPerBlock + warp ) * 4 + grp;
            const bool     live = i < b.n;
            const uint32_t ni   = live ? b.nbrCount[ i ] : 0u;
            const size_t   row  = (size_t)i * b.cap;
            uint32_t       vis = 0, part = 0, full = 0;
            for ( uint32_t s0 = 0; s0 < ni; s0 += 8 * kHeld )
            {
                uint32_t j[ kHeld ], r[ kHeld ], t[ kHeld ];
#pragma unroll
                for ( uint32_t h = 0; h < kHeld; h++ )
                {
                    const uint32_t s = s0 + gl + 8 * h;
                    j[ h ] = r[ h ] = 0;
                    t[ h ]          = 0xffffffffu;
                    if ( s < ni )
                    {
                        j[ h ] = b.nbr[ row + s ];
                        r[ h ] = b.status[ row + s ];
                        // the slot of i in the list of j, left in slotTrim by k_visibility
                        // for the mirrored circles (k_emit fills slotTrim later)
                        if ( b.mode == 0 )
                            t[ h ] = b.slotTrim[ row + s ];
                    }
                }
#pragma unroll
                for ( uint32_t h = 0; h < kHeld; h++ )
                    if ( ( r[ h ] & kVisMirror ) )
                    {
                        // the status of (j, i): its flags, or the status another warp already
                        // made of them (which has no kVisEvaluated bit)
                        const uint32_t q = t[ h ] < b.cap ? b.status[ (size_t)j[ h ] * b.cap + t[ h ] ] : 0u;
                        r[ h ] = ( q & kVisEvaluated ) ? q
                                                       : ( q == 0 ? kVisEvaluated | kVisBuried
                                                                  : q == 1 ? kVisEvaluated | kVisTouched : kVisEvaluated );
                    }
#pragma unroll
                for ( uint32_t h = 0; h < kHeld; h++ )
                {
                    const uint32_t s = s0 + gl + 8 * h;
                    if ( s < ni )
                    {
                        const uint8_t st = ( r[ h ] & kVisEvaluated ) ? ( ( r[ h ] & kVisBuried ) ? 0 : ( ( r[ h ] & kVisTouched ) ? 1 : 2 ) ) : 0;
                        b.status[ row + s ] = st;
                        vis += st != 0;
                        part += ( st == 1 && i < j[ h ] );
                        full += ( st == 2 && i < j[ h ] );
                    }
                }
            }
            for ( int o = 4; o > 0; o >>= 1 )
            {
                vis += __shfl_xor_sync( 0xffffffffu, vis, o );
                part += __shfl_xor_sync( 0xffffffffu, part, o );
                full += __shfl_xor_sync( 0xffffffffu, full, o );
            }
            if ( live && gl == 0 )
            {
                b.visCnt[ i ]  = vis;
                b.partCnt[ i ] = part;
                b.fullCnt[ i ] = full;
            }
        }

        __host__ inline size_t visibility_smem( uint32_t cap, int warps ) { return vis_smem_per_warp( cap ) * (size_t)warps; }

        // ---- sectors, complete circles, partial-circle numbering -----------
        // sector of buildConvexPatchesSectors (operations.inl:186-213) in
        // coordinates relative to atom i
        __device__ float4 sector_of( const Build & b, const float4 & ai, const float4 & aj )
        {
            const float rirp   = ai.w + b.rp;
            const float sqrirp = rirp * rirp;
            const f3    dj     = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
            const float Rj     = aj.w + b.rp;
            const float d      = dot( dj, dj );
            const float t      = ( rirp * rirp - Rj * Rj + d ) / ( 2.f * d );
            const f3    cij    = dj * t;
            const float radius = sqrtf( fmaxf( sqrirp - dot( cij, cij ), 0.f ) );
            const f3    cicj   = normalize( dj );
            f3          ref    = F3( 1.f, 0.f, 0.f );
            if ( fabsf( dot( cicj, ref ) ) > 1.f - 1e-4f )
                ref = F3( 0.f, 1.f, 0.f );
            const f3    nn = normalize( cross( cicj, ref ) );
            const f3    x  = cij + nn * radius;
            const float c  = fmaxf( -1.f, fminf( dot( cicj, x * ( 1.f / rirp ) ), 1.f ) );
            return make_float4( cicj.x, cicj.y, cicj.z, acosf( c ) );
        }

        // four atoms per warp, eight lanes per atom (neighbour rows of ~35 slots fill the lanes)
        constexpr uint32_t kEmitGroup = 8;

        __global__ void __launch_bounds__( 32 * kWarpsPerBlock ) k_emit( Build b )
        {
            pdl_begin();
            const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t grp = lane / kEmitGroup, gl = lane % kEmitGroup;
            const uint32_t gmask = ( ( 1u << kEmitGroup ) - 1u ) << ( grp * kEmitGroup );
            const uint32_t i     = ( blockIdx.x * kWarpsPerBlock + warp ) * ( 32 / kEmitGroup ) + grp;
            const bool     live  = i < b.n;
            const uint32_t ni    = live ? b.nbrCount[ i ] : 0u;
            const float4   ai    = live ? b.atoms[ i ] : make_float4( 0.f, 0.f, 0.f, 0.f );
            uint32_t       visBase  = live ? b.visOff[ i ] : 0u;
            uint32_t       partBase = live ? b.partOff[ i ] : 0u;
            uint32_t       fullBase = live ? b.fullOff[ i ] : 0u;
            uint32_t       most     = ni;
            for ( int o = 16; o > 0; o >>= 1 )
                most = max( most, __shfl_xor_sync( 0xffffffffu, most, o ) );
            uint32_t       ovf = 0;
            const uint32_t lt  = lanemask_lt() & gmask;
            for ( uint32_t base = 0; base < most; base += kEmitGroup )
            {
                const uint32_t s     = base + gl;
                const bool     valid = s < ni;
                const size_t   slot  = (size_t)i * b.cap + s;
                uint32_t       j     = 0;
                uint8_t        st    = 0;
                if ( valid )
                {
                    j  = b.nbr[ slot ];
                    st = b.status[ slot ];
                }
                const bool     vis  = valid && st != 0;
                const bool     part = valid && st == 1 && i < j;
                const bool     full = valid && st == 2 && i < j;
                const uint32_t mv   = __ballot_sync( 0xffffffffu, vis ) & gmask;
                const uint32_t mp   = __ballot_sync( 0xffffffffu, part ) & gmask;
                const uint32_t mf   = __ballot_sync( 0xffffffffu, full ) & gmask;
                if ( valid )
                    b.slotTrim[ slot ] = partBase + __popc( mp & lt );
                if ( vis && b.mode == 0 )
                {
                    const uint32_t idx = visBase + __popc( mv & lt );
                    if ( idx < b.capSectors )
                        b.sectors[ idx ] = sector_of( b, ai, b.atoms[ j ] );
                    else
                        ovf |= kOverflowSectors;
                }
                if ( part )
                {
                    const uint32_t t = partBase + __popc( mp & lt );
                    if ( t < b.capC1 )
                        b.trimSlot[ t ] = (uint32_t)slot;
                    else
                        ovf |= kOverflowC1;
                }
                if ( full && b.mode == 0 )
                {
                    const uint32_t f = fullBase + __popc( mf & lt );
                    if ( f < b.capFull )
                        b.fullCircles[ f ] = make_uint2( i, j );
                    else
                        ovf |= kOverflowFull;
                }
                visBase += __popc( mv );
                partBase += __popc( mp );
                fullBase += __popc( mf );
            }
            if ( live && gl == 0 && b.mode == 0 )
                b.convex[ i ] = make_uint2( b.visOff[ i ], b.visOff[ i ] + b.visCnt[ i ] );
            if ( ovf )
                atomicOr( &b.counts->overflow, ovf );
        }

        // ---- probes: enumeration, float32 screen, double-precision solve -------

        // ---- probe solve -----------------------------------------------------
        // Double-precision triplet point in closed form. With a = c_j - c_i,
        // b = c_k - c_i and n = a x b, the points at distance R_i, R_j, R_k from
        // the three centres are c_i + y0 +- n sqrt(h2 / |n|^2), where
        // y0 = (p (b x n) + q (n x a)) / |n|^2 lies in the plane of the centres
        // (a . y0 = p = (|a|^2 + R_i^2 - R_j^2) / 2, b . y0 = q likewise) and
        // h2 = R_i^2 - |y0|^2. The reference intersects the circles (i, j) and
        // (i, k) for the same points (findIntersectionsBetweenCircles,
        // operations.inl:384-398); the closed form takes one division and one
        // root instead of six and four. h is also the distance of the points
        // from the plane of the centres, the quantity of the singular test.
        // Returns false when h2 < 0 (no point), as the reference's t < 0.
        __device__ __forceinline__ bool solve_d( d3 ci, double ri, d3 cj, double rj, d3 ck, double rk, double rp, d3 & x1, d3 & x2,
                                                 double & h2 )
        {
            const d3     a  = dsub( cj, ci ), bv = dsub( ck, ci );
            const d3     n  = dcross( a, bv );
            const double Ri = __dadd_rn( ri, rp ), Rj = __dadd_rn( rj, rp ), Rk = __dadd_rn( rk, rp );
            const double Ri2 = __dmul_rn( Ri, Ri );
            const double p   = __dmul_rn( __dsub_rn( __dadd_rn( ddot( a, a ), Ri2 ), __dmul_rn( Rj, Rj ) ), 0.5 );
            const double q   = __dmul_rn( __dsub_rn( __dadd_rn( ddot( bv, bv ), Ri2 ), __dmul_rn( Rk, Rk ) ), 0.5 );
            const double inv = __ddiv_rn( 1.0, ddot( n, n ) );
            const d3     y0  = dmul( dadd( dmul( dcross( bv, n ), p ), dmul( dcross( n, a ), q ) ), inv );
            h2               = __dsub_rn( Ri2, ddot( y0, y0 ) );
            if ( !( h2 >= 0.0 ) )
                return false;
            const double s  = __dsqrt_rn( __dmul_rn( h2, inv ) );
            const d3     xc = dadd( ci, y0 );
            x1              = dadd( xc, dmul( n, s ) );
            x2              = dsub( xc, dmul( n, s ) );
            return true;
        }

        // Float-float solve of a kept probe: the closed form of solve_d carried in
        // float-float arithmetic (about 48 bits), with an a-priori bound Ex on the
        // distance of its position from the exact point. The double-precision result
        // lies within far less than Ex of the exact point too, so wherever the
        // float-float coordinate is more than Ex from a float32 rounding boundary
        // both round to the same float32 (and the singular test, more than its own
        // bound from its threshold, decides alike). Returns false otherwise; the
        // caller then solves in double precision (about 0.2 % of the jobs, mostly
        // probes close to the plane of their centres).
        __device__ __forceinline__ ff ff_dot3( ff ax, ff ay, ff az, ff bx, ff by, ff bz )
        {
            return ff_add( ff_add( ff_mul( ax, bx ), ff_mul( ay, by ) ), ff_mul( az, bz ) );
        }
        __device__ __forceinline__ float ff_margin( ff x )
        {
            // distance of x from the nearest boundary between two float32 values
            const float v    = fabsf( x.hi );
            const float up   = __int_as_float( __float_as_int( v ) + 1 ) - v;
            const float down = v > 0.f ? v - __int_as_float( __float_as_int( v ) - 1 ) : up;
            return 0.5f * fminf( up, down ) - fabsf( x.lo );
        }
        __device__ bool solve_ff( float4 ai, float4 aj, float4 ak, float rp, uint32_t side, bool wantSingular, float3 & pos,
                                  bool & singular )
        {
            const ff ax = two_sum( aj.x, -ai.x ), ay = two_sum( aj.y, -ai.y ), az = two_sum( aj.z, -ai.z );
            const ff bx = two_sum( ak.x, -ai.x ), by = two_sum( ak.y, -ai.y ), bz = two_sum( ak.z, -ai.z );
            const ff nx = ff_sub( ff_mul( ay, bz ), ff_mul( az, by ) );
            const ff ny = ff_sub( ff_mul( az, bx ), ff_mul( ax, bz ) );
            const ff nz = ff_sub( ff_mul( ax, by ), ff_mul( ay, bx ) );
            const ff Ri = two_sum( ai.w, rp ), Rj = two_sum( aj.w, rp ), Rk = two_sum( ak.w, rp );
            const ff Ri2 = ff_mul( Ri, Ri ), Rj2 = ff_mul( Rj, Rj ), Rk2 = ff_mul( Rk, Rk );
            const ff aa  = ff_dot3( ax, ay, az, ax, ay, az );
            const ff bb  = ff_dot3( bx, by, bz, bx, by, bz );
            const ff p   = ff_scale( ff_sub( ff_add( aa, Ri2 ), Rj2 ), 0.5f );
            const ff q   = ff_scale( ff_sub( ff_add( bb, Ri2 ), Rk2 ), 0.5f );
            const ff nn  = ff_dot3( nx, ny, nz, nx, ny, nz );
            if ( !( nn.hi > 0.f ) )
                return false;
            const ff inv = ff_div( ff_of( 1.f ), nn );
            // y0 = (p (b x n) + q (n x a)) / |n|^2
            const ff cx  = ff_add( ff_mul( p, ff_sub( ff_mul( by, nz ), ff_mul( bz, ny ) ) ), ff_mul( q, ff_sub( ff_mul( ny, az ), ff_mul( nz, ay ) ) ) );
            const ff cy  = ff_add( ff_mul( p, ff_sub( ff_mul( bz, nx ), ff_mul( bx, nz ) ) ), ff_mul( q, ff_sub( ff_mul( nz, ax ), ff_mul( nx, az ) ) ) );
            const ff cz  = ff_add( ff_mul( p, ff_sub( ff_mul( bx, ny ), ff_mul( by, nx ) ) ), ff_mul( q, ff_sub( ff_mul( nx, ay ), ff_mul( ny, ax ) ) ) );
            const ff yx = ff_mul( cx, inv ), yy = ff_mul( cy, inv ), yz = ff_mul( cz, inv );
            const ff h2 = ff_sub( Ri2, ff_dot3( yx, yy, yz, yx, yy, yz ) );
            if ( !( h2.hi > 0.f ) )
                return false;
            const ff s = ff_sqrt( ff_mul( h2, inv ) );
            // error bound, with u = 2^-42 (a float-float operation rounds by at most
            // ~2^-46 relative to the magnitudes bounded below; ~10 of them feed each
            // term, and every term carries a factor >= 4 on top) and
            // kappa = |a| |b| / |n| = 1 / sin(angle at c_i)
            const float u     = 2.2737367544323206e-13f;
            const float A     = sqrtf( aa.hi ), B = sqrtf( bb.hi ), N = sqrtf( nn.hi );
            const float kappa = A * B / N;
            const float Pm    = aa.hi + Ri2.hi + Rj2.hi, Qm = bb.hi + Ri2.hi + Rk2.hi;
            const float Y     = sqrtf( yx.hi * yx.hi + yy.hi * yy.hi + yz.hi * yz.hi );
            const float root  = sqrtf( h2.hi );
            const float Ey0   = u * ( ( Pm * B + Qm * A ) / N + Y ) * ( 4.f + 2.f * kappa );
            const float Eh2   = 2.f * Y * Ey0 + u * ( Ri2.hi + Y * Y );
            const float Eroot = Eh2 / ( 2.f * root ) + u * ( 2.f + 2.f * kappa ) * root;
            const float amax  = fmaxf( fabsf( ai.x ), fmaxf( fabsf( ai.y ), fabsf( ai.z ) ) );
            const float Ex    = Ey0 + Eroot + u * ( amax + Y + root );
            const ff    px = ff_add( ff_add( ff_of( ai.x ), yx ), side ? ff_neg( ff_mul( nx, s ) ) : ff_mul( nx, s ) );
            const ff    py = ff_add( ff_add( ff_of( ai.y ), yy ), side ? ff_neg( ff_mul( ny, s ) ) : ff_mul( ny, s ) );
            const ff    pz = ff_add( ff_add( ff_of( ai.z ), yz ), side ? ff_neg( ff_mul( nz, s ) ) : ff_mul( nz, s ) );
            if ( !( ff_margin( px ) > Ex && ff_margin( py ) > Ex && ff_margin( pz ) > Ex ) )
                return false;
            pos = make_float3( px.hi, py.hi, pz.hi );
            if ( wantSingular )
            {
                // h2 - rp^2 < -1e-4 (the threshold as the double of the float 1e-4)
                const ff    v  = ff_add( ff_sub( h2, two_prod( rp, rp ) ), ff_of( 1e-4f ) );
                const float Ev = Eh2 + u * rp * rp;
                if ( !( fabsf( v.hi ) > Ev ) )
                    return false;
                singular = v.hi < 0.f;
            }
            return true;
        }

        // singular flag (operations.inl:441-451): the point closer than rp to the
        // plane of the centres, d^2 - rp^2 < -1e-4 with d^2 = h2
        __device__ __forceinline__ bool singular_d( double h2, double rp )
        {
            return __dsub_rn( h2, __dmul_rn( rp, rp ) ) < -(double)1e-4f;
        }

        // Occlusion of the double-precision points by N(i) \ {j, k} (operations.inl:401-430):
        // float32 filter around the rounded relative positions, double precision in
        // the band. The neighbours are fetched eight at a time (independent loads in
        // flight instead of one dependent id-then-atom pair per neighbour); the test
        // is an "inside some l" test, so the order does not matter.
        constexpr uint32_t kOccChunk = 8;
        __device__ __forceinline__ void occlusion_d( const Build & b, uint32_t i, const float4 & ai, uint32_t sj, uint32_t sk,
                                                     const d3 x[ 2 ], bool vis[ 2 ], uint32_t & fp64 )
        {
            const double rp = (double)b.rp;
            const d3     ci = D3( ai );
            f3           xr[ 2 ];
            for ( int e = 0; e < 2; e++ )
                xr[ e ] = F3( __double2float_rn( __dsub_rn( x[ e ].x, ci.x ) ), __double2float_rn( __dsub_rn( x[ e ].y, ci.y ) ),
                              __double2float_rn( __dsub_rn( x[ e ].z, ci.z ) ) );
            const uint32_t   ni  = b.nbrCount[ i ];
            const uint32_t * row = b.nbr + (size_t)i * b.cap;
            for ( uint32_t s0 = 0; s0 < ni && ( vis[ 0 ] || vis[ 1 ] ); s0 += kOccChunk )
            {
                uint32_t id[ kOccChunk ];
                float4   al[ kOccChunk ];
#pragma unroll
                for ( uint32_t c = 0; c < kOccChunk; c++ )
                    id[ c ] = s0 + c < ni ? row[ s0 + c ] : 0u;
#pragma unroll
                for ( uint32_t c = 0; c < kOccChunk; c++ )
                    al[ c ] = b.atoms[ id[ c ] ];
#pragma unroll
                for ( uint32_t c = 0; c < kOccChunk; c++ )
                {
                    const uint32_t sl = s0 + c;
                    if ( sl >= ni || sl == sj || sl == sk )
                        continue;
                    const f3    dl  = F3( al[ c ].x - ai.x, al[ c ].y - ai.y, al[ c ].z - ai.z );
                    const float Rl  = al[ c ].w + b.rp;
                    const float Rl2 = Rl * Rl;
                    for ( int e = 0; e < 2; e++ )
                    {
                        if ( !vis[ e ] )
                            continue;
                        const f3    ev = dl - xr[ e ];
                        const float ee = dot( ev, ev );
                        const float m  = ee - Rl2;
                        const float em = kRel * ( ee + Rl2 + 1.f );
                        if ( m < -em )
                            vis[ e ] = false;
                        else if ( !( m > em ) )
                        {
                            const double Rld = __dadd_rn( (double)al[ c ].w, rp );
                            const d3     dv  = dsub( D3( al[ c ] ), x[ e ] );
                            vis[ e ]         = __dsub_rn( ddot( dv, dv ), __dmul_rn( Rld, Rld ) ) > 0.0;
                            fp64++;
                        }
                    }
                }
            }
        }

        // Error scale of the float32 solve (relative, generous: about 60x the
        // accumulated rounding of its ~25 dependent operations).
        constexpr float kSolve = 1.0f / 262144.0f; // 2^-18

        // One warp per block: the work of an atom varies a lot, and a block's slot (its
        // registers and shared memory) is freed only when its last warp ends.
        constexpr int kCandBuf    = 64;  // candidates queued per warp
        constexpr int kProbeBuf   = 128; // probes of one atom (the reference's per-block buffer, operations.inl:248)

        // Per-warp staging of atom i's neighbourhood. For a point x on the SAS
        // sphere of i (|x| = R_i in coordinates relative to i), x lies inside the
        // SAS sphere of neighbour l exactly when x . d_l > K_l with
        // K_l = (R_i^2 + |d_l|^2 - R_l^2) / 2: the occlusion test is one plane test.
        struct ProbeSmem
        {
            float4 *   rel;   // cap: d_l (neighbour centre - centre of i), K_l
            float *    rad;   // cap: R_l (vdW radius + probe radius)
            uint32_t * nid;   // cap: neighbour ids
            uint16_t * plist; // cap: slots of the partial circles (i, j), i < j
            uint8_t *  full;  // cap: 1 if the neighbour list of that neighbour may be truncated
            uint32_t * cand;  // kCandBuf: slot j | slot k << 16
            uint2 *    ent;   // kProbeBuf: (slot j | slot k << 16, side | kind << 1 | (w + 4) << 2)
            uint64_t * touch; // kMaskSlots: slots of the atoms touching the partial circle (i, slot)
            uint16_t * coff;  // kMaskSlots: first candidate of each partial circle (touch-mask enumeration)
        };

        __host__ __device__ inline size_t probe_smem_per_warp( uint32_t cap )
        {
            size_t b = (size_t)staged_rows( cap ) * ( 16 + 4 + 4 + 2 + 1 );
            b        = ( b + 15 ) & ~(size_t)15;
            return b + kCandBuf * 4 + kProbeBuf * 8 + kMaskSlots * ( 8 + 2 );
        }

        __device__ inline ProbeSmem probe_smem( unsigned char * base, uint32_t capacity )
        {
            const size_t cap = staged_rows( capacity );
            ProbeSmem    m;
            m.rel    = reinterpret_cast<float4 *>( base );
            m.rad    = reinterpret_cast<float *>( base + (size_t)cap * 16 );
            m.nid    = reinterpret_cast<uint32_t *>( base + (size_t)cap * 20 );
            m.plist  = reinterpret_cast<uint16_t *>( base + (size_t)cap * 24 );
            m.full   = reinterpret_cast<uint8_t *>( base + (size_t)cap * 26 );
            size_t o = ( (size_t)cap * 27 + 15 ) & ~(size_t)15;
            m.cand   = reinterpret_cast<uint32_t *>( base + o );
            o += kCandBuf * 4;
            m.ent = reinterpret_cast<uint2 *>( base + o );
            o += kProbeBuf * 8;
            m.touch = reinterpret_cast<uint64_t *>( base + o );
            o += kMaskSlots * 8;
            m.coff = reinterpret_cast<uint16_t *>( base + o );
            return m;
        }

        // float32 singular test (operations.inl:441-451) in coordinates relative to
        // atom i: 1 singular, 0 regular, -1 inside the band (decide in double)
        __device__ __forceinline__ int singular_f( f3 dj, f3 dk, f3 x, float ep, float rp )
        {
            const f3    a  = normalize( dj );
            const f3    c  = normalize( dj - dk );
            const f3    cr = cross( a, c );
            const float s2 = dot( cr, cr );
            if ( !( s2 > 1e-6f ) )
                return -1;
            const f3    pn = cr * rsqrtf( s2 );
            const float d  = -dot( x, pn );
            const float xn = sqrtf( dot( x, x ) );
            const float ed = ep + xn * kSolve * ( 4.f + 4.f * rsqrtf( s2 ) );
            const float ms = d * d - rp * rp + 1e-4f;
            const float es = 2.f * ( fabsf( d ) + ed ) * ed + kRel * ( d * d + rp * rp + 1.f );
            if ( ms < -es )
                return 1;
            if ( ms > es )
                return 0;
            return -1;
        }

        // Job of the double-precision pass: entry index, atom, slots, kind.
        enum : uint32_t
        {
            kJobFill = 0, // one side decided visible in float32: exact position (and singular flag if pending)
            kJobBand = 1, // the float32 screen hit the band: solve, occlusion and flags in double precision
        };

        // Bounds of atom i's staged neighbourhood that size the error bands of the
        // float32 screens: the largest |d_l| and |d_l|^2 and the half-width of the
        // plane-test band due to rounding (kRel (R_i^2 + |d_l|^2 + R_l^2 + 1) / 2).
        struct ProbeBounds
        {
            float dmax, d2max, eK;
        };

        // Is k (slot sk) in the neighbour list of j (slot sj)? The lists hold every
        // atom that satisfies the neighbour predicate (k_neighbors decides it
        // exactly), in ascending order, cut at the capacity: for a list that is
        // not full the float32 predicate answers outside its error band; a full
        // list, or a pair inside the band, is searched.
        __device__ __forceinline__ bool pair_is_neighbor( const Build & b, const ProbeSmem & m, const ProbeBounds & pb,
                                                          uint32_t sj, uint32_t sk, uint32_t & fp64 )
        {
            const uint32_t j = m.nid[ sj ], k = m.nid[ sk ];
            if ( m.full[ sj ] )
                return find_in_row( b.nbr + (size_t)j * b.cap, b.nbrCount[ j ], k ) >= 0;
            const float4 qj = m.rel[ sj ], qk = m.rel[ sk ];
            const f3     v  = F3( qj.x - qk.x, qj.y - qk.y, qj.z - qk.z );
            const float  d  = dot( v, v );
            const float  R  = m.rad[ sj ] + m.rad[ sk ];
            const float  mm = d - R * R - 1e-4f;
            // the float32 difference of two relative positions adds at most a few
            // ulps of |d_j| + |d_k| to v: covered by the d2max term
            const float e = kRel * ( d + R * R + pb.d2max + 1.f );
            if ( mm < -e )
                return true;
            if ( mm > e )
                return false;
            fp64++; // inside the band: the list itself answers
            return find_in_row( b.nbr + (size_t)j * b.cap, b.nbrCount[ j ], k ) >= 0;
        }

        // One (i, j, k) candidate, float32 screen in coordinates relative to atom i
        // with a conservative error band. Sets w[e]: 0 none, +-1 regular, +-2
        // singular, +-3 kept with the singular flag undecided; or band = true
        // (both entries reserved for the double-precision pass).
        __device__ __forceinline__ void probe_screen( const ProbeSmem & m, const ProbeBounds & pb, float Ri, float rp,
                                                      uint32_t ni, bool useMask, uint32_t sj, uint32_t sk, int w[ 2 ],
                                                      bool & band )
        {
            const float4 qj = m.rel[ sj ], qk = m.rel[ sk ];
            const f3     dj = F3( qj.x, qj.y, qj.z ), dk = F3( qk.x, qk.y, qk.z );
            // approximate reciprocals and roots (a few ulps) are well inside the kSolve error scale
            const float  dJ = dot( dj, dj ), dK = dot( dk, dk );
            const float  rJ = rsqrtf( dJ ), rK = rsqrtf( dK );
            const f3     cJ = dj * ( qj.w * rJ * rJ ); // (R_i^2 - R_j^2 + |d_j|^2) / (2 |d_j|^2) = K_j / |d_j|^2
            const f3     cK = dk * ( qk.w * rK * rK );
            const f3     nJ = dj * rJ;
            const f3     nK = dk * rK;
            const f3     u  = nK - nJ * dot( nK, nJ );
            const float  den = dot( u, nK ); // sin^2 of the angle between the circle axes
            w[ 0 ] = w[ 1 ] = 0;
            band            = !( den > 1e-3f );
            if ( band )
                return;
            const float iden = __fdividef( 1.f, den );
            const f3    xc   = cJ + u * ( dot( cK - cJ, nK ) * iden );
            const float x2   = dot( xc, xc );
            const float xn   = x2 > 0.f ? x2 * rsqrtf( x2 ) : 0.f;
            const float ex   = kSolve * ( Ri + xn ) * ( 1.f + iden );
            const float tt   = Ri * Ri - x2;
            const float et   = 2.f * ( xn + ex ) * ex + kSolve * Ri * Ri;
            if ( tt < -et )
                return; // no point
            if ( !( tt > et ) )
            {
                band = true;
                return;
            }
            const float rt   = rsqrtf( tt );
            const float root = tt * rt;
            const f3    nn   = normalize( cross( nJ, nK ) );
            const float ep   = ex + 0.5f * et * rt + root * kSolve * rsqrtf( den );
            // x1,2 = xc +- root nn lie within ep of the exact points: a plane test
            // moves by at most ep |d_l|, rounding by at most eK
            const float eh = ep * pb.dmax + pb.eK;
            bool        v1 = true, v2 = true;
            // 0: go on, 1: inside the band, 2: both points buried
            auto occlude = [ & ]( uint32_t sl ) -> int {
                const float4 ql = m.rel[ sl ];
                const float  a  = ql.w - ( xc.x * ql.x + xc.y * ql.y + xc.z * ql.z );
                const float  c  = root * ( nn.x * ql.x + nn.y * ql.y + nn.z * ql.z );
                const float  h1 = a - c, h2 = a + c; // K_l - x . d_l for x1 and x2
                // inside the band, or NaN: left to double precision
                if ( ( v1 && !( fabsf( h1 ) > eh ) ) || ( v2 && !( fabsf( h2 ) > eh ) ) )
                    return 1;
                v1 = v1 && h1 > 0.f;
                v2 = v2 && h2 > 0.f;
                return ( v1 || v2 ) ? 0 : 2;
            };
            if ( useMask )
            {
                // only an atom that touches both circles (i, j) and (i, k) can hold a point of both
                // in ascending slot order, one 32-bit half of the mask at a time
                const uint64_t occ = m.touch[ sj ] & m.touch[ sk ] & ~( ( 1ull << sj ) | ( 1ull << sk ) );
#pragma unroll
                for ( uint32_t h = 0; h < 2; h++ )
                    for ( uint32_t w = (uint32_t)( occ >> ( 32 * h ) ); w; w &= w - 1 )
                    {
                        const int r = occlude( 32u * h + (uint32_t)( __ffs( (int)w ) - 1 ) );
                        if ( r )
                        {
                            band = r == 1;
                            return;
                        }
                    }
            }
            else
            {
                for ( uint32_t sl = 0; sl < ni; sl++ )
                {
                    if ( sl == sj || sl == sk )
                        continue;
                    const int r = occlude( sl );
                    if ( r )
                    {
                        band = r == 1;
                        return;
                    }
                }
            }
            if ( v1 )
            {
                const int sg = singular_f( dj, dk, xc + nn * root, ep, rp );
                w[ 0 ]       = sg < 0 ? 3 : 1 + sg;
            }
            if ( v2 )
            {
                const int sg = singular_f( dj, dk, xc - nn * root, ep, rp );
                w[ 1 ]       = -( sg < 0 ? 3 : 1 + sg );
            }
        }

        // Warp per atom i: every pair of partial circles (i, j), (i, k), i < j < k,
        // whose far atoms are neighbours. Entries of the atom's probe list are kept
        // in order (circle (i, j), then k, then x1 before x2) and written as one
        // chunk; positions and undecided flags are completed by k_probe_jobs.
        __device__ __forceinline__ void probes_of_atom( const Build & b, uint32_t i, unsigned char * smemWarp )
        {
            const uint32_t  lane = lane_id();
            const ProbeSmem m    = probe_smem( smemWarp, b.cap );
            const uint32_t  ni  = b.nbrCount[ i ];
            const float4    ai  = b.atoms[ i ];
            const float     Ri  = ai.w + b.rp;
            const size_t    row = (size_t)i * b.cap;
            const uint32_t  po  = b.pairOff[ i ];

            const bool useMask = ni <= (uint32_t)kMaskSlots;
            uint32_t   p       = 0;
            uint64_t   partial = 0; // slots of the partial circles (i, j), i < j
            float      d2max = 0.f, bmax = 0.f;
            // two rows of 32 neighbours at a time. The rows (ids, statuses) are read up to the
            // capacity without waiting for the count (slots past it are not used), so that they
            // travel with the atom's own loads; the neighbours' atoms, counts and touch masks
            // follow together: two round trips to memory for an atom of up to 64 neighbours
            for ( uint32_t base0 = 0; base0 == 0 || base0 < ni; base0 += 64 )
            {
                uint32_t jj[ 2 ] = { 0u, 0u }, st[ 2 ] = { 0u, 0u }, cn[ 2 ] = { 0u, 0u };
                float4   aa[ 2 ];
                uint64_t tm[ 2 ] = { ~0ull, ~0ull };
#pragma unroll
                for ( int h = 0; h < 2; h++ )
                {
                    const uint32_t s = base0 + 32 * h + lane;
                    if ( s < b.cap )
                    {
                        jj[ h ] = b.nbr[ row + s ];
                        st[ h ] = b.status[ row + s ];
                    }
                }
#pragma unroll
                for ( int h = 0; h < 2; h++ )
                {
                    const uint32_t s = base0 + 32 * h + lane;
                    if ( s < ni )
                    {
                        aa[ h ] = b.atoms[ jj[ h ] ];
                        cn[ h ] = b.nbrCount[ jj[ h ] ];
                        // past the touch buffer's capacity (a build that overflowed P and is built
                        // again) every neighbour counts as touching
                        if ( useMask && po + s < b.capPairs )
                            tm[ h ] = b.touch[ po + s ];
                    }
                }
#pragma unroll
                for ( int h = 0; h < 2; h++ )
                {
                    const uint32_t base = base0 + 32 * h;
                    if ( base >= ni )
                        break;
                    const uint32_t s   = base + lane;
                    bool           isP = false;
                    if ( s < ni )
                    {
                        const uint32_t j  = jj[ h ];
                        const float4   aj = aa[ h ];
                        const f3       d  = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
                        const float    dd = dot( d, d );
                        const float    Rl = aj.w + b.rp;
                        m.rel[ s ]        = make_float4( d.x, d.y, d.z, 0.5f * ( ( Ri * Ri + dd ) - Rl * Rl ) );
                        m.rad[ s ]        = Rl;
                        m.nid[ s ]        = j;
                        m.full[ s ]       = cn[ h ] >= b.cap;
                        isP               = st[ h ] == 1 && i < j;
                        if ( isP && useMask )
                            m.touch[ s ] = tm[ h ];
                        d2max = fmaxf( d2max, dd );
                        bmax  = fmaxf( bmax, Ri * Ri + dd + Rl * Rl );
                    }
                    const uint32_t mk = __ballot_sync( 0xffffffffu, isP );
                    if ( isP )
                        m.plist[ p + __popc( mk & lanemask_lt() ) ] = (uint16_t)s;
                    p += __popc( mk );
                    if ( base < 64 )
                        partial |= (uint64_t)mk << base;
                }
            }
            for ( int o = 16; o > 0; o >>= 1 )
            {
                d2max = fmaxf( d2max, __shfl_xor_sync( 0xffffffffu, d2max, o ) );
                bmax  = fmaxf( bmax, __shfl_xor_sync( 0xffffffffu, bmax, o ) );
            }
            ProbeBounds pb;
            pb.d2max = d2max;
            pb.dmax  = sqrtf( d2max ) * ( 1.f + kRel );
            pb.eK    = 0.5f * kRel * ( bmax + 1.f );
            __syncwarp();

            uint32_t nCand = 0, nEnt = 0, nSing = 0, nReg = 0, cands = 0, fp64 = 0;
            // screens queued candidates 32 at a time (all of them when last)
            auto screen_batches = [ & ]( bool last ) {
                while ( nCand >= 32 || ( last && nCand > 0 ) )
                {
                    const uint32_t batch = nCand < 32 ? nCand : 32;
                    int            w[ 2 ] = { 0, 0 };
                    bool           band   = false;
                    uint32_t       sjk    = 0;
                    if ( lane < batch )
                    {
                        sjk = m.cand[ lane ];
                        probe_screen( m, pb, Ri, b.rp, ni, useMask, sjk & 0xffffu, sjk >> 16, w, band );
                    }
                    const uint32_t need = band ? 2u : ( w[ 0 ] != 0 ) + ( w[ 1 ] != 0 );
                    uint32_t       tot;
                    uint32_t       at = nEnt + warp_exclusive_sum( need, tot );
                    for ( int e = 0; e < 2 && need; e++ )
                    {
                        if ( !band && w[ e ] == 0 )
                            continue;
                        if ( at < (uint32_t)kProbeBuf )
                            m.ent[ at ] = make_uint2( sjk, (uint32_t)e | ( ( band ? kJobBand : kJobFill ) << 1 ) |
                                                               ( (uint32_t)( ( band ? 0 : w[ e ] ) + 4 ) << 2 ) );
                        if ( !band )
                        {
                            const int aw = w[ e ] < 0 ? -w[ e ] : w[ e ];
                            nSing += aw == 2;
                            nReg += aw == 1;
                        }
                        at++;
                    }
                    nEnt += tot;
                    // drop the processed batch from the queue
                    __syncwarp();
                    const uint32_t rest = nCand - batch;
                    uint32_t       keep[ 2 ];
                    for ( uint32_t r = 0; r < 2; r++ )
                        if ( lane + 32 * r < rest )
                            keep[ r ] = m.cand[ batch + lane + 32 * r ];
                    __syncwarp();
                    for ( uint32_t r = 0; r < 2; r++ )
                        if ( lane + 32 * r < rest )
                            m.cand[ lane + 32 * r ] = keep[ r ];
                    __syncwarp();
                    nCand = rest;
                }
            };
            auto enqueue = [ & ]( bool isC, uint32_t sj, uint32_t sk ) {
                const uint32_t mc = __ballot_sync( 0xffffffffu, isC );
                if ( isC )
                    m.cand[ nCand + __popc( mc & lanemask_lt() ) ] = sj | ( sk << 16 );
                nCand += __popc( mc );
                cands += __popc( mc );
                __syncwarp();
            };
            if ( useMask )
            {
                // for each partial circle (i, j): the partial circles (i, k), k > j, whose
                // far atom touches circle (i, j); flattened over the circles in (j, k)
                // slot order, 32 at a time, and kept when k is a neighbour of j
                auto later = [ & ]( uint32_t a ) {
                    const uint32_t sj = m.plist[ a ];
                    return m.touch[ sj ] & partial & ( sj >= 63 ? 0ull : ~0ull << ( sj + 1 ) );
                };
                uint32_t total = 0;
                for ( uint32_t a0 = 0; a0 < p; a0 += 32 )
                {
                    const uint32_t a = a0 + lane;
                    const uint32_t c = a < p ? (uint32_t)__popcll( later( a ) ) : 0u;
                    uint32_t       tot;
                    const uint32_t first = total + warp_exclusive_sum( c, tot );
                    if ( a < p )
                        m.coff[ a ] = (uint16_t)first;
                    total += tot;
                }
                __syncwarp();
                for ( uint32_t c0 = 0; c0 < total; c0 += 32 )
                {
                    const uint32_t c   = c0 + lane;
                    bool           isC = false;
                    uint32_t       sj = 0, sk = 0;
                    if ( c < total )
                    {
                        // last circle whose first candidate is <= c (at most 64 circles here)
                        uint32_t lo = 0;
#pragma unroll
                        for ( uint32_t step = 32; step > 0; step >>= 1 )
                            if ( lo + step < p && m.coff[ lo + step ] <= c )
                                lo += step;
                        // its r-th candidate: the r-th set bit of the mask (r from 0), found by halving
                        const uint64_t w  = later( lo );
                        uint32_t       r  = c - m.coff[ lo ];
                        const uint32_t wl = (uint32_t)w, nl = __popc( wl );
                        uint32_t       word = r < nl ? wl : (uint32_t)( w >> 32 );
                        uint32_t       pos  = r < nl ? 0u : 32u;
                        r                   = r < nl ? r : r - nl;
#pragma unroll
                        for ( uint32_t h = 16; h > 0; h >>= 1 )
                        {
                            const uint32_t cnt = __popc( word & ( ( 1u << h ) - 1u ) );
                            if ( r >= cnt )
                            {
                                r -= cnt;
                                word >>= h;
                                pos += h;
                            }
                        }
                        sj = m.plist[ lo ];
                        sk = pos;
                        isC = pair_is_neighbor( b, m, pb, sj, sk, fp64 );
                    }
                    enqueue( isC, sj, sk );
                    screen_batches( false );
                }
                screen_batches( true );
            }
            else
            {
                const uint32_t pairs = p * ( p > 0 ? p - 1 : 0 ) / 2;
                for ( uint32_t q0 = 0; q0 < pairs || nCand > 0; q0 += 32 )
                {
                    if ( q0 < pairs )
                    {
                        // pair q = (a, bb), a < bb, row-major over the partial circles
                        const uint32_t q   = q0 + lane;
                        bool           isC = false;
                        uint32_t       sj = 0, sk = 0;
                        if ( q < pairs )
                        {
                            const float tp = 2.f * p - 1.f;
                            int         a  = (int)floorf( 0.5f * ( tp - sqrtf( fmaxf( tp * tp - 8.f * (float)q, 0.f ) ) ) );
                            a              = a < 0 ? 0 : a;
                            while ( a > 0 && (uint32_t)( a * ( 2 * (int)p - a - 1 ) / 2 ) > q )
                                a--;
                            while ( (uint32_t)( ( a + 1 ) * ( 2 * (int)p - a - 2 ) / 2 ) <= q )
                                a++;
                            const uint32_t bb = (uint32_t)a + 1 + ( q - (uint32_t)( a * ( 2 * (int)p - a - 1 ) / 2 ) );
                            sj                = m.plist[ a ];
                            sk                = m.plist[ bb ];
                            isC               = pair_is_neighbor( b, m, pb, sj, sk, fp64 );
                        }
                        enqueue( isC, sj, sk );
                    }
                    screen_batches( q0 + 32 >= pairs );
                }
            }
            for ( int o = 16; o > 0; o >>= 1 )
            {
                nSing += __shfl_xor_sync( 0xffffffffu, nSing, o );
                nReg += __shfl_xor_sync( 0xffffffffu, nReg, o );
                fp64 += __shfl_xor_sync( 0xffffffffu, fp64, o );
            }
            __syncwarp();
            // one chunk per atom; one double-precision job per kept side or band candidate.
            // Jobs: a fill entry is one job (counted up from the bottom of the job array); a
            // band candidate's two entries are one job on its first entry (counted down from the
            // top), so that each kind runs with full warps
            const uint32_t kept     = nEnt < (uint32_t)kProbeBuf ? nEnt : (uint32_t)kProbeBuf;
            uint32_t       fillHere = 0, bandHere = 0;
            for ( uint32_t q0 = 0; q0 < kept; q0 += 32 )
            {
                const uint32_t q    = q0 + lane;
                bool           fill = false, band = false;
                if ( q < kept )
                {
                    const uint32_t info = m.ent[ q ].y;
                    fill                = ( ( info >> 1 ) & 1u ) == kJobFill;
                    band                = !fill && ( info & 1u ) == 0u;
                }
                fillHere += __popc( __ballot_sync( 0xffffffffu, fill ) );
                bandHere += __popc( __ballot_sync( 0xffffffffu, band ) );
            }
            // the staging chunk and the fill-job slots in one 64-bit atomic: every atom's warp adds
            // to these counters, and a contended atomic whose result a warp waits for is costly. The
            // low word (staged entries, at most kProbeBuf per atom) cannot carry into the high word
            // below 2^25 atoms; far below that the build's 32-bit capacities overflow and regrow first
            uint32_t chunk = 0, jbase = 0;
            if ( lane == 0 )
            {
                if ( nEnt > (uint32_t)kProbeBuf )
                    atomicOr( &b.counts->overflow, (uint32_t)kOverflowAtomProbes );
                if ( kept )
                {
                    const unsigned long long old = atomicAdd( reinterpret_cast<unsigned long long *>( &b.counts->staged ),
                                                              (unsigned long long)kept | ( (unsigned long long)fillHere << 32 ) );
                    chunk = (uint32_t)old;
                    jbase = (uint32_t)( old >> 32 );
                }
                if ( cands )
                    atomicAdd( &b.counts->cand, cands );
                if ( fp64 )
                    atomicAdd( &b.counts->fp64[ kFp64Neighbor ], fp64 );
            }
            chunk = __shfl_sync( 0xffffffffu, chunk, 0 );
            jbase = __shfl_sync( 0xffffffffu, jbase, 0 );
            // an atom with more entries than the warp holds (an error of the build) places none, so
            // that the probe offsets stay within the staged ones; its fill-job slots get empty jobs
            const bool fits = chunk + kept <= b.capProbes && nEnt <= (uint32_t)kProbeBuf;
            if ( !fits )
            {
                for ( uint32_t t = lane; t < fillHere; t += 32 )
                    if ( jbase + t < b.capProbes )
                        b.jobs[ jbase + t ] = make_uint4( 0u, 0xffffffffu, 0u, 0u );
                bandHere = 0;
            }
            // slot of k in N(j) for every kept entry, found by the whole warp: coalesced
            // passes over the rows of four entries at a time, their loads in flight together
            // (the row is read before its count arrives; slots past the count do not match)
            uint16_t * sjkS = reinterpret_cast<uint16_t *>( m.cand ); // free after the screening (2 kCandBuf slots)
            for ( uint32_t e0 = 0; e0 < kept && fits; e0 += 4 )
            {
                uint32_t jv[ 4 ], kv[ 4 ], nv[ 4 ], pos[ 4 ];
#pragma unroll
                for ( int u = 0; u < 4; u++ )
                {
                    const uint32_t ex = m.ent[ min( e0 + (uint32_t)u, kept - 1u ) ].x;
                    jv[ u ]           = m.nid[ ex & 0xffffu ];
                    kv[ u ]           = m.nid[ ex >> 16 ];
                    pos[ u ]          = 0xffffffffu;
                }
#pragma unroll
                for ( int u = 0; u < 4; u++ )
                    nv[ u ] = b.nbrCount[ jv[ u ] ];
                uint32_t base = 0;
                do
                {
                    const uint32_t s = base + lane;
                    uint32_t       id[ 4 ];
#pragma unroll
                    for ( int u = 0; u < 4; u++ )
                        id[ u ] = s < b.cap ? b.nbr[ (size_t)jv[ u ] * b.cap + s ] : 0xffffffffu;
                    uint32_t span = 0;
#pragma unroll
                    for ( int u = 0; u < 4; u++ )
                    {
                        const uint32_t mk = __ballot_sync( 0xffffffffu, s < nv[ u ] && id[ u ] == kv[ u ] );
                        if ( mk && pos[ u ] == 0xffffffffu )
                            pos[ u ] = base + (uint32_t)( __ffs( mk ) - 1 );
                        if ( pos[ u ] == 0xffffffffu )
                            span = max( span, nv[ u ] );
                    }
                    base += 32;
                    if ( base >= span )
                        break;
                } while ( true );
                if ( lane < 4 && e0 + lane < kept )
                {
                    uint32_t r = pos[ 0 ];
#pragma unroll
                    for ( int u = 1; u < 4; u++ )
                        r = lane == (uint32_t)u ? pos[ u ] : r;
                    sjkS[ e0 + lane ] = (uint16_t)( r == 0xffffffffu ? 0u : r );
                }
            }
            __syncwarp();
            uint32_t gbase = 0;
            if ( lane == 0 && bandHere )
                gbase = atomicAdd( &b.counts->bandJobs, bandHere );
            gbase = __shfl_sync( 0xffffffffu, gbase, 0 );
            for ( uint32_t q0 = 0; q0 < kept; q0 += 32 )
            {
                const uint32_t q     = q0 + lane;
                bool           isJob = false;
                uint2          en    = make_uint2( 0u, 0u );
                if ( q < kept && fits )
                {
                    en                  = m.ent[ q ];
                    const uint32_t sj   = en.x & 0xffffu, sk = en.x >> 16;
                    const uint32_t side = en.y & 1u, kind = ( en.y >> 1 ) & 1u;
                    const int      wv   = (int)( en.y >> 2 ) - 4;
                    const uint32_t j = m.nid[ sj ], k = m.nid[ sk ];
                    const uint32_t sjk  = sjkS[ q ];
                    int4           cid;
                    if ( b.mode == 0 )
                        cid = make_int4( (int)b.slotTrim[ row + sj ], (int)b.slotTrim[ (size_t)j * b.cap + sjk ],
                                         (int)b.slotTrim[ row + sk ], wv );
                    else
                        cid = make_int4( (int)( row + sj ), (int)( row + sk ), (int)( (size_t)j * b.cap + sjk ), wv );
                    b.stageCid[ chunk + q ] = cid;
                    b.stageIds[ chunk + q ] = make_int4( (int)i, (int)j, (int)k, 0 );
                    b.stagePos[ chunk + q ] = make_float4( 0.f, 0.f, 0.f, 0.f );
                    isJob                   = kind == kJobFill || side == 0u;
                    en.y                    = side | ( kind << 8 );
                }
                const bool     fill = isJob && ( en.y >> 8 ) == kJobFill;
                const uint32_t mf   = __ballot_sync( 0xffffffffu, fill );
                const uint32_t mb   = __ballot_sync( 0xffffffffu, isJob && !fill );
                if ( isJob )
                {
                    const uint32_t slot = fill ? jbase + __popc( mf & lanemask_lt() )
                                               : b.capProbes - 1u - ( gbase + __popc( mb & lanemask_lt() ) );
                    if ( slot < b.capProbes )
                        b.jobs[ slot ] = make_uint4( chunk + q, i, en.x, en.y << 16 );
                }
                jbase += __popc( mf );
                gbase += __popc( mb );
            }
            if ( lane == 0 )
            {
                if ( !fits )
                    atomicOr( &b.counts->overflow, (uint32_t)kOverflowProbes );
                b.chunkStart[ i ] = chunk;
                b.chunkLen[ i ]   = fits ? kept : 0u;
                b.singCnt[ i ]    = fits ? nSing : 0u;
                b.regCnt[ i ]     = fits ? nReg : 0u;
            }
        }

        // W warps per block; with kQueue the grid is persistent and its warps take tiles of atoms
        // from a work counter (in sorted order: molecule by molecule, reference-grid cell by cell),
        // else warp w of block k takes atom k W + w (the default: the block scheduler hands out the
        // atoms with no counter atomic, measured 50 us faster at 100k atoms)
        constexpr uint32_t kProbeTile = 4;
        template<int W, bool kQueue>
        __global__ void __launch_bounds__( 32 * W, 32 / W ) k_probes( Build b )
        {
            pdl_begin();
            extern __shared__ __align__( 16 ) unsigned char smemRaw[];
            const uint32_t  warp = threadIdx.x >> 5, lane = lane_id();
            unsigned char * mine = smemRaw + warp * probe_smem_per_warp( b.cap );
            if ( !kQueue )
            {
                const uint32_t i = blockIdx.x * W + warp;
                if ( i < b.n )
                    probes_of_atom( b, i, mine );
                return;
            }
            // work items: tiles of kProbeTile consecutive atoms of the sorted order (molecule by
            // molecule, reference-grid cell by cell), one counter atomic per tile
            for ( uint32_t it = 0; it < b.n; it++ ) // bounded: every turn takes a new tile
            {
                uint32_t t = 0;
                if ( lane == 0 )
                    t = atomicAdd( &b.counts->probeCursor, kProbeTile );
                t = __shfl_sync( 0xffffffffu, t, 0 );
                if ( t >= b.n )
                    break;
                for ( uint32_t i = t; i < t + kProbeTile && i < b.n; i++ )
                {
                    probes_of_atom( b, i, mine );
                    __syncwarp();
                }
            }
        }

        // Exact position of one side of a kept probe in double precision, rounded once to
        // float32; returns the singular flag. Out of line, so that its conversions run
        // only for the few probes whose float-float position cannot be rounded safely.
        __device__ __noinline__ bool fill_position_d( float4 ai, float4 aj, float4 ak, float rpf, uint32_t side, float3 & pf )
        {
            const double rp = (double)rpf;
            d3           x[ 2 ];
            double       h2 = 0.0;
            solve_d( D3( ai ), (double)ai.w, D3( aj ), (double)aj.w, D3( ak ), (double)ak.w, rp, x[ 0 ], x[ 1 ], h2 );
            const d3 xs = side ? x[ 1 ] : x[ 0 ];
            pf          = make_float3( __double2float_rn( xs.x ), __double2float_rn( xs.y ), __double2float_rn( xs.z ) );
            return singular_d( h2, rp );
        }

        // The double-precision pass, one job per thread with full warps: exact
        // probe positions (the solve of findIntersectionsBetweenCircles in IEEE
        // double, rounded once to float32) and the decisions the float32 screen
        // left open.
        __global__ void __launch_bounds__( 128 ) k_probe_jobs( Build b )
        {
            pdl_begin();
            const uint32_t nFill = min( b.counts->jobs, b.capProbes );
            const uint32_t nBand = min( b.counts->bandJobs, b.capProbes - nFill );
            const double   rp    = (double)b.rp;
            const uint32_t lane  = lane_id();
            uint32_t       fp64 = 0, full64 = 0, ffMiss = 0;
            // fill jobs, one per thread: float-float first, double precision only where
            // the float-float result cannot decide
            for ( uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nFill; t += gridDim.x * blockDim.x )
            {
                const uint4    jb   = b.jobs[ t ];
                const uint32_t ent  = jb.x, i = jb.y;
                const uint32_t sj   = jb.z & 0xffffu, sk = jb.z >> 16;
                const uint32_t side = ( jb.w >> 16 ) & 0xffu;
                // the empty jobs of an atom whose entries did not fit (a build that is redone larger)
                if ( i >= b.n || ent >= b.capProbes || sj >= b.cap || sk >= b.cap )
                    continue;
                const size_t   row  = (size_t)i * b.cap;
                const float4   ai = b.atoms[ i ], aj = b.atoms[ b.nbr[ row + sj ] ], ak = b.atoms[ b.nbr[ row + sk ] ];
                int4           cid  = b.stageCid[ ent ];
                int            aw   = cid.w < 0 ? -cid.w : cid.w;
                float3         pf;
                bool           sing = false;
                if ( !solve_ff( ai, aj, ak, b.rp, side, aw == 3, pf, sing ) )
                {
                    ffMiss++;
                    sing = fill_position_d( ai, aj, ak, b.rp, side, pf );
                }
                if ( aw == 3 )
                {
                    aw                = sing ? 2 : 1;
                    cid.w             = cid.w < 0 ? -aw : aw;
                    b.stageCid[ ent ] = cid;
                    atomicAdd( aw == 2 ? &b.singCnt[ i ] : &b.regCnt[ i ], 1u );
                }
                b.stagePos[ ent ] = make_float4( pf.x, pf.y, pf.z, (float)cid.w );
            }
            // band candidates, one per thread (the double-precision solve, occlusion and
            // singular test), stored from the top of the job array
            for ( uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < nBand; g += gridDim.x * blockDim.x )
            {
                const uint4    jb  = b.jobs[ b.capProbes - 1u - g ];
                const uint32_t ent = jb.x, i = jb.y;
                const uint32_t sj  = jb.z & 0xffffu, sk = jb.z >> 16;
                if ( i >= b.n || ent + 1u >= b.capProbes || sj >= b.cap || sk >= b.cap )
                    continue; // an empty job
                const size_t   row = (size_t)i * b.cap;
                const float4   ai = b.atoms[ i ], aj = b.atoms[ b.nbr[ row + sj ] ], ak = b.atoms[ b.nbr[ row + sk ] ];
                d3             x[ 2 ];
                double         h2 = 0.0;
                const bool     ok = solve_d( D3( ai ), (double)ai.w, D3( aj ), (double)aj.w, D3( ak ), (double)ak.w, rp, x[ 0 ], x[ 1 ], h2 );
                full64++;
                if ( !ok )
                    continue;
                bool vis[ 2 ] = { true, true };
                occlusion_d( b, i, ai, sj, sk, x, vis, fp64 );
                for ( int e = 0; e < 2; e++ )
                {
                    if ( !vis[ e ] )
                        continue;
                    int4      cid = b.stageCid[ ent + e ];
                    const int aw  = singular_d( h2, rp ) ? 2 : 1;
                    cid.w         = e == 0 ? aw : -aw;
                    b.stageCid[ ent + e ] = cid;
                    b.stagePos[ ent + e ] = make_float4( __double2float_rn( x[ e ].x ), __double2float_rn( x[ e ].y ),
                                                         __double2float_rn( x[ e ].z ), (float)cid.w );
                    atomicAdd( aw == 2 ? &b.singCnt[ i ] : &b.regCnt[ i ], 1u );
                }
            }
            for ( int o = 16; o > 0; o >>= 1 )
            {
                fp64 += __shfl_xor_sync( 0xffffffffu, fp64, o );
                full64 += __shfl_xor_sync( 0xffffffffu, full64, o );
                ffMiss += __shfl_xor_sync( 0xffffffffu, ffMiss, o );
            }
            if ( lane == 0 )
            {
                if ( fp64 )
                    atomicAdd( &b.counts->fp64[ kFp64Occlusion ], fp64 );
                if ( full64 )
                    atomicAdd( &b.counts->fp64[ kFp64Solve ], full64 );
                if ( ffMiss )
                    atomicAdd( &b.counts->fp64[ kFp64Positions ], ffMiss );
            }
        }

        // Stable placement, singular probes first (the reference partitions with an
        // unstable sort, operations.inl:128-135), and the fill of
        // fillIntersections (operations.cu:206-269; exterior ssesdf/operations.cu:287-329).
        // eight atoms per warp, four lanes per atom (an atom keeps ~2 probes)
        constexpr uint32_t kPlaceGroup = 4;

        __global__ void __launch_bounds__( 32 * kWarpsPerBlock ) k_place( Build b )
        {
            pdl_begin();
            const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t grp = lane / kPlaceGroup, gl = lane % kPlaceGroup;
            const uint32_t gmask = ( ( 1u << kPlaceGroup ) - 1u ) << ( grp * kPlaceGroup );
            const uint32_t i     = ( blockIdx.x * kWarpsPerBlock + warp ) * ( 32 / kPlaceGroup ) + grp;
            if ( i == 0 && gl == 0 )
                b.counts->I = b.counts->Q + b.counts->regTotal;
            const bool     atom  = i < b.n;
            const uint32_t Q     = b.counts->Q;
            const uint32_t cnt   = atom ? b.chunkLen[ i ] : 0u;
            const uint32_t chunk = atom ? b.chunkStart[ i ] : 0u;
            uint32_t       so = atom ? b.singOff[ i ] : 0u, ro = atom ? Q + b.regOff[ i ] : 0u;
            uint32_t       sq = so; // singular index (molecule-major)
            if ( atom && b.nMol > 1 )
            {
                // singular probes first within each molecule of the batch
                const uint32_t m  = mol_of( b, i );
                const uint32_t a0 = b.molStart[ m ], a1 = b.molStart[ m + 1 ];
                const uint32_t s0 = b.singOff[ a0 ], r0 = b.regOff[ a0 ];
                so                = r0 + b.singOff[ i ];
                ro                = s0 + ( b.singOff[ a1 ] - s0 ) + b.regOff[ i ];
            }
            uint32_t most = cnt;
            for ( int o = 16; o > 0; o >>= 1 )
                most = max( most, __shfl_xor_sync( 0xffffffffu, most, o ) );
            const uint32_t lt = lanemask_lt() & gmask;
            for ( uint32_t m0 = 0; m0 < most; m0 += kPlaceGroup )
            {
                const uint32_t m     = m0 + gl;
                const bool     valid = m < cnt;
                int4           cid   = make_int4( 0, 0, 0, 0 );
                if ( valid )
                    cid = b.stageCid[ chunk + m ];
                const bool     live = valid && cid.w != 0; // band entries without a point are holes
                const bool     sing = live && ( cid.w == 2 || cid.w == -2 );
                const uint32_t ms   = __ballot_sync( 0xffffffffu, sing ) & gmask;
                const uint32_t mr   = __ballot_sync( 0xffffffffu, live && !sing ) & gmask;
                const uint32_t dst  = sing ? so + __popc( ms & lt ) : ro + __popc( mr & lt );
                if ( sing && b.nMol > 1 )
                    b.singList[ sq + __popc( ms & lt ) ] = dst;
                so += __popc( ms );
                ro += __popc( mr );
                sq += __popc( ms );
                if ( !live )
                    continue;
                b.probePos[ dst ] = b.stagePos[ chunk + m ];
                b.probeCid[ dst ] = cid;
                b.probeIds[ dst ] = b.stageIds[ chunk + m ];
                if ( b.mode == 0 )
                {
                    // partial-circle numbers beyond the capacity exist only in a build that overflowed
                    // C1 (flagged by k_emit) and is built again after regrowing
                    if ( (uint32_t)cid.x < b.capC1 )
                        atomicAdd( &b.ccount[ cid.x ], 1u );
                    if ( (uint32_t)cid.y < b.capC1 )
                        atomicAdd( &b.ccount[ cid.y ], 1u );
                    if ( (uint32_t)cid.z < b.capC1 )
                        atomicAdd( &b.ccount[ cid.z ], 1u );
                }
                else
                {
                    // exterior: the probe's three circles become tori (status 1 -> 2)
                    if ( b.status[ cid.x ] == 1 )
                        b.status[ cid.x ] = 2;
                    if ( b.status[ cid.y ] == 1 )
                        b.status[ cid.y ] = 2;
                    if ( b.status[ cid.z ] == 1 )
                        b.status[ cid.z ] = 2;
                }
            }
        }

        __global__ void k_lists( Build b )
        {
            pdl_begin();
            const uint32_t I = min( b.counts->I, b.capProbes );
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < I; q += gridDim.x * blockDim.x )
            {
                const int4     cid = b.probeCid[ q ];
                const uint32_t t3[ 3 ] = { (uint32_t)cid.x, (uint32_t)cid.y, (uint32_t)cid.z };
                for ( int e = 0; e < 3; e++ )
                {
                    const uint32_t t = t3[ e ];
                    if ( t >= b.capC1 ) // only in a build that overflowed C1 (see k_place)
                        continue;
                    const uint32_t pos = b.cstart[ t ] + atomicAdd( &b.ccursor[ t ], 1u );
                    b.clist[ pos ]     = q;
                }
            }
        }

        // Segment counts per partial circle, and the list of the circles carrying
        // segments (in any order) for the full-warp segment pass: one counter atomic per
        // block and step (a single counter taken by every warp serialises at L2).
        __global__ void __launch_bounds__( 256 ) k_segment_counts( Build b )
        {
            pdl_begin();
            __shared__ uint32_t warpBase[ 8 ];
            __shared__ uint32_t blockBase;
            const uint32_t      C1   = min( b.counts->C1, b.capC1 );
            const uint32_t      warp = threadIdx.x >> 5, lane = lane_id();
            for ( uint32_t t0 = blockIdx.x * blockDim.x; t0 < C1; t0 += gridDim.x * blockDim.x )
            {
                const uint32_t t  = t0 + threadIdx.x;
                uint32_t       cc = 0;
                if ( t < C1 )
                {
                    cc            = b.ccount[ t ];
                    b.segCnt[ t ] = min( cc, b.segCap ) / 2u;
                    if ( cc > b.segCap )
                        atomicAdd( &b.counts->segTruncated, 1u );
                }
                const uint32_t mk = __ballot_sync( 0xffffffffu, cc >= 2 );
                if ( lane == 0 )
                    warpBase[ warp ] = (uint32_t)__popc( mk );
                __syncthreads();
                if ( threadIdx.x == 0 )
                {
                    uint32_t tot = 0;
                    for ( uint32_t w = 0; w < ( blockDim.x >> 5 ); w++ )
                    {
                        const uint32_t c = warpBase[ w ];
                        warpBase[ w ]    = tot;
                        tot += c;
                    }
                    blockBase = tot ? atomicAdd( &b.counts->segCircles, tot ) : 0u;
                }
                __syncthreads();
                if ( cc >= 2 )
                {
                    const uint32_t at = blockBase + warpBase[ warp ] + __popc( mk & lanemask_lt() );
                    if ( at < b.capC1 )
                        b.segList[ at ] = t;
                }
                __syncthreads(); // warpBase and blockBase are rewritten by the next step
            }
        }

        // ---- segments (buildSegments, operations.inl:552-668) ---------------
        constexpr float kKeyTol = 1.0f / 32768.0f; // 2^-15: float32 pseudo-angles closer than this go to double

        __device__ __forceinline__ ff ff_dot( ff ax, ff ay, ff az, ff bx, ff by, ff bz )
        {
            return ff_add( ff_add( ff_mul( ax, bx ), ff_mul( ay, by ) ), ff_mul( az, bz ) );
        }
        __device__ __forceinline__ bool ff_gt( ff a, ff b ) { return a.hi > b.hi || ( a.hi == b.hi && a.lo > b.lo ); }

        // Float-float pseudo-angle keys of the probes of circle (i, j) (the double-
        // precision keys' formula): their order is the double-precision order whenever
        // every key is more than the bound E away from its neighbours in the order
        // (the start key 0 included) and every side test more than its bound from 0.
        // Returns false otherwise (the caller then sorts in double precision).
        __device__ bool segment_order_ff( const Build & b, const float4 & ai, const float4 & aj, const float4 & spos,
                                          const uint32_t * lst, uint32_t nb, bool reverse, uint8_t * ord )
        {
            const ff R1 = two_sum( ai.w, b.rp ), R2 = two_sum( aj.w, b.rp );
            const ff dx = two_sum( aj.x, -ai.x ), dy = two_sum( aj.y, -ai.y ), dz = two_sum( aj.z, -ai.z );
            const ff d  = ff_dot( dx, dy, dz, dx, dy, dz );
            if ( !( d.hi > 0.f ) )
                return false;
            const ff tt  = ff_div( ff_add( ff_sub( ff_mul( R1, R1 ), ff_mul( R2, R2 ) ), d ), ff_scale( d, 2.f ) );
            const ff cx  = ff_mul( dx, tt ), cy = ff_mul( dy, tt ), cz = ff_mul( dz, tt ); // centre - c_i
            const ff inv = ff_div( ff_of( 1.f ), ff_sqrt( d ) );
            const ff nx = ff_mul( dx, inv ), ny = ff_mul( dy, inv ), nz = ff_mul( dz, inv );
            const ff rx = ff_sub( two_sum( spos.x, -ai.x ), cx ), ry = ff_sub( two_sum( spos.y, -ai.y ), cy ),
                     rz = ff_sub( two_sum( spos.z, -ai.z ), cz );
            const float E = 5.820766091346741e-11f; // 2^-34: 256 float-float roundings on keys of size <= 4
            ff          key[ kSegBuf ];
            key[ 0 ] = ff_of( 0.f );
            ord[ 0 ] = 0;
            for ( uint32_t m = 1; m < nb; m++ )
            {
                const float4 pm = b.probePos[ lst[ m ] ];
                const ff     wx = ff_sub( two_sum( pm.x, -ai.x ), cx ), wy = ff_sub( two_sum( pm.y, -ai.y ), cy ),
                         wz = ff_sub( two_sum( pm.z, -ai.z ), cz );
                const ff ux = reverse ? wx : rx, uy = reverse ? wy : ry, uz = reverse ? wz : rz;
                const ff vx = reverse ? rx : wx, vy = reverse ? ry : wy, vz = reverse ? rz : wz;
                const ff uu = ff_dot( ux, uy, uz, ux, uy, uz ), vv = ff_dot( vx, vy, vz, vx, vy, vz );
                const ff l  = ff_sqrt( ff_mul( uu, vv ) );
                if ( !( l.hi > 0.f ) )
                    return false;
                ff c = ff_div( ff_dot( ux, uy, uz, vx, vy, vz ), l );
                // det = u . (v x n)
                const ff det = ff_dot( ux, uy, uz, ff_sub( ff_mul( vy, nz ), ff_mul( vz, ny ) ), ff_sub( ff_mul( vz, nx ), ff_mul( vx, nz ) ),
                                       ff_sub( ff_mul( vx, ny ), ff_mul( vy, nx ) ) );
                if ( !( fabsf( det.hi ) > E * l.hi ) )
                    return false;
                if ( c.hi > 1.f )
                    c = ff_of( 1.f );
                if ( c.hi < -1.f )
                    c = ff_of( -1.f );
                const ff kv = det.hi > 0.f ? ff_sub( ff_of( 1.f ), c ) : ff_add( ff_of( 3.f ), c );
                uint32_t p  = m;
                while ( p > 0 && ff_gt( key[ p - 1 ], kv ) )
                {
                    key[ p ] = key[ p - 1 ];
                    ord[ p ] = ord[ p - 1 ];
                    p--;
                }
                key[ p ] = kv;
                ord[ p ] = (uint8_t)m;
            }
            for ( uint32_t m = 1; m < nb; m++ )
                if ( !( ff_sub( key[ m ], key[ m - 1 ] ).hi > E ) )
                    return false;
            return true;
        }

        // Orders the probes of circle t along the circle and writes its segments:
        // float32 keys first; when two keys (or a key and the start) are closer than
        // kKeyTol, or a side test is ambiguous, float-float keys, and where even those
        // are too close, the double-precision keys decide.
        __global__ void __launch_bounds__( 128 ) k_segments( Build b )
        {
            pdl_begin();
            const uint32_t nc  = min( b.counts->segCircles, b.capC1 );
            uint32_t       ovf = 0, fp64 = 0;
            for ( uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nc; idx += gridDim.x * blockDim.x )
            {
                const uint32_t t   = b.segList[ idx ];
                const uint32_t cnt = b.ccount[ t ];
                if ( cnt > (uint32_t)kSegBuf )
                {
                    ovf |= kOverflowList;
                    continue;
                }
                uint32_t         lst[ kSegBuf ];
                const uint32_t * src = b.clist + b.cstart[ t ];
                for ( uint32_t m = 0; m < cnt; m++ )
                {
                    // insertion into ascending order
                    const uint32_t v = src[ m ];
                    uint32_t       p = m;
                    while ( p > 0 && lst[ p - 1 ] > v )
                    {
                        lst[ p ] = lst[ p - 1 ];
                        p--;
                    }
                    lst[ p ] = v;
                }
                const uint32_t nb  = min( cnt, b.segCap );
                const uint32_t sIJ = b.trimSlot[ t ];
                const uint32_t i   = sIJ / b.cap;
                const uint32_t j   = b.nbr[ sIJ ];
                const float4   ai = b.atoms[ i ], aj = b.atoms[ j ];

                const uint32_t st          = lst[ 0 ];
                const int4     sids        = b.probeIds[ st ];
                const float4   spos        = b.probePos[ st ];
                const bool     isSecondary = (int)i == sids.x && (int)j == sids.z;
                const bool     reverse     = ( spos.w < 0.f ) != isSecondary; // direction < 0

                // float32 keys, coordinates relative to atom i. Two probes need none: the first
                // probe's key is 0 and every other key is >= 0, so the stable order is (0, 1)
                // whatever the keys (the circles of two probes are most of them)
                float   key[ kSegBuf ];
                uint8_t ord[ kSegBuf ];
                ord[ 0 ]   = 0;
                ord[ 1 ]   = 1;
                bool exact = true;
                if ( nb > 2 )
                {
                    const float Ri = ai.w + b.rp, Rj = aj.w + b.rp;
                    const f3    dj = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
                    const float d  = dot( dj, dj );
                    const f3    c  = dj * ( ( Ri * Ri - Rj * Rj + d ) / ( 2.f * d ) );
                    const f3    n  = dj * rsqrtf( d );
                    const f3    rf = F3( spos.x - ai.x, spos.y - ai.y, spos.z - ai.z ) - c;
                    key[ 0 ]       = 0.f;
                    ord[ 0 ]       = 0;
                    for ( uint32_t m = 1; m < nb && exact; m++ )
                    {
                        const float4 pm = b.probePos[ lst[ m ] ];
                        f3           v1 = rf;
                        f3           v2 = normalize( F3( pm.x - ai.x, pm.y - ai.y, pm.z - ai.z ) - c );
                        if ( reverse )
                        {
                            const f3 tmp = v1;
                            v1           = v2;
                            v2           = tmp;
                        }
                        const float l   = sqrtf( dot( v1, v1 ) * dot( v2, v2 ) );
                        const float cs  = fmaxf( -1.f, fminf( dot( v1, v2 ) / l, 1.f ) );
                        const float det = dot( v1, cross( v2, n ) ) / l;
                        // next to angle 0 the side test decides between key 0 and key 4
                        if ( fabsf( det ) < kKeyTol && cs > 0.f )
                            exact = false;
                        const float kv = det > 0.f ? 1.f - cs : 3.f + cs;
                        uint32_t    p  = m;
                        while ( p > 0 && key[ p - 1 ] > kv )
                        {
                            key[ p ] = key[ p - 1 ];
                            ord[ p ] = ord[ p - 1 ];
                            p--;
                        }
                        key[ p ] = kv;
                        ord[ p ] = (uint8_t)m;
                    }
                    for ( uint32_t m = 1; m < nb && exact; m++ )
                        if ( key[ m ] - key[ m - 1 ] < kKeyTol )
                            exact = false;
                }
                if ( nb > 2 && !exact && !segment_order_ff( b, ai, aj, spos, lst, nb, reverse, ord ) )
                {
                    // double-precision keys (the oracle's), same stable ordering
                    fp64++;
                    const dcircle geo = dcircle_geometry( D3( ai ), (double)ai.w, D3( aj ), (double)aj.w, (double)b.rp );
                    const d3      ref = dsub( D3( spos ), geo.center );
                    double        dk[ kSegBuf ];
                    dk[ 0 ]  = 0.0;
                    ord[ 0 ] = 0;
                    for ( uint32_t m = 1; m < nb; m++ )
                    {
                        d3 v1 = ref;
                        d3 v2 = dnrm( dsub( D3( b.probePos[ lst[ m ] ] ), geo.center ) );
                        if ( reverse )
                        {
                            const d3 tmp = v1;
                            v1           = v2;
                            v2           = tmp;
                        }
                        const double kv = dpseudo_angle( v1, v2, geo.normal );
                        uint32_t     p  = m;
                        while ( p > 0 && dk[ p - 1 ] > kv )
                        {
                            dk[ p ]  = dk[ p - 1 ];
                            ord[ p ] = ord[ p - 1 ];
                            p--;
                        }
                        dk[ p ]  = kv;
                        ord[ p ] = (uint8_t)m;
                    }
                }
                uint32_t out = b.segOff[ t ];
                for ( uint32_t m = 0; m + 1 < nb; m += 2, out++ )
                {
                    uint32_t a1 = lst[ ord[ m ] ], a2 = lst[ ord[ m + 1 ] ];
                    if ( reverse )
                    {
                        const uint32_t tmp = a1;
                        a1                 = a2;
                        a2                 = tmp;
                    }
                    if ( out < b.capSeg )
                        b.segments[ out ] = make_uint4( i, j, a1, a2 );
                    else
                        ovf |= kOverflowSeg;
                }
            }
            if ( ovf )
                atomicOr( &b.counts->overflow, ovf );
            if ( fp64 )
                atomicAdd( &b.counts->fp64[ kFp64Segments ], fp64 );
        }

        // ---- neighbours of singular probes -------------------------------------
        __global__ void __launch_bounds__( 32 * kWarpsPerBlock ) k_probe_neighbors( Build b )
        {
            pdl_begin();
            __shared__ unsigned long long buf[ kWarpsPerBlock ][ kSnbrBuf ];
            __shared__ uint32_t           rowStart[ kWarpsPerBlock ][ 25 ], rowPre[ kWarpsPerBlock ][ 26 ];
            const uint32_t                warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t                Q    = min( b.counts->Q, b.capProbes );
            const float                   t2   = 2.f * b.rp;
            // one molecule: the reference-grid hash has 3 log2(size) bits and the index of a singular
            // probe pBits; when they fit in 31 bits the keys are sorted as 32-bit values
            const uint32_t pBits  = Q > 1 ? 32u - (uint32_t)__clz( (int)( Q - 1u ) ) : 1u;
            const uint32_t hBits  = 3u * ( 31u - (uint32_t)__clz( b.grid.size > 0 ? b.grid.size : 1 ) );
            const bool     narrow = b.nMol <= 1 && hBits + pBits <= 31u;
            uint32_t                      fp64 = 0, trunc = 0;
            for ( uint32_t q = blockIdx.x * kWarpsPerBlock + warp; q < Q; q += gridDim.x * kWarpsPerBlock )
            {
                const uint32_t pi = b.nMol > 1 ? b.singList[ q ] : q; // probe index of singular probe q
                const float4   pq = b.probePos[ pi ];
                const uint32_t m  = b.nMol > 1 ? mol_of( b, (uint32_t)b.probeIds[ pi ].x ) : 0u;
                const FineGrid g  = b.fine[ m ];
                const uint32_t * cells = b.cellStart + cell_base( b, m );
                const bool       span2 = g.span == 2;
                Rows             rows;
                uint32_t         total;
                __syncwarp();
                if ( span2 )
                    total = stencil_rows_span2( g, cells, pq, t2 + 0.005f, rowStart[ warp ], rowPre[ warp ] );
                else
                {
                    stencil_rows( g, cells, fine_cell( g, pq.x, pq.y, pq.z ), rows );
                    total = rows.total;
                }
                uint32_t count = 0;
                for ( uint32_t base = 0; base < total; base += 32 )
                {
                    const uint32_t     f    = base + lane;
                    bool               pass = false;
                    unsigned long long key  = 0;
                    if ( f < total )
                    {
                        const uint32_t idx = span2 ? row_item_span2( rowStart[ warp ], rowPre[ warp ], f ) : row_item( rows, f );
                        const uint32_t p   = b.cellItems[ idx ];
                        if ( p != q )
                        {
                            const float4 pp = b.cellPos[ idx ];
                            const f3     dv = F3( pq.x - pp.x, pq.y - pp.y, pq.z - pp.z );
                            const float  d2 = dot( dv, dv );
                            const float  m  = d2 - t2 * t2;
                            const float  e  = kRel * ( d2 + t2 * t2 + 1.f );
                            if ( m < -e )
                                pass = true;
                            else if ( !( m > e ) )
                            {
                                pass = probe_pair_d( pq, pp, b.rp );
                                fp64++;
                            }
                            if ( pass )
                                key = ( (unsigned long long)__float_as_uint( pp.w ) << 32 ) | p;
                        }
                    }
                    const uint32_t mask = __ballot_sync( 0xffffffffu, pass );
                    const uint32_t pos  = count + __popc( mask & lanemask_lt() );
                    if ( pass && pos < kSnbrBuf )
                        buf[ warp ][ pos ] = key;
                    count += __popc( mask );
                }
                __syncwarp();
                const uint32_t     held = count < kSnbrBuf ? count : kSnbrBuf;
                const uint32_t     kept = held < kMaxProbeNbr ? held : kMaxProbeNbr;
                unsigned long long key0;
                if ( held <= 64 )
                {
                    // in registers (the common case)
                    key0                    = lane < held ? buf[ warp ][ lane ] : ~0ull;
                    unsigned long long key1 = lane + 32 < held ? buf[ warp ][ lane + 32 ] : ~0ull;
                    if ( narrow )
                    {
                        // (hash, index) packed into 32 bits where both fit below the padding value:
                        // the same order with half the shuffles and compares
                        const auto pack = [ & ]( unsigned long long k ) {
                            return k == ~0ull ? 0xffffffffu : ( (uint32_t)( k >> 32 ) << pBits ) | (uint32_t)k;
                        };
                        uint32_t n0 = pack( key0 ), n1 = pack( key1 );
                        warp_sort64( n0, n1, held > 32 );
                        key0 = n0 == 0xffffffffu ? ~0ull
                                                 : ( (unsigned long long)( n0 >> pBits ) << 32 ) | ( n0 & ( ( 1u << pBits ) - 1u ) );
                    }
                    else
                        warp_sort64( key0, key1, held > 32 );
                }
                else
                {
                    warp_bitonic_sort<unsigned long long>( buf[ warp ], held, kSnbrBuf, ~0ull );
                    key0 = buf[ warp ][ lane ];
                }
                if ( lane < kept )
                {
                    const uint32_t p  = (uint32_t)( key0 & 0xffffffffull );
                    const float4   pp = b.probePos[ b.nMol > 1 ? b.singList[ p ] : p ];
                    const float    wv = b.mode == 0 ? __fmul_rn( __fmul_rn( pq.x, pq.y ), pq.z ) : 0.f;
                    b.probeNbrs[ (size_t)q * kMaxProbeNbr + lane ]   = make_float4( pp.x, pp.y, pp.z, wv );
                    b.probeNbrIdx[ (size_t)q * kMaxProbeNbr + lane ] = p;
                }
                if ( lane == 0 )
                {
                    b.probeIds[ pi ].w = (int)kept;
                    if ( count > kMaxProbeNbr )
                        trunc++;
                }
                __syncwarp();
            }
            for ( int o = 16; o > 0; o >>= 1 )
                fp64 += __shfl_xor_sync( 0xffffffffu, fp64, o );
            if ( lane == 0 )
            {
                if ( fp64 )
                    atomicAdd( &b.counts->fp64[ kFp64SingularNbr ], fp64 );
                if ( trunc )
                    atomicAdd( &b.counts->snbrTruncated, trunc );
            }
        }

        // exterior: probe position w becomes the index of its neighbour block
        // (ssesdf/operations.cu:397); done after every neighbour search read xyz
        __global__ void k_probe_w( Build b )
        {
            pdl_begin();
            const uint32_t Q = min( b.counts->Q, b.capProbes );
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < Q; q += gridDim.x * blockDim.x )
            {
                uint32_t pi = q, local = q;
                if ( b.nMol > 1 )
                {
                    // index of the neighbour block within the probe's molecule
                    pi    = b.singList[ q ];
                    local = q - b.singOff[ b.molStart[ mol_of( b, (uint32_t)b.probeIds[ pi ].x ) ] ];
                }
                b.probePos[ pi ].w = (float)(int)( local * kMaxProbeNbr );
            }
        }

        // ---- batches: per-molecule counts and molecule-local ids ----------------
        __global__ void k_mol_counts( Build b )
        {
            pdl_begin();
            for ( uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < b.nMol; m += gridDim.x * blockDim.x )
            {
                const uint32_t a0 = b.molStart[ m ], a1 = b.molStart[ m + 1 ];
                uint32_t *     o  = b.molCounts + (size_t)m * kMolFields;
                const uint32_t q0 = b.singOff[ a0 ], q1 = b.singOff[ a1 ];
                o[ kMolAtoms ]        = a1 - a0;
                o[ kMolSingular ]     = q1 - q0;
                o[ kMolProbes ]       = ( q1 - q0 ) + ( b.regOff[ a1 ] - b.regOff[ a0 ] );
                o[ kMolAtomBase ]     = a0;
                o[ kMolProbeBase ]    = q0 + b.regOff[ a0 ];
                o[ kMolSingularBase ] = q0;
                o[ kMolC1 ]           = b.partOff[ a1 ] - b.partOff[ a0 ];
                o[ kMolC1Base ]       = b.partOff[ a0 ];
                if ( b.mode == 0 )
                {
                    o[ kMolSectors ]     = b.visOff[ a1 ] - b.visOff[ a0 ];
                    o[ kMolSectorBase ]  = b.visOff[ a0 ];
                    o[ kMolFull ]        = b.fullOff[ a1 ] - b.fullOff[ a0 ];
                    o[ kMolFullBase ]    = b.fullOff[ a0 ];
                    // segOff holds min(C1, capC1) + 1 entries (larger C1: a build that is done again)
                    const uint32_t t0    = min( b.partOff[ a0 ], b.capC1 ), t1 = min( b.partOff[ a1 ], b.capC1 );
                    o[ kMolSegments ]    = b.segOff[ t1 ] - b.segOff[ t0 ];
                    o[ kMolSegmentBase ] = b.segOff[ t0 ];
                    o[ kMolTori ] = o[ kMolToriBase ] = 0;
                }
                else
                {
                    o[ kMolTori ]     = b.torOff[ a1 ] - b.torOff[ a0 ];
                    o[ kMolToriBase ] = b.torOff[ a0 ];
                    o[ kMolSectors ] = o[ kMolSectorBase ] = o[ kMolFull ] = o[ kMolFullBase ] = 0;
                    o[ kMolSegments ] = o[ kMolSegmentBase ] = 0;
                }
            }
        }

        // Ids in the output buffers become molecule-local, so that each molecule's
        // slice of a batch reads exactly like the buffers of its own build.
        __global__ void k_mol_rebase( Build b )
        {
            pdl_begin();
            const uint32_t stride = gridDim.x * blockDim.x;
            const uint32_t t0     = blockIdx.x * blockDim.x + threadIdx.x;
            for ( uint32_t s = t0; s < b.n; s += stride )
            {
                const uint32_t m  = mol_of( b, s );
                const uint32_t a0 = b.molStart[ m ];
                b.perm[ s ] -= a0;
                if ( b.mode == 0 )
                {
                    const uint32_t v0 = b.molCounts[ (size_t)m * kMolFields + kMolSectorBase ];
                    uint2          cv = b.convex[ s ];
                    b.convex[ s ]     = make_uint2( cv.x - v0, cv.y - v0 );
                }
            }
            const uint32_t I = min( b.counts->I, b.capProbes );
            for ( uint32_t p = t0; p < I; p += stride )
            {
                int4           id = b.probeIds[ p ];
                const uint32_t a0 = b.molStart[ mol_of( b, (uint32_t)id.x ) ];
                b.probeIds[ p ]   = make_int4( id.x - (int)a0, id.y - (int)a0, id.z - (int)a0, id.w );
            }
            if ( b.mode != 0 )
                return;
            const uint32_t F = min( b.counts->F, b.capFull );
            for ( uint32_t f = t0; f < F; f += stride )
            {
                const uint2    c  = b.fullCircles[ f ];
                const uint32_t a0 = b.molStart[ mol_of( b, c.x ) ];
                b.fullCircles[ f ] = make_uint2( c.x - a0, c.y - a0 );
            }
            const uint32_t S = min( b.counts->S, b.capSeg );
            for ( uint32_t k = t0; k < S; k += stride )
            {
                const uint4    g  = b.segments[ k ];
                const uint32_t m  = mol_of( b, g.x );
                const uint32_t a0 = b.molStart[ m ], p0 = b.molCounts[ (size_t)m * kMolFields + kMolProbeBase ];
                b.segments[ k ]   = make_uint4( g.x - a0, g.y - a0, g.z - p0, g.w - p0 );
            }
        }

        // ---- exterior tori ---------------------------------------------------
        // squared radius of circle (i, j) in double precision from the float32 atoms (out of
        // line: its conversions run only for the nearly tangent circles that need it)
        __device__ __noinline__ float torus_r2_d( float4 ai, float4 aj, float rp )
        {
            const double Rid = (double)ai.w + (double)rp, Rjd = (double)aj.w + (double)rp;
            const double ex = (double)aj.x - (double)ai.x, ey = (double)aj.y - (double)ai.y, ez = (double)aj.z - (double)ai.z;
            const double dd = ex * ex + ey * ey + ez * ez;
            const double td = ( Rid * Rid - Rjd * Rjd + dd ) / ( 2.0 * dd );
            return (float)( Rid * Rid - td * td * dd );
        }

        // status-2 circles per atom: four atoms per warp, eight lanes per atom
        __global__ void __launch_bounds__( 32 * kWarpsPerBlock ) k_tori_count( Build b )
        {
            pdl_begin();
            const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t grp = lane / 8, gl = lane % 8;
            const uint32_t i  = ( blockIdx.x * kWarpsPerBlock + warp ) * 4 + grp;
            const uint32_t ni = i < b.n ? b.nbrCount[ i ] : 0u;
            uint32_t       c  = 0;
#pragma unroll 4
            for ( uint32_t s = gl; s < ni; s += 8 )
                c += b.status[ (size_t)i * b.cap + s ] == 2;
            for ( int o = 4; o > 0; o >>= 1 )
                c += __shfl_xor_sync( 0xffffffffu, c, o );
            if ( i < b.n && gl == 0 )
                b.torCnt[ i ] = c;
        }

        // Torus of circle (i, s) of status 2 (fillCircles, ssesdf/operations.cu:246-285), in
        // coordinates relative to atom i; writes its three records at idx
        __device__ __forceinline__ void torus_of( const Build & b, uint32_t i, uint32_t s, uint32_t idx, uint32_t & ovf,
                                                  uint32_t & degenerate )
        {
            const float4 ai = b.atoms[ i ];
            const float4 aj = b.atoms[ b.nbr[ (size_t)i * b.cap + s ] ];
            const float  Ri = ai.w + b.rp;
            const float  Rj = aj.w + b.rp;
            const f3     dj = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
            const float  d  = dot( dj, dj );
            const float  t  = ( Ri * Ri - Rj * Rj + d ) / ( 2.f * d );
            const f3     c  = dj * t; // circle centre relative to atom i
            float        r2 = Ri * Ri - dot( c, c );
            if ( r2 < 0.004f * Ri * Ri )
                // nearly tangent SAS spheres: the radius is the root of a difference of nearly
                // equal numbers; taken in double precision from the float32 atoms
                r2 = torus_r2_d( ai, aj, b.rp );
            const float r  = sqrtf( fmaxf( r2, 0.f ) );
            const f3    ta = normalize( c );
            f3          cz = cross( ta, F3( 0.f, 0.f, 1.f ) );
            if ( dot( cz, cz ) < 1e-12f )
            {
                // the reference normalises a zero vector here (NaN); use the x axis instead
                cz = cross( ta, F3( 1.f, 0.f, 0.f ) );
                degenerate++;
            }
            const f3    ortho = normalize( cz );
            const f3    P     = c + ortho * r;
            const f3    X     = normalize( P ) * ai.w;
            const float lpi   = sqrtf( dot( P, P ) );
            const f3    Pj    = P - dj;
            const float lpj   = sqrtf( dot( Pj, Pj ) );
            const f3    C     = dj * ( lpi / ( lpj + lpi ) );
            const f3    XC    = X - C;
            const float dist  = sqrtf( dot( XC, XC ) );
            const f3    Cout  = C - c;
            if ( idx < b.capTori )
            {
                b.torPos[ idx ]  = make_float4( ai.x + c.x, ai.y + c.y, ai.z + c.z, r );
                b.torAxis[ idx ] = make_float4( ta.x, ta.y, ta.z, b.rp );
                b.torVs[ idx ]   = make_float4( Cout.x, Cout.y, Cout.z, dist );
            }
            else
                ovf |= kOverflowTori;
        }

        // A warp gathers the status-2 circles of kToriAtoms consecutive atoms into a shared
        // queue (atom, slot, output index) and evaluates them 32 at a time, one per lane (an
        // atom has a few tori among ~40 slots: a lane per slot left most lanes idle)
        constexpr uint32_t kToriAtoms = 8;
        __global__ void __launch_bounds__( 32 * kWarpsPerBlock ) k_tori( Build b )
        {
            pdl_begin();
            __shared__ uint4   queue[ kWarpsPerBlock ][ 64 ];
            __shared__ uint8_t stat[ kWarpsPerBlock ][ 64 * kToriAtoms ];
            const uint32_t     warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t     i0   = ( blockIdx.x * kWarpsPerBlock + warp ) * kToriAtoms;
            uint4 *          q    = queue[ warp ];
            uint32_t         nq = 0, ovf = 0, degenerate = 0;
            auto             drain = [ & ]( bool all ) {
                while ( nq >= 32 || ( all && nq > 0 ) )
                {
                    const uint32_t take = nq < 32 ? nq : 32;
                    if ( lane < take )
                    {
                        const uint4 e = q[ lane ];
                        torus_of( b, e.x, e.y, e.z, ovf, degenerate );
                    }
                    const uint32_t rest = nq - take; // at most 31
                    uint4          keep = make_uint4( 0u, 0u, 0u, 0u );
                    if ( lane < rest )
                        keep = q[ take + lane ];
                    __syncwarp();
                    if ( lane < rest )
                        q[ lane ] = keep;
                    __syncwarp();
                    nq = rest;
                }
            };
            // the atoms' counts, output offsets and first 64 statuses, all loads in flight together
            // (statuses past the count are read within the row's capacity and not used), the
            // statuses into shared memory
            uint32_t myNi = 0, myBase = 0;
            if ( lane < kToriAtoms && i0 + lane < b.n )
            {
                myNi   = b.nbrCount[ i0 + lane ];
                myBase = b.torOff[ i0 + lane ];
            }
            uint8_t * st = stat[ warp ];
#pragma unroll
            for ( uint32_t a = 0; a < kToriAtoms; a++ )
#pragma unroll
                for ( uint32_t h = 0; h < 2; h++ )
                    st[ 64 * a + 32 * h + lane ] =
                        i0 + a < b.n && lane + 32 * h < b.cap ? b.status[ (size_t)( i0 + a ) * b.cap + lane + 32 * h ] : (uint8_t)0;
            __syncwarp();
            for ( uint32_t a = 0; a < kToriAtoms; a++ )
            {
                const uint32_t i    = i0 + a;
                const uint32_t ni   = __shfl_sync( 0xffffffffu, myNi, a );
                uint32_t       base = __shfl_sync( 0xffffffffu, myBase, a );
                for ( uint32_t s0 = 0; s0 < ni; s0 += 32 )
                {
                    const uint32_t s     = s0 + lane;
                    const uint32_t code  = s0 < 64 ? st[ 64 * a + s ] : ( s < ni ? b.status[ (size_t)i * b.cap + s ] : 0u );
                    const bool     valid = s < ni && code == 2;
                    const uint32_t m     = __ballot_sync( 0xffffffffu, valid );
                    const uint32_t r     = __popc( m & lanemask_lt() );
                    if ( valid ) // nq <= 31 here: the queue holds up to 63 entries
                        q[ nq + r ] = make_uint4( i, s, base + r, 0u );
                    nq += __popc( m );
                    base += __popc( m );
                    __syncwarp();
                    drain( false );
                }
            }
            drain( true );
            for ( int o = 16; o > 0; o >>= 1 )
            {
                degenerate += __shfl_xor_sync( 0xffffffffu, degenerate, o );
                ovf |= __shfl_xor_sync( 0xffffffffu, ovf, o );
            }
            if ( lane == 0 && degenerate )
                atomicAdd( &b.counts->torusDegenerate, degenerate );
            if ( lane == 0 && ovf )
                atomicOr( &b.counts->overflow, ovf );
        }

        // ---- reference-layout analysis buffers --------------------------------
        // globalToTrimmedId (operations.inl:46-47): exclusive count of partial
        // slots over the whole N x cap slot array, plus one trailing total
        __global__ void k_reference_fill( Build b, uint32_t * g2t )
        {
            const uint64_t total = (uint64_t)b.n * b.cap;
            for ( uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q <= total; q += (uint64_t)gridDim.x * blockDim.x )
            {
                if ( q == total )
                {
                    if ( g2t )
                        g2t[ q ] = b.counts->C1;
                    continue;
                }
                const uint32_t i = (uint32_t)( q / b.cap ), s = (uint32_t)( q % b.cap );
                const uint32_t ni = b.nbrCount[ i ];
                if ( s >= ni )
                {
                    b.status[ q ] = 0;
                    if ( g2t )
                        g2t[ q ] = b.partOff[ i ] + b.partCnt[ i ];
                }
                else if ( g2t )
                    g2t[ q ] = b.slotTrim[ q ];
            }
        }

        std::atomic<uint64_t> g_launches { 0 };
        inline void counted( uint32_t k = 1 ) { g_launches.fetch_add( k, std::memory_order_relaxed ); }

        inline uint32_t blocks_for( uint64_t n, uint32_t threads )
        {
            return (uint32_t)( ( n + threads - 1 ) / threads );
        }
        inline uint32_t persistent_blocks( uint32_t threads )
        {
            // a few waves over 152 SMs for grid-stride kernels whose length is on the device
            return 152u * ( 2048u / threads );
        }
    } // namespace

    void launch_hash( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_hash, blocks_for( b.n, 256 ), 256, 0, s, b );
        counted();
    }
    void launch_fine_params( const Build & b, float cutoff, uint32_t, cudaStream_t s, int span )
    {
        pdl_launch( k_fine_params, blocks_for( b.nMol, 128 ), 128, 0, s, b, cutoff, span );
        counted();
    }
    void launch_zero2( uint32_t * a, uint32_t * c, uint32_t nHost, const uint32_t * nDevice, cudaStream_t s )
    {
        pdl_launch( k_zero2, min( persistent_blocks( 256 ), blocks_for( (uint64_t)nHost + 1, 256 ) ), 256, 0, s, a, c, nHost, nDevice );
        counted();
    }
    void launch_gather( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_gather, blocks_for( b.n, 256 ), 256, 0, s, b );
        counted();
    }
    void launch_cells( const Build & b, int kind, uint32_t nHost, const uint32_t * nDevice, void * scanScratch,
                       cudaStream_t s )
    {
        {
            // the cells of the grid just sized (one molecule), or every cell of a batch
            const uint32_t * cells = b.nMol > 1 ? nullptr
                                                : reinterpret_cast<const uint32_t *>( reinterpret_cast<const char *>( b.fine ) + offsetof( FineGrid, cells ) );
            launch_zero2( b.cellCount, b.cellCursor, b.capCells, cells, s );
        }
        if ( nHost == 0 )
            return;
        const uint32_t blocks = nDevice ? min( persistent_blocks( 256 ), blocks_for( nHost, 256 ) ) : blocks_for( nHost, 256 );
        pdl_launch( k_cell_count, blocks, 256, 0, s, b, kind, nHost, nDevice );
        if ( b.nMol > 1 )
            exclusive_scan( b.cellCount, b.cellStart, b.capCells, nullptr, nullptr, scanScratch, s ); // all molecules' cells
        else
        {
            const uint32_t * cells = reinterpret_cast<const uint32_t *>( reinterpret_cast<const char *>( b.fine ) + offsetof( FineGrid, cells ) );
            exclusive_scan( b.cellCount, b.cellStart, b.capCells, cells, nullptr, scanScratch, s );
        }
        pdl_launch( k_cell_scatter, blocks, 256, 0, s, b, kind, nHost, nDevice );
        counted( 2 );
    }
    void launch_batch_finish( const Build & b, cudaStream_t s )
    {
        if ( b.nMol <= 1 || !b.n )
            return;
        pdl_launch( k_mol_counts, blocks_for( b.nMol, 128 ), 128, 0, s, b );
        pdl_launch( k_mol_rebase, persistent_blocks( 256 ), 256, 0, s, b );
        counted( 2 );
    }
    void launch_neighbors( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        switch ( b.nbrWarps )
        {
        case 2: pdl_launch( k_neighbors<2>, blocks_for( b.n, 2 ), 64, 0, s, b ); break;
        case 4: pdl_launch( k_neighbors<4>, blocks_for( b.n, 4 ), 128, 0, s, b ); break;
        case 16: pdl_launch( k_neighbors<16>, blocks_for( b.n, 16 ), 512, 0, s, b ); break;
        default: pdl_launch( k_neighbors<8>, blocks_for( b.n, 8 ), 256, 0, s, b ); break;
        }
        counted();
    }
    void launch_visibility( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        switch ( b.visWarps )
        {
        case 2: pdl_launch( k_visibility<2>, blocks_for( b.n, 2 ), 64, visibility_smem( b.cap, 2 ), s, b ); break;
        case 4: pdl_launch( k_visibility<4>, blocks_for( b.n, 4 ), 128, visibility_smem( b.cap, 4 ), s, b ); break;
        default: pdl_launch( k_visibility<1>, blocks_for( b.n, 1 ), 32, visibility_smem( b.cap, 1 ), s, b ); break;
        }
        counted();
    }
    void launch_visibility_resolve( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_visibility_band, min( persistent_blocks( 128 ), blocks_for( b.capVisBand, 128 ) + 1 ), 128, 0, s, b );
        pdl_launch( k_visibility_final, blocks_for( b.n, kWarpsPerBlock * 4 ), 32 * kWarpsPerBlock, 0, s, b );
        counted( 2 );
    }
    void launch_emit( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_emit, blocks_for( b.n, kWarpsPerBlock * ( 32 / kEmitGroup ) ), 32 * kWarpsPerBlock, 0, s, b );
        counted();
    }
    void launch_probes( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        const size_t   smem  = probe_smem_per_warp( b.cap ) * (size_t)b.probeWarps;
        const uint32_t queue = b.probeQueueBlocks; // resident blocks of the persistent variant (0: one warp per atom)
        switch ( b.probeWarps * 2 + ( queue ? 1 : 0 ) )
        {
        case 3: pdl_launch( k_probes<1, true>, min( queue, blocks_for( b.n, 1 ) ), 32, smem, s, b ); break;
        case 4: pdl_launch( k_probes<2, false>, blocks_for( b.n, 2 ), 64, smem, s, b ); break;
        case 5: pdl_launch( k_probes<2, true>, min( queue, blocks_for( b.n, 2 ) ), 64, smem, s, b ); break;
        case 8: pdl_launch( k_probes<4, false>, blocks_for( b.n, 4 ), 128, smem, s, b ); break;
        case 9: pdl_launch( k_probes<4, true>, min( queue, blocks_for( b.n, 4 ) ), 128, smem, s, b ); break;
        default: pdl_launch( k_probes<1, false>, blocks_for( b.n, 1 ), 32, smem, s, b ); break;
        }
        counted();
    }
    void launch_probe_jobs( const Build & b, cudaStream_t s )
    {
        pdl_launch( k_probe_jobs, min( persistent_blocks( 128 ), blocks_for( b.capProbes, 128 ) + 1 ), 128, 0, s, b );
        counted();
    }
    void launch_place( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_place, blocks_for( b.n, kWarpsPerBlock * ( 32 / kPlaceGroup ) ), 32 * kWarpsPerBlock, 0, s, b );
        counted();
    }
    void launch_lists( const Build & b, cudaStream_t s )
    {
        pdl_launch( k_lists, min( persistent_blocks( 256 ), blocks_for( b.capProbes, 256 ) + 1 ), 256, 0, s, b );
        counted();
    }
    void launch_segment_counts( const Build & b, cudaStream_t s )
    {
        pdl_launch( k_segment_counts, min( persistent_blocks( 256 ), blocks_for( b.capC1, 256 ) + 1 ), 256, 0, s, b );
        counted();
    }
    void launch_segments( const Build & b, cudaStream_t s )
    {
        pdl_launch( k_segments, min( persistent_blocks( 128 ), blocks_for( b.capC1, 128 ) + 1 ), 128, 0, s, b );
        counted();
    }
    void launch_probe_neighbors( const Build & b, cudaStream_t s )
    {
        pdl_launch( k_probe_neighbors, min( persistent_blocks( 256 ), blocks_for( b.capProbes, kWarpsPerBlock ) + 1 ), 32 * kWarpsPerBlock, 0, s, b );
        counted();
        if ( b.mode == 1 )
        {
            pdl_launch( k_probe_w, min( persistent_blocks( 256 ), blocks_for( b.capProbes, 256 ) + 1 ), 256, 0, s, b );
            counted();
        }
    }
    void launch_tori( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_tori_count, blocks_for( b.n, kWarpsPerBlock * 4 ), 32 * kWarpsPerBlock, 0, s, b );
        counted();
    }
    void launch_tori_emit( const Build & b, cudaStream_t s )
    {
        if ( !b.n )
            return;
        pdl_launch( k_tori, blocks_for( b.n, kWarpsPerBlock * kToriAtoms ), 32 * kWarpsPerBlock, 0, s, b );
        counted();
    }
    uint64_t launch_count() { return g_launches.load(); }
    void     count_launches( uint32_t k ) { counted( k ); }

    cudaError_t configure_kernels( const Build & b )
    {
        const size_t vs = vis_smem_per_warp( b.cap ), ps = probe_smem_per_warp( b.cap );
        cudaError_t  e  = cudaSuccess;
        auto         set = [ & ]( const void * f, size_t bytes ) {
            if ( e == cudaSuccess )
                e = cudaFuncSetAttribute( f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes );
        };
        set( (const void *)k_visibility<1>, vs );
        set( (const void *)k_visibility<2>, 2 * vs );
        set( (const void *)k_visibility<4>, 4 * vs );
        set( (const void *)k_probes<1, false>, ps );
        set( (const void *)k_probes<1, true>, ps );
        set( (const void *)k_probes<2, false>, 2 * ps );
        set( (const void *)k_probes<2, true>, 2 * ps );
        set( (const void *)k_probes<4, false>, 4 * ps );
        set( (const void *)k_probes<4, true>, 4 * ps );
        return e;
    }

    uint32_t probe_queue_blocks( const Build & b, int warps )
    {
        // blocks of the persistent probe kernel that fit on the GPU at once
        int          dev = 0, sms = 0, per = 0;
        const void * f   = warps == 4 ? (const void *)k_probes<4, true>
                                      : warps == 2 ? (const void *)k_probes<2, true> : (const void *)k_probes<1, true>;
        cudaGetDevice( &dev );
        cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
        if ( cudaOccupancyMaxActiveBlocksPerMultiprocessor( &per, f, 32 * warps, probe_smem_per_warp( b.cap ) * warps )
             != cudaSuccess )
            per = 1;
        return (uint32_t)std::max( 1, sms * std::max( per, 1 ) );
    }
    void launch_reference_fill( const Build & b, uint32_t * globalToTrimmed, cudaStream_t s )
    {
        const uint64_t total = (uint64_t)b.n * b.cap + 1;
        k_reference_fill<<<min( persistent_blocks( 256 ), blocks_for( total, 256 ) ), 256, 0, s>>>( b, globalToTrimmed );
        counted();
    }
} // namespace sesgb

// ---- signed distance to the SES at query points -----------------------------
//
// Definition (project-written; the reference has no SDF). E is the set of
// probe-centre positions that overlap no atom: outside every SAS sphere
// (radius R_i = r_i + rp). With T = rp + kSdfBand:
//   x outside the SAS:  sdf = min_i (|x - c_i| - r_i), clamped to kSdfBand;
//   x inside the SAS:   sdf = rp - min(T, dist(x, dE)).
// dE is the SAS surface: the accessible parts of the SAS spheres, the arcs of
// the visible circles and the probe positions. The nearest point of dE is the
// radial projection of x on a sphere, the nearest point of a circle, or a
// probe, whichever is nearest among those that lie on dE (not strictly inside
// another SAS sphere); only atoms with |x - c_i| <= R_i + T can carry one.
// The gradient with respect to the atoms follows the active primitive: the
// sphere or atom distance directly, a circle point and a probe by the
// Lagrange / implicit-function rule for points constrained to |p - c_m| = R_m.
namespace sesgb
{
    namespace
    {
        constexpr int   kSdfWarps = 4;   // warps per block (one query per warp)
        constexpr int   kSdfList   = 256; // atoms within reach held per query
        constexpr int   kSdfStaged = 128; // neighbour slots staged in shared memory

        enum SdfKind : int
        {
            kSdfClampInside = 0, // deeper than T below dE
            kSdfAtom        = 1, // outside the SAS: nearest vdW sphere
            kSdfClampOutside = 2,
            kSdfSphere      = 3, // radial projection on an accessible SAS sphere patch
            kSdfCircle      = 4, // nearest point of an accessible arc
            kSdfProbe       = 5, // probe position (vertex of dE)
        };

        struct SdfHit
        {
            int    kind;
            int    a, b, c; // sorted atom ids
            float3 q;       // point of dE (or of the vdW sphere)
            float  value;
        };

        struct SdfSmem
        {
            unsigned long long key[ kSdfList ];   // (delta bits << 32) | atom
            float4             nb[ kSdfStaged ];   // neighbourhood of the atom being examined: (c_k, R_k)
            uint16_t           near[ kNbrBuf ];    // its slots whose SAS sphere comes within the current best of x
            uint8_t            vis[ kNbrBuf ];     // status of its circles
        };

        // neighbour slot s of atom i as (c_k, R_k): staged slots from shared memory
        __device__ __forceinline__ float4 sdf_nb( const Build & b, const SdfSmem & sm, size_t row, uint32_t s )
        {
            if ( s < (uint32_t)kSdfStaged )
                return sm.nb[ s ];
            const float4 c = b.atoms[ b.nbr[ row + s ] ];
            return make_float4( c.x, c.y, c.z, c.w + b.rp );
        }

        __device__ __forceinline__ void warp_min_hit( float & best, int & owner )
        {
            // smallest candidate distance, lowest lane on ties
            for ( int o = 16; o > 0; o >>= 1 )
            {
                const float ob = __shfl_xor_sync( 0xffffffffu, best, o );
                const int   oo = __shfl_xor_sync( 0xffffffffu, owner, o );
                if ( ob < best || ( ob == best && oo < owner ) )
                {
                    best  = ob;
                    owner = oo;
                }
            }
        }

        // Float32 error bound of |q - c_k|^2 - R_k^2 for a point q computed in absolute float32
        // coordinates: a few ulps of the coordinates (at most qQ / 4, the query's largest coordinate
        // plus its reach) on every coordinate, times 2 |q - c_k| (taken as R_k: the bound matters only
        // where |q - c_k| is close to R_k), plus the rounding of the squares. Inside it the test is
        // taken again in double precision.
        __device__ __forceinline__ float hidden_band( float qQ, float d2, float Rk )
        {
            return 3.8147e-6f * ( d2 + Rk * ( Rk + qQ ) + 1.f );
        }

        // point q (double) strictly inside the SAS sphere of atom k, in double precision
        __device__ __noinline__ bool point_inside_d( const Build & b, d3 q, uint32_t k )
        {
            const float4 ck = b.atoms[ k ];
            const double Rk = (double)ck.w + (double)b.rp;
            const double dx = q.x - (double)ck.x, dy = q.y - (double)ck.y, dz = q.z - (double)ck.z;
            return dx * dx + dy * dy + dz * dz < Rk * Rk;
        }

        // The radial projection of x on the SAS sphere of i, in double precision, strictly inside the
        // SAS sphere of one of this lane's near neighbours (lanes take every 32nd)
        __device__ __noinline__ bool sphere_point_hidden_d( const Build & b, const SdfSmem & sm, size_t row, uint32_t nn,
                                                            uint32_t i, float3 x, uint32_t lane )
        {
            const float4 ci = b.atoms[ i ];
            const d3     wd = D3( (double)x.x - (double)ci.x, (double)x.y - (double)ci.y, (double)x.z - (double)ci.z );
            const double Rd = (double)ci.w + (double)b.rp;
            const double sc = Rd / sqrt( wd.x * wd.x + wd.y * wd.y + wd.z * wd.z );
            const d3     qd = D3( (double)ci.x + wd.x * sc, (double)ci.y + wd.y * sc, (double)ci.z + wd.z * sc );
            bool         hd = false;
            for ( uint32_t e = lane; e < nn; e += 32 )
                hd = hd || point_inside_d( b, qd, b.nbr[ row + sm.near[ e ] ] );
            return hd;
        }

        // The nearest point of circle (i, neighbour slot s) to x, in double precision, strictly inside
        // the SAS sphere of a near neighbour of i other than that of slot s
        __device__ __noinline__ bool circle_point_hidden_d( const Build & b, const SdfSmem & sm, size_t row, uint32_t nn,
                                                            uint32_t i, uint32_t s, float3 x )
        {
            const float4 ai = b.atoms[ i ], aj = b.atoms[ b.nbr[ row + s ] ];
            const double Ri = (double)ai.w + (double)b.rp, Rj = (double)aj.w + (double)b.rp;
            const d3     d  = D3( (double)aj.x - (double)ai.x, (double)aj.y - (double)ai.y, (double)aj.z - (double)ai.z );
            const double dd = d.x * d.x + d.y * d.y + d.z * d.z;
            const double tt = ( Ri * Ri - Rj * Rj + dd ) / ( 2.0 * dd );
            const double r2 = Ri * Ri - tt * tt * dd;
            if ( !( r2 > 0.0 ) )
                return false;
            const double r   = sqrt( r2 );
            const double inv = 1.0 / sqrt( dd );
            const d3     n   = D3( d.x * inv, d.y * inv, d.z * inv );
            const d3     c   = D3( (double)ai.x + d.x * tt, (double)ai.y + d.y * tt, (double)ai.z + d.z * tt );
            const d3     w   = D3( (double)x.x - c.x, (double)x.y - c.y, (double)x.z - c.z );
            const double h   = w.x * n.x + w.y * n.y + w.z * n.z;
            const d3     v   = D3( w.x - h * n.x, w.y - h * n.y, w.z - h * n.z );
            const double rho = sqrt( v.x * v.x + v.y * v.y + v.z * v.z );
            if ( !( rho > 0.0 ) )
                return false;
            const d3 q = D3( c.x + v.x * ( r / rho ), c.y + v.y * ( r / rho ), c.z + v.z * ( r / rho ) );
            for ( uint32_t e = 0; e < nn; e++ )
            {
                const uint32_t k = sm.near[ e ];
                if ( k != s && point_inside_d( b, q, b.nbr[ row + k ] ) )
                    return true;
            }
            return false;
        }

        // one query, the whole warp; the hit is valid in every lane. A point of dE within the float32
        // error of another SAS sphere is decided in double precision with kExact; without it the
        // query is only marked (exact set, in every lane), for a second pass that runs it with kExact.
        template<bool kExact>
        __device__ SdfHit sdf_query( const Build & b, float3 x, SdfSmem & sm, float band, uint32_t & overflow, bool & exact )
        {
            const uint32_t lane      = lane_id();
            bool           exactLane = false;
            exact                    = false;
            // 4 x (largest coordinate of any point of dE this query examines)
            const float qQ = 4.f * ( fmaxf( fabsf( x.x ), fmaxf( fabsf( x.y ), fabsf( x.z ) ) ) + 12.f );
            const float    T    = b.rp + band;
            const FineGrid g    = b.fine[ 0 ];
            Rows           rows;
            stencil_rows( g, b.cellStart, fine_cell( g, x.x, x.y, x.z ), rows );
            // atoms within reach; minima of |x - c| - R (SAS) and |x - c| - r (vdW)
            uint32_t nl = 0;
            float    smin = 3.4e38f, vmin = 3.4e38f;
            int      vatom = 0x7fffffff;
            for ( uint32_t base = 0; base < rows.total; base += 32 )
            {
                const uint32_t f    = base + lane;
                bool           keep = false;
                uint32_t       i    = 0;
                float          dl   = 0.f;
                if ( f < rows.total )
                {
                    const uint32_t idx = row_item( rows, f );
                    i                  = b.cellItems[ idx ];
                    const float4 c     = b.cellPos[ idx ];
                    const float  ra    = fabsf( c.w );
                    const float  L     = sqrtf( ( x.x - c.x ) * ( x.x - c.x ) + ( x.y - c.y ) * ( x.y - c.y ) + ( x.z - c.z ) * ( x.z - c.z ) );
                    const float  R     = ra + b.rp;
                    if ( L <= R + T )
                    {
                        smin = fminf( smin, L - R );
                        const float v = L - ra;
                        if ( v < vmin || ( v == vmin && (int)i < vatom ) )
                        {
                            vmin  = v;
                            vatom = (int)i;
                        }
                        dl = fabsf( L - R );
                        // fully buried atoms carry no point of dE: only the bounds above use them
                        keep = !signbit( c.w );
                    }
                }
                const uint32_t mk = __ballot_sync( 0xffffffffu, keep );
                const uint32_t at = nl + __popc( mk & lanemask_lt() );
                if ( keep && at < (uint32_t)kSdfList )
                    sm.key[ at ] = ( (unsigned long long)__float_as_uint( dl ) << 32 ) | i;
                nl += __popc( mk );
            }
            if ( nl > (uint32_t)kSdfList )
            {
                overflow = 1;
                nl       = kSdfList;
            }
            for ( int o = 16; o > 0; o >>= 1 )
            {
                smin          = fminf( smin, __shfl_xor_sync( 0xffffffffu, smin, o ) );
                const float v = __shfl_xor_sync( 0xffffffffu, vmin, o );
                const int   a = __shfl_xor_sync( 0xffffffffu, vatom, o );
                if ( v < vmin || ( v == vmin && a < vatom ) )
                {
                    vmin  = v;
                    vatom = a;
                }
            }
            SdfHit hit;
            hit.a = hit.b = hit.c = -1;
            hit.q                 = x;
            if ( !( smin < 0.f ) )
            {
                // outside the SAS (or nothing within reach)
                if ( vatom != 0x7fffffff && vmin <= band )
                {
                    hit.kind  = kSdfAtom;
                    hit.a     = vatom;
                    hit.value = vmin;
                }
                else
                {
                    hit.kind  = kSdfClampOutside;
                    hit.value = band;
                }
                return hit;
            }
            __syncwarp();
            float best  = T;
            hit.kind    = kSdfClampInside;
            // x lies in a SAS sphere with R - |x - c| = -smin: every point of dE is at least that far
            const float floorD = -smin;
            if ( !( floorD < T ) )
            {
                hit.value = b.rp - T;
                return hit;
            }
            // probes (vertices of dE, never hidden) first: an early upper bound for the search
            {
                float  cand = 3.4e38f;
                int    pa = -1, pb = -1, pc = -1;
                float3 pq = x;
                // lane per atom: its probe chunk
                for ( uint32_t e0 = lane; e0 < nl; e0 += 32 )
                {
                    const uint32_t i     = (uint32_t)sm.key[ e0 ];
                    const uint32_t chunk = b.chunkStart[ i ], len = b.chunkLen[ i ];
                    for ( uint32_t e = 0; e < len; e++ )
                    {
                        const int4 cid = b.stageCid[ chunk + e ];
                        if ( cid.w == 0 )
                            continue;
                        const float4 p    = b.stagePos[ chunk + e ];
                        const float  dist = sqrtf( ( x.x - p.x ) * ( x.x - p.x ) + ( x.y - p.y ) * ( x.y - p.y ) + ( x.z - p.z ) * ( x.z - p.z ) );
                        if ( dist < cand )
                        {
                            const int4 ids = b.stageIds[ chunk + e ];
                            cand           = dist;
                            pa             = ids.x;
                            pb             = ids.y;
                            pc             = ids.z;
                            pq             = make_float3( p.x, p.y, p.z );
                        }
                    }
                }
                float wbest = cand;
                int   owner = (int)lane;
                warp_min_hit( wbest, owner );
                if ( wbest < best )
                {
                    best     = wbest;
                    hit.kind = kSdfProbe;
                    hit.a    = __shfl_sync( 0xffffffffu, pa, owner );
                    hit.b    = __shfl_sync( 0xffffffffu, pb, owner );
                    hit.c    = __shfl_sync( 0xffffffffu, pc, owner );
                    hit.q.x  = __shfl_sync( 0xffffffffu, pq.x, owner );
                    hit.q.y  = __shfl_sync( 0xffffffffu, pq.y, owner );
                    hit.q.z  = __shfl_sync( 0xffffffffu, pq.z, owner );
                }
            }
            // atoms in ascending |x - c| - R order (the lower bound of all their candidates),
            // each picked by a warp minimum over the ones left, until the bound reaches best
            for ( uint32_t t = 0; t < nl; t++ )
            {
                unsigned long long key = ~0ull;
                uint32_t           at  = 0;
                for ( uint32_t e = lane; e < nl; e += 32 )
                    if ( sm.key[ e ] < key )
                    {
                        key = sm.key[ e ];
                        at  = e;
                    }
                for ( int o = 16; o > 0; o >>= 1 )
                {
                    const unsigned long long ok = __shfl_xor_sync( 0xffffffffu, key, o );
                    const uint32_t           oa = __shfl_xor_sync( 0xffffffffu, at, o );
                    if ( ok < key )
                    {
                        key = ok;
                        at  = oa;
                    }
                }
                const float dl = __uint_as_float( (uint32_t)( key >> 32 ) );
                if ( !( dl < best ) || !( floorD < best ) )
                    break; // every candidate of this and the remaining atoms is at least dl away
                __syncwarp();
                if ( lane == 0 )
                    sm.key[ at ] = ~0ull; // taken
                const uint32_t i   = (uint32_t)key;
                const float4   ci  = b.atoms[ i ];
                const float    Ri  = ci.w + b.rp;
                const uint32_t ni  = b.nbrCount[ i ];
                const size_t   row = (size_t)i * b.cap;
                // stage N(i); a point q with |x - q| < best can only lie inside the SAS
                // sphere of a neighbour k with |x - c_k| - R_k < best: those are the "near" ones
                uint32_t nn = 0;
                for ( uint32_t s0 = 0; s0 < ni; s0 += 32 )
                {
                    const uint32_t s    = s0 + lane;
                    bool           near = false;
                    if ( s < ni )
                    {
                        sm.vis[ s ]     = b.status[ row + s ];
                        const float4 ck = b.atoms[ b.nbr[ row + s ] ];
                        const float  Rk = ck.w + b.rp;
                        if ( s < (uint32_t)kSdfStaged )
                            sm.nb[ s ] = make_float4( ck.x, ck.y, ck.z, Rk );
                        const float Lk  = sqrtf( ( x.x - ck.x ) * ( x.x - ck.x ) + ( x.y - ck.y ) * ( x.y - ck.y ) + ( x.z - ck.z ) * ( x.z - ck.z ) );
                        near            = Lk - Rk < best;
                    }
                    const uint32_t mk = __ballot_sync( 0xffffffffu, near );
                    if ( near )
                        sm.near[ nn + __popc( mk & lanemask_lt() ) ] = (uint16_t)s;
                    nn += __popc( mk );
                }
                __syncwarp();
                // candidates of this atom, one per lane at most, reduced at the end
                float  cand = 3.4e38f;
                int    ck = 0, cb = -1, cc = -1;
                float3 cq = x;
                // radial projection on sphere i
                {
                    const float3 w = make_float3( x.x - ci.x, x.y - ci.y, x.z - ci.z );
                    const float  L = sqrtf( w.x * w.x + w.y * w.y + w.z * w.z );
                    if ( L > 0.f )
                    {
                        const float3 q = make_float3( ci.x + w.x * ( Ri / L ), ci.y + w.y * ( Ri / L ), ci.z + w.z * ( Ri / L ) );
                        bool         hidden = false, unsure = false;
                        for ( uint32_t e = lane; e < nn; e += 32 )
                        {
                            const float4 nk = sdf_nb( b, sm, row, sm.near[ e ] );
                            const float  dx = q.x - nk.x, dy = q.y - nk.y, dz = q.z - nk.z;
                            const float  d2 = dx * dx + dy * dy + dz * dz;
                            const float  m  = d2 - nk.w * nk.w;
                            const float  eb = hidden_band( qQ, d2, nk.w );
                            hidden          = hidden || m < -eb;
                            unsure          = unsure || !( fabsf( m ) > eb );
                        }
                        bool hid = __any_sync( 0xffffffffu, hidden );
                        if ( !hid && __any_sync( 0xffffffffu, unsure ) )
                        {
                            // a neighbour's sphere passes within the float32 error of the point:
                            // the point and the test in double precision
                            if ( kExact )
                                hid = __any_sync( 0xffffffffu, sphere_point_hidden_d( b, sm, row, nn, i, x, lane ) );
                            else
                                exactLane = true;
                        }
                        if ( !hid && lane == 0 )
                        {
                            cand = dl;
                            ck   = kSdfSphere;
                            cq   = q;
                        }
                    }
                }
                // nearest points of the visible circles of i
                for ( uint32_t s0 = 0; s0 < ni; s0 += 32 )
                {
                    const uint32_t s = s0 + lane;
                    if ( s >= ni || sm.vis[ s ] == 0 )
                        continue;
                    const float4 nj = sdf_nb( b, sm, row, s );
                    {
                        // every point of circle (i, j) is on sphere j too: |x - c_j| - R_j bounds it
                        const float Lj = sqrtf( ( x.x - nj.x ) * ( x.x - nj.x ) + ( x.y - nj.y ) * ( x.y - nj.y ) + ( x.z - nj.z ) * ( x.z - nj.z ) );
                        if ( !( fabsf( Lj - nj.w ) < best ) )
                            continue;
                    }
                    const float3 d  = make_float3( nj.x - ci.x, nj.y - ci.y, nj.z - ci.z );
                    const float  dd = d.x * d.x + d.y * d.y + d.z * d.z;
                    const float  tt = ( Ri * Ri - nj.w * nj.w + dd ) / ( 2.f * dd );
                    const float  r2 = Ri * Ri - tt * tt * dd;
                    if ( !( r2 > 0.f ) )
                        continue;
                    const float  r   = sqrtf( r2 );
                    const float  inv = rsqrtf( dd );
                    const float3 n   = make_float3( d.x * inv, d.y * inv, d.z * inv );
                    const float3 c   = make_float3( ci.x + d.x * tt, ci.y + d.y * tt, ci.z + d.z * tt );
                    const float3 w   = make_float3( x.x - c.x, x.y - c.y, x.z - c.z );
                    const float  h   = w.x * n.x + w.y * n.y + w.z * n.z;
                    const float3 v   = make_float3( w.x - h * n.x, w.y - h * n.y, w.z - h * n.z );
                    const float  rho = sqrtf( v.x * v.x + v.y * v.y + v.z * v.z );
                    float        dist;
                    float3       q = c;
                    if ( rho > 1e-6f )
                    {
                        q    = make_float3( c.x + v.x * ( r / rho ), c.y + v.y * ( r / rho ), c.z + v.z * ( r / rho ) );
                        dist = sqrtf( h * h + ( rho - r ) * ( rho - r ) );
                        if ( !( dist < cand ) || !( dist < best ) )
                            continue;
                        bool hidden = false, unsure = false;
                        for ( uint32_t e = 0; e < nn && !hidden; e++ )
                        {
                            const uint32_t k = sm.near[ e ];
                            if ( k == s )
                                continue;
                            const float4 nk = sdf_nb( b, sm, row, k );
                            const float  dx = q.x - nk.x, dy = q.y - nk.y, dz = q.z - nk.z;
                            const float  d2 = dx * dx + dy * dy + dz * dz;
                            const float  m  = d2 - nk.w * nk.w;
                            const float  eb = hidden_band( qQ, d2, nk.w );
                            hidden          = m < -eb;
                            unsure          = unsure || !( fabsf( m ) > eb );
                        }
                        if ( !hidden && unsure )
                        {
                            if ( kExact )
                                hidden = circle_point_hidden_d( b, sm, row, nn, i, s, x );
                            else
                                exactLane = true;
                        }
                        if ( hidden )
                            continue;
                    }
                    else
                    {
                        // x on the axis: every point of the circle is as near; a visible
                        // circle has an accessible arc
                        dist = sqrtf( h * h + r2 );
                        if ( !( dist < cand ) || !( dist < best ) )
                            continue;
                    }
                    cand = dist;
                    ck   = kSdfCircle;
                    cb   = (int)b.nbr[ row + s ];
                    cq   = q;
                }
                float wbest = cand;
                int   owner = (int)lane;
                warp_min_hit( wbest, owner );
                if ( wbest < best )
                {
                    best     = wbest;
                    hit.kind = __shfl_sync( 0xffffffffu, ck, owner );
                    hit.a    = (int)i;
                    hit.b    = __shfl_sync( 0xffffffffu, cb, owner );
                    hit.c    = __shfl_sync( 0xffffffffu, cc, owner );
                    hit.q.x  = __shfl_sync( 0xffffffffu, cq.x, owner );
                    hit.q.y  = __shfl_sync( 0xffffffffu, cq.y, owner );
                    hit.q.z  = __shfl_sync( 0xffffffffu, cq.z, owner );
                }
                __syncwarp();
            }
            hit.value = b.rp - best;
            exact     = __any_sync( 0xffffffffu, exactLane );
            return hit;
        }

        __device__ __forceinline__ void add_grad( float * g, uint32_t atom, float gx, float gy, float gz, float gr )
        {
            atomicAdd( g + 4 * atom + 0, gx );
            atomicAdd( g + 4 * atom + 1, gy );
            atomicAdd( g + 4 * atom + 2, gz );
            atomicAdd( g + 4 * atom + 3, gr );
        }

        // d sdf / d (c, r) of the active primitive, scaled by gs, into g (sorted order)
        __device__ __noinline__ void sdf_gradient( const Build & b, const SdfHit & h, float3 x, float gs, float * g )
        {
            if ( h.kind == kSdfAtom || h.kind == kSdfSphere )
            {
                // sdf = |x - c_a| - r_a (outside the SAS, or x inside sphere a); the
                // opposite sign when x lies outside sphere a but inside another
                const float4 c = b.atoms[ h.a ];
                const float3 w = make_float3( x.x - c.x, x.y - c.y, x.z - c.z );
                const float  L = sqrtf( w.x * w.x + w.y * w.y + w.z * w.z );
                if ( !( L > 0.f ) )
                    return;
                float sgn = -1.f;
                if ( h.kind == kSdfSphere && L > c.w + b.rp )
                    sgn = 1.f;
                add_grad( g, (uint32_t)h.a, gs * sgn * w.x / L, gs * sgn * w.y / L, gs * sgn * w.z / L, gs * sgn );
                return;
            }
            if ( h.kind != kSdfCircle && h.kind != kSdfProbe )
                return;
            // The multipliers of the constraints |p - c_k|^2 = R_k^2 that hold the point p: a 2x2
            // (circle) or 3x3 (probe) system that is nearly singular when the constraint normals
            // are nearly parallel (two circle centres nearly aligned with p, a probe near the plane
            // of its three centres), where float32 would show in the gradient. Solved in double
            // precision from the float32 values (their differences are exact in double); one lane
            // per query, so the FP64 pipe's rate does not matter.
            const float3 pf = h.q;
            const d3     p  = D3( (double)pf.x, (double)pf.y, (double)pf.z );
            const d3     dv = D3( (double)x.x - p.x, (double)x.y - p.y, (double)x.z - p.z );
            const double D  = sqrt( dv.x * dv.x + dv.y * dv.y + dv.z * dv.z );
            if ( !( D > 0.0 ) )
                return;
            const d3  u = D3( dv.x / D, dv.y / D, dv.z / D );
            const int m = h.kind == kSdfCircle ? 2 : 3;
            const int ids[ 3 ] = { h.a, h.b, h.c };
            d3        a[ 3 ];
            double    R[ 3 ];
            for ( int k = 0; k < m; k++ )
            {
                const float4 c = b.atoms[ ids[ k ] ];
                a[ k ]         = D3( 2.0 * ( p.x - (double)c.x ), 2.0 * ( p.y - (double)c.y ), 2.0 * ( p.z - (double)c.z ) );
                R[ k ]         = (double)c.w + (double)b.rp;
            }
            // multipliers w: sum_k w_k a_k = u (least squares for the circle, exact for the probe)
            double w[ 3 ] = { 0.0, 0.0, 0.0 };
            if ( m == 2 )
            {
                const double g00 = a[ 0 ].x * a[ 0 ].x + a[ 0 ].y * a[ 0 ].y + a[ 0 ].z * a[ 0 ].z;
                const double g01 = a[ 0 ].x * a[ 1 ].x + a[ 0 ].y * a[ 1 ].y + a[ 0 ].z * a[ 1 ].z;
                const double g11 = a[ 1 ].x * a[ 1 ].x + a[ 1 ].y * a[ 1 ].y + a[ 1 ].z * a[ 1 ].z;
                const double r0  = a[ 0 ].x * u.x + a[ 0 ].y * u.y + a[ 0 ].z * u.z;
                const double r1  = a[ 1 ].x * u.x + a[ 1 ].y * u.y + a[ 1 ].z * u.z;
                const double det = g00 * g11 - g01 * g01;
                if ( !( fabs( det ) > 0.0 ) )
                    return;
                w[ 0 ] = ( r0 * g11 - r1 * g01 ) / det;
                w[ 1 ] = ( r1 * g00 - r0 * g01 ) / det;
            }
            else
            {
                // columns a_0, a_1, a_2: Cramer's rule
                const d3     c12 = dcross( a[ 1 ], a[ 2 ] );
                const double det = ddot( a[ 0 ], c12 );
                if ( !( fabs( det ) > 0.0 ) )
                    return;
                w[ 0 ] = ddot( u, c12 ) / det;                    // det[u, a1, a2]
                w[ 1 ] = ddot( a[ 0 ], dcross( u, a[ 2 ] ) ) / det; // det[a0, u, a2]
                w[ 2 ] = ddot( dcross( a[ 0 ], a[ 1 ] ), u ) / det; // det[a0, a1, u]
            }
            // sdf = rp - D: d sdf / d c_k = w_k a_k, d sdf / d r_k = 2 w_k R_k
            for ( int k = 0; k < m; k++ )
                add_grad( g, (uint32_t)ids[ k ], (float)( gs * w[ k ] * a[ k ].x ), (float)( gs * w[ k ] * a[ k ].y ),
                          (float)( gs * w[ k ] * a[ k ].z ), (float)( gs * 2.0 * w[ k ] * R[ k ] ) );
        }

        // grid cell of each query (sort key) and its index
        __global__ void k_sdf_keys( Build b, const float * queries, uint32_t m, uint32_t * keys, uint32_t * order )
        {
            const FineGrid g = b.fine[ 0 ];
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x )
            {
                keys[ q ]  = fine_key( g, fine_cell( g, queries[ 3 * (size_t)q ], queries[ 3 * (size_t)q + 1 ], queries[ 3 * (size_t)q + 2 ] ) );
                order[ q ] = q;
            }
        }

        // First pass over the queries (in grid-cell order: neighbouring warps read the same atoms);
        // a query that needs a double-precision decision is listed for k_sdf_exact instead
        template<bool kBackward>
        __global__ void __launch_bounds__( 32 * kSdfWarps, 8 ) k_sdf( Build b, const float * queries, uint32_t m, float band,
                                                                   float * sdf, const float * gradSdf, float * gradSorted,
                                                                   int * kind, const uint32_t * order, uint32_t * exactList,
                                                                   uint32_t * exactCount )
        {
            __shared__ SdfSmem smem[ kSdfWarps ];
            const uint32_t     warp = threadIdx.x >> 5, lane = lane_id();
            uint32_t           overflow = 0;
            for ( uint32_t qs = blockIdx.x * kSdfWarps + warp; qs < m; qs += gridDim.x * kSdfWarps )
            {
                const uint32_t qi = order[ qs ];
                const float3 x = make_float3( queries[ 3 * (size_t)qi ], queries[ 3 * (size_t)qi + 1 ], queries[ 3 * (size_t)qi + 2 ] );
                bool         exact;
                const SdfHit h = sdf_query<false>( b, x, smem[ warp ], band, overflow, exact );
                if ( lane == 0 )
                {
                    if ( exact )
                        exactList[ atomicAdd( exactCount, 1u ) ] = qi;
                    else if ( kBackward )
                        sdf_gradient( b, h, x, gradSdf[ qi ], gradSorted );
                    else
                    {
                        sdf[ qi ] = h.value;
                        if ( kind )
                            kind[ qi ] = h.kind;
                    }
                }
            }
            if ( lane == 0 && overflow )
                atomicOr( &b.counts->overflow, (uint32_t)kOverflowSdfList );
        }

        // Second pass: the listed queries, with every decision within the float32 band taken in
        // double precision (few queries: a point of dE next to another SAS sphere's surface)
        template<bool kBackward>
        __global__ void __launch_bounds__( 32 * kSdfWarps ) k_sdf_exact( Build b, const float * queries, float band, float * sdf,
                                                                      const float * gradSdf, float * gradSorted, int * kind,
                                                                      const uint32_t * exactList, const uint32_t * exactCount )
        {
            __shared__ SdfSmem smem[ kSdfWarps ];
            const uint32_t     warp = threadIdx.x >> 5, lane = lane_id();
            const uint32_t     count = *exactCount;
            uint32_t           overflow = 0;
            for ( uint32_t e = blockIdx.x * kSdfWarps + warp; e < count; e += gridDim.x * kSdfWarps )
            {
                const uint32_t qi = exactList[ e ];
                const float3 x = make_float3( queries[ 3 * (size_t)qi ], queries[ 3 * (size_t)qi + 1 ], queries[ 3 * (size_t)qi + 2 ] );
                bool         exact;
                const SdfHit h = sdf_query<true>( b, x, smem[ warp ], band, overflow, exact );
                if ( lane == 0 )
                {
                    if ( kBackward )
                        sdf_gradient( b, h, x, gradSdf[ qi ], gradSorted );
                    else
                    {
                        sdf[ qi ] = h.value;
                        if ( kind )
                            kind[ qi ] = h.kind;
                    }
                }
            }
            if ( lane == 0 && overflow )
                atomicOr( &b.counts->overflow, (uint32_t)kOverflowSdfList );
        }

        __global__ void k_sdf_unsort( Build b, const float * gradSorted, float * gradInput )
        {
            for ( uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < b.n; s += gridDim.x * blockDim.x )
            {
                const uint32_t i = b.perm[ s ];
                for ( int k = 0; k < 4; k++ )
                    gradInput[ 4 * (size_t)i + k ] = gradSorted[ 4 * (size_t)s + k ];
            }
        }

        // ---- headless image: sphere tracing of the signed distance ------------------
        // Every pixel's ray x(t) = eye + t d advances by a step that never crosses the SES:
        // inside the SAS (kinds 3-5) the value rp - dist(x, E) bounds the distance to the SES
        // (every SES point lies at rp from E); outside (kinds 1, 2) value - rp bounds the distance
        // to the SAS, which holds the SES. A ray stops when an inside value falls below eps (a hit
        // at t), when it reaches a point deeper than the band (kind 0, taken as a hit), or when t
        // passes tFar; it advances by at least eps / 4. The ray setup, the march (points eye + t d,
        // steps, t) and the normals are in float32 with every operation rounded on its own, in the
        // order the host tracer writes them, so that the image does not depend on contraction
        // choices. The normal of a hit is the normalised central difference of the signed distance
        // (step normalStep) at the hit point.
        __global__ void __launch_bounds__( 32 * kSdfWarps ) k_trace( Build b, TraceParams p, float band, float * depth,
                                                                       float * normals )
        {
            __shared__ SdfSmem smem[ kSdfWarps ];
            const uint32_t     warp = threadIdx.x >> 5, lane = lane_id();
            uint32_t           overflow = 0;
            const uint32_t     pixels   = p.width * p.height;
            const float3       f        = make_float3( (float)p.forward[ 0 ], (float)p.forward[ 1 ], (float)p.forward[ 2 ] );
            const float3       r        = make_float3( (float)p.right[ 0 ], (float)p.right[ 1 ], (float)p.right[ 2 ] );
            const float3       u        = make_float3( (float)p.up[ 0 ], (float)p.up[ 1 ], (float)p.up[ 2 ] );
            const float3       ef       = make_float3( (float)p.eye[ 0 ], (float)p.eye[ 1 ], (float)p.eye[ 2 ] );
            const float        th       = (float)p.tanHalfFov, W = (float)p.width, H = (float)p.height;
            const float        eps      = (float)p.eps, tFar = (float)p.tFar, hn = (float)p.normalStep;
            const float        minStep  = __fmul_rn( 0.25f, eps );
            for ( uint32_t px = blockIdx.x * kSdfWarps + warp; px < pixels; px += gridDim.x * kSdfWarps )
            {
                const uint32_t iy = px / p.width, ix = px - iy * p.width;
                // pinhole ray through the pixel centre, row-major from the top left
                const float xs  = __fdiv_rn( __fmul_rn( __fmul_rn( __fsub_rn( __fdiv_rn( __fmul_rn( 2.f, __fadd_rn( (float)ix, 0.5f ) ), W ), 1.f ),
                                                                  th ),
                                                        W ),
                                             H );
                const float ys  = __fmul_rn( __fsub_rn( 1.f, __fdiv_rn( __fmul_rn( 2.f, __fadd_rn( (float)iy, 0.5f ) ), H ) ), th );
                const float dx  = __fadd_rn( __fadd_rn( f.x, __fmul_rn( r.x, xs ) ), __fmul_rn( u.x, ys ) );
                const float dy  = __fadd_rn( __fadd_rn( f.y, __fmul_rn( r.y, xs ) ), __fmul_rn( u.y, ys ) );
                const float dz  = __fadd_rn( __fadd_rn( f.z, __fmul_rn( r.z, xs ) ), __fmul_rn( u.z, ys ) );
                const float len = __fsqrt_rn( __fadd_rn( __fadd_rn( __fmul_rn( dx, dx ), __fmul_rn( dy, dy ) ), __fmul_rn( dz, dz ) ) );
                const float3 df = make_float3( __fdiv_rn( dx, len ), __fdiv_rn( dy, len ), __fdiv_rn( dz, len ) );
                float        t   = (float)p.tNear;
                float        hit = __int_as_float( 0x7f800000 ); // +inf: background
                // One query call site for the march and the six evaluations of the normal (the
                // query is inlined once). Evaluation k of the normal moves the hit point by +hn
                // (k even) or -hn (k odd) along axis k / 2.
                float3   xh = make_float3( 0.f, 0.f, 0.f ), g = make_float3( 0.f, 0.f, 0.f );
                float    vp = 0.f;
                uint32_t step = 0;
                int      k    = -1; // -1: marching
                while ( true )
                {
                    float3 q;
                    if ( k < 0 )
                    {
                        if ( !( step < p.maxSteps && t <= tFar ) )
                            break;
                        q = make_float3( __fadd_rn( ef.x, __fmul_rn( t, df.x ) ), __fadd_rn( ef.y, __fmul_rn( t, df.y ) ),
                                         __fadd_rn( ef.z, __fmul_rn( t, df.z ) ) );
                    }
                    else
                    {
                        if ( k == 6 )
                            break;
                        const float e = ( k & 1 ) ? -hn : hn;
                        q             = xh;
                        if ( k < 2 )
                            q.x = __fadd_rn( xh.x, e );
                        else if ( k < 4 )
                            q.y = __fadd_rn( xh.y, e );
                        else
                            q.z = __fadd_rn( xh.z, e );
                    }
                    bool         ex;
                    const SdfHit h = sdf_query<true>( b, q, smem[ warp ], band, overflow, ex );
                    if ( k < 0 )
                    {
                        step++;
                        const bool inside = h.kind == kSdfSphere || h.kind == kSdfCircle || h.kind == kSdfProbe;
                        if ( ( inside && h.value < eps ) || h.kind == kSdfClampInside )
                        {
                            hit = t;
                            if ( !normals )
                                break;
                            // the hit point as the march computed it
                            xh = q;
                            k  = 0;
                            continue;
                        }
                        const float st = inside ? h.value : __fsub_rn( h.value, b.rp );
                        t              = __fadd_rn( t, fmaxf( st, minStep ) );
                        continue;
                    }
                    if ( ( k & 1 ) == 0 )
                        vp = h.value;
                    else
                    {
                        const float ga = __fdiv_rn( __fsub_rn( vp, h.value ), __fmul_rn( 2.f, hn ) );
                        if ( k == 1 )
                            g.x = ga;
                        else if ( k == 3 )
                            g.y = ga;
                        else
                            g.z = ga;
                    }
                    k++;
                }
                float3 nrm = make_float3( 0.f, 0.f, 0.f );
                if ( normals && hit < 3.4e38f )
                {
                    const float gl  = __fsqrt_rn( __fadd_rn( __fadd_rn( __fmul_rn( g.x, g.x ), __fmul_rn( g.y, g.y ) ), __fmul_rn( g.z, g.z ) ) );
                    const float inv = gl > 0.f ? gl : 1.f;
                    nrm = make_float3( __fdiv_rn( g.x, inv ), __fdiv_rn( g.y, inv ), __fdiv_rn( g.z, inv ) );
                }
                if ( lane == 0 )
                {
                    depth[ px ] = hit;
                    if ( normals )
                    {
                        normals[ 3 * (size_t)px ]     = nrm.x;
                        normals[ 3 * (size_t)px + 1 ] = nrm.y;
                        normals[ 3 * (size_t)px + 2 ] = nrm.z;
                    }
                }
            }
            if ( lane == 0 && overflow )
                atomicOr( &b.counts->overflow, (uint32_t)kOverflowSdfList );
        }
    } // namespace

    // keys and order of the queries, the list of queries for the exact pass and its counter, radix scratch
    size_t sdf_scratch_bytes( uint32_t m ) { return 3 * ( ( (size_t)m * 4 + 255 ) & ~(size_t)255 ) + 256 + radix_scratch_bytes( m ); }

    // the list of queries for the exact pass (m entries, then its counter)
    static uint32_t * sdf_exact_list( void * scratch, uint32_t m )
    {
        return reinterpret_cast<uint32_t *>( static_cast<char *>( scratch ) + 2 * ( ( (size_t)m * 4 + 255 ) & ~(size_t)255 ) );
    }

    // queries sorted by grid cell into `order` (scratch: sdf_scratch_bytes)
    static const uint32_t * sdf_order( const Build & b, const float * queries, uint32_t m, void * scratch, cudaStream_t s )
    {
        char *     p     = static_cast<char *>( scratch );
        uint32_t * keys  = reinterpret_cast<uint32_t *>( p );
        uint32_t * order = reinterpret_cast<uint32_t *>( p + ( ( (size_t)m * 4 + 255 ) & ~(size_t)255 ) );
        void *     rad   = p + 3 * ( ( (size_t)m * 4 + 255 ) & ~(size_t)255 ) + 256;
        k_sdf_keys<<<min( persistent_blocks( 256 ), blocks_for( m, 256 ) ), 256, 0, s>>>( b, queries, m, keys, order );
        counted();
        radix_sort( keys, order, m, 32, rad, s );
        return order;
    }

    void launch_sdf( const Build & b, const float * queries, uint32_t m, float band, float * sdf, int * kind, void * scratch,
                     cudaStream_t s )
    {
        if ( !m )
            return;
        const uint32_t * order  = sdf_order( b, queries, m, scratch, s );
        uint32_t *       list   = sdf_exact_list( scratch, m );
        uint32_t *       count  = list + ( ( (size_t)m * 4 + 255 ) & ~(size_t)255 ) / 4;
        const uint32_t   blocks = min( persistent_blocks( 32 * kSdfWarps ) * 2, ( m + kSdfWarps - 1 ) / kSdfWarps );
        cudaMemsetAsync( count, 0, sizeof( uint32_t ), s );
        k_sdf<false><<<blocks, 32 * kSdfWarps, 0, s>>>( b, queries, m, band, sdf, nullptr, nullptr, kind, order, list, count );
        k_sdf_exact<false><<<min( blocks, 152u * 4u ), 32 * kSdfWarps, 0, s>>>( b, queries, band, sdf, nullptr, nullptr, kind, list,
                                                                              count );
        counted( 2 );
    }
    void launch_trace( const Build & b, const TraceParams & p, float band, float * depth, float * normals, cudaStream_t s )
    {
        const uint32_t pixels = p.width * p.height;
        if ( !pixels )
            return;
        const uint32_t blocks = min( persistent_blocks( 32 * kSdfWarps ) * 2, ( pixels + kSdfWarps - 1 ) / kSdfWarps );
        k_trace<<<blocks, 32 * kSdfWarps, 0, s>>>( b, p, band, depth, normals );
        counted();
    }

    void launch_sdf_backward( const Build & b, const float * queries, uint32_t m, float band, const float * gradSdf,
                              float * gradSorted, float * gradInput, void * scratch, cudaStream_t s )
    {
        cudaMemsetAsync( gradSorted, 0, sizeof( float ) * 4 * (size_t)b.n, s );
        if ( m )
        {
            const uint32_t * order  = sdf_order( b, queries, m, scratch, s );
            uint32_t *       list   = sdf_exact_list( scratch, m );
            uint32_t *       count  = list + ( ( (size_t)m * 4 + 255 ) & ~(size_t)255 ) / 4;
            const uint32_t   blocks = min( persistent_blocks( 32 * kSdfWarps ) * 2, ( m + kSdfWarps - 1 ) / kSdfWarps );
            cudaMemsetAsync( count, 0, sizeof( uint32_t ), s );
            k_sdf<true><<<blocks, 32 * kSdfWarps, 0, s>>>( b, queries, m, band, nullptr, gradSdf, gradSorted, nullptr, order, list,
                                                           count );
            k_sdf_exact<true><<<min( blocks, 152u * 4u ), 32 * kSdfWarps, 0, s>>>( b, queries, band, nullptr, gradSdf, gradSorted,
                                                                                 nullptr, list, count );
            counted( 2 );
        }
        if ( b.n )
        {
            k_sdf_unsort<<<blocks_for( b.n, 256 ), 256, 0, s>>>( b, gradSorted, gradInput );
            counted();
        }
    }
} // namespace sesgb
