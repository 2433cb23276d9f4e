// sesgb_sort.cu -- scan and radix-sort primitives for the SES build.
//
// Exclusive scan: reduce-then-scan over 2048-element tiles (three launches, no
// inter-block waiting). Radix sort: stable LSD passes over 8-bit digits with a
// per-tile digit histogram, a scan of the (digit, tile) matrix and a scatter
// that ranks equal digits inside a tile with warp match masks, round by round,
// so that the order of equal keys is kept.
#include "sesgb_internal.h"

namespace sesgb
{
    namespace
    {
        constexpr int kScanThreads = 256;
        constexpr int kScanItems   = 8;
        constexpr int kScanTile    = kScanThreads * kScanItems;
        constexpr int kScanArrays  = 3;

        __device__ __forceinline__ uint64_t scan_len( uint64_t nHost, const uint32_t * nDevice )
        {
            if ( !nDevice )
                return nHost;
            const uint64_t n = *nDevice;
            return n < nHost ? n : nHost;
        }

        // block-wide exclusive sum of one value per thread
        __device__ __forceinline__ uint32_t block_exclusive_sum( uint32_t v, uint32_t & total, uint32_t * warpSums )
        {
            uint32_t       wt;
            const uint32_t x    = warp_exclusive_sum( v, wt );
            const uint32_t warp = threadIdx.x >> 5;
            if ( lane_id() == 31 )
                warpSums[ warp ] = wt;
            __syncthreads();
            if ( warp == 0 )
            {
                const uint32_t s = lane_id() < ( blockDim.x >> 5 ) ? warpSums[ lane_id() ] : 0u;
                uint32_t       t;
                const uint32_t e = warp_exclusive_sum( s, t );
                if ( lane_id() < ( blockDim.x >> 5 ) )
                    warpSums[ lane_id() ] = e;
                if ( lane_id() == 0 )
                    warpSums[ 32 ] = t;
            }
            __syncthreads();
            const uint32_t r = x + warpSums[ warp ];
            total            = warpSums[ 32 ];
            __syncthreads();
            return r;
        }

        // Up to kScanArrays independent scans of the same length in one launch
        // (blockIdx.y selects the array).
        struct ScanArrays
        {
            const uint32_t * in[ kScanArrays ];
            uint32_t *       out[ kScanArrays ];
            uint32_t *       total[ kScanArrays ];
        };

        __global__ void __launch_bounds__( kScanThreads ) k_tile_sums( ScanArrays a, uint64_t nHost, const uint32_t * nDevice,
                                                                        uint32_t * tileSums, uint32_t tiles )
        {
            pdl_begin();
            __shared__ uint32_t warpSums[ 33 ];
            const uint64_t      n    = scan_len( nHost, nDevice );
            const uint64_t      base = (uint64_t)blockIdx.x * kScanTile;
            const uint32_t *    in   = a.in[ blockIdx.y ];
            if ( base >= n )
                return;
            uint32_t s = 0;
#pragma unroll
            for ( int k = 0; k < kScanItems; k++ )
            {
                const uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
                if ( i < n )
                    s += in[ i ];
            }
            uint32_t total;
            block_exclusive_sum( s, total, warpSums );
            if ( threadIdx.x == 0 )
                tileSums[ blockIdx.y * tiles + blockIdx.x ] = total;
        }

        // Each tile adds up the sums of the tiles before it (a few hundred at most
        // for the sizes of the build), scans itself, and the tile holding the last
        // element writes out[n] and the total.
        __global__ void __launch_bounds__( kScanThreads ) k_tile_scan( ScanArrays a, uint64_t nHost, const uint32_t * nDevice,
                                                                        const uint32_t * tileSums, uint32_t tiles )
        {
            pdl_begin();
            __shared__ uint32_t tile[ kScanTile + kScanTile / 32 ];
            __shared__ uint32_t warpSums[ 33 ];
            const uint64_t      n    = scan_len( nHost, nDevice );
            const uint64_t      base = (uint64_t)blockIdx.x * kScanTile;
            const uint32_t *    in   = a.in[ blockIdx.y ];
            uint32_t *          out  = a.out[ blockIdx.y ];
            if ( n == 0 )
            {
                if ( blockIdx.x == 0 && threadIdx.x == 0 )
                {
                    out[ 0 ] = 0;
                    if ( a.total[ blockIdx.y ] )
                        *a.total[ blockIdx.y ] = 0;
                }
                return;
            }
            if ( base >= n )
                return;
            // offset of this tile
            uint32_t before = 0;
            for ( uint32_t t = threadIdx.x; t < blockIdx.x; t += kScanThreads )
                before += tileSums[ blockIdx.y * tiles + t ];
            uint32_t offsetTotal;
            block_exclusive_sum( before, offsetTotal, warpSums );
            // coalesced load into a padded tile (index + index / 32 avoids bank conflicts)
#pragma unroll
            for ( int k = 0; k < kScanItems; k++ )
            {
                const uint32_t j = k * kScanThreads + threadIdx.x;
                const uint64_t i = base + j;
                tile[ j + j / 32 ] = i < n ? in[ i ] : 0u;
            }
            __syncthreads();
            uint32_t v[ kScanItems ];
            uint32_t s = 0;
#pragma unroll
            for ( int k = 0; k < kScanItems; k++ )
            {
                const uint32_t j = threadIdx.x * kScanItems + k;
                v[ k ]           = tile[ j + j / 32 ];
                s += v[ k ];
            }
            uint32_t total;
            uint32_t e = block_exclusive_sum( s, total, warpSums ) + offsetTotal;
#pragma unroll
            for ( int k = 0; k < kScanItems; k++ )
            {
                const uint32_t j = threadIdx.x * kScanItems + k;
                tile[ j + j / 32 ] = e;
                e += v[ k ];
            }
            __syncthreads();
#pragma unroll
            for ( int k = 0; k < kScanItems; k++ )
            {
                const uint32_t j = k * kScanThreads + threadIdx.x;
                const uint64_t i = base + j;
                if ( i < n )
                    out[ i ] = tile[ j + j / 32 ];
            }
            if ( threadIdx.x == 0 && base + kScanTile >= n )
            {
                out[ n ] = offsetTotal + total;
                if ( a.total[ blockIdx.y ] )
                    *a.total[ blockIdx.y ] = offsetTotal + total;
            }
        }

        // ---- radix sort ---------------------------------------------------
        constexpr int kRadixThreads = 256;
        constexpr int kRadixRounds  = 8;
        constexpr int kRadixTile    = kRadixThreads * kRadixRounds;
        constexpr int kRadixWarps   = kRadixThreads / 32;

        __global__ void __launch_bounds__( kRadixThreads ) k_radix_hist( const uint32_t * keys, uint32_t n, int shift,
                                                                          uint32_t * hist, uint32_t tiles )
        {
            pdl_begin();
            __shared__ uint32_t h[ 256 ];
            h[ threadIdx.x ] = 0;
            __syncthreads();
            const uint32_t base = blockIdx.x * kRadixTile;
            for ( int r = 0; r < kRadixRounds; r++ )
            {
                const uint32_t i = base + r * kRadixThreads + threadIdx.x;
                if ( i < n )
                    atomicAdd( &h[ ( keys[ i ] >> shift ) & 255u ], 1u );
            }
            __syncthreads();
            hist[ threadIdx.x * tiles + blockIdx.x ] = h[ threadIdx.x ];
        }

        __global__ void __launch_bounds__( kRadixThreads ) k_radix_scatter( const uint32_t * keysIn, const uint32_t * valsIn,
                                                                             uint32_t * keysOut, uint32_t * valsOut, uint32_t n,
                                                                             int shift, const uint32_t * offsets, uint32_t tiles )
        {
            pdl_begin();
            __shared__ uint32_t base[ 256 ];
            __shared__ uint32_t warpCount[ kRadixWarps ][ 256 ];
            const uint32_t      warp = threadIdx.x >> 5;
            base[ threadIdx.x ]      = offsets[ threadIdx.x * tiles + blockIdx.x ];
            const uint32_t tile0     = blockIdx.x * kRadixTile;
            for ( int r = 0; r < kRadixRounds; r++ )
            {
                for ( int w = 0; w < kRadixWarps; w++ )
                    warpCount[ w ][ threadIdx.x ] = 0;
                __syncthreads();
                const uint32_t i     = tile0 + r * kRadixThreads + threadIdx.x;
                const bool     valid = i < n;
                uint32_t       key = 0, val = 0, digit = 256;
                if ( valid )
                {
                    key   = keysIn[ i ];
                    val   = valsIn[ i ];
                    digit = ( key >> shift ) & 255u;
                }
                const uint32_t peers = __match_any_sync( 0xffffffffu, digit );
                const uint32_t rank  = __popc( peers & lanemask_lt() );
                if ( valid && rank == 0 )
                    warpCount[ warp ][ digit ] = __popc( peers );
                __syncthreads();
                // per digit: prefix over warps, then advance the running base
                {
                    const uint32_t d   = threadIdx.x;
                    uint32_t       acc = 0;
                    for ( int w = 0; w < kRadixWarps; w++ )
                    {
                        const uint32_t c  = warpCount[ w ][ d ];
                        warpCount[ w ][ d ] = acc;
                        acc += c;
                    }
                    __syncthreads();
                    if ( valid )
                    {
                        const uint32_t dst = base[ digit ] + warpCount[ warp ][ digit ] + rank;
                        keysOut[ dst ]     = key;
                        valsOut[ dst ]     = val;
                    }
                    __syncthreads();
                    base[ d ] += acc;
                }
                __syncthreads();
            }
        }
    } // namespace

    size_t scan_scratch_bytes( uint64_t n )
    {
        const uint64_t tiles = ( n + kScanTile - 1 ) / kScanTile + 1;
        return ( kScanArrays * tiles * sizeof( uint32_t ) + 255 ) & ~(size_t)255;
    }
    void exclusive_scan_many( const ScanJob * jobs, int count, uint64_t nHost, const uint32_t * nDevice, void * scratch,
                              cudaStream_t stream )
    {
        ScanArrays a = {};
        for ( int k = 0; k < count && k < kScanArrays; k++ )
        {
            a.in[ k ]    = jobs[ k ].in;
            a.out[ k ]   = jobs[ k ].out;
            a.total[ k ] = jobs[ k ].total;
        }
        const uint32_t tiles = (uint32_t)( ( nHost + kScanTile - 1 ) / kScanTile );
        const dim3     grid( tiles > 0 ? tiles : 1u, (unsigned)( count < kScanArrays ? count : kScanArrays ) );
        uint32_t *     tileSums = static_cast<uint32_t *>( scratch );
        if ( tiles > 1 )
        {
            pdl_launch( k_tile_sums, grid, kScanThreads, 0, stream, a, nHost, nDevice, tileSums, tiles );
            count_launches( 1 );
        }
        pdl_launch( k_tile_scan, grid, kScanThreads, 0, stream, a, nHost, nDevice, tileSums, tiles );
        count_launches( 1 );
    }
    void exclusive_scan( const uint32_t * in, uint32_t * out, uint64_t nHost, const uint32_t * nDevice, uint32_t * total,
                         void * scratch, cudaStream_t stream )
    {
        const ScanJob job = { in, out, total };
        exclusive_scan_many( &job, 1, nHost, nDevice, scratch, stream );
    }

    size_t radix_scratch_bytes( uint32_t n )
    {
        const uint64_t tiles = ( (uint64_t)n + kRadixTile - 1 ) / kRadixTile;
        const uint64_t hist  = 256 * ( tiles ? tiles : 1 );
        size_t         b     = 0;
        b += ( 2ull * n * sizeof( uint32_t ) + 255 ) & ~(size_t)255; // ping-pong keys + vals
        b += ( ( hist + 1 ) * sizeof( uint32_t ) + 255 ) & ~(size_t)255;
        b += scan_scratch_bytes( hist );
        return b;
    }

    void radix_sort( uint32_t * keys, uint32_t * vals, uint32_t n, int bits, void * scratch, cudaStream_t stream )
    {
        if ( n <= 1 || bits <= 0 )
            return;
        const uint32_t tiles = ( n + kRadixTile - 1 ) / kRadixTile;
        const uint64_t hist  = 256ull * tiles;
        char *         p     = static_cast<char *>( scratch );
        uint32_t *     keys2 = reinterpret_cast<uint32_t *>( p );
        uint32_t *     vals2 = keys2 + n;
        p += ( 2ull * n * sizeof( uint32_t ) + 255 ) & ~(size_t)255;
        uint32_t * histBuf = reinterpret_cast<uint32_t *>( p );
        p += ( ( hist + 1 ) * sizeof( uint32_t ) + 255 ) & ~(size_t)255;
        void * scanScratch = p;

        uint32_t *ka = keys, *va = vals, *kb = keys2, *vb = vals2;
        int       passes = 0;
        for ( int shift = 0; shift < bits; shift += 8, passes++ )
        {
            pdl_launch( k_radix_hist, tiles, kRadixThreads, 0, stream, ka, n, shift, histBuf, tiles );
            exclusive_scan( histBuf, histBuf, hist, nullptr, nullptr, scanScratch, stream );
            pdl_launch( k_radix_scatter, tiles, kRadixThreads, 0, stream, ka, va, kb, vb, n, shift, histBuf, tiles );
            count_launches( 2 );
            std::swap( ka, kb );
            std::swap( va, vb );
        }
        if ( passes & 1 )
        {
            cudaMemcpyAsync( keys, ka, sizeof( uint32_t ) * n, cudaMemcpyDeviceToDevice, stream );
            cudaMemcpyAsync( vals, va, sizeof( uint32_t ) * n, cudaMemcpyDeviceToDevice, stream );
        }
    }
} // namespace sesgb
