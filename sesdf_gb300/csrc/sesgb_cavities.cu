// sesgb_cavities.cu -- components of the probe-accessible space on the GPU (no counterpart in the
// reference, whose exterior-only build keeps every probe, cavities included:
// sesdf/src/ssesdf/ssesdf.cu:133-187).
//
// E = probe-centre positions outside every SAS sphere (radius R = r + rp). Its component that touches
// the border of a box around the SAS is the exterior; every other one is a cavity. E is sampled at
// the centres of a voxel grid of spacing h (origin lo = min(c - R) - 2h, dims = ceil((hi - lo) / h) + 1,
// hi = max(c + R) + 2h, index v = (ix * ny + iy) * nz + iz) and its 6-connected components are labelled:
//   k_cav_bounds   one block: min and max of c -+ R over the atoms (double)
//   k_cav_raster   one warp per atom, a lane per (ix, iy) column of its bounding box: the run of voxel
//                  centres inside the SAS sphere along z, set in an occupancy bit grid with one atomicOr
//                  per 32-voxel word. The voxel test is ((dx^2 + dy^2) + dz^2) < R^2 in double
//                  precision, dx = (lo_x + ix h) - c_x, evaluated exactly for the voxels next to the
//                  run's ends; voxels two or more inside the ends are well inside the sphere.
//   k_cav_init     label[v] = the first voxel of v's run of accessible voxels along z (-1 when v is
//                  not accessible): every run starts as a tree of depth one
//   k_cav_union    runs joined across y and x: lock-free union-find (one merge per pair of overlapping
//                  runs, at the first voxel of their overlap) in which a root is only ever linked under a
//                  smaller one (atomicMin), with path halving in every find, so the root of a component
//                  ends as its smallest voxel index
//   k_cav_flatten  label[v] = root of v; roots are collected
//   k_cav_relabel  label[v] = 1 + rank of its root among the sorted roots: components numbered in the
//                  order of their first voxel in index order (the numbering of a raster-order labelling);
//                  voxel count and border flag per component
//   k_cav_probes   each probe: the label of the nearest accessible voxel centre among the 5^3 around its
//                  nearest voxel (first minimum in (ox, oy, oz) order), 0 when there is none
// Every loop that follows parent links is bounded (a chain only ever points to smaller indices); a
// kernel that meets its bound sets an error flag instead of looping on.
#include "sesgb_stages.cuh"

namespace sesgb
{
    namespace
    {
        constexpr uint32_t kCavMaxFind = 1u << 28; // parent links followed at most (a chain is shorter than V)

        inline uint32_t cav_blocks( uint64_t n, uint32_t threads, uint32_t cap = 152u * 16u )
        {
            const uint64_t b = ( n + threads - 1 ) / threads;
            return (uint32_t)( b < cap ? ( b ? b : 1 ) : cap );
        }

        __device__ __forceinline__ double sq( double x ) { return __dmul_rn( x, x ); }

        __global__ void k_cav_bounds( const float4 * atoms, uint32_t n, double rp, double * out )
        {
            __shared__ double red[ 6 ][ 32 ];
            double m[ 6 ] = { 1e300, 1e300, 1e300, -1e300, -1e300, -1e300 };
            for ( uint32_t i = threadIdx.x; i < n; i += blockDim.x )
            {
                const float4 a = atoms[ i ];
                const double R = __dadd_rn( (double)a.w, rp );
                const double c[ 3 ] = { (double)a.x, (double)a.y, (double)a.z };
                for ( int k = 0; k < 3; k++ )
                {
                    m[ k ]     = fmin( m[ k ], __dsub_rn( c[ k ], R ) );
                    m[ 3 + k ] = fmax( m[ 3 + k ], __dadd_rn( c[ k ], R ) );
                }
            }
            for ( int k = 0; k < 6; k++ )
                for ( int o = 16; o > 0; o >>= 1 )
                {
                    const double v = __shfl_xor_sync( 0xffffffffu, m[ k ], o );
                    m[ k ]         = k < 3 ? fmin( m[ k ], v ) : fmax( m[ k ], v );
                }
            const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
            if ( lane == 0 )
                for ( int k = 0; k < 6; k++ )
                    red[ k ][ warp ] = m[ k ];
            __syncthreads();
            if ( threadIdx.x < 6 )
            {
                const int k = threadIdx.x;
                double    v = red[ k ][ 0 ];
                for ( uint32_t w = 1; w < blockDim.x / 32; w++ )
                    v = k < 3 ? fmin( v, red[ k ][ w ] ) : fmax( v, red[ k ][ w ] );
                out[ k ] = v;
            }
        }

        // voxel centre (index i) inside the sphere: the exact double test of the host labelling
        __device__ __forceinline__ bool cav_inside( const CavGrid & g, double a, int iz, double cz, double R2 )
        {
            const double dz = __dsub_rn( __dadd_rn( g.lo[ 2 ], __dmul_rn( (double)iz, g.h ) ), cz );
            return __dadd_rn( a, sq( dz ) ) < R2;
        }

        __device__ __forceinline__ void cav_set_run( uint32_t * bits, uint64_t v0, uint64_t v1 ) // [v0, v1]
        {
            for ( uint64_t w = v0 >> 5; w <= ( v1 >> 5 ); w++ )
            {
                const uint64_t lo = w << 5;
                const uint32_t a  = v0 > lo ? (uint32_t)( v0 - lo ) : 0u;
                const uint32_t b  = v1 < lo + 31 ? (uint32_t)( v1 - lo ) : 31u;
                const uint32_t m  = ( b == 31u ? 0xffffffffu : ( ( 1u << ( b + 1 ) ) - 1u ) ) & ~( ( 1u << a ) - 1u );
                atomicOr( bits + w, m );
            }
        }

        __global__ void k_cav_raster( const float4 * atoms, uint32_t n, CavGrid g, uint32_t * bits )
        {
            const uint32_t lane = threadIdx.x & 31u;
            const uint32_t warps = gridDim.x * ( blockDim.x >> 5 );
            for ( uint32_t i = blockIdx.x * ( blockDim.x >> 5 ) + ( threadIdx.x >> 5 ); i < n; i += warps )
            {
                const float4 at = atoms[ i ];
                const double c[ 3 ] = { (double)at.x, (double)at.y, (double)at.z };
                const double R  = __dadd_rn( (double)at.w, g.rp );
                const double R2 = sq( R );
                const int    k  = (int)ceil( __ddiv_rn( R, g.h ) ) + 1;
                int          lo[ 3 ], hi[ 3 ];
                for ( int a = 0; a < 3; a++ )
                {
                    const int base = (int)floor( __ddiv_rn( __dsub_rn( c[ a ], g.lo[ a ] ), g.h ) );
                    lo[ a ]        = max( base - k, 0 );
                    hi[ a ]        = min( base + k, (int)g.dims[ a ] - 1 );
                }
                const int ny = hi[ 1 ] - lo[ 1 ] + 1;
                const int cols = ( hi[ 0 ] - lo[ 0 ] + 1 ) * ny;
                for ( int col = (int)lane; col < cols; col += 32 )
                {
                    const int    ix = lo[ 0 ] + col / ny, iy = lo[ 1 ] + col % ny;
                    const double dx = __dsub_rn( __dadd_rn( g.lo[ 0 ], __dmul_rn( (double)ix, g.h ) ), c[ 0 ] );
                    const double dy = __dsub_rn( __dadd_rn( g.lo[ 1 ], __dmul_rn( (double)iy, g.h ) ), c[ 1 ] );
                    const double a  = __dadd_rn( sq( dx ), sq( dy ) );
                    const double rem = __dsub_rn( R2, a );
                    if ( rem < -1e-9 * R2 )
                        continue;
                    const double w  = sqrt( fmax( rem, 0.0 ) );
                    // approximate run [za, zb] of centres with |dz| <= w, widened by one voxel each way
                    int za = (int)ceil( __ddiv_rn( __dsub_rn( __dsub_rn( c[ 2 ], w ), g.lo[ 2 ] ), g.h ) ) - 1;
                    int zb = (int)floor( __ddiv_rn( __dsub_rn( __dadd_rn( c[ 2 ], w ), g.lo[ 2 ] ), g.h ) ) + 1;
                    za     = max( za, lo[ 2 ] );
                    zb     = min( zb, hi[ 2 ] );
                    if ( za > zb )
                        continue;
                    // exact tests next to both ends; the voxels between are inside
                    int first = -1, last = -1;
                    for ( int iz = za; iz <= min( za + 2, zb ); iz++ )
                        if ( cav_inside( g, a, iz, c[ 2 ], R2 ) )
                        {
                            first = iz;
                            break;
                        }
                    for ( int iz = zb; iz >= max( zb - 2, za ); iz-- )
                        if ( cav_inside( g, a, iz, c[ 2 ], R2 ) )
                        {
                            last = iz;
                            break;
                        }
                    if ( first < 0 && zb - za > 5 )
                        first = za + 3; // cannot happen for a run this long: its inner voxels are inside
                    if ( last < 0 && zb - za > 5 )
                        last = zb - 3;
                    if ( first < 0 || last < 0 || first > last )
                        continue;
                    const uint64_t row = ( (uint64_t)ix * g.dims[ 1 ] + (uint64_t)iy ) * g.dims[ 2 ];
                    cav_set_run( bits, row + (uint64_t)first, row + (uint64_t)last );
                }
            }
        }

        __device__ __forceinline__ bool cav_free( const uint32_t * bits, uint64_t v ) { return !( ( bits[ v >> 5 ] >> ( v & 31u ) ) & 1u ); }

        // largest occupied bit index in [lo, v), or lo - 1 when there is none
        __device__ __forceinline__ int64_t cav_last_occupied( const uint32_t * bits, uint64_t lo, uint64_t v )
        {
            int64_t w = (int64_t)( v >> 5 );
            uint32_t x = bits[ w ] & ( ( v & 31u ) ? ( 0xffffffffu >> ( 32u - ( v & 31u ) ) ) : 0u );
            const int64_t wlo = (int64_t)( lo >> 5 );
            while ( !x && w > wlo )
                x = bits[ --w ];
            if ( !x )
                return (int64_t)lo - 1;
            const int64_t at = w * 32 + ( 31 - __clz( x ) );
            return at >= (int64_t)lo ? at : (int64_t)lo - 1;
        }

        __global__ void k_cav_init( const uint32_t * bits, CavGrid g, int32_t * L )
        {
            const uint64_t nz = g.dims[ 2 ], V = nz * g.dims[ 1 ] * g.dims[ 0 ];
            for ( uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x )
            {
                if ( !cav_free( bits, v ) )
                {
                    L[ v ] = -1;
                    continue;
                }
                const uint64_t row = v - v % nz;
                L[ v ]             = (int32_t)( cav_last_occupied( bits, row, v ) + 1 );
            }
        }

        // root of v, halving the path on the way (labels only decrease: every write keeps an ancestor)
        __device__ __forceinline__ int32_t cav_find( int32_t * L, int32_t v, uint32_t * err )
        {
            for ( uint32_t s = 0; s < kCavMaxFind; s++ )
            {
                const int32_t p = __ldcg( L + v );
                if ( p == v )
                    return v;
                const int32_t gp = __ldcg( L + p );
                if ( gp == p )
                    return p;
                atomicMin( L + v, gp );
                v = gp;
            }
            atomicOr( err, 1u );
            return v;
        }

        __device__ __forceinline__ void cav_merge( int32_t * L, int32_t a, int32_t b, uint32_t * err )
        {
            for ( uint32_t s = 0; s < kCavMaxFind; s++ )
            {
                a = cav_find( L, a, err );
                b = cav_find( L, b, err );
                if ( a == b )
                    return;
                if ( a > b )
                {
                    const int32_t t = a;
                    a               = b;
                    b               = t;
                }
                // link the larger root under the smaller one; done unless b stopped being a root meanwhile
                const int32_t old = atomicMin( L + b, a );
                if ( old == b )
                    return;
                b = old;
            }
            atomicOr( err, 2u );
        }

        __global__ void k_cav_union( const uint32_t * bits, CavGrid g, int32_t * L, uint32_t * err )
        {
            const uint64_t nz = g.dims[ 2 ], nyz = (uint64_t)g.dims[ 1 ] * nz, V = nyz * g.dims[ 0 ];
            for ( uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x )
            {
                if ( !cav_free( bits, v ) )
                    continue;
                const uint64_t iz = v % nz, iy = ( v / nz ) % g.dims[ 1 ], ix = v / nyz;
                const bool     prev = iz > 0 && cav_free( bits, v - 1 );
                // a neighbouring run is joined once, where its overlap with v's run begins
                if ( iy + 1 < g.dims[ 1 ] && cav_free( bits, v + nz ) && !( prev && cav_free( bits, v + nz - 1 ) ) )
                    cav_merge( L, (int32_t)v, (int32_t)( v + nz ), err );
                if ( ix + 1 < g.dims[ 0 ] && cav_free( bits, v + nyz ) && !( prev && cav_free( bits, v + nyz - 1 ) ) )
                    cav_merge( L, (int32_t)v, (int32_t)( v + nyz ), err );
            }
        }

        __global__ void k_cav_flatten( uint64_t V, int32_t * L, uint32_t * roots, uint32_t rootCap, uint32_t * nRoots,
                                       uint32_t * err )
        {
            for ( uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x )
            {
                const int32_t p = L[ v ];
                if ( p < 0 )
                    continue;
                const int32_t r = cav_find( L, p, err );
                L[ v ]          = r;
                if ( r == (int32_t)v )
                {
                    const uint32_t at = atomicAdd( nRoots, 1u );
                    if ( at < rootCap )
                        roots[ at ] = (uint32_t)v;
                    else
                        atomicOr( err, 4u );
                }
            }
        }

        __global__ void k_cav_relabel( CavGrid g, int32_t * L, const uint32_t * roots, uint32_t nRoots, uint32_t * voxels,
                                       uint8_t * border )
        {
            const uint64_t nz = g.dims[ 2 ], nyz = (uint64_t)g.dims[ 1 ] * nz, V = nyz * g.dims[ 0 ];
            const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
            // every lane runs the same number of iterations, so that the warp vote below sees full warps
            for ( uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < V; base += stride )
            {
                const uint64_t v   = base + threadIdx.x;
                int32_t        lab = 0;
                if ( v < V && L[ v ] >= 0 )
                {
                    const uint32_t r = (uint32_t)L[ v ];
                    uint32_t       a = 0, b = nRoots; // lower bound of r in the sorted roots
                    while ( a < b )
                    {
                        const uint32_t m = ( a + b ) >> 1;
                        if ( roots[ m ] < r )
                            a = m + 1;
                        else
                            b = m;
                    }
                    lab = (int32_t)a + 1;
                    const uint64_t iz = v % nz, iy = ( v / nz ) % g.dims[ 1 ], ix = v / nyz;
                    if ( ix == 0 || iy == 0 || iz == 0 || ix + 1 == g.dims[ 0 ] || iy + 1 == g.dims[ 1 ] || iz + 1 == nz )
                        border[ lab ] = 1;
                }
                if ( v < V )
                    L[ v ] = lab;
                // voxel counts, one atomic per distinct label of the warp
                const uint32_t peers = __match_any_sync( 0xffffffffu, lab );
                if ( lab > 0 && ( threadIdx.x & 31u ) == (uint32_t)( __ffs( peers ) - 1 ) )
                    atomicAdd( voxels + lab, (uint32_t)__popc( peers ) );
            }
        }

        __global__ void k_cav_probes( const float4 * probes, uint32_t k, CavGrid g, const int32_t * L, int32_t * out )
        {
            for ( uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < k; q += gridDim.x * blockDim.x )
            {
                const float4 pf = probes[ q ];
                const double p[ 3 ] = { (double)pf.x, (double)pf.y, (double)pf.z };
                int          base[ 3 ];
                for ( int a = 0; a < 3; a++ )
                    base[ a ] = (int)rint( __ddiv_rn( __dsub_rn( p[ a ], g.lo[ a ] ), g.h ) );
                double  best = 1e300;
                int32_t lab  = 0;
                for ( int ox = -2; ox <= 2; ox++ )
                    for ( int oy = -2; oy <= 2; oy++ )
                        for ( int oz = -2; oz <= 2; oz++ )
                        {
                            const int o[ 3 ] = { ox, oy, oz };
                            int       idx[ 3 ];
                            double    d2 = 0.0;
                            for ( int a = 0; a < 3; a++ )
                            {
                                idx[ a ]       = min( max( base[ a ] + o[ a ], 0 ), (int)g.dims[ a ] - 1 );
                                const double d = __dsub_rn( __dadd_rn( g.lo[ a ], __dmul_rn( (double)idx[ a ], g.h ) ), p[ a ] );
                                d2             = a == 0 ? sq( d ) : __dadd_rn( d2, sq( d ) );
                            }
                            const int32_t l = L[ ( (uint64_t)idx[ 0 ] * g.dims[ 1 ] + (uint64_t)idx[ 1 ] ) * g.dims[ 2 ] + (uint64_t)idx[ 2 ] ];
                            if ( l > 0 && d2 < best )
                            {
                                best = d2;
                                lab  = l;
                            }
                        }
                out[ q ] = lab;
            }
        }
    } // namespace

    void launch_cavity_bounds( const Build & b, double rp, double * out, cudaStream_t s )
    {
        k_cav_bounds<<<1, 1024, 0, s>>>( b.atoms, b.n, rp, out );
        count_launches( 1 );
    }

    void launch_cavity_labels( const Build & b, const CavGrid & g, uint32_t * bits, int32_t * labels, uint32_t * roots,
                               uint32_t rootCap, uint32_t * scalars, cudaStream_t s )
    {
        const uint64_t V = (uint64_t)g.dims[ 0 ] * g.dims[ 1 ] * g.dims[ 2 ];
        cudaMemsetAsync( bits, 0, sizeof( uint32_t ) * ( ( V + 31 ) / 32 ), s );
        cudaMemsetAsync( scalars, 0, sizeof( uint32_t ) * 2, s );
        if ( b.n )
            k_cav_raster<<<cav_blocks( (uint64_t)b.n * 32, 256 ), 256, 0, s>>>( b.atoms, b.n, g, bits );
        k_cav_init<<<cav_blocks( V, 256 ), 256, 0, s>>>( bits, g, labels );
        k_cav_union<<<cav_blocks( V, 256 ), 256, 0, s>>>( bits, g, labels, scalars + 1 );
        k_cav_flatten<<<cav_blocks( V, 256 ), 256, 0, s>>>( V, labels, roots, rootCap, scalars, scalars + 1 );
        count_launches( b.n ? 4 : 3 );
    }

    void launch_cavity_relabel( const CavGrid & g, int32_t * labels, const uint32_t * roots, uint32_t nRoots, uint32_t * voxels,
                                uint8_t * border, const float4 * probes, uint32_t k, int32_t * probeLabel, cudaStream_t s )
    {
        const uint64_t V = (uint64_t)g.dims[ 0 ] * g.dims[ 1 ] * g.dims[ 2 ];
        cudaMemsetAsync( voxels, 0, sizeof( uint32_t ) * ( nRoots + 1 ), s );
        cudaMemsetAsync( border, 0, nRoots + 1, s );
        k_cav_relabel<<<cav_blocks( V, 256 ), 256, 0, s>>>( g, labels, roots, nRoots, voxels, border );
        count_launches( 1 );
        if ( k && probeLabel )
        {
            k_cav_probes<<<cav_blocks( k, 128 ), 128, 0, s>>>( probes, k, g, labels, probeLabel );
            count_launches( 1 );
        }
    }
} // namespace sesgb
