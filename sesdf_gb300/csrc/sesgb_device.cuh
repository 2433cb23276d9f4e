// sesgb_device.cuh -- device helpers shared by the SES build kernels.
//
// Two arithmetic layers:
//  * float32 "filter" math in coordinates relative to the atom that owns the
//    work item (differences of nearby float32 coordinates are exact), used for
//    every predicate together with a conservative error band;
//  * double-precision twins of the reference's expressions, written with
//    explicitly rounded intrinsics (__dadd_rn, __dmul_rn, ...) so that no
//    multiply-add contraction happens. They reproduce, operation for
//    operation, the IEEE double evaluation of the reference's formulas; a
//    predicate whose float32 margin falls inside the band is decided here.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sesgb
{
    // ---- float32 -----------------------------------------------------------
    struct f3
    {
        float x, y, z;
    };
    __device__ __forceinline__ f3 F3( float x, float y, float z ) { return { x, y, z }; }
    __device__ __forceinline__ f3 F3( float4 a ) { return { a.x, a.y, a.z }; }
    __device__ __forceinline__ f3 operator+( f3 a, f3 b ) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
    __device__ __forceinline__ f3 operator-( f3 a, f3 b ) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
    __device__ __forceinline__ f3 operator*( f3 a, float s ) { return { a.x * s, a.y * s, a.z * s }; }
    __device__ __forceinline__ float dot( f3 a, f3 b ) { return a.x * b.x + a.y * b.y + a.z * b.z; }
    __device__ __forceinline__ f3 cross( f3 a, f3 b )
    {
        return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
    }
    __device__ __forceinline__ f3 normalize( f3 v ) { return v * rsqrtf( dot( v, v ) ); }

    // ---- double, explicitly rounded (no contraction) ------------------------
    struct d3
    {
        double x, y, z;
    };
    __device__ __forceinline__ d3 D3( double x, double y, double z ) { return { x, y, z }; }
    __device__ __forceinline__ d3 D3( float4 a ) { return { (double)a.x, (double)a.y, (double)a.z }; }
    __device__ __forceinline__ d3 dadd( d3 a, d3 b ) { return { __dadd_rn( a.x, b.x ), __dadd_rn( a.y, b.y ), __dadd_rn( a.z, b.z ) }; }
    __device__ __forceinline__ d3 dsub( d3 a, d3 b ) { return { __dsub_rn( a.x, b.x ), __dsub_rn( a.y, b.y ), __dsub_rn( a.z, b.z ) }; }
    __device__ __forceinline__ d3 dmul( d3 a, double s ) { return { __dmul_rn( a.x, s ), __dmul_rn( a.y, s ), __dmul_rn( a.z, s ) }; }
    // a.x*b.x + a.y*b.y + a.z*b.z, left to right
    __device__ __forceinline__ double ddot( d3 a, d3 b )
    {
        return __dadd_rn( __dadd_rn( __dmul_rn( a.x, b.x ), __dmul_rn( a.y, b.y ) ), __dmul_rn( a.z, b.z ) );
    }
    __device__ __forceinline__ d3 dcross( d3 a, d3 b )
    {
        return { __dsub_rn( __dmul_rn( a.y, b.z ), __dmul_rn( a.z, b.y ) ),
                 __dsub_rn( __dmul_rn( a.z, b.x ), __dmul_rn( a.x, b.z ) ),
                 __dsub_rn( __dmul_rn( a.x, b.y ), __dmul_rn( a.y, b.x ) ) };
    }
    // v * (1 / sqrt(dot(v, v)))
    __device__ __forceinline__ d3 dnrm( d3 v ) { return dmul( v, __ddiv_rn( 1.0, __dsqrt_rn( ddot( v, v ) ) ) ); }

    struct dcircle
    {
        d3     center;
        d3     normal;
        double radius;
    };

    // getCircleGeometry / getCircleCenter of the reference
    // (sesdf/include/bcs/sesdf/data.cuh:98-114, sesdf/include/bcs/cuda/circles.cuh:9-14)
    __device__ __forceinline__ dcircle dcircle_geometry( d3 ci, double ri, d3 cj, double rj, double rp )
    {
        const double R1 = __dadd_rn( ri, rp ), R2 = __dadd_rn( rj, rp );
        const d3     dij = dsub( ci, cj );
        const double d   = ddot( dij, dij );
        const double t   = __ddiv_rn( __dadd_rn( __dsub_rn( __dmul_rn( R1, R1 ), __dmul_rn( R2, R2 ) ), d ), __dmul_rn( 2.0, d ) );
        dcircle      c;
        c.center        = dadd( ci, dmul( dsub( cj, ci ), t ) );
        const d3 toI    = dsub( ci, c.center );
        c.radius        = __dsqrt_rn( __dsub_rn( __dmul_rn( R1, R1 ), ddot( toI, toI ) ) );
        c.normal        = dnrm( dsub( cj, ci ) );
        return c;
    }

    // One k of computeCirclesVisibilityStatus (sesdf/src/sesdf/operations.cu:164-197):
    // bit 0 set if k's SAS sphere holds the whole circle, bit 1 set if it
    // touches the circle (both with the reference's 1e-4f tolerance).
    __device__ __forceinline__ int dcircle_vs_atom( const dcircle & c, d3 ck, double Rk )
    {
        const d3     kToCircle      = dsub( c.center, ck );
        const double distToCircle   = __dsqrt_rn( ddot( kToCircle, kToCircle ) );
        const double secondDistance = ddot( kToCircle, c.normal );
        const double cosTheta       = __ddiv_rn( secondDistance, distToCircle );
        const double sinTheta       = __dsqrt_rn( __dsub_rn( 1.0, __dmul_rn( cosTheta, cosTheta ) ) );
        const double tol            = (double)1e-4f;
        const double Rk2            = __dmul_rn( Rk, Rk );
        int          r              = 0;
        {
            const double first    = __dadd_rn( __dmul_rn( sinTheta, distToCircle ), c.radius );
            const double complete = __dadd_rn( __dmul_rn( first, first ), __dmul_rn( secondDistance, secondDistance ) );
            if ( __dsub_rn( complete, Rk2 ) < tol )
                r |= 1;
        }
        {
            const double first    = __dadd_rn( __dmul_rn( -sinTheta, distToCircle ), c.radius );
            const double complete = __dadd_rn( __dmul_rn( first, first ), __dmul_rn( secondDistance, secondDistance ) );
            if ( __dsub_rn( complete, Rk2 ) < tol )
                r |= 2;
        }
        return r;
    }

    // Neighbour predicate of findCirclesInCell (sesdf/src/sesdf/operations.cu:55-57)
    __device__ __forceinline__ bool dneighbor( d3 ci, double ri, d3 cj, double rj, double rp )
    {
        const d3     v  = dsub( ci, cj );
        const double d  = ddot( v, v );
        const double R  = __dadd_rn( __dadd_rn( ri, rp ), __dadd_rn( rj, rp ) );
        return __dsub_rn( d, __dmul_rn( R, R ) ) <= (double)1e-4f;
    }

    // pseudo-angle ordered like angleBetweenEdges (sesdf/include/bcs/cuda/circles.cuh:27-31)
    __device__ __forceinline__ double dpseudo_angle( d3 u, d3 v, d3 n )
    {
        double c = __ddiv_rn( ddot( u, v ), __dmul_rn( __dsqrt_rn( ddot( u, u ) ), __dsqrt_rn( ddot( v, v ) ) ) );
        c        = fmax( -1.0, fmin( c, 1.0 ) );
        const double det = ddot( u, dcross( v, n ) );
        return copysign( 1.0, det ) > 0.0 ? __dsub_rn( 1.0, c ) : __dadd_rn( 3.0, c );
    }

    // ---- float-float ("double-float") arithmetic -----------------------------
    // A value is hi + lo with two float32 numbers, |lo| <= ulp(hi) / 2: about 48
    // significand bits on the float32 pipes (64x the FP64 rate on GB300). The
    // error-free transforms are Knuth's two-sum, Dekker's fast two-sum and the
    // FMA two-product; add, multiply, divide and square root follow the usual
    // double-word algorithms (as in Dekker 1971 and the QD library of Hida, Li and
    // Bailey, 2001), written here with explicitly rounded float intrinsics so that
    // no contraction changes them.
    struct ff
    {
        float hi, lo;
    };
    __device__ __forceinline__ ff ff_of( float a ) { return { a, 0.f }; }
    __device__ __forceinline__ ff two_sum( float a, float b )
    {
        const float s  = __fadd_rn( a, b );
        const float bb = __fsub_rn( s, a );
        const float e  = __fadd_rn( __fsub_rn( a, __fsub_rn( s, bb ) ), __fsub_rn( b, bb ) );
        return { s, e };
    }
    __device__ __forceinline__ ff fast_two_sum( float a, float b ) // |a| >= |b| (or a = 0)
    {
        const float s = __fadd_rn( a, b );
        return { s, __fsub_rn( b, __fsub_rn( s, a ) ) };
    }
    __device__ __forceinline__ ff two_prod( float a, float b )
    {
        const float p = __fmul_rn( a, b );
        return { p, __fmaf_rn( a, b, -p ) };
    }
    __device__ __forceinline__ ff ff_add( ff x, ff y )
    {
        ff       s = two_sum( x.hi, y.hi );
        const ff t = two_sum( x.lo, y.lo );
        s          = fast_two_sum( s.hi, __fadd_rn( s.lo, t.hi ) );
        return fast_two_sum( s.hi, __fadd_rn( s.lo, t.lo ) );
    }
    __device__ __forceinline__ ff ff_neg( ff x ) { return { -x.hi, -x.lo }; }
    __device__ __forceinline__ ff ff_sub( ff x, ff y ) { return ff_add( x, ff_neg( y ) ); }
    __device__ __forceinline__ ff ff_mul( ff x, ff y )
    {
        ff p = two_prod( x.hi, y.hi );
        p.lo = __fmaf_rn( x.hi, y.lo, __fmaf_rn( x.lo, y.hi, p.lo ) );
        return fast_two_sum( p.hi, p.lo );
    }
    __device__ __forceinline__ ff ff_scale( ff x, float pow2 ) { return { __fmul_rn( x.hi, pow2 ), __fmul_rn( x.lo, pow2 ) }; }
    // x / y: a float quotient refined twice by the float-float remainder
    __device__ __forceinline__ ff ff_div( ff x, ff y )
    {
        const float q1 = __fdiv_rn( x.hi, y.hi );
        ff          r  = ff_sub( x, ff_mul( y, ff_of( q1 ) ) );
        const float q2 = __fdiv_rn( r.hi, y.hi );
        r              = ff_sub( r, ff_mul( y, ff_of( q2 ) ) );
        const float q3 = __fdiv_rn( r.hi, y.hi );
        const ff    q  = fast_two_sum( q1, q2 );
        return ff_add( q, ff_of( q3 ) );
    }
    // sqrt(x), x > 0: the float root corrected by one Newton step in float-float
    __device__ __forceinline__ ff ff_sqrt( ff x )
    {
        const float s = __fsqrt_rn( x.hi );
        const ff    r = ff_sub( x, two_prod( s, s ) );
        return fast_two_sum( s, __fdiv_rn( r.hi, __fmul_rn( 2.f, s ) ) );
    }

    // ---- reference grid hash (GridInfo, sesdf/include/bcs/cuda/grid.inl) ---
    struct GridRef
    {
        float3 origin;
        float3 cell;
        int    size;
    };

    // The reference is compiled with --use_fast_math, under which a float
    // division is the full-range approximate division; the same instruction is
    // used here so that cell assignments agree at cell boundaries.
    __device__ __forceinline__ float div_full( float a, float b )
    {
        float r;
        asm( "div.full.ftz.f32 %0, %1, %2;" : "=f"( r ) : "f"( a ), "f"( b ) );
        return r;
    }
    __device__ __forceinline__ int3 ref_grid_position( const GridRef & g, float x, float y, float z )
    {
        return make_int3( (int)floorf( div_full( x - g.origin.x, g.cell.x ) ), (int)floorf( div_full( y - g.origin.y, g.cell.y ) ),
                          (int)floorf( div_full( z - g.origin.z, g.cell.z ) ) );
    }
    __device__ __forceinline__ uint32_t ref_grid_hash( const GridRef & g, int3 p )
    {
        const int s = g.size;
        const int x = p.x & ( s - 1 ), y = p.y & ( s - 1 ), z = p.z & ( s - 1 );
        return (uint32_t)( z * s * s + y * s + x );
    }

    // ---- warp helpers -------------------------------------------------------
    // Programmatic dependent launch: a kernel launched with
    // cudaLaunchAttributeProgrammaticStreamSerialization right after another one
    // has its launch prepared while that grid runs. It waits here, before it reads
    // anything, until the previous grid has completed and its writes are visible (a
    // no-op when there is no such grid). No kernel triggers its dependents early:
    // measured on GB300, dependents scheduled at the start of a grid take SM slots
    // from its last wave and the build gets 2 % slower, while the prepared launch
    // alone saves about 1 %.
    __device__ __forceinline__ void pdl_begin() { asm volatile( "griddepcontrol.wait;" ::: "memory" ); }

    __device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
    __device__ __forceinline__ uint32_t lanemask_lt() { return ( 1u << lane_id() ) - 1u; }

    template<class T> __device__ __forceinline__ T warp_exclusive_sum( T v, T & total )
    {
        T x = v;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            const T y = __shfl_up_sync( 0xffffffffu, x, o );
            if ( (int)lane_id() >= o )
                x += y;
        }
        total = __shfl_sync( 0xffffffffu, x, 31 );
        return x - v;
    }
} // namespace sesgb
