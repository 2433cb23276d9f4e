// sesgb_area.cu -- solvent-excluded surface area of the primitives of a
// full-surface build, and its adjoint with respect to the atoms.
//
// The reference renders its primitives and computes no area; the area here is
// the area of those primitives: the convex patch of every atom (the directions
// of its SAS sphere outside every other SAS sphere of N(i), scaled to the vdW
// sphere: the sectors of buildConvexPatchesSectors, operations.inl:175-228),
// the torus swept over the accessible arcs of every circle (the segments and
// full circles, operations.inl:552-668), trimmed at its axis when it
// self-intersects, and the concave triangle of every probe (operations.inl:
// 230-486) outside the spheres of its listed neighbour probes
// (findIntersectionsNeighbors, operations.cu:271-338).
//
// Every patch is a region R = {y : |y| = 1, y . w_m <= c_m} of a sphere. By
// Gauss-Bonnet its area is 2 pi chi + sum_m c_m dphi_m - sum_v theta_v, with
// dphi_m the angle of circle m on the boundary of R and theta_v the turning
// angle at a corner. Cut into three lunes of 120 degrees around z, every piece
// has area < 2 pi, so the sum reduced mod 2 pi is the area and the Euler
// characteristic is never needed. The corner terms are written per arc, as the
// change of the boundary tangent's angle against a fixed frame field between the
// arc's ends, so that no corner has to be matched with the arc on its other side
// (several circles through one point, as at the axis points of a self-intersecting
// torus, need no special case, and float32 rounding moves the sum only by as much
// as it moves the arcs). Adjoint: dA/dc_m = dphi_m,
// dA/dw_m = -integral of y over the boundary arcs of m; an arc's angle moves with
// the circles that bound its ends; probe positions follow their atoms by the
// implicit function of |p - c_a|^2 = R_a^2.
//
// Work split: a warp per atom (lanes over the circles of its region), a warp per
// probe (lanes over the triangle edges and neighbour caps), float32 throughout.
#include "sesgb_device.cuh"
#include "sesgb_stages.cuh"

namespace sesgb
{
    namespace
    {
        constexpr float    kPiF       = 3.14159265358979f;
        constexpr float    k2PiF      = 6.28318530717959f;
        constexpr int      kAreaWarps = 4;
        constexpr int      kAreaNbr   = 128;             // neighbour constraints of one atom region
        constexpr int      kAreaIv    = 64 + 2;          // cuts of one constraint circle (a lane's own, local memory)
        constexpr int      kLuneIv    = kAreaNbr + 2;    // cuts of one lune-plane circle (the warp's, shared memory)
        constexpr int      kProbeCons = 3 + (int)kMaxProbeNbr;
        // |tw| below which a torus arc end's angle terms are taken in double precision: its float32
        // position carries rounding ~1e-7 / |tw|, and the terms go as 1 / tw
        constexpr float kShallowCrossing = 0.1f;
        static_assert( kMaxProbeNbr <= 32, "one neighbour cap per lane" );

        struct Circ
        {
            f3    w, e1, e2;
            float c, s;
        };

        // reduces an angle in (-4 pi, 6 pi) to [0, 2 pi)
        __device__ __forceinline__ float wrapf( float a )
        {
            if ( a < 0.f )
                a += k2PiF;
            if ( a < 0.f )
                a += k2PiF;
            if ( a >= k2PiF )
                a -= k2PiF;
            if ( a >= k2PiF )
                a -= k2PiF;
            return a;
        }

        __device__ __forceinline__ Circ circ_of( float4 k )
        {
            Circ         C;
            C.w            = F3( k.x, k.y, k.z );
            C.c            = k.w;
            C.s            = sqrtf( fmaxf( 0.f, ( 1.f - k.w ) * ( 1.f + k.w ) ) );
            const float ax = fabsf( k.x ), ay = fabsf( k.y ), az = fabsf( k.z );
            const f3    t  = ( ax <= ay && ax <= az ) ? F3( 1.f, 0.f, 0.f ) : ( ay <= az ? F3( 0.f, 1.f, 0.f ) : F3( 0.f, 0.f, 1.f ) );
            C.e1           = normalize( cross( C.w, t ) );
            C.e2           = cross( C.w, C.e1 );
            return C;
        }

        // y . w <= 0 bounding lune L (side 0: the plane at 2 pi L / 3, side 1: the next one)
        __device__ __forceinline__ float4 lune_cons( int L, int side )
        {
            float sn, cs;
            sincosf( ( k2PiF / 3.f ) * (float)( L + side ), &sn, &cs );
            return side == 0 ? make_float4( sn, -cs, 0.f, 0.f ) : make_float4( -sn, cs, 0.f, 0.f );
        }

        // Forbidden arc of circle C under constraint k: 0 none, 1 [start, start + len), 2 all of it.
        __device__ __forceinline__ int cut_of( const Circ & C, float4 k, float & start, float & len )
        {
            if ( !( k.w < 1.f ) )
                return 0;
            const f3    wn  = F3( k.x, k.y, k.z );
            const float p1  = dot( C.e1, wn ), p2 = dot( C.e2, wn );
            const float B   = C.s * sqrtf( p1 * p1 + p2 * p2 );
            const float rhs = k.w - C.c * dot( C.w, wn );
            if ( !( B > fabsf( rhs ) ) )
                return rhs < 0.f ? 2 : 0;
            const float delta = atan2f( sqrtf( ( B - rhs ) * ( B + rhs ) ), rhs );
            start             = wrapf( atan2f( p2, p1 ) - delta );
            len               = 2.f * delta;
            return 1;
        }

        __device__ __forceinline__ f3 point_at( const Circ & C, float phi )
        {
            float sn, cs;
            sincosf( phi, &sn, &cs );
            return C.w * C.c + ( C.e1 * cs + C.e2 * sn ) * C.s;
        }

        // Cuts of one circle: start, length, constraint, rounded end, re-measured length.
        struct Cuts
        {
            float    s[ kAreaIv ], l[ kAreaIv ], ev[ kAreaIv ], el[ kAreaIv ];
            uint16_t n[ kAreaIv ];
            int      count;
        };

        // frame field xi(y) = a - (a . y) y, singular only at +-a (a generic direction)
        __device__ __forceinline__ float frame_angle( f3 y, f3 t )
        {
            const f3    a  = F3( 0.32140077f, 0.55410134f, 0.76790185f );
            const float ay = dot( a, y );
            const f3    xi = a - y * ay;
            return atan2f( dot( cross( xi, t ), y ), dot( xi, t ) );
        }

        // tangent-angle change against the frame field along the arc [st, st + ln] of C,
        // traversed with the region on its left (decreasing phi: the cap lies towards w)
        __device__ __forceinline__ float arc_turn( const Circ & C, float st, float ln )
        {
            float s0, c0, s1, c1;
            sincosf( st + ln, &s0, &c0 );
            sincosf( st, &s1, &c1 );
            const f3 y0 = C.w * C.c + ( C.e1 * c0 + C.e2 * s0 ) * C.s, t0 = C.e1 * s0 - C.e2 * c0;
            const f3 y1 = C.w * C.c + ( C.e1 * c1 + C.e2 * s1 ) * C.s, t1 = C.e1 * s1 - C.e2 * c1;
            return frame_angle( y1, t1 ) - frame_angle( y0, t0 );
        }

        // Walks the allowed arcs (gaps between the cuts) of circle C; calls
        // on_arc(start, length, na, nb) for each (na, nb: the constraints whose cuts
        // bound it, -1 for a whole circle) and returns the circle's Gauss-Bonnet terms:
        // c dphi plus the frame-relative tangent turn of every arc. Corners need no
        // partner: the arcs that meet at a corner share its point, so their frame
        // angles add up to its turning angle. An end strictly inside another cut is
        // covered (lengths re-measured from the rounded ends, so that equal ends
        // compare equal); of equal uncovered ends the first one counts.
        template<class OnArc>
        __device__ float circle_arcs( const Circ & C, Cuts & X, OnArc on_arc )
        {
            const int nIv = X.count;
            if ( nIv == 0 )
            {
                on_arc( 0.f, k2PiF, -1, -1 );
                return C.c * k2PiF;
            }
            for ( int q = 0; q < nIv; q++ )
            {
                X.ev[ q ]        = wrapf( X.s[ q ] + X.l[ q ] );
                const float len2 = wrapf( X.ev[ q ] - X.s[ q ] );
                X.el[ q ]        = len2 >= 0.5f * X.l[ q ] ? len2 : X.l[ q ];
            }
            float total = 0.f;
            for ( int a = 0; a < nIv; a++ )
            {
                const float end  = X.ev[ a ];
                bool        skip = false;
                for ( int b = 0; b < nIv && !skip; b++ )
                    skip = b != a && wrapf( end - X.s[ b ] ) < X.el[ b ];
                if ( skip )
                    continue;
                // an equal end of an earlier uncovered cut already walks this gap
                for ( int b = 0; b < a && !skip; b++ )
                {
                    if ( X.ev[ b ] != end )
                        continue;
                    bool covb = false;
                    for ( int q = 0; q < nIv && !covb; q++ )
                        covb = q != b && wrapf( X.ev[ b ] - X.s[ q ] ) < X.el[ q ];
                    skip = !covb;
                }
                if ( skip )
                    continue;
                float gap = k2PiF;
                int   nb  = -1;
                for ( int b = 0; b < nIv; b++ )
                {
                    const float g = wrapf( X.s[ b ] - end );
                    if ( g > 0.f && ( nb < 0 || g < gap ) )
                    {
                        gap = g;
                        nb  = b;
                    }
                }
                if ( nb < 0 )
                    continue;
                total += C.c * gap + arc_turn( C, end, gap );
                on_arc( end, gap, (int)X.n[ a ], (int)X.n[ nb ] );
            }
            return total;
        }

        // Cuts of one lune-plane circle, shared by the warp.
        struct WarpCuts
        {
            float    s[ kLuneIv ], l[ kLuneIv ], ev[ kLuneIv ], el[ kLuneIv ];
            uint8_t  unc[ kLuneIv ];
        };

        // circle_arcs for a circle whose cuts are in shared memory, with the cuts
        // spread over the lanes; returns this lane's part of the Gauss-Bonnet terms
        __device__ float circle_arcs_warp( const Circ & C, WarpCuts & W, int count )
        {
            const int lane = (int)lane_id();
            if ( count == 0 )
                return lane == 0 ? C.c * k2PiF : 0.f;
            for ( int q = lane; q < count; q += 32 )
            {
                W.ev[ q ]        = wrapf( W.s[ q ] + W.l[ q ] );
                const float len2 = wrapf( W.ev[ q ] - W.s[ q ] );
                W.el[ q ]        = len2 >= 0.5f * W.l[ q ] ? len2 : W.l[ q ];
            }
            __syncwarp();
            for ( int a = lane; a < count; a += 32 )
            {
                bool covered = false;
                for ( int b = 0; b < count && !covered; b++ )
                    covered = b != a && wrapf( W.ev[ a ] - W.s[ b ] ) < W.el[ b ];
                W.unc[ a ] = !covered;
            }
            __syncwarp();
            float total = 0.f;
            for ( int a = lane; a < count; a += 32 )
            {
                if ( !W.unc[ a ] )
                    continue;
                const float end = W.ev[ a ];
                bool        dup = false;
                for ( int b = 0; b < a && !dup; b++ )
                    dup = W.unc[ b ] && W.ev[ b ] == end;
                if ( dup )
                    continue;
                float gap = k2PiF;
                bool  any = false;
                for ( int b = 0; b < count; b++ )
                {
                    const float g = wrapf( W.s[ b ] - end );
                    if ( g > 0.f && ( !any || g < gap ) )
                    {
                        gap = g;
                        any = true;
                    }
                }
                if ( any )
                    total += C.c * gap + arc_turn( C, end, gap );
            }
            __syncwarp();
            return total;
        }

        // One region of the unit sphere, held by a warp: constraints cons[0, M) in
        // shared memory; each lane takes circles m = lane, lane + 32, ...; the three
        // lunes add their two planes. per_arc(m, C, start, len, na, nb) is called for
        // every allowed arc of an original circle. Returns the area (all lanes).
        template<class PerArc>
        __device__ float region_area_warp( const float4 * cons, int M, WarpCuts & W, uint32_t & overflow, PerArc per_arc )
        {
            const uint32_t lane = lane_id();
            float          tot[ 3 ] = { 0.f, 0.f, 0.f };
            bool           empty    = false;
            for ( int m = (int)lane; m < M; m += 32 )
                if ( !( cons[ m ].w > -1.f ) )
                    empty = true;
            if ( __any_sync( 0xffffffffu, empty ) )
                return 0.f;
            Cuts X;
            // the original circles, each over the three lunes
            for ( int m = (int)lane; m < M; m += 32 )
            {
                const float4 km = cons[ m ];
                if ( !( km.w < 1.f ) )
                    continue;
                const Circ C    = circ_of( km );
                bool       gone = false;
                int        nIv  = 0;
                for ( int n = 0; n < M && !gone; n++ )
                {
                    if ( n == m )
                        continue;
                    const float4 kn = cons[ n ];
                    if ( kn.x == km.x && kn.y == km.y && kn.z == km.z && kn.w == km.w )
                    {
                        gone = n < m; // the same constraint twice: the first keeps the circle
                        continue;
                    }
                    float      st, ln;
                    const int  r = cut_of( C, kn, st, ln );
                    if ( r == 2 )
                        gone = true;
                    else if ( r == 1 )
                    {
                        if ( nIv < kAreaIv - 2 )
                        {
                            X.s[ nIv ] = st, X.l[ nIv ] = ln, X.n[ nIv ] = (uint16_t)n;
                            nIv++;
                        }
                        else
                            overflow = 1;
                    }
                }
                if ( gone )
                    continue;
                for ( int L = 0; L < 3; L++ )
                {
                    X.count = nIv;
                    bool out = false;
                    for ( int side = 0; side < 2; side++ )
                    {
                        float     st, ln;
                        const int r = cut_of( C, lune_cons( L, side ), st, ln );
                        if ( r == 2 )
                            out = true;
                        else if ( r == 1 )
                        {
                            X.s[ X.count ] = st, X.l[ X.count ] = ln, X.n[ X.count ] = (uint16_t)( M + side );
                            X.count++;
                        }
                    }
                    if ( out )
                        continue;
                    tot[ L ] += circle_arcs( C, X, [ & ]( float st, float ln, int na, int nb ) { per_arc( m, C, st, ln, na, nb ); } );
                }
            }
            // the lune planes: six circles, one after another, each over the whole warp
            for ( int lc = 0; lc < 6; lc++ )
            {
                const int  L = lc >> 1, side = lc & 1;
                const Circ C    = circ_of( lune_cons( L, side ) );
                bool       gone = false;
                int        nIv  = 0;
                for ( int n0 = 0; n0 <= M; n0 += 32 )
                {
                    const int n = n0 + (int)lane;
                    float     st = 0.f, ln = 0.f;
                    int       r  = 0;
                    if ( n <= M )
                        r = cut_of( C, n < M ? cons[ n ] : lune_cons( L, 1 - side ), st, ln );
                    gone |= r == 2;
                    const uint32_t mk  = __ballot_sync( 0xffffffffu, r == 1 );
                    const int      pos = nIv + __popc( mk & lanemask_lt() );
                    if ( r == 1 && pos < kLuneIv )
                    {
                        W.s[ pos ] = st;
                        W.l[ pos ] = ln;
                    }
                    nIv += __popc( mk );
                }
                if ( nIv > kLuneIv )
                {
                    overflow = 1;
                    nIv      = kLuneIv;
                }
                __syncwarp();
                if ( !__any_sync( 0xffffffffu, gone ) )
                    tot[ L ] += circle_arcs_warp( C, W, nIv );
                __syncwarp();
            }
            float area = 0.f;
            for ( int L = 0; L < 3; L++ )
            {
                float t = tot[ L ];
                for ( int o = 16; o > 0; o >>= 1 )
                    t += __shfl_xor_sync( 0xffffffffu, t, o );
                // the sum spans many turns: reduce it with a full modulo
                float r = fmodf( t, k2PiF );
                if ( r < 0.f )
                    r += k2PiF;
                if ( r > 5.f * kPiF / 3.f )
                    r -= k2PiF; // a piece of (nearly) zero area
                area += fmaxf( r, 0.f );
            }
            return area;
        }

        // integral of y over the arc [st, st + ln] of C
        __device__ __forceinline__ f3 arc_integral( const Circ & C, float st, float ln )
        {
            float s0, c0, s1, c1;
            sincosf( st, &s0, &c0 );
            sincosf( st + ln, &s1, &c1 );
            return C.w * ( C.c * ln ) + ( C.e1 * ( s1 - s0 ) - C.e2 * ( c1 - c0 ) ) * C.s;
        }

        // Pair constraint of atom i and neighbour j: w = D / d, c = (R_i^2 - R_j^2 + d^2) / (2 d R_i).
        struct PairGeo
        {
            f3    D;
            float d, Ri, Rj;
        };
        __device__ __forceinline__ float4 pair_cons( const PairGeo & p )
        {
            if ( !( p.d > 0.f ) )
                return make_float4( 0.f, 0.f, 1.f, 2.f ); // coincident centres: ignored
            const f3 w = p.D * ( 1.f / p.d );
            return make_float4( w.x, w.y, w.z, ( p.Ri * p.Ri - p.Rj * p.Rj + p.d * p.d ) / ( 2.f * p.d * p.Ri ) );
        }

        // toroidal patch per unit angle (rp times the integral of max(0, rho - rp cos beta)
        // over [beta_i, beta_j]) and its derivatives by (d, R_i, R_j)
        __device__ __forceinline__ float torus_F( float d, float Ri, float Rj, float rp, float dF[ 3 ] )
        {
            const float hi = ( Ri * Ri - Rj * Rj + d * d ) / ( 2.f * d ), hj = d - hi;
            const float rr = Ri * Ri - hi * hi;
            dF[ 0 ] = dF[ 1 ] = dF[ 2 ] = 0.f;
            if ( !( rr > 0.f ) )
                return 0.f;
            const float rho = sqrtf( rr );
            const float bi = -atan2f( hi, rho ), bj = atan2f( hj, rho );
            float       F  = rho * ( bj - bi ) - rp * ( hj / Rj + hi / Ri );
            float       Fr = ( bj - bi ) - rho * ( hj / ( Rj * Rj ) + hi / ( Ri * Ri ) )
                       + rp * rho * ( hj / ( Rj * Rj * Rj ) + hi / ( Ri * Ri * Ri ) );
            const float Fhi = ( rho * rho / ( Ri * Ri ) ) * ( 1.f - rp / Ri );
            const float Fhj = ( rho * rho / ( Rj * Rj ) ) * ( 1.f - rp / Rj );
            if ( rho < rp && hi > 0.f && hj > 0.f )
            {
                const float b0 = acosf( rho / rp );
                F -= 2.f * rho * b0 - 2.f * rp * sqrtf( ( 1.f - rho / rp ) * ( 1.f + rho / rp ) );
                Fr -= 2.f * b0;
            }
            const float rd = -hi * hj / ( d * rho ), rRi = Ri * hj / ( d * rho ), rRj = Rj * hi / ( d * rho );
            dF[ 0 ] = rp * ( Fr * rd + Fhi * ( hj / d ) + Fhj * ( hi / d ) );
            dF[ 1 ] = rp * ( Fr * rRi + Fhi * ( Ri / d ) - Fhj * ( Ri / d ) );
            dF[ 2 ] = rp * ( Fr * rRj - Fhi * ( Rj / d ) + Fhj * ( Rj / d ) );
            return rp * F;
        }

        __device__ __forceinline__ void add4( float * g, uint32_t a, f3 v, float r )
        {
            atomicAdd( g + 4 * (size_t)a + 0, v.x );
            atomicAdd( g + 4 * (size_t)a + 1, v.y );
            atomicAdd( g + 4 * (size_t)a + 2, v.z );
            if ( r != 0.f )
                atomicAdd( g + 4 * (size_t)a + 3, r );
        }

        // Pair constraint (w, c) of atom i and neighbour atom j in double precision, from the float32 atoms.
        __device__ __forceinline__ void pair_cons_d( float4 ai, float4 aj, double rp, d3 & w, double & c )
        {
            const d3     D  = D3( (double)aj.x - (double)ai.x, (double)aj.y - (double)ai.y, (double)aj.z - (double)ai.z );
            const double d  = sqrt( ddot( D, D ) );
            const double Ri = (double)ai.w + rp, Rj = (double)aj.w + rp;
            w               = dmul( D, 1.0 / d );
            c               = ( Ri * Ri - Rj * Rj + d * d ) / ( 2.0 * d * Ri );
        }

        // Angle part of the torus of circle m at one arc end where circle m crosses the plane of
        // constraint nn at a small angle (|tw| small): there the end's float32 position, and so tw
        // and 1 / tw, carry rounding magnified by the shallow crossing. The end is taken again in
        // double precision as the point of circle m on that plane (the one on the side of the
        // float32 end), with both constraints recomputed from the atoms, and its terms are formed
        // in double precision (coef = Gs / tw; Gs = -G or G by the end): out = gc[nn], gw[nn],
        // gc[m], gw[m].
        __device__ __noinline__ void arc_end_terms_d( const Build & b, uint32_t i, uint32_t jm, uint32_t jn, f3 yf, float Gs,
                                                      double out[ 8 ] )
        {
            const float4 ai = b.atoms[ i ];
            d3           wm, wn;
            double       cm, cn;
            pair_cons_d( ai, b.atoms[ jm ], (double)b.rp, wm, cm );
            pair_cons_d( ai, b.atoms[ jn ], (double)b.rp, wn, cn );
            const double g   = ddot( wm, wn );
            const double den = 1.0 - g * g;
            for ( int k = 0; k < 8; k++ )
                out[ k ] = 0.0;
            if ( !( den > 0.0 ) )
                return;
            const double al = ( cm - g * cn ) / den, be = ( cn - g * cm ) / den;
            const d3     nv = dcross( wm, wn );
            double       g2 = ( 1.0 - ( al * al + be * be + 2.0 * al * be * g ) ) / den;
            g2              = g2 > 0.0 ? g2 : 0.0;
            const double ga = ( (double)yf.x * nv.x + (double)yf.y * nv.y + (double)yf.z * nv.z ) < 0.0 ? -sqrt( g2 ) : sqrt( g2 );
            const d3     y  = dadd( dadd( dmul( wm, al ), dmul( wn, be ) ), dmul( nv, ga ) );
            const d3     yc = dsub( y, dmul( wm, cm ) );
            const double tw = ddot( dcross( wm, yc ), wn );
            if ( !( fabs( tw ) > 0.0 ) )
                return;
            const double coef = (double)Gs / tw;
            const double sm2  = 1.0 - cm * cm;
            out[ 0 ]          = coef;
            out[ 1 ] = -coef * y.x, out[ 2 ] = -coef * y.y, out[ 3 ] = -coef * y.z;
            out[ 4 ]          = -coef * ( g - ( cm / sm2 ) * ddot( yc, wn ) );
            const d3 gwm      = dmul( dsub( dmul( wn, cm ), dmul( yc, g ) ), -coef );
            out[ 5 ] = gwm.x, out[ 6 ] = gwm.y, out[ 7 ] = gwm.z;
        }

        struct AreaSmem
        {
            float4 cons[ kAreaNbr ];
            float  dphi[ kAreaNbr ];
            float4 iy[ kAreaNbr ];
            float  gc[ kAreaNbr ];
            float4 gw[ kAreaNbr ];
            float  dist[ kAreaNbr ];
            float  Rn[ kAreaNbr ];
            WarpCuts cuts;
        };

        // Warp per atom: convex patch and the tori of its circles (i, j), i < j.
        // parts (double[3]) accumulate convex, toroidal (and concave in k_area_probes);
        // atomArea (input order) receives convex + half of each torus. With kGrad,
        // gradSorted (float4 per sorted atom) accumulates gConvex d convex + gTorus d tori.
        template<bool kGrad>
        __global__ void __launch_bounds__( 32 * kAreaWarps ) k_area_atoms( Build b, double * parts, float * atomArea,
                                                                             float gConvex, float gTorus, float * gradSorted )
        {
            __shared__ AreaSmem sm[ kAreaWarps ];
            const uint32_t      warp = threadIdx.x >> 5, lane = lane_id();
            AreaSmem &          S    = sm[ warp ];
            double              convexSum = 0.0, torusSum = 0.0;
            uint32_t            overflow = 0;
            for ( uint32_t i = blockIdx.x * kAreaWarps + warp; i < b.n; i += gridDim.x * kAreaWarps )
            {
                const float4   ai = b.atoms[ i ];
                const float    Ri = ai.w + b.rp, ri = ai.w;
                const uint32_t ni = b.nbrCount[ i ];
                const size_t   row = (size_t)i * b.cap;
                // an atom whose circles are all buried has no accessible patch
                bool open = false;
                for ( uint32_t s = lane; s < ni; s += 32 )
                    open |= b.status[ row + s ] != 0;
                if ( ni > 0 && !__any_sync( 0xffffffffu, open ) )
                    continue;
                if ( ni > (uint32_t)kAreaNbr )
                {
                    overflow = 1;
                    continue;
                }
                const int M = (int)ni;
                for ( int m = (int)lane; m < M; m += 32 )
                {
                    const float4 aj = b.atoms[ b.nbr[ row + m ] ];
                    PairGeo      p;
                    p.D          = F3( aj.x - ai.x, aj.y - ai.y, aj.z - ai.z );
                    p.d          = sqrtf( dot( p.D, p.D ) );
                    p.Ri         = Ri;
                    p.Rj         = aj.w + b.rp;
                    S.cons[ m ]  = pair_cons( p );
                    S.dist[ m ]  = p.d;
                    S.Rn[ m ]    = p.Rj;
                    S.dphi[ m ]  = 0.f;
                    S.iy[ m ]    = make_float4( 0.f, 0.f, 0.f, 0.f );
                    S.gc[ m ]    = 0.f;
                    S.gw[ m ]    = make_float4( 0.f, 0.f, 0.f, 0.f );
                }
                __syncwarp();
                const float U = region_area_warp( S.cons, M, S.cuts, overflow, [ & ]( int m, const Circ & C, float st, float ln, int na, int nb ) {
                    // the lane that owns circle m is the only writer of its sums
                    S.dphi[ m ] += ln;
                    if ( !kGrad )
                        return;
                    const f3 I = arc_integral( C, st, ln );
                    S.iy[ m ].x += I.x, S.iy[ m ].y += I.y, S.iy[ m ].z += I.z;
                    const uint32_t j = b.nbr[ row + m ];
                    if ( !( j > i ) || !( S.dist[ m ] > 0.f ) )
                        return;
                    // angle part of the torus of (i, j): its arc ends move with the circles
                    float       dF[ 3 ];
                    const float G = gTorus * torus_F( S.dist[ m ], Ri, S.Rn[ m ], b.rp, dF );
                    for ( int e = 0; e < 2; e++ )
                    {
                        const int nn = e == 0 ? na : nb;
                        if ( nn < 0 || nn >= M )
                            continue; // whole circle, or a cut between lunes
                        const float  phi = e == 0 ? st : st + ln;
                        const f3     y   = point_at( C, phi );
                        const f3     yc  = y - C.w * C.c;
                        const float4 kn  = S.cons[ nn ];
                        const f3     wn  = F3( kn.x, kn.y, kn.z );
                        const float  tw  = dot( cross( C.w, yc ), wn );
                        if ( fabsf( tw ) < kShallowCrossing )
                        {
                            double t[ 8 ];
                            arc_end_terms_d( b, i, j, b.nbr[ row + nn ], y, e == 0 ? -G : G, t );
                            atomicAdd( &S.gc[ nn ], (float)t[ 0 ] );
                            atomicAdd( &S.gw[ nn ].x, (float)t[ 1 ] );
                            atomicAdd( &S.gw[ nn ].y, (float)t[ 2 ] );
                            atomicAdd( &S.gw[ nn ].z, (float)t[ 3 ] );
                            atomicAdd( &S.gc[ m ], (float)t[ 4 ] );
                            atomicAdd( &S.gw[ m ].x, (float)t[ 5 ] );
                            atomicAdd( &S.gw[ m ].y, (float)t[ 6 ] );
                            atomicAdd( &S.gw[ m ].z, (float)t[ 7 ] );
                            continue;
                        }
                        const float coef = ( e == 0 ? -G : G ) / tw;
                        const float wwn  = dot( C.w, wn );
                        atomicAdd( &S.gc[ nn ], coef );
                        atomicAdd( &S.gw[ nn ].x, -coef * y.x );
                        atomicAdd( &S.gw[ nn ].y, -coef * y.y );
                        atomicAdd( &S.gw[ nn ].z, -coef * y.z );
                        const f3 gwm = ( wn * C.c - yc * wwn ) * ( -coef );
                        atomicAdd( &S.gc[ m ], -coef * ( wwn - ( C.c / ( C.s * C.s ) ) * dot( yc, wn ) ) );
                        atomicAdd( &S.gw[ m ].x, gwm.x );
                        atomicAdd( &S.gw[ m ].y, gwm.y );
                        atomicAdd( &S.gw[ m ].z, gwm.z );
                    }
                } );
                __syncwarp();
                float mine = 0.f, tori = 0.f;
                f3    gi   = F3( 0.f, 0.f, 0.f );
                float gRi  = 0.f;
                for ( int m = (int)lane; m < M; m += 32 )
                {
                    const uint32_t j = b.nbr[ row + m ];
                    if ( j > i && S.dphi[ m ] > 0.f && S.dist[ m ] > 0.f )
                    {
                        float       dF[ 3 ];
                        const float F = torus_F( S.dist[ m ], Ri, S.Rn[ m ], b.rp, dF );
                        const float T = F * S.dphi[ m ];
                        tori += T;
                        mine += 0.5f * T;
                        if ( atomArea )
                            atomicAdd( atomArea + b.perm[ j ], 0.5f * T );
                        if ( kGrad )
                        {
                            const float4 k  = S.cons[ m ];
                            const f3     w  = F3( k.x, k.y, k.z );
                            const float  gs = gTorus * S.dphi[ m ];
                            add4( gradSorted, j, w * ( gs * dF[ 0 ] ), gs * dF[ 2 ] );
                            gi  = gi - w * ( gs * dF[ 0 ] );
                            gRi += gs * dF[ 1 ];
                        }
                    }
                    if ( kGrad && S.dist[ m ] > 0.f )
                    {
                        // convex part and the angle parts gathered above, through (w, c) of the pair
                        const float4 k   = S.cons[ m ];
                        const f3     w   = F3( k.x, k.y, k.z );
                        const float  d   = S.dist[ m ], Rj = S.Rn[ m ];
                        const float  gc  = S.gc[ m ] + gConvex * ri * ri * S.dphi[ m ];
                        const f3     gw  = F3( S.gw[ m ].x, S.gw[ m ].y, S.gw[ m ].z ) - F3( S.iy[ m ].x, S.iy[ m ].y, S.iy[ m ].z ) * ( gConvex * ri * ri );
                        const float  dcd = 1.f / ( 2.f * Ri ) - ( Ri * Ri - Rj * Rj ) / ( 2.f * d * d * Ri );
                        const float  dcRi = ( Ri * Ri + Rj * Rj - d * d ) / ( 2.f * d * Ri * Ri );
                        const float  dcRj = -Rj / ( d * Ri );
                        const f3     gD   = ( gw - w * dot( gw, w ) ) * ( 1.f / d ) + w * ( gc * dcd );
                        add4( gradSorted, j, gD, gc * dcRj );
                        gi  = gi - gD;
                        gRi += gc * dcRi;
                    }
                }
                for ( int o = 16; o > 0; o >>= 1 )
                {
                    mine += __shfl_xor_sync( 0xffffffffu, mine, o );
                    tori += __shfl_xor_sync( 0xffffffffu, tori, o );
                    if ( kGrad )
                    {
                        gi.x += __shfl_xor_sync( 0xffffffffu, gi.x, o );
                        gi.y += __shfl_xor_sync( 0xffffffffu, gi.y, o );
                        gi.z += __shfl_xor_sync( 0xffffffffu, gi.z, o );
                        gRi += __shfl_xor_sync( 0xffffffffu, gRi, o );
                    }
                }
                const float cA = ri * ri * U;
                if ( lane == 0 )
                {
                    convexSum += cA;
                    torusSum += tori;
                    if ( atomArea )
                        atomicAdd( atomArea + b.perm[ i ], cA + mine );
                    if ( kGrad )
                        add4( gradSorted, i, gi, gRi + gConvex * 2.f * ri * U );
                }
                __syncwarp();
            }
            if ( lane == 0 )
            {
                if ( parts && convexSum != 0.0 )
                    atomicAdd( parts + 0, convexSum );
                if ( parts && torusSum != 0.0 )
                    atomicAdd( parts + 1, torusSum );
            }
            overflow = __any_sync( 0xffffffffu, overflow != 0 );
            if ( lane == 0 && overflow )
                atomicOr( &b.counts->overflow, (uint32_t)kOverflowArea );
        }

        // ---- double-precision twin of a probe region's adjoint ------------------------------
        // A neighbour probe closer than kCloseProbe makes a cap of nearly a hemisphere whose terms
        // go as 1 / L (L the distance of the two probes): the float32 arc integrals' rounding shows
        // there. Such a region's adjoint is taken again in double precision: the same constraints
        // from the float32 probe positions and atoms, every constraint's allowed arcs (the gaps
        // between its cuts by the others; the lune split of the area does not change their sums),
        // and the same terms as the float32 path.
        constexpr float kCloseProbe = 0.5f;

        struct dcons
        {
            double x, y, z, w;
        };
        __device__ __forceinline__ dcons dcons_of( double x, double y, double z, double w ) { return { x, y, z, w }; }

        __device__ __forceinline__ double wrap2pi_d( double a )
        {
            a = fmod( a, 2.0 * 3.14159265358979323846 );
            return a < 0.0 ? a + 2.0 * 3.14159265358979323846 : a;
        }

        // allowed-arc length and integral of y over constraint m of the region kd[0, M)
        __device__ void constraint_arcs_d( const dcons * kd, int M, int m, double & dphi, d3 & iy )
        {
            const double k2Pi = 2.0 * 3.14159265358979323846;
            dphi              = 0.0;
            iy                = D3( 0.0, 0.0, 0.0 );
            const double cm   = kd[ m ].w;
            if ( !( cm < 1.0 ) )
                return;
            const d3     wm = D3( kd[ m ].x, kd[ m ].y, kd[ m ].z );
            const double sm = sqrt( ( 1.0 - cm ) * ( 1.0 + cm ) );
            const double ax = fabs( wm.x ), ay = fabs( wm.y ), az = fabs( wm.z );
            const d3     t  = ( ax <= ay && ax <= az ) ? D3( 1.0, 0.0, 0.0 ) : ( ay <= az ? D3( 0.0, 1.0, 0.0 ) : D3( 0.0, 0.0, 1.0 ) );
            d3           e1 = dcross( wm, t );
            e1              = dmul( e1, 1.0 / sqrt( ddot( e1, e1 ) ) );
            const d3 e2     = dcross( wm, e1 );
            double   ivS[ kProbeCons ], ivL[ kProbeCons ], enV[ kProbeCons ], enL[ kProbeCons ];
            bool     unc[ kProbeCons ];
            int      nIv = 0;
            for ( int n = 0; n < M; n++ )
            {
                if ( n == m )
                    continue;
                const double cn = kd[ n ].w;
                if ( !( cn < 1.0 ) )
                    continue;
                const d3 wn = D3( kd[ n ].x, kd[ n ].y, kd[ n ].z );
                if ( wn.x == wm.x && wn.y == wm.y && wn.z == wm.z && cn == cm )
                {
                    if ( n < m )
                        return; // the same constraint twice: the first one keeps the circle
                    continue;
                }
                const double p1 = ddot( e1, wn ), p2 = ddot( e2, wn );
                const double B = sm * sqrt( p1 * p1 + p2 * p2 ), rhs = cn - cm * ddot( wm, wn );
                if ( !( B > fabs( rhs ) ) )
                {
                    if ( rhs < 0.0 )
                        return; // the whole circle lies inside cap n
                    continue;
                }
                const double delta = atan2( sqrt( ( B - rhs ) * ( B + rhs ) ), rhs );
                ivS[ nIv ]         = wrap2pi_d( atan2( p2, p1 ) - delta );
                ivL[ nIv ]         = 2.0 * delta;
                nIv++;
            }
            if ( nIv == 0 )
            {
                dphi = k2Pi;
                iy   = dmul( wm, cm * k2Pi );
                return;
            }
            for ( int q = 0; q < nIv; q++ )
            {
                enV[ q ]          = wrap2pi_d( ivS[ q ] + ivL[ q ] );
                const double len2 = wrap2pi_d( enV[ q ] - ivS[ q ] );
                enL[ q ]          = len2 >= 0.5 * ivL[ q ] ? len2 : ivL[ q ];
            }
            for ( int a = 0; a < nIv; a++ )
            {
                unc[ a ] = true;
                for ( int c = 0; c < nIv && unc[ a ]; c++ )
                    if ( c != a && wrap2pi_d( enV[ a ] - ivS[ c ] ) < enL[ c ] )
                        unc[ a ] = false;
            }
            for ( int a = 0; a < nIv; a++ )
            {
                if ( !unc[ a ] )
                    continue;
                const double end = enV[ a ];
                bool         dup = false;
                for ( int c = 0; c < a && !dup; c++ )
                    dup = unc[ c ] && enV[ c ] == end;
                if ( dup )
                    continue;
                double gap = k2Pi;
                bool   any = false;
                for ( int c = 0; c < nIv; c++ )
                {
                    const double g = wrap2pi_d( ivS[ c ] - end );
                    if ( g > 0.0 && ( !any || g < gap ) )
                    {
                        gap = g;
                        any = true;
                    }
                }
                if ( !any )
                    continue;
                dphi += gap;
                const double c0 = cos( end ), s0 = sin( end ), c1 = cos( end + gap ), s1 = sin( end + gap );
                iy = dadd( iy, dadd( dmul( wm, cm * gap ), dmul( dsub( dmul( e1, s1 - s0 ), dmul( e2, c1 - c0 ) ), sm ) ) );
            }
        }

        // The warp's probe p (a region with a nearly coincident neighbour): its adjoint terms in
        // double precision into gradSorted (contact directions) and probeGrad (probe positions).
        // kd, sums: shared memory of kProbeCons entries each.
        __device__ __noinline__ void probe_region_grad_d( const Build & b, uint32_t p, float gConcave, float * gradSorted,
                                                          float4 * probeGrad, dcons * kd, dcons * sums )
        {
            const uint32_t lane = lane_id();
            const double   rp   = (double)b.rp;
            const int4     id   = b.probeIds[ p ];
            const float4   pf   = b.probePos[ p ];
            const d3       P    = D3( (double)pf.x, (double)pf.y, (double)pf.z );
            const int      ia[ 3 ] = { id.x, id.y, id.z };
            d3             v[ 3 ];
            double         Lv[ 3 ];
            for ( int a = 0; a < 3; a++ )
            {
                const float4 c = b.atoms[ ia[ a ] ];
                const d3     D = D3( (double)c.x - P.x, (double)c.y - P.y, (double)c.z - P.z );
                Lv[ a ]        = sqrt( ddot( D, D ) );
                v[ a ]         = dmul( D, 1.0 / Lv[ a ] );
            }
            d3     u[ 3 ];
            double ul[ 3 ], sg[ 3 ];
            bool   flat = false;
            for ( int e = 0; e < 3; e++ )
            {
                u[ e ]            = dcross( v[ e ], v[ ( e + 1 ) % 3 ] );
                ul[ e ]           = sqrt( ddot( u[ e ], u[ e ] ) );
                const double side = ddot( u[ e ], v[ ( e + 2 ) % 3 ] );
                flat |= !( ul[ e ] > 0.0 ) || side == 0.0;
                sg[ e ] = side > 0.0 ? 1.0 : -1.0;
            }
            if ( flat )
                return; // a flat triangle has no area
            const uint32_t Q   = min( b.counts->Q, b.capProbes );
            const uint32_t cnt = p < Q ? min( (uint32_t)id.w, kMaxProbeNbr ) : 0u;
            const int      M   = 3 + (int)cnt;
            if ( lane < 3 )
            {
                const d3 w  = dmul( u[ lane ], -sg[ lane ] / ul[ lane ] );
                kd[ lane ] = dcons_of( w.x, w.y, w.z, 0.0 );
            }
            uint32_t q = 0;
            double   L = 0.0;
            if ( lane < cnt )
            {
                q               = b.probeNbrIdx[ (size_t)p * kMaxProbeNbr + lane ];
                const float4 pq = b.probePos[ q ];
                const d3     D  = D3( (double)pq.x - P.x, (double)pq.y - P.y, (double)pq.z - P.z );
                L               = sqrt( ddot( D, D ) );
                kd[ 3 + lane ]  = L > 0.0 && L < 2.0 * rp ? dcons_of( D.x / L, D.y / L, D.z / L, L / ( 2.0 * rp ) )
                                                          : dcons_of( 0.0, 0.0, 1.0, 2.0 ); // vacuous
            }
            __syncwarp();
            for ( int m = (int)lane; m < M; m += 32 )
            {
                double dphi;
                d3     iy;
                constraint_arcs_d( kd, M, m, dphi, iy );
                sums[ m ] = dcons_of( iy.x, iy.y, iy.z, dphi );
            }
            __syncwarp();
            const double k2 = (double)gConcave * rp * rp;
            d3           gP = D3( 0.0, 0.0, 0.0 );
            if ( lane == 0 )
            {
                d3 gv[ 3 ] = { D3( 0.0, 0.0, 0.0 ), D3( 0.0, 0.0, 0.0 ), D3( 0.0, 0.0, 0.0 ) };
                for ( int e = 0; e < 3; e++ )
                {
                    const d3  gw = dmul( D3( sums[ e ].x, sums[ e ].y, sums[ e ].z ), -k2 );
                    const d3  wh = dmul( u[ e ], 1.0 / ul[ e ] );
                    const d3  gu = dmul( dsub( gw, dmul( wh, ddot( gw, wh ) ) ), -sg[ e ] / ul[ e ] );
                    const int a = e, c2 = ( e + 1 ) % 3;
                    gv[ a ]     = dadd( gv[ a ], dcross( v[ c2 ], gu ) );
                    gv[ c2 ]    = dadd( gv[ c2 ], dcross( gu, v[ a ] ) );
                }
                for ( int a = 0; a < 3; a++ )
                {
                    const d3 gD = dmul( dsub( gv[ a ], dmul( v[ a ], ddot( gv[ a ], v[ a ] ) ) ), 1.0 / Lv[ a ] );
                    add4( gradSorted, (uint32_t)ia[ a ], F3( (float)gD.x, (float)gD.y, (float)gD.z ), 0.f );
                    gP = dsub( gP, gD );
                }
            }
            if ( lane < cnt && L > 0.0 && L < 2.0 * rp )
            {
                const int    m  = 3 + (int)lane;
                const d3     w  = D3( kd[ m ].x, kd[ m ].y, kd[ m ].z );
                const d3     gw = dmul( D3( sums[ m ].x, sums[ m ].y, sums[ m ].z ), -k2 );
                const double gc = k2 * sums[ m ].w;
                const d3     gD = dadd( dmul( dsub( gw, dmul( w, ddot( gw, w ) ) ), 1.0 / L ), dmul( w, gc / ( 2.0 * rp ) ) );
                gP              = dsub( gP, gD );
                atomicAdd( &probeGrad[ q ].x, (float)gD.x );
                atomicAdd( &probeGrad[ q ].y, (float)gD.y );
                atomicAdd( &probeGrad[ q ].z, (float)gD.z );
            }
            for ( int o = 16; o > 0; o >>= 1 )
            {
                gP.x += __shfl_xor_sync( 0xffffffffu, gP.x, o );
                gP.y += __shfl_xor_sync( 0xffffffffu, gP.y, o );
                gP.z += __shfl_xor_sync( 0xffffffffu, gP.z, o );
            }
            if ( lane == 0 )
            {
                atomicAdd( &probeGrad[ p ].x, (float)gP.x );
                atomicAdd( &probeGrad[ p ].y, (float)gP.y );
                atomicAdd( &probeGrad[ p ].z, (float)gP.z );
            }
            __syncwarp();
        }

        struct ProbeAreaSmem
        {
            dcons kd[ kProbeCons ];   // constraints of a region taken in double precision
            dcons sums[ kProbeCons ]; // and their allowed-arc integrals and lengths
            float4 cons[ kProbeCons ];
            float  dphi[ kProbeCons ];
            float4 iy[ kProbeCons ];
            float  dist[ kProbeCons ];
            uint32_t nq[ kProbeCons ];
            WarpCuts cuts;
        };

        // Warp per probe: its concave triangle outside the listed neighbour probes.
        // With kGrad, probeGrad (float4 per probe) accumulates d/d(position) of every
        // probe involved and gradSorted the direct terms of the contact directions.
        template<bool kGrad>
        __global__ void __launch_bounds__( 32 * kAreaWarps ) k_area_probes( Build b, double * parts, float * atomArea,
                                                                              float gConcave, float * gradSorted, float4 * probeGrad )
        {
            __shared__ ProbeAreaSmem sm[ kAreaWarps ];
            const uint32_t           warp = threadIdx.x >> 5, lane = lane_id();
            ProbeAreaSmem &          S    = sm[ warp ];
            const uint32_t           I    = min( b.counts->I, b.capProbes );
            const uint32_t           Q    = min( b.counts->Q, b.capProbes );
            const float              rp   = b.rp;
            double                   concaveSum = 0.0;
            uint32_t                 overflow   = 0;
            for ( uint32_t p = blockIdx.x * kAreaWarps + warp; p < I; p += gridDim.x * kAreaWarps )
            {
                const int4   id = b.probeIds[ p ];
                const float4 pp = b.probePos[ p ];
                const f3     P  = F3( pp.x, pp.y, pp.z );
                f3           v[ 3 ];
                float        Lv[ 3 ];
                const int    ia[ 3 ] = { id.x, id.y, id.z };
                for ( int a = 0; a < 3; a++ )
                {
                    const float4 c = b.atoms[ ia[ a ] ];
                    const f3     D = F3( c.x - P.x, c.y - P.y, c.z - P.z );
                    Lv[ a ]        = sqrtf( dot( D, D ) );
                    v[ a ]         = D * ( 1.f / Lv[ a ] );
                }
                f3    u[ 3 ];
                float ul[ 3 ], sg[ 3 ];
                bool  flat = false;
                for ( int e = 0; e < 3; e++ )
                {
                    u[ e ]           = cross( v[ e ], v[ ( e + 1 ) % 3 ] );
                    ul[ e ]          = sqrtf( dot( u[ e ], u[ e ] ) );
                    const float side = dot( u[ e ], v[ ( e + 2 ) % 3 ] );
                    flat |= !( ul[ e ] > 0.f ) || side == 0.f;
                    sg[ e ] = side > 0.f ? 1.f : -1.f;
                }
                if ( flat )
                    continue; // a flat triangle has no area
                const uint32_t cnt = p < Q ? min( (uint32_t)id.w, kMaxProbeNbr ) : 0u;
                const int      M   = 3 + (int)cnt;
                if ( lane < 3 )
                {
                    const f3 w     = u[ lane ] * ( -sg[ lane ] / ul[ lane ] );
                    S.cons[ lane ] = make_float4( w.x, w.y, w.z, 0.f );
                }
                // neighbour caps at 3 .. M - 1 (up to 35 constraints: lane + 3 covers them in one pass)
                if ( lane < cnt )
                {
                    const int      m  = 3 + (int)lane;
                    const uint32_t q  = b.probeNbrIdx[ (size_t)p * kMaxProbeNbr + lane ];
                    const float4   pq = b.probePos[ q ];
                    const f3       D  = F3( pq.x - P.x, pq.y - P.y, pq.z - P.z );
                    const float    L  = sqrtf( dot( D, D ) );
                    S.dist[ m ]       = L;
                    S.nq[ m ]         = q;
                    if ( L > 0.f && L < 2.f * rp )
                    {
                        const f3 w  = D * ( 1.f / L );
                        S.cons[ m ] = make_float4( w.x, w.y, w.z, L / ( 2.f * rp ) );
                    }
                    else
                        S.cons[ m ] = make_float4( 0.f, 0.f, 1.f, 2.f ); // vacuous
                }
                for ( int m = (int)lane; m < M; m += 32 )
                {
                    S.dphi[ m ] = 0.f;
                    S.iy[ m ]   = make_float4( 0.f, 0.f, 0.f, 0.f );
                }
                __syncwarp();
                const float U = region_area_warp( S.cons, M, S.cuts, overflow, [ & ]( int m, const Circ & C, float st, float ln, int, int ) {
                    if ( !kGrad )
                        return;
                    S.dphi[ m ] += ln;
                    const f3 Iy = arc_integral( C, st, ln );
                    S.iy[ m ].x += Iy.x, S.iy[ m ].y += Iy.y, S.iy[ m ].z += Iy.z;
                } );
                __syncwarp();
                const float cA = rp * rp * U;
                if ( lane == 0 )
                {
                    concaveSum += cA;
                    if ( atomArea )
                        for ( int a = 0; a < 3; a++ )
                            atomicAdd( atomArea + b.perm[ ia[ a ] ], cA * ( 1.f / 3.f ) );
                }
                // a nearly coincident neighbour probe: the region's adjoint in double precision
                const bool close = kGrad && __any_sync( 0xffffffffu, lane < cnt && S.dist[ 3 + lane ] < kCloseProbe );
                if ( close )
                    probe_region_grad_d( b, p, gConcave, gradSorted, probeGrad, S.kd, S.sums );
                if ( kGrad && !close )
                {
                    const float k2 = gConcave * rp * rp;
                    f3          gP = F3( 0.f, 0.f, 0.f );
                    if ( lane == 0 )
                    {
                        f3 gv[ 3 ] = { F3( 0.f, 0.f, 0.f ), F3( 0.f, 0.f, 0.f ), F3( 0.f, 0.f, 0.f ) };
                        for ( int e = 0; e < 3; e++ )
                        {
                            const f3  gw = F3( S.iy[ e ].x, S.iy[ e ].y, S.iy[ e ].z ) * ( -k2 );
                            const f3  wh = u[ e ] * ( 1.f / ul[ e ] );
                            const f3  gu = ( gw - wh * dot( gw, wh ) ) * ( -sg[ e ] / ul[ e ] );
                            const int a = e, c2 = ( e + 1 ) % 3;
                            gv[ a ]     = gv[ a ] + cross( v[ c2 ], gu );
                            gv[ c2 ]    = gv[ c2 ] + cross( gu, v[ a ] );
                        }
                        for ( int a = 0; a < 3; a++ )
                        {
                            const f3 gD = ( gv[ a ] - v[ a ] * dot( gv[ a ], v[ a ] ) ) * ( 1.f / Lv[ a ] );
                            add4( gradSorted, (uint32_t)ia[ a ], gD, 0.f );
                            gP = gP - gD;
                        }
                    }
                    if ( lane < cnt )
                    {
                        const int   m = 3 + (int)lane;
                        const float L = S.dist[ m ];
                        if ( L > 0.f && L < 2.f * rp )
                        {
                            const float4 k  = S.cons[ m ];
                            const f3     w  = F3( k.x, k.y, k.z );
                            const f3     gw = F3( S.iy[ m ].x, S.iy[ m ].y, S.iy[ m ].z ) * ( -k2 );
                            const float  gc = k2 * S.dphi[ m ];
                            const f3     gD = ( gw - w * dot( gw, w ) ) * ( 1.f / L ) + w * ( gc / ( 2.f * rp ) );
                            gP              = gP - gD;
                            atomicAdd( &probeGrad[ S.nq[ m ] ].x, gD.x );
                            atomicAdd( &probeGrad[ S.nq[ m ] ].y, gD.y );
                            atomicAdd( &probeGrad[ S.nq[ m ] ].z, gD.z );
                        }
                    }
                    for ( int o = 16; o > 0; o >>= 1 )
                    {
                        gP.x += __shfl_xor_sync( 0xffffffffu, gP.x, o );
                        gP.y += __shfl_xor_sync( 0xffffffffu, gP.y, o );
                        gP.z += __shfl_xor_sync( 0xffffffffu, gP.z, o );
                    }
                    if ( lane == 0 )
                    {
                        atomicAdd( &probeGrad[ p ].x, gP.x );
                        atomicAdd( &probeGrad[ p ].y, gP.y );
                        atomicAdd( &probeGrad[ p ].z, gP.z );
                    }
                }
                __syncwarp();
            }
            if ( lane == 0 && parts && concaveSum != 0.0 )
                atomicAdd( parts + 2, concaveSum );
            overflow = __any_sync( 0xffffffffu, overflow != 0 );
            if ( lane == 0 && overflow )
                atomicOr( &b.counts->overflow, (uint32_t)kOverflowArea );
        }

        // probe positions follow their atoms: M^T lambda = g with rows p - c_a;
        // d/dc_a = lambda_a (p - c_a), d/dR_a = lambda_a R_a. The 3x3 solve is in double
        // precision: for a probe near the plane of its three centres (its mirror probe about to
        // merge with it) M is nearly singular and lambda grows as 1 / det, so float32 rounding of
        // the rows and of det would show in the atoms' gradients. One solve per probe: the FP64
        // pipe's rate does not matter here.
        __global__ void k_area_probe_back( Build b, const float4 * probeGrad, float * gradSorted )
        {
            const uint32_t I = min( b.counts->I, b.capProbes );
            for ( uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < I; p += gridDim.x * blockDim.x )
            {
                const float4 g4 = probeGrad[ p ];
                if ( g4.x == 0.f && g4.y == 0.f && g4.z == 0.f )
                    continue;
                const d3     g  = D3( (double)g4.x, (double)g4.y, (double)g4.z );
                const int4   id = b.probeIds[ p ];
                const float4 pp = b.probePos[ p ];
                const int    ia[ 3 ] = { id.x, id.y, id.z };
                d3           r[ 3 ];
                double       R[ 3 ];
                for ( int k = 0; k < 3; k++ )
                {
                    const float4 c = b.atoms[ ia[ k ] ];
                    // differences of float32 values: exact in double
                    r[ k ] = D3( (double)pp.x - (double)c.x, (double)pp.y - (double)c.y, (double)pp.z - (double)c.z );
                    R[ k ] = (double)c.w + (double)b.rp;
                }
                const double det = ddot( r[ 0 ], dcross( r[ 1 ], r[ 2 ] ) );
                if ( !( fabs( det ) > 0.0 ) )
                    continue;
                const double lam[ 3 ] = { ddot( g, dcross( r[ 1 ], r[ 2 ] ) ) / det, ddot( r[ 0 ], dcross( g, r[ 2 ] ) ) / det,
                                          ddot( r[ 0 ], dcross( r[ 1 ], g ) ) / det };
                for ( int k = 0; k < 3; k++ )
                    add4( gradSorted, (uint32_t)ia[ k ],
                          F3( (float)( r[ k ].x * lam[ k ] ), (float)( r[ k ].y * lam[ k ] ), (float)( r[ k ].z * lam[ k ] ) ),
                          (float)( lam[ k ] * R[ k ] ) );
            }
        }

        __global__ void k_area_unsort( Build b, const float * gradSorted, float * gradInput )
        {
            for ( uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < b.n; s += gridDim.x * blockDim.x )
            {
                const uint32_t i = b.perm[ s ];
                for ( int k = 0; k < 4; k++ )
                    gradInput[ 4 * (size_t)i + k ] = gradSorted[ 4 * (size_t)s + k ];
            }
        }

        inline uint32_t area_blocks( uint64_t items )
        {
            const uint64_t want = ( items + kAreaWarps - 1 ) / kAreaWarps;
            const uint64_t cap  = 152ull * 16ull;
            return (uint32_t)( want < 1 ? 1 : ( want < cap ? want : cap ) );
        }
    } // namespace

    size_t area_scratch_bytes( const Build & b ) { return sizeof( float4 ) * (size_t)b.capProbes + 256; }

    void launch_area( const Build & b, double * parts, float * atomArea, cudaStream_t s )
    {
        cudaMemsetAsync( parts, 0, 3 * sizeof( double ), s );
        if ( atomArea )
            cudaMemsetAsync( atomArea, 0, sizeof( float ) * (size_t)b.n, s );
        if ( !b.n )
            return;
        k_area_atoms<false><<<area_blocks( b.n ), 32 * kAreaWarps, 0, s>>>( b, parts, atomArea, 0.f, 0.f, nullptr );
        k_area_probes<false><<<area_blocks( b.capProbes ), 32 * kAreaWarps, 0, s>>>( b, parts, atomArea, 0.f, nullptr, nullptr );
        count_launches( 2 );
    }

    void launch_area_backward( const Build & b, const float gParts[ 3 ], float * gradSorted, float * gradInput, void * scratch,
                               cudaStream_t s )
    {
        cudaMemsetAsync( gradSorted, 0, sizeof( float ) * 4 * (size_t)b.n, s );
        if ( !b.n )
        {
            return;
        }
        float4 * probeGrad = static_cast<float4 *>( scratch );
        cudaMemsetAsync( probeGrad, 0, sizeof( float4 ) * (size_t)b.capProbes, s );
        k_area_atoms<true><<<area_blocks( b.n ), 32 * kAreaWarps, 0, s>>>( b, nullptr, nullptr, gParts[ 0 ], gParts[ 1 ], gradSorted );
        k_area_probes<true><<<area_blocks( b.capProbes ), 32 * kAreaWarps, 0, s>>>( b, nullptr, nullptr, gParts[ 2 ], gradSorted, probeGrad );
        k_area_probe_back<<<min( 152u * 8u, ( b.capProbes + 255 ) / 256 + 1 ), 256, 0, s>>>( b, probeGrad, gradSorted );
        k_area_unsort<<<( b.n + 255 ) / 256, 256, 0, s>>>( b, gradSorted, gradInput );
        count_launches( 4 );
    }
} // namespace sesgb
