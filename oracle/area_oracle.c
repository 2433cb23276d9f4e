/* area_oracle.c -- TEST ORACLE (test infrastructure only): FP64 restatement of
 * the solvent-excluded surface area of a full-surface build and of its
 * gradient with respect to the atoms. The reference renders the surface from
 * its primitives and computes no area; the area here is the area of those
 * primitives:
 *
 *  - convex patch of atom i: the directions of the SAS sphere of i outside every
 *    other SAS sphere of N(i) (the accessible sphere patch the sectors of
 *    buildConvexPatchesSectors describe, operations.inl:175-228), scaled to the
 *    vdW sphere: r_i^2 U_i;
 *  - toroidal patch of circle (i, j): the probe swept over the accessible arcs
 *    of the circle (the segments of buildSegments, operations.inl:552-668, and
 *    the full circles), between its contact points with i and j, trimmed at
 *    the axis where the torus self-intersects (rho < rp);
 *  - concave patch of a probe: the geodesic triangle of its three contact
 *    directions (findIntersectionsBetweenCircles, operations.inl:230-486),
 *    outside the spheres of the probe's listed neighbours (the singular
 *    neighbour lists of findIntersectionsNeighbors, operations.cu:271-338).
 *
 * Every patch is a region of a sphere of the form R = {y : |y| = 1,
 * y . w_m <= c_m for all m}. Its area follows from Gauss-Bonnet,
 *   A = 2 pi chi + sum_m c_m dphi_m - sum_v theta_v,
 * where dphi_m is the angle of the circle y . w_m = c_m left on the boundary
 * and theta_v = acos((w_m . w_n - c_m c_n) / (s_m s_n)) the turning angle at a
 * corner where circles m and n meet (s = sqrt(1 - c^2)). The Euler
 * characteristic is never needed: R is cut into three lunes of 120 degrees
 * around the z axis (two more constraints each); a lune has area 4 pi / 3 < 2 pi,
 * so the area of each piece is the Gauss-Bonnet sum reduced mod 2 pi. The
 * corner terms are written per arc, as the change of the boundary tangent's
 * angle against a fixed frame field between the arc's two ends: no corner has to
 * be matched with the arc on its other side, and several circles through one
 * point (the axis points of a self-intersecting torus) need no special case.
 *
 * Gradient: moving constraint m changes the area by dA/dc_m = dphi_m and
 * dA/dw_m = -integral of y dphi over the arcs of m on the boundary (the
 * boundary moves by the constraint change over |grad_tangent|). The angle of
 * an accessible arc moves with its end points (intersections with the circles
 * that bound it). Probe positions follow their atoms through the implicit
 * function of |p - c_a|^2 = R_a^2. */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct
{
    double x, y, z;
} a3;
static inline a3     A3( double x, double y, double z ) { a3 r = { x, y, z }; return r; }
static inline a3     aadd( a3 a, a3 b ) { return A3( a.x + b.x, a.y + b.y, a.z + b.z ); }
static inline a3     asub( a3 a, a3 b ) { return A3( a.x - b.x, a.y - b.y, a.z - b.z ); }
static inline a3     amul( a3 a, double s ) { return A3( a.x * s, a.y * s, a.z * s ); }
static inline double adot( a3 a, a3 b ) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline a3     across( a3 a, a3 b ) { return A3( a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x ); }
static inline double alen( a3 a ) { return sqrt( adot( a, a ) ); }

#define AREA_MAXC 256 /* constraints of one region (neighbours, or 3 edges + 32 probes) */
static const double kPi = 3.14159265358979323846;

typedef struct
{
    a3     w;
    double c;
} cons_t;

/* per constraint of a region: the boundary angle and the integral of y over it */
typedef struct
{
    double dphi;
    a3     iy;
} cons_sum_t;

/* an accessible arc of circle m: angles [pa, pa + len] in the frame (e1, e2) of
 * the circle, start bounded by circle na, end by nb (-1: whole circle) */
typedef struct
{
    int    m, na, nb;
    double pa, len;
} arc_t;

typedef struct
{
    cons_t k[ AREA_MAXC + 2 ];
    a3     e1[ AREA_MAXC + 2 ], e2[ AREA_MAXC + 2 ];
    double s[ AREA_MAXC + 2 ];
    double ivS[ AREA_MAXC + 2 ], ivL[ AREA_MAXC + 2 ], enV[ AREA_MAXC + 2 ], enL[ AREA_MAXC + 2 ];
    int    ivN[ AREA_MAXC + 2 ], enN[ AREA_MAXC + 2 ];
    int    M;       /* constraints of the region (without the lune pair) */
    arc_t  arcs[ 4 * ( AREA_MAXC + 2 ) ];
    int    nArcs;   /* arcs of the original constraints, all lunes */
    int    overflow;
} region_t;

static void frame_of( a3 w, a3 * e1, a3 * e2 )
{
    const double ax = fabs( w.x ), ay = fabs( w.y ), az = fabs( w.z );
    const a3     t  = ( ax <= ay && ax <= az ) ? A3( 1, 0, 0 ) : ( ay <= az ? A3( 0, 1, 0 ) : A3( 0, 0, 1 ) );
    a3           u  = across( w, t );
    u               = amul( u, 1.0 / alen( u ) );
    *e1             = u;
    *e2             = across( w, u );
}

static double wrap2pi( double a )
{
    a = fmod( a, 2.0 * kPi );
    return a < 0.0 ? a + 2.0 * kPi : a;
}

/* Tangent-angle change of the boundary along the arc [pa, pa + len] of a circle,
 * traversed with the region on its left (decreasing phi, the cap lies towards w),
 * measured against the frame field xi(y) = a - (a . y) y (singular only at
 * +-a): alpha(end) - alpha(start) with alpha = atan2((xi x t) . y, xi . t). At a
 * corner the arcs meeting there share y, so the differences of their alphas
 * are the corner's turning angle and no corner needs to know its partner. */
static const a3 kFrameAxis = { 0.32140077, 0.55410134, 0.76790185 }; /* a generic unit direction */

static double frame_angle( a3 y, a3 t )
{
    const a3 xi = asub( kFrameAxis, amul( y, adot( kFrameAxis, y ) ) );
    return atan2( adot( across( xi, t ), y ), adot( xi, t ) );
}

static double arc_turn( a3 w, double c, double s, a3 e1, a3 e2, double pa, double len )
{
    const double p0 = pa + len, p1 = pa; /* traversal from p0 down to p1 */
    const a3     y0 = aadd( amul( w, c ), amul( aadd( amul( e1, cos( p0 ) ), amul( e2, sin( p0 ) ) ), s ) );
    const a3     y1 = aadd( amul( w, c ), amul( aadd( amul( e1, cos( p1 ) ), amul( e2, sin( p1 ) ) ), s ) );
    const a3     t0 = asub( amul( e1, sin( p0 ) ), amul( e2, cos( p0 ) ) );
    const a3     t1 = asub( amul( e1, sin( p1 ) ), amul( e2, cos( p1 ) ) );
    return frame_angle( y1, t1 ) - frame_angle( y0, t0 );
}

/* area of R cut to lune L (azimuth in [2 pi L / 3, 2 pi (L + 1) / 3]); adds the
 * boundary angles and y-integrals of the original constraints to sums and
 * records their arcs */
static double region_lune( region_t * R, int L, cons_sum_t * sums )
{
    const int    M = R->M, K = M + 2;
    const double al = 2.0 * kPi * L / 3.0, be = al + 2.0 * kPi / 3.0;
    /* y . u1 >= 0 and y . u2 >= 0, u1 = (-sin al, cos al, 0), u2 = (sin be, -cos be, 0) */
    R->k[ M ].w     = A3( sin( al ), -cos( al ), 0.0 );
    R->k[ M ].c     = 0.0;
    R->k[ M + 1 ].w = A3( -sin( be ), cos( be ), 0.0 );
    R->k[ M + 1 ].c = 0.0;
    for ( int m = M; m < K; m++ )
    {
        R->s[ m ] = 1.0;
        frame_of( R->k[ m ].w, &R->e1[ m ], &R->e2[ m ] );
    }
    double total = 0.0;
    for ( int m = 0; m < K; m++ )
    {
        const double cm = R->k[ m ].c;
        if ( !( cm < 1.0 ) || !( cm > -1.0 ) )
            continue; /* vacuous (an empty region is caught by the caller) */
        const double sm = R->s[ m ];
        const a3     wm = R->k[ m ].w, e1 = R->e1[ m ], e2 = R->e2[ m ];
        int          nIv = 0, gone = 0;
        for ( int n = 0; n < K && !gone; n++ )
        {
            if ( n == m )
                continue;
            const double cn = R->k[ n ].c;
            if ( !( cn < 1.0 ) )
                continue;
            const a3 wn = R->k[ n ].w;
            if ( wn.x == wm.x && wn.y == wm.y && wn.z == wm.z && cn == cm )
            {
                if ( n < m )
                    gone = 1; /* the same constraint twice: the first one keeps the circle */
                continue;
            }
            const double p1 = adot( e1, wn ), p2 = adot( e2, wn );
            const double A = cm * adot( wm, wn ), B = sm * sqrt( p1 * p1 + p2 * p2 ), rhs = cn - A;
            if ( !( B > fabs( rhs ) ) )
            {
                if ( rhs < 0.0 )
                    gone = 1; /* the whole circle lies inside cap n */
                continue;
            }
            /* y . w_n > c_n on (phi0 - delta, phi0 + delta) */
            const double delta = atan2( sqrt( ( B - rhs ) * ( B + rhs ) ), rhs );
            const double phi0  = atan2( p2, p1 );
            R->ivS[ nIv ]      = wrap2pi( phi0 - delta );
            R->ivL[ nIv ]      = 2.0 * delta;
            R->ivN[ nIv ]      = n;
            nIv++;
        }
        if ( gone )
            continue;
        if ( nIv == 0 )
        {
            total += cm * 2.0 * kPi;
            if ( m < M )
            {
                sums[ m ].dphi += 2.0 * kPi;
                sums[ m ].iy = aadd( sums[ m ].iy, amul( wm, cm * 2.0 * kPi ) );
                if ( R->nArcs < (int)( sizeof( R->arcs ) / sizeof( R->arcs[ 0 ] ) ) )
                {
                    arc_t * a = &R->arcs[ R->nArcs++ ];
                    a->m = m, a->na = -1, a->nb = -1, a->pa = 0.0, a->len = 2.0 * kPi;
                }
                else
                    R->overflow = 1;
            }
            continue;
        }
        /* allowed arcs: the gaps between the cuts. An end strictly inside another
         * cut is covered (lengths re-measured from the rounded ends, so that equal
         * ends compare equal); of equal uncovered ends the first one counts. */
        for ( int q = 0; q < nIv; q++ )
        {
            R->enV[ q ]       = wrap2pi( R->ivS[ q ] + R->ivL[ q ] );
            const double len2 = wrap2pi( R->enV[ q ] - R->ivS[ q ] );
            R->enL[ q ]       = len2 >= 0.5 * R->ivL[ q ] ? len2 : R->ivL[ q ];
        }
        for ( int a = 0; a < nIv; a++ )
        {
            R->enN[ a ] = 1;
            for ( int b = 0; b < nIv && R->enN[ a ]; b++ )
                if ( b != a && wrap2pi( R->enV[ a ] - R->ivS[ b ] ) < R->enL[ b ] )
                    R->enN[ a ] = 0;
        }
        for ( int a = 0; a < nIv; a++ )
        {
            if ( !R->enN[ a ] )
                continue;
            const double end = R->enV[ a ];
            int          dup = 0;
            for ( int b = 0; b < a && !dup; b++ )
                dup = R->enN[ b ] && R->enV[ b ] == end;
            if ( dup )
                continue;
            double gap = 2.0 * kPi;
            int    nb  = -1;
            for ( int b = 0; b < nIv; b++ )
            {
                const double g = wrap2pi( R->ivS[ b ] - end );
                if ( g > 0.0 && ( nb < 0 || g < gap ) )
                {
                    gap = g;
                    nb  = b;
                }
            }
            if ( nb < 0 )
                continue;
            const int na = R->ivN[ a ], nbc = R->ivN[ nb ];
            total += cm * gap + arc_turn( wm, cm, sm, e1, e2, end, gap );
            if ( m < M )
            {
                sums[ m ].dphi += gap;
                const double c0 = cos( end ), s0 = sin( end ), c1 = cos( end + gap ), s1 = sin( end + gap );
                sums[ m ].iy = aadd( sums[ m ].iy, aadd( amul( wm, cm * gap ), amul( asub( amul( e1, s1 - s0 ), amul( e2, c1 - c0 ) ), sm ) ) );
                if ( R->nArcs < (int)( sizeof( R->arcs ) / sizeof( R->arcs[ 0 ] ) ) )
                {
                    arc_t * r = &R->arcs[ R->nArcs++ ];
                    r->m = m, r->na = na, r->nb = nbc, r->pa = end, r->len = gap;
                }
                else
                    R->overflow = 1;
            }
        }
    }
    double r = wrap2pi( total );
    if ( r > 5.0 * kPi / 3.0 )
        r -= 2.0 * kPi; /* a piece of (nearly) zero area */
    return r > 0.0 ? r : 0.0;
}

/* area of R (unit sphere); sums[m] (M entries) receive dphi and the y-integral */
static double region_area( region_t * R, cons_sum_t * sums )
{
    const int M = R->M;
    for ( int m = 0; m < M; m++ )
    {
        sums[ m ].dphi = 0.0;
        sums[ m ].iy   = A3( 0, 0, 0 );
    }
    R->nArcs    = 0;
    R->overflow = 0;
    for ( int m = 0; m < M; m++ )
        if ( !( R->k[ m ].c > -1.0 ) )
            return 0.0; /* one cap holds the whole sphere */
    for ( int m = 0; m < M; m++ )
    {
        const double c = R->k[ m ].c;
        R->s[ m ]      = ( c < 1.0 ) ? sqrt( ( 1.0 - c ) * ( 1.0 + c ) ) : 0.0;
        if ( c < 1.0 )
            frame_of( R->k[ m ].w, &R->e1[ m ], &R->e2[ m ] );
    }
    double A = 0.0;
    for ( int L = 0; L < 3; L++ )
        A += region_lune( R, L, sums );
    return A;
}

/* ---- atom-sphere constraints ------------------------------------------------ */
typedef struct
{
    a3     D;  /* c_j - c_i */
    double d, Ri, Rj;
} pair_t;

/* w = D / d, c = (R_i^2 - R_j^2 + d^2) / (2 d R_i) */
static cons_t pair_cons( const pair_t * p )
{
    cons_t k;
    k.w = amul( p->D, 1.0 / p->d );
    k.c = ( p->Ri * p->Ri - p->Rj * p->Rj + p->d * p->d ) / ( 2.0 * p->d * p->Ri );
    return k;
}

/* d(loss) through (w, c) of a pair constraint into atoms i and j (grad: x, y, z, R) */
static void pair_back( const pair_t * p, a3 gw, double gc, double * gi, double * gj )
{
    const a3     w   = amul( p->D, 1.0 / p->d );
    const double d = p->d, Ri = p->Ri, Rj = p->Rj;
    const double dcd = 1.0 / ( 2.0 * Ri ) - ( Ri * Ri - Rj * Rj ) / ( 2.0 * d * d * Ri );
    const double dcRi = ( Ri * Ri + Rj * Rj - d * d ) / ( 2.0 * d * Ri * Ri );
    const double dcRj = -Rj / ( d * Ri );
    const a3     gD   = aadd( amul( asub( gw, amul( w, adot( gw, w ) ) ), 1.0 / d ), amul( w, gc * dcd ) );
    gj[ 0 ] += gD.x, gj[ 1 ] += gD.y, gj[ 2 ] += gD.z;
    gi[ 0 ] -= gD.x, gi[ 1 ] -= gD.y, gi[ 2 ] -= gD.z;
    gi[ 3 ] += gc * dcRi;
    gj[ 3 ] += gc * dcRj;
}

/* toroidal patch per unit angle: rp * integral over [beta_i, beta_j] of
 * max(0, rho - rp cos beta) d beta, beta_i = -atan2(h_i, rho), beta_j = atan2(h_j, rho);
 * dF receives dF/d(d, R_i, R_j) */
static double torus_F( double d, double Ri, double Rj, double rp, double dF[ 3 ] )
{
    const double hi = ( Ri * Ri - Rj * Rj + d * d ) / ( 2.0 * d ), hj = d - hi;
    const double rr = Ri * Ri - hi * hi;
    dF[ 0 ] = dF[ 1 ] = dF[ 2 ] = 0.0;
    if ( !( rr > 0.0 ) )
        return 0.0;
    const double rho = sqrt( rr );
    const double bi = -atan2( hi, rho ), bj = atan2( hj, rho );
    double       F  = rho * ( bj - bi ) - rp * ( hj / Rj + hi / Ri );
    double       Fr = ( bj - bi ) - rho * ( hj / ( Rj * Rj ) + hi / ( Ri * Ri ) ) + rp * rho * ( hj / ( Rj * Rj * Rj ) + hi / ( Ri * Ri * Ri ) );
    const double Fhi = ( rho * rho / ( Ri * Ri ) ) * ( 1.0 - rp / Ri );
    const double Fhj = ( rho * rho / ( Rj * Rj ) ) * ( 1.0 - rp / Rj );
    if ( rho < rp && hi > 0.0 && hj > 0.0 )
    {
        /* the torus crosses its axis: the part with rho - rp cos beta < 0 is not surface */
        const double b0 = acos( rho / rp );
        F -= 2.0 * rho * b0 - 2.0 * rp * sqrt( ( 1.0 - rho / rp ) * ( 1.0 + rho / rp ) );
        Fr -= 2.0 * b0;
    }
    /* (rho, h_i, h_j) from (d, R_i, R_j) */
    const double rd = -hi * hj / ( d * rho ), rRi = Ri * hj / ( d * rho ), rRj = Rj * hi / ( d * rho );
    dF[ 0 ] = rp * ( Fr * rd + Fhi * ( hj / d ) + Fhj * ( hi / d ) );
    dF[ 1 ] = rp * ( Fr * rRi + Fhi * ( Ri / d ) + Fhj * ( -Ri / d ) );
    dF[ 2 ] = rp * ( Fr * rRj + Fhi * ( -Rj / d ) + Fhj * ( Rj / d ) );
    return rp * F;
}

static void atomic_add( double * p, double v )
{
#pragma omp atomic
    *p += v;
}

/* d(loss) at a probe position p = P(atoms a, b, c) into the atoms: solve
 * M^T lambda = g with rows M_k = p - c_k; d/dc_k = lambda_k (p - c_k),
 * d/dR_k = lambda_k R_k */
static void probe_back( const float * atoms, const int32_t * ids, const double * pos, double rp, a3 g, double * grad )
{
    const a3 p = A3( pos[ 0 ], pos[ 1 ], pos[ 2 ] );
    a3       r[ 3 ];
    double   R[ 3 ];
    for ( int k = 0; k < 3; k++ )
    {
        const float * c = atoms + 4 * (size_t)ids[ k ];
        r[ k ]          = A3( p.x - c[ 0 ], p.y - c[ 1 ], p.z - c[ 2 ] );
        R[ k ]          = (double)c[ 3 ] + rp;
    }
    /* M^T lambda = g: columns r_k; Cramer's rule */
    const double det = adot( r[ 0 ], across( r[ 1 ], r[ 2 ] ) );
    if ( !( fabs( det ) > 0.0 ) )
        return;
    double lam[ 3 ];
    lam[ 0 ] = adot( g, across( r[ 1 ], r[ 2 ] ) ) / det;
    lam[ 1 ] = adot( r[ 0 ], across( g, r[ 2 ] ) ) / det;
    lam[ 2 ] = adot( r[ 0 ], across( r[ 1 ], g ) ) / det;
    for ( int k = 0; k < 3; k++ )
    {
        double * gk = grad + 4 * (size_t)ids[ k ];
        atomic_add( gk + 0, lam[ k ] * r[ k ].x );
        atomic_add( gk + 1, lam[ k ] * r[ k ].y );
        atomic_add( gk + 2, lam[ k ] * r[ k ].z );
        atomic_add( gk + 3, lam[ k ] * R[ k ] );
    }
}

/* Total SES area of the primitives of a full-surface build (sorted atoms xyzr,
 * CSR neighbour lists with their circle statuses (an atom whose circles are all
 * buried has no accessible patch), probes: ids (i, j, k, neighbour count), FP64 positions,
 * the first Q probes singular with neighbour lists snbrIdx[32 q + t]).
 * parts: convex, toroidal, concave. atomArea (n, optional): convex area of the
 * atom + half of its tori + a third of its probes' concave patches. With grad
 * (4n, sorted order, accumulated): d (sum_k gParts[k] parts[k]) / d (x, y, z, r).
 * Returns the number of regions whose arc list overflowed (0 when complete). */
int ora_area( const float * atoms, uint32_t n, const uint32_t * noff, const uint32_t * nbr, const uint8_t * status, const int32_t * ids,
              const double * posd, uint32_t I, uint32_t Q, const uint32_t * snbrIdx, float rpf, const double * gParts,
              double * parts, double * atomArea, double * grad, int threads )
{
    const double rp = rpf;
    /* loss weights of the convex, toroidal and concave areas */
    const double gConvex = gParts ? gParts[ 0 ] : 0.0, gTorus = gParts ? gParts[ 1 ] : 0.0, gConcave = gParts ? gParts[ 2 ] : 0.0;
    double       convex = 0.0, toroidal = 0.0, concave = 0.0;
    int          overflow = 0;
    if ( atomArea )
        memset( atomArea, 0, sizeof( double ) * n );
    double * probeGrad = grad ? (double *)calloc( 3 * (size_t)( I ? I : 1 ), sizeof( double ) ) : NULL;
    if ( threads > 0 )
        omp_set_num_threads( threads );
#pragma omp parallel reduction( + : convex, toroidal, concave, overflow )
    {
        region_t *   R    = (region_t *)malloc( sizeof( region_t ) );
        cons_sum_t * sums = (cons_sum_t *)malloc( sizeof( cons_sum_t ) * AREA_MAXC );
        pair_t *     pr   = (pair_t *)malloc( sizeof( pair_t ) * AREA_MAXC );
        double *     gcs  = (double *)malloc( sizeof( double ) * AREA_MAXC );
        a3 *         gws  = (a3 *)malloc( sizeof( a3 ) * AREA_MAXC );
        double *     gloc = (double *)malloc( sizeof( double ) * 4 * ( AREA_MAXC + 1 ) );
#pragma omp for schedule( dynamic, 16 )
        for ( int64_t ii = 0; ii < (int64_t)n; ii++ )
        {
            const uint32_t i  = (uint32_t)ii;
            const float *  ai = atoms + 4 * (size_t)i;
            const double   Ri = (double)ai[ 3 ] + rp, ri = ai[ 3 ];
            const uint32_t b0 = noff[ i ], ni = noff[ i + 1 ] - b0;
            int            M  = 0;
            /* an atom whose circles are all buried (status 0) has no accessible patch */
            int open = ni == 0;
            for ( uint32_t s = 0; s < ni && !open; s++ )
                open = status[ b0 + s ] != 0;
            if ( !open )
                continue;
            for ( uint32_t s = 0; s < ni && M < AREA_MAXC; s++ )
            {
                const float * aj = atoms + 4 * (size_t)nbr[ b0 + s ];
                pair_t        p;
                p.D  = A3( (double)aj[ 0 ] - ai[ 0 ], (double)aj[ 1 ] - ai[ 1 ], (double)aj[ 2 ] - ai[ 2 ] );
                p.d  = alen( p.D );
                p.Ri = Ri;
                p.Rj = (double)aj[ 3 ] + rp;
                if ( !( p.d > 0.0 ) )
                    p.D = A3( 0, 0, 1 ), p.d = 0.0;
                pr[ s ]   = p;
                R->k[ M ] = p.d > 0.0 ? pair_cons( &p ) : ( cons_t ) { A3( 0, 0, 1 ), 2.0 }; /* coincident centres: ignored */
                M++;
            }
            R->M           = M;
            const double U = region_area( R, sums );
            overflow += R->overflow;
            const double cA = ri * ri * U;
            convex += cA;
            double mine = cA;
            /* tori of the circles (i, j), i < j */
            for ( int m = 0; m < M; m++ )
            {
                gcs[ m ] = 0.0;
                gws[ m ] = A3( 0, 0, 0 );
            }
            for ( int m = 0; m < M; m++ )
            {
                const uint32_t j = nbr[ b0 + m ];
                if ( !( j > i ) || !( sums[ m ].dphi > 0.0 ) )
                    continue;
                double       dF[ 3 ];
                const double F = torus_F( pr[ m ].d, Ri, pr[ m ].Rj, rp, dF );
                const double T = F * sums[ m ].dphi;
                toroidal += T;
                mine += 0.5 * T;
                if ( atomArea )
                    atomic_add( atomArea + j, 0.5 * T );
                if ( !grad )
                    continue;
                /* F part: through d, R_i, R_j */
                const double gs = gTorus * sums[ m ].dphi;
                const a3     w  = amul( pr[ m ].D, 1.0 / pr[ m ].d );
                double *     gj = grad + 4 * (size_t)j;
                double *     gi = grad + 4 * (size_t)i;
                atomic_add( gj + 0, gs * dF[ 0 ] * w.x );
                atomic_add( gj + 1, gs * dF[ 0 ] * w.y );
                atomic_add( gj + 2, gs * dF[ 0 ] * w.z );
                atomic_add( gi + 0, -gs * dF[ 0 ] * w.x );
                atomic_add( gi + 1, -gs * dF[ 0 ] * w.y );
                atomic_add( gi + 2, -gs * dF[ 0 ] * w.z );
                atomic_add( gi + 3, gs * dF[ 1 ] );
                atomic_add( gj + 3, gs * dF[ 2 ] );
                /* angle part: every arc end bounded by another neighbour moves with both circles */
                const double G  = gTorus * F;
                const double c  = R->k[ m ].c, s = R->s[ m ];
                const a3     wm = R->k[ m ].w;
                for ( int q = 0; q < R->nArcs; q++ )
                {
                    const arc_t * a = &R->arcs[ q ];
                    if ( a->m != m )
                        continue;
                    for ( int e = 0; e < 2; e++ )
                    {
                        const int nn = e == 0 ? a->na : a->nb;
                        if ( nn < 0 || nn >= M )
                            continue; /* whole circle, or a cut between lunes */
                        const double phi = e == 0 ? a->pa : a->pa + a->len;
                        const a3     yc  = amul( aadd( amul( R->e1[ m ], cos( phi ) ), amul( R->e2[ m ], sin( phi ) ) ), s );
                        const a3     y   = aadd( amul( wm, c ), yc );
                        const a3     t   = across( wm, yc );
                        const a3     wn  = R->k[ nn ].w;
                        const double tw  = adot( t, wn );
                        if ( !( fabs( tw ) > 0.0 ) )
                            continue;
                        const double coef = ( e == 0 ? -G : G ) / tw;
                        const double wwn  = adot( wm, wn );
                        gcs[ nn ] += coef;
                        gws[ nn ] = asub( gws[ nn ], amul( y, coef ) );
                        gcs[ m ] -= coef * ( wwn - ( c / ( s * s ) ) * adot( yc, wn ) );
                        gws[ m ] = asub( gws[ m ], amul( asub( amul( wn, c ), amul( yc, wwn ) ), coef ) );
                    }
                }
            }
            if ( atomArea )
                atomic_add( atomArea + i, mine );
            if ( !grad )
                continue;
            /* convex part: r_i^2 U_i */
            atomic_add( grad + 4 * (size_t)i + 3, gConvex * 2.0 * ri * U );
            memset( gloc, 0, sizeof( double ) * 4 * ( M + 1 ) );
            for ( int m = 0; m < M; m++ )
            {
                if ( !( pr[ m ].d > 0.0 ) )
                    continue;
                const double gc = gcs[ m ] + gConvex * ri * ri * sums[ m ].dphi;
                const a3     gw = asub( gws[ m ], amul( sums[ m ].iy, gConvex * ri * ri ) );
                pair_back( &pr[ m ], gw, gc, gloc + 4 * M, gloc + 4 * m );
            }
            for ( int m = 0; m < M; m++ )
                for ( int a = 0; a < 4; a++ )
                    if ( gloc[ 4 * m + a ] != 0.0 )
                        atomic_add( grad + 4 * (size_t)nbr[ b0 + m ] + a, gloc[ 4 * m + a ] );
            for ( int a = 0; a < 4; a++ )
                atomic_add( grad + 4 * (size_t)i + a, gloc[ 4 * M + a ] );
        }

        /* concave patches */
#pragma omp for schedule( dynamic, 64 )
        for ( int64_t pp = 0; pp < (int64_t)I; pp++ )
        {
            const int32_t * id = ids + 4 * pp;
            const a3        P  = A3( posd[ 4 * pp ], posd[ 4 * pp + 1 ], posd[ 4 * pp + 2 ] );
            a3              Dv[ 3 ], v[ 3 ];
            double          Lv[ 3 ];
            for ( int a = 0; a < 3; a++ )
            {
                const float * c = atoms + 4 * (size_t)id[ a ];
                Dv[ a ]         = A3( c[ 0 ] - P.x, c[ 1 ] - P.y, c[ 2 ] - P.z );
                Lv[ a ]         = alen( Dv[ a ] );
                v[ a ]          = amul( Dv[ a ], 1.0 / Lv[ a ] );
            }
            /* edges (a, b) with the third vertex on the inner side */
            a3     u[ 3 ];
            double ul[ 3 ], sg[ 3 ];
            int    bad = 0;
            for ( int e = 0; e < 3; e++ )
            {
                const int a = e, b = ( e + 1 ) % 3, c = ( e + 2 ) % 3;
                u[ e ]      = across( v[ a ], v[ b ] );
                ul[ e ]     = alen( u[ e ] );
                const double side = adot( u[ e ], v[ c ] );
                if ( !( ul[ e ] > 0.0 ) || side == 0.0 )
                    bad = 1;
                sg[ e ]          = side > 0.0 ? 1.0 : -1.0;
                R->k[ e ].w = amul( u[ e ], -sg[ e ] / ( ul[ e ] > 0.0 ? ul[ e ] : 1.0 ) );
                R->k[ e ].c = 0.0;
            }
            if ( bad )
                continue; /* a flat triangle has no area */
            int      M   = 3;
            uint32_t cnt = ( pp < (int64_t)Q ) ? (uint32_t)id[ 3 ] : 0u;
            if ( cnt > 32 )
                cnt = 32;
            uint32_t nq[ 32 ];
            a3       Dq[ 32 ];
            double   Lq[ 32 ];
            for ( uint32_t t = 0; t < cnt; t++ )
            {
                const uint32_t q = snbrIdx[ 32 * (size_t)pp + t ];
                Dq[ t ]          = A3( posd[ 4 * (size_t)q ] - P.x, posd[ 4 * (size_t)q + 1 ] - P.y, posd[ 4 * (size_t)q + 2 ] - P.z );
                Lq[ t ]          = alen( Dq[ t ] );
                nq[ t ]          = q;
                if ( Lq[ t ] > 0.0 && Lq[ t ] < 2.0 * rp )
                {
                    R->k[ M ].w = amul( Dq[ t ], 1.0 / Lq[ t ] );
                    R->k[ M ].c = Lq[ t ] / ( 2.0 * rp );
                }
                else
                {
                    R->k[ M ].w = A3( 0, 0, 1 );
                    R->k[ M ].c = 2.0; /* vacuous */
                }
                M++;
            }
            R->M           = M;
            const double U = region_area( R, sums );
            overflow += R->overflow;
            const double cA = rp * rp * U;
            concave += cA;
            if ( atomArea )
                for ( int a = 0; a < 3; a++ )
                    atomic_add( atomArea + id[ a ], cA / 3.0 );
            if ( !grad )
                continue;
            const double k2 = gConcave * rp * rp;
            a3           gP = A3( 0, 0, 0 );
            a3           gv[ 3 ] = { A3( 0, 0, 0 ), A3( 0, 0, 0 ), A3( 0, 0, 0 ) };
            for ( int e = 0; e < 3; e++ )
            {
                const a3 gw = amul( sums[ e ].iy, -k2 );
                const a3 wh = amul( u[ e ], 1.0 / ul[ e ] );
                /* w = -sg u / |u| */
                const a3  gu = amul( asub( gw, amul( wh, adot( gw, wh ) ) ), -sg[ e ] / ul[ e ] );
                const int a = e, b = ( e + 1 ) % 3;
                gv[ a ]     = aadd( gv[ a ], across( v[ b ], gu ) );
                gv[ b ]     = aadd( gv[ b ], across( gu, v[ a ] ) );
            }
            for ( int a = 0; a < 3; a++ )
            {
                /* v = D / |D|, D = c_a - P */
                const a3 gD = amul( asub( gv[ a ], amul( v[ a ], adot( gv[ a ], v[ a ] ) ) ), 1.0 / Lv[ a ] );
                double * ga = grad + 4 * (size_t)id[ a ];
                atomic_add( ga + 0, gD.x );
                atomic_add( ga + 1, gD.y );
                atomic_add( ga + 2, gD.z );
                gP = asub( gP, gD );
            }
            for ( uint32_t t = 0; t < cnt; t++ )
            {
                if ( !( Lq[ t ] > 0.0 && Lq[ t ] < 2.0 * rp ) )
                    continue;
                const int    m  = 3 + (int)t;
                const a3     w  = R->k[ m ].w;
                const a3     gw = amul( sums[ m ].iy, -k2 );
                const double gc = k2 * sums[ m ].dphi;
                const a3     gD = aadd( amul( asub( gw, amul( w, adot( gw, w ) ) ), 1.0 / Lq[ t ] ), amul( w, gc / ( 2.0 * rp ) ) );
                gP              = asub( gP, gD );
                atomic_add( probeGrad + 3 * (size_t)nq[ t ] + 0, gD.x );
                atomic_add( probeGrad + 3 * (size_t)nq[ t ] + 1, gD.y );
                atomic_add( probeGrad + 3 * (size_t)nq[ t ] + 2, gD.z );
            }
            atomic_add( probeGrad + 3 * pp + 0, gP.x );
            atomic_add( probeGrad + 3 * pp + 1, gP.y );
            atomic_add( probeGrad + 3 * pp + 2, gP.z );
        }
        if ( grad )
        {
#pragma omp for schedule( static )
            for ( int64_t pp = 0; pp < (int64_t)I; pp++ )
            {
                const a3 g = A3( probeGrad[ 3 * pp ], probeGrad[ 3 * pp + 1 ], probeGrad[ 3 * pp + 2 ] );
                if ( g.x != 0.0 || g.y != 0.0 || g.z != 0.0 )
                    probe_back( atoms, ids + 4 * pp, posd + 4 * pp, rp, g, grad );
            }
        }
        free( R );
        free( sums );
        free( pr );
        free( gcs );
        free( gws );
        free( gloc );
    }
    free( probeGrad );
    parts[ 0 ] = convex;
    parts[ 1 ] = toroidal;
    parts[ 2 ] = concave;
    return overflow;
}

/* Area of one region {y . w_m <= c_m} of the unit sphere (test hook): cons is
 * 4M doubles (w, c); sums (optional) 4M doubles (dphi, integral of y). */
double ora_region_area( const double * cons, int M, double * sums )
{
    if ( M > AREA_MAXC )
        return -1.0;
    region_t *   R = (region_t *)malloc( sizeof( region_t ) );
    cons_sum_t * s = (cons_sum_t *)malloc( sizeof( cons_sum_t ) * ( M ? M : 1 ) );
    R->M           = M;
    for ( int m = 0; m < M; m++ )
    {
        R->k[ m ].w = A3( cons[ 4 * m ], cons[ 4 * m + 1 ], cons[ 4 * m + 2 ] );
        R->k[ m ].c = cons[ 4 * m + 3 ];
    }
    const double A = region_area( R, s );
    if ( sums )
        for ( int m = 0; m < M; m++ )
        {
            sums[ 4 * m ]     = s[ m ].dphi;
            sums[ 4 * m + 1 ] = s[ m ].iy.x;
            sums[ 4 * m + 2 ] = s[ m ].iy.y;
            sums[ 4 * m + 3 ] = s[ m ].iy.z;
        }
    free( R );
    free( s );
    return A;
}
