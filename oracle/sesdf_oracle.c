/*
 * sesdf_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU restatement of the Solvent-Excluded Surface build of PlathC/SESDF
 * (full surface: bcs::Sesdf::build, sesdf/src/sesdf/sesdf.cu:172-264; exterior
 * only: bcs::Ssesdf::build, sesdf/src/ssesdf/ssesdf.cu:133-187). It is the
 * checker for the GPU build in sesdf_gb300/ and is never part of the product
 * path: only tests, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 * Every predicate of the reference is evaluated in IEEE double precision on the
 * float32 inputs, with the reference's own formulas, constants (1e-4f, 3.48f,
 * ...) and operation order, and with floating-point contraction disabled
 * (-ffp-contract=off). The GPU build re-evaluates every decision that its
 * float32 filter cannot settle with the same double-precision expressions, so
 * its topology must agree with this file bit for bit.
 *
 * Where the reference's output order is decided by atomics or by an unstable
 * sort, this file fixes one deterministic order (documented at each stage);
 * the GPU build uses the same order.
 *
 * Parity pin: outputs of the reference's own CUDA kernels (built from its
 * sources by oracle/Makefile and driven by oracle/ref/ref_driver.cu) are
 * compared with this file in tests/test_oracle_golden.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORA_MODE_FULL 0
#define ORA_MODE_EXTERIOR 1

/* band counters (number of predicate evaluations whose FP64 margin lies
 * within the stated degeneracy band) */
enum
{
    BAND_NEIGHBOR = 0,   /* d^2 - (Ri+Rj)^2 <= 1e-4       operations.cu:57 */
    BAND_BURIED,         /* circle covered by k           operations.cu:183 */
    BAND_COMPLETE,       /* circle touched by k           operations.cu:194 */
    BAND_PROBE_T,        /* t >= 0 in the triplet solve   operations.inl:392 */
    BAND_OCCLUSION,      /* |c_l - x|^2 - R_l^2 > 0       operations.inl:428 */
    BAND_SINGULAR,       /* d^2 - rp^2 < -1e-4            operations.inl:451 */
    BAND_SINGULAR_NBR,   /* |x - y| < 2 rp                operations.cu:319 */
    BAND_ANGLE_TIE,      /* segment angles closer than the reference's resolution */
    BAND_ORTHO,          /* |n.x| > 1 - 1e-4              math.cuh:35 */
    ILL_CONDITIONED,     /* triplet solves with condition estimate > 1e3 */
    TORUS_DEGENERATE,    /* torus axis parallel to z      ssesdf/operations.cu:268 */
    NBR_TRUNCATED,       /* atoms whose neighbour list hit the capacity */
    SEG_TRUNCATED,       /* circles with more intersections than the segment cap */
    SNBR_TRUNCATED,      /* singular probes with more than 32 neighbours */
    GRID_OUTSIDE,        /* atoms outside the reference grid (wrapped hash) */
    ORA_NCOUNTER
};

static const double kEps32 = 1.1920928955078125e-07; /* 2^-23 */
static const double kBand  = 64.0;                    /* band width in units of eps32 * magnitude */

typedef struct
{
    double x, y, z;
} v3;

static inline v3 mk( double x, double y, double z )
{
    v3 r = { x, y, z };
    return r;
}
static inline v3 add( v3 a, v3 b ) { return mk( a.x + b.x, a.y + b.y, a.z + b.z ); }
static inline v3 sub( v3 a, v3 b ) { return mk( a.x - b.x, a.y - b.y, a.z - b.z ); }
static inline v3 mul( v3 a, double s ) { return mk( a.x * s, a.y * s, a.z * s ); }
/* helper_math.h dot: a.x*b.x + a.y*b.y + a.z*b.z, evaluated left to right */
static inline double dot( v3 a, v3 b ) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross( v3 a, v3 b ) { return mk( a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x ); }
/* helper_math.h normalize: v * rsqrt(dot(v, v)); restated as v * (1 / sqrt(dot)) */
static inline v3 nrm( v3 v ) { return mul( v, 1.0 / sqrt( dot( v, v ) ) ); }
/* helper_math.h clamp: fmaxf(a, fminf(f, b)) (a NaN argument yields b) */
static inline double clampd( double x, double lo, double hi ) { return fmax( lo, fmin( x, hi ) ); }

typedef struct
{
    v3     center;
    v3     normal;
    double radius;
} circle_t;

/* SesdfContext::getCircleGeometry (sesdf/include/bcs/sesdf/data.cuh:98-114) with
 * getCircleCenter (sesdf/include/bcs/cuda/circles.cuh:9-14). */
static circle_t circle_geometry( v3 ci, double ri, v3 cj, double rj, double rp )
{
    const double R1 = ri + rp, R2 = rj + rp;
    const double d  = dot( sub( ci, cj ), sub( ci, cj ) );
    const double t  = ( R1 * R1 - R2 * R2 + d ) / ( 2.0 * d );
    circle_t     c;
    c.center             = add( ci, mul( sub( cj, ci ), t ) );
    const v3 circleToI   = sub( ci, c.center );
    const double sqDist  = dot( circleToI, circleToI );
    c.radius             = sqrt( R1 * R1 - sqDist );
    c.normal             = nrm( sub( cj, ci ) );
    return c;
}

/* ------------------------------------------------------------------------ */
typedef struct
{
    /* inputs */
    uint32_t n;
    int      mode;
    float    rp;
    uint32_t maxNbr; /* neighbour capacity per atom (reference: 128) */
    uint32_t segCap; /* intersections per circle used by the segment stage */
    float    aabb[ 6 ];

    /* reference grid (sesdf.cu:23-33) */
    float    origin[ 3 ], cell[ 3 ];
    uint32_t gsize;

    uint32_t * perm;  /* sorted id -> original id */
    uint32_t * hash;  /* reference cell hash per sorted atom */
    float *    atoms; /* sorted atoms, xyzr */

    /* neighbour lists, CSR in sorted ids (ascending) */
    uint32_t * noff; /* n + 1 */
    uint32_t * nbr;  /* P */
    uint32_t * slotAtom;
    uint8_t *  status; /* P, after exterior promotion */
    uint8_t *  status0; /* P, before exterior promotion */
    uint64_t   P;

    /* convex patches (full) */
    uint32_t * convex; /* 2n */
    double *   sectors; /* 4V */
    uint64_t   V;
    uint32_t * fullCircles; /* 2F */
    uint64_t   F;

    /* partial (trimmed) circles */
    uint32_t * slotTrim; /* P: exclusive count of partial slots before the slot */
    uint32_t * trimSlot; /* C1: CSR slot of each partial circle */
    uint64_t   C1;

    /* intersections, final order (singular first) */
    uint64_t  I, Q;
    int32_t * ids;    /* 4I: final ids (i, j, k, w) */
    int32_t * cids;   /* 4I: circle ids before the fill (full: trimmed ids; exterior: CSR slots) and w */
    float *   posf;   /* 4I: stored position float4 */
    double *  posd;   /* 4I: FP64 position and condition estimate */

    /* per partial circle (full) */
    uint32_t * ccount, *cstart, *clist;

    /* segments (full) */
    uint64_t   S;
    uint32_t * seg; /* 4S */

    /* singular probe neighbours */
    float *    snbr;    /* 32 * 4 * Q */
    uint32_t * snbrIdx; /* 32 * Q: singular index of each listed neighbour */

    /* exterior tori */
    uint64_t T;
    double * tori; /* 12T: position (c, R), axis (ta, rp), visibility sphere */

    uint64_t counters[ ORA_NCOUNTER ];
} ora_t;

static uint32_t floor_log2( uint64_t v )
{
    uint32_t e = 0;
    while ( v >>= 1 )
        e++;
    return e;
}
static uint32_t next_pow2( uint64_t v )
{
    uint64_t i = 1;
    while ( v > i )
        i <<= 1;
    return (uint32_t)i;
}

/* GridInfo::getGridPosition (sesdf/include/bcs/cuda/grid.inl:8-15), IEEE float32 */
static void grid_position( const ora_t * o, float x, float y, float z, int g[ 3 ] )
{
    g[ 0 ] = (int)floorf( ( x - o->origin[ 0 ] ) / o->cell[ 0 ] );
    g[ 1 ] = (int)floorf( ( y - o->origin[ 1 ] ) / o->cell[ 1 ] );
    g[ 2 ] = (int)floorf( ( z - o->origin[ 2 ] ) / o->cell[ 2 ] );
}
/* GridInfo::getHash (grid.inl:22-28): wrapping power-of-two grid */
static uint32_t grid_hash( const ora_t * o, const int g[ 3 ] )
{
    const int s = (int)o->gsize;
    const int x = g[ 0 ] & ( s - 1 ), y = g[ 1 ] & ( s - 1 ), z = g[ 2 ] & ( s - 1 );
    return (uint32_t)( z * s * s + y * s + x );
}

/* ---- stage A1: reference grid and stable hash sort ------------------------
 * Sesdf::Sesdf (sesdf/src/sesdf/sesdf.cu:23-33) and AccelerationGrid::build
 * (sesdf/src/cuda/grid.cu:99-132): hash per atom, stable radix sort by hash,
 * atoms reordered; every later id is a sorted id (operations.inl:23-24). */
static void stage_sort( ora_t * o, const float * in )
{
    const float maxVdw = 3.48f;
    for ( int a = 0; a < 3; a++ )
    {
        o->origin[ a ]     = ( o->aabb[ a ] - maxVdw ) - o->rp;
        const float size   = fabsf( ( ( o->aabb[ 3 + a ] + maxVdw ) + o->rp ) - o->origin[ a ] );
        o->gsize           = next_pow2( floor_log2( o->n ) );
        o->cell[ a ]       = size / (float)o->gsize;
    }
    uint32_t * h = (uint32_t *)malloc( sizeof( uint32_t ) * ( o->n ? o->n : 1 ) );
    for ( uint32_t i = 0; i < o->n; i++ )
    {
        int g[ 3 ];
        grid_position( o, in[ 4 * i ], in[ 4 * i + 1 ], in[ 4 * i + 2 ], g );
        if ( g[ 0 ] < 0 || g[ 1 ] < 0 || g[ 2 ] < 0 || g[ 0 ] >= (int)o->gsize || g[ 1 ] >= (int)o->gsize
             || g[ 2 ] >= (int)o->gsize )
            o->counters[ GRID_OUTSIDE ]++;
        h[ i ] = grid_hash( o, g );
    }
    /* stable counting sort by hash */
    const uint32_t cells = o->gsize * o->gsize * o->gsize;
    uint32_t *     cnt   = (uint32_t *)calloc( cells + 1, sizeof( uint32_t ) );
    for ( uint32_t i = 0; i < o->n; i++ )
        cnt[ h[ i ] + 1 ]++;
    for ( uint32_t c = 0; c < cells; c++ )
        cnt[ c + 1 ] += cnt[ c ];
    for ( uint32_t i = 0; i < o->n; i++ )
    {
        const uint32_t s = cnt[ h[ i ] ]++;
        o->perm[ s ]     = i;
    }
    for ( uint32_t s = 0; s < o->n; s++ )
    {
        const uint32_t i = o->perm[ s ];
        memcpy( o->atoms + 4 * s, in + 4 * i, 4 * sizeof( float ) );
        o->hash[ s ] = h[ i ];
    }
    free( cnt );
    free( h );
}

static inline v3 atom_pos( const ora_t * o, uint32_t i )
{
    return mk( o->atoms[ 4 * i ], o->atoms[ 4 * i + 1 ], o->atoms[ 4 * i + 2 ] );
}
static inline double atom_r( const ora_t * o, uint32_t i ) { return (double)o->atoms[ 4 * i + 3 ]; }

/* ---- stage A2: neighbour lists --------------------------------------------
 * findCirclesBetweenAtoms / findCirclesInCell (sesdf/src/sesdf/operations.cu:34-124):
 * j is a neighbour of i iff |ci - cj|^2 - ((ri + rp) + (rj + rp))^2 <= 1e-4 and
 * j lies in the reference's cell stencil around i. The list is in ascending
 * sorted id (the order in which the reference visits cells and atoms) and is
 * truncated at maxNbr entries. A finer grid is used here only to find the
 * candidates; the predicate and order are the reference's. */
typedef struct
{
    double     h;
    double     org[ 3 ];
    int        dim[ 3 ];
    uint32_t * start; /* cells + 1 */
    uint32_t * items; /* sorted ids, ascending within a cell */
} fine_grid_t;

static void fine_cell( const fine_grid_t * g, double x, double y, double z, int c[ 3 ] )
{
    const double p[ 3 ] = { x, y, z };
    for ( int a = 0; a < 3; a++ )
    {
        int k = (int)floor( ( p[ a ] - g->org[ a ] ) / g->h );
        if ( k < 0 )
            k = 0;
        if ( k >= g->dim[ a ] )
            k = g->dim[ a ] - 1;
        c[ a ] = k;
    }
}

static void fine_build( fine_grid_t * g, const float * pts, uint32_t count, double h )
{
    double lo[ 3 ] = { 1e300, 1e300, 1e300 }, hi[ 3 ] = { -1e300, -1e300, -1e300 };
    for ( uint32_t i = 0; i < count; i++ )
        for ( int a = 0; a < 3; a++ )
        {
            const double v = pts[ 4 * i + a ];
            lo[ a ]        = v < lo[ a ] ? v : lo[ a ];
            hi[ a ]        = v > hi[ a ] ? v : hi[ a ];
        }
    if ( count == 0 )
        for ( int a = 0; a < 3; a++ )
            lo[ a ] = hi[ a ] = 0.0;
    g->h = h;
    size_t cells = 1;
    for ( int a = 0; a < 3; a++ )
    {
        g->org[ a ] = lo[ a ] - h;
        g->dim[ a ] = (int)( ( hi[ a ] - lo[ a ] ) / h ) + 3;
        cells *= (size_t)g->dim[ a ];
    }
    g->start = (uint32_t *)calloc( cells + 1, sizeof( uint32_t ) );
    g->items = (uint32_t *)malloc( sizeof( uint32_t ) * ( count ? count : 1 ) );
    uint32_t * cellOf = (uint32_t *)malloc( sizeof( uint32_t ) * ( count ? count : 1 ) );
    for ( uint32_t i = 0; i < count; i++ )
    {
        int c[ 3 ];
        fine_cell( g, pts[ 4 * i ], pts[ 4 * i + 1 ], pts[ 4 * i + 2 ], c );
        cellOf[ i ] = (uint32_t)( ( (size_t)c[ 2 ] * g->dim[ 1 ] + c[ 1 ] ) * g->dim[ 0 ] + c[ 0 ] );
        g->start[ cellOf[ i ] + 1 ]++;
    }
    for ( size_t c = 0; c < cells; c++ )
        g->start[ c + 1 ] += g->start[ c ];
    uint32_t * fill = (uint32_t *)malloc( sizeof( uint32_t ) * ( cells + 1 ) );
    memcpy( fill, g->start, sizeof( uint32_t ) * ( cells + 1 ) );
    for ( uint32_t i = 0; i < count; i++ )
        g->items[ fill[ cellOf[ i ] ]++ ] = i;
    free( fill );
    free( cellOf );
}

static void fine_free( fine_grid_t * g )
{
    free( g->start );
    free( g->items );
}

static int cmp_u32( const void * a, const void * b )
{
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : ( x > y ? 1 : 0 );
}

/* candidates of atom i that pass the reference predicate, ascending; returns count */
static uint32_t neighbors_of( const ora_t * o, const fine_grid_t * g, uint32_t i, uint32_t * buf, uint32_t bufCap,
                              uint64_t * bandCount )
{
    const v3     ci = atom_pos( o, i );
    const double rp = o->rp;
    const double Ri = atom_r( o, i ) + rp;
    int          c[ 3 ];
    fine_cell( g, ci.x, ci.y, ci.z, c );

    /* reference stencil (operations.cu:78-84) */
    int gp[ 3 ];
    grid_position( o, o->atoms[ 4 * i ], o->atoms[ 4 * i + 1 ], o->atoms[ 4 * i + 2 ], gp );
    const float range = ( o->atoms[ 4 * i + 3 ] + 3.48f ) + 2.f * o->rp;
    int         lo[ 3 ], hi[ 3 ];
    for ( int a = 0; a < 3; a++ )
    {
        int r = (int)ceilf( range / o->cell[ a ] );
        if ( r < 1 )
            r = 1;
        lo[ a ] = gp[ a ] - r < 0 ? 0 : gp[ a ] - r;
        hi[ a ] = gp[ a ] + r > (int)o->gsize - 1 ? (int)o->gsize - 1 : gp[ a ] + r;
    }

    uint32_t count = 0;
    for ( int dz = -1; dz <= 1; dz++ )
        for ( int dy = -1; dy <= 1; dy++ )
            for ( int dx = -1; dx <= 1; dx++ )
            {
                const int x = c[ 0 ] + dx, y = c[ 1 ] + dy, z = c[ 2 ] + dz;
                if ( x < 0 || y < 0 || z < 0 || x >= g->dim[ 0 ] || y >= g->dim[ 1 ] || z >= g->dim[ 2 ] )
                    continue;
                const size_t cell = ( (size_t)z * g->dim[ 1 ] + y ) * g->dim[ 0 ] + x;
                for ( uint32_t q = g->start[ cell ]; q < g->start[ cell + 1 ]; q++ )
                {
                    const uint32_t j = g->items[ q ];
                    if ( j == i )
                        continue;
                    const v3     cj = atom_pos( o, j );
                    const double Rj = atom_r( o, j ) + rp;
                    const double d  = dot( sub( ci, cj ), sub( ci, cj ) );
                    const double R  = Ri + Rj;
                    const double m  = d - R * R - (double)1e-4f;
                    if ( fabs( m ) < kBand * kEps32 * ( d + R * R ) )
                        ( *bandCount )++;
                    if ( !( d - R * R <= (double)1e-4f ) )
                        continue;
                    /* stencil membership of j's (wrapped) cell */
                    int gj[ 3 ];
                    grid_position( o, o->atoms[ 4 * j ], o->atoms[ 4 * j + 1 ], o->atoms[ 4 * j + 2 ], gj );
                    const int s   = (int)o->gsize;
                    int       inb = 1;
                    for ( int a = 0; a < 3; a++ )
                    {
                        const int w = gj[ a ] & ( s - 1 );
                        if ( w < lo[ a ] || w > hi[ a ] )
                            inb = 0;
                    }
                    if ( !inb )
                        continue;
                    if ( count < bufCap )
                        buf[ count ] = j;
                    count++;
                }
            }
    const uint32_t kept = count < bufCap ? count : bufCap;
    qsort( buf, kept, sizeof( uint32_t ), cmp_u32 );
    return count;
}

static void stage_neighbors( ora_t * o )
{
    double rmax = 0.0;
    for ( uint32_t i = 0; i < o->n; i++ )
        rmax = atom_r( o, i ) > rmax ? atom_r( o, i ) : rmax;
    fine_grid_t g;
    fine_build( &g, o->atoms, o->n, 2.0 * ( rmax + (double)o->rp ) + 0.01 );

    uint32_t * cnt = (uint32_t *)calloc( o->n + 1, sizeof( uint32_t ) );
    uint64_t   band = 0, trunc = 0;
#pragma omp parallel reduction( + : band, trunc )
    {
        uint32_t * buf = (uint32_t *)malloc( sizeof( uint32_t ) * 4096 );
#pragma omp for schedule( dynamic, 256 )
        for ( int64_t i = 0; i < (int64_t)o->n; i++ )
        {
            uint64_t       b = 0;
            const uint32_t c = neighbors_of( o, &g, (uint32_t)i, buf, 4096, &b );
            band += b;
            cnt[ i ] = c < o->maxNbr ? c : o->maxNbr;
            if ( c > o->maxNbr )
                trunc++;
        }
        free( buf );
    }
    o->counters[ BAND_NEIGHBOR ] += band;
    o->counters[ NBR_TRUNCATED ] += trunc;
    o->noff = (uint32_t *)malloc( sizeof( uint32_t ) * ( o->n + 1 ) );
    uint64_t acc = 0;
    for ( uint32_t i = 0; i < o->n; i++ )
    {
        o->noff[ i ] = (uint32_t)acc;
        acc += cnt[ i ];
    }
    o->noff[ o->n ] = (uint32_t)acc;
    o->P            = acc;
    o->nbr          = (uint32_t *)malloc( sizeof( uint32_t ) * ( acc ? acc : 1 ) );
    o->slotAtom     = (uint32_t *)malloc( sizeof( uint32_t ) * ( acc ? acc : 1 ) );
#pragma omp parallel
    {
        uint32_t * buf = (uint32_t *)malloc( sizeof( uint32_t ) * 4096 );
#pragma omp for schedule( dynamic, 256 )
        for ( int64_t i = 0; i < (int64_t)o->n; i++ )
        {
            uint64_t b = 0;
            neighbors_of( o, &g, (uint32_t)i, buf, 4096, &b );
            memcpy( o->nbr + o->noff[ i ], buf, sizeof( uint32_t ) * cnt[ i ] );
            for ( uint32_t s = 0; s < cnt[ i ]; s++ )
                o->slotAtom[ o->noff[ i ] + s ] = (uint32_t)i;
        }
        free( buf );
    }
    free( cnt );
    fine_free( &g );
}

/* ---- stage B: circle visibility --------------------------------------------
 * computeCirclesVisibilityStatus (full: sesdf/src/sesdf/operations.cu:126-204;
 * exterior: sesdf/src/ssesdf/operations.cu:169-244). Status of the directed
 * circle (i, j): 0 buried (some k's SAS sphere holds the whole circle),
 * 1 partial, 2 complete (no k touches it). The exterior build evaluates only
 * i < j; its j < i slots are left unwritten by the reference and are 0 here. */
static uint8_t circle_status( const ora_t * o, uint32_t i, uint32_t s, uint64_t * bandB, uint64_t * bandC )
{
    const double   rp   = o->rp;
    const uint32_t base = o->noff[ i ];
    const uint32_t ni   = o->noff[ i + 1 ] - base;
    const uint32_t j    = o->nbr[ base + s ];
    const circle_t c    = circle_geometry( atom_pos( o, i ), atom_r( o, i ), atom_pos( o, j ), atom_r( o, j ), rp );
    int            isVisible = 1, isComplete = 1;
    for ( uint32_t k = 0; k < ni; k++ )
    {
        if ( k == s )
            continue;
        const uint32_t kid            = o->nbr[ base + k ];
        const double   Rk             = atom_r( o, kid ) + rp;
        const v3       kToCircle      = sub( c.center, atom_pos( o, kid ) );
        const double   distToCircle   = sqrt( dot( kToCircle, kToCircle ) );
        const double   secondDistance = dot( kToCircle, c.normal );
        const double   cosTheta       = secondDistance / distToCircle;
        const double   sinTheta       = sqrt( 1.0 - cosTheta * cosTheta );
        {
            const double firstDistance    = sinTheta * distToCircle + c.radius;
            const double completeDistance = firstDistance * firstDistance + secondDistance * secondDistance;
            const double m                = completeDistance - Rk * Rk - (double)1e-4f;
            if ( fabs( m ) < kBand * kEps32 * ( completeDistance + Rk * Rk ) )
                ( *bandB )++;
            if ( completeDistance - Rk * Rk < (double)1e-4f )
            {
                isVisible = 0;
                break;
            }
        }
        if ( isComplete )
        {
            const double firstDistance    = ( -sinTheta ) * distToCircle + c.radius;
            const double completeDistance = firstDistance * firstDistance + secondDistance * secondDistance;
            const double m                = completeDistance - Rk * Rk - (double)1e-4f;
            if ( fabs( m ) < kBand * kEps32 * ( completeDistance + Rk * Rk + 2.0 * distToCircle * c.radius ) )
                ( *bandC )++;
            if ( completeDistance - Rk * Rk < (double)1e-4f )
                isComplete = 0;
        }
    }
    return (uint8_t)( isVisible * ( 1 + isComplete ) );
}

static int32_t find_slot( const ora_t * o, uint32_t atom, uint32_t target );

/* Full build: circles (i, j) and (j, i) are one circle (the intersection of the
 * SAS spheres of i and j), so that, where neither neighbour list is cut at the
 * capacity, the circle is evaluated once, from its lower atom (i < j), and the
 * slot of (j, i) takes that status. Every atom that can touch the circle is a
 * neighbour of both i and j (its SAS sphere reaches a point of both spheres), so
 * the two evaluations of the reference differ only where a test lies within
 * float32 rounding, or the 1e-4 margin, of its threshold. A list cut at the
 * capacity misses neighbours the other side may hold: such circles are
 * evaluated from both sides, as the reference does. */
static int mirrored_circle( const ora_t * o, uint32_t i, uint32_t j )
{
    return o->mode == ORA_MODE_FULL && j < i && o->noff[ i + 1 ] - o->noff[ i ] < o->maxNbr &&
           o->noff[ j + 1 ] - o->noff[ j ] < o->maxNbr;
}

static void stage_visibility( ora_t * o )
{
    o->status  = (uint8_t *)calloc( o->P ? o->P : 1, 1 );
    o->status0 = (uint8_t *)calloc( o->P ? o->P : 1, 1 );
    uint64_t bandB = 0, bandC = 0;
#pragma omp parallel for schedule( dynamic, 64 ) reduction( + : bandB, bandC )
    for ( int64_t i = 0; i < (int64_t)o->n; i++ )
    {
        const uint32_t base = o->noff[ i ], ni = o->noff[ i + 1 ] - base;
        for ( uint32_t s = 0; s < ni; s++ )
        {
            const uint32_t j = o->nbr[ base + s ];
            if ( o->mode == ORA_MODE_EXTERIOR && !( (uint32_t)i < j ) )
                continue;
            if ( mirrored_circle( o, (uint32_t)i, j ) )
                continue;
            uint64_t b = 0, c = 0;
            o->status[ base + s ] = circle_status( o, (uint32_t)i, s, &b, &c );
            bandB += b;
            bandC += c;
        }
    }
#pragma omp parallel for schedule( dynamic, 256 )
    for ( int64_t i = 0; i < (int64_t)o->n; i++ )
    {
        const uint32_t base = o->noff[ i ], ni = o->noff[ i + 1 ] - base;
        for ( uint32_t s = 0; s < ni; s++ )
        {
            const uint32_t j = o->nbr[ base + s ];
            if ( !mirrored_circle( o, (uint32_t)i, j ) )
                continue;
            /* both lists are complete and the neighbour predicate is symmetric: i is in N(j) */
            const int32_t t       = find_slot( o, j, (uint32_t)i );
            o->status[ base + s ] = t >= 0 ? o->status[ o->noff[ j ] + (uint32_t)t ] : 0;
        }
    }
    o->counters[ BAND_BURIED ] += bandB;
    o->counters[ BAND_COMPLETE ] += bandC;
}

/* ---- stage C: convex sectors, full circles, partial-circle numbering -------
 * buildConvexPatchesSectors (sesdf/include/bcs/sesdf/operations.inl:175-228),
 * orthogonalVector (sesdf/include/bcs/cuda/math.cuh:32-38), the scans of
 * findCircles (operations.inl:46-67) and the full-circle append
 * (operations.cu:200-201; here in (i, slot) order instead of atomic order). */
static void stage_convex( ora_t * o )
{
    const double rp = o->rp;
    /* partial circles: status 1 and i < j, in (i, slot) order */
    o->slotTrim = (uint32_t *)malloc( sizeof( uint32_t ) * ( o->P ? o->P : 1 ) );
    uint64_t c1 = 0, F = 0, V = 0;
    for ( uint64_t p = 0; p < o->P; p++ )
    {
        o->slotTrim[ p ]  = (uint32_t)c1;
        const uint32_t i  = o->slotAtom[ p ];
        const uint32_t j  = o->nbr[ p ];
        const uint8_t  st = o->status[ p ];
        if ( st == 1 && i < j )
            c1++;
        if ( st == 2 && i < j )
            F++;
        if ( st != 0 )
            V++;
    }
    o->C1          = c1;
    o->F           = F;
    o->trimSlot    = (uint32_t *)malloc( sizeof( uint32_t ) * ( c1 ? c1 : 1 ) );
    o->fullCircles = (uint32_t *)malloc( sizeof( uint32_t ) * 2 * ( F ? F : 1 ) );
    uint64_t t = 0, f = 0;
    for ( uint64_t p = 0; p < o->P; p++ )
    {
        const uint32_t i = o->slotAtom[ p ], j = o->nbr[ p ];
        if ( o->status[ p ] == 1 && i < j )
            o->trimSlot[ t++ ] = (uint32_t)p;
        if ( o->status[ p ] == 2 && i < j )
        {
            o->fullCircles[ 2 * f ]     = i;
            o->fullCircles[ 2 * f + 1 ] = j;
            f++;
        }
    }
    if ( o->mode != ORA_MODE_FULL )
        return;

    o->V       = V;
    o->sectors = (double *)malloc( sizeof( double ) * 4 * ( V ? V : 1 ) );
    o->convex  = (uint32_t *)malloc( sizeof( uint32_t ) * 2 * ( o->n ? o->n : 1 ) );
    uint64_t acc = 0, bandOrtho = 0;
    for ( uint32_t i = 0; i < o->n; i++ )
    {
        const uint32_t base = o->noff[ i ], ni = o->noff[ i + 1 ] - base;
        o->convex[ 2 * i ]  = (uint32_t)acc;
        const v3     ci     = atom_pos( o, i );
        const double rirp   = atom_r( o, i ) + rp;
        const double sqrirp = rirp * rirp;
        for ( uint32_t s = 0; s < ni; s++ )
        {
            if ( o->status[ base + s ] == 0 )
                continue;
            const uint32_t j      = o->nbr[ base + s ];
            const v3       cj     = atom_pos( o, j );
            const circle_t geo    = circle_geometry( ci, atom_r( o, i ), cj, atom_r( o, j ), rp );
            const v3       cijci  = sub( ci, geo.center );
            const double   radius = sqrt( sqrirp - dot( cijci, cijci ) );
            const v3       cicj   = nrm( sub( cj, ci ) );
            v3             ref    = mk( 1.0, 0.0, 0.0 );
            const double   ax     = fabs( dot( cicj, ref ) );
            if ( fabs( ax - ( 1.0 - (double)1e-4f ) ) < kBand * kEps32 )
                bandOrtho++;
            if ( ax > 1.0 - (double)1e-4f )
                ref = mk( 0.0, 1.0, 0.0 );
            const v3 nn = nrm( cross( cicj, ref ) );
            const v3 x  = add( geo.center, mul( nn, radius ) );
            double * dst = o->sectors + 4 * acc;
            dst[ 0 ]     = cicj.x;
            dst[ 1 ]     = cicj.y;
            dst[ 2 ]     = cicj.z;
            dst[ 3 ]     = acos( clampd( dot( cicj, mul( sub( x, ci ), 1.0 / rirp ) ), -1.0, 1.0 ) );
            acc++;
        }
        o->convex[ 2 * i + 1 ] = (uint32_t)acc;
    }
    o->counters[ BAND_ORTHO ] += bandOrtho;
}

/* ---- stage D: circle intersections (concave probes) ------------------------
 * findIntersectionsBetweenCircles (full: sesdf/include/bcs/sesdf/operations.inl:230-486;
 * exterior: sesdf/include/bcs/ssesdf/operation.inl:100-351). For each partial
 * circle (i, j) and each k in N(i) with k > j, (i, k) partial and k in N(j):
 * the two points at distance R_i, R_j, R_k from the three centres, kept when
 * outside every other SAS sphere of N(i); singular when closer than rp to the
 * plane of the three centres. Order here: partial circle, then k in slot
 * order, then x1 before x2 (the reference appends in atomic order). */
typedef struct
{
    uint32_t t;      /* trimmed id of (i, j) */
    uint32_t slotJK; /* CSR slot of (j, k) */
    uint32_t slotIK; /* CSR slot of (i, k) */
    int32_t  w;      /* +-(1 + singular) */
    double   x[ 3 ];
    double   cond;
} probe_t;

typedef struct
{
    probe_t * v;
    size_t    n, cap;
} probe_vec_t;

static void pv_push( probe_vec_t * pv, const probe_t * p )
{
    if ( pv->n == pv->cap )
    {
        pv->cap = pv->cap ? 2 * pv->cap : 16;
        pv->v   = (probe_t *)realloc( pv->v, sizeof( probe_t ) * pv->cap );
    }
    pv->v[ pv->n++ ] = *p;
}

static int32_t find_slot( const ora_t * o, uint32_t atom, uint32_t target )
{
    uint32_t lo = o->noff[ atom ], hi = o->noff[ atom + 1 ];
    while ( lo < hi )
    {
        const uint32_t mid = ( lo + hi ) / 2;
        if ( o->nbr[ mid ] < target )
            lo = mid + 1;
        else
            hi = mid;
    }
    if ( lo < o->noff[ atom + 1 ] && o->nbr[ lo ] == target )
        return (int32_t)( lo - o->noff[ atom ] );
    return -1;
}

static void circle_intersections( const ora_t * o, uint32_t t, probe_vec_t * out, uint64_t * counters )
{
    const double   rp    = o->rp;
    const uint32_t slot  = o->trimSlot[ t ];
    const uint32_t i     = o->slotAtom[ slot ];
    const uint32_t base  = o->noff[ i ];
    const uint32_t ni    = o->noff[ i + 1 ] - base;
    const uint32_t sj    = slot - base;
    const uint32_t j     = o->nbr[ slot ];
    const v3       ci    = atom_pos( o, i );
    const double   ri    = atom_r( o, i );
    const v3       cj    = atom_pos( o, j );
    const double   Ri    = ri + rp;
    const double   Rj    = atom_r( o, j ) + rp;
    const double   Ri2   = Ri * Ri;
    const v3       a     = sub( cj, ci );
    const double   aa    = dot( a, a );
    const double   p     = ( aa + Ri2 - Rj * Rj ) * 0.5;
    for ( uint32_t sk = 0; sk < ni; sk++ )
    {
        const uint32_t k = o->nbr[ base + sk ];
        if ( !( j < k ) )
            continue;
        if ( o->status0[ base + sk ] != 1 )
            continue;
        const int32_t sjk = find_slot( o, j, k );
        if ( sjk < 0 )
            continue;
        /* The points at distance R_i, R_j, R_k from the centres, in closed form
         * (the reference intersects the circles (i, j), (i, k) for the same
         * points, operations.inl:384-398): with a = c_j - c_i, b = c_k - c_i and
         * n = a x b, x = c_i + y0 +- n sqrt(tt / |n|^2), where
         * y0 = (p (b x n) + q (n x a)) / |n|^2 lies in the plane of the centres
         * (a . y0 = p = (|a|^2 + R_i^2 - R_j^2) / 2, b . y0 = q likewise) and
         * tt = R_i^2 - |y0|^2 is the squared height of the points over that plane. */
        const v3       ck  = atom_pos( o, k );
        const double   Rk  = atom_r( o, k ) + rp;
        const v3       b   = sub( ck, ci );
        const v3       n   = cross( a, b );
        const double   bb  = dot( b, b );
        const double   q   = ( bb + Ri2 - Rk * Rk ) * 0.5;
        const double   inv = 1.0 / dot( n, n );
        const v3       y0  = mul( add( mul( cross( b, n ), p ), mul( cross( n, a ), q ) ), inv );
        const double   tt  = Ri2 - dot( y0, y0 );
        const double   den = dot( n, n ) / ( aa * bb ); /* sin^2 of the angle at c_i (diagnostics) */
        const double   cond = 1.0 / fabs( den ) + ( tt > 0.0 ? sqrt( Ri2 ) / sqrt( tt ) : 1e30 );
        if ( fabs( tt ) < kBand * kEps32 * Ri2 * ( 1.0 / fabs( den ) ) )
            counters[ BAND_PROBE_T ]++;
        if ( !( tt >= 0.0 ) )
            continue;
        if ( cond > 1e3 )
            counters[ ILL_CONDITIONED ]++;
        const double s    = sqrt( tt * inv );
        const v3     xc   = add( ci, y0 );
        const v3     x1   = add( xc, mul( n, s ) );
        const v3     x2   = sub( xc, mul( n, s ) );
        int          vis1 = 1, vis2 = 1;
        for ( uint32_t sl = 0; sl < ni && ( vis1 || vis2 ); sl++ )
        {
            if ( sl == sj || sl == sk )
                continue;
            const uint32_t l  = o->nbr[ base + sl ];
            const v3       cl = atom_pos( o, l );
            double         Rl = atom_r( o, l ) + rp;
            Rl *= Rl;
            const double m1 = dot( sub( cl, x1 ), sub( cl, x1 ) ) - Rl;
            const double m2 = dot( sub( cl, x2 ), sub( cl, x2 ) ) - Rl;
            if ( vis1 && fabs( m1 ) < kBand * kEps32 * ( m1 + 2.0 * Rl ) * cond )
                counters[ BAND_OCCLUSION ]++;
            if ( vis2 && fabs( m2 ) < kBand * kEps32 * ( m2 + 2.0 * Rl ) * cond )
                counters[ BAND_OCCLUSION ]++;
            vis1 = vis1 && m1 > 0.0;
            vis2 = vis2 && m2 > 0.0;
        }
        if ( !vis1 && !vis2 )
            continue;
        /* singular (operations.inl:441-451): d^2 - rp^2 < -1e-4 with d the
         * distance of the point from the plane of the centres, d^2 = tt */
        for ( int side = 0; side < 2; side++ )
        {
            if ( side == 0 && !vis1 )
                continue;
            if ( side == 1 && !vis2 )
                continue;
            const v3     x  = side == 0 ? x1 : x2;
            const double ms = tt - (double)rp * rp - ( -(double)1e-4f );
            if ( fabs( ms ) < kBand * kEps32 * ( tt + (double)rp * rp ) * cond )
                counters[ BAND_SINGULAR ]++;
            const int singular = tt - (double)rp * rp < -(double)1e-4f;
            probe_t   p;
            p.t      = t;
            p.slotJK = o->noff[ j ] + (uint32_t)sjk;
            p.slotIK = base + sk;
            p.w      = ( side == 0 ? 1 : -1 ) * ( 1 + singular );
            p.x[ 0 ] = x.x;
            p.x[ 1 ] = x.y;
            p.x[ 2 ] = x.z;
            p.cond   = cond;
            pv_push( out, &p );
        }
    }
}

/* pseudo-angle with the order of angleBetweenEdges
 * (sesdf/include/bcs/cuda/circles.cuh:27-31): theta = acos(u.v / |u||v|),
 * angle = theta if sign(det(u, v, n)) > 0 else 2 pi - theta. The key
 * (1 - cos) or (3 + cos) is monotone in that angle and needs no acos. */
static double pseudo_angle( v3 u, v3 v, v3 n )
{
    const double c   = clampd( dot( u, v ) / ( sqrt( dot( u, u ) ) * sqrt( dot( v, v ) ) ), -1.0, 1.0 );
    const double det = dot( u, cross( v, n ) );
    return copysign( 1.0, det ) > 0.0 ? 1.0 - c : 3.0 + c;
}

static int cmp_key( const void * a, const void * b )
{
    const double * x = (const double *)a;
    const double * y = (const double *)b;
    if ( x[ 0 ] < y[ 0 ] )
        return -1;
    if ( x[ 0 ] > y[ 0 ] )
        return 1;
    return x[ 1 ] < y[ 1 ] ? -1 : ( x[ 1 ] > y[ 1 ] ? 1 : 0 );
}

static void stage_intersections( ora_t * o )
{
    const double rp = o->rp;
    memcpy( o->status0, o->status, o->P );

    /* per partial circle, in parallel, then concatenated in circle order */
    probe_vec_t * per  = (probe_vec_t *)calloc( o->C1 ? o->C1 : 1, sizeof( probe_vec_t ) );
    uint64_t      cnts[ ORA_NCOUNTER ];
    memset( cnts, 0, sizeof( cnts ) );
    uint64_t bT = 0, bO = 0, bS = 0, bIll = 0;
#pragma omp parallel for schedule( dynamic, 64 ) reduction( + : bT, bO, bS, bIll )
    for ( int64_t t = 0; t < (int64_t)o->C1; t++ )
    {
        uint64_t c[ ORA_NCOUNTER ];
        memset( c, 0, sizeof( c ) );
        circle_intersections( o, (uint32_t)t, &per[ t ], c );
        bT += c[ BAND_PROBE_T ];
        bO += c[ BAND_OCCLUSION ];
        bS += c[ BAND_SINGULAR ];
        bIll += c[ ILL_CONDITIONED ];
    }
    o->counters[ BAND_PROBE_T ] += bT;
    o->counters[ BAND_OCCLUSION ] += bO;
    o->counters[ BAND_SINGULAR ] += bS;
    o->counters[ ILL_CONDITIONED ] += bIll;

    uint64_t total = 0, nsing = 0;
    for ( uint64_t t = 0; t < o->C1; t++ )
    {
        total += per[ t ].n;
        for ( size_t q = 0; q < per[ t ].n; q++ )
            nsing += ( per[ t ].v[ q ].w == 2 || per[ t ].v[ q ].w == -2 );
    }
    o->I    = total;
    o->Q    = nsing;
    o->ids  = (int32_t *)malloc( sizeof( int32_t ) * 4 * ( total ? total : 1 ) );
    o->cids = (int32_t *)malloc( sizeof( int32_t ) * 4 * ( total ? total : 1 ) );
    o->posf = (float *)malloc( sizeof( float ) * 4 * ( total ? total : 1 ) );
    o->posd = (double *)malloc( sizeof( double ) * 4 * ( total ? total : 1 ) );

    /* stable partition: singular probes (|w| == 2) first
     * (operations.inl:128-135 uses an unstable sort for the same purpose) */
    uint64_t a = 0, b = nsing;
    for ( uint64_t t = 0; t < o->C1; t++ )
        for ( size_t q = 0; q < per[ t ].n; q++ )
        {
            const probe_t * p   = &per[ t ].v[ q ];
            const int       sng = p->w == 2 || p->w == -2;
            const uint64_t  idx = sng ? a++ : b++;
            const uint32_t  sij = o->trimSlot[ p->t ];
            const uint32_t  i   = o->slotAtom[ sij ];
            const uint32_t  j   = o->nbr[ sij ];
            const uint32_t  k   = o->nbr[ p->slotIK ];
            if ( o->mode == ORA_MODE_FULL )
            {
                o->cids[ 4 * idx + 0 ] = (int32_t)p->t;
                o->cids[ 4 * idx + 1 ] = (int32_t)o->slotTrim[ p->slotJK ];
                o->cids[ 4 * idx + 2 ] = (int32_t)o->slotTrim[ p->slotIK ];
            }
            else
            {
                o->cids[ 4 * idx + 0 ] = (int32_t)sij;
                o->cids[ 4 * idx + 1 ] = (int32_t)p->slotIK;
                o->cids[ 4 * idx + 2 ] = (int32_t)p->slotJK;
            }
            o->cids[ 4 * idx + 3 ] = p->w;
            o->ids[ 4 * idx + 0 ]  = (int32_t)i;
            o->ids[ 4 * idx + 1 ]  = (int32_t)j;
            o->ids[ 4 * idx + 2 ]  = (int32_t)k;
            o->ids[ 4 * idx + 3 ]  = 0;
            o->posd[ 4 * idx + 0 ] = p->x[ 0 ];
            o->posd[ 4 * idx + 1 ] = p->x[ 1 ];
            o->posd[ 4 * idx + 2 ] = p->x[ 2 ];
            o->posd[ 4 * idx + 3 ] = p->cond;
            o->posf[ 4 * idx + 0 ] = (float)p->x[ 0 ];
            o->posf[ 4 * idx + 1 ] = (float)p->x[ 1 ];
            o->posf[ 4 * idx + 2 ] = (float)p->x[ 2 ];
            o->posf[ 4 * idx + 3 ] = (float)p->w;
        }
    for ( uint64_t t = 0; t < o->C1; t++ )
        free( per[ t ].v );
    free( per );

    if ( o->mode == ORA_MODE_EXTERIOR )
    {
        /* ssesdf fillIntersections (sesdf/src/ssesdf/operations.cu:287-329):
         * the three circles of each probe move from status 1 to 2 */
        for ( uint64_t q = 0; q < o->I; q++ )
            for ( int c = 0; c < 3; c++ )
            {
                const uint32_t s = (uint32_t)o->cids[ 4 * q + c ];
                if ( o->status[ s ] == 1 )
                    o->status[ s ] = 2;
            }
        return;
    }

    /* sesdf fillIntersections (sesdf/src/sesdf/operations.cu:206-269): per
     * partial circle, the list of probes lying on it (here in ascending probe
     * index; the reference fills it with atomics) */
    o->ccount = (uint32_t *)calloc( o->C1 ? o->C1 : 1, sizeof( uint32_t ) );
    o->cstart = (uint32_t *)calloc( o->C1 + 1, sizeof( uint32_t ) );
    for ( uint64_t q = 0; q < o->I; q++ )
        for ( int c = 0; c < 3; c++ )
            o->ccount[ o->cids[ 4 * q + c ] ]++;
    for ( uint64_t t = 0; t < o->C1; t++ )
        o->cstart[ t + 1 ] = o->cstart[ t ] + o->ccount[ t ];
    o->clist       = (uint32_t *)malloc( sizeof( uint32_t ) * ( 3 * o->I + 1 ) );
    uint32_t * put = (uint32_t *)calloc( o->C1 ? o->C1 : 1, sizeof( uint32_t ) );
    for ( uint64_t q = 0; q < o->I; q++ )
        for ( int c = 0; c < 3; c++ )
        {
            const uint32_t t                       = (uint32_t)o->cids[ 4 * q + c ];
            o->clist[ o->cstart[ t ] + put[ t ]++ ] = (uint32_t)q;
        }
    free( put );

    /* ---- stage F: segments (buildSegments, operations.inl:552-668) ------- */
    uint64_t S = 0, segTrunc = 0;
    for ( uint64_t t = 0; t < o->C1; t++ )
    {
        uint32_t c = o->ccount[ t ];
        if ( c > o->segCap )
        {
            segTrunc++;
            c = o->segCap;
        }
        S += c / 2;
    }
    o->counters[ SEG_TRUNCATED ] += segTrunc;
    o->S           = S;
    o->seg         = (uint32_t *)malloc( sizeof( uint32_t ) * 4 * ( S ? S : 1 ) );
    uint64_t out   = 0, ties = 0;
    double * keys  = (double *)malloc( sizeof( double ) * 2 * ( o->segCap + 1 ) );
    for ( uint64_t t = 0; t < o->C1; t++ )
    {
        uint32_t nb = o->ccount[ t ];
        if ( nb > o->segCap )
            nb = o->segCap;
        if ( nb < 2 )
            continue;
        const uint32_t   sij  = o->trimSlot[ t ];
        const uint32_t   i    = o->slotAtom[ sij ];
        const uint32_t   j    = o->nbr[ sij ];
        const circle_t   geo  = circle_geometry( atom_pos( o, i ), atom_r( o, i ), atom_pos( o, j ), atom_r( o, j ), rp );
        const uint32_t * list = o->clist + o->cstart[ t ];
        const uint32_t   st   = list[ 0 ];
        const int        isSecondary = ( (int32_t)i == o->ids[ 4 * st ] && (int32_t)j == o->ids[ 4 * st + 2 ] );
        const double     direction   = copysign( 1.0, (double)o->posf[ 4 * st + 3 ] ) * ( isSecondary ? -1.0 : 1.0 );
        const v3 startPos = mk( o->posf[ 4 * st ], o->posf[ 4 * st + 1 ], o->posf[ 4 * st + 2 ] );
        const v3 ref      = sub( startPos, geo.center );
        keys[ 0 ]         = 0.0;
        keys[ 1 ]         = 0.0;
        for ( uint32_t m = 1; m < nb; m++ )
        {
            const uint32_t q  = list[ m ];
            const v3       cp = mk( o->posf[ 4 * q ], o->posf[ 4 * q + 1 ], o->posf[ 4 * q + 2 ] );
            v3             v1 = ref;
            v3             v2 = nrm( sub( cp, geo.center ) );
            if ( direction < 0.0 )
            {
                const v3 tmp = v1;
                v1           = v2;
                v2           = tmp;
            }
            keys[ 2 * m ]     = pseudo_angle( v1, v2, geo.normal );
            keys[ 2 * m + 1 ] = (double)m;
        }
        qsort( keys, nb, 2 * sizeof( double ), cmp_key );
        for ( uint32_t m = 1; m < nb; m++ )
            if ( keys[ 2 * m ] - keys[ 2 * m - 2 ] < 1e-8 )
                ties++;
        for ( uint32_t m = 0; m + 1 < nb; m += 2 )
        {
            uint32_t a1 = list[ (uint32_t)keys[ 2 * m + 1 ] ];
            uint32_t a2 = list[ (uint32_t)keys[ 2 * m + 3 ] ];
            if ( direction < 0.0 )
            {
                const uint32_t tmp = a1;
                a1                 = a2;
                a2                 = tmp;
            }
            o->seg[ 4 * out + 0 ] = i;
            o->seg[ 4 * out + 1 ] = j;
            o->seg[ 4 * out + 2 ] = a1;
            o->seg[ 4 * out + 3 ] = a2;
            out++;
        }
    }
    o->counters[ BAND_ANGLE_TIE ] += ties;
    free( keys );
}

/* ---- stage G: neighbours of singular probes ---------------------------------
 * handleIntersectionSingularities + findIntersectionsNeighbors (full:
 * sesdf/src/sesdf/operations.cu:14-32,271-338; exterior:
 * sesdf/src/ssesdf/operations.cu:57-75,331-399). Over the Q singular probes
 * (stored float positions): neighbours closer than 2 rp, ordered by the
 * reference grid hash of the neighbour then by probe index, at most 32. */
typedef struct
{
    uint32_t hash, idx;
} hk_t;

static int cmp_hk( const void * a, const void * b )
{
    const hk_t * x = (const hk_t *)a;
    const hk_t * y = (const hk_t *)b;
    if ( x->hash != y->hash )
        return x->hash < y->hash ? -1 : 1;
    return x->idx < y->idx ? -1 : ( x->idx > y->idx ? 1 : 0 );
}

static void stage_singular( ora_t * o )
{
    const uint32_t maxN = 32;
    const double   twoRp = 2.0 * (double)o->rp;
    o->snbr              = (float *)calloc( 4 * maxN * ( o->Q ? o->Q : 1 ), sizeof( float ) );
    o->snbrIdx           = (uint32_t *)calloc( maxN * ( o->Q ? o->Q : 1 ), sizeof( uint32_t ) );
    if ( o->Q == 0 )
        return;
    fine_grid_t g;
    fine_build( &g, o->posf, (uint32_t)o->Q, twoRp + 0.01 );
    uint32_t * qhash = (uint32_t *)malloc( sizeof( uint32_t ) * o->Q );
    for ( uint64_t q = 0; q < o->Q; q++ )
    {
        int gp[ 3 ];
        grid_position( o, o->posf[ 4 * q ], o->posf[ 4 * q + 1 ], o->posf[ 4 * q + 2 ], gp );
        qhash[ q ] = grid_hash( o, gp );
    }
    uint64_t band = 0, trunc = 0;
#pragma omp parallel reduction( + : band, trunc )
    {
        hk_t * buf = (hk_t *)malloc( sizeof( hk_t ) * 65536 );
#pragma omp for schedule( dynamic, 64 )
        for ( int64_t q = 0; q < (int64_t)o->Q; q++ )
        {
            const float * pq = o->posf + 4 * q;
            int           c[ 3 ];
            fine_cell( &g, pq[ 0 ], pq[ 1 ], pq[ 2 ], c );
            uint32_t found = 0;
            for ( int dz = -1; dz <= 1; dz++ )
                for ( int dy = -1; dy <= 1; dy++ )
                    for ( int dx = -1; dx <= 1; dx++ )
                    {
                        const int x = c[ 0 ] + dx, y = c[ 1 ] + dy, z = c[ 2 ] + dz;
                        if ( x < 0 || y < 0 || z < 0 || x >= g.dim[ 0 ] || y >= g.dim[ 1 ] || z >= g.dim[ 2 ] )
                            continue;
                        const size_t cell = ( (size_t)z * g.dim[ 1 ] + y ) * g.dim[ 0 ] + x;
                        for ( uint32_t e = g.start[ cell ]; e < g.start[ cell + 1 ]; e++ )
                        {
                            const uint32_t p = g.items[ e ];
                            if ( p == (uint32_t)q )
                                continue;
                            const float * pp = o->posf + 4 * p;
                            const v3      dv = mk( (double)pq[ 0 ] - pp[ 0 ], (double)pq[ 1 ] - pp[ 1 ], (double)pq[ 2 ] - pp[ 2 ] );
                            const double  d  = sqrt( dot( dv, dv ) );
                            if ( fabs( d - twoRp ) < kBand * kEps32 * twoRp )
                                band++;
                            if ( !( d < twoRp ) )
                                continue;
                            if ( found < 65536 )
                            {
                                buf[ found ].hash = qhash[ p ];
                                buf[ found ].idx  = p;
                            }
                            found++;
                        }
                    }
            const uint32_t kept = found < 65536 ? found : 65536;
            qsort( buf, kept, sizeof( hk_t ), cmp_hk );
            const uint32_t count = kept < maxN ? kept : maxN;
            if ( found > maxN )
                trunc++;
            for ( uint32_t m = 0; m < count; m++ )
            {
                const float * pp  = o->posf + 4 * buf[ m ].idx;
                float *       dst = o->snbr + 4 * ( maxN * q + m );
                o->snbrIdx[ maxN * q + m ] = buf[ m ].idx;
                dst[ 0 ]          = pp[ 0 ];
                dst[ 1 ]          = pp[ 1 ];
                dst[ 2 ]          = pp[ 2 ];
                dst[ 3 ]          = o->mode == ORA_MODE_FULL ? ( pq[ 0 ] * pq[ 1 ] ) * pq[ 2 ] : 0.f;
            }
            o->ids[ 4 * q + 3 ] = (int32_t)count;
        }
        free( buf );
    }
    if ( o->mode == ORA_MODE_EXTERIOR )
        for ( uint64_t q = 0; q < o->Q; q++ )
            o->posf[ 4 * q + 3 ] = (float)(int32_t)( q * maxN );
    o->counters[ BAND_SINGULAR_NBR ] += band;
    o->counters[ SNBR_TRUNCATED ] += trunc;
    free( qhash );
    fine_free( &g );
}

/* ---- stage H: exterior tori -------------------------------------------------
 * count_if/copy_if(status == 2) + fillCircles
 * (sesdf/include/bcs/ssesdf/operation.inl:73-97; sesdf/src/ssesdf/operations.cu:246-285). */
static void stage_tori( ora_t * o )
{
    const double rp = o->rp;
    uint64_t     T  = 0;
    for ( uint64_t p = 0; p < o->P; p++ )
        T += o->status[ p ] == 2;
    o->T        = T;
    o->tori     = (double *)malloc( sizeof( double ) * 12 * ( T ? T : 1 ) );
    uint64_t t  = 0, degenerate = 0;
    for ( uint64_t p = 0; p < o->P; p++ )
    {
        if ( o->status[ p ] != 2 )
            continue;
        const uint32_t i   = o->slotAtom[ p ], j = o->nbr[ p ];
        const v3       ci  = atom_pos( o, i ), cj = atom_pos( o, j );
        const double   ri  = atom_r( o, i );
        const circle_t c   = circle_geometry( ci, ri, cj, atom_r( o, j ), rp );
        const v3       ta  = nrm( sub( c.center, ci ) );
        const v3       tc  = c.center;
        const v3       cz  = cross( ta, mk( 0.0, 0.0, 1.0 ) );
        if ( dot( cz, cz ) < 1e-12 )
            degenerate++;
        const v3     ortho = nrm( cz );
        const v3     P     = add( tc, mul( ortho, c.radius ) );
        const v3     X     = mul( nrm( sub( P, ci ) ), ri );
        const double lpi   = sqrt( dot( sub( P, ci ), sub( P, ci ) ) );
        const double lpj   = sqrt( dot( sub( P, cj ), sub( P, cj ) ) );
        v3           C     = mul( sub( cj, ci ), lpi / ( lpj + lpi ) );
        const double dist  = sqrt( dot( sub( X, C ), sub( X, C ) ) );
        C                  = sub( add( C, ci ), tc );
        double * dst       = o->tori + 12 * t;
        dst[ 0 ]           = tc.x;
        dst[ 1 ]           = tc.y;
        dst[ 2 ]           = tc.z;
        dst[ 3 ]           = c.radius;
        dst[ 4 ]           = ta.x;
        dst[ 5 ]           = ta.y;
        dst[ 6 ]           = ta.z;
        dst[ 7 ]           = rp;
        dst[ 8 ]           = C.x;
        dst[ 9 ]           = C.y;
        dst[ 10 ]          = C.z;
        dst[ 11 ]          = dist;
        t++;
    }
    o->counters[ TORUS_DEGENERATE ] += degenerate;
}

/* ------------------------------------------------------------------------ */
void * ora_build( const float * atoms, uint32_t n, const float * aabb, float rp, int mode, uint32_t maxNbr, uint32_t segCap,
                  int threads )
{
#ifdef _OPENMP
    if ( threads > 0 )
        omp_set_num_threads( threads );
#else
    (void)threads;
#endif
    ora_t * o  = (ora_t *)calloc( 1, sizeof( ora_t ) );
    o->n       = n;
    o->mode    = mode;
    o->rp      = rp;
    o->maxNbr  = maxNbr ? maxNbr : 128u;
    o->segCap  = segCap ? segCap : 32u;
    memcpy( o->aabb, aabb, sizeof( o->aabb ) );
    o->perm  = (uint32_t *)malloc( sizeof( uint32_t ) * ( n ? n : 1 ) );
    o->hash  = (uint32_t *)malloc( sizeof( uint32_t ) * ( n ? n : 1 ) );
    o->atoms = (float *)malloc( sizeof( float ) * 4 * ( n ? n : 1 ) );
    stage_sort( o, atoms );
    stage_neighbors( o );
    stage_visibility( o );
    stage_convex( o );
    stage_intersections( o );
    stage_singular( o );
    if ( mode == ORA_MODE_EXTERIOR )
        stage_tori( o );
    return o;
}

/* getAabb (sesdf/src/core/molecule.cpp:132-143) in float32 */
void ora_aabb( const float * atoms, uint32_t n, float * out )
{
    for ( int a = 0; a < 3; a++ )
    {
        out[ a ]     = 3.402823466e+38f;
        out[ 3 + a ] = -3.402823466e+38f;
    }
    for ( uint32_t i = 0; i < n; i++ )
        for ( int a = 0; a < 3; a++ )
        {
            const float lo = atoms[ 4 * i + a ] - atoms[ 4 * i + 3 ];
            const float hi = atoms[ 4 * i + a ] + atoms[ 4 * i + 3 ];
            out[ a ]       = lo < out[ a ] ? lo : out[ a ];
            out[ 3 + a ]   = hi > out[ 3 + a ] ? hi : out[ 3 + a ];
        }
}

/* array accessor: returns a pointer and element count for a named output */
int ora_array( void * h, const char * name, void ** ptr, uint64_t * count )
{
    ora_t * o = (ora_t *)h;
#define ORA_ARR( nm, p, c )                                                                                              \
    if ( strcmp( name, nm ) == 0 )                                                                                       \
    {                                                                                                                    \
        *ptr   = (void *)( p );                                                                                          \
        *count = ( c );                                                                                                  \
        return 0;                                                                                                        \
    }
    ORA_ARR( "perm", o->perm, o->n )
    ORA_ARR( "hash", o->hash, o->n )
    ORA_ARR( "atoms", o->atoms, 4ull * o->n )
    ORA_ARR( "noff", o->noff, o->n + 1ull )
    ORA_ARR( "nbr", o->nbr, o->P )
    ORA_ARR( "status", o->status, o->P )
    ORA_ARR( "status0", o->status0, o->P )
    ORA_ARR( "convex", o->convex, o->convex ? 2ull * o->n : 0 )
    ORA_ARR( "sectors", o->sectors, 4ull * o->V )
    ORA_ARR( "full", o->fullCircles, 2ull * o->F )
    ORA_ARR( "slot_trim", o->slotTrim, o->P )
    ORA_ARR( "trim_slot", o->trimSlot, o->C1 )
    ORA_ARR( "ids", o->ids, 4ull * o->I )
    ORA_ARR( "cids", o->cids, 4ull * o->I )
    ORA_ARR( "posf", o->posf, 4ull * o->I )
    ORA_ARR( "posd", o->posd, 4ull * o->I )
    ORA_ARR( "ccount", o->ccount, o->ccount ? o->C1 : 0 )
    ORA_ARR( "cstart", o->cstart, o->cstart ? o->C1 + 1 : 0 )
    ORA_ARR( "clist", o->clist, o->clist ? 3ull * o->I : 0 )
    ORA_ARR( "segments", o->seg, 4ull * o->S )
    ORA_ARR( "snbr", o->snbr, 4ull * 32ull * o->Q )
    ORA_ARR( "snbr_idx", o->snbrIdx, 32ull * o->Q )
    ORA_ARR( "tori", o->tori, 12ull * o->T )
    ORA_ARR( "counters", o->counters, (uint64_t)ORA_NCOUNTER )
#undef ORA_ARR
    return -1;
}

void ora_grid( void * h, float * origin, float * cell, uint32_t * gsize )
{
    ora_t * o = (ora_t *)h;
    memcpy( origin, o->origin, sizeof( o->origin ) );
    memcpy( cell, o->cell, sizeof( o->cell ) );
    *gsize = o->gsize;
}

void ora_free( void * h )
{
    ora_t * o = (ora_t *)h;
    if ( !o )
        return;
    free( o->perm );
    free( o->hash );
    free( o->atoms );
    free( o->noff );
    free( o->nbr );
    free( o->slotAtom );
    free( o->status );
    free( o->status0 );
    free( o->convex );
    free( o->sectors );
    free( o->fullCircles );
    free( o->slotTrim );
    free( o->trimSlot );
    free( o->ids );
    free( o->cids );
    free( o->posf );
    free( o->posd );
    free( o->ccount );
    free( o->cstart );
    free( o->clist );
    free( o->seg );
    free( o->snbr );
    free( o->snbrIdx );
    free( o->tori );
    free( o );
}

/* ---- SDF at query points (test oracle, FP64) ---------------------------------
 * The project's definition of the signed distance to the SES (no reference
 * counterpart): E = probe-centre positions outside every SAS sphere
 * (R_i = r_i + rp); with T = rp + band, outside the SAS sdf = min_i(|x - c_i| -
 * r_i) clamped to band; inside, sdf = rp - min(T, dist(x, dE)), dE the SAS
 * surface made of the accessible sphere patches (radial projections of x that
 * no other SAS sphere strictly contains), the visible circles' arcs (nearest
 * circle points likewise) and the probe positions. Inputs are the build's
 * sorted atoms, neighbour lists, statuses and probes (ids, FP64 positions).
 * kind: 0 clamped inside, 1 atom (outside the SAS), 2 clamped outside, 3 sphere
 * patch, 4 circle arc, 5 probe. With gq, grad (4n, sorted order) receives
 * sum_q gq[q] d sdf_q / d (c, r) of the active primitive: the atom or sphere
 * distance directly, a circle point and a probe by the Lagrange /
 * implicit-function rule on their sphere constraints |p - c_m|^2 = R_m^2. */
static double d3len( const double v[ 3 ] ) { return sqrt( v[ 0 ] * v[ 0 ] + v[ 1 ] * v[ 1 ] + v[ 2 ] * v[ 2 ] ); }
static void   sdf_cross( const double a[ 3 ], const double b[ 3 ], double o[ 3 ] )
{
    o[ 0 ] = a[ 1 ] * b[ 2 ] - a[ 2 ] * b[ 1 ];
    o[ 1 ] = a[ 2 ] * b[ 0 ] - a[ 0 ] * b[ 2 ];
    o[ 2 ] = a[ 0 ] * b[ 1 ] - a[ 1 ] * b[ 0 ];
}

static int sdf_hidden( const float * atoms, const uint32_t * row, uint32_t ni, uint32_t skip, double rp, const double q[ 3 ] )
{
    for ( uint32_t k = 0; k < ni; k++ )
    {
        if ( k == skip )
            continue;
        const float * c  = atoms + 4 * (size_t)row[ k ];
        const double  dx = q[ 0 ] - c[ 0 ], dy = q[ 1 ] - c[ 1 ], dz = q[ 2 ] - c[ 2 ];
        const double  R  = (double)c[ 3 ] + rp;
        if ( dx * dx + dy * dy + dz * dz < R * R )
            return 1;
    }
    return 0;
}

typedef struct
{
    int    kind;
    int    a, b, c;
    double q[ 3 ];
    double value;
} ora_hit_t;

static void sdf_grad( const float * atoms, double rp, const ora_hit_t * h, const double x[ 3 ], double gs, double * grad )
{
    if ( h->kind == 1 || h->kind == 3 )
    {
        const float * c = atoms + 4 * (size_t)h->a;
        double        w[ 3 ] = { x[ 0 ] - c[ 0 ], x[ 1 ] - c[ 1 ], x[ 2 ] - c[ 2 ] };
        const double  L = d3len( w );
        if ( !( L > 0.0 ) )
            return;
        double sgn = -1.0;
        if ( h->kind == 3 && L > (double)c[ 3 ] + rp )
            sgn = 1.0;
        for ( int a = 0; a < 3; a++ )
            grad[ 4 * (size_t)h->a + a ] += gs * sgn * w[ a ] / L;
        grad[ 4 * (size_t)h->a + 3 ] += gs * sgn;
        return;
    }
    if ( h->kind != 4 && h->kind != 5 )
        return;
    const double u0[ 3 ] = { x[ 0 ] - h->q[ 0 ], x[ 1 ] - h->q[ 1 ], x[ 2 ] - h->q[ 2 ] };
    const double D       = d3len( u0 );
    if ( !( D > 0.0 ) )
        return;
    const double u[ 3 ] = { u0[ 0 ] / D, u0[ 1 ] / D, u0[ 2 ] / D };
    const int    m      = h->kind == 4 ? 2 : 3;
    const int    ids[ 3 ] = { h->a, h->b, h->c };
    double       A[ 3 ][ 3 ], R[ 3 ], w[ 3 ] = { 0, 0, 0 };
    for ( int k = 0; k < m; k++ )
    {
        const float * c = atoms + 4 * (size_t)ids[ k ];
        for ( int a = 0; a < 3; a++ )
            A[ k ][ a ] = 2.0 * ( h->q[ a ] - c[ a ] );
        R[ k ] = (double)c[ 3 ] + rp;
    }
    if ( m == 2 )
    {
        double g00 = 0, g01 = 0, g11 = 0, r0 = 0, r1 = 0;
        for ( int a = 0; a < 3; a++ )
        {
            g00 += A[ 0 ][ a ] * A[ 0 ][ a ];
            g01 += A[ 0 ][ a ] * A[ 1 ][ a ];
            g11 += A[ 1 ][ a ] * A[ 1 ][ a ];
            r0 += A[ 0 ][ a ] * u[ a ];
            r1 += A[ 1 ][ a ] * u[ a ];
        }
        const double det = g00 * g11 - g01 * g01;
        if ( !( fabs( det ) > 0.0 ) )
            return;
        w[ 0 ] = ( r0 * g11 - r1 * g01 ) / det;
        w[ 1 ] = ( r1 * g00 - r0 * g01 ) / det;
    }
    else
    {
        /* sum_k w_k A_k = u (A_k as columns): Cramer's rule */
        double c12[ 3 ], cu2[ 3 ], c01[ 3 ];
        sdf_cross( A[ 1 ], A[ 2 ], c12 );
        sdf_cross( u, A[ 2 ], cu2 );
        sdf_cross( A[ 0 ], A[ 1 ], c01 );
        const double det = A[ 0 ][ 0 ] * c12[ 0 ] + A[ 0 ][ 1 ] * c12[ 1 ] + A[ 0 ][ 2 ] * c12[ 2 ];
        if ( !( fabs( det ) > 0.0 ) )
            return;
        w[ 0 ] = ( u[ 0 ] * c12[ 0 ] + u[ 1 ] * c12[ 1 ] + u[ 2 ] * c12[ 2 ] ) / det;               /* det[u, A1, A2] */
        w[ 1 ] = ( A[ 0 ][ 0 ] * cu2[ 0 ] + A[ 0 ][ 1 ] * cu2[ 1 ] + A[ 0 ][ 2 ] * cu2[ 2 ] ) / det; /* det[A0, u, A2] */
        w[ 2 ] = ( c01[ 0 ] * u[ 0 ] + c01[ 1 ] * u[ 1 ] + c01[ 2 ] * u[ 2 ] ) / det;               /* det[A0, A1, u] */
    }
    for ( int k = 0; k < m; k++ )
    {
        for ( int a = 0; a < 3; a++ )
            grad[ 4 * (size_t)ids[ k ] + a ] += gs * w[ k ] * A[ k ][ a ];
        grad[ 4 * (size_t)ids[ k ] + 3 ] += gs * 2.0 * w[ k ] * R[ k ];
    }
}

static int cmp_dkey( const void * a, const void * b )
{
    const double * x = (const double *)a;
    const double * y = (const double *)b;
    if ( x[ 0 ] != y[ 0 ] )
        return x[ 0 ] < y[ 0 ] ? -1 : 1;
    return x[ 1 ] < y[ 1 ] ? -1 : ( x[ 1 ] > y[ 1 ] );
}

int ora_sdf( const float * atoms, uint32_t n, const uint32_t * noff, const uint32_t * nbr, const uint8_t * status,
             const int32_t * ids, const double * posd, uint32_t I, float rpf, float bandf, const float * queries,
             uint32_t m, const double * gq, double * sdf, int32_t * kind, double * grad, int threads )
{
    const double rp = rpf, band = bandf, T = rp + band;
    double       lo[ 3 ] = { 1e300, 1e300, 1e300 }, hi[ 3 ] = { -1e300, -1e300, -1e300 }, rmax = 0;
    if ( n == 0 )
    {
        for ( uint32_t q = 0; q < m; q++ )
        {
            sdf[ q ] = band;
            if ( kind )
                kind[ q ] = 2;
        }
        return 0;
    }
    for ( uint32_t i = 0; i < n; i++ )
    {
        for ( int a = 0; a < 3; a++ )
        {
            lo[ a ] = atoms[ 4 * i + a ] < lo[ a ] ? atoms[ 4 * i + a ] : lo[ a ];
            hi[ a ] = atoms[ 4 * i + a ] > hi[ a ] ? atoms[ 4 * i + a ] : hi[ a ];
        }
        rmax = atoms[ 4 * i + 3 ] > rmax ? atoms[ 4 * i + 3 ] : rmax;
    }
    /* atom grid with cell >= the reach R + T */
    const double h = rmax + rp + T + 1e-3;
    int          dims[ 3 ];
    for ( int a = 0; a < 3; a++ )
    {
        lo[ a ] -= h;
        dims[ a ] = (int)( ( hi[ a ] + h - lo[ a ] ) / h ) + 1;
    }
    const uint64_t cells = (uint64_t)dims[ 0 ] * dims[ 1 ] * dims[ 2 ];
    uint32_t *     start = (uint32_t *)calloc( cells + 1, sizeof( uint32_t ) );
    uint32_t *     item  = (uint32_t *)malloc( sizeof( uint32_t ) * n );
    uint32_t *     cell  = (uint32_t *)malloc( sizeof( uint32_t ) * n );
    /* probes by their first atom */
    uint32_t * pstart = (uint32_t *)calloc( n + 1, sizeof( uint32_t ) );
    uint32_t * pitem  = (uint32_t *)malloc( sizeof( uint32_t ) * ( I ? I : 1 ) );
    if ( !start || !item || !cell || !pstart || !pitem )
        return -1;
    for ( uint32_t i = 0; i < n; i++ )
    {
        int c[ 3 ];
        for ( int a = 0; a < 3; a++ )
            c[ a ] = (int)( ( atoms[ 4 * i + a ] - lo[ a ] ) / h );
        cell[ i ] = (uint32_t)( ( (uint64_t)c[ 2 ] * dims[ 1 ] + c[ 1 ] ) * dims[ 0 ] + c[ 0 ] );
        start[ cell[ i ] + 1 ]++;
    }
    for ( uint64_t k = 0; k < cells; k++ )
        start[ k + 1 ] += start[ k ];
    {
        uint32_t * cur = (uint32_t *)malloc( sizeof( uint32_t ) * ( cells + 1 ) );
        memcpy( cur, start, sizeof( uint32_t ) * ( cells + 1 ) );
        for ( uint32_t i = 0; i < n; i++ )
            item[ cur[ cell[ i ] ]++ ] = i;
        free( cur );
    }
    for ( uint32_t p = 0; p < I; p++ )
        pstart[ ids[ 4 * p ] + 1 ]++;
    for ( uint32_t i = 0; i < n; i++ )
        pstart[ i + 1 ] += pstart[ i ];
    {
        uint32_t * cur = (uint32_t *)malloc( sizeof( uint32_t ) * ( n + 1 ) );
        memcpy( cur, pstart, sizeof( uint32_t ) * ( n + 1 ) );
        for ( uint32_t p = 0; p < I; p++ )
            pitem[ cur[ ids[ 4 * p ] ]++ ] = p;
        free( cur );
    }
    if ( grad )
        memset( grad, 0, sizeof( double ) * 4 * n );
    int nthreads = threads > 0 ? threads : omp_get_max_threads();
    /* per-thread gradient accumulators, summed at the end (deterministic per thread count) */
    double * gpriv = grad ? (double *)calloc( (size_t)nthreads * 4 * n, sizeof( double ) ) : NULL;
#pragma omp parallel num_threads( nthreads )
    {
        const int tid  = omp_get_thread_num();
        double *  gmy  = gpriv ? gpriv + (size_t)tid * 4 * n : NULL;
        double *  keys = (double *)malloc( sizeof( double ) * 2 * ( n < 4096 ? n : 4096 ) );
#pragma omp for schedule( dynamic, 256 )
        for ( uint32_t qi = 0; qi < m; qi++ )
        {
            const double x[ 3 ] = { queries[ 3 * (size_t)qi ], queries[ 3 * (size_t)qi + 1 ], queries[ 3 * (size_t)qi + 2 ] };
            int          c[ 3 ];
            for ( int a = 0; a < 3; a++ )
                c[ a ] = (int)( ( x[ a ] - lo[ a ] ) / h );
            uint32_t  nl = 0;
            double    smin = 1e300, vmin = 1e300;
            int       vatom = -1;
            for ( int dz = -1; dz <= 1; dz++ )
                for ( int dy = -1; dy <= 1; dy++ )
                    for ( int dx = -1; dx <= 1; dx++ )
                    {
                        const int cx = c[ 0 ] + dx, cy = c[ 1 ] + dy, cz = c[ 2 ] + dz;
                        if ( cx < 0 || cy < 0 || cz < 0 || cx >= dims[ 0 ] || cy >= dims[ 1 ] || cz >= dims[ 2 ] )
                            continue;
                        const uint64_t k = ( (uint64_t)cz * dims[ 1 ] + cy ) * dims[ 0 ] + cx;
                        for ( uint32_t e = start[ k ]; e < start[ k + 1 ]; e++ )
                        {
                            const uint32_t i  = item[ e ];
                            const double   w[ 3 ] = { x[ 0 ] - atoms[ 4 * i ], x[ 1 ] - atoms[ 4 * i + 1 ], x[ 2 ] - atoms[ 4 * i + 2 ] };
                            const double   L  = d3len( w );
                            const double   R  = (double)atoms[ 4 * i + 3 ] + rp;
                            if ( !( L <= R + T ) )
                                continue;
                            smin           = L - R < smin ? L - R : smin;
                            const double v = L - atoms[ 4 * i + 3 ];
                            if ( v < vmin || ( v == vmin && (int)i < vatom ) )
                            {
                                vmin  = v;
                                vatom = (int)i;
                            }
                            if ( nl < 4096 )
                            {
                                keys[ 2 * nl ]     = fabs( L - R );
                                keys[ 2 * nl + 1 ] = (double)i;
                                nl++;
                            }
                        }
                    }
            ora_hit_t hit;
            hit.a = hit.b = hit.c = -1;
            hit.q[ 0 ] = x[ 0 ], hit.q[ 1 ] = x[ 1 ], hit.q[ 2 ] = x[ 2 ];
            if ( !( smin < 0.0 ) )
            {
                if ( vatom >= 0 && vmin <= band )
                {
                    hit.kind  = 1;
                    hit.a     = vatom;
                    hit.value = vmin;
                }
                else
                {
                    hit.kind  = 2;
                    hit.value = band;
                }
            }
            else
            {
                qsort( keys, nl, 2 * sizeof( double ), cmp_dkey );
                double best = T;
                hit.kind    = 0;
                for ( uint32_t t = 0; t < nl; t++ )
                {
                    const double   dl = keys[ 2 * t ];
                    const uint32_t i  = (uint32_t)keys[ 2 * t + 1 ];
                    if ( !( dl < best ) )
                        break;
                    const float *    ci  = atoms + 4 * (size_t)i;
                    const double     Ri  = (double)ci[ 3 ] + rp;
                    const uint32_t * row = nbr + noff[ i ];
                    const uint32_t   ni  = noff[ i + 1 ] - noff[ i ];
                    /* sphere patch */
                    {
                        double       w[ 3 ] = { x[ 0 ] - ci[ 0 ], x[ 1 ] - ci[ 1 ], x[ 2 ] - ci[ 2 ] };
                        const double L      = d3len( w );
                        if ( L > 0.0 )
                        {
                            const double q[ 3 ] = { ci[ 0 ] + w[ 0 ] * ( Ri / L ), ci[ 1 ] + w[ 1 ] * ( Ri / L ), ci[ 2 ] + w[ 2 ] * ( Ri / L ) };
                            if ( !sdf_hidden( atoms, row, ni, 0xffffffffu, rp, q ) && dl < best )
                            {
                                best     = dl;
                                hit.kind = 3;
                                hit.a    = (int)i;
                                memcpy( hit.q, q, sizeof( q ) );
                            }
                        }
                    }
                    /* visible circles */
                    for ( uint32_t s = 0; s < ni; s++ )
                    {
                        if ( status[ noff[ i ] + s ] == 0 )
                            continue;
                        const float * cj = atoms + 4 * (size_t)row[ s ];
                        const double  Rj = (double)cj[ 3 ] + rp;
                        const double  d[ 3 ] = { (double)cj[ 0 ] - ci[ 0 ], (double)cj[ 1 ] - ci[ 1 ], (double)cj[ 2 ] - ci[ 2 ] };
                        const double  dd = d[ 0 ] * d[ 0 ] + d[ 1 ] * d[ 1 ] + d[ 2 ] * d[ 2 ];
                        const double  tt = ( Ri * Ri - Rj * Rj + dd ) / ( 2.0 * dd );
                        const double  r2 = Ri * Ri - tt * tt * dd;
                        if ( !( r2 > 0.0 ) )
                            continue;
                        const double r    = sqrt( r2 );
                        const double dl2  = sqrt( dd );
                        const double nn[ 3 ] = { d[ 0 ] / dl2, d[ 1 ] / dl2, d[ 2 ] / dl2 };
                        const double cc[ 3 ] = { ci[ 0 ] + d[ 0 ] * tt, ci[ 1 ] + d[ 1 ] * tt, ci[ 2 ] + d[ 2 ] * tt };
                        const double w[ 3 ]  = { x[ 0 ] - cc[ 0 ], x[ 1 ] - cc[ 1 ], x[ 2 ] - cc[ 2 ] };
                        const double hh      = w[ 0 ] * nn[ 0 ] + w[ 1 ] * nn[ 1 ] + w[ 2 ] * nn[ 2 ];
                        const double v[ 3 ]  = { w[ 0 ] - hh * nn[ 0 ], w[ 1 ] - hh * nn[ 1 ], w[ 2 ] - hh * nn[ 2 ] };
                        const double rho     = d3len( v );
                        double       dist, q[ 3 ] = { cc[ 0 ], cc[ 1 ], cc[ 2 ] };
                        if ( rho > 1e-6 )
                        {
                            for ( int a = 0; a < 3; a++ )
                                q[ a ] = cc[ a ] + v[ a ] * ( r / rho );
                            dist = sqrt( hh * hh + ( rho - r ) * ( rho - r ) );
                            if ( !( dist < best ) || sdf_hidden( atoms, row, ni, s, rp, q ) )
                                continue;
                        }
                        else
                        {
                            dist = sqrt( hh * hh + r2 );
                            if ( !( dist < best ) )
                                continue;
                        }
                        best     = dist;
                        hit.kind = 4;
                        hit.a    = (int)i;
                        hit.b    = (int)row[ s ];
                        memcpy( hit.q, q, sizeof( q ) );
                    }
                    /* probes whose first atom is i */
                    for ( uint32_t e = pstart[ i ]; e < pstart[ i + 1 ]; e++ )
                    {
                        const uint32_t p    = pitem[ e ];
                        const double * pp   = posd + 4 * (size_t)p;
                        const double   w[ 3 ] = { x[ 0 ] - pp[ 0 ], x[ 1 ] - pp[ 1 ], x[ 2 ] - pp[ 2 ] };
                        const double   dist = d3len( w );
                        if ( dist < best )
                        {
                            best     = dist;
                            hit.kind = 5;
                            hit.a    = ids[ 4 * p ];
                            hit.b    = ids[ 4 * p + 1 ];
                            hit.c    = ids[ 4 * p + 2 ];
                            memcpy( hit.q, pp, 3 * sizeof( double ) );
                        }
                    }
                }
                hit.value = rp - best;
            }
            sdf[ qi ] = hit.value;
            if ( kind )
                kind[ qi ] = hit.kind;
            if ( gmy && gq )
                sdf_grad( atoms, rp, &hit, x, gq[ qi ], gmy );
        }
        free( keys );
    }
    if ( grad )
    {
        for ( int t = 0; t < nthreads; t++ )
            for ( size_t k = 0; k < 4 * (size_t)n; k++ )
                grad[ k ] += gpriv[ (size_t)t * 4 * n + k ];
        free( gpriv );
    }
    free( start );
    free( item );
    free( cell );
    free( pstart );
    free( pitem );
    return 0;
}
