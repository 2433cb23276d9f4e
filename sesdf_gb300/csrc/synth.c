/*
 * Seeded synthetic molecules for the SES build workloads.
 *
 * The reference benchmarks PDB entries (app/benchmarks/main.cu:97-113); these
 * generators stand in for them with protein-like density (0.045 atoms/A^3) and
 * element mix (C/N/O/S 62/17/19/2 %, vdW radii 1.70/1.55/1.52/1.80 A).
 *
 * Globule: a self-avoiding random chain with bond length 1.53 A, bond angle
 * 111 degrees and uniform random torsion, confined to a sphere of radius
 * (3N / (4 pi 0.045))^(1/3); a step is rejected when it comes within 3.0 A of a
 * non-bonded atom (every atom except the two previous ones) or leaves the
 * sphere. Plain sequential growth jams far below protein density (the chain
 * end gets trapped in a pocket), so when 200 consecutive trial steps are
 * rejected the chain starts a new segment at a uniformly drawn free point of
 * the sphere (every atom of a segment except its first keeps the bond,
 * angle and torsion rules). This reaches the target density exactly.
 *
 * Only +, -, *, / and sqrt are used (no libm transcendental calls) and the file
 * is compiled with -ffp-contract=off, so x86-64 and aarch64 hosts generate
 * bit-identical coordinates from the same seed.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SYN_DENSITY 0.045
#define SYN_BOND 1.53
#define SYN_CLASH 3.0

/* cos and sin of (180 - 111) degrees: the new bond makes a 111 degree angle
 * with the previous bond, i.e. deviates 69 degrees from its direction. */
static const double kCos69 = 0.35836794954530027;
static const double kSin69 = 0.93358042649720174;

typedef struct
{
    uint64_t s[ 4 ];
} rng_t;

static uint64_t splitmix64( uint64_t * x )
{
    uint64_t z = ( *x += 0x9E3779B97F4A7C15ull );
    z          = ( z ^ ( z >> 30 ) ) * 0xBF58476D1CE4E5B9ull;
    z          = ( z ^ ( z >> 27 ) ) * 0x94D049BB133111EBull;
    return z ^ ( z >> 31 );
}

static void rng_seed( rng_t * r, uint64_t seed )
{
    uint64_t x = seed;
    for ( int i = 0; i < 4; i++ )
        r->s[ i ] = splitmix64( &x );
}

static inline uint64_t rotl( uint64_t x, int k ) { return ( x << k ) | ( x >> ( 64 - k ) ); }

/* xoshiro256** */
static uint64_t rng_next( rng_t * r )
{
    uint64_t * s      = r->s;
    const uint64_t rs = rotl( s[ 1 ] * 5, 7 ) * 9;
    const uint64_t t  = s[ 1 ] << 17;
    s[ 2 ] ^= s[ 0 ];
    s[ 3 ] ^= s[ 1 ];
    s[ 1 ] ^= s[ 2 ];
    s[ 0 ] ^= s[ 3 ];
    s[ 2 ] ^= t;
    s[ 3 ] = rotl( s[ 3 ], 45 );
    return rs;
}

/* uniform in [0, 1) with 53 random bits */
static double rng_uniform( rng_t * r ) { return (double)( rng_next( r ) >> 11 ) * ( 1.0 / 9007199254740992.0 ); }

/* uniform point on the unit circle (rejection from the square) */
static void rng_circle( rng_t * r, double * c, double * s )
{
    for ( ;; )
    {
        const double x  = 2.0 * rng_uniform( r ) - 1.0;
        const double y  = 2.0 * rng_uniform( r ) - 1.0;
        const double q2 = x * x + y * y;
        if ( q2 > 1e-6 && q2 <= 1.0 )
        {
            const double q = sqrt( q2 );
            *c             = x / q;
            *s             = y / q;
            return;
        }
    }
}

/* uniform direction on the unit sphere (rejection from the cube) */
static void rng_sphere( rng_t * r, double v[ 3 ] )
{
    for ( ;; )
    {
        const double x  = 2.0 * rng_uniform( r ) - 1.0;
        const double y  = 2.0 * rng_uniform( r ) - 1.0;
        const double z  = 2.0 * rng_uniform( r ) - 1.0;
        const double q2 = x * x + y * y + z * z;
        if ( q2 > 1e-6 && q2 <= 1.0 )
        {
            const double q = sqrt( q2 );
            v[ 0 ]         = x / q;
            v[ 1 ]         = y / q;
            v[ 2 ]         = z / q;
            return;
        }
    }
}

/* natural logarithm from frexp (exact) and the atanh series, so that no libm
 * approximation enters the generated coordinates */
static double ln_series( double x )
{
    int          e;
    const double m = frexp( x, &e ); /* x = m 2^e, m in [0.5, 1) */
    const double z = ( m - 1.0 ) / ( m + 1.0 );
    const double z2 = z * z;
    double       term = z, sum = 0.0;
    for ( int k = 1; k < 80; k += 2 )
    {
        sum += term / (double)k;
        term *= z2;
    }
    return 2.0 * sum + (double)e * 0.69314718055994530942;
}

/* standard normal by the Marsaglia polar method */
static double rng_gauss( rng_t * r )
{
    for ( ;; )
    {
        const double u = 2.0 * rng_uniform( r ) - 1.0;
        const double v = 2.0 * rng_uniform( r ) - 1.0;
        const double q = u * u + v * v;
        if ( q > 0.0 && q < 1.0 )
            return u * sqrt( -2.0 * ln_series( q ) / q );
    }
}

static float element_radius( rng_t * r )
{
    const double u = rng_uniform( r );
    if ( u < 0.62 )
        return 1.70f; /* C */
    if ( u < 0.79 )
        return 1.55f; /* N */
    if ( u < 0.98 )
        return 1.52f; /* O */
    return 1.80f;     /* S */
}

/* ---- clash grid: cubic cells of SYN_CLASH A holding atom indices ---------- */
typedef struct
{
    int        dim;
    double     origin;
    int32_t *  head; /* dim^3 */
    int32_t *  next; /* capacity */
    int32_t *  cell; /* capacity: cell of each atom or -1 */
} clash_grid_t;

static int cg_cell_of( const clash_grid_t * g, const double p[ 3 ], int c[ 3 ] )
{
    for ( int a = 0; a < 3; a++ )
    {
        const double t = ( p[ a ] - g->origin ) / SYN_CLASH;
        int          k = (int)floor( t );
        if ( k < 0 || k >= g->dim )
            return 0;
        c[ a ] = k;
    }
    return 1;
}

static void cg_insert( clash_grid_t * g, int32_t idx, const double p[ 3 ] )
{
    int c[ 3 ];
    if ( !cg_cell_of( g, p, c ) )
    {
        g->cell[ idx ] = -1;
        return;
    }
    const int32_t h = ( c[ 2 ] * g->dim + c[ 1 ] ) * g->dim + c[ 0 ];
    g->cell[ idx ]  = h;
    g->next[ idx ]  = g->head[ h ];
    g->head[ h ]    = idx;
}

/* 1 if p lies inside the grid and farther than SYN_CLASH from every stored
 * atom other than skipA and skipB */
static int cg_free( const clash_grid_t * g, const double * xyz, const double p[ 3 ], int32_t skipA, int32_t skipB )
{
    int c[ 3 ];
    if ( !cg_cell_of( g, p, c ) )
        return 0;
    for ( int dz = -1; dz <= 1; dz++ )
        for ( int dy = -1; dy <= 1; dy++ )
            for ( int dx = -1; dx <= 1; dx++ )
            {
                const int x = c[ 0 ] + dx, y = c[ 1 ] + dy, z = c[ 2 ] + dz;
                if ( x < 0 || y < 0 || z < 0 || x >= g->dim || y >= g->dim || z >= g->dim )
                    continue;
                for ( int32_t j = g->head[ ( z * g->dim + y ) * g->dim + x ]; j >= 0; j = g->next[ j ] )
                {
                    if ( j == skipA || j == skipB )
                        continue;
                    const double ex = xyz[ 3 * j ] - p[ 0 ], ey = xyz[ 3 * j + 1 ] - p[ 1 ], ez = xyz[ 3 * j + 2 ] - p[ 2 ];
                    if ( ex * ex + ey * ey + ez * ez < SYN_CLASH * SYN_CLASH )
                        return 0;
                }
            }
    return 1;
}

static void cross3( const double a[ 3 ], const double b[ 3 ], double o[ 3 ] )
{
    o[ 0 ] = a[ 1 ] * b[ 2 ] - a[ 2 ] * b[ 1 ];
    o[ 1 ] = a[ 2 ] * b[ 0 ] - a[ 0 ] * b[ 2 ];
    o[ 2 ] = a[ 0 ] * b[ 1 ] - a[ 1 ] * b[ 0 ];
}

static void normalize3( double v[ 3 ] )
{
    const double q = sqrt( v[ 0 ] * v[ 0 ] + v[ 1 ] * v[ 1 ] + v[ 2 ] * v[ 2 ] );
    v[ 0 ] /= q;
    v[ 1 ] /= q;
    v[ 2 ] /= q;
}

/* cube root by Newton iterations (x > 0) */
static double cbrt_newton( double x )
{
    double y = x > 1.0 ? x / 3.0 : 1.0;
    for ( int i = 0; i < 200; i++ )
    {
        const double ny = y - ( y * y * y - x ) / ( 3.0 * y * y );
        if ( ny == y )
            break;
        y = ny;
    }
    return y;
}

/*
 * Grows an n-atom globule centred on the origin.
 * out: n * 4 floats (x, y, z, vdW radius). Returns the number of chain
 * segments (>= 1), or -1 if the sphere could not be filled.
 */
int sesgb_synth_globule( uint32_t n, uint64_t seed, float * out )
{
    if ( n == 0 )
        return 0;
    rng_t rng;
    rng_seed( &rng, seed );

    const double radius = cbrt_newton( 3.0 * (double)n / ( 4.0 * 3.14159265358979323846 * SYN_DENSITY ) );
    double *     xyz    = (double *)malloc( sizeof( double ) * 3 * n );
    clash_grid_t g;
    g.dim    = (int)( 2.0 * ( radius + 4.0 ) / SYN_CLASH ) + 3;
    g.origin = -( radius + 4.0 ) - SYN_CLASH;
    g.head   = (int32_t *)malloc( sizeof( int32_t ) * (size_t)g.dim * g.dim * g.dim );
    g.next   = (int32_t *)malloc( sizeof( int32_t ) * n );
    g.cell   = (int32_t *)malloc( sizeof( int32_t ) * n );
    for ( size_t c = 0; c < (size_t)g.dim * g.dim * g.dim; c++ )
        g.head[ c ] = -1;

    const uint32_t maxTries    = 200;
    const uint64_t maxSegments = 64ull * n + 1000ull;
    uint32_t       count       = 0;
    uint32_t       segStart    = 0;
    uint64_t       segments    = 1;
    int            ok          = 1;
    while ( count < n )
    {
        const uint32_t segLen = count - segStart;
        int            placed = 0;
        for ( uint32_t t = 0; t < maxTries && !placed; t++ )
        {
            double  p[ 3 ];
            int32_t skipA = -1, skipB = -1; /* bonded predecessors, exempt from the clash test */
            if ( segLen == 0 )
            {
                for ( int a = 0; a < 3; a++ )
                    p[ a ] = ( 2.0 * rng_uniform( &rng ) - 1.0 ) * radius;
            }
            else if ( segLen == 1 )
            {
                double d[ 3 ];
                rng_sphere( &rng, d );
                for ( int a = 0; a < 3; a++ )
                    p[ a ] = xyz[ 3 * ( count - 1 ) + a ] + SYN_BOND * d[ a ];
                skipA = (int32_t)count - 1;
            }
            else
            {
                const double * a1     = xyz + 3 * ( count - 1 );
                const double * a2     = xyz + 3 * ( count - 2 );
                double         b[ 3 ] = { a1[ 0 ] - a2[ 0 ], a1[ 1 ] - a2[ 1 ], a1[ 2 ] - a2[ 2 ] };
                normalize3( b );
                /* orthonormal frame perpendicular to the previous bond */
                double ref[ 3 ] = { 1.0, 0.0, 0.0 };
                if ( fabs( b[ 0 ] ) > 0.9 )
                {
                    ref[ 0 ] = 0.0;
                    ref[ 1 ] = 1.0;
                }
                double e1[ 3 ], e2[ 3 ];
                cross3( b, ref, e1 );
                normalize3( e1 );
                cross3( b, e1, e2 );
                double c, s; /* uniform torsion */
                rng_circle( &rng, &c, &s );
                for ( int a = 0; a < 3; a++ )
                    p[ a ] = a1[ a ] + SYN_BOND * ( kCos69 * b[ a ] + kSin69 * ( c * e1[ a ] + s * e2[ a ] ) );
                skipA = (int32_t)count - 1;
                skipB = (int32_t)count - 2;
            }
            if ( p[ 0 ] * p[ 0 ] + p[ 1 ] * p[ 1 ] + p[ 2 ] * p[ 2 ] > radius * radius )
                continue;
            if ( !cg_free( &g, xyz, p, skipA, skipB ) )
                continue;
            memcpy( xyz + 3 * count, p, sizeof( p ) );
            cg_insert( &g, (int32_t)count, p );
            count++;
            placed = 1;
        }
        if ( !placed )
        {
            /* the chain end is trapped: start a new segment */
            segStart = count;
            if ( ++segments > maxSegments )
            {
                ok = 0;
                break;
            }
        }
    }

    if ( ok )
    {
        /* element radii come from a second stream so that they do not depend
         * on the number of rejected steps */
        rng_t rr;
        rng_seed( &rr, seed ^ 0x5DEECE66Dull );
        for ( uint32_t i = 0; i < n; i++ )
        {
            out[ 4 * i + 0 ] = (float)xyz[ 3 * i + 0 ];
            out[ 4 * i + 1 ] = (float)xyz[ 3 * i + 1 ];
            out[ 4 * i + 2 ] = (float)xyz[ 3 * i + 2 ];
            out[ 4 * i + 3 ] = element_radius( &rr );
        }
    }
    free( xyz );
    free( g.head );
    free( g.next );
    free( g.cell );
    return ok ? (int)segments : -1;
}

/* radius of the ball around the origin that holds every atom's vdW sphere */
static double globule_extent( const float * atoms, uint32_t n )
{
    double m = 0.0;
    for ( uint32_t i = 0; i < n; i++ )
    {
        const double x = atoms[ 4 * i ], y = atoms[ 4 * i + 1 ], z = atoms[ 4 * i + 2 ];
        const double d = sqrt( x * x + y * y + z * z ) + atoms[ 4 * i + 3 ];
        if ( d > m )
            m = d;
    }
    return m;
}

/*
 * Assembly of g globules of n atoms each (globule k uses seed seed0 + k),
 * placed one by one next to a randomly chosen earlier globule with a surface
 * gap drawn uniformly in [2, 8] A; a placement is rejected if any other
 * globule comes closer than 2 A or if it leaves the enclosing sphere.
 * out: g * n * 4 floats. Returns 0 on success.
 */
int sesgb_synth_assembly( uint32_t g, uint32_t n, uint64_t seed0, uint64_t placementSeed, float * out )
{
    double * centers = (double *)malloc( sizeof( double ) * 3 * ( g ? g : 1 ) );
    double * radii   = (double *)malloc( sizeof( double ) * ( g ? g : 1 ) );
    rng_t    rng;
    rng_seed( &rng, placementSeed );
    int ok = 0;
    for ( uint32_t k = 0; k < g && ok == 0; k++ )
    {
        float * dst = out + (size_t)k * n * 4;
        if ( sesgb_synth_globule( n, seed0 + k, dst ) < 0 )
        {
            ok = -1;
            break;
        }
        radii[ k ] = globule_extent( dst, n );
    }
    if ( ok == 0 && g > 0 )
    {
        const double enclosing = 2.5 * radii[ 0 ] * cbrt_newton( (double)g ) + 2.0 * radii[ 0 ];
        centers[ 0 ] = centers[ 1 ] = centers[ 2 ] = 0.0;
        for ( uint32_t k = 1; k < g && ok == 0; k++ )
        {
            int placed = 0;
            for ( int t = 0; t < 100000 && !placed; t++ )
            {
                const uint32_t h   = (uint32_t)( rng_uniform( &rng ) * k );
                const double   gap = 2.0 + 6.0 * rng_uniform( &rng );
                double         u[ 3 ];
                rng_sphere( &rng, u );
                double c[ 3 ];
                for ( int a = 0; a < 3; a++ )
                    c[ a ] = centers[ 3 * h + a ] + u[ a ] * ( radii[ k ] + radii[ h ] + gap );
                if ( sqrt( c[ 0 ] * c[ 0 ] + c[ 1 ] * c[ 1 ] + c[ 2 ] * c[ 2 ] ) + radii[ k ] > enclosing )
                    continue;
                int clash = 0;
                for ( uint32_t o = 0; o < k && !clash; o++ )
                {
                    if ( o == h )
                        continue;
                    const double dx = c[ 0 ] - centers[ 3 * o ], dy = c[ 1 ] - centers[ 3 * o + 1 ],
                                 dz = c[ 2 ] - centers[ 3 * o + 2 ];
                    if ( sqrt( dx * dx + dy * dy + dz * dz ) < radii[ k ] + radii[ o ] + 2.0 )
                        clash = 1;
                }
                if ( clash )
                    continue;
                memcpy( centers + 3 * k, c, sizeof( c ) );
                placed = 1;
            }
            if ( !placed )
                ok = -1;
        }
        for ( uint32_t k = 0; k < g && ok == 0; k++ )
        {
            float * dst = out + (size_t)k * n * 4;
            for ( uint32_t i = 0; i < n; i++ )
                for ( int a = 0; a < 3; a++ )
                    dst[ 4 * i + a ] = (float)( (double)dst[ 4 * i + a ] + centers[ 3 * k + a ] );
        }
    }
    free( centers );
    free( radii );
    return ok;
}

/*
 * Shell of g globules of n atoms (globule k uses seed seed0 + k) whose centres
 * lie on a Fibonacci sphere of the given radius. The golden-angle rotation is
 * applied by repeated complex multiplication so that no libm call is needed.
 */
int sesgb_synth_shell( uint32_t g, uint32_t n, uint64_t seed0, double shellRadius, float * out )
{
    /* cos and sin of the golden angle pi (3 - sqrt 5) */
    const double ca = -0.73736887807831974, sa = 0.67549029426152364;
    double       c = 1.0, s = 0.0;
    for ( uint32_t k = 0; k < g; k++ )
    {
        float * dst = out + (size_t)k * n * 4;
        if ( sesgb_synth_globule( n, seed0 + k, dst ) < 0 )
            return -1;
        const double y  = 1.0 - 2.0 * ( (double)k + 0.5 ) / (double)g;
        const double rr = sqrt( 1.0 - y * y );
        const double cx = shellRadius * rr * c, cy = shellRadius * y, cz = shellRadius * rr * s;
        for ( uint32_t i = 0; i < n; i++ )
        {
            dst[ 4 * i + 0 ] = (float)( (double)dst[ 4 * i + 0 ] + cx );
            dst[ 4 * i + 1 ] = (float)( (double)dst[ 4 * i + 1 ] + cy );
            dst[ 4 * i + 2 ] = (float)( (double)dst[ 4 * i + 2 ] + cz );
        }
        const double nc = c * ca - s * sa;
        const double ns = c * sa + s * ca;
        c               = nc;
        s               = ns;
    }
    return 0;
}

/* Adds independent N(0, sigma^2) noise to every coordinate (radii unchanged). */
void sesgb_synth_jitter( float * atoms, uint32_t n, double sigma, uint64_t seed )
{
    rng_t rng;
    rng_seed( &rng, seed );
    for ( uint32_t i = 0; i < n; i++ )
        for ( int a = 0; a < 3; a++ )
            atoms[ 4 * i + a ] = (float)( (double)atoms[ 4 * i + a ] + sigma * rng_gauss( &rng ) );
}

/* uniform doubles in [0, 1) from the same generator (used for batch sizes and queries) */
void sesgb_synth_uniform( uint64_t seed, uint32_t count, double * out )
{
    rng_t rng;
    rng_seed( &rng, seed );
    for ( uint32_t i = 0; i < count; i++ )
        out[ i ] = rng_uniform( &rng );
}

/* Query points for the SDF: uniform in the atoms' bounding box (getAabb:
 * min(c - r), max(c + r)), kept when |min_i(|x - c_i| - r_i)| <= band. Draws
 * until m points are kept (at most 10000 m draws); returns the number kept. */
uint32_t sesgb_synth_queries( const float * atoms, uint32_t n, uint32_t m, uint64_t seed, float band, float * out )
{
    if ( n == 0 || m == 0 )
        return 0;
    double lo[ 3 ] = { 1e300, 1e300, 1e300 }, hi[ 3 ] = { -1e300, -1e300, -1e300 }, rmax = 0.0;
    for ( uint32_t i = 0; i < n; i++ )
        for ( int a = 0; a < 3; a++ )
        {
            const double c = atoms[ 4 * i + a ], r = atoms[ 4 * i + 3 ];
            lo[ a ]        = c - r < lo[ a ] ? c - r : lo[ a ];
            hi[ a ]        = c + r > hi[ a ] ? c + r : hi[ a ];
            rmax           = r > rmax ? r : rmax;
        }
    /* cell grid over the box, cell >= band + rmax: the 27 cells around x hold every atom within band of its surface */
    const double h = (double)band + rmax + 1e-3;
    int          dims[ 3 ];
    for ( int a = 0; a < 3; a++ )
    {
        dims[ a ] = (int)( ( hi[ a ] - lo[ a ] ) / h ) + 1;
        if ( dims[ a ] < 1 )
            dims[ a ] = 1;
    }
    const uint64_t cells = (uint64_t)dims[ 0 ] * dims[ 1 ] * dims[ 2 ];
    uint32_t *     start = (uint32_t *)calloc( cells + 1, sizeof( uint32_t ) );
    uint32_t *     item  = (uint32_t *)malloc( sizeof( uint32_t ) * n );
    uint32_t *     cell  = (uint32_t *)malloc( sizeof( uint32_t ) * n );
    if ( !start || !item || !cell )
    {
        free( start );
        free( item );
        free( cell );
        return 0;
    }
    for ( uint32_t i = 0; i < n; i++ )
    {
        int c[ 3 ];
        for ( int a = 0; a < 3; a++ )
        {
            c[ a ] = (int)( ( atoms[ 4 * i + a ] - lo[ a ] ) / h );
            c[ a ] = c[ a ] < 0 ? 0 : ( c[ a ] >= dims[ a ] ? dims[ a ] - 1 : c[ a ] );
        }
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
    rng_t    r;
    uint32_t kept = 0;
    rng_seed( &r, seed );
    for ( uint64_t draw = 0; kept < m && draw < 10000ull * m; draw++ )
    {
        float x[ 3 ];
        int   c[ 3 ];
        for ( int a = 0; a < 3; a++ )
        {
            x[ a ] = (float)( lo[ a ] + ( hi[ a ] - lo[ a ] ) * rng_uniform( &r ) );
            c[ a ] = (int)( ( x[ a ] - lo[ a ] ) / h );
            c[ a ] = c[ a ] < 0 ? 0 : ( c[ a ] >= dims[ a ] ? dims[ a ] - 1 : c[ a ] );
        }
        double best = 1e300;
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
                        const double   ex = (double)x[ 0 ] - atoms[ 4 * i ], ey = (double)x[ 1 ] - atoms[ 4 * i + 1 ],
                                     ez = (double)x[ 2 ] - atoms[ 4 * i + 2 ];
                        const double d = sqrt( ex * ex + ey * ey + ez * ez ) - atoms[ 4 * i + 3 ];
                        best           = d < best ? d : best;
                    }
                }
        if ( best <= (double)band && best >= -(double)band )
        {
            out[ 3 * kept + 0 ] = x[ 0 ];
            out[ 3 * kept + 1 ] = x[ 1 ];
            out[ 3 * kept + 2 ] = x[ 2 ];
            kept++;
        }
    }
    free( start );
    free( item );
    free( cell );
    return kept;
}
