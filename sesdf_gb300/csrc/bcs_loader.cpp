// bcs_loader.cpp -- atoms of an MMTF structure file, host side: sesgb_load_mmtf (C ABI) and
// bcs::load (the reference's loader, sesdf/src/core/loader.cpp:14-71, for MMTF files).
//
// The reference reads a structure through chemfiles: the atoms of the first frame, residue by
// residue in file order, each with the vdW radius of its element (bcs::getRadius,
// sesdf/src/core/molecule.cpp:9-131; the symbol is upper-cased and looked up as the enumerator
// "A_<symbol>" of bcs::SYMBOL, sesdf/include/bcs/core/molecule.hpp:13-140, an unknown symbol taking
// the UNKNOWN radius). The MessagePack container and the binary codecs are decoded here from the MMTF
// 1.0 specification; coordinates are the file's integers divided by the codec parameter in float32.
// Portable C++17: bytes are read as uint8_t and assembled big-endian by shifts.
#include <cctype>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bcs/core/loader.hpp"
#include "sesgb.h"

namespace
{
    // bcs::SYMBOL in enumerator order (index = atomic number, 0 = UNKNOWN); the codes past 104
    // are the reference's own and kept so that the lookup answers the same
    const char * const kSymbols[] = {
        "UNKNOWN", "H",  "HE", "LI", "BE", "B",  "C",  "N",  "O",  "F",  "NE", "NA", "MG", "AL", "SI", "P",   "S",
        "CL",      "AR", "K",  "CA", "SC", "TI", "V",  "CR", "MN", "FE", "CO", "NI", "CU", "ZN", "GA", "GE",  "AS",
        "SE",      "BR", "KR", "RB", "SR", "Y",  "ZR", "NB", "MO", "TC", "RU", "RH", "PD", "AG", "CD", "IN",  "SN",
        "SB",      "TE", "I",  "XE", "CS", "BA", "LA", "CE", "PR", "ND", "PM", "SM", "EU", "GD", "TB", "DY",  "HO",
        "ER",      "TM", "YB", "LU", "HF", "TA", "W",  "RE", "OS", "IR", "PT", "AU", "HG", "TL", "PB", "BI",  "PO",
        "AT",      "RN", "FR", "RA", "AC", "TH", "PA", "U",  "NP", "PU", "AM", "CM", "BK", "CF", "ES", "FM",  "MD",
        "NO",      "LR", "RF", "DD", "SG", "BHJ", "HS", "MT", "DS", "RG", "UUB", "UUT", "UUQ", "UUP", "UUH", "UUS", "UUO" };
    // vdW radius (A) by the index above, as bcs::getRadius returns it (0 where the reference has none)
    const float kRadius[] = {
        1.20f, 1.20f, 1.43f, 2.12f, 1.98f, 1.91f, 1.77f, 1.66f, 1.50f, 1.46f, 1.58f, 2.50f, 2.51f, 2.25f, 2.19f, 1.90f,
        1.89f, 1.82f, 1.83f, 2.73f, 2.62f, 2.58f, 2.46f, 2.42f, 2.45f, 2.45f, 2.44f, 2.40f, 2.40f, 2.38f, 2.39f, 2.32f,
        2.29f, 1.88f, 1.82f, 1.86f, 2.25f, 3.21f, 2.84f, 2.75f, 2.52f, 2.56f, 2.45f, 2.44f, 2.46f, 2.44f, 2.15f, 2.53f,
        2.49f, 2.43f, 2.42f, 2.47f, 1.99f, 2.04f, 2.06f, 3.48f, 3.03f, 2.98f, 2.88f, 2.92f, 2.95f, 0.00f, 2.90f, 2.87f,
        2.83f, 2.79f, 2.87f, 2.81f, 2.83f, 2.79f, 2.80f, 2.74f, 2.63f, 2.53f, 2.57f, 2.49f, 2.48f, 2.41f, 2.29f, 2.32f,
        2.45f, 2.47f, 2.60f, 2.54f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 2.80f, 2.93f, 2.88f, 2.71f, 2.82f, 2.81f, 2.83f,
        3.05f, 3.40f, 3.05f, 2.70f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f,
        0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f, 0.00f };
    static_assert( sizeof( kSymbols ) / sizeof( kSymbols[ 0 ] ) == 119, "119 enumerators" );
    static_assert( sizeof( kRadius ) / sizeof( kRadius[ 0 ] ) == 119, "one radius per enumerator" );

    float radius_of( const std::string & symbol )
    {
        std::string up = symbol;
        for ( char & c : up )
            c = (char)std::toupper( (unsigned char)c );
        for ( int k = 1; k < 119; k++ )
            if ( up == kSymbols[ k ] )
                return kRadius[ k ];
        return kRadius[ 0 ];
    }

    // ---- MessagePack (the forms MMTF uses) ---------------------------------------------------
    struct Value
    {
        enum Kind
        {
            Nil,
            Bool,
            Int,
            Float,
            Str,
            Bin,
            Array,
            Map
        } kind = Nil;
        int64_t                                   i = 0;
        double                                    f = 0.0;
        std::string                               s; // Str, and Bin bytes
        std::vector<Value>                        arr;
        std::vector<std::pair<std::string, Value>> map;

        const Value * get( const char * key ) const
        {
            for ( const auto & kv : map )
                if ( kv.first == key )
                    return &kv.second;
            return nullptr;
        }
    };

    struct Reader
    {
        const uint8_t * p;
        size_t          n, at = 0;

        const uint8_t * take( size_t k )
        {
            if ( k > n - at )
                throw std::runtime_error( "truncated MessagePack data" );
            const uint8_t * q = p + at;
            at += k;
            return q;
        }
        uint64_t be( size_t k )
        {
            const uint8_t * q = take( k );
            uint64_t        v = 0;
            for ( size_t j = 0; j < k; j++ )
                v = ( v << 8 ) | q[ j ];
            return v;
        }
        int64_t sbe( size_t k )
        {
            const uint64_t v = be( k );
            const int      s = 64 - 8 * (int)k;
            return (int64_t)( v << s ) >> s; // sign-extend the k-byte value
        }
        Value value( int depth = 0 )
        {
            if ( depth > 64 )
                throw std::runtime_error( "MessagePack nesting too deep" );
            Value         v;
            const uint8_t t = *take( 1 );
            auto          str = [ & ]( size_t k ) {
                const uint8_t * q = take( k );
                return std::string( reinterpret_cast<const char *>( q ), k );
            };
            auto array = [ & ]( uint64_t k ) {
                v.kind = Value::Array;
                for ( uint64_t j = 0; j < k; j++ )
                    v.arr.push_back( value( depth + 1 ) );
            };
            auto dict = [ & ]( uint64_t k ) {
                v.kind = Value::Map;
                for ( uint64_t j = 0; j < k; j++ )
                {
                    Value key = value( depth + 1 );
                    Value val = value( depth + 1 );
                    v.map.emplace_back( key.s, std::move( val ) );
                }
            };
            if ( t <= 0x7F )
                v.kind = Value::Int, v.i = t;
            else if ( t >= 0xE0 )
                v.kind = Value::Int, v.i = (int64_t)t - 0x100;
            else if ( t <= 0x8F )
                dict( t & 0x0F );
            else if ( t <= 0x9F )
                array( t & 0x0F );
            else if ( t <= 0xBF )
                v.kind = Value::Str, v.s = str( t & 0x1F );
            else
                switch ( t )
                {
                case 0xC0: break;
                case 0xC2:
                case 0xC3: v.kind = Value::Bool, v.i = t == 0xC3; break;
                case 0xC4: v.kind = Value::Bin, v.s = str( be( 1 ) ); break;
                case 0xC5: v.kind = Value::Bin, v.s = str( be( 2 ) ); break;
                case 0xC6: v.kind = Value::Bin, v.s = str( be( 4 ) ); break;
                case 0xCA:
                {
                    const uint32_t b = (uint32_t)be( 4 );
                    float          f;
                    std::memcpy( &f, &b, 4 );
                    v.kind = Value::Float, v.f = f;
                    break;
                }
                case 0xCB:
                {
                    const uint64_t b = be( 8 );
                    std::memcpy( &v.f, &b, 8 );
                    v.kind = Value::Float;
                    break;
                }
                case 0xCC: v.kind = Value::Int, v.i = (int64_t)be( 1 ); break;
                case 0xCD: v.kind = Value::Int, v.i = (int64_t)be( 2 ); break;
                case 0xCE: v.kind = Value::Int, v.i = (int64_t)be( 4 ); break;
                case 0xCF: v.kind = Value::Int, v.i = (int64_t)be( 8 ); break;
                case 0xD0: v.kind = Value::Int, v.i = sbe( 1 ); break;
                case 0xD1: v.kind = Value::Int, v.i = sbe( 2 ); break;
                case 0xD2: v.kind = Value::Int, v.i = sbe( 4 ); break;
                case 0xD3: v.kind = Value::Int, v.i = sbe( 8 ); break;
                case 0xD9: v.kind = Value::Str, v.s = str( be( 1 ) ); break;
                case 0xDA: v.kind = Value::Str, v.s = str( be( 2 ) ); break;
                case 0xDB: v.kind = Value::Str, v.s = str( be( 4 ) ); break;
                case 0xDC: array( be( 2 ) ); break;
                case 0xDD: array( be( 4 ) ); break;
                case 0xDE: dict( be( 2 ) ); break;
                case 0xDF: dict( be( 4 ) ); break;
                default: throw std::runtime_error( "MessagePack type not used by MMTF" );
                }
            return v;
        }
    };

    // ---- MMTF codecs (12-byte big-endian header: codec, length, parameter) --------------------
    int64_t be_int( const std::string & b, size_t at, size_t k )
    {
        uint64_t v = 0;
        for ( size_t j = 0; j < k; j++ )
            v = ( v << 8 ) | (uint8_t)b[ at + j ];
        const int s = 64 - 8 * (int)k;
        return (int64_t)( v << s ) >> s;
    }

    struct Decoded
    {
        std::vector<int64_t> ints;   // integer codecs
        std::vector<float>   floats; // float codecs
    };

    Decoded decode( const std::string & b )
    {
        if ( b.size() < 12 )
            throw std::runtime_error( "MMTF binary field shorter than its header" );
        const int32_t codec = (int32_t)be_int( b, 0, 4 ), length = (int32_t)be_int( b, 4, 4 ),
                      param = (int32_t)be_int( b, 8, 4 );
        const size_t body = b.size() - 12;
        auto         ints = [ & ]( size_t k ) {
            std::vector<int64_t> v( body / k );
            for ( size_t j = 0; j < v.size(); j++ )
                v[ j ] = be_int( b, 12 + j * k, k );
            return v;
        };
        auto run_length = []( const std::vector<int64_t> & pairs ) {
            std::vector<int64_t> v;
            for ( size_t j = 0; j + 1 < pairs.size(); j += 2 )
                for ( int64_t c = 0; c < pairs[ j + 1 ]; c++ )
                    v.push_back( pairs[ j ] );
            return v;
        };
        auto recursive = []( const std::vector<int64_t> & in, int64_t lo, int64_t hi ) {
            std::vector<int64_t> v;
            int64_t              acc = 0;
            for ( int64_t x : in )
            {
                acc += x;
                if ( x != lo && x != hi )
                {
                    v.push_back( acc );
                    acc = 0;
                }
            }
            return v;
        };
        auto divide = [ & ]( const std::vector<int64_t> & in ) {
            std::vector<float> v( in.size() );
            for ( size_t j = 0; j < in.size(); j++ )
                v[ j ] = (float)in[ j ] / (float)param;
            return v;
        };
        Decoded d;
        switch ( codec )
        {
        case 1:
        {
            for ( int64_t x : ints( 4 ) )
            {
                const uint32_t u = (uint32_t)x;
                float          f;
                std::memcpy( &f, &u, 4 );
                d.floats.push_back( f );
            }
            break;
        }
        case 2: d.ints = ints( 1 ); break;
        case 3: d.ints = ints( 2 ); break;
        case 4: d.ints = ints( 4 ); break;
        case 7: d.ints = run_length( ints( 4 ) ); break;
        case 8:
        {
            d.ints = run_length( ints( 4 ) );
            for ( size_t j = 1; j < d.ints.size(); j++ )
                d.ints[ j ] += d.ints[ j - 1 ];
            break;
        }
        case 9: d.floats = divide( run_length( ints( 4 ) ) ); break;
        case 10:
        {
            std::vector<int64_t> v = recursive( ints( 2 ), -32768, 32767 );
            for ( size_t j = 1; j < v.size(); j++ )
                v[ j ] += v[ j - 1 ];
            d.floats = divide( v );
            break;
        }
        case 11: d.floats = divide( ints( 2 ) ); break;
        case 12: d.floats = divide( recursive( ints( 2 ), -32768, 32767 ) ); break;
        case 13: d.ints = recursive( ints( 1 ), -128, 127 ); break;
        case 14: d.ints = recursive( ints( 2 ), -32768, 32767 ); break;
        default: throw std::runtime_error( "MMTF codec not supported" );
        }
        const size_t got = d.ints.size() + d.floats.size();
        if ( got != (size_t)length )
            throw std::runtime_error( "MMTF codec length differs from its header" );
        return d;
    }

    std::vector<float> float_field( const Value & doc, const char * key )
    {
        const Value * v = doc.get( key );
        if ( !v || v->kind != Value::Bin )
            throw std::runtime_error( std::string( "MMTF field missing: " ) + key );
        Decoded d = decode( v->s );
        if ( d.floats.empty() && !d.ints.empty() )
            throw std::runtime_error( std::string( "MMTF field is not a float list: " ) + key );
        return d.floats;
    }

    std::vector<int64_t> int_field( const Value & doc, const char * key )
    {
        const Value * v = doc.get( key );
        if ( !v )
            throw std::runtime_error( std::string( "MMTF field missing: " ) + key );
        if ( v->kind == Value::Bin )
            return decode( v->s ).ints;
        std::vector<int64_t> out;
        if ( v->kind != Value::Array )
            throw std::runtime_error( std::string( "MMTF field is not a list: " ) + key );
        for ( const Value & x : v->arr )
            out.push_back( x.i );
        return out;
    }

    // atoms (x, y, z, r) of the first model
    std::vector<float> load_atoms( const uint8_t * data, size_t size )
    {
        if ( size >= 2 && data[ 0 ] == 0x1F && data[ 1 ] == 0x8B )
            throw std::runtime_error( "gzip-compressed MMTF: decompress it first" );
        Reader      r { data, size };
        const Value doc = r.value();
        if ( doc.kind != Value::Map || !doc.get( "xCoordList" ) )
            throw std::runtime_error( "not an MMTF document" );
        const std::vector<float>   x = float_field( doc, "xCoordList" ), y = float_field( doc, "yCoordList" ),
                                 z = float_field( doc, "zCoordList" );
        const std::vector<int64_t> types = int_field( doc, "groupTypeList" );
        const std::vector<int64_t> chainsPerModel = int_field( doc, "chainsPerModel" );
        const std::vector<int64_t> groupsPerChain = int_field( doc, "groupsPerChain" );
        const Value *              groups = doc.get( "groupList" );
        if ( !groups || groups->kind != Value::Array )
            throw std::runtime_error( "MMTF field missing: groupList" );
        int64_t nGroups = 0;
        if ( !chainsPerModel.empty() )
            for ( int64_t c = 0; c < chainsPerModel[ 0 ] && c < (int64_t)groupsPerChain.size(); c++ )
                nGroups += groupsPerChain[ (size_t)c ];
        std::vector<float> out;
        size_t             a = 0;
        for ( int64_t g = 0; g < nGroups && g < (int64_t)types.size(); g++ )
        {
            const int64_t t = types[ (size_t)g ];
            if ( t < 0 || t >= (int64_t)groups->arr.size() )
                throw std::runtime_error( "MMTF group type out of range" );
            const Value * el = groups->arr[ (size_t)t ].get( "elementList" );
            if ( !el || el->kind != Value::Array )
                throw std::runtime_error( "MMTF group without elementList" );
            for ( const Value & e : el->arr )
            {
                if ( a >= x.size() || a >= y.size() || a >= z.size() )
                    throw std::runtime_error( "MMTF groups hold more atoms than the coordinate lists" );
                out.insert( out.end(), { x[ a ], y[ a ], z[ a ], radius_of( e.s ) } );
                a++;
            }
        }
        return out;
    }
} // namespace

namespace bcs
{
    Molecule load( const std::string & path )
    {
        std::ifstream f( path, std::ios::binary );
        if ( !f )
            throw std::runtime_error( "cannot open " + path );
        const std::vector<uint8_t> bytes( ( std::istreambuf_iterator<char>( f ) ), std::istreambuf_iterator<char>() );
        const std::vector<float>   a = load_atoms( bytes.data(), bytes.size() );
        Molecule                   m;
        m.reserve( a.size() / 4 );
        for ( size_t i = 0; i + 3 < a.size(); i += 4 )
            m.emplace_back( Vec4f { a[ i ], a[ i + 1 ], a[ i + 2 ], a[ i + 3 ] } );
        return m;
    }
} // namespace bcs

extern "C" int sesgb_load_mmtf( const void * data, size_t size, float * atoms, uint32_t capacity, uint32_t * n )
{
    if ( !data || !n || ( capacity && !atoms ) )
        return SESGB_ERR_INVALID;
    try
    {
        const std::vector<float> a = load_atoms( static_cast<const uint8_t *>( data ), size );
        *n                         = (uint32_t)( a.size() / 4 );
        if ( *n > capacity )
            return SESGB_ERR_OVERFLOW;
        if ( !a.empty() )
            std::memcpy( atoms, a.data(), a.size() * sizeof( float ) );
        return SESGB_OK;
    }
    catch ( const std::exception & )
    {
        *n = 0;
        return SESGB_ERR_INVALID;
    }
}
