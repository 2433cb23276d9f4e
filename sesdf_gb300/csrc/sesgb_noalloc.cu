// sesgb_noalloc.cu -- reference-grid atom sort that allocates no memory.
//
// Some callers cannot allocate device memory at the time they need the sort:
// a plugin whose host application owns a fixed device-memory budget and hands
// it every buffer, or a real-time loop that must never enter the allocator
// (cudaMalloc can synchronise the device and take milliseconds). For them,
// sesgb_sort_atoms_noalloc sorts atoms into the order of the build's `atoms`
// output (the reference grid's stable cell order, the order getAtomIndices()
// describes) using only the buffers the caller passes plus one fixed scratch
// array that lives in this library's device image.
//
// The scratch array below is a file-scope __device__ array: every GPU that
// loads the library keeps its SESGB_NOALLOC_MAX_ATOMS-sized copy (about 3.3 MB)
// until the process exits. Host code must not use the array's symbol as a
// device address; the device address is fetched once per device with
// cudaGetSymbolAddress (the first call of the entry point on a device does it,
// with that device current) and passed to the kernels. The stored address
// belongs to the device's context of that moment: resetting the device
// (cudaDeviceReset) while the library is loaded is not supported. Every call
// on a device shares the one array and leaves its contents behind: two calls
// whose work overlaps on the GPU (different streams, or different host threads
// on one device) race on it and must be serialised by the caller. No part of
// the scratch has to start at zero (every pass writes the whole histogram and
// key arrays it reads afterwards).
#include <cstring>
#include <mutex>

#include "../../include/sesgb.h"
#include "sesgb_internal.h"

namespace sesgb
{
    namespace
    {
        constexpr uint32_t kMaxAtoms = SESGB_NOALLOC_MAX_ATOMS;
        // keys (n) + radix ping-pong (2n) + digit histogram (256 x tiles + 1) + tile sums
        constexpr size_t kRadixTile    = 2048;
        constexpr size_t kTiles        = ( kMaxAtoms + kRadixTile - 1 ) / kRadixTile;
        constexpr size_t align256( size_t b ) { return ( b + 255 ) & ~(size_t)255; }
        constexpr size_t kKeyBytes     = align256( (size_t)kMaxAtoms * 4 );
        constexpr size_t kScratchBytes = kKeyBytes + align256( 2ull * kMaxAtoms * 4 ) + align256( ( 256 * kTiles + 1 ) * 4 )
                                         + align256( ( ( 256 * kTiles + 2047 ) / 2048 + 1 ) * 4 ) + 4096;

        static __device__ __align__( 256 ) unsigned char g_noallocScratch[ kScratchBytes ];

        constexpr int kMaxDevices = 64;
        std::mutex    g_setupLock;
        void *        g_scratch[ kMaxDevices ] = {};

        // device address of the scratch array on the current device (set up once per device)
        cudaError_t scratch_address( void ** out )
        {
            int dev = 0;
            cudaError_t e = cudaGetDevice( &dev );
            if ( e != cudaSuccess )
                return e;
            if ( dev < 0 || dev >= kMaxDevices )
                return cudaErrorInvalidDevice;
            std::lock_guard<std::mutex> g( g_setupLock );
            if ( !g_scratch[ dev ] )
            {
                void * p = nullptr;
                e        = cudaGetSymbolAddress( &p, g_noallocScratch );
                if ( e != cudaSuccess )
                    return e;
                g_scratch[ dev ] = p;
            }
            *out = g_scratch[ dev ];
            return cudaSuccess;
        }

        __global__ void k_noalloc_hash( const float4 * atoms, uint32_t n, GridRef grid, uint32_t * keys, uint32_t * order )
        {
            const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
            if ( i >= n )
                return;
            const float4 a = atoms[ i ];
            keys[ i ]      = ref_grid_hash( grid, ref_grid_position( grid, a.x, a.y, a.z ) );
            order[ i ]     = i;
        }

        __global__ void k_noalloc_gather( const float4 * atoms, const uint32_t * order, uint32_t n, float4 * sorted )
        {
            const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
            if ( s < n )
                sorted[ s ] = atoms[ order[ s ] ];
        }
    } // namespace
} // namespace sesgb

using namespace sesgb;

extern "C" int sesgb_sort_atoms_noalloc( const void * device_atoms, uint32_t n, const float * aabb, float probe_radius,
                                         void * device_sorted_atoms, uint32_t * device_sorted_to_input, void * stream )
{
    if ( n > kMaxAtoms )
        return SESGB_ERR_TOO_LARGE;
    if ( !aabb || !( probe_radius >= 0.f ) || ( n && ( !device_atoms || !device_sorted_atoms || !device_sorted_to_input ) ) )
        return SESGB_ERR_INVALID;
    if ( radix_scratch_bytes( n ) > kScratchBytes - kKeyBytes )
        return SESGB_ERR_TOO_LARGE;
    void * scratch = nullptr;
    if ( scratch_address( &scratch ) != cudaSuccess )
        return SESGB_ERR_CUDA;
    if ( n == 0 )
        return SESGB_OK;
    // a launch error left pending on this thread by earlier work is returned here, before anything
    // is launched, so that the check after the launches below judges only this call's own
    if ( cudaGetLastError() != cudaSuccess )
        return SESGB_ERR_CUDA;

    // reference grid of Sesdf::Sesdf (sesdf/src/sesdf/sesdf.cu:23-33)
    GridRef        grid;
    const float    maxVdw = 3.48f;
    uint64_t       e = 0, v = n;
    while ( v >>= 1 )
        e++;
    uint32_t gs = 1;
    while ( e > gs )
        gs <<= 1;
    for ( int a = 0; a < 3; a++ )
    {
        const float origin = ( aabb[ a ] - maxVdw ) - probe_radius;
        float       size   = ( ( aabb[ 3 + a ] + maxVdw ) + probe_radius ) - origin;
        size               = size < 0.f ? -size : size;
        ( &grid.origin.x )[ a ] = origin;
        ( &grid.cell.x )[ a ]   = size / (float)gs;
    }
    grid.size  = (int)gs;
    int bits   = 0;
    for ( uint32_t g = gs; g > 1; g >>= 1 )
        bits += 3;

    cudaStream_t s    = static_cast<cudaStream_t>( stream );
    uint32_t *   keys = static_cast<uint32_t *>( scratch );
    void *       rad  = static_cast<unsigned char *>( scratch ) + kKeyBytes;
    const uint32_t blocks = ( n + 255 ) / 256;
    k_noalloc_hash<<<blocks, 256, 0, s>>>( static_cast<const float4 *>( device_atoms ), n, grid, keys, device_sorted_to_input );
    radix_sort( keys, device_sorted_to_input, n, bits, rad, s );
    k_noalloc_gather<<<blocks, 256, 0, s>>>( static_cast<const float4 *>( device_atoms ), device_sorted_to_input, n,
                                            static_cast<float4 *>( device_sorted_atoms ) );
    count_launches( 2 );
    return cudaGetLastError() == cudaSuccess ? SESGB_OK : SESGB_ERR_CUDA;
}
