// bcs/cuda/memory.hpp -- DeviceBuffer of the drop-in API.
// The reference's DeviceBuffer (sesdf/include/bcs/cuda/memory.cuh:119-161) owns
// stream-ordered device memory; here the build owns all memory and a
// DeviceBuffer is a typed view of one of its buffers, with the same accessors.
#ifndef BCS_CUDA_MEMORY_HPP
#define BCS_CUDA_MEMORY_HPP

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime_api.h>

namespace bcs
{
    class DeviceBuffer
    {
      public:
        DeviceBuffer() = default;
        DeviceBuffer( void * ptr, std::size_t bytes ) : m_ptr( static_cast<uint8_t *>( ptr ) ), m_size( bytes ) {}

        uint8_t *       get() { return m_ptr; }
        const uint8_t * get() const { return m_ptr; }
        template<class Type> Type *       get( std::size_t offset = 0 ) { return reinterpret_cast<Type *>( m_ptr + offset ); }
        template<class Type> const Type * get( std::size_t offset = 0 ) const
        {
            return reinterpret_cast<const Type *>( m_ptr + offset );
        }

        explicit operator bool() const { return m_ptr != nullptr; }
        std::size_t size() const { return m_size; }
        template<class Type> std::size_t size() const { return m_size / sizeof( Type ); }

        template<class Type> std::vector<Type> toHost() const
        {
            std::vector<Type> out( m_size / sizeof( Type ) );
            if ( !out.empty() )
                cudaMemcpy( out.data(), m_ptr, out.size() * sizeof( Type ), cudaMemcpyDeviceToHost );
            return out;
        }

      private:
        uint8_t *   m_ptr  = nullptr;
        std::size_t m_size = 0;
    };
} // namespace bcs

#endif // BCS_CUDA_MEMORY_HPP
