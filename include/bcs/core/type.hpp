// bcs/core/type.hpp -- span types of the drop-in API (sesdf/include/bcs/core/type.hpp:9-53).
#ifndef BCS_CORE_TYPE_HPP
#define BCS_CORE_TYPE_HPP

#include <cstddef>
#include <vector>

namespace bcs
{
    template<class Type> struct Span
    {
        Type *      ptr  = nullptr;
        std::size_t size = 0;
        Span()           = default;
        Span( Type * p, std::size_t s ) : ptr( p ), size( s ) {}
        Span( std::vector<Type> & data ) : ptr( data.data() ), size( data.size() ) {}
    };

    template<class Type> struct ConstSpan
    {
        const Type * ptr  = nullptr;
        std::size_t  size = 0;
        ConstSpan()       = default;
        ConstSpan( const Type * p, std::size_t s ) : ptr( p ), size( s ) {}
        ConstSpan( const std::vector<Type> & data ) : ptr( data.data() ), size( data.size() ) {}
        ConstSpan( const Span<Type> data ) : ptr( data.ptr ), size( data.size ) {}
    };

    template<class HandleType> struct HandleSpan
    {
        HandleType  handle {};
        std::size_t offset = 0;
        std::size_t size   = 0;
        HandleSpan()       = default;
        HandleSpan( HandleType h, std::size_t o, std::size_t s ) : handle( h ), offset( o ), size( s ) {}
        HandleSpan( HandleType h, std::size_t s ) : handle( h ), offset( 0 ), size( s ) {}
    };

    template<class Type> struct RangeBase
    {
        Type start;
        Type end;
        Type size() const { return end - start; }
    };
    using Range = RangeBase<std::size_t>;
} // namespace bcs

#endif // BCS_CORE_TYPE_HPP
